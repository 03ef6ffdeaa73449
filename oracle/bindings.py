"""ctypes bindings of the CPU restatement (oracle/liboracle.so) and, when it
was built from the reference's sources on this machine, of the reference
harness (oracle/_ref/libhelp_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the help_gb300 package.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libhelp_ref.so")
REF_BIN = os.path.join(HERE, "_ref", "help_ref")
REF_LINDEP_BIN = os.path.join(HERE, "_ref", "help_ref_lindep")

PIVOT_GREEDY = 0
PIVOT_GIVEN = 1

_lib = None
_ref = None


def P(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


class Pchol(C.Structure):
    _fields_ = [("m", C.c_int), ("k", C.c_int), ("perm", C.POINTER(C.c_int)), ("L", C.POINTER(C.c_double)),
                ("D", C.POINTER(C.c_double)), ("diag_s", C.POINTER(C.c_double)),
                ("l11inv", C.POINTER(C.c_double)), ("beg", C.POINTER(C.c_int)), ("end", C.POINTER(C.c_int))]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            raise RuntimeError("oracle not built: make -C oracle")
        L = C.CDLL(ORACLE_SO)
        vp = C.c_void_p
        L.oracle_csrmv_n.argtypes = [C.c_int, C.c_int, C.c_double, vp, vp, vp, vp, vp, C.c_double, vp]
        L.oracle_csrmv_t.argtypes = [C.c_int, C.c_int, C.c_double, vp, vp, vp, vp, vp, C.c_double, vp]
        L.oracle_adat_symbolic.argtypes = [C.c_int, C.c_int, vp, vp, vp, vp, vp, vp]
        L.oracle_adat_symbolic.restype = C.c_int64
        L.oracle_adat_numeric.argtypes = [C.c_int, C.c_int] + [vp] * 10
        L.oracle_adat_numeric_threads.argtypes = [C.c_int, C.c_int] + [vp] * 10 + [C.c_int]
        L.oracle_adat_numeric_threads.restype = C.c_int
        L.oracle_pchol_build.argtypes = [C.c_int, C.c_int, vp, vp, vp, vp, C.c_double, C.c_double, C.c_int, C.c_int,
                                         vp, C.POINTER(Pchol)]
        L.oracle_pchol_free.argtypes = [C.POINTER(Pchol)]
        L.oracle_precond_apply.argtypes = [C.POINTER(Pchol), vp, vp]
        L.oracle_pcg.argtypes = [C.c_int, C.c_int, vp, vp, vp, vp, C.c_double, C.c_double, vp, vp, C.c_int, C.c_int,
                                 vp, C.c_double, C.c_int64]
        L.oracle_pcg.restype = C.c_int64
        L.oracle_ne_create.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int64]
        L.oracle_ne_create.restype = vp
        L.oracle_ne_construct.argtypes = [vp, C.c_int32, C.c_int32, vp, vp, vp]
        L.oracle_ne_renew.argtypes = [vp, vp]
        L.oracle_ne_solve.argtypes = [vp, vp, vp, vp, vp, vp]
        L.oracle_ne_destruct.argtypes = [vp]
        L.oracle_ne_free.argtypes = [vp]
        L.oracle_ne_free.restype = None
        L.oracle_ne_last_iters.argtypes = [vp]
        L.oracle_ne_last_iters.restype = C.c_int64
        L.oracle_ne_total_iters.argtypes = [vp]
        L.oracle_ne_total_iters.restype = C.c_int64
        L.oracle_topk_pivots.argtypes = [C.c_int, vp, C.c_int, vp]
        L.oracle_diag_adat.argtypes = [C.c_int, vp, vp, vp, vp, C.c_double, C.c_double, vp]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref_lindep_available() -> bool:
    return os.path.exists(REF_LINDEP_BIN)


def ref_lindep(mps_path: str, timeout: float = 600.0) -> dict:
    """The reference's own dependent-row presolve (Presolve_Lindep.cpp with its
    LUSOL, oracle/ref/ref_lindep.cpp) on one MPS file: {"rows", "dependent",
    "status" (0 ok, 1 primal infeasible), "disabled"}, or {"error": ...} when
    the reference program stops (LUSOL's fixed factor space runs out on
    near-square random matrices: LUSOL_ANEEDMEM)."""
    import json
    import subprocess

    r = subprocess.run([REF_LINDEP_BIN, mps_path], capture_output=True, text=True, timeout=timeout)
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    if r.returncode != 0 or not lines:
        tail = (r.stdout + r.stderr).strip().splitlines()
        return {"error": "exit %d: %s" % (r.returncode, tail[-1] if tail else "")}
    return json.loads(lines[-1])


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_SO)
        vp = C.c_void_p
        R.ref_load.argtypes = [C.c_int, C.c_int, vp, vp, vp]
        R.ref_solve.argtypes = [vp] * 5
        R.ref_solve.restype = C.c_longlong
        R.ref_csrmv_n.argtypes = [C.c_int, C.c_int, C.c_double, vp, vp, vp, vp, vp, C.c_double, vp]
        R.ref_csrmv_t.argtypes = [C.c_int, C.c_int, C.c_double, vp, vp, vp, vp, vp, C.c_double, vp]
        R.ref_pchol.argtypes = [vp, C.c_double, C.c_double, vp, vp, vp, vp]
        R.ref_precond.argtypes = [vp, vp]
        R.ref_adat.argtypes = [vp, vp, vp, vp, C.c_int]
        R.ref_pchol_cols.restype = C.c_int
        R.ref_construct.restype = C.c_int
        _ref = R
    return _ref


# ---------------------------------------------------------------- helpers

def csrmv_n(rp, ci, v, x, m, n, alpha=1.0, beta=0.0, y=None):
    y = np.zeros(m) if y is None else y.copy()
    beg, end = np.ascontiguousarray(rp[:-1]), np.ascontiguousarray(rp[1:])  # keep alive across the call
    x = np.ascontiguousarray(x, dtype=np.float64)
    lib().oracle_csrmv_n(m, n, alpha, P(v), P(ci), P(beg), P(end), P(x), beta, P(y))
    return y


def csrmv_t(rp, ci, v, x, m, n, alpha=1.0, beta=0.0, y=None):
    y = np.zeros(n) if y is None else y.copy()
    beg, end = np.ascontiguousarray(rp[:-1]), np.ascontiguousarray(rp[1:])
    x = np.ascontiguousarray(x, dtype=np.float64)
    lib().oracle_csrmv_t(m, n, alpha, P(v), P(ci), P(beg), P(end), P(x), beta, P(y))
    return y


def diag_adat(rp, ci, v, d, m, gamma=0.0, delta=0.0):
    out = np.zeros(m)
    lib().oracle_diag_adat(m, P(rp), P(ci), P(v), P(d), gamma, delta, P(out))
    return out


def adat(rp, ci, v, col_ptr, row_ind, val, w, m, n):
    """Upper triangle of A diag(w) A^T: ADAt_Allocate + ADAt_Calc restated
    (Helper.cpp:215-377).  Returns (row_ptr, col, val) with the columns of
    every row sorted (the restatement keeps the reference's pattern order;
    the values are the reference's sums, in its order, unchanged)."""
    orp = np.zeros(m + 1, np.int32)
    nnz = lib().oracle_adat_symbolic(m, n, P(rp), P(ci), P(col_ptr), P(row_ind), P(orp), None)
    ocol = np.zeros(max(nnz, 1), np.int32)
    lib().oracle_adat_symbolic(m, n, P(rp), P(ci), P(col_ptr), P(row_ind), P(orp), P(ocol))
    oval = np.zeros(max(nnz, 1))
    lib().oracle_adat_numeric(m, n, P(rp), P(ci), P(v), P(col_ptr), P(row_ind), P(val), P(w), P(orp), P(ocol),
                              P(oval))
    row = np.repeat(np.arange(m, dtype=np.int64), np.diff(orp))
    o = np.lexsort((ocol[:nnz], row))
    return orp, ocol[:nnz][o], oval[:nnz][o]


def adat_timed(rp, ci, v, col_ptr, row_ind, val, w, m, n, threads):
    """ADAt_Allocate (symbolic, one thread) then ADAt_Calc (numeric, the
    reference's OpenMP row loop with `threads` threads), each timed; the
    values in the restatement's pattern order."""
    import time
    t0 = time.perf_counter()
    orp = np.zeros(m + 1, np.int32)
    nnz = lib().oracle_adat_symbolic(m, n, P(rp), P(ci), P(col_ptr), P(row_ind), P(orp), None)
    ocol = np.zeros(max(nnz, 1), np.int32)
    lib().oracle_adat_symbolic(m, n, P(rp), P(ci), P(col_ptr), P(row_ind), P(orp), P(ocol))
    t1 = time.perf_counter()
    oval = np.zeros(max(nnz, 1))
    used = lib().oracle_adat_numeric_threads(m, n, P(rp), P(ci), P(v), P(col_ptr), P(row_ind), P(val), P(w), P(orp),
                                             P(ocol), P(oval), threads)
    t2 = time.perf_counter()
    if used < 0:
        raise MemoryError("oracle_adat_numeric_threads")
    return {"nnz": int(nnz), "symbolic_s": t1 - t0, "numeric_s": t2 - t1, "threads": int(used)}


def topk(diag, k):
    m = len(diag)
    piv = np.zeros(max(k, 1), np.int32)
    kk = lib().oracle_topk_pivots(m, P(np.ascontiguousarray(diag)), k, P(piv))
    return piv[:kk]


class PartialCholesky:
    """RenewPartialCholesky restated (PCG.cpp:38-177); frees itself."""

    def __init__(self, rp, ci, v, d, m, n, k, rule=PIVOT_GREEDY, given=None, gamma=0.0, delta=0.0):
        self.pc = Pchol()
        self._keep = (rp, ci, v, d, given)
        g = np.ascontiguousarray(given, dtype=np.int32) if given is not None else None
        self._g = g
        rc = lib().oracle_pchol_build(m, n, P(rp), P(ci), P(v), P(d), gamma, delta, k, rule, P(g), C.byref(self.pc))
        if rc != 0:
            raise RuntimeError("oracle_pchol_build failed")
        self.m, self.k = m, self.pc.k

    @property
    def perm(self):
        return np.ctypeslib.as_array(self.pc.perm, (self.m,)).copy()

    @property
    def diag_s(self):
        return np.ctypeslib.as_array(self.pc.diag_s, (self.m,)).copy()

    @property
    def L(self):
        return np.ctypeslib.as_array(self.pc.L, (self.m * max(self.k, 1),)).reshape(self.m, max(self.k, 1))[:, :self.k].copy()

    @property
    def D(self):
        return np.ctypeslib.as_array(self.pc.D, (max(self.k, 1),))[:self.k].copy()

    def apply_permuted(self, r_perm):
        out = np.zeros(self.m)
        lib().oracle_precond_apply(C.byref(self.pc), P(np.ascontiguousarray(r_perm)), P(out))
        return out

    def apply(self, r):
        """M^-1 r with r and the result in the original row order."""
        perm = self.perm
        zp = self.apply_permuted(np.ascontiguousarray(r)[perm])
        z = np.empty(self.m)
        z[perm] = zp
        return z

    def __del__(self):
        try:
            lib().oracle_pchol_free(C.byref(self.pc))
        except Exception:
            pass


def pcg(rp, ci, v, d, b, m, n, k, rule=PIVOT_GREEDY, given=None, tol=1e-20, max_iter=10**12, gamma=0.0, delta=0.0):
    x = np.zeros(m)
    g = np.ascontiguousarray(given, dtype=np.int32) if given is not None else None
    it = lib().oracle_pcg(m, n, P(rp), P(ci), P(v), P(d), gamma, delta, P(np.ascontiguousarray(b)), P(x), k, rule,
                          P(g), tol, max_iter)
    return x, int(it)


class OracleNormalEquations:
    """The reference PCG backend restated (UsePCG_CPU.cpp:26-183)."""

    def __init__(self, pivots=10, rule=PIVOT_GREEDY, tol=1e-20, max_iter=10**12):
        self.L = lib()
        self.ctx = self.L.oracle_ne_create(pivots, rule, tol, max_iter)

    def LinearEquation_Construct(self, lp):
        self._keep = (np.ascontiguousarray(lp.col_ptr), np.ascontiguousarray(lp.row_ind), np.ascontiguousarray(lp.val))
        self.m, self.n = lp.m, lp.n
        return self.L.oracle_ne_construct(self.ctx, lp.m, lp.n, *[P(a) for a in self._keep])

    def RenewLinearEquation(self, d):
        return self.L.oracle_ne_renew(self.ctx, P(np.ascontiguousarray(d, dtype=np.float64)))

    def SolveLinearEquation(self, d, b_1, b_2):
        x1, x2 = np.zeros(self.n), np.zeros(self.m)
        rc = self.L.oracle_ne_solve(self.ctx, P(np.ascontiguousarray(d, dtype=np.float64)),
                                    P(np.ascontiguousarray(b_1, dtype=np.float64)),
                                    P(np.ascontiguousarray(b_2, dtype=np.float64)), P(x1), P(x2))
        if rc != 0:
            raise RuntimeError("oracle_ne_solve failed")
        return x1, x2

    def LinearEquation_Destruct(self):
        return self.L.oracle_ne_destruct(self.ctx)

    def last_iters(self):
        return int(self.L.oracle_ne_last_iters(self.ctx))

    def total_iters(self):
        return int(self.L.oracle_ne_total_iters(self.ctx))

    def ne_backend(self):
        from help_gb300 import native
        L = self.L
        be = native.NeBackend(ctx=self.ctx, construct=C.cast(L.oracle_ne_construct, C.c_void_p).value,
                              renew=C.cast(L.oracle_ne_renew, C.c_void_p).value,
                              solve=C.cast(L.oracle_ne_solve, C.c_void_p).value,
                              destruct=C.cast(L.oracle_ne_destruct, C.c_void_p).value)
        be._owner = self  # the table holds self.ctx: keep the context alive as long as the table
        return be

    def __del__(self):
        try:
            self.L.oracle_ne_free(self.ctx)
        except Exception:
            pass
