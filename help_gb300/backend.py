"""Python mirror of the reference's normal-equations backend interface.

The reference (Tian-Xie/HELP) links one backend exposing four functions
(LP.h:157-160); the PCG backend implements them in UsePCG_CPU.cpp:26-183.
:class:`GpuNormalEquations` exposes the same four operations, with the same
names and argument meaning, over the C ABI of ``libhelp_gpu.so``:

=================================  ==========================================
reference (UsePCG_CPU.cpp)         here
=================================  ==========================================
``LinearEquation_Construct()``     ``LinearEquation_Construct(lp)`` (A given
                                   explicitly instead of through globals)
``RenewLinearEquation(d)``         ``RenewLinearEquation(d)``
``SolveLinearEquation(d, b_1,      ``x_1, x_2 = SolveLinearEquation(d, b_1,
b_2, x_1, x_2)``                   b_2)``
``LinearEquation_Destruct()``      ``LinearEquation_Destruct()``
=================================  ==========================================

Errors: every native call returns a status; a non-zero status raises
:class:`BackendError` with the library's message (the reference exits the
process through CheckError, Helper.cpp:24-35).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native


class BackendError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("help_gpu error %d: %s" % (code, msg))
        self.code = code


def _f64(a, n=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    if n is not None and a.shape != (n,):
        raise ValueError("expected a vector of length %d, got shape %s" % (n, a.shape))
    return a


def pcg_options(lib, pivots: int = 10, precision: str = "fp64", cg_tol: float = 1e-20,
                cg_max_iter: int = 1_000_000, delta: float = 0.0, ir_tol: float = 1e-10,
                ir_max_outer: int = 10, inner_tol: float = 1e-5, inner_max_iter: int = 200_000,
                warm_start: bool = False, fallback: bool = True, device: int = 0, cg_path: str = "auto",
                cap_ok: bool = False, mixed_max_d_spread: float = 1e8) -> native.PcgOptions:
    """help_pcg_options from the library defaults and these arguments."""
    o = native.PcgOptions()
    lib.help_pcg_default_options(C.byref(o))
    o.device = device
    o.pivots = int(pivots)
    o.precision = {"fp64": native.HELP_PREC_FP64, "mixed": native.HELP_PREC_MIXED}[precision]
    o.cg_tol = cg_tol
    o.cg_max_iter = int(cg_max_iter)
    o.delta = delta
    o.ir_tol = ir_tol
    o.ir_max_outer = ir_max_outer
    o.inner_tol = inner_tol
    o.inner_max_iter = int(inner_max_iter)
    o.warm_start = int(bool(warm_start))
    o.fallback = int(bool(fallback))
    o.cg_path = {"auto": 0, "graph": 1, "cluster": 2, "resident": 3}[cg_path]
    o.cap_ok = int(bool(cap_ok))
    o.mixed_max_d_spread = float(mixed_max_d_spread)
    return o


class GpuPairNormalEquations:
    """Two contexts on one GB300 for the HSD driver's paired solves
    (help_pcg_pair: the bottom system and the first search direction of
    every IPM iteration solved at the same time, each on its own context,
    host thread and stream).  Same options as GpuNormalEquations except the
    warm start, which the pairing would reorder.  Use through ne_backend()."""

    def __init__(self, **kw):
        if kw.get("warm_start"):
            raise ValueError("the pair runs every solve from a cold start")
        self.lib = native.gpu_lib()
        self.options = pcg_options(self.lib, **kw)
        h = C.c_void_p()
        rc = self.lib.help_pcg_pair_create(C.byref(self.options), C.byref(h))
        if rc != 0:
            raise BackendError(rc, "help_pcg_pair_create")
        self.pair = h

    def context(self, which: int):
        return self.lib.help_pcg_pair_context(self.pair, which)

    def stats(self, which: int = 0) -> dict:
        s = native.PcgStats()
        rc = self.lib.help_pcg_get_stats(self.context(which), C.byref(s))
        if rc != 0:
            raise BackendError(rc, "help_pcg_get_stats")
        return {f: getattr(s, f) for f, _ in native.PcgStats._fields_}

    def ne_backend(self) -> native.NeBackend:
        """Backend table for help_hsd_solve with solve2 set."""
        lib = self.lib
        f = lambda fn: C.cast(fn, C.c_void_p).value
        be = native.NeBackend(ctx=self.pair.value, construct=f(lib.help_pcg_pair_construct),
                              renew=f(lib.help_pcg_pair_renew), solve=f(lib.help_pcg_pair_solve),
                              destruct=f(lib.help_pcg_pair_destruct), matvec=f(lib.help_pcg_pair_matvec),
                              solve2=f(lib.help_pcg_pair_solve2))
        be._owner = self
        return be

    def close(self) -> None:
        if getattr(self, "pair", None):
            self.lib.help_pcg_pair_free(self.pair)
            self.pair = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class GpuNormalEquations:
    """Normal-equations backend on one GB300 (plain FP64 PCG or mixed precision)."""

    def __init__(self, **kw):
        self.lib = native.gpu_lib()
        o = pcg_options(self.lib, **kw)
        self.options = o
        h = C.c_void_p()
        self._check(self.lib.help_pcg_create(C.byref(o), C.byref(h)), None)
        self.ctx = h
        self.m = self.n = 0

    # -- plumbing
    def _check(self, rc: int, ctx=None) -> None:
        if rc != 0:
            msg = self.lib.help_pcg_last_error(ctx if ctx is not None else self.ctx)
            raise BackendError(rc, msg.decode() if msg else "")

    def close(self) -> None:
        if getattr(self, "ctx", None):
            self.lib.help_pcg_free(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- the four boundary operations
    def LinearEquation_Construct(self, lp=None, *, m=None, n=None, col_ptr=None, row_ind=None, val=None) -> int:
        if lp is not None:
            m, n, col_ptr, row_ind, val = lp.m, lp.n, lp.col_ptr, lp.row_ind, lp.val
        self._cp = np.ascontiguousarray(col_ptr, dtype=np.int32)
        self._ri = np.ascontiguousarray(row_ind, dtype=np.int32)
        self._v = np.ascontiguousarray(val, dtype=np.float64)
        self._check(self.lib.help_pcg_construct(self.ctx, int(m), int(n), native.ptr(self._cp),
                                                native.ptr(self._ri), native.ptr(self._v)))
        self.m, self.n = int(m), int(n)
        return 0

    def RenewLinearEquation(self, d) -> None:
        self._d = _f64(d, self.n)
        self._check(self.lib.help_pcg_renew(self.ctx, native.ptr(self._d)))

    def SolveLinearEquation(self, d, b_1, b_2):
        d = _f64(d, self.n)
        if getattr(self, "_d", None) is not None and d is not self._d and np.array_equal(d, self._d):
            d = self._d  # same values as renewed: keep the renewed preconditioner
        else:
            self._d = d
        b1 = _f64(b_1, self.n)
        b2 = _f64(b_2, self.m)
        x1 = np.empty(self.n)
        x2 = np.empty(self.m)
        self._check(self.lib.help_pcg_solve(self.ctx, native.ptr(d), native.ptr(b1), native.ptr(b2),
                                            native.ptr(x1), native.ptr(x2)))
        return x1, x2

    def LinearEquation_Destruct(self) -> int:
        self._check(self.lib.help_pcg_destruct(self.ctx))
        return 0

    # -- building blocks
    def stats(self) -> dict:
        s = native.PcgStats()
        self._check(self.lib.help_pcg_get_stats(self.ctx, C.byref(s)))
        return {f: getattr(s, f) for f, _ in native.PcgStats._fields_}

    def matvec(self, op: str, x) -> np.ndarray:
        opc = {"A": native.HELP_OP_A, "AT": native.HELP_OP_AT, "ADAT": native.HELP_OP_ADAT,
               "B": native.HELP_OP_B, "BT": native.HELP_OP_BT}[op]
        nin = self.n if op in ("A", "B") else self.m
        nout = self.n if op in ("AT", "BT") else self.m
        x = _f64(x, nin)
        y = np.empty(nout)
        self._check(self.lib.help_pcg_matvec(self.ctx, opc, native.ptr(x), native.ptr(y)))
        return y

    def matvec_dev(self, op: str, x_ptr: int, y_ptr: int, fp32: bool = False, stream: int = 0) -> None:
        opc = {"A": native.HELP_OP_A, "AT": native.HELP_OP_AT, "ADAT": native.HELP_OP_ADAT,
               "B": native.HELP_OP_B, "BT": native.HELP_OP_BT}[op]
        self._check(self.lib.help_pcg_matvec_dev(self.ctx, opc, int(fp32), C.c_void_p(x_ptr),
                                                 C.c_void_p(y_ptr), C.c_void_p(stream or None)))

    def precond_apply(self, r) -> np.ndarray:
        r = _f64(r, self.m)
        z = np.empty(self.m)
        self._check(self.lib.help_pcg_precond_apply(self.ctx, native.ptr(r), native.ptr(z)))
        return z

    def pivots(self):
        k = self.stats()["pivots"]
        piv = np.empty(max(k, 1), np.int32)
        dg = np.empty(self.m)
        ds = np.empty(self.m)
        self._check(self.lib.help_pcg_get_pivots(self.ctx, native.ptr(piv), native.ptr(dg), native.ptr(ds)))
        return piv[:k], dg, ds

    def cg(self, b, fp32: bool = False):
        b = _f64(b, self.m)
        x = np.empty(self.m)
        it = C.c_int64()
        fn = self.lib.help_pcg_cg_f32 if fp32 else self.lib.help_pcg_cg
        self._check(fn(self.ctx, native.ptr(b), native.ptr(x), C.byref(it)))
        return x, int(it.value)

    def adat(self, w):
        """Upper triangle of A diag(w) A^T as CSR (row_ptr, col, val)."""
        w = _f64(w, self.n)
        rp = np.empty(self.m + 1, np.int32)
        nnz = C.c_int64()
        self._check(self.lib.help_adat_assemble(self.ctx, native.ptr(w), native.ptr(rp), None, None,
                                                C.byref(nnz)))
        col = np.empty(max(nnz.value, 1), np.int32)
        val = np.empty(max(nnz.value, 1))
        self._check(self.lib.help_adat_assemble(self.ctx, native.ptr(w), native.ptr(rp), native.ptr(col),
                                                native.ptr(val), C.byref(nnz)))
        return rp, col[:nnz.value], val[:nnz.value]

    def ne_backend(self, gpu_matvec: bool = True) -> native.NeBackend:
        """Function-pointer table for the native HSD driver (help_hsd_solve).
        gpu_matvec: the driver's own A x / A^T y products run on this
        context's device copy of A (help_pcg_matvec_acc); False keeps the
        driver's host loops (the reference's summation order)."""
        lib = self.lib
        be = native.NeBackend(
            ctx=self.ctx.value,
            construct=C.cast(lib.help_pcg_construct, C.c_void_p).value,
            renew=C.cast(lib.help_pcg_renew, C.c_void_p).value,
            solve=C.cast(lib.help_pcg_solve, C.c_void_p).value,
            destruct=C.cast(lib.help_pcg_destruct, C.c_void_p).value,
            matvec=C.cast(lib.help_pcg_matvec_acc, C.c_void_p).value if gpu_matvec else None,
        )
        be._owner = self  # the table holds self.ctx: keep the context alive as long as the table
        return be
