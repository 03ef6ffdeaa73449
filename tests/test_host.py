"""Host-side pieces: generator determinism and feasibility, MPS round trip,
C-ABI symbol exports (no GPU compute), HSD driver on small LPs vs scipy."""
import ctypes as C
import hashlib
import os
import re
import tempfile

import numpy as np
import pytest

from help_gb300 import hsd, lp as L, native
from oracle import bindings as ob

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _digest(lp):
    h = hashlib.sha256()
    for a in (lp.col_ptr, lp.row_ind, lp.val, lp.b, lp.c):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:16]


def test_generator_deterministic():
    a = L.generate(L.spec_random(300, 900, 5), 42)
    b = L.generate(L.spec_random(300, 900, 5), 42)
    c = L.generate(L.spec_random(300, 900, 5), 43)
    assert _digest(a) == _digest(b)
    assert _digest(a) != _digest(c)


@pytest.mark.parametrize("spec", [
    L.spec_random(500, 1500, 5),
    L.spec_zipf(2000, 8000, 6),
    L.spec_block(3, 200, 900, 5, 30, 0.05),
])
def test_generator_feasible_by_construction(spec):
    lp = L.generate(spec, 9)
    assert lp.col_ptr[0] == 0 and np.all(np.diff(lp.col_ptr) >= 0)
    for j in range(lp.n):
        r = lp.row_ind[lp.col_ptr[j]:lp.col_ptr[j + 1]]
        assert np.all(np.diff(r) > 0)
    rows_hit = np.bincount(lp.row_ind, minlength=lp.m)
    assert rows_hit.min() >= 1, "empty row"
    assert np.all(lp.val != 0)
    # values on the 1e-6 grid
    assert np.all(np.abs(lp.val * 1e6 - np.round(lp.val * 1e6)) < 1e-6)


def test_zipf_rows_are_skewed():
    lp = L.generate(L.spec_zipf(20000, 80000, 6), 1)
    cnt = np.bincount(lp.row_ind, minlength=lp.m)
    assert cnt.max() > 20 * cnt.mean()


def test_mcf_shape():
    lp = L.generate(L.spec_mcf(10, 2, 3), 1)
    arcs = 4 * 10 * 9
    assert lp.n == 2 * arcs + arcs and lp.n_struct == 2 * arcs
    assert lp.m == 2 * (100 - 1) + arcs
    assert lp.row_type.count(b"L") == arcs


def test_mps_round_trip():
    lp = L.generate(L.spec_random(30, 90, 4), 5)
    with tempfile.TemporaryDirectory() as t:
        p = os.path.join(t, "a.mps")
        lp.write_mps(p)
        txt = open(p).read().splitlines()
    # fixed card positions 4 / 14 / 24, each line short enough not to carry a second pair
    cols = [l for l in txt if l.startswith("    C")]
    assert all(len(l) <= 39 for l in cols)
    vals = {}
    for l in cols:
        name, row, v = l[4:12].strip(), l[14:22].strip(), float(l[24:])
        if row != "COST":
            vals[(int(row[1:]), int(name[1:]))] = v
    for j in range(lp.n):
        for p_ in range(lp.col_ptr[j], lp.col_ptr[j + 1]):
            assert vals[(lp.row_ind[p_], j)] == lp.val[p_]


def _declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"\b(help_[a-z0-9_]+)\s*\(", txt)))


def test_gpu_library_exports_every_declared_symbol():
    path = os.path.join(native.LIBDIR, "libhelp_gpu.so")
    lib = C.CDLL(path)  # loads without a GPU (no compute)
    names = _declared("help_gpu.h")
    assert len(names) >= 14
    for s in names:
        getattr(lib, s)


def test_default_options_match_the_reference_and_the_header_layout():
    """help_pcg_default_options runs without a GPU: the reference's PCG
    settings (10 pivots, FP64, 1e-20; PCG.h:19-20), an iteration cap that is
    an error by default (cap_ok = 0), and the ctypes mirror the same size as
    the C struct (the C compiler's sizeof, from the header)."""
    lib = native.gpu_lib()
    o = native.PcgOptions()
    C.memset(C.byref(o), 0x5A, C.sizeof(o))
    lib.help_pcg_default_options(C.byref(o))
    assert (o.pivots, o.precision, o.cg_tol, o.cap_ok, o.fallback) == (10, native.HELP_PREC_FP64, 1e-20, 0, 1)
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "s.c")
        with open(src, "w") as f:
            f.write('#include "help_gpu.h"\n#include <stdio.h>\n'
                    'int main(void){printf("%zu\\n", sizeof(help_pcg_options)); return 0;}\n')
        exe = os.path.join(tmp, "s")
        import subprocess
        subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        size = int(subprocess.run([exe], capture_output=True, text=True, check=True).stdout)
    assert size == C.sizeof(native.PcgOptions)


def test_lp_library_exports_every_declared_symbol():
    lib = C.CDLL(os.path.join(native.LIBDIR, "libhelp_lp.so"))
    for s in _declared("help_lp.h"):
        getattr(lib, s)


@pytest.mark.skipif(not ob.ref_available(), reason="the reference's sources were not built here")
def test_reference_program_links_against_gpu_backend():
    """The reference program (every source but UsePCG_CPU.cpp + PCG.cpp) links
    with help_gb300/csrc/UsePCG_GPU.cpp over libhelp_gpu.so: all four LP.h
    entry points resolve to the shim and nothing is left undefined."""
    import subprocess
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), "../_ref/help_ref_gpu"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    exe = os.path.join(ROOT, "oracle", "_ref", "help_ref_gpu")
    syms = subprocess.run(["nm", "-C", exe], capture_output=True, text=True).stdout
    for f in ("LinearEquation_Construct()", "LinearEquation_Destruct()", "RenewLinearEquation(double*)",
              "SolveLinearEquation(double*, double*, double*, double*, double*)"):
        assert re.search(r" T " + re.escape(f), syms), f
    assert "ConjugateGradient" not in syms  # the reference's CPU PCG is not linked in
    dyn = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True, text=True).stdout
    assert "help_pcg_solve" in dyn


def test_hsd_driver_objective_matches_scipy():
    scipy_opt = pytest.importorskip("scipy.optimize")
    import scipy.sparse as sp
    lp = L.generate(L.spec_random(80, 240, 5), 3)
    ora = ob.OracleNormalEquations(pivots=10, tol=1e-14, max_iter=10**6)
    res = hsd.solve_lp(lp, ora.ne_backend())
    A = sp.csc_matrix((lp.val, lp.row_ind, lp.col_ptr), shape=(lp.m, lp.n))
    r = scipy_opt.linprog(lp.c, A_eq=A, b_eq=lp.b, bounds=(0, None), method="highs")
    assert res["status"] == 0
    assert abs(res["primal_obj"] - r.fun) / (1 + abs(r.fun)) < 1e-8


def test_hsd_driver_uses_backend_matvec():
    """The optional matvec of the backend table replaces the driver's host
    products: a numpy matvec (dest += sign A v / A^T v) is called for every
    product and the run matches the host loops to rounding."""
    import ctypes as C
    import scipy.sparse as sp
    from help_gb300 import native
    lp = L.generate(L.spec_random(80, 240, 5), 3)
    A = sp.csc_matrix((lp.val, lp.row_ind, lp.col_ptr), shape=(lp.m, lp.n))
    calls = []

    def matvec(_c, transpose, sign, v, dest):
        nin, nout = (lp.m, lp.n) if transpose else (lp.n, lp.m)
        vv = np.ctypeslib.as_array(C.cast(v, C.POINTER(C.c_double)), (nin,))
        dd = np.ctypeslib.as_array(C.cast(dest, C.POINTER(C.c_double)), (nout,))
        dd += sign * ((A.T if transpose else A) @ vv)
        calls.append(transpose)
        return 0

    fn = native.MATVEC_FN(matvec)
    ora = ob.OracleNormalEquations(pivots=10, tol=1e-14, max_iter=10**6)
    be = ora.ne_backend()
    be.matvec = C.cast(fn, C.c_void_p).value
    res = hsd.solve_lp(lp, be)
    ora2 = ob.OracleNormalEquations(pivots=10, tol=1e-14, max_iter=10**6)
    ref = hsd.solve_lp(lp, ora2.ne_backend())
    assert res["status"] == ref["status"] == 0
    assert calls.count(0) > 0 and calls.count(1) > 0
    assert abs(res["primal_obj"] - ref["primal_obj"]) <= 1e-9 * (1 + abs(ref["primal_obj"]))


def test_hsd_driver_wall_clock_cap():
    """max_seconds stops the driver before the next renew once it has run out
    (status 2, as at the iteration limit); 0 means no cap."""
    lp = L.generate(L.spec_random(300, 900, 5), 4)
    ora = ob.OracleNormalEquations(pivots=10, tol=1e-10)
    full = hsd.solve_lp(lp, ora.ne_backend())
    assert full["status"] == 0
    ora2 = ob.OracleNormalEquations(pivots=10, tol=1e-10)
    capped = hsd.solve_lp(lp, ora2.ne_backend(), max_seconds=1e-9)
    assert capped["status"] == 2 and capped["iterations"] == 1 and capped["renews"] <= 1


def test_hsd_driver_paired_solves_give_the_same_run():
    """With a backend that offers solve2, the driver computes the bottom
    system's and the first direction's right-hand sides and solves them in
    one call; every value it computes is the same as in the reference's
    order.  Here solve2 is the CPU oracle's solve done twice, so the run must
    equal the sequential one bit for bit."""
    import ctypes as C
    from help_gb300 import native
    lp = L.generate(L.spec_random(80, 240, 5), 3)
    seq = ob.OracleNormalEquations(pivots=10, tol=1e-14, max_iter=10**6)
    r1 = hsd.solve_lp(lp, seq.ne_backend(), want_solution=True)
    ora = ob.OracleNormalEquations(pivots=10, tol=1e-14, max_iter=10**6)
    base = ora.ne_backend()
    solve = native.SOLVE_FN(base.solve)
    pairs = []

    def solve2(ctx, d, b1a, b2a, x1a, x2a, b1b, b2b, x1b, x2b):
        pairs.append(1)
        rc = solve(ctx, d, b1a, b2a, x1a, x2a)
        return rc if rc else solve(ctx, d, b1b, b2b, x1b, x2b)

    fn = native.SOLVE2_FN(solve2)
    be = native.NeBackend(ctx=base.ctx, construct=base.construct, renew=base.renew, solve=base.solve,
                          destruct=base.destruct, solve2=C.cast(fn, C.c_void_p).value)
    r2 = hsd.solve_lp(lp, be, want_solution=True)
    assert r1["status"] == r2["status"] == 0 and r1["iterations"] == r2["iterations"]
    assert r1["solves"] == r2["solves"] and len(pairs) == r1["iterations"]
    assert r1["primal_obj"] == r2["primal_obj"] and r1["rel_gap"] == r2["rel_gap"]
    assert np.array_equal(r1["x"], r2["x"]) and np.array_equal(r1["y"], r2["y"])


def test_pair_and_slot_entry_points_reject_bad_arguments():
    """The paired backend and the solve-slot entry points check their
    arguments before any device work (no GPU needed): a pair refuses the
    warm_start option, null contexts and out-of-range slots are errors."""
    import ctypes as C
    from help_gb300 import backend, native
    lib = native.gpu_lib()
    opt = backend.pcg_options(lib, pivots=4, warm_start=True)
    out = C.c_void_p()
    assert lib.help_pcg_pair_create(C.byref(opt), C.byref(out)) == native.HELP_E_ARG and not out.value
    slots = (C.c_int32 * 2)(0, 7)
    assert lib.help_pcg_set_solve_slots(None, slots, 2) == native.HELP_E_ARG
    assert lib.help_pcg_share_solution(None, 0, None, 0) == native.HELP_E_ARG
    assert lib.help_pcg_pair_context(None, 0) is None
    for fn in (lib.help_pcg_pair_renew, lib.help_pcg_pair_destruct):
        fn.restype = C.c_int
    assert lib.help_pcg_pair_renew(None, None) == native.HELP_E_ARG
    assert lib.help_pcg_pair_destruct(None) == native.HELP_E_ARG


def test_hsd_driver_stops_on_a_failed_paired_solve():
    """A backend whose solve2 fails ends the driver's run with the backend
    error code (the same handling as a failed solve), after one call."""
    import ctypes as C
    from help_gb300 import native
    lp = L.generate(L.spec_random(60, 180, 5), 4)
    ora = ob.OracleNormalEquations(pivots=10, tol=1e-14, max_iter=10**6)
    base = ora.ne_backend()
    calls = []

    def solve2(*_args):
        calls.append(1)
        return -1

    fn = native.SOLVE2_FN(solve2)
    be = native.NeBackend(ctx=base.ctx, construct=base.construct, renew=base.renew, solve=base.solve,
                          destruct=base.destruct, solve2=C.cast(fn, C.c_void_p).value)
    r = hsd.solve_lp(lp, be)
    assert r["rc"] == -2 and len(calls) == 1
