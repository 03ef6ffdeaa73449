"""The HSD driver's own products on the device (help_pcg_matvec_acc, the
optional matvec of the backend table) against numpy and against the driver's
host loops.

Tolerances: dest += sign * A v to 1e-13 relative (row sums in a different
order); IPM runs with device and host products reach the same status and
iteration count and objectives within 1e-9 relative (the products differ in
rounding only).
"""
import ctypes as C

import numpy as np
import pytest

from help_gb300 import backend, hsd, native, lp as L

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("transpose", [0, 1])
@pytest.mark.parametrize("sign", [1, -1])
def test_matvec_acc(transpose, sign):
    lp = L.generate(L.spec_zipf(800, 3000, 6, 1.3, 40), 2)  # ragged rows
    A = np.zeros((lp.m, lp.n))
    for j in range(lp.n):
        A[lp.row_ind[lp.col_ptr[j]:lp.col_ptr[j + 1]], j] = lp.val[lp.col_ptr[j]:lp.col_ptr[j + 1]]
    rng = np.random.default_rng(transpose * 2 + (sign > 0))
    v = rng.standard_normal(lp.m if transpose else lp.n)
    dest = rng.standard_normal(lp.n if transpose else lp.m)
    want = dest + sign * ((A.T if transpose else A) @ v)
    with backend.GpuNormalEquations(pivots=4) as g:
        g.LinearEquation_Construct(lp)
        out = dest.copy()
        rc = g.lib.help_pcg_matvec_acc(g.ctx, transpose, sign, native.ptr(v), native.ptr(out))
        assert rc == native.HELP_OK
        assert rel(out, want) < 1e-13
        assert g.lib.help_pcg_matvec_acc(g.ctx, transpose, 2, native.ptr(v), native.ptr(out)) != native.HELP_OK


@pytest.mark.parametrize("name,spec,seed", [("random", L.spec_random(300, 900, 5), 1),
                                            ("mcf", L.spec_mcf(8, 3, 2), 4)])
def test_ipm_device_products_match_host_loops(name, spec, seed):
    lp = L.generate(spec, seed)
    runs = {}
    for dev in (True, False):
        with backend.GpuNormalEquations(pivots=10, cg_tol=1e-12, cg_max_iter=200000) as g:
            runs[dev] = hsd.solve_lp(lp, g.ne_backend(gpu_matvec=dev))
    a, b = runs[True], runs[False]
    assert a["status"] == b["status"] == 0
    assert a["iterations"] == b["iterations"]
    assert abs(a["primal_obj"] - b["primal_obj"]) <= 1e-9 * (1 + abs(b["primal_obj"]))
    assert a["rel_gap"] < 1e-8 and a["primal_infeas"] < 1e-7


def test_host_arrays_at_8_byte_offsets():
    """Host arrays that are not 16-byte aligned (the direct-copy path then
    moves 8-byte words)."""
    lp = L.generate(L.spec_random(300, 900, 5), 9)
    rng = np.random.default_rng(9)
    A = np.zeros((lp.m, lp.n))
    for j in range(lp.n):
        A[lp.row_ind[lp.col_ptr[j]:lp.col_ptr[j + 1]], j] = lp.val[lp.col_ptr[j]:lp.col_ptr[j + 1]]
    xb = rng.standard_normal(lp.n + 1)
    yb = np.zeros(lp.m + 1)
    x, y = xb[1:], yb[1:]
    assert x.ctypes.data % 16 == 8 or xb.ctypes.data % 16 == 8
    with backend.GpuNormalEquations(pivots=4) as g:
        g.LinearEquation_Construct(lp)
        rc = g.lib.help_pcg_matvec(g.ctx, native.HELP_OP_A, native.ptr(x), native.ptr(y))
        assert rc == native.HELP_OK
    assert rel(y, A @ x) < 1e-13 and yb[0] == 0.0


def test_ungrounded_flow_presolved_then_solved():
    """Multicommodity flow with every node row kept is one row per commodity
    short of full rank; after the dependent-row presolve the GPU backend and
    the HSD driver reach the grounded instance's optimum, and x is feasible
    for the full rows too (objectives within 1e-7 relative: two IPM runs to
    a 1e-8 gap on different but equivalent row sets)."""
    full = L.generate(L.spec_mcf(8, 3, 2, grounded=False), 4)
    grounded = L.generate(L.spec_mcf(8, 3, 2), 4)
    red, removed = L.remove_dependent_rows(full)
    assert removed.sum() == 3
    runs = []
    for lp in (red, grounded):
        with backend.GpuNormalEquations(pivots=10, cg_tol=1e-12, cg_max_iter=200000) as g:
            runs.append(hsd.solve_lp(lp, g.ne_backend(), want_solution=True))
    assert all(r["status"] == 0 and r["rel_gap"] < 1e-8 for r in runs)
    assert abs(runs[0]["primal_obj"] - runs[1]["primal_obj"]) <= 1e-7 * (1 + abs(runs[1]["primal_obj"]))
    A = np.zeros((full.m, full.n))
    for j in range(full.n):
        A[full.row_ind[full.col_ptr[j]:full.col_ptr[j + 1]], j] = full.val[full.col_ptr[j]:full.col_ptr[j + 1]]
    assert np.linalg.norm(A @ runs[0]["x"] - full.b) <= 1e-7 * (1 + np.linalg.norm(full.b))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name, spec, seed", [("random", L.spec_random(400, 1200, 5), 21),
                                              ("mcf", L.spec_mcf(10, 3, 3), 22)])
def test_paired_solves_give_the_same_run(precision, name, spec, seed):
    """The bottom system and the first direction of every iteration solved
    at once on two contexts (backend solve2, help_pcg_pair) give bitwise the
    run of one context solving them one after the other: each solve is a cold
    start, and the driver computes the same values in the same order."""
    lp = L.generate(spec, seed)
    kw = dict(pivots=10, precision=precision, cg_tol=1e-10, ir_tol=1e-10, cg_max_iter=200_000)
    with backend.GpuNormalEquations(**kw) as g:
        one = hsd.solve_lp(lp, g.ne_backend(), want_solution=True)
    with backend.GpuPairNormalEquations(**kw) as p:
        two = hsd.solve_lp(lp, p.ne_backend(), want_solution=True)
        s0, s1 = p.stats(0), p.stats(1)
    assert one["status"] == two["status"] == 0 and one["iterations"] == two["iterations"], (name, one, two)
    assert one["solves"] == two["solves"]
    assert one["primal_obj"] == two["primal_obj"] and one["rel_gap"] == two["rel_gap"]
    assert np.array_equal(one["x"], two["x"]) and np.array_equal(one["y"], two["y"])
    # context 1 took the second system of every pair: one per direction computed
    assert s1["solves"] > 0 and s0["solves"] + s1["solves"] == one["solves"]


def test_pair_rejects_warm_start():
    with pytest.raises(ValueError):
        backend.GpuPairNormalEquations(pivots=4, warm_start=True)
