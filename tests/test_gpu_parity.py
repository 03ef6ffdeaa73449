"""GPU parity: every building block of the path through the C ABI against the
CPU oracle (a restatement of the reference pinned to the reference itself in
test_oracle_pin.py).

Tolerances: FP64 kernels agree with the oracle to 1e-12 relative (summation
order differs); iterative solves are compared after both reach the same
stopping rule, to 1e-8 relative; index work (pivots, ADA^T pattern) is exact.
"""
import numpy as np
import pytest

from help_gb300 import backend, lp as L
from oracle import bindings as ob

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


CASES = {
    "random": lambda: L.generate(L.spec_random(400, 1200, 5), 3),
    "zipf": lambda: L.generate(L.spec_zipf(3000, 12000, 6, 1.3, 70), 4),
    "block": lambda: L.generate(L.spec_block(4, 300, 1200, 5, 40, 0.05), 5),
    "mcf": lambda: L.generate(L.spec_mcf(12, 3, 3), 6),
    # 4 linking rows of ~19k nonzeros: long rows split over 2 CTAs each, and
    # pivot columns of C with ~8k entries (long rows of C^T, one CTA each)
    "longrows": lambda: L.generate(L.spec_block(8, 1000, 4000, 5, 4, 0.6), 8),
}


# cases whose vectors fit one cluster's shared memory with rows of <= 32 G
# nonzeros (the resident CG path); the others fall back to the auto choice
RESIDENT_CASES = {"random", "mcf"}
PATH_USED = {
    "graph": lambda name: {1},
    "cluster": lambda name: {2},
    "resident": lambda name: {3} if name in RESIDENT_CASES else {1, 2},
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    lp = CASES[request.param]()
    rng = np.random.default_rng(11)
    d = np.exp(rng.uniform(-6, 6, lp.n))
    return request.param, lp, d, rng


def test_mkl_known_answer():
    # [1 0 2; 0 3 0; 4 0 5] * [3 5 7]^T = [17 15 47]^T (Main.cpp:19-35)
    col_ptr = np.array([0, 2, 3, 5], np.int32)
    row_ind = np.array([0, 2, 1, 0, 2], np.int32)
    val = np.array([1.0, 4.0, 3.0, 2.0, 5.0])
    with backend.GpuNormalEquations(pivots=1) as g:
        g.LinearEquation_Construct(m=3, n=3, col_ptr=col_ptr, row_ind=row_ind, val=val)
        y = g.matvec("A", np.array([3.0, 5.0, 7.0]))
    assert np.array_equal(y, [17.0, 15.0, 47.0])


def test_spmv_and_adat(case):
    name, lp, d, rng = case
    rp, ci, v = lp.csr()
    with backend.GpuNormalEquations(pivots=8) as g:
        g.LinearEquation_Construct(lp)
        x = rng.standard_normal(lp.n)
        w = rng.standard_normal(lp.m)
        assert rel(g.matvec("A", x), ob.csrmv_n(rp, ci, v, x, lp.m, lp.n)) < 1e-13
        assert rel(g.matvec("AT", w), ob.csrmv_t(rp, ci, v, w, lp.m, lp.n)) < 1e-13
        g.RenewLinearEquation(d)
        y = g.matvec("ADAT", w)
        t = ob.csrmv_t(rp, ci, v, w, lp.m, lp.n) / d
        assert rel(y, ob.csrmv_n(rp, ci, v, t, lp.m, lp.n)) < 1e-11


@pytest.mark.parametrize("k", [0, 1, 10, 64])
def test_pivots_diag_schur_precond(case, k):
    name, lp, d, rng = case
    rp, ci, v = lp.csr()
    with backend.GpuNormalEquations(pivots=k) as g:
        g.LinearEquation_Construct(lp)
        g.RenewLinearEquation(d)
        piv, dg, ds = g.pivots()
        dg_ref = ob.diag_adat(rp, ci, v, d, lp.m)
        assert rel(dg, dg_ref) < 1e-13
        assert np.array_equal(piv, ob.topk(dg, k))          # same rule on the same diagonal: exact
        pc = ob.PartialCholesky(rp, ci, v, d, lp.m, lp.n, k, ob.PIVOT_GIVEN, piv)
        non = np.ones(lp.m, bool)
        non[piv] = False
        ds_ref = pc.diag_s
        good = non & (ds_ref > 1e-6 * dg_ref)              # rows whose Schur diagonal is not pure cancellation
        assert np.max(np.abs(ds[good] - ds_ref[good]) / dg_ref[good]) < 1e-9
        r = rng.standard_normal(lp.m)
        z = g.precond_apply(r)
        assert rel(z, pc.apply(r)) < 1e-8


@pytest.mark.parametrize("path", ["graph", "cluster", "resident"])
def test_cg_matches_oracle(case, path):
    name, lp, d, rng = case
    rp, ci, v = lp.csr()
    k = 16
    b = rng.standard_normal(lp.m)
    with backend.GpuNormalEquations(pivots=k, cg_tol=1e-10, cg_max_iter=20000, cg_path=path) as g:
        g.LinearEquation_Construct(lp)
        g.RenewLinearEquation(d)
        piv, _, _ = g.pivots()
        x, it = g.cg(b)
        st = g.stats()
    assert st["cluster_ctas"] in (8, 16)
    assert st["cg_path_used"] in PATH_USED[path](name)
    xo, ito = ob.pcg(rp, ci, v, d, b, lp.m, lp.n, k, ob.PIVOT_GIVEN, piv, tol=1e-10, max_iter=20000)
    assert rel(x, xo) < 1e-6
    assert abs(it - ito) <= max(3, 0.05 * ito)


@pytest.mark.parametrize("path", ["graph", "cluster", "resident"])
def test_solve_linear_equation(case, path):
    name, lp, d, rng = case
    b1 = rng.standard_normal(lp.n)
    b2 = rng.standard_normal(lp.m)
    with backend.GpuNormalEquations(pivots=10, cg_tol=1e-12, cg_max_iter=50000, cg_path=path) as g:
        g.LinearEquation_Construct(lp)
        g.RenewLinearEquation(d)
        x1, x2 = g.SolveLinearEquation(d, b1, b2)
        st = g.stats()
    ora = ob.OracleNormalEquations(pivots=10, rule=ob.PIVOT_GIVEN, tol=1e-12, max_iter=50000)
    ora.LinearEquation_Construct(lp)
    ox1, ox2 = ora.SolveLinearEquation(d, b1, b2)
    assert st["converged"] == 1
    assert rel(x2, ox2) < 1e-6
    assert rel(x1, ox1) < 1e-6


@pytest.mark.parametrize("path", ["graph", "cluster", "resident"])
def test_mixed_precision_solve(case, path):
    name, lp, d, rng = case
    b1 = rng.standard_normal(lp.n)
    b2 = rng.standard_normal(lp.m)
    with backend.GpuNormalEquations(pivots=16, precision="mixed", ir_tol=1e-10, inner_tol=1e-4,
                                    cg_tol=1e-14, cg_path=path) as g:
        g.LinearEquation_Construct(lp)
        g.RenewLinearEquation(d)
        x1, x2 = g.SolveLinearEquation(d, b1, b2)
        st = g.stats()
    ora = ob.OracleNormalEquations(pivots=16, rule=ob.PIVOT_GIVEN, tol=1e-14, max_iter=100000)
    ora.LinearEquation_Construct(lp)
    ox1, ox2 = ora.SolveLinearEquation(d, b1, b2)
    assert st["rel_residual"] < 1e-9
    assert rel(x2, ox2) < 1e-5


def test_adat_assembly_bitwise(case):
    name, lp, d, rng = case
    rp, ci, v = lp.csr()
    w = np.exp(rng.uniform(-2, 2, lp.n))
    with backend.GpuNormalEquations(pivots=1) as g:
        g.LinearEquation_Construct(lp)
        grp, gcol, gval = g.adat(w)
        grp2, gcol2, gval2 = g.adat(w)  # the heavy rows' accumulator slots are reused
    orp, ocol, oval = ob.adat(rp, ci, v, lp.col_ptr, lp.row_ind, lp.val, w, lp.m, lp.n)
    assert np.array_equal(grp, orp)
    assert np.array_equal(gcol, ocol)
    assert np.array_equal(gval, oval)   # same products, same order: bit-exact
    assert np.array_equal(gcol2, gcol) and np.array_equal(gval2, gval)
    if name in ("zipf", "longrows"):
        # rows with more than the per-warp sort's 2,048 contributions (entries
        # k >= i of the columns the row touches) went through the heavy-row kernel
        col = np.repeat(np.arange(lp.n), np.diff(lp.col_ptr))
        contrib = np.bincount(lp.row_ind, weights=lp.col_ptr[col + 1] - np.arange(lp.nnz), minlength=lp.m)
        assert contrib.max() > 2048


def test_bad_d_is_an_error():
    lp = CASES["random"]()
    with backend.GpuNormalEquations(pivots=4) as g:
        g.LinearEquation_Construct(lp)
        d = np.ones(lp.n)
        d[7] = 0.0
        with pytest.raises(backend.BackendError) as e:
            g.RenewLinearEquation(d)
        assert e.value.code == -4
        d[7] = np.nan
        with pytest.raises(backend.BackendError):
            g.RenewLinearEquation(d)
        g.RenewLinearEquation(np.ones(lp.n))          # context still usable afterwards
        assert g.stats()["pivots"] == 4


def test_long_rows_repeatable_and_fp32():
    """Rows split over several CTAs give bitwise the same product on every
    call (partials added in segment order, tickets reset by the last CTA),
    in FP64 and in the FP32 copy, and FP32 agrees with FP64 to 1e-5."""
    torch = pytest.importorskip("torch")
    lp = CASES["longrows"]()
    rng = np.random.default_rng(12)
    d = np.exp(rng.uniform(-6, 6, lp.n))
    rp, ci, v = lp.csr()
    with backend.GpuNormalEquations(pivots=4, precision="mixed") as g:
        g.LinearEquation_Construct(lp)
        g.RenewLinearEquation(d)
        w = rng.standard_normal(lp.m)
        y1, y2 = g.matvec("ADAT", w), g.matvec("ADAT", w)
        assert np.array_equal(y1, y2)
        t = ob.csrmv_t(rp, ci, v, w, lp.m, lp.n) / d
        assert rel(y1, ob.csrmv_n(rp, ci, v, t, lp.m, lp.n)) < 1e-11
        x32 = torch.from_numpy(w.astype(np.float32)).cuda()
        outs = []
        for _ in range(2):
            y32 = torch.empty(lp.m, dtype=torch.float32, device="cuda")
            g.matvec_dev("ADAT", x32.data_ptr(), y32.data_ptr(), fp32=True)
            torch.cuda.synchronize()
            outs.append(y32.cpu().numpy().astype(np.float64))
        assert np.array_equal(outs[0], outs[1])
        assert rel(outs[0], y1) < 1e-5


@pytest.mark.parametrize("name", ["random", "mcf"])
def test_cg_f32_agrees_with_fp64(name):
    """The mixed form's FP32 inner CG alone (help_pcg_cg_f32) reaches the FP64
    solution to FP32 accuracy: 1e-3 relative at a 1e-5 residual reduction."""
    lp = CASES[name]()
    rng = np.random.default_rng(13)
    d = np.exp(rng.uniform(-3, 3, lp.n))
    b = rng.standard_normal(lp.m)
    with backend.GpuNormalEquations(pivots=16, precision="mixed", cg_tol=1e-5, cg_max_iter=20000) as g:
        g.LinearEquation_Construct(lp)
        g.RenewLinearEquation(d)
        x64, it64 = g.cg(b)
        x32, it32 = g.cg(b, fp32=True)
    assert it32 < 20000
    assert rel(x32, x64) < 1e-3


@pytest.mark.parametrize("name", ["random", "block"])
def test_direct_form_all_rows_pivots(name):
    """pivots = m: the partial Cholesky becomes the full factorisation of
    A D^-1 A^T, CG converges in one or two iterations, and the solve agrees
    with the oracle's (a direct solve; the second oracle for the PCG path)."""
    lp = CASES[name]()
    rng = np.random.default_rng(14)
    d = np.exp(rng.uniform(-4, 4, lp.n))
    b1 = rng.standard_normal(lp.n)
    b2 = rng.standard_normal(lp.m)
    with backend.GpuNormalEquations(pivots=lp.m, cg_tol=1e-12, cg_max_iter=100) as g:
        g.LinearEquation_Construct(lp)
        g.RenewLinearEquation(d)
        x1, x2 = g.SolveLinearEquation(d, b1, b2)
        st = g.stats()
    assert st["pivots"] == lp.m and st["nnz_c"] == 0
    assert st["cg_iterations"] <= 3
    ora = ob.OracleNormalEquations(pivots=10, rule=ob.PIVOT_GREEDY, tol=1e-14, max_iter=200000)
    ora.LinearEquation_Construct(lp)
    ox1, ox2 = ora.SolveLinearEquation(d, b1, b2)
    assert rel(x2, ox2) < 1e-8
    assert rel(x1, ox1) < 1e-8


@pytest.mark.parametrize("name", ["zipf", "longrows", "block"])
def test_graph_cg_bitwise_repeatable(name):
    """Two CG solves of the same system on the multi-kernel graph path give
    bitwise the same solution and iteration count, in FP64 and FP32: every
    reduction adds its blocks' partials in block order in the last block,
    which takes its ticket only after every warp of every block has written
    (k_p3's last block reads all of w = r_P - C^T z_N; these cases have C^T
    rows taken by a warp each or split over CTAs)."""
    lp = CASES[name]()
    rng = np.random.default_rng(15)
    d = np.exp(rng.uniform(-4, 4, lp.n))
    b = rng.standard_normal(lp.m)
    with backend.GpuNormalEquations(pivots=32, precision="mixed", cg_tol=1e-10, cg_max_iter=3000,
                                    cg_path="graph") as g:
        g.LinearEquation_Construct(lp)
        g.RenewLinearEquation(d)
        assert g.stats()["nnz_c"] > 0
        for fp32 in (False, True):
            (x1, i1), (x2, i2) = g.cg(b, fp32=fp32), g.cg(b, fp32=fp32)
            assert g.stats()["cg_path_used"] == 1
            assert i1 == i2 and np.array_equal(x1, x2), (name, fp32)
