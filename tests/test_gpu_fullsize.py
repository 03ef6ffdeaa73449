"""The benchmark's configurations at full size (configs 1-4: up to 1.9M x 8M
with 104M nonzeros, Zipf rows of ~43k entries in config 2, 4,000 linking rows
of ~16k entries in config 4).

Against the oracle (the reference's own loops restated, O(nnz) per product):
  * A x, A^T y (CSRMV_N / CSRMV_T, Helper.cpp:57-81) to 1e-12 relative and
    A D^-1 A^T v (CSRMV_T, scale, CSRMV_N) to 1e-11;
  * diag(A D^-1 A^T) (PCG.cpp:41-46) to 1e-13, and the k largest of it --
    the pivots at the configuration's own k -- exactly;
  * the explicit upper triangle of A D^-1 A^T (ADAt_Allocate + ADAt_Calc,
    Helper.cpp:215-377) bit for bit at configs 1-3 (config 2 has 2,137 rows
    past the per-warp sort, up to 245,908 contributions each); at config 4
    (~430M entries) its diagonal against diag(G) to 1e-13 and 40 rows, the
    linking rows among them, against numpy to 1e-13;
  * at k = 8 given pivots: the Schur diagonal D_S (PCG.cpp:60-120) to 1e-9 of
    diag(G), one preconditioner application (PCG.cpp:183-196) to 1e-8, and
    10 CG iterations (PCG.cpp:333-394; tolerance 1e-30 so both run exactly 10)
    to 1e-6 -- a small k keeps the oracle's O(k nnz) factor build in seconds.

And through properties that hold whatever the size:

  * G = A D^-1 A^T is symmetric:      x . G y == y . G x
  * and linear:                      G (a x + b y) == a G x + b G y
  * the fused product equals A (D^-1 (A^T x)) from the separate A^T and A
    products (the reference's CSRMV_T, scale, CSRMV_N order)
  * FP32 copies agree with FP64 to FP32 accuracy
  * the preconditioner is symmetric and positive: r . M^-1 s == s . M^-1 r,
    r . M^-1 r > 0
  * CG lowers the energy 1/2 x.Gx - b.x below its value at x = 0 (the
    quantity CG minimises; the residual's 2-norm need not fall)

Tolerances: 1e-12 relative for FP64 identities (sums of up to ~10^5 terms
per row in different orders), 1e-5 for FP32 against FP64.
"""
import numpy as np
import pytest

from help_gb300 import backend, lp as L
from oracle import bindings as ob

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module", params=[1, 2, 3, 4])
def system(request):
    config = request.param
    lp = L.make_lp(config, 0)
    rng = np.random.default_rng(100 + config)
    d = np.exp(rng.uniform(np.log(1e-8), np.log(1e8), lp.n))
    k = L.config_pivots(config)
    g = backend.GpuNormalEquations(pivots=k, precision="mixed", cg_tol=1e-6, cg_max_iter=200)
    g.LinearEquation_Construct(lp)
    g.RenewLinearEquation(d)
    yield config, lp, d, g, rng
    g.close()


@pytest.fixture(scope="module")
def csr(system):
    config, lp, d, g, rng = system
    return lp.csr()


def test_products_match_oracle(system, csr):
    config, lp, d, g, rng = system
    rp, ci, v = csr
    x, w = rng.standard_normal(lp.n), rng.standard_normal(lp.m)
    assert rel(g.matvec("A", x), ob.csrmv_n(rp, ci, v, x, lp.m, lp.n)) < 1e-12
    assert rel(g.matvec("AT", w), ob.csrmv_t(rp, ci, v, w, lp.m, lp.n)) < 1e-12
    want = ob.csrmv_n(rp, ci, v, ob.csrmv_t(rp, ci, v, w, lp.m, lp.n) / d, lp.m, lp.n)
    assert rel(g.matvec("ADAT", w), want) < 1e-11


def test_diagonal_and_pivots_match_oracle(system, csr):
    config, lp, d, g, rng = system
    rp, ci, v = csr
    piv, dg, ds = g.pivots()
    dg_ref = ob.diag_adat(rp, ci, v, d, lp.m)
    assert rel(dg, dg_ref) < 1e-13
    assert len(piv) == L.config_pivots(config)
    assert np.array_equal(piv, ob.topk(dg, len(piv)))


def test_adat_assembly_matches_oracle(system, csr):
    config, lp, d, g, rng = system
    rp, ci, v = csr
    w = 1.0 / d
    grp, gcol, gval = g.adat(w)
    if config != 4:
        orp, ocol, oval = ob.adat(rp, ci, v, lp.col_ptr, lp.row_ind, lp.val, w, lp.m, lp.n)
        assert np.array_equal(grp, orp) and np.array_equal(gcol, ocol) and np.array_equal(gval, oval)
        return
    rows = np.arange(lp.m)
    assert np.all(gcol[grp[:-1]] == rows)  # the diagonal leads every row (columns ascending, k >= i)
    dg = ob.diag_adat(rp, ci, v, d, lp.m)
    assert np.max(np.abs(gval[grp[:-1]] - dg) / dg) < 1e-13
    picks = np.concatenate([rng.choice(lp.m - 4000, 30, replace=False), lp.m - 4000 + rng.choice(4000, 10, replace=False)])
    for i in picks:
        acc = {}
        for e in range(rp[i], rp[i + 1]):
            j = ci[e]
            q = np.arange(lp.col_ptr[j], lp.col_ptr[j + 1])
            q = q[lp.row_ind[q] >= i]
            for k, a in zip(lp.row_ind[q], v[e] * w[j] * lp.val[q]):
                acc[k] = acc.get(k, 0.0) + a
        ks = np.array(sorted(acc), np.int64)
        want = np.array([acc[k] for k in ks])
        assert np.array_equal(gcol[grp[i]:grp[i + 1]], ks), i
        assert np.max(np.abs(gval[grp[i]:grp[i + 1]] - want)) <= 1e-13 * np.max(np.abs(want)), i


def test_schur_precond_and_capped_cg_match_oracle(system, csr):
    config, lp, d, g0, rng = system
    rp, ci, v = csr
    k, iters = 8, 10
    b = rng.standard_normal(lp.m)
    r = rng.standard_normal(lp.m)
    with backend.GpuNormalEquations(pivots=k, cg_tol=1e-30, cg_max_iter=iters) as g:
        g.LinearEquation_Construct(lp)
        g.RenewLinearEquation(d)
        piv, dg, ds = g.pivots()
        z = g.precond_apply(r)
        x, it = g.cg(b)
    pc = ob.PartialCholesky(rp, ci, v, d, lp.m, lp.n, k, ob.PIVOT_GIVEN, piv)
    non = np.ones(lp.m, bool)
    non[piv] = False
    ds_ref = pc.diag_s
    good = non & (ds_ref > 1e-6 * dg)  # rows whose Schur diagonal is not pure cancellation
    assert np.max(np.abs(ds[good] - ds_ref[good]) / dg[good]) < 1e-9
    assert rel(z, pc.apply(r)) < 1e-8
    del pc
    xo, ito = ob.pcg(rp, ci, v, d, b, lp.m, lp.n, k, ob.PIVOT_GIVEN, piv, tol=1e-30, max_iter=iters)
    assert it == ito == iters
    assert rel(x, xo) < 1e-6


def test_product_symmetric_and_linear(system):
    config, lp, d, g, rng = system
    x, y = rng.standard_normal(lp.m), rng.standard_normal(lp.m)
    gx, gy = g.matvec("ADAT", x), g.matvec("ADAT", y)
    assert abs(x @ gy - y @ gx) <= 1e-12 * np.linalg.norm(x) * np.linalg.norm(gy)
    a, b = 0.75, -1.5
    assert rel(g.matvec("ADAT", a * x + b * y), a * gx + b * gy) < 1e-12


def test_fused_product_matches_separate_passes(system):
    config, lp, d, g, rng = system
    x = rng.standard_normal(lp.m)
    t = g.matvec("AT", x) / d
    assert rel(g.matvec("ADAT", x), g.matvec("A", t)) < 1e-12


def test_fp32_copy_agrees_with_fp64(system):
    torch = pytest.importorskip("torch")
    config, lp, d, g, rng = system
    x = rng.standard_normal(lp.m)
    y64 = g.matvec("ADAT", x)
    x32 = torch.from_numpy(x.astype(np.float32)).cuda()
    y32 = torch.empty(lp.m, dtype=torch.float32, device="cuda")
    g.matvec_dev("ADAT", x32.data_ptr(), y32.data_ptr(), fp32=True)
    torch.cuda.synchronize()
    assert rel(y32.cpu().numpy().astype(np.float64), y64) < 1e-5


def test_preconditioner_symmetric_positive(system):
    config, lp, d, g, rng = system
    r, s = rng.standard_normal(lp.m), rng.standard_normal(lp.m)
    mr, ms = g.precond_apply(r), g.precond_apply(s)
    assert abs(r @ ms - s @ mr) <= 1e-9 * np.linalg.norm(r) * np.linalg.norm(ms)
    assert r @ mr > 0 and s @ ms > 0


def test_cg_lowers_the_energy(system):
    config, lp, d, g, rng = system
    b = rng.standard_normal(lp.m)
    x, it = g.cg(b)
    assert it > 0
    energy = 0.5 * (x @ g.matvec("ADAT", x)) - b @ x
    assert energy < 0.0
