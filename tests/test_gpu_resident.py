"""The shared-memory-resident cluster CG (cg_path "resident") against the
multi-kernel graph path and dense solves: pivot counts 0..64, delta > 0,
systems smaller than the cluster (CTAs with no rows), runs that span several
launches (state saved and restored), the iteration cap, and FP32.

Tolerances: the two paths add the same products in different orders, so
solutions agree to 1e-8 relative (FP64, after reaching the same stopping
rule) and 1e-4 (FP32); iteration counts within 3.
"""
import numpy as np
import pytest

from help_gb300 import backend, lp as L

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def system():
    lp = L.generate(L.spec_random(400, 1200, 5), 3)
    rng = np.random.default_rng(21)
    d = np.exp(rng.uniform(-6, 6, lp.n))
    b = rng.standard_normal(lp.m)
    return lp, d, b


def _cg(lp, d, b, path, fp32=False, **kw):
    with backend.GpuNormalEquations(precision="mixed" if fp32 else "fp64", cg_path=path, **kw) as g:
        g.LinearEquation_Construct(lp)
        g.RenewLinearEquation(d)
        x, it = g.cg(b, fp32=fp32)
        st = g.stats()
    return x, it, st


@pytest.mark.parametrize("k", [0, 1, 10, 64])
@pytest.mark.parametrize("delta", [0.0, 1e-3])
def test_resident_matches_graph(system, k, delta):
    lp, d, b = system
    kw = dict(pivots=k, delta=delta, cg_tol=1e-10, cg_max_iter=20000)
    xr, itr, st = _cg(lp, d, b, "resident", **kw)
    assert st["cg_path_used"] == 3
    xg, itg, _ = _cg(lp, d, b, "graph", **kw)
    assert itr > 64  # more than the first launch's 64 iterations: state carried between launches
    assert abs(itr - itg) <= 3
    assert rel(xr, xg) < 1e-8


def test_resident_iteration_cap(system):
    lp, d, b = system
    xr, itr, st = _cg(lp, d, b, "resident", pivots=10, cg_tol=1e-30, cg_max_iter=77)
    xg, itg, _ = _cg(lp, d, b, "graph", pivots=10, cg_tol=1e-30, cg_max_iter=77)
    assert st["cg_path_used"] == 3 and itr == itg == 77
    # mid-run iterates of an ill-conditioned system: the paths' different
    # summation orders grow to ~1e-8 by iteration 77
    assert rel(xr, xg) < 1e-6


def test_resident_fp32(system):
    lp, d, b = system
    xr, itr, st = _cg(lp, d, b, "resident", fp32=True, pivots=16, cg_tol=1e-5, cg_max_iter=20000)
    assert st["cg_path_used"] == 3
    xg, itg, _ = _cg(lp, d, b, "graph", fp32=True, pivots=16, cg_tol=1e-5, cg_max_iter=20000)
    assert abs(itr - itg) <= 3
    assert rel(xr, xg) < 1e-4


@pytest.mark.parametrize("m,n", [(3, 7), (10, 30), (67, 150)])
def test_resident_small_systems(m, n):
    """Fewer rows than 4 per CTA: most CTAs own no rows or columns."""
    rng = np.random.default_rng(m)
    A = rng.standard_normal((m, n)) * (rng.random((m, n)) < 0.4)
    A[np.arange(m), rng.integers(0, n, m)] = 1.0  # no empty rows
    cp, ri, v = [0], [], []
    for j in range(n):
        nz = np.nonzero(A[:, j])[0]
        ri += nz.tolist()
        v += A[nz, j].tolist()
        cp.append(len(ri))
    d = np.exp(rng.uniform(-2, 2, n))
    b = rng.standard_normal(m)
    for k in (0, min(3, m)):
        with backend.GpuNormalEquations(pivots=k, cg_tol=1e-13, cg_max_iter=10000, cg_path="resident") as g:
            g.LinearEquation_Construct(m=m, n=n, col_ptr=np.array(cp, np.int32), row_ind=np.array(ri, np.int32),
                                       val=np.array(v))
            g.RenewLinearEquation(d)
            x, it = g.cg(b)
            assert g.stats()["cg_path_used"] == 3
        G = (A / d) @ A.T
        assert rel(x, np.linalg.solve(G, b)) < 1e-8


@pytest.mark.parametrize("name,spec,seed", [("random 8000 x 24000", L.spec_random(8000, 24000, 5), 5),
                                            ("mcf 48 x 48 x 4", L.spec_mcf(48, 4, 3), 6)])
@pytest.mark.parametrize("fp32", [False, True])
def test_resident_matrix_in_l2(name, spec, seed, fp32):
    """Systems whose matrix slices do not fit in shared memory next to the
    vectors (FP64 slices alone: 12 bytes x 2 nnz / 16 CTAs > 227 KB with the
    8 m bytes of p) run the resident kernel with the matrix read from L2."""
    lp = L.generate(spec, seed)
    assert 8 * lp.m + 12 * 2 * lp.nnz / 16 > 227 * 1024 or fp32
    rng = np.random.default_rng(seed)
    d = np.exp(rng.uniform(-5, 5, lp.n))
    b = rng.standard_normal(lp.m)
    tol = 1e-5 if fp32 else 1e-10
    kw = dict(pivots=16, cg_tol=tol, cg_max_iter=50000)
    xr, itr, st = _cg(lp, d, b, "resident", fp32=fp32, **kw)
    assert st["cg_path_used"] == 3
    xg, itg, _ = _cg(lp, d, b, "graph", fp32=fp32, **kw)
    assert abs(itr - itg) <= max(3, 0.02 * itg)
    assert rel(xr, xg) < (1e-4 if fp32 else 1e-8)


@pytest.mark.parametrize("name,spec,seed", [("smem matrix", L.spec_random(400, 1200, 5), 3),
                                            ("L2 matrix", L.spec_random(8000, 24000, 5), 5)])
def test_resident_repeatable(name, spec, seed):
    """The same solve twice gives the same bits (every reduction in a fixed
    order, no atomics on values)."""
    lp = L.generate(spec, seed)
    rng = np.random.default_rng(seed)
    d = np.exp(rng.uniform(-5, 5, lp.n))
    b = rng.standard_normal(lp.m)
    with backend.GpuNormalEquations(pivots=16, cg_tol=1e-10, cg_max_iter=50000, cg_path="resident") as g:
        g.LinearEquation_Construct(lp)
        g.RenewLinearEquation(d)
        x1, i1 = g.cg(b)
        x2, i2 = g.cg(b)
        assert g.stats()["cg_path_used"] == 3
    assert i1 == i2 and np.array_equal(x1, x2)
