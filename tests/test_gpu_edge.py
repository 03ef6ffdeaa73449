"""Edge cases through the C ABI: degenerate and ragged inputs, bad input
rejected with a clear error, the context usable afterwards.  Small systems,
checked against dense numpy solves (1e-10 relative; products 1e-13)."""
import numpy as np
import pytest

from help_gb300 import backend

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def _csc(dense):
    m, n = dense.shape
    cp, ri, v = [0], [], []
    for j in range(n):
        for i in range(m):
            if dense[i, j] != 0.0:
                ri.append(i)
                v.append(dense[i, j])
        cp.append(len(ri))
    return (np.array(cp, np.int32), np.array(ri, np.int32), np.array(v, np.float64))


def _solve_ref(dense, d, b1, b2, delta=0.0):
    G = (dense / d) @ dense.T + delta * np.eye(dense.shape[0])
    x2 = np.linalg.solve(G, (dense / d) @ b1 - b2)
    x1 = (b1 - dense.T @ x2) / d
    return x1, x2


def test_one_by_one():
    cp, ri, v = _csc(np.array([[2.5]]))
    with backend.GpuNormalEquations(pivots=1, cg_tol=1e-14) as g:
        g.LinearEquation_Construct(m=1, n=1, col_ptr=cp, row_ind=ri, val=v)
        d = np.array([4.0])
        g.RenewLinearEquation(d)
        x1, x2 = g.SolveLinearEquation(d, np.array([1.0]), np.array([3.0]))
    r1, r2 = _solve_ref(np.array([[2.5]]), d, np.array([1.0]), np.array([3.0]))
    assert rel(x2, r2) < 1e-14 and rel(x1, r1) < 1e-14


@pytest.mark.parametrize("pivots", [0, 2])
def test_empty_columns(pivots):
    rng = np.random.default_rng(1)
    A = rng.standard_normal((5, 9))
    A[:, [1, 4, 8]] = 0.0  # columns without nonzeros
    A[rng.random(A.shape) < 0.3] = 0.0
    A[:, 0] = rng.standard_normal(5)  # keep every row non-empty
    cp, ri, v = _csc(A)
    d = np.exp(rng.uniform(-2, 2, 9))
    b1, b2 = rng.standard_normal(9), rng.standard_normal(5)
    with backend.GpuNormalEquations(pivots=pivots, cg_tol=1e-14, cg_max_iter=1000) as g:
        g.LinearEquation_Construct(m=5, n=9, col_ptr=cp, row_ind=ri, val=v)
        g.RenewLinearEquation(d)
        x1, x2 = g.SolveLinearEquation(d, b1, b2)
    r1, r2 = _solve_ref(A, d, b1, b2)
    assert rel(x2, r2) < 1e-10 and rel(x1, r1) < 1e-10


def test_empty_row_is_an_error_unless_regularised():
    rng = np.random.default_rng(2)
    A = rng.standard_normal((4, 7))
    A[2, :] = 0.0  # a row without nonzeros: A D^-1 A^T is singular
    cp, ri, v = _csc(A)
    d = np.exp(rng.uniform(-1, 1, 7))
    b1, b2 = rng.standard_normal(7), rng.standard_normal(4)
    with backend.GpuNormalEquations(pivots=1) as g:
        g.LinearEquation_Construct(m=4, n=7, col_ptr=cp, row_ind=ri, val=v)
        with pytest.raises(backend.BackendError, match="no nonzeros"):
            g.RenewLinearEquation(d)
        # the context stays usable
        y = g.matvec("A", np.ones(7))
        assert rel(y, A @ np.ones(7)) < 1e-14
    with backend.GpuNormalEquations(pivots=1, delta=1e-3, cg_tol=1e-14, cg_max_iter=1000) as g:
        g.LinearEquation_Construct(m=4, n=7, col_ptr=cp, row_ind=ri, val=v)
        g.RenewLinearEquation(d)
        x1, x2 = g.SolveLinearEquation(d, b1, b2)
    r1, r2 = _solve_ref(A, d, b1, b2, delta=1e-3)
    assert rel(x2, r2) < 1e-10


def test_bad_matrices_are_rejected():
    cp = np.array([0, 2, 3], np.int32)
    v = np.ones(3)
    with backend.GpuNormalEquations(pivots=1) as g:
        with pytest.raises(backend.BackendError, match="strictly increasing"):
            g.LinearEquation_Construct(m=3, n=2, col_ptr=cp, row_ind=np.array([2, 1, 0], np.int32), val=v)
        with pytest.raises(backend.BackendError, match="out of range"):
            g.LinearEquation_Construct(m=3, n=2, col_ptr=cp, row_ind=np.array([0, 3, 1], np.int32), val=v)
        with pytest.raises(backend.BackendError, match="monotone"):
            g.LinearEquation_Construct(m=3, n=2, col_ptr=np.array([0, 2, 1], np.int32),
                                       row_ind=np.array([0, 1, 2], np.int32), val=v)
        g.LinearEquation_Construct(m=3, n=2, col_ptr=cp, row_ind=np.array([0, 1, 2], np.int32), val=v)
        with pytest.raises(backend.BackendError, match="already constructed"):
            g.LinearEquation_Construct(m=3, n=2, col_ptr=cp, row_ind=np.array([0, 1, 2], np.int32), val=v)


def test_solve_before_construct_and_renew():
    with backend.GpuNormalEquations(pivots=1) as g:
        g.m, g.n = 1, 2  # shapes for the Python wrapper; the library has no matrix yet
        with pytest.raises(backend.BackendError, match="construct first"):
            g.SolveLinearEquation(np.ones(2), np.ones(2), np.ones(1))
        with pytest.raises(backend.BackendError, match="renew first"):
            g.cg(np.ones(1))


def test_ragged_matrix_product():
    """One row with every column, the others with one or two entries."""
    rng = np.random.default_rng(3)
    m, n = 60, 400
    A = np.zeros((m, n))
    A[0, :] = rng.standard_normal(n)
    for i in range(1, m):
        A[i, rng.choice(n, size=1 + (i % 2), replace=False)] = rng.standard_normal(1 + (i % 2))
    cp, ri, v = _csc(A)
    d = np.exp(rng.uniform(-3, 3, n))
    w = rng.standard_normal(m)
    with backend.GpuNormalEquations(pivots=4) as g:
        g.LinearEquation_Construct(m=m, n=n, col_ptr=cp, row_ind=ri, val=v)
        g.RenewLinearEquation(d)
        y = g.matvec("ADAT", w)
    assert rel(y, (A / d) @ (A.T @ w)) < 1e-13


def test_iteration_cap_is_an_error_unless_cap_ok():
    """A solve whose CG stops at cg_max_iter before cg_tol returns
    HELP_E_NOT_CONVERGED (x_1, x_2 still written); with cap_ok it returns
    HELP_OK and stats.converged = 0.  The reference's CG has no cap
    (PCG.cpp:333-394 runs until ||r|| < 1e-20 ||r0||)."""
    from help_gb300 import lp as L, native

    lp = L.generate(L.spec_random(300, 900, 5), 3)
    rng = np.random.default_rng(3)
    d = np.exp(rng.uniform(-3, 3, lp.n))
    b1, b2 = rng.standard_normal(lp.n), rng.standard_normal(lp.m)
    for precision in ("fp64", "mixed"):
        with backend.GpuNormalEquations(pivots=4, precision=precision, cg_tol=1e-14, cg_max_iter=3,
                                        inner_max_iter=3, ir_max_outer=1) as g:
            g.LinearEquation_Construct(lp)
            g.RenewLinearEquation(d)
            with pytest.raises(backend.BackendError) as e:
                g.SolveLinearEquation(d, b1, b2)
            assert e.value.code == native.HELP_E_NOT_CONVERGED
            assert g.stats()["converged"] == 0
        with backend.GpuNormalEquations(pivots=4, precision=precision, cg_tol=1e-14, cg_max_iter=3,
                                        inner_max_iter=3, ir_max_outer=1, cap_ok=True) as g:
            g.LinearEquation_Construct(lp)
            g.RenewLinearEquation(d)
            x1, x2 = g.SolveLinearEquation(d, b1, b2)
            st = g.stats()
            assert st["converged"] == 0 and np.all(np.isfinite(x2)) and np.all(np.isfinite(x1))
        # the same context solves fully when the cap allows it
        with backend.GpuNormalEquations(pivots=4, precision=precision, cg_tol=1e-12, cg_max_iter=100000) as g:
            g.LinearEquation_Construct(lp)
            g.RenewLinearEquation(d)
            g.SolveLinearEquation(d, b1, b2)
            assert g.stats()["converged"] == 1


def test_context_with_fewer_pivots_leaves_an_earlier_one_usable():
    """Kernel launch limits (dynamic shared memory sized by the pivot count)
    are per function, shared by every context: constructing a second
    context with fewer pivots must not lower them under the first, whose
    CG graph is captured afterwards."""
    from help_gb300 import lp as L

    lp = L.generate(L.spec_random(2000, 6000, 5), 5)
    rng = np.random.default_rng(5)
    d = np.exp(rng.uniform(-4, 4, lp.n))
    b = rng.standard_normal(lp.m)
    with backend.GpuNormalEquations(pivots=512, cg_tol=1e-10, cg_max_iter=20000, cg_path="graph") as big:
        big.LinearEquation_Construct(lp)
        big.RenewLinearEquation(d)
        with backend.GpuNormalEquations(pivots=2, cg_tol=1e-10, cg_max_iter=20000, cg_path="graph") as small:
            small.LinearEquation_Construct(lp)
            small.RenewLinearEquation(d)
            xs, _ = small.cg(b)
        xb, _ = big.cg(b)
        z = big.precond_apply(b)
        gx = big.matvec("ADAT", xb)
    assert rel(gx, b) < 1e-8 and rel(xb, xs) < 1e-6 and np.all(np.isfinite(z))


def test_mixed_form_chooses_fp32_only_where_it_can_pay():
    """The mixed form runs FP32 refinement only on the bandwidth-bound graph
    path and while max(d)/min(d) <= mixed_max_d_spread; otherwise it goes to
    plain FP64 PCG up front.  Either way the FP64 residual meets ir_tol."""
    from help_gb300 import lp as L

    rng = np.random.default_rng(8)
    big = L.generate(L.spec_random(20000, 80000, 8), 8)      # graph path
    small = L.generate(L.spec_random(300, 900, 5), 8)        # resident path
    cases = [(big, 1e2, "graph", 1), (big, 1e12, "graph", 0), (small, 1e2, "auto", 0)]
    for lp, spread, path, want in cases:
        d = np.exp(rng.uniform(0.0, np.log(spread), lp.n))
        b1, b2 = rng.standard_normal(lp.n), rng.standard_normal(lp.m)
        with backend.GpuNormalEquations(pivots=16, precision="mixed", ir_tol=1e-10, cg_tol=1e-10,
                                        cg_path=path) as g:
            g.LinearEquation_Construct(lp)
            g.RenewLinearEquation(d)
            g.SolveLinearEquation(d, b1, b2)
            st = g.stats()
        assert st["fp32_chosen"] == want, (lp.m, spread, st["fp32_chosen"])
        assert abs(st["d_spread"] - d.max() / d.min()) <= 1e-12 * st["d_spread"]
        assert st["rel_residual"] < 1e-9
        assert (st["cg_iterations_fp32"] > 0) == bool(want)
