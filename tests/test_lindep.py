"""Linear-dependency presolve (help_lp_remove_dependent_rows, the purpose of
the reference's Presolve_Lindep.cpp): as many rows dropped as A is short of
full row rank (numpy's SVD rank is the independent check), on every path of
the elimination -- sparse only, the direct dense finish and the sketched
dense finish; b checked along each dependency (primal infeasibility
reported); full-rank instances pass unchanged; the reduced LP has the
original's optimum (HiGHS); random sparse matrices at 10^4 rows are reported
as beyond the presolve's limits."""
import time

import numpy as np
import pytest

from help_gb300 import lp as L


def dense(lp):
    A = np.zeros((lp.m, lp.n))
    for j in range(lp.n):
        A[lp.row_ind[lp.col_ptr[j]:lp.col_ptr[j + 1]], j] = lp.val[lp.col_ptr[j]:lp.col_ptr[j + 1]]
    return A


def from_dense(A, b, c, row_type=None, n_struct=None):
    m, n = A.shape
    cp, ri, v = [0], [], []
    for j in range(n):
        nz = np.nonzero(A[:, j])[0]
        ri += nz.tolist()
        v += A[nz, j].tolist()
        cp.append(len(ri))
    return L.LP(m=m, n=n, n_struct=n if n_struct is None else n_struct, col_ptr=np.array(cp, np.int32),
                row_ind=np.array(ri, np.int32), val=np.array(v), b=np.array(b, float), c=np.array(c, float),
                row_type=row_type or b"E" * m)


def check_reduced(lp, red, removed):
    """red is lp without the flagged rows, in order, every column kept."""
    keep = ~removed
    assert red.m == int(keep.sum()) and red.n == lp.n and red.n_struct == lp.n_struct
    assert np.array_equal(dense(red), dense(lp)[keep])
    assert np.array_equal(red.b, lp.b[keep]) and np.array_equal(red.c, lp.c)


@pytest.mark.parametrize("spec,seed", [(L.spec_random(200, 600, 5), 1), (L.spec_mcf(6, 2, 2), 2),
                                       (L.spec_zipf(300, 900, 4, 1.3, 20), 3)])
def test_full_rank_unchanged(spec, seed):
    lp = L.generate(spec, seed)
    red, removed = L.remove_dependent_rows(lp)
    assert not removed.any()
    for f in ("col_ptr", "row_ind", "val", "b", "c"):
        assert np.array_equal(getattr(red, f), getattr(lp, f)), f


# (m, n, nonzeros per column, seed): random instances that finish sparse
# (300 x 330), through the direct dense finish (600 x 660, 1000 x 1100: few
# active columns left) and the sketched one (600 x 1800: many); the seeds of
# 600 x 700 x 4 and 1000 x 1100 x 5 include rank-deficient ones (rows that
# share their only columns)
@pytest.mark.parametrize("m,n,k,seed", [(300, 330, 5, 0), (600, 660, 5, 0), (600, 700, 4, 0), (600, 700, 4, 2),
                                        (1000, 1100, 5, 2), (600, 1800, 5, 1)])
def test_rows_removed_equal_rank_deficiency(m, n, k, seed):
    lp = L.generate(L.spec_random(m, n, k), seed)
    red, removed = L.remove_dependent_rows(lp)
    A = dense(lp)
    assert int(removed.sum()) == m - np.linalg.matrix_rank(A)
    assert np.linalg.matrix_rank(dense(red)) == red.m
    check_reduced(lp, red, removed)


@pytest.mark.parametrize("m,n", [(60, 200), (600, 1800)])
def test_combinations_duplicates_and_empty_rows_dropped(m, n):
    lp = L.generate(L.spec_random(m, n, 4 if m < 100 else 5), 5)
    A, b = dense(lp), lp.b.copy()
    rng = np.random.default_rng(5)
    i1, i2, i3, i4 = rng.choice(m, 4, replace=False)
    extra = [1.5 * A[i1] - 0.25 * A[i2] + 2.0 * A[i3],  # a combination
             -2.0 * A[i4],                               # a scaled duplicate
             np.zeros(lp.n)]                             # an empty row
    eb = [1.5 * b[i1] - 0.25 * b[i2] + 2.0 * b[i3], -2.0 * b[i4], 0.0]
    big = from_dense(np.vstack([A] + extra), np.append(b, eb), lp.c)
    red, removed = L.remove_dependent_rows(big)
    assert removed.sum() == 3 and removed[-1]
    # which row of a dependent set goes is the elimination's choice; the rank
    # and the row space are what must hold
    assert red.m == m and np.linalg.matrix_rank(dense(red)) == m
    check_reduced(big, red, removed)


def test_infeasible_dependency_reported():
    lp = L.generate(L.spec_random(40, 120, 4), 6)
    A, b = dense(lp), lp.b.copy()
    big = from_dense(np.vstack([A, A[2] + A[5]]), np.append(b, b[2] + b[5] + 1e-3), lp.c)
    with pytest.raises(ValueError, match="infeasible"):
        L.remove_dependent_rows(big)
    with pytest.raises(ValueError, match="infeasible"):
        L.remove_dependent_rows(from_dense(np.vstack([A, np.zeros(lp.n)]), np.append(b, 3.0), lp.c))
    # the bound on y^T b is 1e-8 sqrt(1 + |b|_2^2): half of it passes, twice fails
    rhs = b[2] + b[5]
    bound = 1e-8 * np.sqrt(1.0 + b @ b + rhs * rhs)
    ok = from_dense(np.vstack([A, A[2] + A[5]]), np.append(b, rhs + 0.5 * bound), lp.c)
    red, removed = L.remove_dependent_rows(ok)
    assert removed.sum() == 1
    with pytest.raises(ValueError, match="infeasible"):
        L.remove_dependent_rows(from_dense(np.vstack([A, A[2] + A[5]]), np.append(b, rhs + 2.0 * bound), lp.c))


def test_ungrounded_flow_one_row_per_commodity_and_same_optimum():
    """Multicommodity flow with every node row kept (each commodity's rows sum
    to zero, so A is K rows short of full rank): one node row per commodity
    dropped, and the reduced LP has the optimum of the grounded one."""
    scipy_opt = pytest.importorskip("scipy.optimize")
    G, K = 4, 2
    full = L.generate(L.spec_mcf(G, K, 2, grounded=False), 7)
    grounded = L.generate(L.spec_mcf(G, K, 2), 7)
    N = G * G
    red, removed = L.remove_dependent_rows(full)
    assert removed.sum() == K
    for k in range(K):
        assert removed[k * N:(k + 1) * N].sum() == 1
    assert not removed[K * N:].any()
    check_reduced(full, red, removed)
    assert np.linalg.matrix_rank(dense(red)) == red.m
    opt = [scipy_opt.linprog(x.c, A_eq=dense(x), b_eq=x.b, bounds=(0, None), method="highs")
           for x in (full, red, grounded)]
    assert all(r.status == 0 for r in opt)
    assert abs(opt[0].fun - opt[1].fun) <= 1e-9 * (1 + abs(opt[0].fun))
    assert abs(opt[1].fun - opt[2].fun) <= 1e-9 * (1 + abs(opt[1].fun))
    # duals of the reduced LP, zero on the dropped rows, are duals of the full one
    y_red = -opt[1].eqlin.marginals
    y = L.expand_duals(y_red, removed)
    assert np.allclose(dense(full).T @ y, dense(red).T @ y_red)
    assert abs(full.b @ y - red.b @ y_red) <= 1e-9 * (1 + abs(opt[1].fun))


def test_ungrounded_flow_200x200_grid_8_commodities():
    """The 200 x 200 grid, 8-commodity flow (479,200 rows, 4.0M nonzeros) with
    every node row kept: the network rows eliminate without fill, one row per
    commodity goes, in seconds."""
    G, K = 200, 8
    lp = L.generate(L.spec_mcf(G, K, grounded=False), 0)
    t = time.perf_counter()
    red, removed = L.remove_dependent_rows(lp)
    elapsed = time.perf_counter() - t
    N = G * G
    assert removed.sum() == K
    assert all(removed[k * N:(k + 1) * N].sum() == 1 for k in range(K))
    assert red.m == lp.m - K and red.nnz == lp.nnz - int(
        sum(np.count_nonzero(lp.row_ind == i) for i in np.nonzero(removed)[0]))
    assert elapsed < 30.0


def test_random_10k_rows_beyond_limits():
    """Random sparse A at 8,000 x 24,000 fills in past the sparse limits and
    leaves a remainder too large for the dense finish: reported quickly, no
    rows removed."""
    lp = L.generate(L.spec_random(8000, 24000, 5), 1)
    t = time.perf_counter()
    with pytest.raises(L.PresolveNotApplicable):
        L.remove_dependent_rows(lp)
    assert time.perf_counter() - t < 30.0


def test_ungrounded_flow_presolved_then_solved_by_hsd():
    """The whole flow on the host: presolve, then the HSD driver over the
    oracle's normal-equations backend reaches the grounded instance's
    optimum, and its x is feasible for the full (unreduced) rows too."""
    from help_gb300 import hsd
    from oracle import bindings as ob

    full = L.generate(L.spec_mcf(8, 3, 2, grounded=False), 4)
    grounded = L.generate(L.spec_mcf(8, 3, 2), 4)
    red, removed = L.remove_dependent_rows(full)
    assert removed.sum() == 3
    runs = [hsd.solve_lp(lp, ob.OracleNormalEquations(pivots=10, tol=1e-14, max_iter=10**6).ne_backend(),
                         want_solution=True) for lp in (red, grounded)]
    assert all(r["status"] == 0 and r["rel_gap"] < 1e-8 for r in runs)
    assert abs(runs[0]["primal_obj"] - runs[1]["primal_obj"]) <= 1e-7 * (1 + abs(runs[1]["primal_obj"]))
    x = runs[0]["x"]
    assert np.linalg.norm(dense(full) @ x - full.b) <= 1e-7 * (1 + np.linalg.norm(full.b))


def test_bad_arguments_rejected():
    """Non-positive tol, or an LP with no rows or columns: -1, nothing allocated."""
    import ctypes as C

    from help_gb300 import native

    lib = native.lp_lib()
    lp = L.generate(L.spec_random(20, 60, 3), 1)
    out = native.LpStruct()
    st = lp.as_struct()
    for tol in (0.0, -1e-8, float("nan")):
        assert lib.help_lp_remove_dependent_rows(C.byref(st), tol, C.byref(out), None) == -1
    empty = native.LpStruct()
    assert lib.help_lp_remove_dependent_rows(C.byref(empty), 1e-8, C.byref(out), None) == -1
    assert lib.help_lp_remove_dependent_rows(None, 1e-8, C.byref(out), None) == -1
    with pytest.raises(ValueError, match="bad arguments"):
        L.remove_dependent_rows(lp, tol=0.0)


def test_config3_generated_full_then_presolved():
    """Config 3 as specified: every node row (479,200), one per commodity
    removed by the presolve, leaving 479,192 rows and every column."""
    lp = L.make_lp(3, 0)
    assert lp.m == 479192 and lp.n == 1432800 and lp.name == "config3-seed0"
    assert np.all(np.diff(lp.col_ptr) > 0)


def test_hsd_driver_presolve_switch():
    """help_hsd_options.presolve_lindep (the reference's PRESOLVE_LINDEP): the
    driver removes the dependent rows itself, reaches the grounded optimum,
    reports how many rows went, and returns y for all m rows (0 on the
    dropped ones) -- b^T y over the full rows equals the objective; with b
    moved along a dependency it reports primal infeasibility and runs no
    iteration."""
    from help_gb300 import hsd
    from oracle import bindings as ob

    def backend():
        return ob.OracleNormalEquations(pivots=10, tol=1e-14, max_iter=10**6).ne_backend()

    full = L.generate(L.spec_mcf(8, 3, 2, grounded=False), 4)
    grounded = L.generate(L.spec_mcf(8, 3, 2), 4)
    r = hsd.solve_lp(full, backend(), presolve_lindep=True, want_solution=True)
    g = hsd.solve_lp(grounded, backend())
    assert r["rc"] == 0 and r["status"] == 0 and r["lp_status"] == 0 and r["rows_removed"] == 3
    assert abs(r["primal_obj"] - g["primal_obj"]) <= 1e-7 * (1 + abs(g["primal_obj"]))
    assert len(r["y"]) == full.m and np.count_nonzero(r["y"] == 0.0) >= 3
    assert abs(full.b @ r["y"] - r["primal_obj"]) <= 1e-6 * (1 + abs(r["primal_obj"]))
    assert np.linalg.norm(dense(full) @ r["x"] - full.b) <= 1e-7 * (1 + np.linalg.norm(full.b))
    bad = L.generate(L.spec_mcf(8, 3, 2, grounded=False), 4)
    bad.b = bad.b.copy()
    bad.b[70] += 0.5
    r = hsd.solve_lp(bad, backend(), presolve_lindep=True)
    assert r["rc"] == 0 and r["lp_status"] == 1 and r["iterations"] == 0
    # on a full-rank LP the switch leaves the run as it is
    r0 = hsd.solve_lp(grounded, backend(), presolve_lindep=True)
    assert r0["rows_removed"] == 0 and r0["iterations"] == g["iterations"] and r0["primal_obj"] == g["primal_obj"]
