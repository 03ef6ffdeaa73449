"""Pin the CPU oracle to the reference.

1. Against the golden fixtures produced by the reference itself
   (tests/golden/make_golden.py runs the reference's own sources): the
   restatement must reproduce them bit for bit.
2. Against the known answers the reference's sources carry in comments:
   MKLTest (Main.cpp:19-35) and the 5 x 5 partial-Cholesky example of
   UnitTest (PCG.cpp:402-457).
3. Against the live reference harness when it was built on this machine.
"""
import json
import os

import numpy as np
import pytest

from help_gb300 import hsd, lp as L
from oracle import bindings as ob


def test_known_answer_csrmv():
    # [1 0 2; 0 3 0; 4 0 5] * [3 5 7]^T = [17 15 47]^T
    rp = np.array([0, 2, 3, 5], np.int32)
    ci = np.array([0, 2, 1, 0, 2], np.int32)
    v = np.array([1.0, 2.0, 3.0, 4.0, 5.0])
    assert np.array_equal(ob.csrmv_n(rp, ci, v, np.array([3.0, 5.0, 7.0]), 3, 3), [17.0, 15.0, 47.0])


def _unit_test_matrix():
    # PCG.cpp:406-411 with zero-based columns (the reference's arrays are one-based
    # by mistake, PCG.cpp:409): A = lower-triangular M, d = 1 / diag(4,1,5,3,2)^2,
    # so A D^-1 A^T = M diag(4,1,5,3,2)^2 M^T (PCG.cpp:416-418).
    rp = np.array([0, 1, 3, 6, 10, 15], np.int32)
    ci = np.array([0, 0, 1, 0, 1, 2, 0, 1, 2, 3, 0, 1, 2, 3, 4], np.int32)
    v = np.array([1, 2, 1, 3, 5, 1, 2, 4, 3, 1, 3, 3, 0, 2, 1], np.float64)
    d = np.array([0.25 * 0.25, 1, 0.2 * 0.2, 1.0 / 9.0, 0.25])
    return rp, ci, v, d


def test_known_answer_partial_cholesky():
    rp, ci, v, d = _unit_test_matrix()
    pc1 = ob.PartialCholesky(rp, ci, v, d, 5, 5, 1)
    # first pivot: row 4 (one-based), G = [4 2 3 1 5] in PCG.cpp:420
    assert pc1.perm[0] == 3
    L1 = pc1.L[:, 0]
    # L(:,1) = [1.0000, 0.2166, 0.6083, 0.1019, 0.4013] in the order G (PCG.cpp:424-432)
    np.testing.assert_allclose(L1[[3, 1, 2, 0, 4]], [1.0, 0.2166, 0.6083, 0.1019, 0.4013], atol=5e-5)
    # Schur diagonal after the first pivot: 50.2739, 77.8185, 12.7389, 142.4395 (PCG.cpp:436-442)
    np.testing.assert_allclose(pc1.diag_s[[1, 2, 0, 4]], [50.2739, 77.8185, 12.7389, 142.4395], atol=5e-5)
    # the greedy rule then takes row 5 (one-based): G = [4 5 3 1 2] (PCG.cpp:448)
    pc2 = ob.PartialCholesky(rp, ci, v, d, 5, 5, 2)
    assert list(pc2.perm[:2]) == [3, 4]


@pytest.fixture(scope="module")
def golden(golden_dir):
    return np.load(os.path.join(golden_dir, "ref_kernels.npz"))


@pytest.fixture(scope="module")
def glp(golden):
    m, n, k, seed = (int(x) for x in golden["gen"])
    return L.generate(L.spec_random(m, n, k), seed)


def test_oracle_csrmv_bitwise(golden, glp):
    rp, ci, v = glp.csr()
    yN = ob.csrmv_n(rp, ci, v, golden["x_n"], glp.m, glp.n, 1.5, -0.5, golden["y0"])
    yT = ob.csrmv_t(rp, ci, v, golden["x_t"], glp.m, glp.n)
    assert np.array_equal(yN, golden["yN"])
    assert np.array_equal(yT, golden["yT"])


def test_oracle_partial_cholesky_bitwise(golden, glp):
    rp, ci, v = glp.csr()
    pc = ob.PartialCholesky(rp, ci, v, golden["d"], glp.m, glp.n, int(golden["k"]))
    assert np.array_equal(pc.perm, golden["perm"])
    assert np.array_equal(pc.L, golden["L"])
    assert np.array_equal(pc.D, golden["D"])
    assert np.array_equal(pc.diag_s, golden["diag_s"])
    assert np.array_equal(pc.apply_permuted(golden["r_perm"]), golden["z_perm"])


def test_oracle_adat_bitwise(golden, glp):
    rp, ci, v = glp.csr()
    orp = np.zeros(glp.m + 1, np.int32)
    nnz = ob.lib().oracle_adat_symbolic(glp.m, glp.n, ob.P(rp), ob.P(ci), ob.P(glp.col_ptr), ob.P(glp.row_ind),
                                        ob.P(orp), None)
    col = np.zeros(nnz, np.int32)
    ob.lib().oracle_adat_symbolic(glp.m, glp.n, ob.P(rp), ob.P(ci), ob.P(glp.col_ptr), ob.P(glp.row_ind), ob.P(orp),
                                  ob.P(col))
    val = np.zeros(nnz)
    ob.lib().oracle_adat_numeric(glp.m, glp.n, ob.P(rp), ob.P(ci), ob.P(v), ob.P(glp.col_ptr), ob.P(glp.row_ind),
                                 ob.P(glp.val), ob.P(golden["w"]), ob.P(orp), ob.P(col), ob.P(val))
    assert np.array_equal(orp, golden["adat_rp"])
    assert np.array_equal(col, golden["adat_col"])
    assert np.array_equal(val, golden["adat_val"])


def test_oracle_solve_bitwise(golden, glp):
    ora = ob.OracleNormalEquations(pivots=10)
    ora.LinearEquation_Construct(glp)
    x1, x2 = ora.SolveLinearEquation(golden["d"], golden["b1"], golden["b2"])
    assert ora.last_iters() == int(golden["iters"])
    assert np.array_equal(x1, golden["x1"])
    assert np.array_equal(x2, golden["x2"])


def test_hsd_driver_with_oracle_reproduces_reference_program(golden_dir):
    """The native HSD driver + the oracle backend replays every solve the reference
    program made on a 50 x 150 LP, bit for bit (inputs, outputs, CG counts)."""
    rec = np.load(os.path.join(golden_dir, "ref_hsd_small.npz"))
    lp = L.generate(L.spec_random(50, 150, 5), 1)
    ora = ob.OracleNormalEquations(pivots=10)
    calls = []
    import ctypes as C
    from help_gb300 import native

    base = ora.ne_backend()
    solve_raw = native.SOLVE_FN(base.solve)

    def solve(ctx, d, b1, b2, x1, x2):
        rc = solve_raw(ctx, d, b1, b2, x1, x2)
        arr = lambda p, k: np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_double)), (k,)).copy()
        calls.append((arr(d, lp.n), arr(b1, lp.n), arr(b2, lp.m), arr(x1, lp.n), arr(x2, lp.m),
                      ora.last_iters()))
        return rc

    cb = native.SOLVE_FN(solve)
    be = native.NeBackend(ctx=base.ctx, construct=base.construct, renew=base.renew,
                          solve=C.cast(cb, C.c_void_p).value, destruct=base.destruct)
    res = hsd.solve_lp(lp, be)
    assert res["status"] == 0
    assert len(calls) == len(rec["iters"])
    for i, (d, b1, b2, x1, x2, it) in enumerate(calls):
        assert np.array_equal(d, rec["d"][i]), i
        assert np.array_equal(b1, rec["b1"][i]), i
        assert np.array_equal(b2, rec["b2"][i]), i
        assert np.array_equal(x1, rec["x1"][i]), i
        assert np.array_equal(x2, rec["x2"][i]), i
        assert it == rec["iters"][i], i


def test_hsd_tables_match_reference_program(golden_dir):
    """Iteration tables of the driver + oracle equal the reference program's
    (values as printed: 8 and 2 significant digits)."""
    tables = json.load(open(os.path.join(golden_dir, "ref_hsd.json")))
    for name in ("random-50x150-k5-seed1", "random-200x600-k5-seed2"):
        t = tables[name]
        lp = L.generate(L.spec_random(t["m"], t["n"], 5), t["seed"])
        ora = ob.OracleNormalEquations(pivots=10)
        rows = []
        hsd.solve_lp(lp, ora.ne_backend(), on_iter=lambda it, s: rows.append([it] + s[:5]))
        assert len(rows) == len(t["rows"])
        for got, want in zip(rows, t["rows"]):
            np.testing.assert_allclose(got[1:3], want[1:3], rtol=6e-8)
            np.testing.assert_allclose(got[3:6], want[3:6], rtol=6e-2)


def test_hsd_final_iterate_matches_reference_program_bitwise(golden_dir):
    """The driver + oracle end where the reference program ended: status,
    iteration and solve counts, total CG iterations, objectives, gap,
    infeasibilities, tau and kappa, all bit for bit (the reference's values
    read from its globals at HSD_Main's end, HSDSolver.cpp:881)."""
    tables = json.load(open(os.path.join(golden_dir, "ref_hsd.json")))
    for name in ("random-50x150-k5-seed1", "random-200x600-k5-seed2"):
        t = tables[name]
        ref = t["final"]
        lp = L.generate(L.spec_random(t["m"], t["n"], 5), t["seed"])
        ora = ob.OracleNormalEquations(pivots=10)
        be = ora.ne_backend()
        res = hsd.solve_lp(lp, be)
        assert res["status"] == ref["status"] and res["iterations"] == ref["iterations"]
        assert res["solves"] == ref["solves"]
        for key in ("primal_obj", "dual_obj", "rel_gap", "primal_infeas", "dual_infeas", "tau", "kappa"):
            assert res[key] == ref[key], (name, key, res[key], ref[key])


@pytest.mark.skipif(not ob.ref_available(), reason="reference harness not built on this machine")
def test_live_reference_random_instances():
    R = ob.ref()
    for seed in range(3):
        lp = L.generate(L.spec_random(60, 200, 4), 100 + seed)
        R.ref_load(lp.m, lp.n, ob.P(lp.col_ptr), ob.P(lp.row_ind), ob.P(lp.val))
        R.ref_construct()
        rng = np.random.default_rng(seed)
        d = np.exp(rng.uniform(-5, 5, lp.n))
        b1, b2 = rng.standard_normal(lp.n), rng.standard_normal(lp.m)
        x1, x2 = np.zeros(lp.n), np.zeros(lp.m)
        it = R.ref_solve(ob.P(d), ob.P(b1), ob.P(b2), ob.P(x1), ob.P(x2))
        ora = ob.OracleNormalEquations(pivots=10)
        ora.LinearEquation_Construct(lp)
        ox1, ox2 = ora.SolveLinearEquation(d, b1, b2)
        assert ora.last_iters() == it
        assert np.array_equal(ox1, x1) and np.array_equal(ox2, x2)


def test_threaded_adat_calc_equals_serial():
    """The threaded ADAt_Calc port (the reference's OpenMP row loop) gives the
    serial restatement's values bit for bit, rows being independent."""
    lp = L.generate(L.spec_zipf(3000, 12000, 6, 1.3, 70), 4)
    rp, ci, v = lp.csr()
    w = np.exp(np.random.default_rng(2).uniform(-2, 2, lp.n))
    outs = []
    for threads in (1, 4):
        orp = np.zeros(lp.m + 1, np.int32)
        nnz = ob.lib().oracle_adat_symbolic(lp.m, lp.n, ob.P(rp), ob.P(ci), ob.P(lp.col_ptr), ob.P(lp.row_ind),
                                            ob.P(orp), None)
        ocol = np.zeros(nnz, np.int32)
        ob.lib().oracle_adat_symbolic(lp.m, lp.n, ob.P(rp), ob.P(ci), ob.P(lp.col_ptr), ob.P(lp.row_ind), ob.P(orp),
                                      ob.P(ocol))
        oval = np.zeros(nnz)
        used = ob.lib().oracle_adat_numeric_threads(lp.m, lp.n, ob.P(rp), ob.P(ci), ob.P(v), ob.P(lp.col_ptr),
                                                    ob.P(lp.row_ind), ob.P(lp.val), ob.P(w), ob.P(orp), ob.P(ocol),
                                                    ob.P(oval), threads)
        assert used == threads
        outs.append(oval)
    assert np.array_equal(outs[0], outs[1])
