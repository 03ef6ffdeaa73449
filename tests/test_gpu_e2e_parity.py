"""End to end on the GPU against the reference program itself.

The HSD driver (the reference's HSD_Main, HSDSolver.cpp:869-883, restated in
hsd.cpp) runs on the GPU backend with the reference's own settings (10
pivots, CG to ||r|| < 1e-20 ||r0||, PCG.h:19-20, PCG.cpp:333-340) on the LPs
whose reference-program runs are recorded in tests/golden/ref_hsd.json: the
final iterate the reference program reached (read from its globals when
HSD_Main destructs the backend, HSDSolver.cpp:881, printed at %.17g;
tests/golden/make_golden.py) is the target.

Tolerances (the GPU's CG sums in a different order, so its iterates differ
from the reference's in rounding):
  * same status (solved) and the same number of interior-point iterations;
  * primal and dual objective within 1e-8 relative of the reference's;
  * relative gap and primal / dual infeasibility within the reference's
    stopping tolerances (1e-8, LP.h:88-91) and within 1e-8 of the
    reference's values.
"""
import json
import os

import numpy as np
import pytest

from help_gb300 import backend, hsd, lp as L

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
TABLES = json.load(open(os.path.join(HERE, "golden", "ref_hsd.json")))


def _lp(name):
    t = TABLES[name]
    if name.startswith("config0"):
        return L.generate(L.CONFIGS[0][0](), t["seed"])
    return L.generate(L.spec_random(t["m"], t["n"], 5), t["seed"])


@pytest.mark.parametrize("name", sorted(TABLES))
def test_gpu_ipm_reaches_the_reference_programs_final_iterate(name):
    t = TABLES[name]
    ref = t["final"]
    lp = _lp(name)
    assert (lp.m, lp.n) == (t["m"], t["n"])
    with backend.GpuNormalEquations(pivots=10, cg_tol=1e-20) as g:
        r = hsd.solve_lp(lp, g.ne_backend())
    assert r["status"] == ref["status"] == 0
    assert r["iterations"] == ref["iterations"]
    for key in ("primal_obj", "dual_obj"):
        assert abs(r[key] - ref[key]) <= 1e-8 * abs(ref[key]), (key, r[key], ref[key])
    for key in ("rel_gap", "primal_infeas", "dual_infeas"):
        assert r[key] <= 1e-8 and abs(r[key] - ref[key]) <= 1e-8, (key, r[key], ref[key])
    # the objectives agree far inside the bar: print what was reached
    print("%s: iterations %d, primal obj %.17g (reference %.17g, rel diff %.2e)" % (
        name, r["iterations"], r["primal_obj"], ref["primal_obj"],
        abs(r["primal_obj"] - ref["primal_obj"]) / abs(ref["primal_obj"])))
