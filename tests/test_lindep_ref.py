"""The dependent-row presolve against the reference's own
(Presolve_Lindep.cpp with its vendored LUSOL, run by oracle/ref/ref_lindep.cpp
after the reference's MPS reader, crushing and presolve set-up) on the same
MPS files: the same number of dependent rows and the same feasibility
verdict.  Which row of a dependent set goes is each method's own choice (the
reference: the artificial basis columns it cannot replace), so the counts and
the verdicts are compared, and both reduced row sets have full rank.

The reference's factor space is fixed (LUSOL_MULT_nz_a x nnz); on
near-square random matrices (m x 1.1 m, 4-5 nonzeros per column) it runs out
and the reference program stops with LUSOL_ANEEDMEM -- those instances are
checked against numpy's rank instead (tests/test_lindep.py)."""
import os
import tempfile

import numpy as np
import pytest

from help_gb300 import lp as L
from oracle import bindings as ob

pytestmark = pytest.mark.skipif(not ob.ref_lindep_available(),
                                reason="reference presolve not built on this machine")


def reference(lp):
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "lp.mps")
        lp.write_mps(path)
        return ob.ref_lindep(path)


@pytest.mark.parametrize("name,spec,seed,want", [
    ("flow 4x4, 2 commodities, every node row", L.spec_mcf(4, 2, 2, grounded=False), 7, 2),
    ("flow 8x8, 3 commodities, every node row", L.spec_mcf(8, 3, 2, grounded=False), 4, 3),
    ("flow 24x24, 4 commodities, every node row", L.spec_mcf(24, 4, 3, grounded=False), 11, 4),
    ("flow 24x24, 4 commodities, grounded", L.spec_mcf(24, 4, 3), 11, 0),
    ("random 2,000 x 6,000 (config 0)", L.spec_random(2000, 6000, 5), 0, 0),
])
def test_same_dependent_row_count_as_reference(name, spec, seed, want):
    lp = L.generate(spec, seed)
    ref = reference(lp)
    assert "error" not in ref, ref
    assert ref["status"] == 0 and ref["rows"] == lp.m
    red, removed = L.remove_dependent_rows(lp)
    assert int(removed.sum()) == ref["dependent"] == want
    # the reference's kept rows carry the same flow structure: one node row of
    # each commodity dropped
    if want:
        N = spec.grid * spec.grid
        dis = np.array(ref["disabled"])
        assert sorted(set(dis // N)) == list(range(spec.commodities))


def test_same_infeasibility_verdict_as_reference():
    """A supply moved by 0.5 in one node row: each commodity's rows no longer
    sum to its balance, and both presolves call the LP primal infeasible."""
    lp = L.generate(L.spec_mcf(8, 3, 2, grounded=False), 4)
    lp.b = lp.b.copy()
    lp.b[70] += 0.5
    ref = reference(lp)
    assert "error" not in ref, ref
    assert ref["status"] == 1
    with pytest.raises(ValueError, match="infeasible"):
        L.remove_dependent_rows(lp)
