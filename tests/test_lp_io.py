"""LP input: the MPS reader (help_lp_read_mps, the reference's MPSRead.cpp and
row standardisation restated for E/L/G rows and x >= 0) and the binary fast
path (help_lp_write_bin / help_lp_read_bin).  Exact comparisons: values on
the generators' 1e-6 grid parse back bit-identical."""
import os

import numpy as np
import pytest

from help_gb300 import lp as L


def same(a, b):
    assert (a.m, a.n, a.n_struct) == (b.m, b.n, b.n_struct)
    for f in ("col_ptr", "row_ind", "val", "b", "c"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    assert a.row_type == b.row_type


@pytest.mark.parametrize("spec,seed", [(L.spec_random(60, 200, 4), 1), (L.spec_mcf(5, 2, 2), 2),
                                       (L.spec_zipf(80, 300, 3, 1.3, 10), 3)])
def test_mps_round_trip(tmp_path, spec, seed):
    lp = L.generate(spec, seed)
    p = str(tmp_path / "a.mps")
    lp.write_mps(p)
    same(L.read_mps(p), lp)


@pytest.mark.parametrize("spec,seed", [(L.spec_random(60, 200, 4), 1), (L.spec_mcf(5, 2, 2), 2)])
def test_binary_round_trip(tmp_path, spec, seed):
    lp = L.generate(spec, seed)
    p = str(tmp_path / "a.bin")
    lp.write_bin(p)
    same(L.read_bin(p), lp)


FREE = """* free-layout MPS with every supported feature
NAME small
ROWS
 N  obj
 E  r1
 L  r2
 G  r3
 N  freerow
COLUMNS
 x1 obj 1.5 r1 2.0
 x1 r3 -1.0 nosuchrow 7.0
 x2 r2 3.0 obj -2.0
 x2 r1 1e-12
 x1 r2 4.0
 x3 r3 0.5
RHS
 rhs r1 4.0 r2 10.0
 r3 1.0
BOUNDS
 PL bnd x1
 LO bnd x2 0
ENDATA
"""


def test_free_layout_rows_slacks_and_dropped_entries(tmp_path):
    p = tmp_path / "f.mps"
    p.write_text(FREE)
    lp = L.read_mps(str(p))
    assert (lp.m, lp.n_struct, lp.n) == (3, 3, 5)  # slacks for the L and G rows
    assert lp.row_type == b"ELG"
    assert np.array_equal(lp.c, [1.5, -2.0, 0.0, 0.0, 0.0])
    assert np.array_equal(lp.b, [4.0, 10.0, 1.0])
    dense = np.zeros((lp.m, lp.n))
    for j in range(lp.n):
        dense[lp.row_ind[lp.col_ptr[j]:lp.col_ptr[j + 1]], j] = lp.val[lp.col_ptr[j]:lp.col_ptr[j + 1]]
    want = np.array([[2.0, 0.0, 0.0, 0.0, 0.0],     # x2's 1e-12 in r1 dropped
                     [4.0, 3.0, 0.0, 1.0, 0.0],     # slack +1 for L
                     [-1.0, 0.0, 0.5, 0.0, -1.0]])  # slack -1 for G; unknown row dropped
    assert np.array_equal(dense, want)


@pytest.mark.parametrize("text,why", [
    (FREE.replace("BOUNDS\n PL bnd x1", "RANGES\n rng r2 1.0\nBOUNDS\n PL bnd x1"), "RANGES"),
    (FREE.replace(" PL bnd x1", " UP bnd x1 4.0"), "BOUNDS"),
    (FREE.replace(" x3 r3 0.5", " m 'MARKER' 'INTORG'\n x3 r3 0.5"), "marker"),
    (FREE.replace(" x3 r3 0.5", " x3 r3 0.5 r3 1.0"), "repeated"),
    (FREE.replace("ENDATA\n", ""), "ENDATA"),
    (FREE.replace(" N  obj\n", "").replace(" N  freerow\n", ""), "objective"),
    (FREE.replace("4.0 r2 10.0", "4.0 r2 1O.0"), "bad value"),
    (FREE.replace(" E  r1", " X  r1"), "row type"),
    ("OBJSENSE\n    MAX\n" + FREE, "OBJSENSE"),
    (FREE.replace("COLUMNS\n", "COLUMNS\n x9 r1\n"), "COLUMNS"),
])
def test_mps_errors(tmp_path, text, why):
    p = tmp_path / "bad.mps"
    p.write_text(text)
    with pytest.raises(ValueError, match=why):
        L.read_mps(str(p))


def test_binary_errors(tmp_path):
    lp = L.generate(L.spec_random(30, 90, 3), 5)
    p = str(tmp_path / "a.bin")
    lp.write_bin(p)
    raw = open(p, "rb").read()
    (tmp_path / "trunc.bin").write_bytes(raw[:-7])
    with pytest.raises(ValueError, match="truncated"):
        L.read_bin(str(tmp_path / "trunc.bin"))
    (tmp_path / "magic.bin").write_bytes(b"NOTALP01" + raw[8:])
    with pytest.raises(ValueError, match="HELPLP01"):
        L.read_bin(str(tmp_path / "magic.bin"))
    bad = bytearray(raw)
    bad[64 + 4 * 5:64 + 4 * 6] = (10**6).to_bytes(4, "little")  # col_ptr[5] out of order
    (tmp_path / "ptr.bin").write_bytes(bytes(bad))
    with pytest.raises(ValueError, match="inconsistent"):
        L.read_bin(str(tmp_path / "ptr.bin"))
    with pytest.raises(ValueError, match="cannot open"):
        L.read_mps(os.path.join(str(tmp_path), "missing.mps"))


def test_hsd_on_an_mps_read_instance_matches_the_generated_one(tmp_path):
    from help_gb300 import hsd
    from oracle import bindings as ob
    lp = L.generate(L.spec_mcf(5, 2, 2), 7)
    p = str(tmp_path / "a.mps")
    lp.write_mps(p)
    back = L.read_mps(p)
    r1 = hsd.solve_lp(lp, ob.OracleNormalEquations(pivots=4, tol=1e-14, max_iter=10**6).ne_backend())
    r2 = hsd.solve_lp(back, ob.OracleNormalEquations(pivots=4, tol=1e-14, max_iter=10**6).ne_backend())
    assert r1["status"] == r2["status"] == 0
    assert r1["primal_obj"] == r2["primal_obj"] and r1["iterations"] == r2["iterations"]


def test_rhs_on_the_objective_row_is_ignored(tmp_path):
    """An RHS entry on the objective row (a constant offset) does not enter b."""
    p = tmp_path / "o.mps"
    p.write_text(FREE.replace(" r3 1.0\n", " r3 1.0\n rhs obj 5.0\n"))
    lp = L.read_mps(str(p))
    assert np.array_equal(lp.b, [4.0, 10.0, 1.0])
