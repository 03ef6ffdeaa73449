"""Seeded LP instances for the benchmark configurations (native generator).

``make_lp(config, seed)`` returns an :class:`LP` holding CSC arrays (numpy,
owned by Python).  The five configurations are the benchmark's:

* ``0`` random sparse LP, m=2,000, n=6,000, 5 nonzeros per column;
* ``1`` same generator, m=100,000, n=400,000, 8 per column (k=512 pivots);
* ``2`` Zipf(1.3) row law, m=500,000, n=2,000,000, 6 per column (k=1,024);
* ``3`` multicommodity flow, 200x200 grid, 8 commodities: every node row
  (479,200 rows, each commodity's rows summing to zero), then the
  dependent-row presolve removes one row per commodity (479,192 rows);
* ``4`` block-angular: 32 blocks of 60,000 x 250,000 (5 per column) plus
  4,000 linking rows with P(column in row) = 0.002 (k=2,048).

All instances are feasible and bounded by construction (x0 ~ U(0.5, 2),
b = A x0, y0 ~ N(0, 1), s0 ~ U(0.5, 2), c = A^T y0 + s0), values on a 1e-6 grid.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import native


@dataclass
class LP:
    m: int
    n: int
    n_struct: int
    col_ptr: np.ndarray  # int32[n+1]
    row_ind: np.ndarray  # int32[nnz]
    val: np.ndarray      # float64[nnz]
    b: np.ndarray        # float64[m]
    c: np.ndarray        # float64[n]
    row_type: bytes
    name: str = ""

    @property
    def nnz(self) -> int:
        return int(self.col_ptr[-1])

    def csr(self):
        """(row_ptr, col_ind, val) of the same matrix."""
        m, n = self.m, self.n
        rp = np.zeros(m + 1, np.int32)
        ci = np.zeros(self.nnz, np.int32)
        v = np.zeros(self.nnz, np.float64)
        native.lp_lib().help_csc_to_csr(m, n, native.ptr(self.col_ptr), native.ptr(self.row_ind),
                                        native.ptr(self.val), native.ptr(rp), native.ptr(ci), native.ptr(v))
        return rp, ci, v

    def as_struct(self) -> native.LpStruct:
        s = native.LpStruct()
        s.m, s.n, s.n_struct, s.nnz = self.m, self.n, self.n_struct, self.nnz
        s.col_ptr = self.col_ptr.ctypes.data_as(C.POINTER(C.c_int32))
        s.row_ind = self.row_ind.ctypes.data_as(C.POINTER(C.c_int32))
        s.val = self.val.ctypes.data_as(C.POINTER(C.c_double))
        s.b = self.b.ctypes.data_as(C.POINTER(C.c_double))
        s.c = self.c.ctypes.data_as(C.POINTER(C.c_double))
        self._rt = C.create_string_buffer(self.row_type, len(self.row_type))
        s.row_type = C.cast(self._rt, C.POINTER(C.c_char))
        return s

    def write_mps(self, path: str) -> None:
        rc = native.lp_lib().help_lp_write_mps(C.byref(self.as_struct()), path.encode())
        if rc != 0:
            raise RuntimeError("help_lp_write_mps failed (%d)" % rc)

    def write_bin(self, path: str) -> None:
        """Binary fast path (help_lp_write_bin): the CSC arrays, b, c, row types."""
        lib = native.lp_lib()
        rc = lib.help_lp_write_bin(C.byref(self.as_struct()), path.encode())
        if rc != 0:
            raise OSError("help_lp_write_bin failed (%d): %s" % (rc, lib.help_lp_last_error().decode()))


def spec_random(m: int, n: int, k: int) -> native.LpSpec:
    return native.LpSpec(kind=native.HELP_LP_RANDOM, m=m, n=n, nnz_per_col=k)


def spec_zipf(m: int, n: int, k: int, s: float = 1.3, offset: int = 70) -> native.LpSpec:
    return native.LpSpec(kind=native.HELP_LP_ZIPF, m=m, n=n, nnz_per_col=k, zipf_s=s, zipf_offset=offset)


def spec_mcf(grid: int, commodities: int, pairs: int = 4, grounded: bool = True) -> native.LpSpec:
    return native.LpSpec(kind=native.HELP_LP_MCF, grid=grid, commodities=commodities,
                         pairs_per_commodity=pairs, mcf_ungrounded=0 if grounded else 1)


def spec_block(blocks: int, block_rows: int, block_cols: int, k: int, link_rows: int,
               link_prob: float) -> native.LpSpec:
    return native.LpSpec(kind=native.HELP_LP_BLOCK, blocks=blocks, block_rows=block_rows,
                         block_cols=block_cols, nnz_per_col=k, link_rows=link_rows, link_prob=link_prob)


# Benchmark configurations: (spec, partial-Cholesky pivot count k)
CONFIGS = {
    0: (lambda: spec_random(2000, 6000, 5), 10),
    1: (lambda: spec_random(100_000, 400_000, 8), 512),
    2: (lambda: spec_zipf(500_000, 2_000_000, 6), 1024),
    3: (lambda: spec_mcf(200, 8, grounded=False), 512),
    4: (lambda: spec_block(32, 60_000, 250_000, 5, 4000, 0.002), 2048),
}


def _from_struct(lib, s, name: str) -> LP:
    try:
        n, nnz, m = s.n, s.nnz, s.m
        lp = LP(
            m=m, n=n, n_struct=s.n_struct,
            col_ptr=np.ctypeslib.as_array(s.col_ptr, (n + 1,)).copy(),
            row_ind=np.ctypeslib.as_array(s.row_ind, (max(nnz, 1),))[:nnz].copy(),
            val=np.ctypeslib.as_array(s.val, (max(nnz, 1),))[:nnz].copy(),
            b=np.ctypeslib.as_array(s.b, (m,)).copy(),
            c=np.ctypeslib.as_array(s.c, (n,)).copy(),
            row_type=C.string_at(s.row_type, m),
            name=name,
        )
    finally:
        lib.help_lp_free(C.byref(s))
    return lp


def generate(spec: native.LpSpec, seed: int = 0, name: str = "") -> LP:
    lib = native.lp_lib()
    s = native.LpStruct()
    rc = lib.help_lp_generate(C.byref(spec), C.c_uint64(seed), C.byref(s))
    if rc != 0:
        raise ValueError("help_lp_generate failed (%d)" % rc)
    return _from_struct(lib, s, name)


def read_mps(path: str) -> LP:
    """An MPS file in the standard form the HSD driver takes (help_lp_read_mps:
    E/L/G rows, slacks appended for L/G rows, x >= 0 only)."""
    lib = native.lp_lib()
    s = native.LpStruct()
    rc = lib.help_lp_read_mps(path.encode(), C.byref(s))
    if rc != 0:
        raise ValueError("help_lp_read_mps failed (%d): %s" % (rc, lib.help_lp_last_error().decode()))
    return _from_struct(lib, s, path)


class PresolveNotApplicable(ValueError):
    """The dependent-row presolve gave up: its elimination fills in past its
    limits (random sparse matrices at 10^5 rows); solve the LP as it is."""


def remove_dependent_rows(lp: LP, tol: float = 1e-8):
    """(reduced LP, mask of the removed rows): the rows that are linear
    combinations of the other rows dropped (help_lp_remove_dependent_rows;
    the purpose of the reference's Presolve_Lindep.cpp:316).  Raises
    ValueError when b disagrees with a dependency (primal infeasible) and
    PresolveNotApplicable when the elimination passes its fill or work limit."""
    lib = native.lp_lib()
    s = native.LpStruct()
    removed = np.zeros(lp.m, np.int32)
    st = lp.as_struct()
    rc = lib.help_lp_remove_dependent_rows(C.byref(st), tol, C.byref(s), native.ptr(removed))
    if rc == -4:
        raise PresolveNotApplicable("help_lp_remove_dependent_rows (-4): the elimination passed its fill or "
                                    "work limit; no rows removed")
    if rc < 0:
        why = {-3: "primal infeasible: b disagrees with a dependent row", -2: "out of memory"}.get(rc, "bad arguments")
        raise ValueError("help_lp_remove_dependent_rows failed (%d): %s" % (rc, why))
    return _from_struct(lib, s, lp.name), removed.astype(bool)


def expand_duals(y_reduced: np.ndarray, removed: np.ndarray) -> np.ndarray:
    """Duals of the original LP from those of the reduced one: a dropped row is
    a combination of kept rows, so y = 0 there keeps A^T y and b^T y."""
    y = np.zeros(len(removed))
    y[~np.asarray(removed, bool)] = y_reduced
    return y


def read_bin(path: str) -> LP:
    """An instance written by LP.write_bin / help_lp_write_bin."""
    lib = native.lp_lib()
    s = native.LpStruct()
    rc = lib.help_lp_read_bin(path.encode(), C.byref(s))
    if rc != 0:
        raise ValueError("help_lp_read_bin failed (%d): %s" % (rc, lib.help_lp_last_error().decode()))
    return _from_struct(lib, s, path)


# Configurations generated rank-deficient and passed through the dependent-row
# presolve, as HELP does with PRESOLVE_LINDEP set (Presolve.cpp:1254-1260)
PRESOLVED = {3}


def make_lp(config: int, seed: int = 0) -> LP:
    spec_fn, _ = CONFIGS[config]
    name = "config%d-seed%d" % (config, seed)
    lp = generate(spec_fn(), seed, name=name)
    if config in PRESOLVED:
        lp, _ = remove_dependent_rows(lp)
        lp.name = name
    return lp


def config_pivots(config: int) -> int:
    return CONFIGS[config][1]
