"""The no-allocation product y = A D^-1 A^T x (help_adat_matvec_noalloc).

It exists for callers that cannot allocate device memory: the caller hands
over every array as a device pointer and the intermediate vector lives in a
fixed device array inside the library.  This file is collected last so a
run that stops at the first failure has run every other test already; it
passes alone in a fresh process as well.

Checked to 1e-12 relative against the backend's allocating entry point
(HELP_OP_ADAT, which computes the same product as B B^T x with
B = A D^-1/2) and against the oracle's CSRMV_T / scale / CSRMV_N
(Helper.cpp:57-81), on two calls in a row with different inputs (the shared
scratch array keeps the previous call's contents); the second call takes no
device memory (free memory before and after it is the same).
"""
import ctypes as C

import numpy as np
import pytest

from help_gb300 import backend, lp as L, native
from oracle import bindings as ob

pytestmark = pytest.mark.gpu


def _skewed_csc(m, n, seed):
    """Sparse random columns plus three dense columns and two dense rows:
    rows and columns far longer than 32 lanes x 8 nonzeros, m != n."""
    rng = np.random.default_rng(seed)
    cols = []
    for j in range(n):
        if j in (5, n // 2, n - 1):
            rows = np.arange(m)
        else:
            rows = np.sort(rng.choice(m, size=int(rng.integers(1, 6)), replace=False))
            rows = np.union1d(rows, [0, m - 1]) if j % 3 == 0 else rows
        cols.append(rows)
    cp = np.zeros(n + 1, np.int32)
    cp[1:] = np.cumsum([len(c) for c in cols])
    ri = np.concatenate(cols).astype(np.int32)
    val = rng.standard_normal(ri.size)
    return cp, ri, val


def _csr(m, n, cp, ri, val):
    order = np.lexsort((np.repeat(np.arange(n), np.diff(cp)), ri))
    rp = np.zeros(m + 1, np.int32)
    np.add.at(rp, ri + 1, 1)
    rp = np.cumsum(rp).astype(np.int32)
    ci = np.repeat(np.arange(n, dtype=np.int32), np.diff(cp))[order]
    return rp, ci, val[order]


CASES = {
    "random-3000x9000": lambda: (lambda lp: (lp.m, lp.n, lp.col_ptr, lp.row_ind, lp.val))(
        L.generate(L.spec_random(3000, 9000, 5), 21)),
    "dense-rows-cols-1200x5000": lambda: (1200, 5000) + _skewed_csc(1200, 5000, 8),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_noalloc_product_matches_allocating_entry_point_twice(case):
    import torch

    m, n, cp, ri, val = CASES[case]()
    rp, ci, v = _csr(m, n, cp, ri, val)
    nnz = int(cp[-1])
    assert np.diff(rp).max() > 32 * 8 or case.startswith("random")
    rng = np.random.default_rng(4)
    d = np.exp(rng.uniform(np.log(1e-6), np.log(1e6), n))
    dev = torch.device("cuda", 0)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    rp_d, ci_d, v_d = T(rp), T(ci), T(v)
    cp_d, ri_d, vt_d = T(cp), T(ri), T(val)
    d_d = T(d)
    lib = native.gpu_lib()
    with backend.GpuNormalEquations(pivots=4) as g:
        g.LinearEquation_Construct(m=m, n=n, col_ptr=cp, row_ind=ri, val=val)
        g.RenewLinearEquation(d)
        for call in range(2):
            x = torch.randn(m, dtype=torch.float64, device=dev)
            y = torch.full((m,), float("nan"), dtype=torch.float64, device=dev)
            y_ref = torch.empty_like(y)
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info(0)[0]
            rc = lib.help_adat_matvec_noalloc(m, n, nnz, rp_d.data_ptr(), ci_d.data_ptr(), v_d.data_ptr(),
                                              cp_d.data_ptr(), ri_d.data_ptr(), vt_d.data_ptr(), d_d.data_ptr(),
                                              x.data_ptr(), y.data_ptr(), None)
            assert rc == native.HELP_OK
            torch.cuda.synchronize()
            free_after = torch.cuda.mem_get_info(0)[0]
            if call == 1:  # the first call may load the library's device code
                assert free_after == free_before
            g.matvec_dev("ADAT", x.data_ptr(), y_ref.data_ptr())
            torch.cuda.synchronize()
            err = float((y - y_ref).norm() / y_ref.norm())
            assert err < 1e-12, (call, err)
            xh = x.cpu().numpy()
            want = ob.csrmv_n(rp, ci, v, ob.csrmv_t(rp, ci, v, xh, m, n) / d, m, n)
            err_o = np.linalg.norm(y.cpu().numpy() - want) / np.linalg.norm(want)
            assert err_o < 1e-12, (call, err_o)


def test_noalloc_rejects_oversized_n():
    lib = native.gpu_lib()
    one = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.help_adat_matvec_noalloc(10, (1 << 20) + 1, 10, one, one, one, one, one, one, one, one, one, None)
    assert rc == native.HELP_E_ARG
