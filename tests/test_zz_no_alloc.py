"""The no-allocation product y = A D^-1 A^T x (help_adat_matvec_noalloc).

It exists for callers that cannot allocate device memory: the caller hands
over every array as a device pointer and the intermediate vector lives in a
fixed device array inside the library.  This file is collected last so a
run that stops at the first failure has run every other test already; it
passes alone in a fresh process as well.

Checked against the backend's allocating entry point (HELP_OP_ADAT, which
computes the same product as B B^T x with B = A D^-1/2) to 1e-12 relative,
on two calls in a row with different inputs (the shared scratch array keeps
the previous call's contents).
"""
import ctypes as C

import numpy as np
import pytest

from help_gb300 import backend, lp as L, native

pytestmark = pytest.mark.gpu


def test_noalloc_product_matches_allocating_entry_point_twice():
    import torch

    lp = L.generate(L.spec_random(3000, 9000, 5), 21)
    rng = np.random.default_rng(4)
    d = np.exp(rng.uniform(np.log(1e-6), np.log(1e6), lp.n))
    rp, ci, v = lp.csr()
    dev = torch.device("cuda", 0)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    rp_d, ci_d, v_d = T(rp), T(ci), T(v)
    cp_d, ri_d, vt_d = T(lp.col_ptr), T(lp.row_ind), T(lp.val)
    d_d = T(d)
    lib = native.gpu_lib()
    with backend.GpuNormalEquations(pivots=4) as g:
        g.LinearEquation_Construct(lp)
        g.RenewLinearEquation(d)
        for call in range(2):
            x = torch.randn(lp.m, dtype=torch.float64, device=dev)
            y = torch.full((lp.m,), float("nan"), dtype=torch.float64, device=dev)
            y_ref = torch.empty_like(y)
            rc = lib.help_adat_matvec_noalloc(lp.m, lp.n, lp.nnz, rp_d.data_ptr(), ci_d.data_ptr(), v_d.data_ptr(),
                                              cp_d.data_ptr(), ri_d.data_ptr(), vt_d.data_ptr(), d_d.data_ptr(),
                                              x.data_ptr(), y.data_ptr(), None)
            assert rc == native.HELP_OK
            g.matvec_dev("ADAT", x.data_ptr(), y_ref.data_ptr())
            torch.cuda.synchronize()
            err = float((y - y_ref).norm() / y_ref.norm())
            assert err < 1e-12, (call, err)


def test_noalloc_rejects_oversized_n():
    lib = native.gpu_lib()
    one = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.help_adat_matvec_noalloc(10, (1 << 20) + 1, 10, one, one, one, one, one, one, one, one, one, None)
    assert rc == native.HELP_E_ARG
