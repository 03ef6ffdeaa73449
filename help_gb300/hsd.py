"""The HSD interior-point driver (native, help_lp.h) over any normal-equations backend."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native


def solve_lp(lp, backend: native.NeBackend, *, verbose: bool = False, max_iterations: int = 10000,
             gap_tol: float = 1e-8, on_iter=None, want_solution: bool = False,
             presolve_lindep: bool = False, max_seconds: float = 0.0) -> dict:
    """Run HSD_Main (HSDSolver.cpp:869-883) on ``lp`` with ``backend``'s four entry points.

    Returns a dict with status, iterations, objective values, gap, infeasibilities,
    total and backend wall time, lp_status / rows_removed of the dependent-row
    presolve (``presolve_lindep``: the reference's PRESOLVE_LINDEP switch,
    LP.h:72), and x, y when ``want_solution``.
    """
    lib = native.lp_lib()
    opt = native.HsdOptions()
    lib.help_hsd_default_options(C.byref(opt))
    opt.max_iterations = max_iterations
    opt.gap_tol = gap_tol
    opt.verbose = int(verbose)
    opt.presolve_lindep = int(presolve_lindep)
    opt.max_seconds = float(max_seconds)
    cb = None
    if on_iter is not None:
        def _cb(user, it, s6):
            on_iter(int(it), [s6[i] for i in range(6)])
        cb = native.ONITER_FN(_cb)
        opt.on_iter = C.cast(cb, C.c_void_p).value
    res = native.HsdResult()
    s = lp.as_struct()
    x = np.empty(lp.n) if want_solution else None
    y = np.empty(lp.m) if want_solution else None
    rc = lib.help_hsd_solve(C.byref(s), C.byref(backend), C.byref(opt), C.byref(res),
                            native.ptr(x) if x is not None else None, native.ptr(y) if y is not None else None)
    out = {f: getattr(res, f) for f, _ in native.HsdResult._fields_}
    out["rc"] = rc
    if want_solution:
        out["x"], out["y"] = x, y
    return out
