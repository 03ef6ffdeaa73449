"""ctypes bindings of the two native libraries (include/help_gpu.h, include/help_lp.h).

The GPU library is the product path: there is no fallback.  If
``libhelp_gpu.so`` is missing or cannot load (no CUDA runtime), loading
raises ``NativeLibraryError`` instead of silently computing elsewhere.
"""
from __future__ import annotations

import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(_PKG, "_lib")

# ---- learned part (help_gpu.h HELP_MLP_*)
MLP_IN, MLP_HIDDEN, MLP_OUT = 16, 64, 2
MLP_OFF_W1, MLP_OFF_B1, MLP_OFF_W2, MLP_OFF_B2, MLP_OFF_W3, MLP_OFF_B3 = 0, 1024, 1088, 5184, 5248, 5376
MLP_OFF_MEAN, MLP_OFF_SCALE, MLP_PARAMS = 5378, 5394, 5410

# ---- error codes (help_gpu.h)
HELP_OK = 0
HELP_E_ARG = -1
HELP_E_CUDA = -2
HELP_E_NOMEM = -3
HELP_E_NUMERIC = -4
HELP_E_TIMEOUT = -5
HELP_E_NOT_CONVERGED = -6
HELP_PREC_FP64 = 0
HELP_PREC_MIXED = 1
HELP_OP_A = 0
HELP_OP_AT = 1
HELP_OP_ADAT = 2
HELP_OP_B = 3
HELP_OP_BT = 4

# ---- instance families (help_lp.h)
HELP_LP_RANDOM = 0
HELP_LP_ZIPF = 1
HELP_LP_MCF = 2
HELP_LP_BLOCK = 3


class NativeLibraryError(RuntimeError):
    pass


class PcgOptions(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("pivots", C.c_int32),
        ("precision", C.c_int32),
        ("cg_tol", C.c_double),
        ("cg_max_iter", C.c_int64),
        ("delta", C.c_double),
        ("ir_tol", C.c_double),
        ("ir_max_outer", C.c_int32),
        ("inner_tol", C.c_double),
        ("inner_max_iter", C.c_int64),
        ("warm_start", C.c_int32),
        ("fallback", C.c_int32),
        ("cg_path", C.c_int32),
        ("cap_ok", C.c_int32),
        ("mixed_max_d_spread", C.c_double),
    ]


class PcgStats(C.Structure):
    _fields_ = [
        ("cg_iterations", C.c_int64),
        ("cg_iterations_total", C.c_int64),
        ("ir_outer", C.c_int32),
        ("fell_back", C.c_int32),
        ("converged", C.c_int32),
        ("pivots", C.c_int32),
        ("rel_residual", C.c_double),
        ("renew_ms", C.c_double),
        ("solve_ms", C.c_double),
        ("nnz_c", C.c_int64),
        ("solves", C.c_int32),
        ("renews", C.c_int32),
        ("cg_kernel_ms", C.c_double),
        ("cg_kernel_ms_total", C.c_double),
        ("cg_iterations_fp32", C.c_int64),
        ("cg_launches", C.c_int32),
        ("dense_regularised", C.c_int32),
        ("cg_path_used", C.c_int32),
        ("cluster_ctas", C.c_int32),
        ("learned_warm", C.c_int32),
        ("learned_fallbacks", C.c_int32),
        ("fp32_chosen", C.c_int32),
        ("d_spread", C.c_double),
    ]


class LpSpec(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("m", C.c_int32),
        ("n", C.c_int32),
        ("nnz_per_col", C.c_int32),
        ("zipf_s", C.c_double),
        ("zipf_offset", C.c_int32),
        ("grid", C.c_int32),
        ("commodities", C.c_int32),
        ("pairs_per_commodity", C.c_int32),
        ("blocks", C.c_int32),
        ("block_rows", C.c_int32),
        ("block_cols", C.c_int32),
        ("link_rows", C.c_int32),
        ("link_prob", C.c_double),
        ("mcf_ungrounded", C.c_int32),
    ]


class LpStruct(C.Structure):
    _fields_ = [
        ("m", C.c_int32),
        ("n", C.c_int32),
        ("n_struct", C.c_int32),
        ("nnz", C.c_int64),
        ("col_ptr", C.POINTER(C.c_int32)),
        ("row_ind", C.POINTER(C.c_int32)),
        ("val", C.POINTER(C.c_double)),
        ("b", C.POINTER(C.c_double)),
        ("c", C.POINTER(C.c_double)),
        ("row_type", C.POINTER(C.c_char)),
    ]


CONSTRUCT_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p)
RENEW_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p)
SOLVE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p)
DESTRUCT_FN = C.CFUNCTYPE(C.c_int, C.c_void_p)
MATVEC_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p)
SOLVE2_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, *([C.c_void_p] * 8))
ONITER_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int32, C.POINTER(C.c_double))


class NeBackend(C.Structure):
    _fields_ = [
        ("ctx", C.c_void_p),
        ("construct", C.c_void_p),
        ("renew", C.c_void_p),
        ("solve", C.c_void_p),
        ("destruct", C.c_void_p),
        ("matvec", C.c_void_p),  # optional: dest += sign * A v / A^T v (NULL: the driver's host loops)
        ("solve2", C.c_void_p),  # optional: two solves at once (NULL: one after the other)
    ]


class HsdOptions(C.Structure):
    _fields_ = [
        ("max_iterations", C.c_int32),
        ("gap_tol", C.c_double),
        ("pinf_tol", C.c_double),
        ("dinf_tol", C.c_double),
        ("verbose", C.c_int32),
        ("on_iter", C.c_void_p),
        ("user", C.c_void_p),
        ("presolve_lindep", C.c_int32),
        ("max_seconds", C.c_double),
    ]


class HsdResult(C.Structure):
    _fields_ = [
        ("status", C.c_int32),
        ("iterations", C.c_int32),
        ("solves", C.c_int32),
        ("renews", C.c_int32),
        ("primal_obj", C.c_double),
        ("dual_obj", C.c_double),
        ("rel_gap", C.c_double),
        ("primal_infeas", C.c_double),
        ("dual_infeas", C.c_double),
        ("tau", C.c_double),
        ("kappa", C.c_double),
        ("wall_s", C.c_double),
        ("backend_s", C.c_double),
        ("lp_status", C.c_int32),
        ("rows_removed", C.c_int32),
    ]


_gpu = None
_lp = None

GPU_SYMBOLS = [
    "help_pcg_default_options", "help_pcg_create", "help_pcg_free", "help_pcg_construct",
    "help_pcg_renew", "help_pcg_solve", "help_pcg_destruct", "help_pcg_get_stats",
    "help_pcg_last_error", "help_pcg_matvec", "help_pcg_matvec_dev", "help_pcg_matvec_acc", "help_pcg_precond_apply",
    "help_pcg_get_pivots", "help_pcg_cg", "help_pcg_cg_f32", "help_adat_assemble", "help_adat_matvec_noalloc",
    "help_mlp_create", "help_mlp_free", "help_mlp_last_error", "help_mlp_set_params", "help_mlp_get_params",
    "help_mlp_forward", "help_mlp_loss_grad", "help_mlp_train_step", "help_pcg_attach_mlp", "help_pcg_features",
    "help_pcg_pair_create", "help_pcg_pair_free", "help_pcg_pair_context", "help_pcg_pair_construct",
    "help_pcg_pair_renew", "help_pcg_pair_solve", "help_pcg_pair_solve2", "help_pcg_pair_destruct",
    "help_pcg_pair_matvec", "help_pcg_set_solve_slots", "help_pcg_share_solution",
]
LP_SYMBOLS = [
    "help_lp_generate", "help_lp_free", "help_lp_write_mps", "help_csc_to_csr", "help_lp_read_mps",
    "help_lp_write_bin", "help_lp_read_bin", "help_lp_last_error", "help_lp_remove_dependent_rows",
    "help_hsd_default_options", "help_hsd_solve",
]


def _load(name: str) -> C.CDLL:
    path = os.path.join(LIBDIR, name)
    if not os.path.exists(path):
        raise NativeLibraryError(
            "%s is not built; run `python -c 'import __graft_entry__ as g; g.build()'`" % path)
    try:
        return C.CDLL(path)
    except OSError as e:
        raise NativeLibraryError("cannot load %s: %s" % (path, e)) from e


def gpu_lib() -> C.CDLL:
    """The sm_103a backend library (raises if unavailable; never falls back)."""
    global _gpu
    if _gpu is None:
        lib = _load("libhelp_gpu.so")
        vp, i32, i64, dp = C.c_void_p, C.c_int32, C.c_int64, C.c_void_p
        lib.help_pcg_default_options.argtypes = [C.POINTER(PcgOptions)]
        lib.help_pcg_default_options.restype = None
        lib.help_pcg_create.argtypes = [C.POINTER(PcgOptions), C.POINTER(C.c_void_p)]
        lib.help_pcg_free.argtypes = [vp]
        lib.help_pcg_free.restype = None
        lib.help_pcg_construct.argtypes = [vp, i32, i32, dp, dp, dp]
        lib.help_pcg_renew.argtypes = [vp, dp]
        lib.help_pcg_solve.argtypes = [vp, dp, dp, dp, dp, dp]
        lib.help_pcg_destruct.argtypes = [vp]
        lib.help_pcg_get_stats.argtypes = [vp, C.POINTER(PcgStats)]
        lib.help_pcg_last_error.argtypes = [vp]
        lib.help_pcg_last_error.restype = C.c_char_p
        lib.help_pcg_matvec.argtypes = [vp, i32, dp, dp]
        lib.help_pcg_matvec_dev.argtypes = [vp, i32, i32, vp, vp, vp]
        lib.help_pcg_matvec_acc.argtypes = [vp, i32, i32, dp, dp]
        lib.help_pcg_precond_apply.argtypes = [vp, dp, dp]
        lib.help_pcg_get_pivots.argtypes = [vp, dp, dp, dp]
        lib.help_pcg_cg.argtypes = [vp, dp, dp, C.POINTER(C.c_int64)]
        lib.help_pcg_cg_f32.argtypes = [vp, dp, dp, C.POINTER(C.c_int64)]
        lib.help_adat_assemble.argtypes = [vp, dp, dp, dp, dp, C.POINTER(C.c_int64)]
        lib.help_adat_matvec_noalloc.argtypes = [i32, i32, i64] + [vp] * 10
        lib.help_pcg_pair_create.argtypes = [C.POINTER(PcgOptions), C.POINTER(C.c_void_p)]
        lib.help_pcg_pair_free.argtypes = [vp]
        lib.help_pcg_pair_free.restype = None
        lib.help_pcg_pair_context.argtypes = [vp, i32]
        lib.help_pcg_pair_context.restype = vp
        lib.help_pcg_set_solve_slots.argtypes = [vp, vp, i32]
        lib.help_pcg_share_solution.argtypes = [vp, i32, vp, i32]
        lib.help_mlp_create.argtypes = [i32, C.POINTER(C.c_void_p)]
        lib.help_mlp_free.argtypes = [vp]
        lib.help_mlp_last_error.argtypes = [vp]
        lib.help_mlp_last_error.restype = C.c_char_p
        lib.help_mlp_set_params.argtypes = [vp, dp]
        lib.help_mlp_get_params.argtypes = [vp, dp]
        lib.help_mlp_forward.argtypes = [vp, vp, i64, vp, vp]
        lib.help_mlp_loss_grad.argtypes = [vp, vp, vp, vp, i64, C.POINTER(C.c_double), dp]
        lib.help_mlp_train_step.argtypes = [vp, vp, vp, vp, i64, C.c_float, C.POINTER(C.c_double)]
        lib.help_pcg_attach_mlp.argtypes = [vp, vp]
        lib.help_pcg_features.argtypes = [vp, C.c_int32, vp]
        for s in GPU_SYMBOLS:
            getattr(lib, s)
        _gpu = lib
    return _gpu


def lp_lib() -> C.CDLL:
    global _lp
    if _lp is None:
        lib = _load("libhelp_lp.so")
        lib.help_lp_generate.argtypes = [C.POINTER(LpSpec), C.c_uint64, C.POINTER(LpStruct)]
        lib.help_lp_free.argtypes = [C.POINTER(LpStruct)]
        lib.help_lp_free.restype = None
        lib.help_lp_write_mps.argtypes = [C.POINTER(LpStruct), C.c_char_p]
        lib.help_lp_read_mps.argtypes = [C.c_char_p, C.POINTER(LpStruct)]
        lib.help_lp_write_bin.argtypes = [C.POINTER(LpStruct), C.c_char_p]
        lib.help_lp_read_bin.argtypes = [C.c_char_p, C.POINTER(LpStruct)]
        lib.help_lp_remove_dependent_rows.argtypes = [C.POINTER(LpStruct), C.c_double, C.POINTER(LpStruct),
                                                      C.c_void_p]
        lib.help_lp_last_error.argtypes = []
        lib.help_lp_last_error.restype = C.c_char_p
        lib.help_csc_to_csr.argtypes = [C.c_int32, C.c_int32] + [C.c_void_p] * 6
        lib.help_hsd_default_options.argtypes = [C.POINTER(HsdOptions)]
        lib.help_hsd_default_options.restype = None
        lib.help_hsd_solve.argtypes = [C.POINTER(LpStruct), C.POINTER(NeBackend), C.POINTER(HsdOptions),
                                       C.POINTER(HsdResult), C.c_void_p, C.c_void_p]
        for s in LP_SYMBOLS:
            getattr(lib, s)
        _lp = lib
    return _lp


def ptr(a) -> C.c_void_p:
    """Raw data pointer of a contiguous numpy array."""
    return C.c_void_p(a.ctypes.data)
