"""ctypes binding of ``libtfx_gb300.so`` (the C ABI declared in include/tfx_gb300.h).

The library is the only compute path: every public routine of this package calls
into it and raises if it is missing or if no CUDA device is present.
"""
import ctypes
import os
from ctypes import POINTER, c_double, c_int, c_longlong, c_size_t, c_void_p, c_char_p

MAX_ORDER = 12
F32, F64 = 0, 1

STATUS = {0: "ok", 1: "invalid argument", 2: "numeric error", 3: "timeout", 4: "CUDA error",
          5: "unsupported configuration"}


class TfxError(RuntimeError):
    """Raised when an entry point of the C ABI returns a non-zero status."""


def check_solve_status(result_rows):
    """Raise if any solved problem reports a non-zero status (``result[:, 2]``),
    e.g. a bounded device wait of the engine that ran out."""
    import numpy as _np
    st = _np.asarray(result_rows)[..., 2]
    if _np.any(st != 0):
        raise TfxError("dGN engine reported status %d (3 = a bounded device wait ran out)" % int(st.max()))


class DgnProblem(ctypes.Structure):
    _fields_ = [("L", c_int), ("R", c_int), ("dims", c_int * MAX_ORDER),
                ("tensor", c_void_p), ("x", c_void_p), ("best", c_void_p), ("work", c_void_p),
                ("budgets", c_void_p), ("damp_sched", c_void_p), ("stats", c_void_p),
                ("result", c_void_p), ("info", c_void_p), ("prof", c_void_p)]


class DgnOptions(ctypes.Structure):
    _fields_ = [("maxiter", c_int), ("tol", c_double), ("tol_step", c_double), ("tol_improv", c_double),
                ("tol_grad", c_double), ("tol_jump", c_double), ("cg_tol", c_double),
                ("init_damp", c_double), ("use_damp_sched", c_int), ("symm", c_int),
                ("factors_norm", c_double), ("tile", c_int), ("aliased", c_int), ("fixed", c_int)]


_LIB = None


def lib_path():
    from ._build import LIB
    return LIB


def load():
    """Loads the compiled library (building it first if it is absent)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        from ._build import build
        build()
    lib = ctypes.CDLL(path)
    _declare(lib)
    _LIB = lib
    return lib


def _declare(lib):
    lib.tfx_last_error.restype = c_char_p
    lib.tfx_launch_count.restype = c_longlong
    lib.tfx_version.restype = c_int
    lib.tfx_dgn_workspace_bytes.restype = c_size_t
    lib.tfx_dgn_workspace_bytes.argtypes = [c_int, c_int, POINTER(c_int), c_int]
    lib.tfx_dgn_solve.restype = c_int
    lib.tfx_dgn_solve.argtypes = [c_int, POINTER(DgnProblem), c_void_p, c_int, POINTER(DgnOptions), c_int,
                                  c_void_p]
    lib.tfx_jtj_matvec.restype = c_int
    lib.tfx_jtj_matvec.argtypes = [c_int, POINTER(DgnProblem), c_void_p, POINTER(DgnOptions), c_int, c_double,
                                   c_void_p, c_void_p, c_void_p, c_void_p]
    lib.tfx_dgn_dogleg.restype = c_int
    lib.tfx_dgn_dogleg.argtypes = [c_int, POINTER(DgnProblem), c_void_p, POINTER(DgnOptions), c_int, c_double,
                                   c_double, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                   c_void_p]
    for name, args in _EXTRA_SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = c_int
        fn.argtypes = args
    for name, args in _SIZE_FUNCS.items():
        fn = getattr(lib, name)
        fn.restype = c_size_t
        fn.argtypes = args


def call(name, *args):
    """Calls an int-status entry point and raises TfxError on failure."""
    check(getattr(load(), name)(*args))


# Remaining entry points: (name -> argtypes); all return an int status.
_P = c_void_p
_I = c_int
_LL = c_longlong
_D = c_double
_SZ = c_size_t
_EXTRA_SIGNATURES = {
    "tfx_mode_gram": [_I, _P, _LL, _I, _LL, _P, _P, _SZ, _P],
    "tfx_wait_probe": [ctypes.c_uint, _P, _P],
    "tfx_coo_dgn_cg": [_I, _I, POINTER(c_int), _I, _P, _P, _D, _I, _D, _P, _P, _P, _P, _P, _SZ, _P],
    "tfx_coo_model_error": [_I, _I, POINTER(c_int), _I, _P, _P, _D, _P, _P, _SZ, _P],
    "tfx_factors_to_rows": [_I, _I, POINTER(c_int), _I, _P, _P, _P],
    "tfx_dogleg_dots": [_LL, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "tfx_dogleg_trial": [_I, _LL, _P, _P, _P, _D, _D, _D, _P, _P, _P, _P, _P],
    "tfx_step_sums": [_I, _LL, _P, _P, _P, _D, _P, _P, _P],
    "tfx_step_revert": [_I, _LL, _P, _P, _P, _P],
    "tfx_step_update_wide": [_I, _I, POINTER(c_int), _I, _P, _P, _P, _P, _D, _P, _P, _SZ, _P],
    "tfx_mttkrp_tc": [_P, _I, POINTER(c_int), _I, _P, _I, _P, _I, _P, _SZ, _P, _P],
    "tfx_factors_bf16": [_I, POINTER(c_int), _I, _P, _P, _P, _P],
    "tfx_coo_mttkrp_bf16": [_P, _P, _LL, _P, _I, POINTER(c_int), _I, _I, _P, _P, _P, _P],
    "tfx_gemm": [_I, _P, _P, _P, _LL, _LL, _LL, _LL, POINTER(c_longlong), _D, _D, _P],
    "tfx_orthonormalize": [_I, _P, _I, _I, _P],
    "tfx_ttm": [_I, _P, _LL, _I, _LL, _P, _I, _P, _P],
    "tfx_ttm_tc": [_P, _LL, _I, _LL, _P, _I, _P, _P, _P],
    "tfx_sym_eig": [_I, _P, _I, _P, _P, _I, _P, _P],
    "tfx_flip_signs": [_I, _P, _I, _I, _P],
    "tfx_cp_residual": [_I, _P, _I, POINTER(c_int), _I, _P, _P, _P, _P],
    "tfx_tensor_norms": [_I, _P, _LL, _P, _P, _P],
    "tfx_coo_encode": [_P, _LL, _I, POINTER(c_int), _P, _P, _P],
    "tfx_mode_gram_tc": [_P, _LL, _I, _LL, _P, _P, _SZ, _P, _P],
    "tfx_coo_sort_mode": [_I, _P, _P, _LL, _I, POINTER(c_int), _I, _P, _P, _P, _P, _P],
    "tfx_coo_mttkrp": [_I, _P, _P, _LL, _P, _I, POINTER(c_int), _I, _I, _P, _P, _P],
    "tfx_sparse_residual": [_I, _P, _P, _LL, _I, POINTER(c_int), _I, _P, _P, _P, _P],
    "tfx_coo_gram": [_I, _P, _P, _LL, _P, _P, _I, POINTER(c_int), _I, _P, _P, _SZ, _P, _P],
    "tfx_sparse_ttmc": [_I, _P, _P, _LL, _I, POINTER(c_int), POINTER(c_int), _P, _P, _P, _SZ, _P],
    "tfx_als_solve": [_I, _P, _I, POINTER(c_int), _I, _P, _P, _P, _P, _P, POINTER(DgnOptions), _I, _P, _SZ, _P],
    "tfx_als_sweep": [_I, _P, _I, POINTER(c_int), _I, _P, _I, _P, _SZ, _P],
    "tfx_dgn_direct_step": [_I, _P, _I, POINTER(c_int), _I, _P, _D, _P, _P, _P, _SZ, _P],
    "tfx_dgn_step_update": [_I, _I, POINTER(c_int), _I, _P, _P, _P, _P, _D, _I, _I, _D, _I, _I, _P, _P, _P],
}
_SIZE_FUNCS = {
    "tfx_mode_gram_scratch_bytes": [_I, _LL, _I, _LL],
    "tfx_sym_eig_smem_bytes": [_I, _I],
    "tfx_mode_gram_tc_scratch_bytes": [_LL, _I, _LL],
    "tfx_cp_residual_scratch_bytes": [],
    "tfx_sparse_residual_scratch_bytes": [],
    "tfx_coo_gram_scratch_bytes": [_LL, _I],
    "tfx_sparse_ttmc_scratch_bytes": [_I, _LL, _I, POINTER(c_int)],
    "tfx_als_workspace_bytes": [_I, _I, POINTER(c_int), _I],
    "tfx_dgn_direct_workspace_bytes": [_I, _I, POINTER(c_int), _I],
    "tfx_coo_dgn_cg_workspace_bytes": [_I, _I, POINTER(c_int), _I],
    "tfx_coo_model_error_scratch_bytes": [_I, _I],
    "tfx_dogleg_scratch_bytes": [],
    "tfx_ttm_tc_supported": [_LL, _I, _LL, _I],
    "tfx_step_update_wide_scratch_bytes": [_I, POINTER(c_int), _I],
    "tfx_mttkrp_tc_scratch_bytes": [_I, POINTER(c_int), _I, _I],
}


def check(status):
    if status != 0:
        msg = _LIB.tfx_last_error().decode() if _LIB is not None else ""
        raise TfxError("%s: %s" % (STATUS.get(status, "status %d" % status), msg))


def launch_count():
    return int(load().tfx_launch_count())
