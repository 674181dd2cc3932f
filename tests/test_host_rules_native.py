"""Host-side rules of the C ABI that run before any device work (no GPU
needed): which shapes the tensor-core mode product takes, the scratch sizes the
direct solver's step update and COO error ask for, and argument errors returned
as status codes instead of launches."""
import ctypes

import pytest

from tensorfox_gb300 import _build

ERR_ARG = 1


@pytest.fixture(scope="module")
def lib():
    L = ctypes.CDLL(_build.build())
    L.tfx_ttm_tc_supported.argtypes = [ctypes.c_longlong, ctypes.c_int, ctypes.c_longlong, ctypes.c_int]
    L.tfx_step_update_wide_scratch_bytes.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int]
    L.tfx_step_update_wide_scratch_bytes.restype = ctypes.c_size_t
    L.tfx_step_update_wide.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                       ctypes.c_void_p]
    L.tfx_coo_model_error_scratch_bytes.argtypes = [ctypes.c_int, ctypes.c_int]
    L.tfx_coo_model_error_scratch_bytes.restype = ctypes.c_size_t
    return L


def dims_arg(dims):
    return (ctypes.c_int * len(dims))(*dims)


@pytest.mark.parametrize("P,D,Q,n,ok", [
    (1, 512, 262144, 50, True),      # the headline truncation
    (50, 512, 512, 50, True),        # the second mode of the same MLSVD
    (2500, 512, 1, 50, False),       # the last mode: no q tile
    (1, 500, 4096, 50, False),       # D not a multiple of 32
    (1, 512, 4096, 65, False),       # more than 64 columns of U
    (1, 512, 130, 7, False),         # Q not a multiple of 4 (TMA strides)
    (1, 32, 128, 1, True),           # one chunk, one tile
    (1, 4096, 1024, 64, True),       # U^T streamed per chunk: no bound on D
])
def test_ttm_tc_shape_rule(lib, P, D, Q, n, ok):
    assert bool(lib.tfx_ttm_tc_supported(P, D, Q, n)) == ok


def test_step_update_wide_scratch_sizes(lib):
    # one column-norm partial per (column, 256-row segment), four scalars per CTA, L R factors
    small = lib.tfx_step_update_wide_scratch_bytes(3, dims_arg([10, 9, 8]), 4)
    large = lib.tfx_step_update_wide_scratch_bytes(3, dims_arg([20000, 20000, 20000]), 16)
    assert small > 0 and large > small
    assert large >= (3 * 16 * ((20000 + 255) // 256)) * 8
    # rank above 64 and order 1 are refused (size 0)
    assert lib.tfx_step_update_wide_scratch_bytes(3, dims_arg([10, 9, 8]), 65) == 0
    assert lib.tfx_step_update_wide_scratch_bytes(1, dims_arg([10]), 4) == 0


def test_step_update_wide_refuses_bad_arguments_without_a_launch(lib):
    # null buffers and a scratch below the size asked for come back as argument errors
    d = dims_arg([10, 9, 8])
    assert lib.tfx_step_update_wide(0, 3, d, 4, None, None, None, None, 0.0, None, None, 0, None) == ERR_ARG
    fake = ctypes.c_void_p(16)  # never dereferenced: the size check fails first
    need = lib.tfx_step_update_wide_scratch_bytes(3, d, 4)
    assert lib.tfx_step_update_wide(0, 3, d, 4, fake, fake, fake, fake, 0.0, fake, fake, need - 1,
                                    None) == ERR_ARG
    assert lib.tfx_step_update_wide(0, 3, d, 65, fake, fake, fake, fake, 0.0, fake, fake, 1 << 20, None) == ERR_ARG


def test_coo_model_error_scratch_grows_with_rank(lib):
    a = lib.tfx_coo_model_error_scratch_bytes(3, 8)
    b = lib.tfx_coo_model_error_scratch_bytes(3, 16)
    assert 0 < a < b
