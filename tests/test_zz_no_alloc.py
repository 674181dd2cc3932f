"""The allocation-free mode Gram (tfx_mode_gram_noalloc) agrees with tfx_mode_gram
and with the FP64 NumPy product of the unfolding with its transpose.

It exists for callers that cannot allocate device memory at call time (a host
whose memory pool owns the device, a latency-critical path, a no-allocation
policy after start-up).  This file is named so that pytest collects it last,
and it also passes when run alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _lib():
    from tensorfox_gb300 import _lib as L
    lib = L.load()
    fn = lib.tfx_mode_gram_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int, ctypes.c_longlong,
                   ctypes.c_void_p, ctypes.c_void_p]
    lib.tfx_mode_gram_noalloc_capacity_bytes.restype = ctypes.c_size_t
    return L, lib


@pytest.mark.parametrize("dtype,shape,l", [(torch.float32, (300, 40, 30), 0), (torch.float32, (20, 64, 50), 1),
                                           (torch.float64, (64, 30, 20), 2)])
def test_noalloc_matches_allocating_entry_point(dtype, shape, l):
    L, lib = _lib()
    from tensorfox_gb300 import kernels
    rng = np.random.default_rng(123)
    T = torch.from_numpy(rng.standard_normal(shape)).to("cuda", dtype)
    P = int(np.prod(shape[:l]))
    D = int(shape[l])
    Q = int(np.prod(shape[l + 1:]))
    ref = kernels.mode_gram(T, list(shape), l).double().cpu().numpy()
    # the same Gram in FP64 NumPy: the (P, D, Q) view's mode unfolding times its transpose
    U = np.moveaxis(T.double().cpu().numpy().reshape(P, D, Q), 1, 0).reshape(D, P * Q)
    exact = U @ U.T
    code = L.F64 if dtype == torch.float64 else L.F32
    stream = ctypes.c_void_p(int(torch.cuda.current_stream().cuda_stream))
    tol = 1e-12 if dtype == torch.float64 else 2e-5
    for _ in range(2):  # two calls in a row share the built-in scratch
        G = torch.full((D, D), float("nan"), dtype=dtype, device="cuda")
        status = lib.tfx_mode_gram_noalloc(code, ctypes.c_void_p(T.data_ptr()), P, D, Q,
                                           ctypes.c_void_p(G.data_ptr()), stream)
        assert status == 0, lib.tfx_last_error()
        torch.cuda.synchronize()
        got = G.double().cpu().numpy()
        np.testing.assert_allclose(got, ref, rtol=tol, atol=tol * np.abs(ref).max())
        np.testing.assert_allclose(got, exact, rtol=tol, atol=tol * np.abs(exact).max())


def test_noalloc_rejects_a_gram_larger_than_its_scratch():
    L, lib = _lib()
    assert lib.tfx_mode_gram_noalloc_capacity_bytes() == 32 << 20
    T = torch.zeros(8, device="cuda")
    G = torch.zeros(8, device="cuda")
    # 4096 x 4096 float32 partials need 64 MiB: refused before any launch
    status = lib.tfx_mode_gram_noalloc(L.F32, ctypes.c_void_p(T.data_ptr()), 1, 4096, 1,
                                       ctypes.c_void_p(G.data_ptr()), None)
    assert status == 1
    assert b"32 MiB" in lib.tfx_last_error()
