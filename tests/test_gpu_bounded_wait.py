"""A bounded device wait that runs out reports TFX_STATUS_ERR_TIMEOUT and
leaves the context usable.

The wait polls an mbarrier that nothing arrives on (no copy or MMA in flight),
with the same bounded-wait helper the tensor-core kernels use for their copy
and MMA barriers; afterwards the same process runs a tensor-core Gram and gets
the right answer, so the context survived."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("limit", [1, 64, 4096])
def test_wait_that_runs_out_reports_timeout(limit):
    from tensorfox_gb300 import _lib, _dev, kernels
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    _lib.call("tfx_wait_probe", limit, ctypes.c_void_p(status.data_ptr()), ctypes.c_void_p(_dev.stream()))
    torch.cuda.synchronize()
    assert int(status.item()) == 3      # TFX_STATUS_ERR_TIMEOUT
    # the context is intact: a tcgen05 Gram right after is correct
    rng = np.random.default_rng(1)
    T = torch.from_numpy(rng.standard_normal((4, 128, 64)).astype(np.float32)).cuda()
    G = kernels.mode_gram_tc(T, [4, 128, 64], 1).double().cpu().numpy()
    U = np.moveaxis(T.double().cpu().numpy(), 1, 0).reshape(128, -1)
    ref = U @ U.T
    np.testing.assert_allclose(G, ref, rtol=1e-2, atol=1e-2 * np.abs(ref).max())


def test_wait_probe_rejects_bad_limits():
    from tensorfox_gb300 import _lib
    lib = _lib.load()
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert lib.tfx_wait_probe(0, ctypes.c_void_p(status.data_ptr()), None) == 1
    assert lib.tfx_wait_probe(1 << 27, ctypes.c_void_p(status.data_ptr()), None) == 1
