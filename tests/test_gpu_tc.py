"""Tensor-core (tcgen05, TF32) mode Gram vs the FP32 SIMT Gram and FP64 NumPy."""
import numpy as np
import pytest

import tfx_oracle as orc

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
from tensorfox_gb300 import kernels  # noqa: E402


@pytest.mark.parametrize("shape,l", [((256, 64, 32), 0), ((128, 4096), 0), ((300, 40, 36), 0), ((20, 200, 64), 1),
                                     ((7, 130, 5, 32), 1), ((512, 96, 64), 0), ((700, 8, 32), 0)])
def test_tc_gram_matches_fp64(shape, l):
    rng = np.random.default_rng(7)
    T = rng.standard_normal(shape).astype(np.float32)
    Td = torch.from_numpy(T).cuda()
    assert kernels.tc_gram_supported(Td, list(shape), l)
    G = kernels.mode_gram_tc(Td, list(shape), l).double().cpu().numpy()
    U = orc.unfold(T.astype(np.float64), l + 1)
    ref = U @ U.T
    # TF32 operands (10-bit mantissa): entries agree to ~1e-3 of the largest entry
    np.testing.assert_allclose(G, ref, rtol=0, atol=3e-3 * np.abs(ref).max())
    # and the diagonal (sums of squares) to a few 1e-4 relative
    np.testing.assert_allclose(np.diag(G), np.diag(ref), rtol=2e-3)
    Gs = kernels.mode_gram(Td, list(shape), l).double().cpu().numpy()
    np.testing.assert_allclose(G, Gs, rtol=0, atol=3e-3 * np.abs(ref).max())


def test_tc_gram_leading_subspace_matches():
    """What the MLSVD needs: the leading eigenvectors of the TF32 Gram match FP64's."""
    rng = np.random.default_rng(8)
    dims, R = (256, 128, 64), 10
    W = [rng.standard_normal((d, R)) for d in dims]
    T = orc.cpd2tens(W) + 1e-2 * rng.standard_normal(dims)
    Td = torch.from_numpy(T.astype(np.float32)).cuda()
    G = kernels.mode_gram_tc(Td, list(dims), 0).double().cpu().numpy()
    U = orc.unfold(T, 1)
    ref = U @ U.T
    ev, V = np.linalg.eigh(G)
    evr, Vr = np.linalg.eigh(ref)
    Vt, Vrt = V[:, -R:], Vr[:, -R:]
    s = np.linalg.svd(Vt.T @ Vrt, compute_uv=False)
    assert s.min() > 1 - 1e-5      # principal angles below ~5e-3 rad


def test_mixed_precision_cpd_c2_like():
    """precision='mixed' (TF32 tensor-core compression): same final error as FP32 within 1e-2 relative."""
    import tensorfox_gb300 as tfx
    rng = np.random.default_rng(12)
    dims, R = (128, 96, 64), 8
    W = [rng.standard_normal((d, R)) for d in dims]
    T = orc.cpd2tens(W)
    E = rng.standard_normal(dims)
    T = (T + 1e-2 * np.linalg.norm(T) / np.linalg.norm(E) * E).astype(np.float32)
    o = tfx.make_options(None)
    o.precision = 'mixed'
    np.random.seed(0)
    _, out_m = tfx.cpd(T, R, o)
    o.precision = 'fp32'
    np.random.seed(0)
    _, out_f = tfx.cpd(T, R, o)
    assert abs(out_m.rel_error - out_f.rel_error) <= 1e-2 * out_f.rel_error
