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


@pytest.mark.parametrize("dims,R", [((64, 48, 40), 10), ((300, 128, 8), 64), ((130, 70, 36), 33),
                                    ((30, 20, 16, 12), 7), ((512, 96, 64), 50), ((9, 260, 300), 5)])
def test_tc_mttkrp_all_modes_vs_fp64(dims, R):
    """The tcgen05 MTTKRP (TMA-fed tensor tiles, 3xTF32, FP32 accumulation) of
    every mode against the FP64 oracle's T_(l) KR_l: within 1e-5 relative
    (norm-wise and entry-wise against the largest entry); the last mode reads
    the copy with that mode moved first."""
    from tensorfox_gb300 import kernels
    rng = np.random.default_rng(14)
    T = rng.standard_normal(dims).astype(np.float32)
    W = [rng.standard_normal((d, R)).astype(np.float32) for d in dims]
    Td = torch.from_numpy(T).cuda()
    flat = torch.from_numpy(orc.cpd2flat([w.astype(np.float64) for w in W])).cuda().float()
    Tl = [orc.unfold(T.astype(np.float64), l + 1) for l in range(len(dims))]
    W64 = [w.astype(np.float64) for w in W]
    for l in range(len(dims)):
        assert kernels.mttkrp_tc_supported(Td, list(dims), R, l)
        got, err = kernels.mttkrp_tc(Td, list(dims), flat, R, l)
        assert int(err.item()) == 0
        got = got.double().cpu().numpy()
        ref = orc.mttkrp(Tl, W64, l)
        assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(ref)
        assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
        gc, _ = kernels.mttkrp_tc(Td, list(dims), flat, R, l, col_major=True)
        np.testing.assert_array_equal(gc.cpu().numpy().T, got.astype(np.float32))


@pytest.mark.parametrize("shape,l,n", [((512, 64, 64), 0, 50), ((3, 64, 300), 1, 64), ((96, 40, 128), 0, 7),
                                       ((5, 32, 129, 4), 1, 33), ((2, 512, 1000), 1, 50)])
def test_tc_ttm_matches_fp64(shape, l, n):
    """The tcgen05 mode product (3xTF32: operands split hi + lo, FP32
    accumulation; precision 'mixed') against FP64: within 1e-5 of the
    product's norm like the FP32 SIMT product, every tile tail (Q not a
    multiple of 128, n below 64 and odd) included."""
    rng = np.random.default_rng(3)
    T = rng.standard_normal(shape).astype(np.float32)
    D = shape[l]
    U = rng.standard_normal((D, n)).astype(np.float32)
    Td = torch.from_numpy(T).cuda()
    Ut = torch.from_numpy(np.ascontiguousarray(U.T)).cuda()
    P, Q = int(np.prod(shape[:l], dtype=np.int64)), int(np.prod(shape[l + 1:], dtype=np.int64))
    from tensorfox_gb300 import _lib
    assert _lib.load().tfx_ttm_tc_supported(P, D, Q, n)
    got, new_shape = kernels.ttm(Td, list(shape), l, Ut, tensor_cores=True)
    kernels.check_ttm_flag()
    ref = np.moveaxis(np.tensordot(T.astype(np.float64), U.astype(np.float64), axes=([l], [0])), -1, l)
    assert list(ref.shape) == list(new_shape)
    got = got.double().cpu().numpy()
    assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(ref)
    # the FP32 SIMT product of the same call, for comparison
    simt, _ = kernels.ttm(Td, list(shape), l, Ut)
    assert np.linalg.norm(simt.double().cpu().numpy() - ref) <= 1e-5 * np.linalg.norm(ref)
