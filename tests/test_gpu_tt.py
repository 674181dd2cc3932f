"""Tensor-train CPD (method='ttcpd') on the device vs the reference's golden
runs and the oracle (TensorFox.py:256-421, 658-817, 1042-1065)."""
import numpy as np
import pytest
import torch

import tfx_oracle as orc
from conftest import load_golden, split_x
from test_oracle_golden import congruence

pytestmark = pytest.mark.gpu

tfx = pytest.importorskip("tensorfox_gb300")
from tensorfox_gb300 import tt  # noqa: E402


def test_tt_cores_match_reference():
    """The device TT-SVD equals the reference's cores and leaves the RNG where
    the reference leaves it."""
    g = load_golden("tt_cores")
    for k in range(int(g["n"])):
        T, R = g["T%d" % k], int(g["R%d" % k])
        np.random.seed(int(g["seed"]) + k)
        G = tt.cpdtt_device(torch.from_numpy(T).cuda(), R)
        assert np.random.rand() == float(g["after%d" % k])
        assert len(G) == int(g["ncores%d" % k])
        for j, c in enumerate(G):
            np.testing.assert_allclose(c.cpu().numpy(), g["G%d_%d" % (k, j)], rtol=1e-7, atol=1e-9)


def test_tt_cores_large_unfoldings_vs_oracle():
    """Both sides of a middle unfolding above the Jacobi limit (Rayleigh-Ritz
    route): a low-rank tensor's cores against the oracle's exact SVD."""
    rng = np.random.default_rng(3)
    dims, R = (12, 12, 12, 12), 10     # middle unfolding 120 x 144
    W = [rng.standard_normal((d, R)) for d in dims]
    T = orc.cpd2tens(W) + 1e-8 * rng.standard_normal(dims)
    np.random.seed(1)
    G0 = orc.cpdtt(T, R)
    np.random.seed(1)
    G1 = tt.cpdtt_device(torch.from_numpy(T).cuda(), R)
    # the TT is fixed up to signs of the rank index: compare the contracted tensor
    A = G1[0].cpu().numpy()
    for c in G1[1:-1]:
        A = np.tensordot(A, c.cpu().numpy(), axes=(-1, 0))
    A = np.tensordot(A, G1[-1].cpu().numpy(), axes=(-1, 0))
    np.testing.assert_allclose(A, T, rtol=0, atol=1e-6 * np.abs(T).max())
    for a, b in zip(G0, G1):
        assert a.shape == tuple(b.shape)


@pytest.mark.parametrize("name", ["cpd_tt_L3", "cpd_tt_L4", "cpd_tt_L5", "cpd_tt_dgn_L4"])
def test_cpd_tt_matches_reference(name):
    g = load_golden(name)
    T, R = g["T"], int(g["R"])
    o = tfx.Options()
    o.method = 'ttcpd'
    np.random.seed(int(g["seed"]))
    f, out = tfx.cpd(T, R, o)
    ref = float(g["rel_error"])
    assert abs(out.rel_error - ref) <= 1e-2 * ref
    assert congruence(f, split_x(g["factors"], T.shape, R)) > 0.999
    assert congruence(f, split_x(g["planted"], T.shape, R)) > 0.999
    assert len(out.cpd_output) == T.ndim - 2


def test_als_fixed_mode_matches_oracle():
    """bicpd's solver: ALS with one factor fixed (Alternating_Least_Squares.py:236-264)."""
    rng = np.random.default_rng(9)
    dims, R = (5, 9, 5), 4
    W = [rng.standard_normal((d, R)) for d in dims]
    T = orc.cpd2tens(W) + 1e-3 * rng.standard_normal(dims)
    init = [w + 0.3 * rng.standard_normal(w.shape) for w in W]
    for fl in (0, 2):
        class O:
            maxiter = 30
        a = [w.copy() for w in init]
        a[fl] = [W[fl].copy(), fl]
        b = [w.copy() for w in init]
        b[fl] = [W[fl].copy(), fl]
        f0, ss0, er0, _, _, st0 = orc.als(T, a, R, orc.make_options(O))
        f1, ss1, er1, _, _, st1 = tfx.als(T, b, R, tfx.make_options(O))
        assert st1 == st0 and len(er1) == len(er0)
        np.testing.assert_allclose(er1, er0, rtol=1e-8)
        np.testing.assert_allclose(f1[fl], W[fl], rtol=0, atol=0)


def test_cpd_tt_sparse_matches_reference():
    """method='ttcpd' on [data, idxs, dims] (every entry stored): the sparse
    MLSVD, the TT path on the dense core, the error on the stored entries."""
    g = load_golden("cpd_tt_sparse")
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    o = tfx.Options()
    o.method = 'ttcpd'
    np.random.seed(int(g["seed"]))
    f, out = tfx.cpd([g["data"], g["idxs"], np.array(dims)], R, o)
    ref = float(g["rel_error"])
    assert abs(out.rel_error - ref) <= 1e-2 * ref
    assert congruence(f, split_x(g["factors"], dims, R)) > 0.999
