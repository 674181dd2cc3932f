"""The conversions users of the CPD path call on its results (cpd2tens,
cpd2unfold1, unfold, foldback) on the device vs the oracle."""
import numpy as np
import pytest

import tfx_oracle as orc

pytestmark = pytest.mark.gpu

tfx = pytest.importorskip("tensorfox_gb300")


def test_cpd2tens_and_unfoldings_vs_oracle():
    rng = np.random.default_rng(11)
    dims, R = (6, 5, 4, 3), 3
    W = [rng.standard_normal((d, R)) for d in dims]
    T = tfx.cpd2tens(W)
    np.testing.assert_allclose(T, orc.cpd2tens(W), rtol=1e-12, atol=1e-12)
    for m in range(1, 5):
        np.testing.assert_array_equal(tfx.unfold(T, m), orc.unfold(T, m))
        back = tfx.foldback(np.empty(dims), tfx.unfold(T, m), m)
        np.testing.assert_array_equal(back, T)
    T1 = np.empty((dims[0], int(np.prod(dims[1:]))))
    np.testing.assert_allclose(tfx.cpd2unfold1(T1, W), orc.cpd2unfold1(W), rtol=1e-12, atol=1e-12)


def test_dense2sparse_sparse2dense_vs_reference_rules():
    rng = np.random.default_rng(13)
    T = rng.standard_normal((5, 4, 3))
    T[rng.random(T.shape) < 0.5] = 0.0
    data, idxs, dims = tfx.dense2sparse(T)
    nz = np.nonzero(T)
    np.testing.assert_array_equal(idxs, np.stack(nz, axis=1))
    np.testing.assert_array_equal(data, T[nz])
    assert dims == [5, 4, 3]
    np.testing.assert_array_equal(tfx.sparse2dense(data, idxs, dims), T)


def test_multilinear_products_vs_oracle():
    """multilin_mult / multilin_mult_cpd / sparse_multilin_mult
    (MultilinearAlgebra.py:42-190) on the device vs the oracle."""
    rng = np.random.default_rng(14)
    dims = (6, 5, 4)
    T = rng.standard_normal(dims)
    UT = [rng.standard_normal((n, d)) for n, d in zip((3, 2, 4), dims)]
    np.testing.assert_allclose(tfx.multilin_mult(UT, orc.unfold(T, 1), dims), orc.multilin_mult(UT, T),
                               rtol=1e-12, atol=1e-12)
    U = [u.T for u in UT]
    W = [rng.standard_normal((n, 2)) for n in (3, 2, 4)]
    np.testing.assert_allclose(tfx.multilin_mult_cpd(U, W, (3, 2, 4)),
                               orc.cpd2tens([u @ w for u, w in zip(U, W)]), rtol=1e-12, atol=1e-12)
    lin = rng.choice(int(np.prod(dims)), size=40, replace=False)
    idxs = np.stack(np.unravel_index(lin, dims), axis=1)
    data = rng.standard_normal(40)
    np.testing.assert_allclose(tfx.sparse_multilin_mult(UT, data, idxs, dims),
                               orc.sparse_multilin_mult(UT, data, idxs, dims), rtol=1e-10, atol=1e-12)
