"""Index rules of the conversions (unfold / foldback) against the reference's
own unfoldings (golden fixture) -- the permutations run on CPU tensors here;
the same code runs on the device for the package's arrays."""
import numpy as np
import pytest
import torch

from conftest import load_golden

conv = pytest.importorskip("tensorfox_gb300.conversion")


def test_unfold_matches_reference_kolda_order():
    g = load_golden("kr_unfold")
    T = torch.from_numpy(g["T"])
    flat = np.concatenate([conv.unfold_tensor(T, m + 1).numpy().flatten() for m in range(T.dim())])
    np.testing.assert_array_equal(flat, g["unf"])


@pytest.mark.parametrize("dims", [(3, 4), (2, 3, 4), (4, 2, 3, 5), (2, 2, 3, 2, 3)])
def test_foldback_inverts_unfold(dims):
    T = torch.from_numpy(np.random.default_rng(len(dims)).standard_normal(dims))
    for m in range(1, len(dims) + 1):
        Tl = conv.unfold_tensor(T, m)
        assert tuple(Tl.shape) == (dims[m - 1], int(np.prod(dims)) // dims[m - 1])
        assert torch.equal(conv.foldback_tensor(Tl, m, dims), T)


def test_foldback_fills_the_given_array():
    T = torch.from_numpy(np.random.default_rng(9).standard_normal((3, 4, 5)))
    out = torch.zeros_like(T)
    assert conv.foldback(out, conv.unfold_tensor(T, 2), 2) is out
    assert torch.equal(out, T)


def test_mode_out_of_range():
    with pytest.raises(ValueError):
        conv.unfold_tensor(torch.zeros(2, 3), 3)


def test_dense2sparse_row_major_and_back():
    rng = np.random.default_rng(12)
    T = rng.standard_normal((4, 3, 5))
    T[rng.random(T.shape) < 0.6] = 0.0
    vals, idx = conv.dense2sparse_tensor(torch.from_numpy(T))
    nz = np.nonzero(T)                      # the reference's order (Conversion.py:174-204)
    np.testing.assert_array_equal(idx.numpy(), np.stack(nz, axis=1))
    np.testing.assert_array_equal(vals.numpy(), T[nz])
    back = conv.sparse2dense_tensor(vals, idx, T.shape)
    np.testing.assert_array_equal(back.numpy(), T)


def test_sparse2dense_sums_repeated_coordinates():
    vals = torch.tensor([1.0, 2.0, 5.0], dtype=torch.float64)
    idx = torch.tensor([[0, 1], [0, 1], [1, 0]])
    out = conv.sparse2dense_tensor(vals, idx, (2, 2))
    np.testing.assert_array_equal(out.numpy(), [[0.0, 3.0], [5.0, 0.0]])
