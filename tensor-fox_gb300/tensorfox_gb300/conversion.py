"""Conversions of Tensor Fox's public namespace that users of the CPD path call
on its inputs and results (Conversion.py:52-315): ``cpd2tens``, ``cpd2unfold1``,
``unfold``, ``foldback``, and the COO converters ``dense2sparse`` /
``sparse2dense`` of the sparse input format ``[data, idxs, dims]``.

``cpd2tens`` forms the tensor on the device (``tfx_cp_full``).  ``unfold`` and
``foldback`` are index permutations, done on whichever device holds the
tensor (a NumPy input is permuted on the GPU and returned as NumPy, like the
reference's arrays).  The mode-m unfolding uses Kolda's column order
(Critical.py:124+): the column of entry (i_1, ..., i_L) is
sum_{k != m} i_k prod_{j < k, j != m} d_j, so the remaining axes are flattened
with the first one varying fastest.
"""
import numpy as np
import torch

from . import _dev


def _as_tensor(T):
    """(tensor, was_numpy): NumPy input goes to the GPU as float64."""
    if isinstance(T, torch.Tensor):
        return T, False
    return _dev.to_device(np.asarray(T), torch.float64), True


def unfold_tensor(t, mode):
    """Mode-``mode`` (1-based) unfolding of a torch tensor, same device, as a
    (d_mode, N / d_mode) tensor in Kolda's column order."""
    L = t.dim()
    m = int(mode) - 1
    if not 0 <= m < L:
        raise ValueError("mode must be between 1 and the order of the tensor")
    rest = [k for k in range(L) if k != m]
    # the remaining axes reversed and flattened row-major = flattened with the
    # first remaining axis fastest
    return t.permute(m, *reversed(rest)).reshape(t.shape[m], -1)


def foldback_tensor(Tl, mode, dims):
    """Inverse of ``unfold_tensor``: the tensor of shape ``dims``."""
    L = len(dims)
    m = int(mode) - 1
    if not 0 <= m < L:
        raise ValueError("mode must be between 1 and the order of the tensor")
    rest = [k for k in range(L) if k != m]
    order = [m] + list(reversed(rest))
    t = Tl.reshape([int(dims[k]) for k in order])
    inv = [0] * L
    for pos, k in enumerate(order):
        inv[k] = pos
    return t.permute(*inv).contiguous()


def unfold(T, mode):
    """Drop-in for Conversion.unfold (Conversion.py:207-228): the mode-``mode``
    unfolding (1 <= mode <= L), a Fortran-ordered NumPy array for NumPy input,
    a device tensor for a torch tensor."""
    t, was_np = _as_tensor(T)
    out = unfold_tensor(t, mode)
    if was_np:
        return np.asfortranarray(out.cpu().numpy())
    return out


def foldback(T, Tl, mode):
    """Drop-in for Conversion.foldback (Conversion.py:305-315): fills ``T``
    (whose shape gives the dimensions) from its mode-``mode`` unfolding ``Tl``
    and returns it."""
    dims = tuple(int(d) for d in T.shape)
    tl, was_np = _as_tensor(Tl)
    out = foldback_tensor(tl, mode, dims)
    if isinstance(T, torch.Tensor):
        T.copy_(out.to(device=T.device, dtype=T.dtype))
        return T
    T[...] = out.cpu().numpy()
    return T


def cpd2tens(factors):
    """Drop-in for Conversion.cpd2tens (Conversion.py:52-79): the tensor of the
    CPD ``factors`` ((d_l, R) arrays), formed on the device in FP64 and returned
    as NumPy (torch factors give a device tensor of their dtype)."""
    from .autograd import cp_full
    if all(isinstance(W, torch.Tensor) for W in factors):
        return cp_full([W.to(device=_dev.device()) for W in factors])
    Wd = [_dev.to_device(np.asarray(W, dtype=np.float64), torch.float64) for W in factors]
    return cp_full(Wd).cpu().numpy()


def cpd2unfold1(T1_approx, factors):
    """Drop-in for Conversion.cpd2unfold1 (Conversion.py:117-141): the first
    unfolding of the CPD's tensor, written into ``T1_approx`` and returned."""
    from .autograd import cp_full
    Wd = [_dev.to_device(np.asarray(W, dtype=np.float64), torch.float64) for W in factors]
    out = unfold_tensor(cp_full(Wd), 1)
    if isinstance(T1_approx, torch.Tensor):
        T1_approx.copy_(out.to(device=T1_approx.device, dtype=T1_approx.dtype))
        return T1_approx
    T1_approx[...] = out.cpu().numpy()
    return T1_approx


def dense2sparse_tensor(t):
    """(values, indices (nnz, L) int64) of the nonzero entries of a torch tensor,
    in row-major (C) order, on its device."""
    idx = torch.nonzero(t)
    return t[tuple(idx.t())], idx


def sparse2dense_tensor(vals, idx, dims, dtype=torch.float64):
    """Dense tensor of shape ``dims`` from values and (nnz, L) indices on the
    same device (a repeated coordinate keeps the sum of its values)."""
    out = torch.zeros([int(d) for d in dims], dtype=dtype, device=vals.device)
    if idx.numel():
        out.index_put_(tuple(idx.t().long()), vals.to(dtype), accumulate=True)
    return out


def dense2sparse(T):
    """Drop-in for Conversion.dense2sparse (Conversion.py:174-204):
    ``[data, idxs, dims]`` of the nonzero entries of ``T``, in row-major order."""
    if isinstance(T, torch.Tensor):
        t = T
    else:
        arr = np.asarray(T)
        t = _dev.to_device(arr, torch.float32 if arr.dtype == np.float32 else torch.float64)
    vals, idx = dense2sparse_tensor(t)
    return [vals.cpu().numpy(), idx.cpu().numpy(), list(int(d) for d in t.shape)]


def sparse2dense(data, idxs, dims):
    """Drop-in for Conversion.sparse2dense (Conversion.py:144-171): the dense
    FP64 tensor of ``[data, idxs, dims]``."""
    vals = _dev.to_device(np.asarray(data, dtype=np.float64), torch.float64)
    idx = torch.as_tensor(np.asarray(idxs, dtype=np.int64).reshape(-1, len(dims)), device=vals.device)
    return sparse2dense_tensor(vals, idx, dims).cpu().numpy()


def multilin_mult(UT, T1, dims):
    """Drop-in for MultilinearAlgebra.multilin_mult (MultilinearAlgebra.py:72-105):
    (U[0]^T, ..., U[L-1]^T) * T from the first unfolding ``T1`` of T (shape
    ``dims``); UT[l] is (n_l, d_l).  The mode products run on the device
    (``tfx_ttm``) in FP64; returns NumPy."""
    from . import kernels
    dims = [int(d) for d in dims]
    t1, _ = _as_tensor(T1)
    S = foldback_tensor(t1.to(torch.float64), 1, dims)
    cur = list(dims)
    for l in range(len(dims)):
        Ut = _dev.to_device(np.asarray(UT[l], dtype=np.float64), torch.float64)
        S, cur = kernels.ttm(S.contiguous(), cur, l, Ut)
    return S.reshape(cur).cpu().numpy()


def multilin_mult_cpd(U, W, dims):
    """Drop-in for MultilinearAlgebra.multilin_mult_cpd (MultilinearAlgebra.py:42-69):
    the tensor of the CPD (U[0] W[0], ..., U[L-1] W[L-1])."""
    from . import kernels
    from .autograd import cp_full
    UW = []
    for Ul, Wl in zip(U, W):
        Ud = _dev.to_device(np.asarray(Ul, dtype=np.float64), torch.float64)
        Wd = _dev.to_device(np.asarray(Wl, dtype=np.float64), torch.float64)
        UW.append(kernels.matmul(Ud, Wd))
    return cp_full(UW).cpu().numpy()


def sparse_multilin_mult(UT, data, idxs, dims):
    """Drop-in for MultilinearAlgebra.sparse_multilin_mult (MultilinearAlgebra.py:
    145-190): the dense core (U[0]^T, ..., U[L-1]^T) * T of the COO tensor
    ``[data, idxs, dims]``, UT[l] (n_l, d_l), computed on the device in FP64
    (``tfx_sparse_ttmc``); returns NumPy."""
    from .sparse import DeviceCOO, sparse_ttmc
    X = DeviceCOO(data, idxs, dims, torch.float64)
    Uts = [_dev.to_device(np.asarray(u, dtype=np.float64), torch.float64) for u in UT]
    return sparse_ttmc(X, Uts).cpu().numpy()
