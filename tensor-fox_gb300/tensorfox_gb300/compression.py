"""Truncated MLSVD on the device (Compression.py:48-189).

Per mode, the reference runs a randomized SVD that streams the unfolding
several times.  Here the unfolding's Gram matrix ``S_(l) S_(l)^T`` is formed in
one pass over the tensor (``tfx_mode_gram``); its leading eigenvectors come from
a Rayleigh-Ritz step on ``span(G^3 Omega)`` -- the same Krylov depth as the
reference's two power iterations -- solved by an in-project Jacobi eigensolver,
or by Jacobi on ``G`` itself when the mode is small.  ``Omega`` is the very
Gaussian block the reference draws from NumPy's global RNG, so seeded runs keep
the RNG in step with the reference (the starting point drawn next is identical).

Singular vectors get the reference's sign convention (largest |entry| of every
column positive) and the same energy truncation (``clean_compression``).
"""
import numpy as np
import torch

from . import _dev, kernels
from .options import make_options


def _draw_omega(rows, n_random):
    """The reference's range-finder draw (Compression.py:382), as float64."""
    return np.random.normal(size=(rows, n_random))


def clean_compression(sigma, tol_mlsvd, L):
    """Smallest i with sum(sigma[i:]^2)/sum(sigma^2) < tol/L (Compression.py:261-301)."""
    eps = tol_mlsvd / L
    tot = np.sum(sigma ** 2)
    for i in range(1, len(sigma)):
        if np.sum(sigma[i:] ** 2) / tot < eps:
            return i
    return len(sigma)


def top_eig(G, n, omega=None, host=True):
    """Leading ``n`` eigenpairs of the symmetric D x D device matrix ``G``.

    Returns ``(Ut, lam)``: Ut is (n, D) (rows = eigenvectors, signs fixed),
    lam a float64 NumPy array (descending), or a device tensor with
    ``host=False`` (no wait for the device).
    """
    D = G.shape[0]
    n = min(n, D)
    direct = 64 if G.dtype == torch.float32 else 32
    k = min(n + 10, D)
    if D <= direct or k >= D:
        ev, V = kernels.sym_eig(G)
        Ut = V[:n].contiguous()
        lam = ev[:n]
    else:
        if omega is not None and omega.shape[0] == D:
            Yt = _dev.h2d(omega[:, :k].T, G.dtype, G.device)
        else:
            rng = np.random.default_rng(D * 7919 + k)
            Yt = _dev.h2d(rng.standard_normal((k, D)), G.dtype, G.device)
        for _ in range(3):
            Yt = kernels.matmul(Yt, G)          # (G Y)^T, G symmetric
            kernels.orthonormalize(Yt)
        Ht = kernels.matmul(Yt, G)
        B = kernels.matmul(Yt, Ht, transB=True)  # Y^T G Y
        ev, V = kernels.sym_eig(B)
        Ut = kernels.matmul(V[:n].contiguous(), Yt)
        lam = ev[:n]
    kernels.flip_signs(Ut)
    if not host:
        return Ut, lam
    lam = lam.double().cpu().numpy()
    return Ut, lam


def _mode_svd(S, shape, l, n, tol_mlsvd, L, draw_cols, tensor_cores=False):
    """One mode: Gram, eigenpairs, signs, truncation. Returns (Ut, sigma, dim).

    ``tensor_cores`` selects the TF32 tcgen05 Gram when the mode allows it."""
    omega = _draw_omega(draw_cols, n + 10)
    if tensor_cores and kernels.tc_gram_supported(S, shape, l):
        G = kernels.mode_gram_tc(S, shape, l)
    else:
        G = kernels.mode_gram(S, shape, l)
    Ut, lam = top_eig(G, n, omega)
    sigma = np.sqrt(np.maximum(lam, 0.0))
    dim = clean_compression(sigma, tol_mlsvd, L)
    return Ut[:dim].contiguous(), sigma[:dim], dim


def _ref_draw_cols(shape, l):
    """Row count of the reference's Gaussian block for this unfolding (Compression.py:487-493)."""
    D = int(shape[l])
    other = int(np.prod(shape, dtype=np.int64)) // D
    return D if D < other else other


def mlsvd_device(Td, R, options, speculate=True):
    """Device MLSVD of a dense C-order tensor. Returns (S, Ut_list, sigmas, shape).

    The sequential method is issued as one stream of device work with a single
    read at the end (``mlsvd_launch`` / ``mlsvd_confirm``); ``speculate=False``,
    or an energy truncation that cuts a mode, takes the mode-by-mode path."""
    o = options
    shape = [int(d) for d in Td.shape]
    L = len(shape)
    tol_mlsvd = o.tol_mlsvd
    if isinstance(tol_mlsvd, list):
        tol_mlsvd = tol_mlsvd[0] if L > 3 else tol_mlsvd[1]
    if tol_mlsvd == -1:
        eye = [torch.eye(d, dtype=Td.dtype, device=Td.device) for d in shape]
        return Td, eye, [np.ones(d) for d in shape], shape
    Uts, sigmas = [], []
    tc = getattr(o, 'precision', None) == 'mixed'
    if o.mlsvd_method in ('seq', 'gpu'):
        p = mlsvd_launch(Td, R, o) if speculate else None
        if p is not None:
            sig = mlsvd_confirm(p)
            if sig is not None:
                return _finish(p.S, p.Uts, sig, p.cur, o, L)
        S, cur = Td, list(shape)
        for l in range(L):
            n = o.svd_n_components if o.svd_n_components is not None else min(R, shape[l])
            Ut, sig, dim = _mode_svd(S, cur, l, n, tol_mlsvd, L, _ref_draw_cols(cur, l), tc)
            Uts.append(Ut)
            sigmas.append(sig)
            S, cur = kernels.ttm(S, cur, l, Ut, tensor_cores=tc)
        kernels.check_ttm_flag()
    elif o.mlsvd_method == 'classic':
        for l in range(L):
            n = o.svd_n_components if o.svd_n_components is not None else min(R, shape[l])
            Ut, sig, dim = _mode_svd(Td, shape, l, n, tol_mlsvd, L, _ref_draw_cols(shape, l), tc)
            Uts.append(Ut)
            sigmas.append(sig)
        S, cur = Td, list(shape)
        for l in range(L):
            S, cur = kernels.ttm(S, cur, l, Uts[l], tensor_cores=tc)
        kernels.check_ttm_flag()
    else:
        raise NotImplementedError("mlsvd_method %r" % (o.mlsvd_method,))
    return _finish(S, Uts, sigmas, cur, o, L)


class Pending:
    """A sequential MLSVD issued to the device and not yet checked: the core
    ``S`` (shape ``cur``) and the bases ``Uts`` assume every mode keeps
    n = min(R, d_l) singular vectors."""

    def __init__(self, S, Uts, cur, lams, errs, ns, state, tol_mlsvd):
        self.S, self.Uts, self.cur = S, Uts, cur
        self.lams, self.errs, self.ns = lams, errs, ns
        self.state, self.tol_mlsvd = state, tol_mlsvd


def mlsvd_launch(Td, R, o):
    """Issues the sequential MLSVD without waiting for the device, or returns
    None where that path does not apply (no compression, 'classic', user
    truncation).  Every mode is assumed to keep n = min(R, d_l) vectors; the
    eigenvalues stay on the device until ``mlsvd_confirm``."""
    shape = [int(d) for d in Td.shape]
    L = len(shape)
    tol_mlsvd = o.tol_mlsvd
    if isinstance(tol_mlsvd, list):
        tol_mlsvd = tol_mlsvd[0] if L > 3 else tol_mlsvd[1]
    if tol_mlsvd == -1 or o.mlsvd_method not in ('seq', 'gpu') or isinstance(o.trunc_dims, list):
        return None
    tc = getattr(o, 'precision', None) == 'mixed'
    state = np.random.get_state()
    S, cur = Td, list(shape)
    Uts, lams, errs, ns = [], [], [], []
    for l in range(L):
        n = o.svd_n_components if o.svd_n_components is not None else min(R, shape[l])
        omega = _draw_omega(_ref_draw_cols(cur, l), n + 10)
        if tc and kernels.tc_gram_supported(S, cur, l):
            G, err = kernels.mode_gram_tc(S, cur, l, check=False)
            errs.append(err)
        else:
            G = kernels.mode_gram(S, cur, l)
        Ut, lam = top_eig(G, n, omega, host=False)
        Uts.append(Ut)
        lams.append(lam.double())
        ns.append(int(lam.shape[0]))
        S, cur = kernels.ttm(S, cur, l, Ut, tensor_cores=tc)
    return Pending(S.contiguous().view(*cur), Uts, cur, lams, errs, ns, state, tol_mlsvd)


def mlsvd_confirm(p):
    """Reads the eigenvalues of a pending MLSVD in one transfer and applies the
    energy truncation (``clean_compression``).  Returns the singular values per
    mode, or None when some mode keeps fewer vectors than assumed -- NumPy's
    RNG is then put back to where it was before the MLSVD, and the caller
    redoes the work mode by mode (the reference's order of draws)."""
    host = torch.cat(p.lams).cpu().numpy()
    for err in p.errs:
        kernels.check_gram_flag(err)
    kernels.check_ttm_flag()
    L = len(p.ns)
    sigmas, off = [], 0
    for l in range(L):
        sigma = np.sqrt(np.maximum(host[off:off + p.ns[l]], 0.0))
        off += p.ns[l]
        if clean_compression(sigma, p.tol_mlsvd, L) != p.ns[l]:
            np.random.set_state(p.state)
            return None
        sigmas.append(sigma)
    return sigmas


def _finish(S, Uts, sigmas, cur, o, L):
    """User truncation (``trunc_dims``) and the core's final shape."""
    if isinstance(o.trunc_dims, list):
        sl = []
        for l in range(L):
            sl.append(slice(0, o.trunc_dims[l]))
            Uts[l] = Uts[l][:min(o.trunc_dims[l], Uts[l].shape[0])].contiguous()
        S = S[tuple(sl)].contiguous()
        cur = list(S.shape)
    return S.contiguous().view(*cur), Uts, sigmas, cur


def mlsvd(T, Tsize, R, options=None):
    """Drop-in for Compression.mlsvd: returns ``(S, U, T1, sigmas)`` as NumPy arrays.

    ``T1`` is the first unfolding of ``T`` (a layout view, Conversion.py:231).
    """
    _dev.require_cuda()
    o = make_options(options) if not hasattr(options, 'bi_method_parameters') else options
    if isinstance(T, list):
        from .sparse import DeviceCOO, mlsvd_sparse_device
        data, idxs, dims = T
        prec = o.precision if o.precision in ('fp64', 'fp32') else 'fp64'
        X = DeviceCOO(data, idxs, dims, _dev.torch_dtype(prec))
        S, Uts, sigmas = mlsvd_sparse_device(X, R, o)
        T1 = None
    else:
        prec = o.precision or ('fp64' if np.asarray(T).dtype == np.float64 else 'fp32')
        Td = _dev.to_device(T, _dev.torch_dtype(prec))
        S, Uts, sigmas, _ = mlsvd_device(Td, R, o)
        T1 = np.moveaxis(np.asarray(T, dtype=np.float64), 0, 0).reshape(T.shape[0], -1, order='F')
    U = [u.double().cpu().numpy().T.copy() for u in Uts]
    return S.double().cpu().numpy(), U, T1, sigmas
