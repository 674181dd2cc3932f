"""Sparse (COO) tensors on the device (TensorFox.py:476-481, Compression.py:123-137,
Critical.py:25-53, MultilinearAlgebra.py:145-190).

A sparse tensor is given as ``[data, idxs, dims]`` like in Tensor Fox.  On the
device the coordinates are re-encoded once to int32 structure-of-arrays
(``tfx_coo_encode``, bounds-checked) and per-mode row-sorted copies are built on
demand (``tfx_coo_sort_mode``).

``tricpd_sparse`` follows the reference's semantics exactly: absent entries are
zeros of the data, the MLSVD works on the dense Gram ``T_(l) T_(l)^T`` of every
unfolding, the core is the sparse multilinear product, dGN runs on the dense
core and the final error counts the stored entries only.
"""
import ctypes

import numpy as np
import torch

from . import _dev, _lib, kernels
from .compression import clean_compression, top_eig, _draw_omega


def _vp(t):
    return ctypes.c_void_p(_dev.ptr(t))


def _st():
    return ctypes.c_void_p(_dev.stream())


def _cint(vals):
    vals = [int(v) for v in vals]
    return (ctypes.c_int * len(vals))(*vals)


class DeviceCOO:
    """COO tensor resident on the device: int32 SoA coordinates and values."""

    def __init__(self, data, idxs, dims, dtype, perm=None):
        """``perm``: the modes of ``dims`` are the input coordinates' columns
        ``perm[0], perm[1], ...`` (applied on the device, after the copy)."""
        dims = [int(d) for d in dims]
        self.dims = dims
        self.L = len(dims)
        if max(dims) >= 2 ** 31:
            raise ValueError("dimensions must be below 2^31")
        dev = _dev.device()
        idx = torch.as_tensor(np.ascontiguousarray(np.asarray(idxs, dtype=np.int64).reshape(-1, self.L)),
                              device=dev)
        if perm is not None and [int(v) for v in perm] != list(range(self.L)):
            idx = idx[:, torch.as_tensor(np.asarray(perm, dtype=np.int64), device=dev)].contiguous()
        self.nnz = int(idx.shape[0])
        # the values go over in their own type when it is the working one
        # (float32 -> float64 -> float32 is exact, so the result is the same)
        dv = np.asarray(data)
        if not ((dv.dtype == np.float32 and dtype == torch.float32) or
                (dv.dtype == np.float64 and dtype == torch.float64)):
            dv = np.asarray(dv, dtype=np.float64)
        self.vals = torch.as_tensor(np.ascontiguousarray(dv), device=dev).to(dtype).contiguous()
        self.idx32 = torch.empty((self.L, max(self.nnz, 1)), dtype=torch.int32, device=dev)
        err = torch.zeros(1, dtype=torch.int32, device=dev)
        _lib.call("tfx_coo_encode", _vp(idx), self.nnz, self.L, _cint(dims), _vp(self.idx32), _vp(err), _st())
        if int(err.item()) != 0:
            raise ValueError("sparse index out of range")
        self.sorted = {}

    def dt(self):
        return _lib.F64 if self.vals.dtype == torch.float64 else _lib.F32

    def sort_mode(self, mode):
        """(rowptr, sorted int32 SoA coordinates, sorted values) for ``mode``."""
        if mode not in self.sorted:
            d = self.dims[mode]
            dev = self.vals.device
            counts = torch.empty(2 * d, dtype=torch.int32, device=dev)
            rowptr = torch.empty(d + 1, dtype=torch.int64, device=dev)
            sidx = torch.empty_like(self.idx32)
            svals = torch.empty_like(self.vals)
            _lib.call("tfx_coo_sort_mode", self.dt(), _vp(self.idx32), _vp(self.vals), self.nnz, self.L,
                      _cint(self.dims), int(mode), _vp(counts), _vp(rowptr), _vp(sidx), _vp(svals), _st())
            self.sorted[mode] = (rowptr, sidx, svals)
        return self.sorted[mode]

    def gram(self, mode):
        """Dense T_(l) T_(l)^T (d_l x d_l) on the device."""
        if self.nnz >= 2 ** 31:
            raise ValueError("the sparse Gram takes fewer than 2^31 stored entries")
        rowptr, sidx, svals = self.sort_mode(mode)
        d = self.dims[mode]
        lib = _lib.load()
        nb = int(lib.tfx_coo_gram_scratch_bytes(self.nnz, d))
        scratch = torch.empty(nb, dtype=torch.uint8, device=self.vals.device)
        G = torch.empty((d, d), dtype=self.vals.dtype, device=self.vals.device)
        err = torch.zeros(1, dtype=torch.int32, device=self.vals.device)
        _lib.call("tfx_coo_gram", self.dt(), _vp(self.idx32), _vp(self.vals), self.nnz, _vp(svals), _vp(rowptr),
                  self.L, _cint(self.dims), int(mode), _vp(G), _vp(scratch), nb, _vp(err), _st())
        if int(err.item()) != 0:
            raise RuntimeError("fibre hash table overflow in the sparse Gram")
        return G


def _row_major_ptrs(factors_rm):
    arr = torch.tensor([_dev.ptr(w) for w in factors_rm], dtype=torch.int64, device=factors_rm[0].device)
    return arr


def coo_mttkrp(X, factors_rm, mode):
    """Sparse MTTKRP ``T_(l) (KR of the other factors)`` as a (d_l, R) row-major tensor.

    ``factors_rm`` are the (d_m, R) row-major device factor matrices."""
    rowptr, sidx, svals = X.sort_mode(mode)
    R = int(factors_rm[0].shape[1])
    out = torch.empty((X.dims[mode], R), dtype=X.vals.dtype, device=X.vals.device)
    ptrs = _row_major_ptrs(factors_rm)
    _lib.call("tfx_coo_mttkrp", X.dt(), _vp(sidx), _vp(svals), X.nnz, _vp(rowptr), X.L, _cint(X.dims), R, int(mode),
              _vp(ptrs), _vp(out), _st())
    return out


def sparse_residual_sq(X, factors_rm):
    """sum over stored entries of (value - model)^2 (float64 device scalar)."""
    R = int(factors_rm[0].shape[1])
    lib = _lib.load()
    scratch = torch.empty(int(lib.tfx_sparse_residual_scratch_bytes()), dtype=torch.uint8, device=X.vals.device)
    out = torch.empty(1, dtype=torch.float64, device=X.vals.device)
    ptrs = _row_major_ptrs(factors_rm)
    _lib.call("tfx_sparse_residual", X.dt(), _vp(X.idx32), _vp(X.vals), X.nnz, X.L, _cint(X.dims), R, _vp(ptrs),
              _vp(out), _vp(scratch), _st())
    return out


def sparse_ttmc(X, Uts):
    """Dense core S = T x_1 U_1^T ... from COO; Uts[l] is (n_l, d_l) row-major."""
    U_rm = [u.t().contiguous() for u in Uts]        # (d_l, n_l) row-major
    n = [int(u.shape[0]) for u in Uts]
    lib = _lib.load()
    nb = int(lib.tfx_sparse_ttmc_scratch_bytes(X.dt(), X.nnz, X.L, _cint(n)))
    scratch = torch.empty(max(nb, 16), dtype=torch.uint8, device=X.vals.device)
    S = torch.empty(n, dtype=X.vals.dtype, device=X.vals.device)
    ptrs = _row_major_ptrs(U_rm)
    _lib.call("tfx_sparse_ttmc", X.dt(), _vp(X.idx32), _vp(X.vals), X.nnz, X.L, _cint(X.dims), _cint(n), _vp(ptrs),
              _vp(S), _vp(scratch), nb, _st())
    return S


def mlsvd_sparse_device(X, R, options):
    """Reference sparse MLSVD (Compression.py:123-137, 211-222) on a DeviceCOO."""
    o = options
    L = X.L
    tol = o.tol_mlsvd
    if isinstance(tol, list):
        tol = tol[0] if L > 3 else tol[1]
    if tol < 0:
        tol = 1e-16
    Uts, sigmas = [], []
    for l in range(L):
        d = X.dims[l]
        low = min(R, d)
        n = o.svd_n_components if o.svd_n_components is not None else int(max(L, np.log10(d * d * L)) * low)
        omega = _draw_omega(d, n + 10)
        G = X.gram(l)
        Ut, lam = top_eig(G, n, omega)
        # the reference takes sqrt of the Gram's singular values (Compression.py:222)
        sig = np.sqrt(np.maximum(lam, 0.0))
        dim = clean_compression(sig, tol, L)
        Uts.append(Ut[:dim].contiguous())
        sigmas.append(sig[:dim])
    S = sparse_ttmc(X, Uts)
    return S, Uts, sigmas


def coo_provider(X, R):
    """MTTKRP provider of a DeviceCOO for ``mttkrp_dgn.dgn_mttkrp``: writes
    T_(l) KR_l (row-major) into the mode-l block of ``Mrm``."""
    dims = X.dims
    es = X.vals.element_size()
    offs = np.concatenate([[0], np.cumsum([R * d for d in dims])])
    cache = {}

    def provide(W, Wrm, Mrm, modes, low=False):
        if low and modes:
            # BF16 factor rows, per-column power-of-two scales, FP32 sums
            if 'bf' not in cache:
                cache['bf'] = torch.empty(W.numel(), dtype=torch.bfloat16, device=W.device)
                cache['scale'] = torch.empty(X.L * R, dtype=torch.float32, device=W.device)
                cache['bptrs'] = torch.tensor([cache['bf'].data_ptr() + int(offs[l]) * 2 for l in range(X.L)],
                                              dtype=torch.int64, device=W.device)
            _lib.call("tfx_factors_bf16", X.L, _cint(dims), int(R), _vp(W), _vp(cache['bf']), _vp(cache['scale']),
                      _st())
            for l in modes:
                rowptr, sidx, svals = X.sort_mode(l)
                _lib.call("tfx_coo_mttkrp_bf16", _vp(sidx), _vp(svals), X.nnz, _vp(rowptr), X.L, _cint(dims),
                          int(R), int(l), _vp(cache['bptrs']), _vp(cache['scale']),
                          ctypes.c_void_p(Mrm.data_ptr() + int(offs[l]) * es), _st())
            return
        key = Wrm.data_ptr()
        if cache.get('key') != key:
            cache['key'] = key
            cache['ptrs'] = torch.tensor([key + int(offs[l]) * es for l in range(X.L)], dtype=torch.int64,
                                         device=Wrm.device)
        for l in modes:
            rowptr, sidx, svals = X.sort_mode(l)
            _lib.call("tfx_coo_mttkrp", X.dt(), _vp(sidx), _vp(svals), X.nnz, _vp(rowptr), X.L, _cint(dims), int(R),
                      int(l), _vp(cache['ptrs']), ctypes.c_void_p(Mrm.data_ptr() + int(offs[l]) * es), _st())
    return provide


def tricpd_sparse_direct(X, data, R, o, prec, ordering, sdims, Tsize):
    """dGN on the COO tensor itself (``options.sparse_solver = 'direct'``): no
    compression; the start is drawn in the full space like the reference's
    random start, the gradient and error come from COO MTTKRPs
    (``mttkrp_dgn.dgn_mttkrp``).  The objective is the reference's (absent
    entries are zeros of the data)."""
    from .api import starting_point_random
    from .mttkrp_dgn import dgn_mttkrp
    dt = X.vals.dtype
    dims = [int(d) for d in sdims]
    if isinstance(o.initialization, list):
        init = [np.asarray(o.initialization[ordering[l]], dtype=np.float64) for l in range(len(dims))]
    elif o.initialization == 'random':
        init = starting_point_random(dims, R, o)
    else:
        raise NotImplementedError("sparse_solver='direct' takes a 'random' or given start")
    x0 = torch.from_numpy(_dev.flat_factors(init)).to(device=X.vals.device, dtype=dt)
    nrm = kernels.tensor_norms(X.vals).cpu().numpy()
    meanabs = float(nrm[1]) / float(np.prod(np.array(dims, dtype=np.float64)))
    # precision 'mixed': BF16 gathers while the error falls fast, then FP32
    ladder = o.precision == 'mixed' and dt == torch.float32 and R in (8, 16, 32, 64)
    return dgn_mttkrp(coo_provider(X, R), dims, R, x0, o, prec, float(nrm[0]), meanabs, ladder=ladder)


def tricpd_sparse(T, R, options):
    """``tricpd`` for ``[data, idxs, dims]`` (TensorFox.py:424-655, sparse branches)."""
    from .api import Output, starting_point_core, _decompress, _run_dgn, _run_als, unsort_dims
    o = options
    if o.method not in ('dGN', 'als'):
        raise NotImplementedError("method %r is outside the damped Gauss-Newton and ALS paths" % (o.method,))
    data, idxs, dims = T
    data_in = np.asarray(data)
    in_f32 = data_in.dtype == np.float32
    data = np.asarray(data, dtype=np.float64)
    idxs = np.asarray(idxs, dtype=np.int64).reshape(len(data), -1)
    dims = np.asarray(dims)
    # the input's own precision unless the options name one ('mixed' computes in FP32)
    if o.precision in ('fp64', 'fp32'):
        prec = o.precision
    elif o.precision == 'mixed' or in_f32:
        prec = 'fp32'
    else:
        prec = 'fp64'
    dt = _dev.torch_dtype(prec)
    ordering = np.argsort(-dims)
    sdims = dims[ordering]
    X = DeviceCOO(data_in, idxs, sdims, dt, perm=ordering)
    Tsize = float(np.linalg.norm(data))
    if getattr(o, 'sparse_solver', None) == 'direct':
        if o.method != 'dGN':
            raise NotImplementedError("sparse_solver='direct' runs method 'dGN'")
        best, ss, er, im, gr, st, _ = tricpd_sparse_direct(X, data, R, o, prec, ordering, sdims, Tsize)
        factors = _dev.unflat(best.double().cpu().numpy(), [int(d) for d in sdims], R)
        return _sparse_output(X, factors, ordering, Tsize, ss, er, im, gr, st, o)
    S, Uts, sigmas = mlsvd_sparse_device(X, R, o)
    core = [int(u.shape[0]) for u in Uts]
    if isinstance(o.initialization, list):
        init = []
        for l in range(len(core)):
            W = torch.from_numpy(np.asarray(o.initialization[ordering[l]], dtype=np.float64)).to(S.device, dt)
            init.append(kernels.matmul(Uts[l], W).double().cpu().numpy())
    else:
        init = starting_point_core(S, core, R, o)
    x0 = torch.from_numpy(_dev.flat_factors(init)).to(device=S.device, dtype=dt)
    if o.method == 'als':
        best, ss, er, im, gr, st = _run_als(S, x0, R, o, prec)
    else:
        alias = bool(o.symm) and float(o.factors_norm) <= 0 and not isinstance(o.initialization, list)
        best, ss, er, im, gr, st = _run_dgn(S, x0, R, o, prec, aliased=alias)
    Wf = _decompress(Uts, best, core, R)
    factors = _dev.unflat(Wf.double().cpu().numpy(), [int(d) for d in sdims], R)
    return _sparse_output(X, factors, ordering, Tsize, ss, er, im, gr, st, o)


def _sparse_output(X, factors, ordering, Tsize, ss, er, im, gr, st, o):
    """Final error on the stored entries (Auxiliar.py:155-159) and the output
    object; ``factors`` in the sorted mode order."""
    from .api import Output, unsort_dims
    dt = X.vals.dtype
    frm = [torch.from_numpy(np.ascontiguousarray(f)).to(X.vals.device, dt) for f in factors]
    res = float(sparse_residual_sq(X, frm).cpu().numpy()[0])
    factors = unsort_dims(factors, ordering)
    out = Output()
    out.num_steps = len(ss)
    out.rel_error = float(np.sqrt(res)) / Tsize
    out.accuracy = max(0, 100 * (1 - out.rel_error))
    out.step_sizes = [ss, np.array([0])]
    out.errors = [er, np.array([0])]
    out.improv = [im, np.array([0])]
    out.gradients = [gr, np.array([0])]
    out.stop = [st, 8]
    out.options = o
    return factors, out
