"""Differentiable CP layer (torch.autograd.Function) on the GB300 kernels.

* ``cp_reconstruct(factors)`` returns the dense tensor [[W_0, ..., W_{L-1}]]
  (Conversion.py:52-79 ``cpd2tens``); its backward for an incoming gradient G is
  ``dL/dW_l = MTTKRP(G, l)`` computed by ``tfx_mttkrp``.
* ``cp_fit_loss(T, factors)`` returns ``||[[W]] - T||^2`` (fused residual, the
  model is never materialised); its backward is
  ``2 (W_l P1_l - MTTKRP(T, l))`` -- twice the gradient ``g`` of
  GaussNewton.py:401-427 -- and ``2 (T - [[W]])`` for ``T`` when requested.

Both recompute the Khatri-Rao rows inside the kernels instead of storing them.
Factors are CUDA tensors of shape (d_l, R), float32 or float64.
"""
import ctypes

import torch

from . import _dev, _lib


def _vp(t):
    return ctypes.c_void_p(_dev.ptr(t))


def _st():
    return ctypes.c_void_p(_dev.stream())


def _dt(t):
    return _lib.F64 if t.dtype == torch.float64 else _lib.F32


def _cint(v):
    return (ctypes.c_int * len(v))(*[int(a) for a in v])


def _flat(factors):
    return torch.cat([W.detach().t().contiguous().reshape(-1) for W in factors])


_DECLARED = None


def _declare():
    global _DECLARED
    if _DECLARED is not None:
        return _DECLARED
    lib = _lib.load()
    P, I, SZ = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
    lib.tfx_mttkrp.argtypes = [I, P, I, ctypes.POINTER(ctypes.c_int), I, P, I, P, P, SZ, P]
    lib.tfx_mttkrp_scratch_bytes.restype = SZ
    lib.tfx_mttkrp_scratch_bytes.argtypes = [I, I, ctypes.POINTER(ctypes.c_int), I, I]
    lib.tfx_cp_full.argtypes = [I, I, ctypes.POINTER(ctypes.c_int), I, P, P, P]
    lib.tfx_cp_wp1.argtypes = [I, I, ctypes.POINTER(ctypes.c_int), I, P, P, P, P]
    lib.tfx_cp_wp1_scratch_bytes.restype = SZ
    lib.tfx_cp_wp1_scratch_bytes.argtypes = [I, I]
    lib.tfx_cp_fit_grad.argtypes = [I, P, I, ctypes.POINTER(ctypes.c_int), I, P, P, P, SZ, P]
    lib.tfx_cp_fit_grad_scratch_bytes.restype = SZ
    lib.tfx_cp_fit_grad_scratch_bytes.argtypes = [I, I, ctypes.POINTER(ctypes.c_int), I]
    _DECLARED = lib
    return lib


def mttkrp(T, factors, mode):
    """T_(l) times the Khatri-Rao product of the other factors, as (d_l, R)."""
    lib = _declare()
    T = T.contiguous()
    dims = list(T.shape)
    R = int(factors[0].shape[1])
    W = _flat(factors).to(T.dtype)
    nb = int(lib.tfx_mttkrp_scratch_bytes(_dt(T), len(dims), _cint(dims), R, int(mode)))
    scratch = torch.empty(max(nb, 16), dtype=torch.uint8, device=T.device)
    out = torch.empty((R, dims[mode]), dtype=T.dtype, device=T.device)
    _lib.check(lib.tfx_mttkrp(_dt(T), _vp(T), len(dims), _cint(dims), R, _vp(W), int(mode), _vp(out), _vp(scratch),
                              nb, _st()))
    return out.t()


def cp_full(factors):
    lib = _declare()
    dims = [int(W.shape[0]) for W in factors]
    R = int(factors[0].shape[1])
    W = _flat(factors)
    out = torch.empty(dims, dtype=W.dtype, device=W.device)
    _lib.check(lib.tfx_cp_full(_dt(W), len(dims), _cint(dims), R, _vp(W), _vp(out), _st()))
    return out


def _wp1(factors):
    lib = _declare()
    dims = [int(W.shape[0]) for W in factors]
    R = int(factors[0].shape[1])
    W = _flat(factors)
    out = torch.empty_like(W)
    scratch = torch.empty(int(lib.tfx_cp_wp1_scratch_bytes(len(dims), R)), dtype=torch.uint8, device=W.device)
    _lib.check(lib.tfx_cp_wp1(_dt(W), len(dims), _cint(dims), R, _vp(W), _vp(out), _vp(scratch), _st()))
    res, s = [], 0
    for d in dims:
        res.append(out[s:s + d * R].view(R, d).t())
        s += d * R
    return res


class CPReconstruct(torch.autograd.Function):
    @staticmethod
    def forward(ctx, *factors):
        ctx.save_for_backward(*factors)
        return cp_full(factors)

    @staticmethod
    def backward(ctx, G):
        factors = ctx.saved_tensors
        G = G.contiguous().to(factors[0].dtype)
        return tuple(mttkrp(G, factors, l) if ctx.needs_input_grad[l] else None for l in range(len(factors)))


def fit_grad(T, W_flat, dims, R):
    """Flat gradient of ||T - [[W]]||^2: 2 (W_l P1_l - MTTKRP(T, l)) per mode
    (one ``tfx_cp_fit_grad`` call)."""
    lib = _declare()
    cd = _cint(dims)
    nb = int(lib.tfx_cp_fit_grad_scratch_bytes(_dt(T), len(dims), cd, R))
    scratch = torch.empty(nb, dtype=torch.uint8, device=T.device)
    out = torch.empty_like(W_flat)
    _lib.check(lib.tfx_cp_fit_grad(_dt(T), _vp(T), len(dims), cd, R, _vp(W_flat), _vp(out), _vp(scratch), nb, _st()))
    return out


class CPFitLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, T, *factors):
        from .kernels import cp_residual_sq
        T = T.contiguous()
        R = int(factors[0].shape[1])
        W_flat = _flat(factors).to(T.dtype)
        ctx.save_for_backward(T, W_flat, *factors)
        return cp_residual_sq(T, list(T.shape), W_flat, R)[0].to(T.dtype)

    @staticmethod
    def backward(ctx, gl):
        T, W_flat, *factors = ctx.saved_tensors
        dims = [int(W.shape[0]) for W in factors]
        R = int(factors[0].shape[1])
        grads = [None] * len(factors)
        if any(ctx.needs_input_grad[1:]):
            g = fit_grad(T, W_flat, dims, R).mul_(gl.to(T.dtype))
            s = 0
            for l, d in enumerate(dims):
                if ctx.needs_input_grad[l + 1]:
                    grads[l] = g[s:s + d * R].view(R, d).t().to(factors[l].dtype)
                s += d * R
        gT = 2.0 * gl * (T - cp_full(factors)) if ctx.needs_input_grad[0] else None
        return (gT, *grads)


def cp_reconstruct(factors):
    """Dense [[W_0, ..., W_{L-1}]] with an MTTKRP backward."""
    _dev.require_cuda()
    return CPReconstruct.apply(*factors)


def cp_fit_loss(T, factors):
    """||[[W]] - T||^2 with the Gauss-Newton gradient as backward."""
    _dev.require_cuda()
    return CPFitLoss.apply(T, *factors)
