"""Alternating least squares on the device (Alternating_Least_Squares.py:18-235).

``als(T, factors, R, options)`` keeps the reference's signature and return tuple
``(factors, step_sizes, errors, improv, gradients, stop)``; like the reference it
returns the LAST iterate.  The solve is one call of ``tfx_als_solve``: a CUDA
graph whose while-node runs one ALS iteration per pass (per mode the MTTKRP
``T_(l) KR_l``, the R x R inverse of ``o_{m != l} G_m`` and the factor update)
until the reference's stop tests fire on the device.
"""
import ctypes

import torch

from . import _dev, _lib
from .options import make_options


def _opts_struct(o):
    s = _lib.DgnOptions()
    s.maxiter = int(o.maxiter)
    s.tol, s.tol_step, s.tol_improv, s.tol_grad = float(o.tol), float(o.tol_step), float(o.tol_improv), float(o.tol_grad)
    s.tol_jump, s.cg_tol, s.init_damp, s.use_damp_sched = 0.0, 0.0, 0.0, 0
    s.symm = 1 if o.symm else 0
    s.factors_norm = float(o.factors_norm)
    return s


def als_device(Td, x0, R, options, precision, fix_mode=-1):
    """ALS on device-resident inputs.  ``x0`` (flat layout) is not modified;
    ``fix_mode`` >= 0 keeps that factor as given (bicpd).
    Returns ``(x_last, best, stats, result, info)``: device vectors and NumPy
    arrays (stats = errors | step sizes | improvements | gradients)."""
    lib = _lib.load()
    o = options
    dims = [int(d) for d in Td.shape]
    L = len(dims)
    cd = (ctypes.c_int * L)(*dims)
    dt = _dev.lib_dtype(precision)
    nb = int(lib.tfx_als_workspace_bytes(dt, L, cd, int(R)))
    work = torch.empty(nb + 256, dtype=torch.uint8, device=Td.device)
    base = (work.data_ptr() + 255) // 256 * 256
    x = x0.clone()
    best = torch.empty_like(x)
    m = int(o.maxiter)
    stats = torch.zeros(4 * m, dtype=torch.float64, device=Td.device)
    result = torch.zeros(4, dtype=torch.int32, device=Td.device)
    info = torch.zeros(8, dtype=torch.float64, device=Td.device)
    opt = _opts_struct(o)
    _lib.check(lib.tfx_als_solve(dt, ctypes.c_void_p(_dev.ptr(Td)), L, cd, int(R), ctypes.c_void_p(_dev.ptr(x)),
                                 ctypes.c_void_p(_dev.ptr(best)), ctypes.c_void_p(_dev.ptr(stats)),
                                 ctypes.c_void_p(_dev.ptr(result)), ctypes.c_void_p(_dev.ptr(info)),
                                 ctypes.byref(opt), int(fix_mode), ctypes.c_void_p(base), nb,
                                 ctypes.c_void_p(_dev.stream())))
    res = result.cpu().numpy()
    _lib.check_solve_status(res)
    return x, best, stats.cpu().numpy(), res, info.cpu().numpy()


def split_stats(stats, maxiter, n):
    """(step_sizes, errors, improv, gradients) of the first ``n`` iterations."""
    m = maxiter
    return (stats[m:m + n].copy(), stats[:n].copy(), stats[2 * m:2 * m + n].copy(), stats[3 * m:3 * m + n].copy())


def als(T, factors, R, options=None, precision=None):
    """Drop-in for Alternating_Least_Squares.als: ``(factors, step_sizes, errors,
    improv, gradients, stop)`` with NumPy float64 arrays; ``factors`` is the
    last iterate."""
    _dev.require_cuda()
    from .gauss_newton import _precision_of
    options = make_options(options) if not hasattr(options, 'bi_method_parameters') else options
    if precision is not None:
        options.precision = precision
    prec = _precision_of(T, options)
    dt = _dev.torch_dtype(prec)
    Td = _dev.to_device(T, dt)
    dims = tuple(int(d) for d in Td.shape)
    factors = list(factors)
    fix = -1
    for l in range(len(factors)):        # [W, l] marks a fixed factor, as in the reference
        if isinstance(factors[l], list):
            fix, factors[l] = l, factors[l][0]
    x0 = torch.from_numpy(_dev.flat_factors(factors)).to(device=Td.device, dtype=dt)
    x, best, stats, res, info = als_device(Td, x0, R, options, prec, fix)
    n = int(res[1])
    ss, er, im, gr = split_stats(stats, int(options.maxiter), n)
    f = _dev.unflat(x.double().cpu().numpy(), dims, R)
    return f, ss, er, im, gr, int(res[0])
