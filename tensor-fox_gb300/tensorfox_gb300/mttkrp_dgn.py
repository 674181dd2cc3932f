"""Damped Gauss-Newton driven by MTTKRPs (GaussNewton.py:29-251, 315-398,
472-517, 713-795), for tensors the persistent engine does not hold.

The dGN iteration touches the tensor in two places only: the gradient
``g_l = W_l P1_l - T_(l) KR_l`` and the error.  With the reference's objective
(for a COO tensor, absent entries are zeros of the data)

    ||T - [[W]]||^2 = ||T||^2 - 2 <W_0, T_(0) KR_0> + sum_{a,b} prod_l G_l[a, b],

so both come from the MTTKRPs ``T_(l) KR_l``; the CG inner solve needs the
factors' Gramians only.  ``dgn_mttkrp`` runs the reference's loop with a
caller's MTTKRP provider, one host step per iteration:

1. the provider's MTTKRPs at the current factors (mode 0 is kept from the
   previous error evaluation);
2. ``tfx_coo_dgn_cg``: Gramians, regularisation, preconditioner, gradient,
   J^T J grad and the preconditioned CG as one cooperative launch;
3. ``tfx_step_update_wide``: x += y and column balancing over the whole
   grid (``tfx_dgn_step_update``, one CTA, above rank 64);
4. the mode-0 MTTKRP at the new factors and ``tfx_coo_model_error``;
5. the host reads the iteration's scalars once and applies the gain ratio,
   damping, best-iterate and stop rules (shared with the stepped loop); after
   a jump it runs the reference's dogleg trials (``tfx_dogleg_dots`` /
   ``tfx_dogleg_trial``, each trial's error from a mode-0 MTTKRP).

The 'cg' caps are drawn like the engine draws them (a copy of NumPy's RNG
state), and the RNG is advanced by the draws the reference makes.
"""
import ctypes

import numpy as np
import torch

from . import _dev, _lib
from .gauss_newton import cg_budgets, advance_rng, _inner_of
from .stepped import _gain_ratio, _update_damp, _stop_code


def _vp(t):
    return ctypes.c_void_p(_dev.ptr(t) if t is not None else None)


def _cint(vals):
    vals = [int(v) for v in vals]
    return (ctypes.c_int * len(vals))(*vals)


class _Aligned:
    def __init__(self, nbytes, dev):
        self.buf = torch.empty(int(nbytes) + 256, dtype=torch.uint8, device=dev)
        self.ptr = (self.buf.data_ptr() + 255) // 256 * 256
        self.nbytes = int(nbytes)


def dgn_mttkrp(provider, dims, R, x0, options, precision, tnorm2, meanabs, error_fn=None, ladder=False):
    """dGN from the flat start ``x0`` (device, working precision).

    ``provider(W, Wrm, Mrm, modes)`` writes ``T_(l) KR_l`` for every l in
    ``modes`` into the row-major block of ``Mrm`` at offset R*sum(dims[:l]),
    from the factors (flat ``W``, or their row-major copy ``Wrm`` at the same
    offsets).  ``tnorm2`` = ||T||^2, ``meanabs`` = mean |T| over every entry of
    the tensor (absent ones included).  ``error_fn(W, out)``, when given,
    writes ||T - [[W]]||^2 (a device double at address ``out``) instead of the
    MTTKRP identity -- a dense tensor's direct residual keeps the error's
    precision where the identity would cancel.  ``ladder``: start with the
    provider's low-precision MTTKRPs (``provider(..., low=True)``: BF16 factor
    rows with per-column scales for a COO tensor) and switch to the working
    precision for good at the first iteration that lowers the error by less
    than 1% -- far from the solution the cheap gradient steers as well, near
    it every digit counts.  Returns ``(best, step_sizes, errors, improv,
    gradients, stop, matvecs)`` with ``best`` a device vector; the number of
    low-precision iterations is ``dgn_mttkrp.low_iterations``."""
    o = options
    lib = _lib.load()
    L = len(dims)
    n = R * sum(dims)
    cd = _cint(dims)
    dt = _dev.lib_dtype(precision)
    dev = x0.device
    st = ctypes.c_void_p(_dev.stream())
    if o.symm or float(o.factors_norm) > 0:
        raise NotImplementedError("the MTTKRP-driven dGN runs without symm / factors_norm")
    kinds = {_inner_of(o, it) for it in range(int(o.maxiter))}
    if not kinds <= {'cg', 'cg_static'}:
        raise NotImplementedError("the MTTKRP-driven dGN runs the 'cg' and 'cg_static' inner methods")
    maxiter = int(o.maxiter)
    budgets = cg_budgets(o, L)
    x = x0.clone()
    W = x0.clone()
    best = W.clone()
    x_prev = torch.empty_like(x0)
    xa, xb = torch.empty_like(x0), torch.empty_like(x0)
    Wrm = torch.empty_like(x0)
    Mrm = torch.empty_like(x0)
    f64 = dict(dtype=torch.float64, device=dev)
    y, grad, jtj = torch.zeros(n, **f64), torch.zeros(n, **f64), torch.zeros(n, **f64)
    bY = torch.zeros(n, **f64)
    scal = torch.zeros(32, **f64)          # [0:3] CG, [4:8] step, [8:11] error, [12:15] dots, [16:18] trial
    cgw = _Aligned(lib.tfx_coo_dgn_cg_workspace_bytes(dt, L, cd, int(R)), dev)
    errw = torch.empty(int(lib.tfx_coo_model_error_scratch_bytes(L, int(R))), dtype=torch.uint8, device=dev)
    dgw = torch.empty(int(lib.tfx_dogleg_scratch_bytes()), dtype=torch.uint8, device=dev)
    # the whole-grid step update (rank <= 64); the one-CTA one otherwise
    wide = R <= 64
    upw = torch.empty(int(lib.tfx_step_update_wide_scratch_bytes(L, cd, int(R))) if wide else 1,
                      dtype=torch.uint8, device=dev)
    sp = scal.data_ptr()

    def rows(src):
        _lib.call("tfx_factors_to_rows", dt, L, cd, int(R), _vp(src), _vp(Wrm), st)

    low = bool(ladder)
    n_low = 0

    def model_error(Wsrc):
        if error_fn is not None:
            error_fn(Wsrc, sp + 8 * 8)
            return
        rows(Wsrc)
        provider(Wsrc, Wrm, Mrm, [0], low=low)
        _lib.call("tfx_coo_model_error", dt, L, cd, int(R), _vp(Wsrc), _vp(Mrm), float(tnorm2),
                  ctypes.c_void_p(sp + 8 * 8), _vp(errw), int(errw.numel()), st)

    Tsize = float(np.sqrt(tnorm2))
    init_damp = o.init_damp
    damp = float(init_damp[0]) if isinstance(init_damp, list) else float(init_damp) * float(meanabs)
    tol, tol_step, tol_improv, tol_grad = o.tol, o.tol_step, o.tol_improv, o.tol_grad
    if n <= 100:                     # GaussNewton.py:117-121
        tol = tol_step = tol_improv = tol_grad = 0
    const = 1 + int(maxiter / 10)
    errors, step_sizes = np.zeros(maxiter), np.zeros(maxiter)
    improv, gradients = np.zeros(maxiter), np.zeros(maxiter)
    error, best_error, stop = 1.0, np.inf, 5
    m0_valid = False
    matvecs = 0
    it = 0
    for it in range(maxiter):
        old_error = error
        rows(W)
        provider(W, Wrm, Mrm, list(range(1 if m0_valid else 0, L)), low=low)
        _lib.call("tfx_coo_dgn_cg", dt, L, cd, int(R), _vp(W), _vp(Mrm), ctypes.c_double(damp),
                  int(budgets[it]), ctypes.c_double(float(o.cg_tol)), _vp(y), _vp(grad), _vp(jtj),
                  ctypes.c_void_p(sp), ctypes.c_void_p(cgw.ptr), cgw.nbytes, st)
        x_prev.copy_(x)
        if wide:
            _lib.call("tfx_step_update_wide", dt, L, cd, int(R), _vp(x), _vp(W), _vp(y), _vp(grad),
                      ctypes.c_double(damp), ctypes.c_void_p(sp + 4 * 8), _vp(upw), int(upw.numel()), st)
        else:
            _lib.call("tfx_dgn_step_update", dt, L, cd, int(R), _vp(x), _vp(W), _vp(y), _vp(grad),
                      ctypes.c_double(damp), 0, 0, ctypes.c_double(0.0), 0, -1, None,
                      ctypes.c_void_p(sp + 4 * 8), st)
        model_error(W)
        s = scal.cpu().numpy()
        if int(s[2]) != 0:
            raise _lib.TfxError("MTTKRP dGN: a bounded grid barrier of the CG ran out")
        matvecs += int(s[0])
        error = float(np.sqrt(max(s[8], 0.0))) / Tsize
        den, ss2, xo2, gmax = float(s[6]), float(s[4]), float(s[5]), float(s[7])
        m0_valid = error_fn is None
        if it > 3 and error > o.tol_jump * old_error:
            error = _dogleg(lib, dt, n, x, y, grad, jtj, W, bY, xa, xb, error, damp, Tsize, model_error,
                            scal, dgw, st)
            m0_valid = False
            _lib.call("tfx_step_sums", dt, n, _vp(x), _vp(x_prev), _vp(grad), ctypes.c_double(damp),
                      ctypes.c_void_p(sp + 12 * 8), _vp(dgw), st)
            s = scal.cpu().numpy()
            den, ss2, xo2, gmax = float(s[12]), float(s[13]), float(s[14]), float(s[15])
        if low:
            n_low += 1
            if old_error - error < 1e-2 * old_error:
                low = False
                m0_valid = False     # the kept mode-0 MTTKRP is a low-precision one
        gain = _gain_ratio(damp, old_error, error, Tsize, den)
        damp = _update_damp(damp, init_damp, gain, it)
        if error < best_error:
            best_error = error
            best.copy_(W)
        errors[it] = error
        step_sizes[it] = np.sqrt(ss2) / np.sqrt(xo2)
        gradients[it] = gmax
        improv[it] = errors[it] if it == 0 else abs(errors[it] - errors[it - 1])
        code = _stop_code(it, errors, step_sizes, improv, gradients, error, Tsize, tol, tol_step, tol_improv,
                          tol_grad, const)
        if code is not None:
            stop = code
            break
    k = it + 1
    advance_rng(o, k)
    dgn_mttkrp.low_iterations = n_low
    return best, step_sizes[:k].copy(), errors[:k].copy(), improv[:k].copy(), gradients[:k].copy(), stop, matvecs


def _dogleg(lib, dt, n, x, y, grad, jtj, W, bY, xa, xb, error, damp, Tsize, model_error, scal, dgw, st):
    """The reference's dogleg trials after a rejected step (GaussNewton.py:713-795):
    on entry ``x`` = x_old + y and ``W`` the rejected factors; on exit ``x``,
    ``y`` and ``W`` hold the best trial (or the reverted point and the rejected
    factors when no trial improves).  Returns the best error."""
    sp = scal.data_ptr()
    _lib.call("tfx_step_revert", dt, n, _vp(x), _vp(y), _vp(xa), st)
    bX, bW = xa.clone(), W.clone()
    bY.copy_(y)
    best_error = error
    _lib.call("tfx_dogleg_dots", n, _vp(grad), _vp(grad), _vp(grad), _vp(jtj), _vp(y), _vp(y),
              ctypes.c_void_p(sp + 12 * 8), _vp(dgw), st)
    s = scal.cpu().numpy()
    g2, gj = float(s[12]), float(s[13])
    alpha = g2 / gj
    gnorm = np.sqrt(g2)
    gain, delta, count = 1.0, 1.0, 0
    xc, xn = xa, xb
    while gain > 0:
        old_error = error
        _lib.call("tfx_dogleg_dots", n, _vp(y), _vp(y), _vp(y), _vp(grad), _vp(grad), _vp(grad),
                  ctypes.c_void_p(sp + 12 * 8), _vp(dgw), st)
        s = scal.cpu().numpy()
        yy, yg = float(s[12]), float(s[13])
        c1 = abs(alpha) * gnorm
        c2 = alpha * yg - alpha * alpha * g2
        c3 = yy - 2 * alpha * yg + alpha * alpha * g2
        c4 = delta ** 2 - c1 ** 2
        m = c2 ** 2 + c3 * c4
        if np.sqrt(yy) < delta:
            ca, cb = 1.0, 0.0
        elif c1 >= delta:
            ca, cb = 0.0, (delta / c1) * alpha
        elif m < 0:
            ca, cb = 1.0, 0.0
        else:
            c5 = np.sqrt(m)
            coef = (-c2 + c5) / c3 if c2 <= 0 else c4 / (c2 + c5)
            ca, cb = coef, (1.0 - coef) * alpha
        _lib.call("tfx_dogleg_trial", dt, n, _vp(xc), _vp(y), _vp(grad), ctypes.c_double(ca), ctypes.c_double(cb),
                  ctypes.c_double(damp), _vp(xn), _vp(W), ctypes.c_void_p(sp + 16 * 8), _vp(dgw), st)
        model_error(W)
        s = scal.cpu().numpy()
        error = float(np.sqrt(max(s[8], 0.0))) / Tsize
        gain = _gain_ratio(damp, old_error, error, Tsize, float(s[16]))
        if error < old_error:
            bX.copy_(xn)
            bY.copy_(y)
            bW.copy_(W)
            best_error = error
        step = np.sqrt(float(s[17]))
        if gain > 0.75:
            delta = max(delta, 2 * step)
        else:
            sigma = 0.25 / (1 + np.exp(-14 * (gain - 0.75))) + 0.75
            delta = min(sigma * delta, delta)
        count += 1
        if count > 10:
            break
        xc, xn = xn, xc
    x.copy_(bX)
    y.copy_(bY)
    W.copy_(bW)
    return best_error


def dense_provider(Td, dims, R):
    """MTTKRP provider of a dense FP32 tensor on the tensor cores
    (``tfx_mttkrp_tc``); the last mode reads a copy of the tensor with that
    mode moved first, made once."""
    from . import kernels
    dims = [int(d) for d in dims]
    L = len(dims)
    offs = np.concatenate([[0], np.cumsum([R * d for d in dims])])
    state = {}

    def provide(W, Wrm, Mrm, modes, low=False):
        for l in modes:
            if l == L - 1 and 'last' not in state:
                state['last'] = kernels.last_mode_first(Td, dims)
            blk = Mrm[int(offs[l]):int(offs[l + 1])].view(dims[l], R)
            _, err = kernels.mttkrp_tc(Td, dims, W, R, l, T_last=state.get('last'), out=blk)
            state.setdefault('errs', []).append(err)
    return provide


def dense_supported(Td, R, options, precision):
    """The tensor-core MTTKRP path applies to this full-tensor dGN run."""
    from . import kernels
    dims = [int(d) for d in Td.shape]
    if precision != 'fp32' or Td.dtype != torch.float32 or len(dims) < 3 or R > 64:
        return False
    if options.symm or float(options.factors_norm) > 0 or isinstance(options.init_damp, list):
        return False
    if not {_inner_of(options, it) for it in range(int(options.maxiter))} <= {'cg', 'cg_static'}:
        return False
    return all(kernels.mttkrp_tc_supported(Td, dims, R, l) for l in range(len(dims)))


def dgn_dense(Td, x0, R, options):
    """dGN on a large dense FP32 tensor (the refinement on the full tensor,
    TensorFox.py:583-604, or a run without compression): gradients from the
    tensor-core MTTKRP, the error from the direct residual (``tfx_cp_residual``),
    CG on the Gramians.  Same return values as ``dgn_mttkrp``."""
    from . import kernels
    dims = [int(d) for d in Td.shape]
    nrm = kernels.tensor_norms(Td).cpu().numpy()
    lib = _lib.load()
    scratch = torch.empty(int(lib.tfx_cp_residual_scratch_bytes()), dtype=torch.uint8, device=Td.device)
    cd = _cint(dims)
    L = len(dims)

    def error_fn(W, out_addr):
        _lib.call("tfx_cp_residual", _lib.F32, _vp(Td), L, cd, int(R), _vp(W), ctypes.c_void_p(out_addr),
                  _vp(scratch), ctypes.c_void_p(_dev.stream()))
    return dgn_mttkrp(dense_provider(Td, dims, R), dims, R, x0, options, 'fp32', float(nrm[0]),
                      float(nrm[1]) / Td.numel(), error_fn=error_fn)
