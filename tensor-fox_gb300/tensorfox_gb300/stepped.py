"""dGN with the 'als' and 'direct' inner methods (GaussNewton.py:29-251, 254-312).

The persistent engine (``tfx_dgn_solve``) runs the 'cg' and 'cg_static' inner
methods.  The two others solve a different sub-problem per iteration and run
here, one iteration per host step, every array on the device:

* 'als' (GaussNewton.py:275-278): one ALS sweep of the factors
  (``tfx_als_sweep``), x = the swept factors, no step, gradient NaN;
* 'direct' (GaussNewton.py:630-653): the damped Gauss-Newton system formed
  explicitly and solved by LU (``tfx_dgn_direct_step``);

then ``tfx_dgn_step_update`` (x2cpd, balancing, transform, fixed factor, the
scalars of the step) and ``tfx_cp_residual`` (the error).  The host reads five
scalars per iteration and applies the reference's gain ratio, damping update,
best-iterate rule and stop tests.  Lists of inner methods may mix 'als' and
'direct'; mixing either with 'cg'/'cg_static' raises NotImplementedError.

The reference keeps the factors in a Python list that, after a symmetrising
``transform``, holds ONE array L times; its in-place ``x2cpd`` and
``transform`` then behave differently (the last block wins, the sum doubles).
That state is tracked here (``aliased``) and reproduced by the update kernel.
"""
import ctypes

import numpy as np
import torch

from . import _dev, _lib

STEPPED = ('als', 'direct')


def inner_kinds(options):
    """The set of inner methods of the run (a list of methods counts per entry
    over ``maxiter`` iterations)."""
    im = options.inner_method
    if isinstance(im, list):
        return set(im[:int(options.maxiter)])
    return {im}


def uses_stepped(options):
    """True when the run needs this module: every inner method is 'als' or
    'direct'.  A mix with the engine's methods is refused."""
    kinds = inner_kinds(options)
    if kinds <= set(STEPPED):
        return True
    if kinds & set(STEPPED):
        raise NotImplementedError("inner_method lists mixing %s with 'cg'/'cg_static' are not supported"
                                  % sorted(kinds & set(STEPPED)))
    return False


def _stop_code(it, errors, step_sizes, improv, gradients, error, Tsize, tol, tol_step, tol_improv, tol_grad,
               const):
    """The stop tests of GaussNewton.py:213-242; None to continue."""
    if it <= 1:
        return None
    if errors[it] < tol:
        return 0
    if step_sizes[it] < tol_step:
        return 1
    if improv[it] < tol_improv:
        return 2
    if gradients[it] < tol_grad:
        return 3
    if it > 2 * const and it % const == 0:
        mean1 = np.mean(errors[it - 2 * const: it - const])
        mean2 = np.mean(errors[it - const: it])
        if mean1 - mean2 <= tol_improv:
            return 4
        mean3 = np.mean(improv[it - const: it])
        if mean3 < 1e-3 * mean2:
            return 7
    if error > max(1, Tsize ** 2) / (1e-16 + tol):
        return 6
    return None


def _gain_ratio(damp, old_error, error, Tsize, den):
    """GaussNewton.py:472-487 with the denominator computed on the device."""
    num = (Tsize ** 2) * (old_error ** 2 - error ** 2)
    if den != 0.0:          # NaN (the 'als' step) takes this branch too
        return num / den
    if num != 0.0:
        return np.sign(num) * np.inf
    return -np.inf


def _update_damp(damp, init_damp, gain_ratio, it):
    """GaussNewton.py:490-503."""
    if isinstance(init_damp, list):
        return init_damp[it]
    if gain_ratio < 0.25:
        return 3 * damp
    if gain_ratio > 0.75:
        return damp / 3
    return damp


def dgn_stepped(Td, x0, R, options, precision, fix_mode=-1, aliased=False):
    """dGN on device-resident inputs for the 'als' / 'direct' inner methods.

    ``x0``: start point (flat layout, not modified); ``fix_mode`` >= 0 keeps
    that factor as given (third order, as bicpd uses it); ``aliased``: the
    caller's factor list holds one array L times.  Returns ``(best, step_sizes,
    errors, improv, gradients, stop)`` with ``best`` a device vector."""
    lib = _lib.load()
    o = options
    dims = [int(d) for d in Td.shape]
    L = len(dims)
    n = R * sum(dims)
    cd = (ctypes.c_int * L)(*dims)
    dt = _dev.lib_dtype(precision)
    dev = Td.device
    st = ctypes.c_void_p(_dev.stream())
    symm = bool(o.symm)
    fn = float(o.factors_norm)
    if fix_mode >= 0 and (L != 3 or symm or aliased):
        raise NotImplementedError("a fixed factor needs a third-order, non-symmetric problem")
    if (symm or aliased) and len(set(dims)) != 1:
        raise ValueError("symm needs equal dimensions")
    maxiter = int(o.maxiter)
    kinds = inner_kinds(o)

    def aligned(nbytes):
        buf = torch.empty(int(nbytes) + 256, dtype=torch.uint8, device=dev)
        return buf, (buf.data_ptr() + 255) // 256 * 256

    ws_als = ws_dir = None
    if 'als' in kinds:
        ws_als = aligned(lib.tfx_als_workspace_bytes(dt, L, cd, int(R)))
    if 'direct' in kinds:
        ws_dir = aligned(lib.tfx_dgn_direct_workspace_bytes(dt, L, cd, int(R)))
    res_scratch = torch.empty(int(lib.tfx_cp_residual_scratch_bytes()), dtype=torch.uint8, device=dev)

    x = x0.clone()
    W = x0.clone()
    Wfix = x0.clone() if fix_mode >= 0 else None
    best = W.clone()
    y = torch.zeros(n, dtype=torch.float64, device=dev)
    grad = torch.zeros(n, dtype=torch.float64, device=dev)
    out = torch.zeros(8, dtype=torch.float64, device=dev)
    _lib.check(lib.tfx_tensor_norms(dt, ctypes.c_void_p(_dev.ptr(Td)), int(Td.numel()),
                                    ctypes.c_void_p(_dev.ptr(out) + 48), ctypes.c_void_p(_dev.ptr(res_scratch)), st))
    tn = out.cpu().numpy()
    Tsize = float(np.sqrt(tn[6]))
    init_damp = o.init_damp
    damp = float(init_damp[0]) if isinstance(init_damp, list) else float(init_damp) * float(tn[7]) / Td.numel()
    tol, tol_step, tol_improv, tol_grad = o.tol, o.tol_step, o.tol_improv, o.tol_grad
    if R * sum(dims) <= 100:                     # GaussNewton.py:117-121
        tol = tol_step = tol_improv = tol_grad = 0
    const = 1 + int(maxiter / 10)
    errors, step_sizes = np.zeros(maxiter), np.zeros(maxiter)
    improv, gradients = np.zeros(maxiter), np.zeros(maxiter)
    error, best_error, stop = 1.0, np.inf, 5
    im = o.inner_method
    it = 0
    for it in range(maxiter):
        inner = im[it] if isinstance(im, list) else im
        old_error = error
        if inner == 'als':
            _lib.check(lib.tfx_als_sweep(dt, ctypes.c_void_p(_dev.ptr(Td)), L, cd, int(R),
                                         ctypes.c_void_p(_dev.ptr(W)), int(fix_mode), ctypes.c_void_p(ws_als[1]),
                                         int(ws_als[0].numel() - 256), st))
            from_W, yp, gp, alias_in = 1, None, None, 0   # the sweep gives every mode a new array
        elif inner == 'direct':
            _lib.check(lib.tfx_dgn_direct_step(dt, ctypes.c_void_p(_dev.ptr(Td)), L, cd, int(R),
                                               ctypes.c_void_p(_dev.ptr(W)), ctypes.c_double(damp),
                                               ctypes.c_void_p(_dev.ptr(y)), ctypes.c_void_p(_dev.ptr(grad)),
                                               ctypes.c_void_p(ws_dir[1]), int(ws_dir[0].numel() - 256), st))
            from_W, yp, gp, alias_in = 0, _dev.ptr(y), _dev.ptr(grad), int(aliased)
        else:
            raise NotImplementedError("inner_method %r" % (inner,))
        _lib.check(lib.tfx_dgn_step_update(dt, L, cd, int(R), ctypes.c_void_p(_dev.ptr(x)),
                                           ctypes.c_void_p(_dev.ptr(W)), ctypes.c_void_p(yp), ctypes.c_void_p(gp),
                                           ctypes.c_double(damp), from_W, int(symm), ctypes.c_double(fn), alias_in,
                                           int(fix_mode), ctypes.c_void_p(_dev.ptr(Wfix)),
                                           ctypes.c_void_p(_dev.ptr(out)), st))
        # the list's state after transform: symmetrising makes it one array;
        # the fixed-norm rescaling gives every mode its own
        aliased = (symm or bool(alias_in)) and fn <= 0
        _lib.check(lib.tfx_cp_residual(dt, ctypes.c_void_p(_dev.ptr(Td)), L, cd, int(R),
                                       ctypes.c_void_p(_dev.ptr(W)), ctypes.c_void_p(_dev.ptr(out) + 32),
                                       ctypes.c_void_p(_dev.ptr(res_scratch)), st))
        s = out.cpu().numpy()
        error = float(np.sqrt(max(s[4], 0.0))) / Tsize
        gain = _gain_ratio(damp, old_error, error, Tsize, float(s[2]))
        damp = _update_damp(damp, init_damp, gain, it)
        if error < best_error:
            best_error = error
            best.copy_(W)
        errors[it] = error
        step_sizes[it] = np.sqrt(s[0]) / np.sqrt(s[1])
        gradients[it] = s[3]
        improv[it] = errors[it] if it == 0 else abs(errors[it] - errors[it - 1])
        code = _stop_code(it, errors, step_sizes, improv, gradients, error, Tsize, tol, tol_step, tol_improv,
                          tol_grad, const)
        if code is not None:
            stop = code
            break
    k = it + 1
    return best, step_sizes[:k].copy(), errors[:k].copy(), improv[:k].copy(), gradients[:k].copy(), stop
