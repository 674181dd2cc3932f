"""User API: ``cpd`` / ``tricpd`` with the reference's semantics (TensorFox.py:69-655).

``cpd(T, R, options)`` returns ``(factors, output)`` exactly like Tensor Fox:
factors are NumPy float64 ``(d_l, R)`` arrays in the caller's mode order and
``output`` carries num_steps, rel_error, accuracy, step_sizes, errors, improv,
gradients, stop and options.  Invalid input raises ``SystemExit`` with the
reference's messages (Auxiliar.py:24-78), without its one-second pause.
"""
import sys

import numpy as np
import torch

from . import _dev, _lib, kernels
from .compression import mlsvd_device
from .gauss_newton import _Batch, advance_rng, auto_cluster
from .options import make_options


class Output:
    """Result record of ``cpd`` (Auxiliar.py:161-218)."""

    def stop_msg(self):
        msgs = {0: '0 - Relative error is small enough.', 1: '1 - Steps are small enough.',
                2: '2 - Improvement in the relative error is small enough.', 3: '3 - Gradient is small enough.',
                4: '4 - Average error increased.', 5: '5 - Limit of iterations was reached.',
                6: '6 - dGN diverged.', 7: '7 - Average improvement is too small compared to the average error.',
                8: '8 - No refinement was performed.'}
        print()
        print('Main stop:')
        print(msgs.get(self.stop[0], str(self.stop[0])))
        print()
        print('Refinement stop:')
        print(msgs.get(self.stop[1], str(self.stop[1])))
        return ''


def consistency(R, dims, options):
    """Input checks of Auxiliar.py:24-78 (same messages, no sleep)."""
    L = len(dims)
    if L > 12:
        sys.exit('Tensor Fox does not work with tensors of order higher than 12.')
    for l in range(L):
        if dims[l] == 1:
            sys.exit('At least one dimension is equal to 1. This situation not supported by Tensor Fox.')
    if (type(R) != int) or (R < 1):
        sys.exit('Rank must be a positive integer.')
    if L == 3:
        m, n, p = int(dims[0]), int(dims[1]), int(dims[2])
        if R > min(m * n, m * p, n * p):
            sys.exit('Rank must satisfy 1 <= rank <= min(m*n, m*p, n*p) = ' + str(min(m * n, m * p, n * p)) + '.')
    if L > 3 and R == 1:
        sys.exit('Rank must be greater than 1 for tensor with order greater than 3.')
    if options.symm:
        for i in range(L):
            for j in range(L):
                if dims[i] != dims[j]:
                    sys.exit('Symmetric tensors must have equal dimensions.')
    if options.method != 'dGN' and options.method != 'als' and options.method != 'ttcpd':
        sys.exit("Wrong method name. Must be 'dGN', 'als' or 'ttcpd'.")


def sort_dims(shape):
    """Mode permutation into decreasing sizes (Auxiliar.py:93-115)."""
    return np.argsort(-np.array(shape))


def unsort_dims(factors, ordering):
    out = [None] * len(factors)
    for l in range(len(factors)):
        out[ordering[l]] = factors[l]
    return out


def _precision(T, options):
    p = options.precision
    if p in ('fp64', 'fp32'):
        return p
    if p == 'mixed':
        return 'fp32'
    if isinstance(T, torch.Tensor):
        return 'fp64' if T.dtype == torch.float64 else 'fp32'
    if isinstance(T, list):
        return 'fp64'
    return 'fp64' if np.asarray(T).dtype == np.float64 else 'fp32'


def starting_point_random(dims, R, options, vectorized=False):
    """'random' initialisation in the compressed space (Initialization.py:61-94).

    ``vectorized`` balances all columns at once; its column norms may differ
    from the per-column ones in the last bit of a float64, which a float32
    engine never sees."""
    f = [np.random.randn(dims[l], R) for l in range(len(dims))]
    for l in range(len(dims)):             # clean_zeros (Initialization.py:361-386)
        W = f[l]
        for i, r in zip(*np.nonzero(W == 0.0)):
            W[i, r] = 1e-4 * np.random.randn() * np.linalg.norm(W)
    L = len(dims)
    if vectorized:                          # equalize, all columns together
        nr = np.stack([np.linalg.norm(f[l], axis=0) for l in range(L)])
        p = np.prod(nr, axis=0)
        ok = p != 0.0
        g = np.where(ok, p, 1.0) ** (1 / L)
        for l in range(L):
            f[l] = np.where(ok, g / np.where(ok, nr[l], 1.0), 1.0) * f[l]
    else:
        for r in range(R):                  # equalize (Conversion.py:361-387)
            nr = np.array([np.linalg.norm(f[l][:, r]) for l in range(L)])
            if np.prod(nr) != 0.0:
                g = np.prod(nr) ** (1 / L)
                for l in range(L):
                    f[l][:, r] = (g / nr[l]) * f[l][:, r]
    if options.symm:
        s = f[0]
        for l in range(1, len(dims)):
            s = s + f[l]
        f = [s / len(dims)] * len(dims)
    if options.factors_norm > 0:
        f = [options.factors_norm * (1 / np.linalg.norm(W)) * W for W in f]
    return f


def starting_point_core(S, core, R, options, vectorized=False):
    """'random', 'smart_random' or 'smart' start in the compressed space
    (Initialization.py:20-94); S is the device core."""
    init = options.initialization
    if init == 'random':
        return starting_point_random(core, R, options, vectorized=vectorized)
    if init in ('smart_random', 'smart'):
        from .initialization import clean_and_balance, smart, smart_random
        Sh = S.double().cpu().numpy()
        f = smart_random(Sh, R) if init == 'smart_random' else smart(Sh, R)
        return clean_and_balance(f, R, options, vectorized=vectorized)
    sys.exit('Error with init parameter initialization.')


def _flat_dev(factors, dtype, device):
    return _dev.h2d(_dev.flat_factors(factors), dtype, device)


def _run_dgn(Td, x0, R, options, prec, aliased=False, fix_mode=-1):
    """dGN on device inputs: the persistent engine for the 'cg'/'cg_static'
    inner methods, the stepped loop for 'als'/'direct'.  ``aliased``: the
    reference would hand dGN one factor array L times (a symmetric start);
    ``fix_mode`` >= 0: that factor is put back after every step (bicpd)."""
    from .stepped import uses_stepped, dgn_stepped
    if uses_stepped(options):
        return dgn_stepped(Td, x0, R, options, prec, fix_mode=fix_mode, aliased=aliased)
    if Td.numel() >= DENSE_MTTKRP_MIN and fix_mode < 0 and not aliased:
        # a large FP32 tensor (the refinement on the full tensor, or no
        # compression): tensor-core MTTKRPs and a grid-wide CG instead of one
        # thread-block cluster streaming the whole tensor
        from .mttkrp_dgn import dense_supported, dgn_dense
        if dense_supported(Td, R, options, prec):
            return dgn_dense(Td, x0, R, options)[:6]
    return _engine_collect(_engine_launch(Td, x0, R, options, prec, aliased, fix_mode), options)


# tensors of at least this many entries take the MTTKRP-driven dGN when it applies
DENSE_MTTKRP_MIN = 1 << 22


def _engine_launch(Td, x0, R, options, prec, aliased=False, fix_mode=-1):
    """Queues one engine solve on the current stream; nothing is read back."""
    b = _Batch([Td], [x0], [R], options, prec, aliased=aliased, fix_mode=fix_mode)
    b.launch(options.cluster or auto_cluster(tuple(Td.shape), R))
    return b


def _engine_collect(b, options):
    """Reads a launched engine solve: (best, step_sizes, errors, improv,
    gradients, stop), the global RNG advanced past the 'cg' caps' draws."""
    res = b.result[0].cpu().numpy()
    _lib.check_solve_status(res)
    stats = b.stats[0].cpu().numpy()
    n = int(res[1])
    advance_rng(options, n)
    m = options.maxiter
    return (b.best[0], stats[m:m + n].copy(), stats[:n].copy(), stats[2 * m:2 * m + n].copy(),
            stats[3 * m:3 * m + n].copy(), int(res[0]))


def _decompress(Uts, best_flat, core_dims, R):
    """factors_l = U_l W_l on the device (TensorFox.py:573-574); returns the flat layout."""
    outs, s = [], 0
    for l, Ut in enumerate(Uts):
        n = core_dims[l]
        WcT = best_flat[s:s + n * R].view(R, n)   # column-major (n x R) core factor
        outs.append(kernels.matmul(WcT, Ut).reshape(-1))   # (R, d) = column-major (d x R)
        s += n * R
    return torch.cat(outs)


def _run_als(Td, x0, R, options, prec):
    from .als import als_device, split_stats
    x, best, stats, res, info = als_device(Td, x0, R, options, prec)
    n = int(res[1])
    ss, er, im, gr = split_stats(stats, int(options.maxiter), n)
    return (x, ss, er, im, gr, int(res[0]))


def tricpd(T, R, options):
    """Compression, starting point, dGN or ALS, decompression, refinement, final
    error (TensorFox.py:424-655)."""
    o = options
    if isinstance(T, list):
        from .sparse import tricpd_sparse
        return tricpd_sparse(T, R, o)
    if o.method not in ('dGN', 'als'):
        raise NotImplementedError("method %r is outside the damped Gauss-Newton and ALS paths" % (o.method,))
    solve = _run_als if o.method == 'als' else _run_dgn
    prec = _precision(T, o)
    dt = _dev.torch_dtype(prec)
    shape = tuple(int(d) for d in T.shape)
    L = len(shape)
    ordering = sort_dims(shape)
    if isinstance(T, torch.Tensor):
        Td = T.to(device=_dev.device(), dtype=dt).permute(*[int(i) for i in ordering]).contiguous()
    else:
        Td = _dev.to_device(np.transpose(np.asarray(T), ordering), dt)
    dims = tuple(int(d) for d in Td.shape)
    nrm_dev = kernels.tensor_norms(Td)       # read with the final error (no wait here)
    # Pipelined path (engine solve, random start): the MLSVD, the start point,
    # the engine, the decompression and the final residual are all queued
    # before the first read from the device.
    pipelined, tried = None, False
    if o.method == 'dGN' and isinstance(o.initialization, str) and o.initialization == 'random':
        from .stepped import uses_stepped
        from .compression import mlsvd_launch
        if not uses_stepped(o):
            pend = mlsvd_launch(Td, R, o)
            if pend is not None:
                tried = True
                pipelined = _pipelined(Td, dims, R, o, prec, dt, pend)
    if pipelined is not None:
        best, ss, er, im, gr, st, Wf, r2 = pipelined
    else:
        # after a failed speculation the MLSVD runs mode by mode straight away
        best, ss, er, im, gr, st, Wf, r2 = _staged(Td, dims, R, o, prec, dt, ordering, solve, speculate=not tried)
    if o.refine:
        Wf, ss2, er2, im2, gr2, st2 = solve(Td, Wf, R, o, prec)
    else:
        ss2, er2, im2, gr2, st2 = np.array([0]), np.array([0]), np.array([0]), np.array([0]), 8
    if o.refine:
        rel_error = float(er2[-1])
    else:
        # one transfer: ||T - [[W]]||^2, ||T||^2
        r2n = torch.cat([r2, nrm_dev[:1]]).cpu().numpy()
        rel_error = float(np.sqrt(r2n[0])) / float(np.sqrt(r2n[1]))
    factors = _dev.unflat(Wf.double().cpu().numpy(), dims, R)
    factors = unsort_dims(factors, ordering)
    out = Output()
    out.num_steps = len(ss) + (len(ss2) if o.refine else 0)
    out.rel_error = rel_error
    out.accuracy = max(0, 100 * (1 - rel_error))
    out.step_sizes = [ss, ss2]
    out.errors = [er, er2]
    out.improv = [im, im2]
    out.gradients = [gr, gr2]
    out.stop = [st, st2]
    out.options = o
    return factors, out


def _symm_core(S, Uts, core, L):
    """TensorFox.py:519-523: with symm the core keeps min(core) in every mode."""
    Rm = min(core)
    S = S[tuple(slice(Rm) for _ in range(L))].contiguous()
    return S, [u[:Rm].contiguous() for u in Uts], [Rm] * L


def _pipelined(Td, dims, R, o, prec, dt, pend):
    """The engine path with no read from the device until everything is queued.
    Returns None (NumPy's RNG put back) when the MLSVD's energy truncation cuts
    a mode, so the staged path must run instead."""
    from .compression import mlsvd_confirm
    L = len(dims)
    S, Uts, core = pend.S, pend.Uts, list(pend.cur)
    if o.symm:
        S, Uts, core = _symm_core(S, Uts, core, L)
    init = starting_point_core(S, core, R, o, vectorized=(prec == 'fp32'))
    x0 = _flat_dev(init, dt, Td.device)
    alias = bool(o.symm) and float(o.factors_norm) <= 0     # Initialization.py:83
    b = _engine_launch(S, x0, R, o, prec, aliased=alias)
    Wf = _decompress(Uts, b.best[0], core, R)
    r2 = None if o.refine else kernels.cp_residual_sq(Td, dims, Wf, R)
    if mlsvd_confirm(pend) is None:
        return None
    best, ss, er, im, gr, st = _engine_collect(b, o)
    return best, ss, er, im, gr, st, Wf, r2


def _staged(Td, dims, R, o, prec, dt, ordering, solve, speculate=True):
    """MLSVD, start point, solve, decompression and residual one after the other."""
    L = len(dims)
    S, Uts, sigmas, core = mlsvd_device(Td, R, o, speculate=speculate)
    if o.symm:
        S, Uts, core = _symm_core(S, Uts, core, L)
    if isinstance(o.initialization, list):
        init = []
        for l in range(L):
            W = torch.from_numpy(np.asarray(o.initialization[ordering[l]], dtype=np.float64)).to(Td.device, dt)
            init.append(kernels.matmul(Uts[l], W).double().cpu().numpy())
    else:
        init = starting_point_core(S, core, R, o, vectorized=(prec == 'fp32'))
    x0 = _flat_dev(init, dt, Td.device)
    if o.method == 'als':
        best, ss, er, im, gr, st = solve(S, x0, R, o, prec)
    else:
        # Initialization.py:83: a symmetrising transform leaves one array L times
        alias = bool(o.symm) and float(o.factors_norm) <= 0 and not isinstance(o.initialization, list)
        best, ss, er, im, gr, st = solve(S, x0, R, o, prec, aliased=alias)
    Wf = _decompress(Uts, best, core, R)
    r2 = None if o.refine else kernels.cp_residual_sq(Td, dims, Wf, R)
    return best, ss, er, im, gr, st, Wf, r2


def cpd(T, R, options=False):
    """Drop-in for TensorFox.cpd (TensorFox.py:69-255): methods 'dGN', 'als' and
    'ttcpd'."""
    _dev.require_cuda()
    if isinstance(T, list):
        dims_orig = T[2]
    else:
        dims_orig = T.shape
    o = make_options(options)
    consistency(R, dims_orig, o)
    if o.method in ('dGN', 'als'):
        return tricpd(T, R, o)
    if o.method == 'ttcpd':
        from .tt import cpd_tt
        return cpd_tt(T, R, o)
    raise NotImplementedError("method %r" % (o.method,))
