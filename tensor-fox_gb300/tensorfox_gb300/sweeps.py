"""Rank search and statistics sweeps (TensorFox.py:820-1039) on the batched engine.

The reference's ``rank(T)`` and ``stats(T, R)`` call ``cpd`` once per trial,
one after the other.  Here every CPD of the same tensor shares its work:

* ``stats(T, R, options, num_samples)`` compresses ``T`` once (MLSVD), draws
  ``num_samples`` random starting points in the compressed space and solves
  all of them in ONE launch of the dGN engine (one thread-block cluster per
  sample); decompression and the final errors follow per sample.
* ``rank(T, options, plot, trials)`` evaluates ranks in windows (1, 2, 4, ...
  up to 16 ranks at a time): one compression per rank, then one engine launch
  for every (rank, trial) of the window.  The reference's stopping rules are
  then applied rank by rank in order, so the result is the same as running the
  ranks one by one; at most the rest of the last window is computed in vain.

Differences from the reference, both deliberate:

* RNG order.  The reference interleaves each trial's draws (range finder,
  starting point, CG caps); here a window or a sample set draws its range
  finders, then all starting points, then the CG caps iteration by iteration
  (one value per problem).  Every draw has the reference's distribution.
* ``times`` of ``stats``: the samples run concurrently, so a per-sample wall
  time does not exist; each entry is the wall time of the whole call divided
  by ``num_samples``.
* Nothing is printed or plotted (``plot`` is accepted and ignored).

The 'als' method solves each problem with its own graph launch; sparse
``[data, idxs, dims]`` input and ``method='ttcpd'`` run ``cpd`` per trial.
"""
import time

import numpy as np
import torch

from . import _dev, kernels
from .api import _decompress, _flat_dev, _precision, _run_als, _run_dgn, consistency, sort_dims, starting_point_core, cpd
from .compression import mlsvd_device
from .gauss_newton import _Batch, _inner_of, auto_cluster
from .options import make_options


def rank_bounds(dims, method='dGN'):
    """(Rmin, Rmax) of the rank search (TensorFox.py:863-873)."""
    L = len(dims)
    if L > 3:
        if method == 'dGN':
            return 1, int(np.prod(np.sort(np.array(dims))[1:]))
        return 2, int(np.min(dims))
    m, n, p = [int(d) for d in dims]
    return 1, int(min(m * n, m * p, n * p))


def _draw_caps(options, L, n):
    """CG caps for ``n`` problems, iteration-major (GaussNewton.py:267 distribution)."""
    m = int(options.maxiter)
    caps = np.zeros((n, m), dtype=np.int32)
    for it in range(m):
        inner = _inner_of(options, it)
        if inner == 'cg':
            draw = np.random.randint(int(1 + it ** 0.4), int(2 + it ** 0.9), size=n)
            caps[:, it] = 1 + (L - 2) * (options.cg_factor * draw).astype(np.int64)
        elif inner == 'cg_static':
            caps[:, it] = options.cg_maxiter
        else:
            raise NotImplementedError("inner_method %r" % (inner,))
    return caps


class _Dense:
    """A dense tensor on the device in the reference's sorted mode order."""

    def __init__(self, T, options):
        self.prec = _precision(T, options)
        self.dt = _dev.torch_dtype(self.prec)
        shape = tuple(int(d) for d in T.shape)
        self.ordering = sort_dims(shape)
        if isinstance(T, torch.Tensor):
            self.Td = T.to(device=_dev.device(), dtype=self.dt).permute(*[int(i) for i in self.ordering]).contiguous()
        else:
            self.Td = _dev.to_device(np.transpose(np.asarray(T), self.ordering), self.dt)
        self.dims = tuple(int(d) for d in self.Td.shape)
        self.Tsize = float(np.sqrt(kernels.tensor_norms(self.Td).cpu().numpy()[0]))

    def compress(self, R, o):
        S, Uts, sigmas, core = mlsvd_device(self.Td, R, o)
        L = len(self.dims)
        if o.symm:
            Rm = min(core)
            S = S[tuple(slice(Rm) for _ in range(L))].contiguous()
            Uts = [u[:Rm].contiguous() for u in Uts]
            core = [Rm] * L
        return S, Uts, [int(c) for c in core]

    def start(self, R, o, Uts, core, S):
        L = len(self.dims)
        if isinstance(o.initialization, list):
            init = []
            for l in range(L):
                W = torch.from_numpy(np.asarray(o.initialization[self.ordering[l]], dtype=np.float64))
                init.append(kernels.matmul(Uts[l], W.to(self.Td.device, self.dt)).double().cpu().numpy())
        else:
            init = starting_point_core(S, core, R, o, vectorized=(self.prec == 'fp32'))
        return _flat_dev(init, self.dt, self.Td.device)

    def solve(self, problems, o):
        """problems: list of (S, Uts, core, R, x0).  Returns per problem
        (rel_error, num_steps, factors_flat_device)."""
        n = len(problems)
        L = len(self.dims)
        from .stepped import uses_stepped
        stepped = o.method != 'als' and uses_stepped(o)
        if o.method == 'als' or stepped:
            bests = []
            steps = []
            alias = stepped and bool(o.symm) and float(o.factors_norm) <= 0 and not isinstance(o.initialization, list)
            for (S, Uts, core, R, x0) in problems:
                if stepped:
                    x, ss, er, im, gr, st = _run_dgn(S, x0, R, o, self.prec, aliased=alias)
                else:
                    x, ss, er, im, gr, st = _run_als(S, x0, R, o, self.prec)
                bests.append(x)
                steps.append(len(ss))
        else:
            caps = _draw_caps(o, L, n)
            alias = bool(o.symm) and float(o.factors_norm) <= 0 and not isinstance(o.initialization, list)
            b = _Batch([p[0] for p in problems], [p[4] for p in problems], [p[3] for p in problems], o, self.prec,
                       budgets=list(caps), aliased=alias)
            c = o.cluster or min(auto_cluster(tuple(p[2]), p[3]) for p in problems)
            b.launch(c)
            res = b.result.cpu().numpy()
            from . import _lib
            _lib.check_solve_status(res)
            bests = b.best
            steps = [int(r[1]) for r in res]
        out = []
        full = [_decompress(p[1], bests[k], p[2], p[3]) for k, p in enumerate(problems)]
        if o.refine:
            if o.method == 'als' or stepped:
                run = _run_dgn if stepped else _run_als
                ref = [run(self.Td, f, p[3], o, self.prec) for f, p in zip(full, problems)]
                for k, r in enumerate(ref):
                    out.append((float(r[2][-1]), steps[k] + len(r[1]), r[0]))
                return out
            caps = _draw_caps(o, L, n)
            b2 = _Batch([self.Td] * n, full, [p[3] for p in problems], o, self.prec, budgets=list(caps))
            b2.launch(o.cluster or auto_cluster(self.dims, max(p[3] for p in problems)))
            res2 = b2.result.cpu().numpy()
            st2 = b2.stats.cpu().numpy()
            m = int(o.maxiter)
            for k in range(n):
                k2 = int(res2[k, 1])
                out.append((float(st2[k, k2 - 1]), steps[k] + k2, b2.best[k]))
            return out
        for k, p in enumerate(problems):
            r2 = float(kernels.cp_residual_sq(self.Td, self.dims, full[k], p[3]).cpu().numpy()[0])
            out.append((float(np.sqrt(max(r2, 0.0))) / self.Tsize, steps[k], full[k]))
        return out


def stats(T, R, options=False, num_samples=100):
    """Drop-in for TensorFox.stats (TensorFox.py:942-1039): ``num_samples`` CPDs
    of ``T`` from random starting points.  Returns ``(times, steps, errors)``."""
    _dev.require_cuda()
    t0 = time.perf_counter()
    o = make_options(options)
    n = int(num_samples)
    if isinstance(T, list) or o.method not in ('dGN', 'als'):
        # COO input and the tensor-train method: one cpd per sample
        times, steps, errors = np.empty(n), np.empty(n), np.empty(n)
        for k in range(n):
            t = time.perf_counter()
            _, out = cpd(T, R, o)
            times[k] = time.perf_counter() - t
            steps[k] = out.num_steps
            errors[k] = out.rel_error
        return times, steps, errors
    consistency(R, T.shape, o)
    X = _Dense(T, o)
    S, Uts, core = X.compress(R, o)
    probs = [(S, Uts, core, R, X.start(R, o, Uts, core, S)) for _ in range(n)]
    res = X.solve(probs, o)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    times = np.full(n, wall / n)
    steps = np.array([r[1] for r in res], dtype=np.float64)
    errors = np.array([r[0] for r in res], dtype=np.float64)
    return times, steps, errors


def rank_search(dims, method, best_errors_of):
    """The reference's rank search (TensorFox.py:854-926) over windows of ranks.

    ``best_errors_of(ranks)`` returns, for each rank of the list, the best
    relative error over the trials.  Order > 3 at rank 1 counts as error 1
    without a CPD.  Returns ``(final_rank, error_per_rank)``."""
    L = len(dims)
    Rmin, Rmax = rank_bounds(dims, method)
    epr = np.empty(Rmax)
    final = None
    r = 1
    width = 1
    while r <= Rmax and final is None:
        window = [q for q in range(r, min(Rmax, r + width - 1) + 1) if not (L > 3 and q == 1)]
        got = dict(zip(window, best_errors_of(window))) if window else {}
        for q in range(r, min(Rmax, r + width - 1) + 1):
            epr[q - 1] = 1.0 if (L > 3 and q == 1) else got[q]
            best = epr[q - 1]
            last = q
            if best < 1e-14:
                final = q
                break
            if q > Rmin and abs(epr[q - 1] - epr[q - 2]) < 1e-5 and best < 0.5:
                final = int(np.nanargmin(epr[0:q])) + 1
                break
            if q > 2:
                prev = abs(epr[q - 2] - epr[q - 3])
                cur = abs(epr[q - 1] - epr[q - 2])
                ratio = (np.inf if prev > 0 else np.nan) if cur == 0 else prev / cur
                if ratio > 100 and best < 0.5:
                    final = q - 1
                    break
        r = last + 1
        width = min(2 * width, 16)
    epr = epr[0:last]
    if final is None:
        final = int(np.nanargmin(epr)) + 1
    return int(final), epr


def rank(T, options=False, plot=True, trials=3):
    """Drop-in for TensorFox.rank (TensorFox.py:820-939).  Returns
    ``(final_rank, error_per_rank)``."""
    _dev.require_cuda()
    o = make_options(options)
    if isinstance(T, list) or o.method not in ('dGN', 'als'):
        # COO input and the tensor-train method: trials run one cpd at a time
        dims = [int(d) for d in (T[2] if isinstance(T, list) else T.shape)]

        def best_errors_of(ranks):
            out = []
            for q in ranks:
                out.append(min(cpd(T, q, o)[1].rel_error for _ in range(trials)))
            return out
        return rank_search(dims, o.method, best_errors_of)
    dims = [int(d) for d in T.shape]
    X = _Dense(T, o)

    def best_errors_of(ranks):
        probs, owner = [], []
        for q in ranks:
            S, Uts, core = X.compress(q, o)
            for _ in range(trials):
                probs.append((S, Uts, core, q, X.start(q, o, Uts, core, S)))
                owner.append(q)
        res = X.solve(probs, o)
        best = {q: np.inf for q in ranks}
        for q, r in zip(owner, res):
            if r[0] < best[q]:
                best[q] = r[0]
        return [best[q] for q in ranks]
    return rank_search(dims, o.method, best_errors_of)
