"""Damped Gauss-Newton on the device (GaussNewton.py:29 ``dGN``).

``dGN(T, factors, R, options)`` keeps the reference's signature and return
tuple.  The whole iteration (CG inner solves, dogleg fallback, damping updates
and stop tests) runs as one launch of the cluster-persistent engine
(``tfx_dgn_solve``); the host only prepares the CG caps and reads the results.

The 'cg' inner method draws its CG cap from NumPy's global RNG once per
iteration (GaussNewton.py:267).  The caps are drawn here from a copy of the RNG
state, and afterwards the real RNG is advanced by exactly the draws the
reference would have made, so seeded runs stay in step with it.
"""
import ctypes

import numpy as np
import torch

from . import _dev, _lib
from .options import make_options


def _inner_of(options, it):
    im = options.inner_method
    return im[it] if isinstance(im, list) else im


def cg_budgets(options, L):
    """CG caps for every iteration, drawn without consuming the global RNG."""
    state = np.random.get_state()
    out = np.zeros(options.maxiter, dtype=np.int32)
    try:
        for it in range(options.maxiter):
            inner = _inner_of(options, it)
            if inner == 'cg':
                out[it] = 1 + (L - 2) * int(options.cg_factor * np.random.randint(1 + it ** 0.4, 2 + it ** 0.9))
            elif inner == 'cg_static':
                out[it] = options.cg_maxiter
            else:
                raise NotImplementedError(
                    "inner_method %r is outside the damped Gauss-Newton CG path" % (inner,))
    finally:
        np.random.set_state(state)
    return out


def advance_rng(options, iterations):
    """Consumes the RNG draws the reference's 'cg' caps make in ``iterations`` steps."""
    for it in range(iterations):
        if _inner_of(options, it) == 'cg':
            np.random.randint(1 + it ** 0.4, 2 + it ** 0.9)


def auto_cluster(dims, R):
    """CTAs per problem (one thread-block cluster): about one CTA per 1.2 million
    multiply-adds of per-iteration MTTKRP work, at most 16 and at most R (every
    CTA owns whole factor columns).  Measured on the 50^3, R=50 core of a
    512^3 problem: 16 CTAs beat 10 and 8 despite the uneven column split."""
    n = int(np.prod(dims))
    work = n * R * len(dims)
    return int(max(1, min(16, R, work // 1200000)))


def _cluster_candidates(c, R):
    cands = [c] + [x for x in (1, 2, 4, 8, 12, 16) if x > c and x <= max(R, 1)]
    return [x for x in cands if x <= max(R, 1)] or [1]


class _Batch:
    """Device buffers for a set of dGN problems solved in one engine launch."""

    def __init__(self, tensors, xs, R_list, options, precision, budgets=None, aliased=False, fix_mode=-1):
        self.precision = precision
        dt = _dev.torch_dtype(precision)
        self.es = 8 if precision == "fp64" else 4
        lib = _lib.load()
        self.n = len(tensors)
        self.options = options
        self.maxiter = int(options.maxiter)
        self.tensors = tensors
        self.xs = xs
        self.dims = [tuple(int(d) for d in t.shape) for t in tensors]
        self.R = R_list
        self.best = [torch.empty_like(x) for x in xs]
        self.ws = []
        for t, R in zip(tensors, R_list):
            L = t.dim()
            dims_c = (ctypes.c_int * L)(*t.shape)
            nb = lib.tfx_dgn_workspace_bytes(_dev.lib_dtype(precision), L, dims_c, int(R))
            self.ws.append(torch.empty(int(nb), dtype=torch.uint8, device=t.device))
        # host -> device copies through pinned staging: they queue behind the
        # device work instead of waiting for it
        if budgets is None:
            self.budgets = [_dev.h2d(cg_budgets(options, t.dim()), None, t.device) for t in tensors]
        else:   # per-problem caps drawn by the caller (maxiter ints each)
            self.budgets = [_dev.h2d(np.asarray(b, dtype=np.int32), None, t.device)
                            for b, t in zip(budgets, tensors)]
        sched = options.init_damp if isinstance(options.init_damp, list) else None
        self.sched = None
        if sched is not None:
            self.sched = _dev.h2d(np.asarray(sched, dtype=np.float64), torch.float64, tensors[0].device)
        self.stats = torch.zeros((self.n, 4 * self.maxiter), dtype=torch.float64, device=tensors[0].device)
        self.result = torch.zeros((self.n, 4), dtype=torch.int32, device=tensors[0].device)
        self.info = torch.zeros((self.n, 8), dtype=torch.float64, device=tensors[0].device)
        self.prof = torch.zeros((self.n, 24), dtype=torch.int64, device=tensors[0].device)
        # the descriptors live in pinned memory, so the library's copy of them
        # to the device is asynchronous (this object keeps the buffer alive
        # until the results are read)
        self._desc_host = torch.zeros(ctypes.sizeof(_lib.DgnProblem) * self.n, dtype=torch.uint8).pin_memory()
        self.desc = (_lib.DgnProblem * self.n).from_address(self._desc_host.data_ptr())
        for p in range(self.n):
            d = self.desc[p]
            d.L = len(self.dims[p])
            d.R = int(R_list[p])
            for l, v in enumerate(self.dims[p]):
                d.dims[l] = v
            d.tensor = _dev.ptr(tensors[p])
            d.x = _dev.ptr(xs[p])
            d.best = _dev.ptr(self.best[p])
            d.work = _dev.ptr(self.ws[p])
            d.budgets = _dev.ptr(self.budgets[p])
            d.damp_sched = _dev.ptr(self.sched) if self.sched is not None else None
            d.stats = _dev.ptr(self.stats[p])
            d.result = _dev.ptr(self.result[p])
            d.info = _dev.ptr(self.info[p])
            d.prof = _dev.ptr(self.prof[p])
        self.d_desc = torch.empty(ctypes.sizeof(_lib.DgnProblem) * self.n, dtype=torch.uint8,
                                  device=tensors[0].device)
        o = _lib.DgnOptions()
        o.maxiter = self.maxiter
        o.tol, o.tol_step, o.tol_improv = float(options.tol), float(options.tol_step), float(options.tol_improv)
        o.tol_grad, o.tol_jump, o.cg_tol = float(options.tol_grad), float(options.tol_jump), float(options.cg_tol)
        o.init_damp = 0.0 if sched is not None else float(options.init_damp)
        o.use_damp_sched = 1 if sched is not None else 0
        o.symm = 1 if options.symm else 0
        o.factors_norm = float(options.factors_norm)
        o.tile = int(getattr(options, 'tile', None) or 0)
        o.aliased = 1 if aliased else 0
        o.fixed = int(fix_mode) + 1
        self.opts = o

    def launch(self, cluster, stream=None):
        lib = _lib.load()
        st = _dev.stream() if stream is None else stream
        cands = _cluster_candidates(cluster, min(self.R))
        last = None
        for c in cands:
            status = lib.tfx_dgn_solve(_dev.lib_dtype(self.precision), self.desc, ctypes.c_void_p(_dev.ptr(self.d_desc)),
                                       self.n, ctypes.byref(self.opts), c, ctypes.c_void_p(st))
            if status == 5:      # does not fit: retry with a wider cluster
                last = status
                continue
            _lib.check(status)
            return c
        _lib.check(last)


def _precision_of(T, options):
    p = getattr(options, 'precision', None)
    if p in ('fp64', 'fp32'):
        return p
    if p == 'mixed':
        return 'fp32'
    if p not in (None, 'auto'):
        raise ValueError("precision must be 'fp64', 'fp32', 'mixed' or None")
    if isinstance(T, torch.Tensor):
        return 'fp64' if T.dtype == torch.float64 else 'fp32'
    return 'fp64' if np.asarray(T).dtype == np.float64 else 'fp32'


def dGN_device(Td, x0d, R, options, precision, cluster=None, aliased=False, fix_mode=-1):
    """Runs the engine on device-resident inputs; returns device results."""
    b = _Batch([Td], [x0d], [R], options, precision, aliased=aliased, fix_mode=fix_mode)
    c = cluster if cluster is not None else (options.cluster or auto_cluster(Td.shape, R))
    b.launch(c)
    return b


class _Single:
    """One problem's descriptor and workspace for the standalone evaluations."""

    def __init__(self, T, x_flat, R, precision):
        self.precision = precision
        self.dt = _dev.torch_dtype(precision)
        self.Td = _dev.to_device(T, self.dt)
        self.dims = tuple(int(d) for d in self.Td.shape)
        dev = self.Td.device
        self.x = (x_flat if isinstance(x_flat, torch.Tensor) else torch.from_numpy(np.asarray(x_flat)))
        self.x = self.x.to(dev, self.dt).contiguous()
        lib = _lib.load()
        L = len(self.dims)
        dims_c = (ctypes.c_int * L)(*self.dims)
        self.ws = torch.empty(int(lib.tfx_dgn_workspace_bytes(_dev.lib_dtype(precision), L, dims_c, int(R))),
                              dtype=torch.uint8, device=dev)
        self.result = torch.zeros(4, dtype=torch.int32, device=dev)
        d = _lib.DgnProblem()
        d.L, d.R = L, int(R)
        for l, v in enumerate(self.dims):
            d.dims[l] = v
        d.tensor, d.x, d.work, d.result = _dev.ptr(self.Td), _dev.ptr(self.x), _dev.ptr(self.ws), _dev.ptr(self.result)
        self.desc = d
        self.d_desc = torch.empty(ctypes.sizeof(_lib.DgnProblem), dtype=torch.uint8, device=dev)
        o = _lib.DgnOptions()
        o.maxiter = 1
        self.opts = o

    def vec(self, v):
        t = v if isinstance(v, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(v))
        return t.to(self.Td.device, self.dt).contiguous()

    def check(self):
        _lib.check_solve_status(self.result.cpu().numpy())


def _vp(t):
    return ctypes.c_void_p(_dev.ptr(t) if t is not None else None)


def jtj_matvec(T, factors, R, v=None, damp=1.0, cluster=None, precision=None, gradient=True):
    """The solver's per-iteration products at one point, computed by the same
    device code as the solve (``tfx_jtj_matvec``): the gradient ``g`` of
    GaussNewton.py:401-427 (``compute_grad``) and ``J^T J v`` of
    GaussNewton.py:551-581 (``matvec``), both in the flat layout.

    ``T`` and ``v`` may be NumPy arrays or torch tensors; the results are
    device tensors of the working precision (``None`` for a skipped product)."""
    _dev.require_cuda()
    if precision is None:
        precision = 'fp64' if (getattr(T, 'dtype', None) in (np.float64, torch.float64)) else 'fp32'
    s = _Single(T, _dev.flat_factors(list(factors)), R, precision)
    vd = s.vec(v) if v is not None else None
    jv = torch.empty_like(s.x) if v is not None else None
    g = torch.empty_like(s.x) if gradient else None
    c = cluster if cluster is not None else auto_cluster(s.dims, R)
    _lib.call("tfx_jtj_matvec", _dev.lib_dtype(precision), ctypes.byref(s.desc), _vp(s.d_desc),
              ctypes.byref(s.opts), int(c), float(damp), _vp(vd), _vp(jv), _vp(g), ctypes.c_void_p(_dev.stream()))
    s.check()
    return g, jv


def dogleg_steps(T, x, y, grad, jtj, error, damp, R, cluster=None, precision=None, symm=False, factors_norm=0):
    """The dogleg trials after a rejected step (GaussNewton.py:713-795
    ``compute_dogleg_steps``) on the device, by the solver's own code.  Returns
    ``(best_factors_flat, best_x, best_y, best_error)`` as device tensors and a
    float."""
    _dev.require_cuda()
    if precision is None:
        precision = 'fp64' if (getattr(T, 'dtype', None) in (np.float64, torch.float64)) else 'fp32'
    s = _Single(T, x, R, precision)
    s.opts.symm = 1 if symm else 0
    s.opts.factors_norm = float(factors_norm)
    yd, gd, jd = s.vec(y), s.vec(grad), s.vec(jtj)
    bx, by, bw = torch.empty_like(s.x), torch.empty_like(s.x), torch.empty_like(s.x)
    be = torch.empty(1, dtype=torch.float64, device=s.x.device)
    c = cluster if cluster is not None else auto_cluster(s.dims, R)
    _lib.call("tfx_dgn_dogleg", _dev.lib_dtype(precision), ctypes.byref(s.desc), _vp(s.d_desc), ctypes.byref(s.opts),
              int(c), float(damp), float(error), _vp(yd), _vp(gd), _vp(jd), _vp(bx), _vp(by), _vp(bw), _vp(be),
              ctypes.c_void_p(_dev.stream()))
    s.check()
    return bw, bx, by, float(be.item())


def dGN(T, factors, R, options=None, precision=None):
    """Damped Gauss-Newton (GaussNewton.py:29-251) on the device.

    Returns ``(best_factors, step_sizes, errors, improv, gradients, stop)`` with
    NumPy float64 arrays, exactly like the reference.
    """
    _dev.require_cuda()
    options = make_options(options) if not hasattr(options, 'bi_method_parameters') else options
    if precision is not None:
        options.precision = precision
    prec = _precision_of(T, options)
    dt = _dev.torch_dtype(prec)
    Td = _dev.to_device(T, dt)
    dims = tuple(Td.shape)
    factors = list(factors)
    L = len(factors)
    aliased = L > 1 and all(f is factors[0] for f in factors)   # one array L times (symmetric start)
    fix = -1
    for l in range(L):        # [W] marks a fixed factor (bicpd), GaussNewton.py:92-99
        if isinstance(factors[l], list):
            fix, factors[l] = l, factors[l][0]
    x0 = torch.from_numpy(_dev.flat_factors(factors)).to(device=Td.device, dtype=dt)
    from .stepped import uses_stepped, dgn_stepped
    if uses_stepped(options):
        best, ss, er, im, gr, st = dgn_stepped(Td, x0, R, options, prec, fix_mode=fix, aliased=aliased)
        return (_dev.unflat(best.double().cpu().numpy(), dims, R), ss, er, im, gr, st)
    if aliased and len(set(dims)) != 1:
        raise ValueError("one factor array for every mode needs equal dimensions")
    b = dGN_device(Td, x0, R, options, prec, aliased=aliased, fix_mode=fix)
    res = b.result[0].cpu().numpy()
    _lib.check_solve_status(res)
    stats = b.stats[0].cpu().numpy()
    n = int(res[1])
    advance_rng(options, n)
    best = _dev.unflat(b.best[0].double().cpu().numpy(), dims, R)
    m = options.maxiter
    return (best, stats[m:m + n].copy(), stats[:n].copy(), stats[2 * m:2 * m + n].copy(),
            stats[3 * m:3 * m + n].copy(), int(res[0]))
