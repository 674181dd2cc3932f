"""Many small dense CPDs in a handful of launches.

Tensor Fox's ``rank`` and ``stats`` drivers (TensorFox.py:820-1039) call ``cpd``
once per trial, serially.  ``cpd_batch(tensors, ranks, options)`` computes the
same per-problem results for a list of small dense tensors (every dimension at
most 64) with one launch per stage for the whole batch:

1. ``tfx_batch_mlsvd``: one CTA per problem runs the sequentially truncated MLSVD;
2. the random starting points are drawn on the host (NumPy's global RNG, one
   problem after the other, each exactly like Initialization.py:61-83);
3. ``tfx_dgn_solve``: the dGN engine with one CTA per problem;
4. ``tfx_batch_decompress`` and ``tfx_batch_residual``.

RNG order differs from a serial loop of ``cpd`` calls (the serial loop draws each
problem's CG caps before the next problem's start): the starting points are drawn
from NumPy's global RNG problem by problem, then the CG caps iteration by
iteration, one value per problem for each iteration (same distribution as
GaussNewton.py:267).
"""
import ctypes
import os

import numpy as np
import torch

from . import _dev, _lib, tuner
from .api import Output, consistency
from .gauss_newton import _inner_of
from .options import make_options

_BATCH_DT = np.dtype([('L', 'i4'), ('R', 'i4'), ('dims', 'i4', 12), ('tensor', 'u8'), ('work', 'u8'),
                      ('work_elems', 'i8'), ('Ut', 'u8'), ('core', 'u8'), ('core_dims', 'u8'), ('sigma', 'u8')],
                     align=True)
_DGN_DT = np.dtype([('L', 'i4'), ('R', 'i4'), ('dims', 'i4', 12), ('tensor', 'u8'), ('x', 'u8'), ('best', 'u8'),
                    ('work', 'u8'), ('budgets', 'u8'), ('damp_sched', 'u8'), ('stats', 'u8'), ('result', 'u8'),
                    ('info', 'u8'), ('prof', 'u8')], align=True)


def _al(n, a=64):
    return (int(n) + a - 1) // a * a


def _random_starts(core_dims, Rs, x_off, xh):
    """Random starting points of every problem, in problem order, written into
    ``xh`` (the engines' flat layout, column-major per mode).

    The draws are one ``np.random.randn`` call for the whole batch, which
    yields the same values as the per-problem, per-mode calls of
    Initialization.py:61-83 taken one after the other.  Column balancing
    (Conversion.py:361-387) is applied to all columns at once.  A draw that
    hits an exact zero (probability ~0) falls back to the per-problem path,
    whose zero replacement draws extra values."""
    n = len(Rs)
    L = core_dims.shape[1]
    sizes = core_dims.astype(np.int64) * Rs.astype(np.int64)[:, None]          # (n, L) block sizes
    total = int(sizes.sum())
    state = np.random.get_state()
    vals = np.random.randn(total)
    if np.any(vals == 0.0):
        np.random.set_state(state)
        for p in range(n):
            f = _equalize_random([int(d) for d in core_dims[p]], int(Rs[p]))
            xh[x_off[p]:x_off[p] + sum(W.size for W in f)] = np.concatenate([W.flatten('F') for W in f])
        return
    # block (p, l): d x R values, row-major as drawn
    bsz = sizes.ravel()
    bstart = np.concatenate([[0], np.cumsum(bsz)[:-1]])
    bd = np.repeat(core_dims.ravel().astype(np.int64), bsz)                    # d of each value's block
    bR = np.repeat(np.repeat(Rs.astype(np.int64), L), bsz)                      # R of each value's block
    within = np.arange(total, dtype=np.int64) - np.repeat(bstart, bsz)
    row, col = within // bR, within % bR
    # column ids: problem p, column r -> one id per (p, r); block ids -> (p, l)
    prob = np.repeat(np.repeat(np.arange(n, dtype=np.int64), L), bsz)
    roff = np.concatenate([[0], np.cumsum(Rs.astype(np.int64))[:-1]])
    pc = roff[prob] + col                                                        # (p, r) id
    mode = np.repeat(np.tile(np.arange(L, dtype=np.int64), n), bsz)
    lc = pc * L + mode                                                           # (p, r, l) id
    nrm = np.sqrt(np.bincount(lc, weights=vals * vals, minlength=int(Rs.sum()) * L)).reshape(-1, L)
    prod = np.prod(nrm, axis=1)
    ok = prod != 0.0
    g = np.where(ok, prod, 1.0) ** (1.0 / L)
    scale = np.where(ok[:, None], g[:, None] / np.where(nrm == 0, 1.0, nrm), 1.0)   # (sum R, L)
    scaled = vals * scale.ravel()[lc]
    # destination: problem offset + mode offset + column-major position r * d + i
    moff = np.concatenate([np.zeros((n, 1), dtype=np.int64), np.cumsum(sizes, axis=1)[:, :-1]], axis=1).ravel()
    dst = x_off[prob] + np.repeat(moff, bsz) + col * bd + row
    xh[dst] = scaled


def _equalize_random(dims, R):
    f = [np.random.randn(d, R) for d in dims]
    for l in range(len(dims)):
        W = f[l]
        z = np.argwhere(W == 0.0)
        for i, r in z:
            W[i, r] = 1e-4 * np.random.randn() * np.linalg.norm(W)
    nr = np.stack([np.linalg.norm(W, axis=0) for W in f])      # (L, R)
    p = np.prod(nr, axis=0)
    ok = p != 0.0
    g = np.where(ok, p, 1.0) ** (1.0 / len(dims))
    for l in range(len(dims)):
        scale = np.where(ok, g / np.where(nr[l] == 0, 1.0, nr[l]), 1.0)
        f[l] = f[l] * scale[None, :]
    return f


def _tuned_launch(prec, L, core_dims, Rs, work, dd, launch):
    """(tile, order) for this batch from the autotuner, timing candidates on a
    sample of the batch's own problems (their outputs are rewritten by the
    full launch)."""
    import torch
    n = len(Rs)
    mc, mr = int(core_dims.max()), int(Rs.max())
    key = tuner.signature(prec, L, mc, mr, n)
    tu = tuner.tuner()
    hit = tu.lookup(key)
    cands = tuner.candidates(mc, mr)
    if hit is not None and hit in cands:
        return hit
    sm = torch.cuda.get_device_properties(0).multi_processor_count
    idx = tuner.sample_indices(n, 2 * sm)

    def run(c):
        tile, order = c
        sel = idx[tuner.order_largest_first(work[idx])] if order == 'largest_first' else idx
        stream = torch.cuda.current_stream()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        launch(dd[sel], tile)            # warm-up (first use of a kernel variant)
        a.record(stream)
        launch(dd[sel], tile)
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b) / 1e3
    return tu.choose(key, cands, run)


def cpd_batch(tensors, ranks, options=None, timings=None, tune=True):
    """CPD of every tensor in ``tensors`` with the matching rank in ``ranks``.

    Returns a list of ``(factors, output)`` pairs like ``cpd``.  Dense FP32 or
    FP64 inputs (NumPy or torch); every dimension <= 64; method 'dGN'.
    ``timings`` (a dict), when given, receives the wall seconds of each stage
    (the device is synchronised between stages, so only for profiling).
    ``tune``: pick the engine's tile and problem order with the autotuner
    (``tuner.py``; the first batch of a new size class pays for the timing);
    ``options.tile`` (1, 2 or 4) forces a tile with the largest-first order.
    Methods the batched engine does not run (``method='als'``, the 'als' and
    'direct' inner methods) are solved problem by problem with ``cpd``.
    """
    _dev.require_cuda()
    import time as _time
    _t = [_time.perf_counter()]

    def _mark(name):
        if timings is not None:
            torch.cuda.synchronize()
            now = _time.perf_counter()
            timings[name] = timings.get(name, 0.0) + now - _t[0]
            _t[0] = now
    o = make_options(options)
    n = len(tensors)
    if n == 0:
        return []
    if isinstance(ranks, int):
        ranks = [ranks] * n
    from .stepped import uses_stepped
    if o.method != 'dGN' or uses_stepped(o):
        from .api import cpd
        return [cpd(T, int(r), o) for T, r in zip(tensors, ranks)]
    lib = _lib.load()
    prec = o.precision if o.precision in ('fp64', 'fp32') else (
        'fp64' if (tensors[0].dtype == np.float64 or tensors[0].dtype == torch.float64) else 'fp32')
    dt = _dev.torch_dtype(prec)
    es = 8 if prec == 'fp64' else 4
    dev = _dev.device()
    L = len(tensors[0].shape)
    if any(len(T.shape) != L for T in tensors):
        raise ValueError("all tensors of a batch must have the same order")
    D = np.array([T.shape for T in tensors], dtype=np.int64)              # (n, L)
    Rs = np.array([int(r) for r in ranks], dtype=np.int64)
    # the input checks of Auxiliar.py:24-78, vectorised; the first problem that
    # fails is passed to consistency() for the reference's message
    bad = np.any(D == 1, axis=1) | (Rs < 1) | np.array([type(r) != int and not isinstance(r, np.integer)
                                                        for r in ranks])
    if L == 3:
        bad |= Rs > np.min(np.stack([D[:, 0] * D[:, 1], D[:, 0] * D[:, 2], D[:, 1] * D[:, 2]]), axis=0)
    if L > 3:
        bad |= Rs == 1
    if o.symm:
        bad |= np.any(D != D[:, :1], axis=1)
    consistency(int(Rs[0]) if not np.any(bad) else ranks[int(np.argmax(bad))],
                tuple(int(v) for v in D[int(np.argmax(bad)) if np.any(bad) else 0]), o)
    if np.any(bad):     # consistency() above raised unless the vector test was stricter
        raise ValueError("problem %d failed the input checks" % int(np.argmax(bad)))
    # sort_dims per problem (stable order on ties, as NumPy's argsort of a short array)
    order_arr = np.argsort(-D, axis=1, kind='stable')
    S_arr = np.take_along_axis(D, order_arr, axis=1)
    orders = list(order_arr)
    shapes = S_arr.tolist()
    if int(S_arr.max()) > 64:
        raise ValueError("cpd_batch handles dimensions up to 64; use cpd for larger tensors")
    N = np.prod(S_arr, axis=1)
    M_arr = np.minimum(Rs[:, None], S_arr)                                # min(R, d_l)
    mins = M_arr.tolist()

    def _offsets(sizes, a=64):
        al = (sizes + a - 1) // a * a
        return np.concatenate([[0], np.cumsum(al)]).astype(np.int64)
    # one allocation per field, per-problem offsets (elements)
    t_off = _offsets(N)
    w_off = _offsets(2 * N)
    u_off = _offsets(np.sum(M_arr * S_arr, axis=1))
    c_off = _offsets(np.prod(M_arr, axis=1))
    s_off = _offsets(np.sum(M_arr, axis=1), 8)
    # pinned staging buffer: each tensor copied as it is (contiguous copies,
    # several host threads), one H2D copy, then the mode permutation of every
    # problem on the device (tfx_batch_permute)
    pinned = torch.empty(int(t_off[-1]), dtype=torch.float64 if prec == 'fp64' else torch.float32, pin_memory=True)
    host = pinned.numpy()

    hd = host.dtype
    arrs = []
    for T in tensors:
        a = T.detach().cpu().numpy() if isinstance(T, torch.Tensor) else np.asarray(T)
        if a.dtype != hd or not a.flags.c_contiguous:
            a = np.ascontiguousarray(a, dtype=hd)
        arrs.append(a)
    srcp = np.array([a.ctypes.data for a in arrs], dtype=np.uint64)
    nbytes = (N * hd.itemsize).astype(np.int64)
    doff = (t_off[:-1] * hd.itemsize).astype(np.int64)
    lib.tfx_host_gather.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                    ctypes.c_int]
    _lib.check(lib.tfx_host_gather(ctypes.c_void_p(srcp.ctypes.data), ctypes.c_void_p(nbytes.ctypes.data),
                                   ctypes.c_void_p(doff.ctypes.data), n, ctypes.c_void_p(host.ctypes.data),
                                   min(32, os.cpu_count() or 4)))
    _mark('stage_host')
    Traw = pinned.to(dev, non_blocking=False)
    Tbuf = torch.empty_like(Traw)
    _mark('h2d')
    work = torch.empty(int(w_off[-1]), dtype=dt, device=dev)
    Ubuf = torch.empty(int(u_off[-1]), dtype=dt, device=dev)
    Cbuf = torch.empty(max(1, int(c_off[-1])), dtype=dt, device=dev)
    cdims = torch.zeros((n, L), dtype=torch.int32, device=dev)
    sig = torch.zeros(int(s_off[-1]) + 8, dtype=torch.float64, device=dev)
    bd = np.zeros(n, dtype=_BATCH_DT)
    bd['L'] = L
    bd['R'] = Rs
    bd['dims'][:, :L] = S_arr
    bd['tensor'] = Tbuf.data_ptr() + t_off[:-1] * es
    bd['work'] = work.data_ptr() + w_off[:-1] * es
    bd['work_elems'] = w_off[1:] - w_off[:-1]
    bd['Ut'] = Ubuf.data_ptr() + u_off[:-1] * es
    bd['core'] = Cbuf.data_ptr() + c_off[:-1] * es
    bd['core_dims'] = cdims.data_ptr() + np.arange(n) * L * 4
    bd['sigma'] = sig.data_ptr() + s_off[:-1] * 8
    d_bd = torch.empty(n * _BATCH_DT.itemsize, dtype=torch.uint8, device=dev)
    tol = o.tol_mlsvd[0] if isinstance(o.tol_mlsvd, list) else o.tol_mlsvd
    if tol < 0:
        raise NotImplementedError("cpd_batch compresses every problem (tol_mlsvd >= 0)")
    st = ctypes.c_void_p(_dev.stream())
    perm = torch.from_numpy(np.concatenate([np.asarray(od, dtype=np.int32) for od in orders])).to(dev)
    srcp = torch.from_numpy((Traw.data_ptr() + t_off[:-1] * es).astype(np.uint64).view(np.int64)).to(dev)
    lib.tfx_batch_permute.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p]
    _lib.check(lib.tfx_batch_permute(_dev.lib_dtype(prec), ctypes.c_void_p(bd.ctypes.data),
                                     ctypes.c_void_p(d_bd.data_ptr()), n, ctypes.c_void_p(srcp.data_ptr()),
                                     ctypes.c_void_p(perm.data_ptr()), st))
    lib.tfx_batch_mlsvd.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_int, ctypes.c_void_p]
    _lib.check(lib.tfx_batch_mlsvd(_dev.lib_dtype(prec), ctypes.c_void_p(bd.ctypes.data),
                                   ctypes.c_void_p(d_bd.data_ptr()), n, float(tol),
                                   int(o.svd_n_components or 0), st))
    core_dims = cdims.cpu().numpy()
    _mark('mlsvd')
    # starting points (host RNG, problem order) and engine descriptors
    nx = np.array([int(Rs[p]) * int(core_dims[p].sum()) for p in range(n)], dtype=np.int64)
    x_off = np.concatenate([[0], np.cumsum([_al(v) for v in nx])])
    xh = np.zeros(int(x_off[-1]), dtype=np.float64)
    _random_starts(core_dims, Rs, x_off, xh)
    X0 = torch.from_numpy(xh).to(device=dev, dtype=dt)
    best = torch.empty_like(X0)
    ws_b, ws_cache = [], {}
    for p in range(n):       # one query per distinct (core dims, rank)
        key = (tuple(int(d) for d in core_dims[p]), int(Rs[p]))
        v = ws_cache.get(key)
        if v is None:
            dims_c = (ctypes.c_int * L)(*key[0])
            v = ws_cache[key] = int(lib.tfx_dgn_workspace_bytes(_dev.lib_dtype(prec), L, dims_c, key[1]))
        ws_b.append(v)
    ws_off = np.concatenate([[0], np.cumsum([_al(v, 256) for v in ws_b])])
    WS = torch.empty(int(ws_off[-1]), dtype=torch.uint8, device=dev)
    m = int(o.maxiter)
    budgets = np.zeros((n, m), dtype=np.int32)
    for it in range(m):      # one draw per iteration for the whole batch (iteration-major order)
        inner = _inner_of(o, it)
        if inner == 'cg':
            draw = np.random.randint(int(1 + it ** 0.4), int(2 + it ** 0.9), size=n)
            budgets[:, it] = 1 + (L - 2) * (o.cg_factor * draw).astype(np.int64)
        elif inner == 'cg_static':
            budgets[:, it] = o.cg_maxiter
        else:
            raise NotImplementedError("inner_method %r" % (inner,))
    B = torch.from_numpy(budgets).to(dev)
    stats = torch.zeros((n, 4 * m), dtype=torch.float64, device=dev)
    result = torch.zeros((n, 4), dtype=torch.int32, device=dev)
    info = torch.zeros((n, 8), dtype=torch.float64, device=dev)
    dd = np.zeros(n, dtype=_DGN_DT)
    dd['L'] = L
    dd['R'] = Rs
    dd['dims'][:, :L] = core_dims
    dd['tensor'] = Cbuf.data_ptr() + c_off[:-1] * es
    dd['x'] = X0.data_ptr() + x_off[:-1] * es
    dd['best'] = best.data_ptr() + x_off[:-1] * es
    dd['work'] = WS.data_ptr() + ws_off[:-1]
    dd['budgets'] = B.data_ptr() + np.arange(n) * m * 4
    dd['stats'] = stats.data_ptr() + np.arange(n) * 4 * m * 8
    dd['result'] = result.data_ptr() + np.arange(n) * 16
    dd['info'] = info.data_ptr() + np.arange(n) * 64
    d_dd = torch.empty(n * _DGN_DT.itemsize, dtype=torch.uint8, device=dev)
    opt = _lib.DgnOptions()
    opt.maxiter = m
    opt.tol, opt.tol_step, opt.tol_improv = float(o.tol), float(o.tol_step), float(o.tol_improv)
    opt.tol_grad, opt.tol_jump, opt.cg_tol = float(o.tol_grad), float(o.tol_jump), float(o.cg_tol)
    if isinstance(o.init_damp, list):
        raise NotImplementedError("cpd_batch takes a scalar init_damp")
    opt.init_damp = float(o.init_damp)
    opt.symm = 1 if o.symm else 0
    opt.factors_norm = float(o.factors_norm)
    # Initialization.py:83: a symmetrising transform of the start leaves one array L times
    opt.aliased = 1 if (o.symm and float(o.factors_norm) <= 0 and not isinstance(o.initialization, list)) else 0
    cl = int(o.cluster or 1)
    _mark('starts_and_descriptors')

    def _launch(desc, tile):
        opt.tile = int(tile)
        desc = np.ascontiguousarray(desc)
        _lib.check(lib.tfx_dgn_solve(_dev.lib_dtype(prec), ctypes.cast(desc.ctypes.data, ctypes.POINTER(_lib.DgnProblem)),
                                     ctypes.c_void_p(d_dd.data_ptr()), len(desc), ctypes.byref(opt), cl, st))
    work = np.prod(core_dims.astype(np.float64), axis=1) * Rs
    forced = getattr(o, 'tile', None)
    if forced:
        tile, order = int(forced), 'largest_first'
    elif not tune or cl != 1:
        tile, order = 0, 'given'
    else:
        tile, order = _tuned_launch(prec, L, core_dims, Rs, work, dd, _launch)
    perm = tuner.order_largest_first(work) if order == 'largest_first' else np.arange(n)
    _launch(dd[perm], tile)
    if timings is not None:
        timings['engine_config'] = (tile, order)
    _mark('dgn_engine')
    # decompression and final errors
    f_sz = [int(Rs[p]) * sum(shapes[p]) for p in range(n)]
    f_off = np.concatenate([[0], np.cumsum([_al(v) for v in f_sz])])
    WF = torch.empty(int(f_off[-1]), dtype=dt, device=dev)
    pc = torch.from_numpy((best.data_ptr() + x_off[:-1] * es).astype(np.uint64).view(np.int64)).to(dev)
    pf = torch.from_numpy((WF.data_ptr() + f_off[:-1] * es).astype(np.uint64).view(np.int64)).to(dev)
    lib.tfx_batch_decompress.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p]
    lib.tfx_batch_residual.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p]
    _lib.check(lib.tfx_batch_decompress(_dev.lib_dtype(prec), ctypes.c_void_p(d_bd.data_ptr()), n,
                                        ctypes.c_void_p(pc.data_ptr()), ctypes.c_void_p(pf.data_ptr()), st))
    res2 = torch.empty(2 * n, dtype=torch.float64, device=dev)
    _lib.check(lib.tfx_batch_residual(_dev.lib_dtype(prec), ctypes.c_void_p(d_bd.data_ptr()), n,
                                      ctypes.c_void_p(pf.data_ptr()), ctypes.c_void_p(res2.data_ptr()), st))
    wf = WF.double().cpu().numpy()
    r2 = res2.cpu().numpy()
    info_h = info.cpu().numpy()
    st_h = stats.cpu().numpy()
    rs_h = result.cpu().numpy()
    _lib.check_solve_status(rs_h)
    _mark('decompress_residual_d2h')
    out = []
    for p in range(n):
        R = int(Rs[p])
        fl, s0 = [], int(f_off[p])
        for d in shapes[p]:
            fl.append(wf[s0:s0 + d * R].reshape(R, d).T.copy())
            s0 += d * R
        factors = [None] * L
        for l in range(L):
            factors[orders[p][l]] = fl[l]
        k = int(rs_h[p, 1])
        op = Output()
        op.num_steps = k
        op.rel_error = float(np.sqrt(r2[2 * p]) / np.sqrt(r2[2 * p + 1]))
        op.accuracy = max(0, 100 * (1 - op.rel_error))
        op.errors = [st_h[p, :k].copy(), np.array([0])]
        op.step_sizes = [st_h[p, m:m + k].copy(), np.array([0])]
        op.improv = [st_h[p, 2 * m:2 * m + k].copy(), np.array([0])]
        op.gradients = [st_h[p, 3 * m:3 * m + k].copy(), np.array([0])]
        op.stop = [int(rs_h[p, 0]), 8]
        op.options = o
        op.matvecs = int(info_h[p, 4])
        op.core_dims = [int(d) for d in core_dims[p]]
        out.append((factors, op))
    _mark('assemble')
    return out
