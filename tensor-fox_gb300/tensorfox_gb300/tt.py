"""Tensor-train CPD, ``method='ttcpd'`` (TensorFox.py:256-421, 658-817, 1042-1065;
Auxiliar.py:365-527; Conversion.py:460-494).

A tensor of order L is compressed by the MLSVD, split by a TT-SVD into the
cores d_0 x R, R x d_1 x R, ..., R x d_{L-1}; the first inner core gets a full
third-order CPD (``tricpd``, best of ``options.trials``), every further core a
CPD whose first factor is fixed to pinv(Z^T) of the previous core's last factor
(``bicpd``: ALS with a fixed mode when bi_method is 'als', else dGN with the
fixed factor put back after every step), and the factors of the tensor are
assembled from the cores' CPDs.

The TT-SVD runs on the device.  Every unfolding is kept column-major, so the
reference's Fortran-order reshapes cost nothing: a column-major (rows x cols)
matrix is the row-major (cols x rows) tensor ``Mt`` of the same memory.  Its
leading R left singular vectors come from the eigen-decomposition of the small
side's Gram (Jacobi on the device; U = M W / sigma when the columns are the
small side), or, when both sides are large, from a Rayleigh-Ritz step on the
row Gram.  Signs follow the reference's scikit-learn SVD: the largest |entry|
of every left singular vector is positive.  The reference's randomized SVD is
taken at full rank (an exact SVD up to rounding); its Gaussian block is drawn
here too, so NumPy's global RNG stays in step with the reference.

The inner cores' unfoldings are orthonormal, so the MLSVD basis of those modes
is not unique: runs that differ in the last bit of a core can reach the same
CPD with its columns permuted (the reference does the same).  Parity is
therefore checked by the final error and the congruence of the factors.
"""
import numpy as np
import torch

from . import _dev, kernels
from .compression import mlsvd_device, top_eig

_JACOBI_MAX = {torch.float64: 96, torch.float32: 128}


def _left_singular(Mt, rows, cols, r):
    """Leading r left singular vectors of M (rows x cols, column-major, given as
    the row-major (cols, rows) tensor Mt).  Returns Ut (r x rows, row-major:
    U column-major) with the signs fixed."""
    low = min(rows, cols)
    omega = np.random.normal(size=(low, low + 10))      # the reference's draw
    jm = _JACOBI_MAX.get(Mt.dtype, 96)
    if rows <= jm:
        G = kernels.matmul(Mt, Mt, transA=True)          # M M^T (rows x rows)
        ev, V = kernels.sym_eig(G)
        Ut = V[:r].contiguous()
    elif cols <= jm:
        G = kernels.matmul(Mt, Mt, transB=True)          # M^T M (cols x cols)
        ev, V = kernels.sym_eig(G)
        lam = ev[:r].double().cpu().numpy()
        sig = np.sqrt(np.maximum(lam, 0.0))
        inv = np.where(sig > 0, 1.0 / np.where(sig > 0, sig, 1.0), 0.0)
        Ut = kernels.matmul(V[:r].contiguous(), Mt)      # (W^T M^T) = (M W)^T, r x rows
        Ut = Ut * torch.from_numpy(inv).to(Ut.device, Ut.dtype)[:, None]
        Ut = Ut.contiguous()
    else:
        G = kernels.matmul(Mt, Mt, transA=True)
        Ut, _ = top_eig(G, r, omega if omega.shape[0] == rows else None)
        return Ut
    kernels.flip_signs(Ut)
    return Ut


def cpdtt_device(Td, R):
    """TT cores of the C-order device tensor Td (TensorFox.py:1042-1065):
    [G0 (d0 x R), G1 (R x d1 x R), ..., G_{L-1} (R x d_{L-1})], device tensors."""
    dims = [int(d) for d in Td.shape]
    L = len(dims)
    # the F-order memory of Td: its axes reversed, C-contiguous
    Mt = Td.permute(*reversed(range(L))).contiguous().reshape(-1)
    G = []
    r1 = 1
    for l in range(L - 1):
        rows = r1 * dims[l]
        cols = int(np.prod(dims[l + 1:]))
        M2 = Mt.view(cols, rows)
        r2 = R
        Ut = _left_singular(M2, rows, cols, min(r2, rows, cols))
        k = Ut.shape[0]
        if k < r2:   # fewer singular directions than R: zero-padded (rank-deficient unfolding)
            pad = torch.zeros((r2 - k, rows), dtype=Ut.dtype, device=Ut.device)
            Ut = torch.cat([Ut, pad])
        Vn = kernels.matmul(M2, Ut, transB=True)          # (cols x R) row-major = U^T M column-major
        if r1 == 1:
            G.append(Ut.t().contiguous())                 # d0 x R
        else:
            G.append(Ut.view(r2, dims[l], r1).permute(2, 1, 0).contiguous())   # r1 x d_l x R
        Mt = Vn.contiguous().reshape(-1)
        r1 = r2
    G.append(Mt.view(dims[-1], r1).t().contiguous())     # R x d_{L-1}
    return G


def _inflate(S, R, dims):
    """Conversion.py:460-480: modes shorter than R padded with 1e-12 * randn."""
    new = [d if d >= R else R for d in dims]
    out = 1e-12 * np.random.randn(*new)
    out = torch.from_numpy(out).to(S.device, S.dtype)
    out[tuple(slice(d) for d in dims)] = S
    return out


def bicpd(Td, R, fixed, options, prec):
    """Third-order CPD of the device tensor Td with the factor ``fixed = [W, l]``
    kept (TensorFox.py:658-817) on the MLSVD core: ALS when bi_method is 'als'
    (the last iterate), else dGN with the options' inner method (the best
    iterate).  Returns (X, Y, Z, output) as NumPy arrays in Td's mode order."""
    from .api import Output, starting_point_core, _run_dgn
    from .als import als_device
    o = options
    use_als = o.bi_method_parameters[0] == 'als'
    dt = _dev.torch_dtype(prec)
    dims = [int(d) for d in Td.shape]
    Tsize = float(np.sqrt(kernels.tensor_norms(Td).cpu().numpy()[0]))
    S, Uts, sigmas, core = mlsvd_device(Td, R, o)
    init = starting_point_core(S, core, R, o, vectorized=(prec == 'fp32'))
    W, fl = fixed
    Wd = torch.from_numpy(np.asarray(W, dtype=np.float64)).to(Td.device, dt)
    init[fl] = kernels.matmul(Uts[fl], Wd).double().cpu().numpy()
    x0 = torch.from_numpy(_dev.flat_factors(init)).to(Td.device, dt)
    if use_als:
        x, best, stats, res, info = als_device(S, x0, R, o, prec, fl)
        n = int(res[1])
        m = int(o.maxiter)
        ss, er, im, gr, st = (stats[m:m + n].copy(), stats[:n].copy(), stats[2 * m:2 * m + n].copy(),
                              stats[3 * m:3 * m + n].copy(), int(res[0]))
    else:
        x, ss, er, im, gr, st = _run_dgn(S, x0, R, o, prec, fix_mode=fl)
        n = len(er)
    xs = x.double().cpu().numpy()
    out, s = [], 0
    for l in range(3):
        c = core[l]
        f = xs[s:s + c * R].reshape(R, c).T
        s += c * R
        if l == fl:
            out.append(np.asarray(W, dtype=np.float64))
        else:
            U = Uts[l].double().cpu().numpy().T            # d_l x n_l
            out.append(U @ f)
    flat = torch.from_numpy(_dev.flat_factors(out)).to(Td.device, dt)
    r2 = float(kernels.cp_residual_sq(Td, dims, flat, R).cpu().numpy()[0])
    op = Output()
    op.num_steps = n
    op.rel_error = float(np.sqrt(max(r2, 0.0))) / Tsize
    op.accuracy = max(0, 100 * (1 - op.rel_error))
    op.errors = [er, np.array([0])]
    op.step_sizes = [ss, np.array([0])]
    op.improv = [im, np.array([0])]
    op.gradients = [gr, np.array([0])]
    op.stop = [st, 5]
    op.options = o
    return out[0], out[1], out[2], op


def _tricpd(G1, R, options):
    """tricpd on a core: the method is dGN unless it is 'als' (TensorFox.py:564-570)."""
    from .api import tricpd
    saved = options.method
    options.method = 'als' if saved == 'als' else 'dGN'
    try:
        return tricpd(G1, R, options)
    finally:
        options.method = saved


def sweep_schedule(L, epochs):
    """The order in which the inner cores G[1..L-2] are decomposed after the
    first one, as ``(core, fixed_mode, record)`` steps (Auxiliar.py:413-527).

    The epoch count is made odd.  Even epochs walk forward and fix each core's
    first factor (mode 0) from the previous core's last one; odd epochs walk
    backward and fix the last factor (mode 2) from the previous core's first
    one.  Forward walks start at core 2; for order 3 the first backward walk
    moves the start to core 1, and backward walks cover cores 1 .. L-3 (core 1
    for order 3).  ``record``: the step's result is the one kept for its core --
    forward steps of the last epoch, backward steps of the one before it."""
    epochs = epochs + 1 - epochs % 2
    steps = []
    fwd_start = 2
    for e in range(epochs):
        if e % 2 == 0:
            steps += [(l, 0, e == epochs - 1) for l in range(fwd_start, L - 1)]
        else:
            if L == 3:
                fwd_start = 1
            top = L - 1 if L == 3 else L - 2
            steps += [(l, 2, e == epochs - 2) for l in range(top - 1, 0, -1)]
    return steps


def _best_of(max_trials, trial):
    """The trial with the smallest relative error, stopping below 1e-4."""
    best = None
    for _ in range(max_trials):
        f, out = trial()
        if best is None or out.rel_error < best[1].rel_error:
            best = (f, out)
            if out.rel_error < 1e-4:
                break
    return best


def cpd_cores(G, max_trials, epochs, R, options, prec):
    """CPDs of the inner TT cores (Auxiliar.py:413-527): core 1 by ``tricpd``,
    then every step of ``sweep_schedule`` by ``bicpd`` with one factor fixed to
    the pseudo-inverse link of its neighbour's result.  Returns the kept
    factors and outputs per inner core and the last step's third factor."""
    L = len(G)
    kept = [None] * (L - 2)
    outs = [None] * (L - 2)
    link, outs[0] = _best_of(max_trials, lambda: _tricpd(G[1], R, options))
    link = list(link)
    kept[0] = link
    for core, fmode, record in sweep_schedule(L, epochs):
        fixed = np.linalg.pinv((link[2] if fmode == 0 else link[0]).T)

        def trial():
            X, Y, Z, out = bicpd(G[core], R, [fixed, fmode], options, prec)
            return ([fixed, Y, Z] if fmode == 0 else [X, Y, fixed]), out
        link, out = _best_of(max_trials, trial)
        if record:
            kept[core - 1], outs[core - 1] = link, out
    return kept, outs, link[2]


def highcpd(S, R, options, prec):
    """TensorFox.py:368-421: TT cores of S, their CPDs, the factors of S."""
    L = S.dim()
    options.refine = False
    G = cpdtt_device(S, R)
    cpd_list, outputs, bZ = cpd_cores(G, int(options.trials), int(options.epochs), R, options, prec)
    G0 = G[0].double().cpu().numpy()
    GL = G[-1].double().cpu().numpy()
    factors = [G0 @ cpd_list[0][0]]
    for l in range(L - 2):
        factors.append(np.asarray(cpd_list[l][1], dtype=np.float64))
    factors.append(GL.T @ bZ)
    # equalize (Conversion.py:361-387)
    for r in range(R):
        nr = np.array([np.linalg.norm(f[:, r]) for f in factors])
        if np.prod(nr) != 0.0:
            g = np.prod(nr) ** (1 / L)
            for l in range(L):
                factors[l][:, r] = (g / nr[l]) * factors[l][:, r]
    return factors, outputs


def cpd_tt(T, R, options):
    """cpd with method 'ttcpd' (TensorFox.py:256-365), dense or
    ``[data, idxs, dims]`` input (sparse: the reference's sparse MLSVD, and the
    final error on the stored entries)."""
    from .api import Output, _precision, sort_dims, unsort_dims
    o = options
    sparse_in = isinstance(T, list)
    if sparse_in:
        from .sparse import DeviceCOO, mlsvd_sparse_device, sparse_residual_sq
        data, idxs, dims0 = T
        data = np.asarray(data, dtype=np.float64)
        dims0 = np.asarray(dims0)
        idxs = np.asarray(idxs, dtype=np.int64).reshape(len(data), -1)
        prec = o.precision if o.precision in ('fp64', 'fp32') else 'fp64'
        dt = _dev.torch_dtype(prec)
        ordering = np.argsort(-dims0)
        dims = [int(d) for d in dims0[ordering]]
        X = DeviceCOO(data, idxs, dims, dt, perm=ordering)
        Tsize = float(np.linalg.norm(data))
        tol = o.tol_mlsvd[0] if isinstance(o.tol_mlsvd, list) else o.tol_mlsvd
        if tol < 0:            # TensorFox.py:275-280
            o.tol_mlsvd = 1e-16
        S, Uts, sigmas = mlsvd_sparse_device(X, R, o)
        core = [int(u.shape[0]) for u in Uts]
    else:
        prec = _precision(T, o)
        dt = _dev.torch_dtype(prec)
        shape = tuple(int(d) for d in T.shape)
        ordering = sort_dims(shape)
        if isinstance(T, torch.Tensor):
            Td = T.to(device=_dev.device(), dtype=dt).permute(*[int(i) for i in ordering]).contiguous()
        else:
            Td = _dev.to_device(np.transpose(np.asarray(T), ordering), dt)
        dims = [int(d) for d in Td.shape]
        Tsize = float(np.sqrt(kernels.tensor_norms(Td).cpu().numpy()[0]))
        S, Uts, sigmas, core = mlsvd_device(Td, R, o)
        core = [int(c) for c in core]
    infl = R > min(core)
    if infl:
        S = _inflate(S, R, core)
    o.trunc_dims = 0
    factors, outputs = highcpd(S.contiguous(), R, o, prec)
    if infl:
        factors = [factors[l][:core[l], :] for l in range(len(core))]
    full = []
    for l in range(len(dims)):
        U = Uts[l].double().cpu().numpy().T                 # d_l x n_l
        full.append(U @ factors[l])
    if sparse_in:            # error on the stored entries (Auxiliar.py:155-159)
        frm = [torch.from_numpy(np.ascontiguousarray(f)).to(S.device, dt) for f in full]
        r2 = float(sparse_residual_sq(X, frm).cpu().numpy()[0])
    else:
        flat = torch.from_numpy(_dev.flat_factors(full)).to(Td.device, dt)
        r2 = float(kernels.cp_residual_sq(Td, dims, flat, R).cpu().numpy()[0])
    rel = float(np.sqrt(max(r2, 0.0))) / Tsize
    full = unsort_dims(full, ordering)
    out = Output()
    out.num_steps = int(sum(x.num_steps for x in outputs))
    out.rel_error = rel
    out.accuracy = max(0, 100 * (1 - rel))
    out.cpd_output = outputs
    out.options = o
    return full, out
