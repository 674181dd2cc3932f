"""CPU oracle for the damped Gauss-Newton CPD path of Tensor Fox v1.2.1.

TEST INFRASTRUCTURE ONLY.  This module restates, in vectorised NumPy, the
algorithm of the reference's dGN path so that the CUDA implementation can be
checked against it.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
legs of ``bench.py`` may import it; the product package never does.

Parity pin: every function below is compared against golden vectors produced by
running the reference itself (``tests/golden/make_golden.py``), see
``tests/test_oracle_golden.py``.

Conventions shared with the reference
-------------------------------------
* factors ``W[l]`` are ``(d_l, R)`` float arrays; the flat point ``x`` is
  ``concat_l vec_F(W[l])`` (GaussNewton.py:125, Conversion.py:21-44);
* the mode-``m`` unfolding uses Kolda's column order (Critical.py:124-146):
  ``unfold(T, m) == moveaxis(T, m-1, 0).reshape(d_m, -1, order='F')``;
* NumPy's global RNG is used exactly where the reference uses it, so a seeded
  run draws the same numbers in the same order.
"""
from copy import deepcopy

import numpy as np
from numpy.linalg import norm
from scipy.linalg import qr as sp_qr, svd as sp_svd

# ----------------------------------------------------------------------------
# options (Auxiliar.py:242-362)
# ----------------------------------------------------------------------------
_DEFAULTS = dict(maxiter=200, tol=1e-16, tol_step=1e-6, tol_improv=1e-6, tol_grad=1e-6,
                 tol_jump=10, method='dGN', inner_method='cg', cg_maxiter=100, cg_factor=1,
                 cg_tol=1e-16, initialization='random', trunc_dims=0,
                 mlsvd_method='seq', tol_mlsvd=1e-16, init_damp=1, refine=False, symm=False,
                 factors_norm=0, trials=3, display=0, epochs=1, gpu=False, mkl_dot=True,
                 svd_n_components=None)


class Options:
    pass


def make_options(options=None):
    """Defaults overridden by any attribute the caller's object defines (Auxiliar.py:256-353)."""
    out = Options()
    for k, v in _DEFAULTS.items():
        setattr(out, k, v)
    out.bi_method_parameters = ['als', 500, 1e-6]
    if options is None or options is False:
        return out
    names = dir(options)
    for k in _DEFAULTS:
        if k in names:
            setattr(out, k, getattr(options, k))
    if out.gpu and 'mlsvd_method' not in names:          # Auxiliar.py:359-360
        out.mlsvd_method = 'gpu'
    return out


# ----------------------------------------------------------------------------
# layout helpers (Conversion.py, Critical.py)
# ----------------------------------------------------------------------------
def unfold(T, mode):
    """Mode-``mode`` (1-based) unfolding, Kolda order (Conversion.py:207-252).

    Column ``s = sum_{k != m} i_k prod_{j < k, j != m} d_j``: a C-order reshape of
    the axes (m, last other, ..., first other), done as one transposing copy.
    """
    m = mode - 1
    others = [k for k in range(T.ndim) if k != m]
    perm = [m] + others[::-1]
    return np.ascontiguousarray(np.transpose(T, perm), dtype=np.float64).reshape(T.shape[m], -1)


def foldback(Tl, mode, dims):
    """Inverse of :func:`unfold` (Conversion.py:305-315)."""
    dims = tuple(int(v) for v in dims)
    m = mode - 1
    moved = (dims[m],) + tuple(d for i, d in enumerate(dims) if i != m)
    return np.moveaxis(np.asarray(Tl).reshape(moved, order='F'), 0, m).copy()


def khatri_rao(A, B):
    """Row-block Khatri-Rao product: row ``i*b1+k`` is ``A[i]*B[k]`` (MultilinearAlgebra.py:248-274)."""
    return (A[:, None, :] * B[None, :, :]).reshape(A.shape[0] * B.shape[0], A.shape[1])


def kr_chain(mats):
    """``mats[0] ⊙ mats[1] ⊙ ...`` with the first matrix varying slowest."""
    M = mats[0]
    for X in mats[1:]:
        M = khatri_rao(M, X)
    return M


def x2cpd(x, factors, eq=True):
    """Writes the flat point into the factor matrices, then balances them (Conversion.py:21-49)."""
    R = factors[0].shape[1]
    s = 0
    for l in range(len(factors)):
        d = factors[l].shape[0]
        factors[l][:, :] = x[s:s + d * R].reshape(R, d).T
        s += d * R
    if eq:
        factors = equalize(factors, R)
    return factors


def cpd2flat(factors):
    return np.concatenate([W.flatten('F') for W in factors])


def equalize(factors, R):
    """Rescales column r of every mode to the geometric mean of their norms (Conversion.py:361-387)."""
    L = len(factors)
    for r in range(R):
        nr = np.array([norm(factors[l][:, r]) for l in range(L)])
        p = np.prod(nr)
        if p != 0.0:
            g = p ** (1 / L)
            for l in range(L):
                factors[l][:, r] = (g / nr[l]) * factors[l][:, r]
    return factors


def transform(factors, symm, factors_norm):
    """Symmetrisation / fixed-norm rescaling (Conversion.py:412-444); both default off."""
    L = len(factors)
    if symm:
        # in place, as in the reference: ``s`` IS factors[0], and afterwards every
        # entry of the list is the same array.  When the list already holds one
        # array L times (any dGN iteration after the first), ``s += factors[l]``
        # doubles it L - 1 times, so the result is 2^(L-1)/L times the array.
        s = factors[0]
        for l in range(1, L):
            s += factors[l]
        factors[0] = s / L
        for l in range(1, L):
            factors[l] = factors[0]
    if factors_norm > 0:
        for l in range(L):
            factors[l] = factors_norm * (1 / norm(factors[l])) * factors[l]
    return factors


def cpd2unfold1(factors):
    """``W0 · (W_{L-1} ⊙ ... ⊙ W_1)^T`` (Conversion.py:117-141)."""
    L = len(factors)
    M = factors[1]
    for l in range(2, L):
        M = khatri_rao(factors[l], M)
    return factors[0] @ M.T


def cpd2tens(factors):
    """Dense tensor of a CPD (Conversion.py:52-79)."""
    dims = [W.shape[0] for W in factors]
    return foldback(cpd2unfold1(factors), 1, dims)


def fastnorm(A, B):
    """Frobenius norm of ``A - B`` (Critical.py:14-22)."""
    return float(np.sqrt(np.sum((np.asarray(A) - np.asarray(B)) ** 2)))


def sparse_fastnorm(data, idxs, dims, factors):
    """Norm of ``data - model(idxs)`` over the stored entries only (Critical.py:25-53)."""
    idxs = np.asarray(idxs).astype(np.int64)
    R = factors[0].shape[1]
    p = np.ones((len(idxs), R))
    for l in range(len(dims)):
        p *= factors[l][idxs[:, l], :]
    approx = p.sum(axis=1)
    return float(norm(np.asarray(data, dtype=np.float64) - approx))


# ----------------------------------------------------------------------------
# dGN building blocks (GaussNewton.py)
# ----------------------------------------------------------------------------
def sum_dims_of(dims, R):
    return np.array([R * int(sum(dims[:l])) for l in range(len(dims) + 1)])


def gramians(factors):
    """``Gr[l] = W_l^T W_l``; ``P2[l][k] = ∘_{m∉{l,k}} Gr[m]``; ``P1[l] = ∘_{m≠l} Gr[m]``.

    Follows GaussNewton.py:520-548 including the product order and the untouched
    diagonal blocks ``P2[l][l] = 1`` (they are never read).
    """
    L = len(factors)
    R = factors[0].shape[1]
    Gr = np.array([W.T @ W for W in factors])
    P1 = np.ones((L, R, R))
    P2 = np.ones((L, L, R, R))
    for l in range(1, L):
        for ll in range(l):
            acc = np.ones((R, R))
            for m in range(L):
                if m != l and m != ll:
                    acc = acc * Gr[m]
            P2[l, ll] = acc
            P2[ll, l] = acc
        if l < L - 1:
            P1[l] = P2[l, l - 1] * Gr[l - 1]
        else:
            P1[l] = P2[l, 0] * Gr[0]
    P1[0] = P2[0, 1] * Gr[1]
    return Gr, P1, P2


def regularization(P1, dims, R):
    """Tikhonov diagonal (GaussNewton.py:584-607).

    Reproduces the reference exactly: ``gamma[l, r] = tmp * sqrt(|P1[l][r, r]|)``
    where ``tmp`` is max|P1| of the LAST mode (the running max ``s`` is unused).
    """
    L = len(dims)
    tmp = np.max(np.abs(P1[L - 1]))
    gamma = tmp * np.sqrt(np.abs(np.array([np.diag(P1[l]) for l in range(L)])))
    Gamma = np.concatenate([np.repeat(gamma[l], dims[l]) for l in range(L)])
    return Gamma, gamma


def precond(Gamma, gamma, damp, dims):
    """``M = 1/sqrt(gamma^2 + damp^2 Gamma^2)`` per column block (GaussNewton.py:610-627)."""
    L = len(dims)
    g = np.concatenate([np.repeat(gamma[l], dims[l]) for l in range(L)])
    return 1 / np.sqrt(g ** 2 + damp ** 2 * Gamma ** 2)


def mttkrp(Tl, factors, l):
    """``T_(l) · (W_{L-1} ⊙ ... ⊙ W_{l+1} ⊙ W_{l-1} ⊙ ... ⊙ W_0)`` (GaussNewton.py:411-423)."""
    L = len(factors)
    order = [k for k in reversed(range(L)) if k != l]
    return Tl[l] @ kr_chain([factors[k] for k in order])


def compute_grad(Tl, factors, P1):
    """``g_l = W_l P1_l - T_(l) KR_l`` stacked as vec_F (GaussNewton.py:401-427)."""
    return np.concatenate([(factors[l] @ P1[l] - mttkrp(Tl, factors, l)).T.ravel()
                           for l in range(len(factors))])


def _split(v, dims, R):
    sd = sum_dims_of(dims, R)
    return [v[sd[l]:sd[l + 1]].reshape(R, dims[l]) for l in range(len(dims))]


def matvec(factors, P1, P2, v):
    """Jacobian-free ``J^T J v`` (GaussNewton.py:551-581 with the A/B set-up of :371-377)."""
    L = len(factors)
    R = factors[0].shape[1]
    dims = [W.shape[0] for W in factors]
    V = _split(v, dims, R)
    A = [V[l] @ factors[l] for l in range(L)]
    B = [V[l].T @ P1[l] for l in range(L)]
    out = []
    for l in range(L):
        acc = np.zeros((R, R))
        for ll in range(L):
            if ll != l:
                acc += P2[l, ll] * A[ll]
        out.append((factors[l] @ acc + B[l]).T.ravel())
    return np.concatenate(out)


def cg(Tl, factors, damp, maxiter, tol):
    """Preconditioned, regularised CG for the dGN step (GaussNewton.py:315-398).

    Returns ``(M*y, grad, JT_J_grad, itn+1, residualnorm)`` like the reference.
    """
    L = len(factors)
    R = factors[0].shape[1]
    dims = [W.shape[0] for W in factors]
    nx = R * sum(dims)
    if nx > 100:
        maxiter = min(maxiter, nx)
    else:
        tol = 0
    Gr, P1, P2 = gramians(factors)
    Gamma, gamma = regularization(P1, dims, R)
    M = precond(Gamma, gamma, damp, dims)
    y = np.zeros(nx)
    grad = -compute_grad(Tl, factors, P1)
    JT_J_grad = matvec(factors, P1, P2, grad)
    r = M * grad
    P = r
    rn = float(r @ r)
    if rn == 0.0:
        rn = 1e-6
    itn = 0
    for itn in range(maxiter):
        Q = M * P
        z = matvec(factors, P1, P2, Q) + damp * Gamma * Q
        z = M * z
        den = float(P @ z)
        if den == 0.0:
            den = 1e-6
        alpha = rn / den
        y = y + alpha * P
        r = r - alpha * z
        rn_new = float(r @ r)
        beta = rn_new / rn
        rn = rn_new
        if itn == 0:
            # GaussNewton.py:349 binds P to the residual array itself, and the
            # in-place update at :388 moves it along, so the first new direction
            # is (1 + beta) * r instead of r + beta * r_old.
            P = r + beta * r
        else:
            P = r + beta * P
        if rn <= tol:
            break
    return M * y, grad, JT_J_grad, itn + 1, rn


def cg_budget(it, L, cg_factor):
    """CG iteration cap of the 'cg' inner method; draws from NumPy's global RNG (GaussNewton.py:267)."""
    return 1 + (L - 2) * int(cg_factor * np.random.randint(1 + it ** 0.4, 2 + it ** 0.9))


def hessian(factors, P1, P2, exact=False):
    """The reference's Gauss-Newton matrix in the flat point's order
    (GaussNewton.py:656-701).

    Diagonal blocks ``kron(P1[l], I_{d_l})``; block (l, m), l > m, entry
    ((l, r, i), (m, s, j)) = ``P2[l, m][r, s] * W_l[i, s] * W_m[j, r]``, where
    (l, r, i) is position ``sum_dims[l] + r d_l + i`` of the flat point, and
    block (m, l) its transpose.  That is ``J^T J`` -- except that the reference
    fills block (l, m) through ``mlinalg.hadamard`` (MultilinearAlgebra.py:276-289),
    which loops over ``A.shape[0]`` in BOTH indices: only the leading R d_l
    columns of the block are written, the rest keep the zeros ``H`` starts
    with.  This truncation is reproduced (``exact=False``).  With d_l > d_m
    (modes not in decreasing order) the reference indexes past the block; the
    full block is used then."""
    L = len(factors)
    R = factors[0].shape[1]
    dims = [W.shape[0] for W in factors]
    sd = sum_dims_of(dims, R)
    H = np.zeros((sd[-1], sd[-1]))
    for l in range(L):
        H[sd[l]:sd[l + 1], sd[l]:sd[l + 1]] = np.kron(P1[l], np.eye(dims[l]))
        for m in range(l):
            blk = np.einsum('rs,is,jr->risj', P2[l, m], factors[l], factors[m])
            blk = blk.reshape(R * dims[l], R * dims[m])
            if not exact and dims[l] < dims[m]:
                blk[:, R * dims[l]:] = 0.0
            H[sd[l]:sd[l + 1], sd[m]:sd[m + 1]] = blk
            H[sd[m]:sd[m + 1], sd[l]:sd[l + 1]] = blk.T
    return H


def direct(Tl, factors, damp):
    """The 'direct' inner method (GaussNewton.py:630-653): the damped system
    ``(J^T J + damp diag(Gamma)) y = grad`` row-scaled by ``M^2`` and solved by a
    QR factorisation and a triangular solve; ``y = 0`` when that raises."""
    L = len(factors)
    R = factors[0].shape[1]
    dims = [W.shape[0] for W in factors]
    Gr, P1, P2 = gramians(factors)
    Gamma, gamma = regularization(P1, dims, R)
    M = precond(Gamma, gamma, damp, dims)
    grad = -compute_grad(Tl, factors, P1)
    H = hessian(factors, P1, P2)
    Hd = H + damp * np.diag(Gamma)
    MHd = ((Hd.T) * (M ** 2)).T
    Mgrad = (M ** 2) * grad
    try:
        q, r = np.linalg.qr(MHd)
        y = np.linalg.solve(r, q.T @ Mgrad)
    except np.linalg.LinAlgError:
        y = np.zeros(len(grad))
    return y, grad


def update_gain_ratio(damp, old_error, error, Tsize, old_x, x, grad):
    """Gain ratio (GaussNewton.py:472-487)."""
    num = (Tsize ** 2) * (old_error ** 2 - error ** 2)
    den = float(np.dot(x - old_x, grad + damp * (x - old_x)))
    if den != 0.0:
        return num / den
    if num != 0.0:
        return np.sign(num) * np.inf
    return -np.inf


def update_damp(damp, init_damp, gain_ratio, it):
    """×3 below 0.25, ÷3 above 0.75, or the user's schedule (GaussNewton.py:490-503)."""
    if type(init_damp) == list:
        return init_damp[it]
    if gain_ratio < 0.25:
        return 3 * damp
    if gain_ratio > 0.75:
        return damp / 3
    return damp


def update_delta(delta, gain_ratio, step_size):
    """Trust-region radius of the dogleg fallback (GaussNewton.py:506-517)."""
    if gain_ratio > 0.75:
        return max(delta, 2 * step_size)
    sigma = 0.25 / (1 + np.exp(-14 * (gain_ratio - 0.75))) + 0.75
    return min(sigma * delta, delta)


def dogleg(y, grad, JT_J_grad, delta):
    """Dogleg step between the steepest-descent and the CG step (GaussNewton.py:766-795)."""
    alpha = norm(grad) ** 2 / np.dot(grad, JT_J_grad)
    y_sd = alpha * grad
    c1 = norm(y_sd)
    c2 = np.dot(y - y_sd, y_sd)
    c3 = norm(y - y_sd) ** 2
    c4 = delta ** 2 - c1 ** 2
    m = c2 ** 2 + c3 * c4
    if norm(y) < delta:
        return y
    if c1 >= delta:
        return (delta / c1) * y_sd
    if m < 0:
        return y
    c5 = np.sqrt(m)
    beta = (-c2 + c5) / c3 if c2 <= 0 else c4 / (c2 + c5)
    return y_sd + beta * (y - y_sd)


def compute_dogleg_steps(Tsize, T1, factors, grad, JT_J_grad, x, y, error, damp, symm, factors_norm):
    """Up to 11 dogleg trials after a rejected step (GaussNewton.py:713-763)."""
    count = 0
    best_x, best_y, best_error = x.copy(), y.copy(), error
    best_factors = deepcopy(factors)
    gain_ratio, delta = 1, 1
    while gain_ratio > 0:
        old_x, old_error = x, error
        y = dogleg(y, grad, JT_J_grad, delta)
        x = x + y
        factors = x2cpd(x, factors, eq=False)
        factors = transform(factors, symm, factors_norm)
        error = fastnorm(T1, cpd2unfold1(factors)) / Tsize
        gain_ratio = update_gain_ratio(damp, old_error, error, Tsize, old_x, x, grad)
        if error < old_error:
            best_x, best_y, best_error = x.copy(), y.copy(), error
            best_factors = deepcopy(factors)
        delta = update_delta(delta, gain_ratio, norm(x - old_x))
        count += 1
        if count > 10:
            break
    return best_factors, best_x, best_y, best_error


def dGN(T, factors, R, options, budgets=None, trace=None):
    """Damped Gauss-Newton (GaussNewton.py:29-251).

    ``budgets`` optionally fixes the CG cap per iteration instead of drawing it;
    ``trace`` (a list) receives per-iteration ``dict(error, damp, itn, y_norm)``.
    Returns ``(best_factors, step_sizes, errors, improv, gradients, stop)``.
    """
    o = options
    init_damp, maxiter = o.init_damp, o.maxiter
    tol, tol_step, tol_improv, tol_grad = o.tol, o.tol_step, o.tol_improv, o.tol_grad
    L = len(factors)
    fix_mode, orig = -1, None
    factors = list(factors)
    for l in range(L):           # [W] marks a fixed factor (bicpd), GaussNewton.py:92-99
        if type(factors[l]) == list:
            fix_mode = l
            factors[l] = factors[l][0]
            orig = np.array(factors[l], dtype=np.float64)
    # float64 copies that keep the list's aliasing: a list holding one array L
    # times (a symmetric start) stays that way, which matters to ``x2cpd`` and
    # ``transform`` (both work in place, as in the reference)
    copies = {}
    factors = [copies.setdefault(id(W), np.array(W, dtype=np.float64)) for W in factors]
    dims = T.shape
    Tsize = norm(T)
    error = 1
    best_error = np.inf
    stop = 5
    damp = init_damp[0] if type(init_damp) == list else init_damp * np.mean(np.abs(T))
    const = 1 + int(maxiter / 10)
    if R * sum(dims) <= 100:
        tol = tol_step = tol_improv = tol_grad = 0
    x = cpd2flat(factors)
    y = np.zeros(R * sum(dims))
    step_sizes, errors = np.zeros(maxiter), np.zeros(maxiter)
    improv, gradients = np.zeros(maxiter), np.zeros(maxiter)
    best_factors = deepcopy(factors)
    Tl = [unfold(np.asarray(T, dtype=np.float64), l + 1) for l in range(L)]
    it = 0
    for it in range(maxiter):
        old_x, old_error = x, error
        inner = o.inner_method[it] if type(o.inner_method) == list else o.inner_method
        cgmax, itn = 0, 0
        if inner == 'als':
            # GaussNewton.py:275-278: one ALS sweep, x = the swept factors, no step
            factors = als_iteration(Tl, factors, fix_mode)
            x = cpd2flat(factors)
            y = np.zeros(R * sum(dims))
            grad = np.array([np.nan])
        elif inner == 'direct':
            y, grad = direct(Tl, factors, damp)
        else:
            if budgets is not None:
                cgmax = int(budgets[it])
            elif inner == 'cg':
                cgmax = cg_budget(it, L, o.cg_factor)
            elif inner == 'cg_static':
                cgmax = o.cg_maxiter
            else:
                raise NotImplementedError("inner_method " + repr(inner))
            y, grad, JT_J_grad, itn, residualnorm = cg(Tl, factors, damp, cgmax, o.cg_tol)
        x = x + y
        factors = x2cpd(x, factors)
        factors = transform(factors, o.symm, o.factors_norm)
        if L == 3 and fix_mode >= 0:     # GaussNewton.py:293-297
            factors[fix_mode] = orig.copy()
        error = fastnorm(Tl[0], cpd2unfold1(factors)) / Tsize
        if inner in ('cg', 'cg_static') and it > 3 and error > o.tol_jump * old_error:
            x = x - y
            factors, x, y, error = compute_dogleg_steps(Tsize, Tl[0], factors, grad, JT_J_grad,
                                                        x, y, error, damp, o.symm, o.factors_norm)
        gain_ratio = update_gain_ratio(damp, old_error, error, Tsize, old_x, x, grad)
        if trace is not None:
            trace.append(dict(error=error, damp=damp, itn=itn, budget=cgmax))
        damp = update_damp(damp, init_damp, gain_ratio, it)
        if error < best_error:
            best_error = error
            best_factors = deepcopy(factors)
        errors[it] = error
        step_sizes[it] = norm(x - old_x) / norm(old_x)
        gradients[it] = norm(grad, np.inf)
        improv[it] = errors[it] if it == 0 else abs(errors[it] - errors[it - 1])
        if it > 1:
            if errors[it] < tol:
                stop = 0
                break
            if step_sizes[it] < tol_step:
                stop = 1
                break
            if improv[it] < tol_improv:
                stop = 2
                break
            if gradients[it] < tol_grad:
                stop = 3
                break
            if it > 2 * const and it % const == 0:
                mean1 = np.mean(errors[it - 2 * const: it - const])
                mean2 = np.mean(errors[it - const: it])
                if mean1 - mean2 <= tol_improv:
                    stop = 4
                    break
                mean3 = np.mean(improv[it - const: it])
                if mean3 < 1e-3 * mean2:
                    stop = 7
                    break
            if error > max(1, Tsize ** 2) / (1e-16 + tol):
                stop = 6
                break
    n = it + 1
    return best_factors, step_sizes[:n], errors[:n], improv[:n], gradients[:n], stop


def als_iteration(Tl, factors, fix_mode=-1):
    """One ALS sweep (Alternating_Least_Squares.py:204-264): mode by mode,
    ``W_l = T_(l) · pinv(KR_l^T)`` with the freshly updated factors; a fixed
    mode (third order, bicpd) is skipped -- the reference's explicit branches
    update the two other modes in the same order with the same products."""
    L = len(factors)
    for l in range(L):
        if l == fix_mode:
            continue
        order = [m for m in reversed(range(L)) if m != l]
        M = kr_chain([factors[m] for m in order])
        factors[l] = Tl[l] @ np.linalg.pinv(M.T)
    return factors


def als(T, factors, R, options):
    """Alternating least squares (Alternating_Least_Squares.py:18-201).

    Returns ``(factors, step_sizes, errors, improv, gradients, stop)``; unlike
    ``dGN`` the factors returned are the LAST iterate (the reference keeps a
    best copy but does not return it)."""
    o = options
    maxiter = o.maxiter
    tol, tol_step, tol_improv, tol_grad = o.tol, o.tol_step, o.tol_improv, o.tol_grad
    L = len(factors)
    fix_mode, orig = -1, None
    for l in range(L):                      # [W, l] marks a fixed factor (bicpd)
        if type(factors[l]) == list:
            fix_mode = l
            factors[l] = factors[l][0]
            orig = np.array(factors[l], dtype=np.float64)
    factors = [np.array(W, dtype=np.float64) for W in factors]
    Tsize = norm(T)
    error = 1
    stop = 5
    const = 1 + int(maxiter / 10)
    x = cpd2flat(factors)
    step_sizes, errors = np.empty(maxiter), np.empty(maxiter)
    improv, gradients = np.empty(maxiter), np.empty(maxiter)
    Tl = [unfold(np.asarray(T, dtype=np.float64), l + 1) for l in range(L)]
    it = 0
    for it in range(maxiter):
        old_x, old_error = x, error
        factors = als_iteration(Tl, factors, fix_mode)
        x = cpd2flat(factors)
        factors = transform(factors, o.symm, o.factors_norm)
        if L == 3 and fix_mode >= 0:
            factors[fix_mode] = orig.copy()
        error = fastnorm(Tl[0], cpd2unfold1(factors)) / Tsize
        step_sizes[it] = norm(x - old_x)
        errors[it] = error
        with np.errstate(divide='ignore', invalid='ignore'):
            gradients[it] = np.abs(old_error - error) / step_sizes[it]
        improv[it] = errors[it] if it == 0 else np.abs(errors[it - 1] - errors[it])
        if it > 1:
            if errors[it] < tol:
                stop = 0
                break
            if step_sizes[it] < tol_step:
                stop = 1
                break
            if improv[it] < tol_improv:
                stop = 2
                break
            if gradients[it] < tol_grad:
                stop = 3
                break
            if it > 2 * const and it % const == 0:
                mean1 = np.mean(errors[it - 2 * const: it - const])
                mean2 = np.mean(errors[it - const: it])
                if mean1 - mean2 <= tol_improv:
                    stop = 4
                    break
                mean3 = np.mean(improv[it - const: it])
                if mean3 < 1e-3 * mean2:
                    stop = 7
                    break
            if error > max(1, Tsize ** 2) / (1e-16 + tol):
                stop = 6
                break
    n = it + 1
    return factors, step_sizes[:n], errors[:n], improv[:n], gradients[:n], stop


def rank_bounds(dims, method='dGN'):
    """(Rmin, Rmax) of the rank search (TensorFox.py:863-873)."""
    L = len(dims)
    if L > 3:
        if method == 'dGN':
            return 1, int(np.prod(np.sort(np.array(dims))[1:]))
        return 2, int(np.min(dims))
    m, n, p = dims
    return 1, int(min(m * n, m * p, n * p))


def rank(best_error_of, dims, method='dGN'):
    """The rank search of TensorFox.py:820-939 with the CPD replaced by
    ``best_error_of(r)`` (the best relative error over the trials at rank r;
    order > 3 at r = 1 counts as 1 without a CPD).  Returns
    ``(final_rank, error_per_rank)``."""
    L = len(dims)
    Rmin, Rmax = rank_bounds(dims, method)
    epr = np.empty(Rmax)
    final_rank = None
    r = 1
    for r in range(1, Rmax + 1):
        best_error = 1.0 if (L > 3 and r == 1) else best_error_of(r)
        epr[r - 1] = best_error
        if best_error < 1e-14:
            final_rank = r
            break
        if r > Rmin and np.abs(epr[r - 1] - epr[r - 2]) < 1e-5 and best_error < 0.5:
            final_rank = int(np.nanargmin(epr[0:r])) + 1
            break
        if r > 2:
            prev = np.abs(epr[r - 2] - epr[r - 3])
            cur = np.abs(epr[r - 1] - epr[r - 2])
            with np.errstate(divide='ignore', invalid='ignore'):
                if prev / cur > 100 and best_error < 0.5:
                    final_rank = r - 1
                    break
    epr = epr[0:r]
    if final_rank is None:
        final_rank = int(np.nanargmin(epr)) + 1
    return int(final_rank), epr


# ----------------------------------------------------------------------------
# compression (Compression.py)
# ----------------------------------------------------------------------------
def svd_flip(u, v, u_based_decision=True):
    """Deterministic signs: largest |loading| positive (Compression.py:521-564)."""
    if u_based_decision:
        idx = np.argmax(np.abs(u), axis=0)
        signs = np.sign(u[idx, range(u.shape[1])])
    else:
        idx = np.argmax(np.abs(v), axis=1)
        signs = np.sign(v[range(v.shape[0]), idx])
    return u * signs, v * signs[:, None]


def randomized_svd(M, n_components, n_oversamples=10, n_iter=2):
    """Halko et al. range finder with ``n_iter`` power iterations (Compression.py:337-518)."""
    n_random = n_components + n_oversamples
    transpose = M.shape[0] < M.shape[1]
    if transpose:
        M = M.T
    Q = np.random.normal(size=(M.shape[1], n_random))
    if M.dtype.kind == 'f':
        Q = Q.astype(M.dtype, copy=False)
    for _ in range(n_iter):
        Q = M @ Q
        Q = M.T @ Q
    Q, _ = sp_qr(M @ Q, mode='economic')
    B = Q.T @ M
    Uhat, s, V = sp_svd(B, full_matrices=False)
    U = Q @ Uhat
    U, V = svd_flip(U, V, u_based_decision=not transpose)
    if transpose:
        return V[:n_components, :].T, s[:n_components], U[:, :n_components].T
    return U[:, :n_components], s[:n_components], V[:n_components, :]


def clean_compression(U, sigma, Vt, tol_mlsvd, L):
    """Energy truncation: first i with Σσ[i:]²/Σσ² < tol/L (Compression.py:261-301)."""
    eps = tol_mlsvd / L
    tot = np.sum(sigma ** 2)
    for i in range(1, len(sigma)):
        if np.sum(sigma[i:] ** 2) / tot < eps:
            return U[:, :i], sigma[:i], Vt[:i, :], i
    return U, sigma, Vt, sigma.size


def sparse_unfold(data, idxs, dims, mode):
    """COO → CSR mode unfolding with Kolda column keys (Conversion.py:255-302)."""
    from scipy.sparse import coo_matrix
    L = len(dims)
    dims = [int(d) for d in dims]
    others = [l for l in range(L) if l != mode - 1]
    K = np.zeros(L, dtype=np.uint64)
    s = 1
    for l in others:
        K[l] = s
        s *= dims[l]
    idxs = np.asarray(idxs, dtype=np.uint64)
    rows = idxs[:, mode - 1]
    cols = np.sum(K * idxs, axis=1, dtype=np.uint64)
    return coo_matrix((data, (rows, cols)), shape=(dims[mode - 1], s)).tocsr()


def sparse_multilin_mult(UT, data, idxs, dims):
    """Dense core ``S = T ×_1 U_1^T ... ×_L U_L^T`` from COO (MultilinearAlgebra.py:145-190)."""
    idxs = np.asarray(idxs).astype(np.int64)
    L = len(dims)
    G = [UT[l][:, idxs[:, l]] for l in range(L)]            # (n_l, nnz)
    S = G[0] * np.asarray(data, dtype=np.float64)[None, :]
    for l in range(1, L):
        S = np.einsum('...k,jk->...jk', S, G[l])
    return S.sum(axis=-1)


def multilin_mult(UT, T):
    """``(U_1^T, ..., U_L^T) · T`` (MultilinearAlgebra.py:72-105)."""
    S = T
    for l in range(len(UT)):
        S = np.moveaxis(np.tensordot(UT[l], S, axes=(1, l)), 0, l)
    return S


def compute_svd(Tl, dims, R, method, tol_mlsvd, L, l, svd_n_components):
    """SVD of one unfolding (Compression.py:192-237)."""
    low_rank = min(R, int(dims[l]))
    if method == 'sparse':
        G = Tl
        n = svd_n_components if svd_n_components is not None else \
            int(max(L, np.log10(dims[l] * dims[l] * L)) * low_rank)
        U, s, Vt = randomized_svd(G, n, n_oversamples=10, n_iter=2)
        s = np.sqrt(s)
    else:
        n = svd_n_components if svd_n_components is not None else low_rank
        U, s, Vt = randomized_svd(Tl, n, n_oversamples=10, n_iter=2)
    return clean_compression(U, s, Vt, tol_mlsvd, L)


def mlsvd(T, Tsize, R, options):
    """Truncated MLSVD, 'seq' / 'classic' / sparse branches (Compression.py:48-189)."""
    o = make_options(options)
    tol_mlsvd = o.tol_mlsvd
    sparse_in = isinstance(T, list)
    if sparse_in:
        data, idxs, dims = T
        data = np.asarray(data, dtype=np.float64)
        idxs = np.asarray(idxs, dtype=np.uint64)
        dims = np.asarray(dims)
    else:
        dims = T.shape
    L = len(dims)
    if type(tol_mlsvd) == list:
        tol_mlsvd = tol_mlsvd[0] if L > 3 else tol_mlsvd[1]
    U, sigmas = [], []
    if tol_mlsvd == -1:
        return T, [np.identity(dims[l]) for l in range(L)], unfold(T, 1), [np.ones(dims[l]) for l in range(L)]
    if sparse_in:
        T1 = sparse_unfold(data, idxs, dims, 1)
        for l in range(L):
            Tl = sparse_unfold(data, idxs, dims, l + 1)
            G = (Tl @ Tl.T).toarray()
            Ul, sl, _, _ = compute_svd(G, dims, R, 'sparse', tol_mlsvd, L, l, o.svd_n_components)
            U.append(Ul)
            sigmas.append(sl)
        S = sparse_multilin_mult([u.T for u in U], data, idxs, dims)
    elif o.mlsvd_method == 'seq':
        S = np.asarray(T, dtype=np.float64)
        S_dims = list(dims)
        T1 = unfold(S, 1)
        for l in range(L):
            Sl = unfold(S, l + 1)
            Ul, sl, Vlt, dim = compute_svd(Sl, dims, R, 'seq', tol_mlsvd, L, l, o.svd_n_components)
            U.append(Ul)
            sigmas.append(sl)
            S_dims[l] = dim
            S = foldback((Vlt.T * sl).T, l + 1, S_dims)
    elif o.mlsvd_method == 'classic':
        T = np.asarray(T, dtype=np.float64)
        T1 = unfold(T, 1)
        for l in range(L):
            Ul, sl, _, _ = compute_svd(unfold(T, l + 1), dims, R, 'classic', tol_mlsvd, L, l,
                                       o.svd_n_components)
            U.append(Ul)
            sigmas.append(sl)
        S = multilin_mult([u.T for u in U], T)
    else:
        raise NotImplementedError("mlsvd_method " + repr(o.mlsvd_method))
    if type(o.trunc_dims) == list:
        sl_ = []
        for l in range(L):
            sl_.append(slice(0, o.trunc_dims[l]))
            U[l] = U[l][:, :min(o.trunc_dims[l], U[l].shape[1])]
        S = S[tuple(sl_)]
    return S, U, T1, sigmas


# ----------------------------------------------------------------------------
# initialisation and driver (Initialization.py, Auxiliar.py, TensorFox.py)
# ----------------------------------------------------------------------------
def clean_zeros(init_factors, dims, R):
    """Replaces exact zeros by ``1e-4 * randn() * ||W||`` (Initialization.py:361-386)."""
    for l in range(len(dims)):
        W = init_factors[l]
        for i in range(dims[l]):
            for r in range(R):
                if W[i, r] == 0.0:
                    W[i, r] = 1e-4 * np.random.randn() * norm(W)
    return init_factors


def smart_sample(S, dims, R):
    """One draw of Initialization.py:139-183: per mode an index i taken with
    probability proportional to d - i (arr = [d, d-1, ..., 1], one integer in
    [0, sum(arr)) per column), a unit entry at that index in every factor, and
    the core's value at the chosen position in the first factor."""
    L = len(dims)
    f = [np.zeros((dims[l], R)) for l in range(L)]
    arr = [dims[l] * np.ones(dims[l]) - np.arange(dims[l]) for l in range(L)]
    high = [np.sum(arr[l]) for l in range(L)]
    C = [np.random.randint(high[l], size=R) for l in range(L)]
    cum = [np.cumsum(arr[l]) for l in range(L)]
    for r in range(R):
        idx = [int(np.searchsorted(cum[l], C[l][r], side='right')) for l in range(L)]
        for l in range(L):
            f[l][idx[l], r] = 1
        f[0][idx[0], r] = S[tuple(idx)]
    return f


def smart_random(S, dims, R):
    """Best of 1 + int(sqrt(prod(dims))) smart samples by relative error to S
    (Initialization.py:97-136), the first one kept on ties."""
    samples = 1 + int(np.sqrt(np.prod(np.array(dims))))
    S1 = unfold(S, 1)
    Ssize = norm(S)
    best, best_error = None, np.inf
    for _ in range(samples):
        f = smart_sample(S, dims, R)
        e = norm(S1 - cpd2unfold1(f)) / Ssize
        if e < best_error:
            best_error, best = e, [w.copy() for w in f]
    return best


def join_rank1(idx):
    """Initialization.py:289-342: groups of chosen positions that differ in one
    coordinate only (one rank-one term each), with the reference's scan order --
    removals inside the scans shift the lists under the running indices."""
    R, L = len(idx), len(idx[0])
    count = 0
    pool = list(idx)
    groups = [[] for _ in range(L * R)]
    g = 0
    for l in range(L):
        keep = [j for j in range(L) if j != l]
        r = 0
        while r < len(pool):
            key = tuple(pool[r][j] for j in keep)
            rr = r + 1
            while rr < len(pool):
                if tuple(pool[rr][j] for j in keep) == key:
                    groups[g].append(pool[rr])
                    pool.remove(pool[rr])
                    count += 1
                rr += 1
            if groups[g]:
                groups[g].append(pool[r])
                pool.remove(pool[r])
            g += 1
            r += 1
    return count, [x for x in groups if x]


def find_pivot(x):
    """The coordinate that varies inside a group (Initialization.py:345-358)."""
    if len(x) == 1:
        return 0
    for l in range(len(x[0])):
        if x[0][l] != x[1][l]:
            return l


def smart(S, dims, R):
    """Deterministic start from the R largest-magnitude core entries, merged
    into rank-one terms where they share all coordinates but one, and extended
    by the next entries while merges free terms (Initialization.py:186-286)."""
    L = len(dims)
    flat = np.argsort(-np.abs(S).ravel(), kind='stable')
    order = [tuple(int(v) for v in np.unravel_index(k, S.shape)) for k in flat]
    chosen, rest = order[:R], order[R:]
    prev = 0
    joined = []
    for _ in range(100):
        count, joined = join_rank1(chosen)
        if count - prev <= 0:
            break
        chosen = chosen + rest[:count - prev]
        rest = rest[count - prev:]
        prev = count
    terms = [[] for _ in range(R)]
    r = 0
    for grp in joined:
        for y in grp:
            terms[r].append(y)
            chosen.remove(y)
        r += 1
    for x in chosen:
        terms[r].append(x)
        r += 1
    f = [np.zeros((dims[l], R)) for l in range(L)]
    for r in range(R):
        m = find_pivot(terms[r])
        for x in terms[r]:
            for l in range(L):
                if l == m:
                    f[l][x[l], r] += S[x]
                else:
                    f[l][x[l], r] = 1
    return f


def starting_point(S, U, R, ordering, options):
    """User list, 'random', 'smart_random' or 'smart' initial factors in the
    compressed space (Initialization.py:20-94)."""
    init = options.initialization
    dims = S.shape
    L = len(dims)
    if type(init) == list:
        return [U[l].T @ init[ordering[l]] for l in range(L)]
    if init == 'random':
        f = [np.random.randn(dims[l], R) for l in range(L)]
    elif init == 'smart_random':
        f = smart_random(S, dims, R)
    elif init == 'smart':
        f = smart(S, dims, R)
    else:
        raise NotImplementedError("initialization " + repr(init))
    f = clean_zeros(f, dims, R)
    f = equalize(f, R)
    return transform(f, options.symm, options.factors_norm)


def sort_dims(T):
    """Modes in decreasing size (Auxiliar.py:93-115)."""
    if isinstance(T, list):
        data, idxs, dims = T
        idxs = np.asarray(idxs, dtype=np.uint64)
        dims = np.asarray(dims)
        ordering = np.argsort(-dims)
        return [data, idxs[:, ordering], tuple(dims[ordering])], ordering
    dims = np.array(T.shape)
    ordering = np.argsort(-dims)
    return np.moveaxis(T, ordering, np.arange(-len(dims), 0)), ordering


def unsort_dims(factors, ordering):
    """Inverse permutation of :func:`sort_dims` (Auxiliar.py:118-128)."""
    out = [None] * len(factors)
    for l in range(len(factors)):
        out[ordering[l]] = factors[l]
    return out


class Output:
    pass


# ----------------------------------------------------------------------------
# tensor-train CPD (TensorFox.py:256-421, 658-817, 1042-1065; Auxiliar.py:365-527;
# Conversion.py:460-494)
# ----------------------------------------------------------------------------
def tt_core(V, dims, r1, r2, l):
    """One core of the TT-SVD (Auxiliar.py:365-380).  The reference takes a
    randomized SVD at full rank (scikit-learn, no power iteration): an exact SVD
    up to rounding, whose Gaussian block it draws from NumPy's global RNG; the
    block is drawn here too, so the RNG stays in step, and the SVD is LAPACK's.
    Signs: the largest |entry| of every left singular vector is positive."""
    V = np.asarray(V).reshape(r1 * dims[l], int(np.prod(dims[l + 1:])), order='F')
    low = min(V.shape)
    np.random.normal(size=(low, low + 10))
    U, sv, Vt = sp_svd(V, full_matrices=False)
    U, Vt = U[:, :low], Vt[:low]
    for j in range(low):
        k = np.argmax(np.abs(U[:, j]))
        if U[k, j] < 0:
            U[:, j] *= -1
            Vt[j] *= -1
    U = U[:, :r2]
    Vn = (sv[:low, None] * Vt)[:r2, :]
    g = U.reshape(dims[l], r2, order='F') if r1 == 1 else U.reshape(r1, dims[l], r2, order='F')
    return Vn, g


def cpdtt(T, R):
    """TT cores d_0 x R -> R x d_1 x R -> ... -> R x d_{L-1} (TensorFox.py:1042-1065)."""
    dims = np.array(T.shape)
    L = len(dims)
    G = []
    r1, r2 = 1, R
    V = T
    for l in range(L - 1):
        V, g = tt_core(V, dims, r1, r2, l)
        r1, r2 = R, R
        G.append(g)
    G.append(V)
    return G


def inflate(T, R, dims):
    """Pads every mode shorter than R with 1e-12 * randn entries (Conversion.py:460-480)."""
    new = [d if d >= R else R for d in dims]
    out = 1e-12 * np.random.randn(*new)
    out[tuple(slice(d) for d in dims)] = T
    return out


def bicpd(T, R, fixed, options):
    """Third-order CPD with one factor fixed (TensorFox.py:658-817): MLSVD of T,
    a random start whose fixed factor is replaced by the projection of the given
    one, ALS (bi_method 'als') or dGN with the options' inner method (any other
    bi_method, TensorFox.py:762-767) on the core, decompression.  Returns
    (X, Y, Z, output) in T's own mode order (no sort_dims)."""
    o = options
    Tsize = norm(T)
    S, U, T1, _ = mlsvd(T, Tsize, R, o)
    f = starting_point(S, U, R, [0, 1, 2], o)
    W, fl = fixed
    f[fl] = [U[fl].T @ W, fl]
    if o.bi_method_parameters[0] == 'als':
        f, ss, er, im, gr, st = als(S, f, R, o)
    else:
        f, ss, er, im, gr, st = dGN(S, f, R, o)
    out = [None, None, None]
    for l in range(3):
        out[l] = W if l == fl else U[l] @ f[l]
    rel = fastnorm(T1, cpd2unfold1(out)) / Tsize
    res = Output()
    res.num_steps = len(ss)
    res.rel_error = rel
    res.stop = [st, 5]
    return out[0], out[1], out[2], res


def cpd_cores(G, max_trials, epochs, R, options):
    """CPDs of the TT cores (Auxiliar.py:413-527): the first inner core by
    tricpd (best of the trials, early exit below 1e-4), then sweeps of bicpd with
    the factor shared with the neighbouring core fixed to pinv of the
    neighbour's factor."""
    L = len(G)
    if epochs % 2 == 0:
        epochs += 1
    cpd_list = list(range(L - 2))
    outputs = list(range(L - 2))
    best_error = np.inf
    for _ in range(max_trials):
        f, out = _tricpd(G[1], R, options)
        if out.rel_error < best_error:
            best_out, best_error = out, out.rel_error
            bX, bY, bZ = f
            if best_error < 1e-4:
                break
    outputs[0] = best_out
    cpd_list[0] = [bX, bY, bZ]
    low, upp = 2, L - 2
    for epoch in range(epochs):
        if epoch % 2 == 0:
            for l in range(low, L - 1):
                best_error = np.inf
                fX = np.linalg.pinv(bZ.T)
                for _ in range(max_trials):
                    X, Y, Z, out = bicpd(G[l], R, [fX, 0], options)
                    if out.rel_error < best_error:
                        best_out, best_error = out, out.rel_error
                        bX, bY, bZ = fX, Y, Z
                        if best_error < 1e-4:
                            break
                if epoch == epochs - 1:
                    outputs[l - 1] = best_out
                    cpd_list[l - 1] = [fX, bY, bZ]
        else:
            if L == 3:
                low, upp = 1, L - 1
            for l in reversed(range(1, upp)):
                best_error = np.inf
                fZ = np.linalg.pinv(bX.T)
                for _ in range(max_trials):
                    X, Y, Z, out = bicpd(G[l], R, [fZ, 2], options)
                    if out.rel_error < best_error:
                        best_out, best_error = out, out.rel_error
                        bX, bY, bZ = X, Y, fZ
                        if best_error < 1e-4:
                            break
                if epoch == epochs - 2:
                    outputs[l - 1] = best_out
                    cpd_list[l - 1] = [bX, bY, fZ]
    return cpd_list, outputs, bZ


def highcpd(T, R, options):
    """TT cores, their CPDs, and the factors of T (TensorFox.py:368-421)."""
    L = T.ndim
    options.refine = False
    G = cpdtt(T, R)
    cpd_list, outputs, bZ = cpd_cores(G, options.trials, options.epochs, R, options)
    factors = [G[0] @ cpd_list[0][0]]
    for l in range(L - 2):
        factors.append(cpd_list[l][1])
    factors.append(G[-1].T @ bZ)
    return equalize(factors, R), outputs




def cpd(T, R, options=None, timings=None):
    """``cpd`` → ``tricpd`` for methods 'dGN' and 'als' (TensorFox.py:69-255, 424-655).

    Returns ``(factors, output)`` where ``output`` carries num_steps, rel_error,
    accuracy, step_sizes, errors, improv, gradients and stop like the reference's.
    ``timings`` (a dict) receives wall seconds of the 'mlsvd', 'dgn' and 'final'
    phases when given.
    """
    import time as _time
    _t = [_time.perf_counter()]

    def _mark(name):
        now = _time.perf_counter()
        if timings is not None:
            timings[name] = timings.get(name, 0.0) + now - _t[0]
        _t[0] = now

    o = make_options(options)
    if o.method == 'ttcpd':
        return cpd_tt(T, R, o)
    sparse_in = isinstance(T, list)
    if sparse_in:
        data_orig = np.asarray(T[0], dtype=np.float64)
        idxs_orig = np.asarray(T[1], dtype=np.uint64)
        dims_orig = np.asarray(T[2])
    Ts, ordering = sort_dims(T)
    if sparse_in:
        Tsize = norm(Ts[0])
        if (o.tol_mlsvd if type(o.tol_mlsvd) != list else o.tol_mlsvd[0]) < 0:
            o.tol_mlsvd = 1e-16
    else:
        Ts = np.asarray(Ts, dtype=np.float64)
        Tsize = norm(Ts)
    _mark('prepare')
    S, U, T1, sigmas = mlsvd(Ts, Tsize, R, o)
    _mark('mlsvd')
    init = starting_point(S, U, R, ordering, o)
    solver = als if o.method == 'als' else dGN
    factors, ss, er, im, gr, st = solver(S, init, R, o)
    _mark('dgn')
    factors = [U[l] @ factors[l] for l in range(len(factors))]
    refine = o.refine and not sparse_in
    if refine:
        factors, ss2, er2, im2, gr2, st2 = solver(Ts, factors, R, o)
    else:
        ss2, er2, im2, gr2, st2 = np.array([0]), np.array([0]), np.array([0]), np.array([0]), 8
    out = Output()
    if sparse_in:
        factors = unsort_dims(factors, ordering)
        rel_error = sparse_fastnorm(data_orig, idxs_orig, dims_orig, factors) / Tsize
    else:
        approx = cpd2unfold1(factors)
        factors = unsort_dims(factors, ordering)
        rel_error = er2[-1] if refine else fastnorm(unfold(Ts, 1), approx) / Tsize
    out.num_steps = len(ss) + (len(ss2) if refine else 0)
    out.rel_error = rel_error
    out.accuracy = max(0, 100 * (1 - rel_error))
    out.step_sizes = [ss, ss2]
    out.errors = [er, er2]
    out.improv = [im, im2]
    out.gradients = [gr, gr2]
    out.stop = [st, st2]
    out.options = o
    _mark('final')
    return factors, out


def _tricpd(T, R, options):
    """tricpd on a dense third-order tensor with the caller's options object
    (TensorFox.py:424-655): the method is dGN unless it is 'als'."""
    o = options
    saved = o.method
    o.method = 'als' if saved == 'als' else 'dGN'
    try:
        f, out = cpd(T, R, o)
    finally:
        o.method = saved
    return f, out


def cpd_tt(T, R, o):
    """cpd with method 'ttcpd' on a dense tensor (TensorFox.py:256-365)."""
    Ts, ordering = sort_dims(T)
    Ts = np.asarray(Ts, dtype=np.float64)
    Tsize = norm(Ts)
    S, U, T1, _ = mlsvd(Ts, Tsize, R, o)
    S_dims = S.shape
    infl = R > min(S_dims)
    if infl:
        S = inflate(S, R, S_dims)
    o.trunc_dims = 0
    factors, outputs = highcpd(S, R, o)
    if infl:
        factors = [factors[l][:S_dims[l], :] for l in range(len(S_dims))]
    factors = [U[l] @ factors[l] for l in range(len(factors))]
    rel_error = fastnorm(unfold(Ts, 1), cpd2unfold1(factors)) / Tsize
    factors = unsort_dims(factors, ordering)
    out = Output()
    out.num_steps = sum(x.num_steps for x in outputs)
    out.rel_error = rel_error
    out.accuracy = max(0, 100 * (1 - rel_error))
    out.cpd_output = outputs
    out.options = o
    return factors, out
