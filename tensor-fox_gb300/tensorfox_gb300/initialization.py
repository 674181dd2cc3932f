"""'smart_random' and 'smart' starting points (Initialization.py:97-358).

Both build a rank-R tensor from entries of the MLSVD core S (a few thousand
values at most), so they run on the host beside the 'random' start, drawing
from NumPy's global RNG exactly where the reference does:

* ``smart_random``: 1 + int(sqrt(prod(dims))) samples; each picks, per column r
  and mode l, an index i with probability proportional to d_l - i and places
  S at the chosen position as a rank-one spike.  The reference forms every
  sample's full tensor to measure its distance to S; here the distance comes
  in closed form from the chosen entries alone: with c_x columns on position x,
  ||S - S_init||^2 = ||S||^2 - sum_x (2 c_x - c_x^2) S_x^2, all samples at once.
  The kept sample is the first one of least error, like the reference's; only
  two different position sets whose errors tie to the last bit could be ranked
  differently by the two formulas.
* ``smart``: the R largest |S| entries, merged into rank-one terms where they
  share every coordinate but one, extended by the next entries while merges
  free terms (the reference's scan order, Initialization.py:186-358).

Zeros are then replaced by small random values, columns balanced and the
transform applied, as for the random start (Initialization.py:74-84).
"""
import numpy as np


def _interval_draws(dims, R, samples):
    """Per sample and mode, R indices drawn like Initialization.py:166-183
    (randint(sum(arr_l), size=R) mapped through the cumulative sums of
    arr_l = [d, d-1, ..., 1]); the draws follow the reference's order
    (sample-major, then mode).  Returns an int array (samples, L, R)."""
    L = len(dims)
    arr = [dims[l] * np.ones(dims[l]) - np.arange(dims[l]) for l in range(L)]
    high = [np.sum(a) for a in arr]
    cum = [np.cumsum(a) for a in arr]
    out = np.empty((samples, L, R), dtype=np.int64)
    for s in range(samples):
        for l in range(L):
            c = np.random.randint(high[l], size=R)
            out[s, l] = np.searchsorted(cum[l], c, side='right')
    return out


def smart_random(S, R):
    """Initialization.py:97-136 with the closed-form sample error."""
    S = np.asarray(S, dtype=np.float64)
    dims = S.shape
    L = len(dims)
    samples = 1 + int(np.sqrt(np.prod(np.array(dims))))
    idx = _interval_draws(dims, R, samples)                       # (samples, L, R)
    lin = np.ravel_multi_index(tuple(idx[:, l, :] for l in range(L)), dims)   # (samples, R)
    vals = S.ravel()[lin]
    # per sample: multiplicity of each chosen position
    srt = np.sort(lin, axis=1)
    first = np.ones_like(srt, dtype=bool)
    first[:, 1:] = srt[:, 1:] != srt[:, :-1]
    sq = (S.ravel()[srt]) ** 2
    # c_x for every distinct position: run lengths of the sorted positions
    gain = np.zeros(samples)
    for s in range(samples):
        starts = np.flatnonzero(first[s])
        counts = np.diff(np.append(starts, R))
        gain[s] = np.sum((2 * counts - counts * counts) * sq[s, starts])
    nrm2 = float(np.sum(S * S))
    err2 = nrm2 - gain
    best = int(np.argmin(err2))                                   # first of the least
    f = [np.zeros((dims[l], R)) for l in range(L)]
    cols = np.arange(R)
    for l in range(L):
        f[l][idx[best, l], cols] = 1.0
    f[0][idx[best, 0], cols] = vals[best]
    return f


def _merge_groups(pos):
    """Initialization.py:289-342 (join_rank1): positions that differ in one
    coordinate only form one rank-one term.  The scan order, including the
    entries a removal shifts past the running index, is the reference's."""
    R, L = len(pos), len(pos[0])
    count = 0
    pool = list(pos)
    groups = []
    for l in range(L):
        keep = [j for j in range(L) if j != l]
        r = 0
        while r < len(pool):
            key = tuple(pool[r][j] for j in keep)
            grp = []
            rr = r + 1
            while rr < len(pool):
                if tuple(pool[rr][j] for j in keep) == key:
                    grp.append(pool[rr])
                    del pool[rr]
                    count += 1
                rr += 1
            if grp:
                grp.append(pool[r])
                del pool[r]
                groups.append(grp)
            r += 1
    return count, groups


def smart(S, R):
    """Initialization.py:186-286."""
    S = np.asarray(S, dtype=np.float64)
    dims = S.shape
    L = len(dims)
    flat = np.argsort(-np.abs(S).ravel(), kind='stable')   # repeated argmax order
    order = list(zip(*[a.tolist() for a in np.unravel_index(flat, dims)]))
    chosen, rest = order[:R], order[R:]
    prev, groups = 0, []
    for _ in range(100):
        count, groups = _merge_groups(chosen)
        if count - prev <= 0:
            break
        chosen = chosen + rest[:count - prev]
        rest = rest[count - prev:]
        prev = count
    terms = []
    for grp in groups:
        for y in grp:
            chosen.remove(y)
        terms.append(grp)
    terms.extend([x] for x in chosen)
    if len(terms) > R:
        raise ValueError("smart initialization produced more rank-one terms than the rank")
    f = [np.zeros((dims[l], R)) for l in range(L)]
    for r, term in enumerate(terms):
        pivot = 0
        if len(term) > 1:
            pivot = next(l for l in range(L) if term[0][l] != term[1][l])
        for x in term:
            for l in range(L):
                if l == pivot:
                    f[l][x[l], r] += S[x]
                else:
                    f[l][x[l], r] = 1.0
    return f


def clean_and_balance(f, R, options, vectorized=False):
    """Zeros -> 1e-4 * randn * ||W_l|| (sequential, Initialization.py:361-386),
    column balancing (Conversion.py:361-387) and the transform
    (Conversion.py:412-444)."""
    L = len(f)
    for l in range(L):
        W = f[l]
        for i, r in zip(*np.nonzero(W == 0.0)):
            W[i, r] = 1e-4 * np.random.randn() * np.linalg.norm(W)
    if vectorized:
        nr = np.stack([np.linalg.norm(f[l], axis=0) for l in range(L)])
        p = np.prod(nr, axis=0)
        ok = p != 0.0
        g = np.where(ok, p, 1.0) ** (1 / L)
        for l in range(L):
            f[l] = np.where(ok, g / np.where(ok, nr[l], 1.0), 1.0) * f[l]
    else:
        for r in range(R):
            nr = np.array([np.linalg.norm(f[l][:, r]) for l in range(L)])
            if np.prod(nr) != 0.0:
                g = np.prod(nr) ** (1 / L)
                for l in range(L):
                    f[l][:, r] = (g / nr[l]) * f[l][:, r]
    if options.symm:
        s = f[0]
        for l in range(1, L):
            s = s + f[l]
        f = [s / L] * L
    if options.factors_norm > 0:
        f = [options.factors_norm * (1 / np.linalg.norm(W)) * W for W in f]
    return f
