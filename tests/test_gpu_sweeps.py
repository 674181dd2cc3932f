"""rank() and stats() on the batched engine (TensorFox.py:820-1039)."""
import numpy as np
import pytest

import tfx_oracle as orc

pytestmark = pytest.mark.gpu

tfx = pytest.importorskip("tensorfox_gb300")
from tensorfox_gb300 import sweeps  # noqa: E402
from tensorfox_gb300.api import _run_dgn  # noqa: E402


def _planted(dims, R, noise, seed):
    rng = np.random.default_rng(seed)
    W = [rng.standard_normal((d, R)) for d in dims]
    T = orc.cpd2tens(W)
    E = rng.standard_normal(T.shape)
    return T + noise * np.linalg.norm(T) / np.linalg.norm(E) * E, W


class _Static:
    inner_method = 'cg_static'
    cg_maxiter = 10
    maxiter = 60


def test_batched_samples_equal_single_solves():
    """Every sample of one engine launch equals the same start solved alone."""
    T, _ = _planted((12, 10, 9), 3, 1e-4, 1)
    o = tfx.make_options(_Static)
    np.random.seed(0)
    X = sweeps._Dense(T, o)
    S, Uts, core = X.compress(3, o)
    probs = [(S, Uts, core, 3, X.start(3, o, Uts, core, S)) for _ in range(5)]
    res = X.solve(probs, o)
    for p, r in zip(probs, res):
        best, ss, er, im, gr, st = _run_dgn(S, p[4], 3, o, X.prec)
        assert r[1] == len(ss)
        full = tfx.api._decompress(Uts, best, core, 3)
        np.testing.assert_allclose(r[2].cpu().numpy(), full.cpu().numpy(), rtol=1e-10, atol=1e-12)


def test_stats_planted():
    T, _ = _planted((14, 12, 10), 4, 1e-6, 2)
    np.random.seed(1)
    times, steps, errors = tfx.stats(T, 4, None, num_samples=12)
    assert times.shape == steps.shape == errors.shape == (12,)
    assert np.all(steps >= 1)
    assert np.median(errors) < 1e-5
    assert np.all(np.isfinite(errors))


def test_stats_als_and_refine():
    T, _ = _planted((10, 9, 8), 3, 1e-5, 3)

    class O:
        method = 'als'
        maxiter = 100
    np.random.seed(2)
    _, steps, errors = tfx.stats(T, 3, O, num_samples=4)
    assert np.all(np.isfinite(errors))
    assert np.min(errors) < 1e-4          # ALS may stall from some starts (swamps)

    class P:
        refine = True
        maxiter = 40
    np.random.seed(3)
    _, steps2, errors2 = tfx.stats(T, 3, P, num_samples=4)
    assert np.median(errors2) < 1e-4


def test_rank_planted():
    """A rank-3 tensor: the error collapses at R = 3; the decision follows the
    reference's rules applied to the errors found."""
    T, _ = _planted((8, 7, 6), 3, 1e-9, 4)
    np.random.seed(5)
    fr, epr = tfx.rank(T, None, plot=False, trials=2)
    assert epr[2] < 1e-6
    assert fr in (3, 4)
    fr2, epr2 = orc.rank(lambda r: float(epr[r - 1]), (8, 7, 6))
    assert fr2 == fr
    np.testing.assert_array_equal(epr2, epr)
