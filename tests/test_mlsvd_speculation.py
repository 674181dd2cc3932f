"""Host logic of the queued MLSVD (compression.mlsvd_confirm): the energy
truncation decided from all modes' eigenvalues at once, and NumPy's RNG put
back when a mode keeps fewer vectors than the queued work assumed (no GPU)."""
import numpy as np
import pytest
import torch

compression = pytest.importorskip("tensorfox_gb300.compression")


def _pending(lams, tol=1e-6):
    state = np.random.get_state()
    p = compression.Pending(S=None, Uts=None, cur=None, lams=[torch.tensor(v, dtype=torch.float64) for v in lams],
                            errs=[], ns=[len(v) for v in lams], state=state, tol_mlsvd=tol)
    return p


def test_no_truncation_returns_the_singular_values():
    lams = [[9.0, 4.0, 1.0], [16.0, 1.0], [4.0, 4.0, 1.0, 0.25]]
    np.random.seed(3)
    p = _pending(lams)
    np.random.normal(size=(5, 4))           # draws made while the work was queued
    after = np.random.get_state()[1].copy()
    sig = compression.mlsvd_confirm(p)
    assert sig is not None
    for s, v in zip(sig, lams):
        np.testing.assert_allclose(s, np.sqrt(v))
    assert np.array_equal(np.random.get_state()[1], after)    # the RNG is left alone


def test_truncation_puts_the_rng_back():
    lams = [[9.0, 4.0, 1e-30, 0.0], [16.0, 1.0, 0.5, 0.1]]
    np.random.seed(4)
    want = np.random.rand()
    np.random.seed(4)
    p = _pending(lams)
    np.random.normal(size=(7, 3))
    np.random.randn(2, 2)
    assert compression.mlsvd_confirm(p) is None
    assert np.random.rand() == want


def test_decision_matches_clean_compression_per_mode():
    """Each mode keeps all its assumed vectors exactly when clean_compression
    (Compression.py:261-301) would keep them all."""
    rng = np.random.default_rng(5)
    for _ in range(50):
        lams = [np.sort(rng.exponential(size=4) ** rng.integers(1, 12))[::-1].tolist() for _ in range(3)]
        tol = 10.0 ** rng.integers(-16, -2)
        keep_all = all(compression.clean_compression(np.sqrt(np.array(v)), tol, 3) == 4 for v in lams)
        np.random.seed(6)
        p = _pending(lams, tol)
        assert (compression.mlsvd_confirm(p) is not None) == keep_all
