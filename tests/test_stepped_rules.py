"""Host logic of the stepped dGN loop ('als' / 'direct' inner methods): which
runs it takes, the gain ratio, the damping rule and the stop tests, against
the oracle's restatement of GaussNewton.py (no GPU needed)."""
import numpy as np
import pytest

import tfx_oracle as orc

stepped = pytest.importorskip("tensorfox_gb300.stepped")


class _O:
    def __init__(self, inner, maxiter=10):
        self.inner_method = inner
        self.maxiter = maxiter


def test_which_runs_are_stepped():
    assert stepped.uses_stepped(_O('als'))
    assert stepped.uses_stepped(_O('direct'))
    assert stepped.uses_stepped(_O(['direct'] * 3 + ['als'] * 7))
    assert not stepped.uses_stepped(_O('cg'))
    assert not stepped.uses_stepped(_O(['cg'] * 5 + ['cg_static'] * 5))
    # only the first maxiter entries of a list count
    assert not stepped.uses_stepped(_O(['cg'] * 10 + ['als'] * 5))
    with pytest.raises(NotImplementedError):
        stepped.uses_stepped(_O(['cg'] * 5 + ['direct'] * 5))


@pytest.mark.parametrize("case", [(1.0, 0.5, 0.4, 3.0), (0.3, 0.31, 2.0, -1.0), (0.2, 0.2, 1.0, 0.0),
                                  (0.2, 0.1, 1.0, 0.0), (0.5, 0.4, 1.0, np.nan)])
def test_gain_ratio_and_damping_match_oracle(case):
    old_error, error, Tsize, den = case
    damp = 0.7
    # the oracle takes vectors; build x - old_x and grad with the same dot product
    d = np.array([1.0, 0.0])
    grad = np.array([den - damp, 0.0])
    want = orc.update_gain_ratio(damp, old_error, error, Tsize, np.zeros(2), d, grad)
    got = stepped._gain_ratio(damp, old_error, error, Tsize, float(np.dot(d, grad + damp * d)))
    if np.isnan(want):
        assert np.isnan(got)
    else:
        assert got == want
    for it in range(3):
        assert stepped._update_damp(damp, 1.0, got, it) == orc.update_damp(damp, 1.0, want, it)
        assert stepped._update_damp(damp, [0.1, 0.2, 0.3], got, it) == orc.update_damp(damp, [0.1, 0.2, 0.3], want, it)


def test_stop_tests_follow_reference_order():
    m = 30
    const = 1 + int(m / 10)
    e = np.linspace(1.0, 0.5, m)
    ss, im, gr = np.ones(m), np.ones(m), np.full(m, np.nan)
    assert stepped._stop_code(1, e, ss, im, gr, e[1], 1.0, 1e-16, 1e-6, 1e-6, 1e-6, const) is None
    assert stepped._stop_code(5, e, ss, im, gr, e[5], 1.0, 1e-16, 1e-6, 1e-6, 1e-6, const) is None  # NaN gradient
    ss2 = ss.copy()
    ss2[5] = 1e-9
    assert stepped._stop_code(5, e, ss2, im, gr, e[5], 1.0, 1e-16, 1e-6, 1e-6, 1e-6, const) == 1
    e2 = e.copy()
    e2[5] = 1e-20
    assert stepped._stop_code(5, e2, ss2, im, gr, e2[5], 1.0, 1e-16, 1e-6, 1e-6, 1e-6, const) == 0
    flat = np.full(m, 0.3)
    it = 3 * const
    assert stepped._stop_code(it, flat, ss, im, gr, flat[it], 1.0, 1e-16, 1e-6, 1e-6, 1e-6, const) == 4
    assert stepped._stop_code(5, e, ss, im, gr, 1e20, 1.0, 1e-16, 1e-6, 1e-6, 1e-6, const) == 6
