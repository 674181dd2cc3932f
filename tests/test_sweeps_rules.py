"""The rank search's stopping rules (TensorFox.py:854-926) of the package,
evaluated window by window, against the reference's own decisions."""
import numpy as np
import pytest

from conftest import load_golden
from test_oracle_golden import rank_tables

sweeps = pytest.importorskip("tensorfox_gb300.sweeps")


@pytest.mark.parametrize("name", ["rank_rules_L3", "rank_rules_L4"])
def test_rank_search_matches_reference(name):
    g = load_golden(name)
    dims = [int(d) for d in g["dims"]]
    s = 0
    for k, tab in enumerate(rank_tables(g)):
        asked = []

        def best_errors_of(ranks, tab=tab):
            asked.extend(ranks)
            return [float(np.min(tab[q - 1])) for q in ranks]
        fr, epr = sweeps.rank_search(dims, 'dGN', best_errors_of)
        n = int(g["error_lens"][k])
        assert fr == int(g["final_rank"][k])
        np.testing.assert_array_equal(epr, g["errors"][s:s + n])
        # windows never ask twice, and stop within one window of the decision
        assert len(asked) == len(set(asked))
        assert max(asked) < 2 * n + 2
        s += n


def test_rank_bounds():
    assert sweeps.rank_bounds([4, 3, 3]) == (1, 9)
    assert sweeps.rank_bounds([3, 3, 2, 2]) == (1, 18)
    assert sweeps.rank_bounds([5, 4, 3, 2], method='als') == (2, 2)


def test_tuner_picks_fastest_and_caches(tmp_path):
    from tensorfox_gb300 import tuner
    t = tuner.BatchTuner(path=str(tmp_path / "tune.json"))
    key = tuner.signature("fp32", 3, 12, 12, 4096)
    cands = tuner.candidates(12, 12)
    assert cands == [(1, "given"), (1, "largest_first")]
    assert len(tuner.candidates(40, 12)) == 6
    calls = []

    def run(c):
        calls.append(c)
        return {(1, "given"): 2.0, (1, "largest_first"): 1.0}[c]
    assert t.choose(key, cands, run) == (1, "largest_first")
    assert len(calls) == 2
    assert t.choose(key, cands, run) == (1, "largest_first") and len(calls) == 2
    t2 = tuner.BatchTuner(path=str(tmp_path / "tune.json"))      # persisted
    assert t2.lookup(key) == (1, "largest_first")


def test_tuner_sample_and_order():
    from tensorfox_gb300 import tuner
    idx = tuner.sample_indices(4096, 304)
    assert 304 <= len(idx) <= 1024 and idx[0] == 0 and np.all(np.diff(idx) > 0)
    assert list(tuner.sample_indices(100, 304)) == list(range(100))
    assert list(tuner.order_largest_first([3, 9, 1, 9])) == [1, 3, 0, 2]
