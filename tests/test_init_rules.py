"""The package's 'smart_random' and 'smart' starts (host logic) against the
reference's own starting_point outputs (Initialization.py:20-358)."""
import numpy as np
import pytest

from conftest import load_golden

ini = pytest.importorskip("tensorfox_gb300.initialization")
opts = pytest.importorskip("tensorfox_gb300.options")


@pytest.mark.parametrize("method", ["smart_random", "smart"])
def test_smart_starts_match_reference(method):
    g = load_golden("init_smart")
    o = opts.make_options(None)
    for k in range(int(g["n"])):
        S, R = g["S%d" % k], int(g["R%d" % k])
        np.random.seed(int(g["seed"]) + k)
        f = (ini.smart_random if method == "smart_random" else ini.smart)(S, R)
        f = ini.clean_and_balance(f, R, o)
        assert np.random.rand() == float(g["%s_after%d" % (method, k)])
        got = np.concatenate([w.flatten('F') for w in f])
        np.testing.assert_allclose(got, g["%s%d" % (method, k)], rtol=1e-12, atol=1e-15)
