"""dGN with the 'als' and 'direct' inner methods on the device vs the
reference's golden trajectories and the oracle."""
import numpy as np
import pytest

import tfx_oracle as orc
from conftest import load_golden, split_x

pytestmark = pytest.mark.gpu

tfx = pytest.importorskip("tensorfox_gb300")

INNER_CASES = ["dgn_als_L3", "dgn_als_L4", "dgn_als_fix_L3", "dgn_direct_L3", "dgn_direct_L4", "dgn_direct_fix_L3",
               "dgn_direct_symm_L3", "dgn_direct_big_L3", "dgn_mixed_L3", "dgn_symm_direct_alias_L3"]
FIXED_CG_CASES = ["dgn_fix_cg_L3", "dgn_fix_cgr_L3"]


def _opts(g, mod):
    o = mod.Options()
    for k, v in zip(g["opt_names"], g["opt_values"]):
        setattr(o, str(k), eval(str(v)))
    return mod.make_options(o)


def _start(g):
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    f = split_x(g["init_x"], dims, R)
    if "alias" in g and int(g["alias"]):
        return [f[0]] * len(dims)     # one array for every mode
    fix = int(g["fix"]) if "fix" in g else -1
    if fix >= 0:
        f[fix] = [f[fix]]
    return f


@pytest.mark.parametrize("name", INNER_CASES)
def test_inner_methods_fp64_match_reference(name):
    """FP64: stop code, iteration count and every per-iteration statistic as the
    reference's (GaussNewton.py:29-312); the 'direct' solve is LU here and QR
    there, so agreement is to rounding of the step, not bitwise."""
    g = load_golden(name)
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    bf, ss, er, im, gr, st = tfx.dGN(g["T"], _start(g), R, _opts(g, tfx))
    assert st == int(g["stop"])
    assert len(er) == len(g["errors"])
    np.testing.assert_allclose(er, g["errors"], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(ss, g["step_sizes"], rtol=1e-5, atol=1e-12)
    np.testing.assert_allclose(gr, g["gradients"], rtol=1e-5, atol=1e-10)    # NaN where the step was 'als'
    np.testing.assert_allclose(np.concatenate([w.flatten('F') for w in bf]), g["best_x"], rtol=1e-5, atol=1e-8)


@pytest.mark.parametrize("name", FIXED_CG_CASES)
@pytest.mark.parametrize("cluster", [1, 3])
def test_engine_fixed_factor_matches_reference(name, cluster):
    """The engine with a fixed factor (bicpd's dGN, GaussNewton.py:92-99,
    293-297): 'cg' caps from the seeded RNG, the fixed factor put back after
    every step but not inside the dogleg trials."""
    g = load_golden(name)
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    o = _opts(g, tfx)
    o.cluster = cluster
    np.random.seed(int(g["seed"]))
    bf, ss, er, im, gr, st = tfx.dGN(g["T"], _start(g), R, o)
    assert st == int(g["stop"])
    assert len(er) == len(g["errors"])
    np.testing.assert_allclose(er, g["errors"], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(ss, g["step_sizes"], rtol=1e-5, atol=1e-12)
    np.testing.assert_allclose(np.concatenate([w.flatten('F') for w in bf]), g["best_x"], rtol=1e-5, atol=1e-8)


@pytest.mark.parametrize("name", ["dgn_als_L3", "dgn_direct_L3", "dgn_direct_big_L3"])
def test_inner_methods_fp32_within_tolerance(name):
    """FP32 factors and tensor (the direct system is still formed and solved in
    FP64): the first iterations' errors within 1e-4 relative of the reference's,
    the final error within 1.5x."""
    g = load_golden(name)
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    o = _opts(g, tfx)
    o.precision = 'fp32'
    bf, ss, er, im, gr, st = tfx.dGN(g["T"], _start(g), R, o)
    np.testing.assert_allclose(er[:4], g["errors"][:4], rtol=1e-4)
    assert er.min() < 1.5 * g["errors"].min()


@pytest.mark.parametrize("inner", ['als', 'direct'])
def test_cpd_with_inner_method_vs_oracle(inner):
    """tricpd with the inner method set (compression, seeded random start,
    dGN, decompression) against the oracle's cpd on the same seed."""
    rng = np.random.default_rng(40)
    dims, R = (14, 12, 10), 3
    W = [rng.standard_normal((d, R)) for d in dims]
    T = orc.cpd2tens(W) + 1e-4 * rng.standard_normal(dims)

    class O:
        inner_method = inner
        maxiter = 40
    np.random.seed(41)
    f0, out0 = orc.cpd(T, R, orc.make_options(O))
    np.random.seed(41)
    f1, out1 = tfx.cpd(T, R, tfx.make_options(O))
    assert out1.stop[0] == out0.stop[0]
    np.testing.assert_allclose(out1.errors[0], out0.errors[0], rtol=1e-6)
    np.testing.assert_allclose(out1.rel_error, out0.rel_error, rtol=1e-6)


def test_direct_unequal_dims_uses_truncated_hessian():
    """Modes of different size: the reference's truncated off-diagonal blocks
    (not J^T J) decide the step; the oracle's exact-J^T J variant would not
    match the first error."""
    g = load_golden("dgn_direct_L3")
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    o = _opts(g, tfx)
    o.maxiter = 3
    _, _, er, _, _, _ = tfx.dGN(g["T"], _start(g), R, o)
    np.testing.assert_allclose(er, g["errors"][:3], rtol=1e-8)


def test_mixing_engine_and_stepped_methods_is_refused():
    g = load_golden("dgn_direct_L3")
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    o = _opts(g, tfx)
    o.inner_method = ['cg'] * 3 + ['direct'] * 27
    with pytest.raises(NotImplementedError):
        tfx.dGN(g["T"], _start(g), R, o)


def test_stats_with_direct_inner_method():
    """The sweep driver routes 'direct' problems through the stepped loop."""
    rng = np.random.default_rng(42)
    dims, R = (8, 7, 6), 2
    W = [rng.standard_normal((d, R)) for d in dims]
    T = orc.cpd2tens(W) + 1e-5 * rng.standard_normal(dims)

    class O:
        inner_method = 'direct'
        maxiter = 30
    np.random.seed(43)
    times, steps, errors = tfx.stats(T, R, tfx.make_options(O), num_samples=3)
    assert np.all(np.isfinite(errors)) and errors.min() < 1e-3
