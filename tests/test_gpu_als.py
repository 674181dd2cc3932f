"""Device ALS (tfx_als_solve, one graph launch per solve) vs the reference's
golden trajectories and the oracle (Alternating_Least_Squares.py:18-235)."""
import numpy as np
import pytest
import torch

import tfx_oracle as orc
from conftest import load_golden, split_x

pytestmark = pytest.mark.gpu

tfx = pytest.importorskip("tensorfox_gb300")


def _opts(g, mod):
    o = mod.Options()
    for k, v in zip(g["opt_names"], g["opt_values"]):
        setattr(o, str(k), eval(str(v)))
    return mod.make_options(o)


@pytest.mark.parametrize("name", ["als_L3", "als_L4", "als_stall_L3", "als_symm_L3", "als_norm_L3"])
def test_als_fp64_matches_reference_trajectory(name):
    g = load_golden(name)
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    f, ss, er, im, gr, st = tfx.als(g["T"], split_x(g["init_x"], dims, R), R, _opts(g, tfx))
    assert st == int(g["stop"])
    assert len(er) == len(g["errors"])
    np.testing.assert_allclose(er, g["errors"], rtol=1e-7, atol=1e-13)
    np.testing.assert_allclose(ss, g["step_sizes"], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(np.concatenate([w.flatten('F') for w in f]), g["final_x"], rtol=1e-6, atol=1e-9)


def test_als_fp32_within_tolerance():
    """FP32 factors and MTTKRP, FP64 Gramians and inverse: the first iterations'
    errors within 1e-5 relative of the FP64 reference."""
    g = load_golden("als_L3")
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    o = _opts(g, tfx)
    o.precision = 'fp32'
    f, ss, er, im, gr, st = tfx.als(g["T"].astype(np.float32), split_x(g["init_x"], dims, R), R, o)
    np.testing.assert_allclose(er[:6], g["errors"][:6], rtol=1e-5)
    assert er[-1] < 1.05 * g["errors"][-1]


def test_als_larger_and_order5_vs_oracle():
    rng = np.random.default_rng(17)
    for dims, R, maxiter in (((24, 20, 16), 8, 25), ((6, 5, 5, 4, 3), 3, 20)):
        W = [rng.standard_normal((d, R)) for d in dims]
        T = orc.cpd2tens(W) + 1e-3 * rng.standard_normal(dims)
        init = [w + 0.3 * rng.standard_normal(w.shape) for w in W]

        class O:
            pass
        O.maxiter = maxiter
        f0, ss0, er0, _, _, st0 = orc.als(T, [w.copy() for w in init], R, orc.make_options(O))
        f1, ss1, er1, _, _, st1 = tfx.als(T, [w.copy() for w in init], R, tfx.make_options(O))
        assert st1 == st0 and len(er1) == len(er0)
        np.testing.assert_allclose(er1, er0, rtol=1e-8)
        np.testing.assert_allclose(orc.cpd2flat(f1), orc.cpd2flat(f0), rtol=1e-6, atol=1e-9)


def test_als_singular_normal_matrix_takes_pseudo_inverse():
    """Two identical columns in every factor make every H_l singular: the solve
    takes the eigen-decomposition route, and its minimum-norm update matches
    NumPy's pinv in the oracle."""
    from tensorfox_gb300.als import als_device
    rng = np.random.default_rng(23)
    dims, R = (9, 8, 7), 4
    T = rng.standard_normal(dims)
    init = [rng.standard_normal((d, R)) for d in dims]
    for w in init:
        w[:, 3] = w[:, 2]

    class O:
        maxiter = 6
    o = orc.make_options(O)
    f0, ss0, er0, _, _, st0 = orc.als(T, [w.copy() for w in init], R, o)
    Td = torch.from_numpy(T).cuda()
    x0 = torch.from_numpy(orc.cpd2flat(init)).cuda()
    x, best, stats, res, info = als_device(Td, x0, R, tfx.make_options(O), 'fp64')
    assert res[3] > 0                       # pseudo-inverse fallbacks taken
    n = int(res[1])
    np.testing.assert_allclose(stats[:n], er0, rtol=1e-6)


@pytest.mark.parametrize("name", ["cpd_als", "cpd_als_refine"])
def test_cpd_als_matches_reference(name):
    g = load_golden(name)
    T, R = g["T"], int(g["R"])
    o = tfx.Options()
    for k, v in zip(g["opt_names"], g["opt_values"]):
        setattr(o, str(k), eval(str(v)))
    np.random.seed(int(g["seed"]))
    f, out = tfx.cpd(T, R, o)
    ref = float(g["rel_error"])
    assert abs(out.rel_error - ref) <= 1e-2 * ref
    fref = split_x(g["factors"], T.shape, R)
    from test_gpu_dense import _congruence
    assert _congruence(f, fref) > 0.999
    assert _congruence(f, split_x(g["planted"], T.shape, R)) > 0.999
