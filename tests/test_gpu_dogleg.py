"""The device dogleg (GaussNewton.py:713-795), fed the same point, rejected
step, gradient, J^T J grad, error and damping as the reference, through
``tfx_dgn_dogleg`` -- the engine's own trial loop, not a copy of it.

Whole dGN trajectories cannot pin the dogleg past its first use (its first
trial re-evaluates the rejected point, a gain ratio of +-eps), so it is
compared here on inputs where every decision is well conditioned: the
reference's own golden case and oracle cases of several shapes."""
import numpy as np
import pytest

import tfx_oracle as orc
from conftest import load_golden

pytestmark = pytest.mark.gpu

tfx = pytest.importorskip("tensorfox_gb300")
torch = pytest.importorskip("torch")
from tensorfox_gb300 import gauss_newton as gn  # noqa: E402


def device_dogleg(T, x, y, g2, j2, err, damp, R, cluster, precision="fp64"):
    bw, bx, by, be = gn.dogleg_steps(T, x, y, g2, j2, err, damp, R, cluster=cluster, precision=precision)
    return bw.double().cpu().numpy(), bx.double().cpu().numpy(), by.double().cpu().numpy(), be


@pytest.mark.parametrize("cluster", [1, 2, 3])
def test_dogleg_matches_reference_golden(cluster):
    g = load_golden("dogleg_units")
    T = g["T"]
    R = len(g["x"]) // sum(T.shape)
    bf, bx, by, be = device_dogleg(T, g["x"], g["y"], g["g2"], g["j2"], float(g["err"]), float(g["damp"]), R,
                                   cluster)
    np.testing.assert_allclose(be, float(g["best_error"]), rtol=1e-10)
    np.testing.assert_allclose(bx, g["best_x"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(by, g["best_y"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(bf, g["best_f"], rtol=1e-10, atol=1e-12)


def oracle_case(dims, R, seed, step_scale, err_scale):
    rng = np.random.default_rng(seed)
    W = [rng.standard_normal((d, R)) for d in dims]
    T = orc.cpd2tens(W) + 0.05 * rng.standard_normal(dims)
    n = R * sum(dims)
    x = orc.cpd2flat(W) + 0.05 * rng.standard_normal(n)
    y = step_scale * rng.standard_normal(n)
    g2 = rng.standard_normal(n)
    j2 = 50 * g2 + rng.standard_normal(n)
    Tsize = np.linalg.norm(T)
    err = err_scale * np.linalg.norm(T - orc.cpd2tens(orc.x2cpd(x + y, [w.copy() for w in W]))) / Tsize
    return T, x, y, g2, j2, err


@pytest.mark.parametrize("dims,R,seed,step_scale,err_scale,damp",
                         [((9, 8, 7), 4, 1, 3.0, 1.0, 0.3), ((12, 10, 9), 5, 2, 0.5, 1.0, 1.0),
                          ((20, 15, 12), 6, 3, 8.0, 1.0, 0.05), ((6, 5, 4, 3), 3, 4, 2.0, 1.0, 0.3),
                          ((16, 16, 16), 8, 5, 4.0, 1.0, 2.0)])
@pytest.mark.parametrize("cluster", [1, 2])
def test_dogleg_matches_oracle(dims, R, seed, step_scale, err_scale, damp, cluster):
    T, x, y, g2, j2, err = oracle_case(dims, R, seed, step_scale, err_scale)
    ref_f, ref_x, ref_y, ref_e = orc.compute_dogleg_steps(np.linalg.norm(T), orc.unfold(T, 1),
                                                          [np.zeros((d, R)) for d in dims], g2, j2, x.copy(),
                                                          y.copy(), err, damp, False, 0)
    bf, bx, by, be = device_dogleg(T, x, y, g2, j2, err, damp, R, cluster)
    np.testing.assert_allclose(be, ref_e, rtol=1e-9)
    np.testing.assert_allclose(bx, ref_x, rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(by, ref_y, rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(bf, orc.cpd2flat(ref_f), rtol=1e-9, atol=1e-11)
