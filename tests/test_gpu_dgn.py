"""Device dGN engine vs the reference's golden trajectories and the oracle."""
import numpy as np
import pytest

import tfx_oracle as orc
from conftest import load_golden, split_x

pytestmark = pytest.mark.gpu

tfx = pytest.importorskip("tensorfox_gb300")


def _opts(g, mod):
    o = mod.Options()
    for k, v in zip(g["opt_names"], g["opt_values"]):
        setattr(o, str(k), eval(str(v)))
    return mod.make_options(o)


@pytest.mark.parametrize("name", ["dgn_static_L3", "dgn_cg_L3", "dgn_cg_L4", "dgn_small_L3"])
def test_dgn_fp64_matches_reference_trajectory(name):
    g = load_golden(name)
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    np.random.seed(int(g["seed"]))
    bf, ss, er, im, gr, st = tfx.dGN(g["T"], split_x(g["init_x"], dims, R), R, _opts(g, tfx))
    assert st == int(g["stop"])
    assert len(er) == len(g["errors"])
    np.testing.assert_allclose(er, g["errors"], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(ss, g["step_sizes"], rtol=1e-5, atol=1e-12)
    np.testing.assert_allclose(gr, g["gradients"], rtol=1e-5, atol=1e-12)
    np.testing.assert_allclose(np.concatenate([w.flatten('F') for w in bf]), g["best_x"], rtol=1e-5, atol=1e-8)


def test_dgn_rng_stays_in_step_with_reference():
    """After a 'cg' solve the global RNG is where the reference leaves it."""
    g = load_golden("dgn_cg_L3")
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    np.random.seed(5)
    orc.dGN(g["T"], split_x(g["init_x"], dims, R), R, orc.make_options(None))
    want = np.random.rand()
    np.random.seed(5)
    tfx.dGN(g["T"], split_x(g["init_x"], dims, R), R, tfx.make_options(None))
    assert np.random.rand() == want


def test_dgn_until_first_dogleg():
    g = load_golden("dgn_dogleg_L3")
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    np.random.seed(int(g["seed"]))
    _, ss, er, im, gr, st = tfx.dGN(g["T"], split_x(g["init_x"], dims, R), R, _opts(g, tfx))
    np.testing.assert_allclose(er[:7], g["errors"][:7], rtol=1e-8)
    assert np.all(np.isfinite(er))


@pytest.mark.parametrize("cluster", [1, 2, 4])
def test_dgn_cluster_sizes_agree(cluster):
    g = load_golden("dgn_static_L3")
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    o = _opts(g, tfx)
    o.cluster = cluster
    if cluster > R:
        pytest.skip("cluster wider than rank")
    bf, ss, er, im, gr, st = tfx.dGN(g["T"], split_x(g["init_x"], dims, R), R, o)
    np.testing.assert_allclose(er, g["errors"], rtol=1e-6, atol=1e-12)


def test_dgn_fp32_within_tolerance():
    """FP32 engine: per-iteration errors within 1e-5 relative of the FP64 oracle
    for the first iterations (the trajectories then drift apart by rounding)."""
    g = load_golden("dgn_static_L3")
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    o = _opts(g, tfx)
    o.precision = 'fp32'
    bf, ss, er, im, gr, st = tfx.dGN(g["T"], split_x(g["init_x"], dims, R), R, o)
    np.testing.assert_allclose(er[:8], g["errors"][:8], rtol=1e-4)
    assert er[-1] < 1.5 * g["errors"][-1]


def test_dgn_larger_core_vs_oracle():
    """A 24x20x16 core at R=8 with cluster 4 against the oracle (cg_static)."""
    rng = np.random.default_rng(7)
    dims, R = (24, 20, 16), 8
    W = [rng.standard_normal((d, R)) for d in dims]
    T = orc.cpd2tens(W) + 1e-3 * rng.standard_normal(dims)
    init = [w + 0.2 * rng.standard_normal(w.shape) for w in W]

    class O:
        inner_method = 'cg_static'
        cg_maxiter = 12
        maxiter = 25
    _, ss0, er0, _, _, st0 = orc.dGN(T, [w.copy() for w in init], R, orc.make_options(O))
    for c in (1, 4, 8):
        o = tfx.make_options(O)
        o.cluster = c
        _, ss1, er1, _, _, st1 = tfx.dGN(T, [w.copy() for w in init], R, o)
        assert st1 == st0
        np.testing.assert_allclose(er1, er0, rtol=1e-7)


def test_dgn_order12_vs_oracle():
    """The largest order the reference accepts (12): a 2^12 tensor at rank 2."""
    rng = np.random.default_rng(12)
    dims, R = (2,) * 12, 2
    W = [rng.standard_normal((d, R)) for d in dims]
    T = orc.cpd2tens(W) + 1e-4 * rng.standard_normal(dims)
    init = [w + 0.2 * rng.standard_normal(w.shape) for w in W]

    class O:
        inner_method = 'cg_static'
        cg_maxiter = 6
        maxiter = 15
    _, ss0, er0, _, _, st0 = orc.dGN(T, [w.copy() for w in init], R, orc.make_options(O))
    _, ss1, er1, _, _, st1 = tfx.dGN(T, [w.copy() for w in init], R, tfx.make_options(O))
    assert st1 == st0 and len(er1) == len(er0)
    np.testing.assert_allclose(er1, er0, rtol=1e-7)


def _start(g):
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    f = split_x(g["init_x"], dims, R)
    if "alias" in g and int(g["alias"]):
        return [f[0]] * len(dims)     # one array for every mode
    return f


@pytest.mark.parametrize("name", ["dgn_symm_L3", "dgn_symm_alias_L3", "dgn_symm_norm_L3"])
@pytest.mark.parametrize("cluster", [1, 2])
def test_dgn_symm_matches_reference(name, cluster):
    """symm=True on the engine: the reference's in-place x2cpd / transform on a
    factor list that holds one array L times (a symmetric start, then every
    iteration after a symmetrising transform) reproduced, fixed norm included."""
    g = load_golden(name)
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    o = _opts(g, tfx)
    o.cluster = cluster
    bf, ss, er, im, gr, st = tfx.dGN(g["T"], _start(g), R, o)
    assert st == int(g["stop"])
    assert len(er) == len(g["errors"])
    np.testing.assert_allclose(er, g["errors"], rtol=1e-6, atol=1e-12)
    # step sizes late in the run are differences of nearly equal points: the
    # rounding of the engine's reductions shows there first (1.7e-5 seen)
    np.testing.assert_allclose(ss, g["step_sizes"], rtol=1e-4, atol=1e-12)


@pytest.mark.parametrize("name", ["dgn_damp_sched_L3", "dgn_norm_L3"])
def test_dgn_options_match_reference(name):
    """A damping schedule (init_damp as a list, GaussNewton.py:110-111, 490-495)
    and factors_norm (Conversion.py:439-442) on the engine."""
    g = load_golden(name)
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    bf, ss, er, im, gr, st = tfx.dGN(g["T"], _start(g), R, _opts(g, tfx))
    assert st == int(g["stop"])
    assert len(er) == len(g["errors"])
    np.testing.assert_allclose(er, g["errors"], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(ss, g["step_sizes"], rtol=1e-4, atol=1e-12)


@pytest.mark.parametrize("dims,R", [((50, 48, 44), 12), ((50, 50, 50), 50), ((64, 60, 56), 24)])
def test_dgn_large_core_slab_split_gradient_vs_oracle(dims, R):
    """Cores large enough for the slab-split gradient (every CTA streams its own
    slabs for all columns, partials summed through distributed shared memory):
    FP64 trajectories equal the oracle's for several cluster sizes; FP32 stays
    within 1e-3 of them over the first iterations (the FP32 and FP64 paths
    drift apart by rounding as the damping and CG caps compound it)."""
    rng = np.random.default_rng(31)
    W = [rng.standard_normal((d, R)) for d in dims]
    T = orc.cpd2tens(W) + 1e-3 * rng.standard_normal(dims)
    init = [w + 0.2 * rng.standard_normal(w.shape) for w in W]

    class O:
        inner_method = 'cg_static'
        cg_maxiter = 10
        maxiter = 12
    _, ss0, er0, _, gr0, st0 = orc.dGN(T, [w.copy() for w in init], R, orc.make_options(O))
    for c in (None, 4, 12):
        if c is not None and c > R:
            continue
        o = tfx.make_options(O)
        o.cluster = c
        _, ss1, er1, _, gr1, st1 = tfx.dGN(T, [w.copy() for w in init], R, o)
        assert st1 == st0 and len(er1) == len(er0)
        np.testing.assert_allclose(er1, er0, rtol=1e-8)
        np.testing.assert_allclose(gr1, gr0, rtol=1e-6)
        o.precision = 'fp32'
        _, _, er2, _, _, _ = tfx.dGN(T.astype(np.float32), [w.copy() for w in init], R, o)
        np.testing.assert_allclose(er2[:6], er0[:6], rtol=1e-3)


def test_dense_mttkrp_dgn_vs_oracle():
    """The MTTKRP-driven dGN on a dense FP32 tensor (tensor-core MTTKRPs, the
    direct residual, the grid-wide CG) from the same start as the FP64 oracle's
    dGN: the errors agree within 1e-4 over the first iterations (FP32 against
    FP64) and the run ends near the oracle's final error."""
    import torch
    from tensorfox_gb300 import mttkrp_dgn
    rng = np.random.default_rng(41)
    dims, R = (96, 80, 64), 8
    W = [rng.standard_normal((d, R)) for d in dims]
    T = orc.cpd2tens(W) + 1e-3 * rng.standard_normal(dims)
    init = [w + 0.2 * rng.standard_normal(w.shape) for w in W]

    class O:
        inner_method = 'cg_static'
        cg_maxiter = 10
        maxiter = 30
    _, ss0, er0, _, _, st0 = orc.dGN(T, [w.copy() for w in init], R, orc.make_options(O))
    Td = torch.from_numpy(T.astype(np.float32)).cuda()
    x0 = torch.from_numpy(orc.cpd2flat(init)).cuda().float()
    best, ss1, er1, _, gr1, st1, mv = mttkrp_dgn.dgn_dense(Td, x0, R, tfx.make_options(O))
    np.testing.assert_allclose(er1[:8], er0[:8], rtol=1e-4)
    assert abs(min(er1) - min(er0)) <= 1e-2 * min(er0)


def test_cpd_refine_fp32_on_tensor_cores_vs_oracle():
    """cpd(refine=True) on a 256^3 FP32 tensor: the refinement on the full tensor
    takes the MTTKRP-driven dGN (tensor-core MTTKRPs); its final error is
    within 1e-2 of the FP64 oracle's refined error and the factors are
    congruent (> 0.999) to the oracle's and to the planted ones."""
    import torch
    from scipy.optimize import linear_sum_assignment
    rng = np.random.default_rng(43)
    dims, R = (256, 256, 256), 12
    W = [rng.standard_normal((d, R)) for d in dims]
    T = orc.cpd2tens(W)
    T = T + 1e-2 * np.linalg.norm(T) / np.sqrt(T.size) * rng.standard_normal(dims)

    class O:
        refine = True
        maxiter = 60
    np.random.seed(2)
    f0, o0 = orc.cpd(T, R, orc.make_options(O))
    np.random.seed(2)
    f1, o1 = tfx.cpd(torch.from_numpy(T.astype(np.float32)).cuda(), R, tfx.make_options(O))
    assert abs(o1.rel_error - o0.rel_error) <= 1e-2 * o0.rel_error

    def cong(A, B):
        C = np.ones((R, R))
        for a, b in zip(A, B):
            C *= np.abs((a / np.linalg.norm(a, axis=0)).T @ (b / np.linalg.norm(b, axis=0)))
        r, c = linear_sum_assignment(-C)
        return C[r, c].min()
    assert cong(f1, f0) > 0.999 and cong(f1, W) > 0.999
