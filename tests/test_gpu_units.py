"""The solver's per-iteration products (gradient and J^T J v), taken from the
engine's own device code through ``tfx_jtj_matvec``, against the reference's
golden unit vectors (GaussNewton.py:401-427 compute_grad, :551-581 matvec) and
against the FP64 oracle at the compressed size of the 512^3 rank-50 workload.

FP32 criterion: within 1e-5 relative (norm-wise, and entry-wise against the
largest entry) of the FP64 result on the same FP32-rounded inputs."""
import numpy as np
import pytest

import tfx_oracle as orc
from conftest import load_golden, split_x

pytestmark = pytest.mark.gpu

tfx = pytest.importorskip("tensorfox_gb300")
torch = pytest.importorskip("torch")
from tensorfox_gb300 import gauss_newton as gn  # noqa: E402

FP32_TOL = 1e-5


def rel_ok(got, ref, tol):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    nrm = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    ent = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    assert nrm <= tol and ent <= tol, (nrm, ent)


def units(T, W, v, R, precision, cluster):
    g, jv = gn.jtj_matvec(T, W, R, v=v, damp=0.7, cluster=cluster, precision=precision)
    return g.double().cpu().numpy(), jv.double().cpu().numpy()


@pytest.mark.parametrize("name", ["units_L3", "units_L4", "units_L3_big", "units_L5"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_units_vs_reference_golden(name, precision):
    g = load_golden(name)
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    W = split_x(g["x"], dims, R)
    T, v = g["T"], g["v"]
    if precision == "fp64":
        ref_g, ref_mv, tol = g["grad"], g["matvec"], 1e-12
    else:
        # the reference's products on the FP32-rounded inputs (the oracle is
        # pinned to the golden vectors on CPU), so only the arithmetic counts
        W32 = [w.astype(np.float32).astype(np.float64) for w in W]
        T32 = T.astype(np.float32).astype(np.float64)
        v32 = v.astype(np.float32).astype(np.float64)
        Tl = [orc.unfold(T32, l + 1) for l in range(len(dims))]
        _, P1, P2 = orc.gramians(W32)
        ref_g = orc.compute_grad(Tl, W32, P1)
        ref_mv = orc.matvec(W32, P1, P2, v32)
        T, W, v, tol = T32.astype(np.float32), [w.astype(np.float32) for w in W32], v32.astype(np.float32), FP32_TOL
    for cluster in range(1, R + 1):
        got_g, got_mv = units(T, W, v, R, precision, cluster)
        rel_ok(got_g, ref_g, tol)
        rel_ok(got_mv, ref_mv, tol)


@pytest.mark.parametrize("cluster", [None, 8, 16])
def test_units_fp32_at_the_headline_core_size(cluster):
    """50 x 50 x 50 core, rank 50 (the compressed size of the 512^3 workload):
    a planted core with noise and a random start, as in the first dGN
    iteration; the engine's own cluster size (None) and two others."""
    rng = np.random.default_rng(17)
    dims, R = (50, 50, 50), 50
    Wp = [rng.standard_normal((d, R)) for d in dims]
    T = orc.cpd2tens(Wp) + 0.05 * rng.standard_normal(dims)
    W = [rng.standard_normal((d, R)) for d in dims]
    v = rng.standard_normal(R * sum(dims))
    T32 = T.astype(np.float32)
    W32 = [w.astype(np.float32) for w in W]
    v32 = v.astype(np.float32)
    T64, W64, v64 = T32.astype(np.float64), [w.astype(np.float64) for w in W32], v32.astype(np.float64)
    Tl = [orc.unfold(T64, l + 1) for l in range(3)]
    _, P1, P2 = orc.gramians(W64)
    ref_g = orc.compute_grad(Tl, W64, P1)
    ref_mv = orc.matvec(W64, P1, P2, v64)
    got_g, got_mv = units(T32, W32, v32, R, "fp32", cluster)
    rel_ok(got_g, ref_g, FP32_TOL)
    rel_ok(got_mv, ref_mv, FP32_TOL)
    # and the FP64 path to rounding level
    got_g, got_mv = units(T64, W64, v64, R, "fp64", cluster)
    rel_ok(got_g, ref_g, 1e-12)
    rel_ok(got_mv, ref_mv, 1e-12)
