"""The configurations the benchmark measures, against the FP64 oracle on the
same inputs.

* 512^3 FP32, rank 50, congruence 0.5, 40 dB SNR (the headline workload):
  ``precision='mixed'`` (TF32 tensor-core compression) and ``'fp32'`` against
  the FP64 oracle ``cpd`` -- final relative error within 1e-2 relative of the
  oracle's, factors congruent (> 0.999) to the oracle's and to the planted
  ones, and the GPU result's own error re-measured in FP64 on the host.
* 100^3 FP64, rank 10, noise 1e-6: the FP64 path reproduces the oracle's
  trajectory (per-iteration errors to 1e-6 relative)."""
import os
import sys

import numpy as np
import pytest

import tfx_oracle as orc

pytestmark = pytest.mark.gpu

tfx = pytest.importorskip("tensorfox_gb300")
torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
import bench  # noqa: E402


def congruence(A, B):
    """Smallest over matched columns of the product over modes of |cos|."""
    from scipy.optimize import linear_sum_assignment
    R = A[0].shape[1]
    C = np.ones((R, R))
    for a, b in zip(A, B):
        C *= np.abs((a / np.linalg.norm(a, axis=0)).T @ (b / np.linalg.norm(b, axis=0)))
    r, c = linear_sum_assignment(-C)
    return C[r, c].min()


def fp64_rel_error(T64, factors):
    """||T - [[W]]|| / ||T|| in FP64 on the host."""
    return orc.fastnorm(orc.unfold(T64, 1), orc.cpd2unfold1(factors)) / np.linalg.norm(T64)


@pytest.fixture(scope="module")
def headline():
    T, W = bench.make_problem()
    T64 = T.astype(np.float64)
    np.random.seed(0)
    f_ref, out_ref = orc.cpd(T64, bench.RANK)
    return T, T64, W, f_ref, out_ref


@pytest.mark.parametrize("precision", ["mixed", "fp32"])
def test_headline_workload_vs_fp64_oracle(headline, precision):
    T, T64, W, f_ref, out_ref = headline
    o = tfx.make_options(None)
    o.precision = precision
    np.random.seed(0)
    f, out = tfx.cpd(torch.from_numpy(T).cuda(), bench.RANK, o)
    assert abs(out.rel_error - out_ref.rel_error) <= 1e-2 * out_ref.rel_error
    # the GPU result's error measured in FP64 agrees with what it reports
    e64 = fp64_rel_error(T64, f)
    assert abs(e64 - out.rel_error) <= 1e-4 * e64
    assert abs(e64 - out_ref.rel_error) <= 1e-2 * out_ref.rel_error
    assert congruence(f, f_ref) > 0.999
    assert congruence(f, W) > 0.999


def test_c1_fp64_trajectory_equals_oracle():
    rng = np.random.default_rng(101)
    dims, R = (100, 100, 100), 10
    W = [rng.standard_normal((d, R)) for d in dims]
    T = np.einsum("ir,jr,kr->ijk", *W)
    E = rng.standard_normal(dims)
    T += 1e-6 * np.linalg.norm(T) / np.linalg.norm(E) * E
    np.random.seed(0)
    f_ref, o_ref = orc.cpd(T, R, None)
    np.random.seed(0)
    f, o = tfx.cpd(torch.from_numpy(T).cuda(), R, None)
    er, er_ref = np.asarray(o.errors[0]), np.asarray(o_ref.errors[0])
    n = min(len(er), len(er_ref))
    np.testing.assert_allclose(er[:n], er_ref[:n], rtol=1e-6)
    assert abs(o.rel_error - o_ref.rel_error) <= 1e-6 * o_ref.rel_error
    assert congruence(f, f_ref) > 0.999999
    assert congruence(f, W) > 0.9999
