"""Dense device kernels (Gram, TTM, eigensolver, residual) and the full cpd vs the reference."""
import numpy as np
import pytest

import tfx_oracle as orc
from conftest import load_golden, split_x

pytestmark = pytest.mark.gpu

tfx = pytest.importorskip("tensorfox_gb300")
torch = pytest.importorskip("torch")
from tensorfox_gb300 import kernels  # noqa: E402


def dev(a, dt=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dt)


@pytest.mark.parametrize("shape,l", [((37, 23, 19), 0), ((37, 23, 19), 1), ((37, 23, 19), 2),
                                     ((130, 70, 5), 0), ((9, 8, 7, 6), 2), ((300, 4, 3), 0)])
@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
def test_mode_gram(shape, l, dt):
    rng = np.random.default_rng(1)
    T = rng.standard_normal(shape)
    G = kernels.mode_gram(dev(T, dt), list(shape), l).double().cpu().numpy()
    U = orc.unfold(T, l + 1)
    ref = U @ U.T
    tol = 1e-12 if dt == torch.float64 else 2e-5
    np.testing.assert_allclose(G, ref, rtol=tol, atol=tol * np.abs(ref).max())


@pytest.mark.parametrize("shape,l,n", [((37, 23, 19), 0, 5), ((37, 23, 19), 1, 7), ((37, 23, 19), 2, 19),
                                       ((40, 30, 5), 2, 3), ((9, 8, 7, 6), 1, 4)])
def test_ttm(shape, l, n):
    rng = np.random.default_rng(2)
    T = rng.standard_normal(shape)
    U = np.linalg.qr(rng.standard_normal((shape[l], n)))[0]
    out, new_shape = kernels.ttm(dev(T), list(shape), l, dev(U.T.copy()))
    ref = np.moveaxis(np.tensordot(U.T, T, axes=(1, l)), 0, l)
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("n", [1, 2, 5, 16, 33, 64, 90])
def test_sym_eig(n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    A = A + A.T
    ev, V = kernels.sym_eig(dev(A))
    ev, V = ev.cpu().numpy(), V.cpu().numpy()
    ref = np.sort(np.linalg.eigvalsh(A))[::-1]
    np.testing.assert_allclose(ev, ref, rtol=1e-10, atol=1e-10)
    # A v = lambda v for every returned pair, V orthonormal
    np.testing.assert_allclose(A @ V.T, V.T * ev, atol=1e-9)
    np.testing.assert_allclose(V @ V.T, np.eye(n), atol=1e-10)


def test_orthonormalize():
    rng = np.random.default_rng(3)
    Y = rng.standard_normal((20, 500))
    Yd = dev(Y)
    kernels.orthonormalize(Yd)
    Q = Yd.cpu().numpy()
    np.testing.assert_allclose(Q @ Q.T, np.eye(20), atol=1e-12)
    # same span
    P = Q.T @ Q
    np.testing.assert_allclose(P @ Y.T, Y.T, atol=1e-9)


@pytest.mark.parametrize("dims,R", [((20, 15, 12), 4), ((9, 8, 7, 6), 3), ((70, 3, 66), 5), ((100, 40, 30), 7),
                                    ((65, 33, 17), 20), ((12, 300, 2), 50)])
@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
def test_cp_residual_and_norms(dims, R, dt):
    rng = np.random.default_rng(4)
    W = [rng.standard_normal((d, R)) for d in dims]
    T = rng.standard_normal(dims)
    x = np.concatenate([w.flatten('F') for w in W])
    got = float(kernels.cp_residual_sq(dev(T, dt), dims, dev(x, dt), R).cpu().numpy()[0])
    ref = orc.fastnorm(orc.unfold(T, 1), orc.cpd2unfold1(W)) ** 2
    tol = 1e-12 if dt == torch.float64 else 1e-5
    assert abs(got - ref) <= tol * ref
    nrm = kernels.tensor_norms(dev(T, dt)).cpu().numpy()
    assert abs(nrm[0] - np.sum(T ** 2)) <= tol * np.sum(T ** 2)
    assert abs(nrm[1] - np.sum(np.abs(T))) <= tol * np.sum(np.abs(T))


@pytest.mark.parametrize("name", ["mlsvd_seq", "mlsvd_classic", "mlsvd_seq_L4"])
def test_mlsvd_matches_reference(name):
    g = load_golden(name)
    T, R = g["T"], int(g["R"])
    o = tfx.make_options(None)
    o.mlsvd_method = str(g["method"])
    np.random.seed(int(g["seed"]))
    S, U, T1, sig = tfx.mlsvd(T, np.linalg.norm(T), R, o)
    assert [u.shape[1] for u in U] == list(g["ranks"])
    np.testing.assert_allclose(np.concatenate(sig), g["sigmas"], rtol=1e-6)
    Uref = np.concatenate([u.flatten('F') for u in U])
    # same singular vectors (signs fixed by the shared convention)
    np.testing.assert_allclose(Uref, g["U"], atol=1e-6)
    np.testing.assert_allclose(S, g["S"], rtol=1e-5, atol=1e-6 * np.abs(g["S"]).max())


def test_mlsvd_keeps_rng_in_step():
    g = load_golden("mlsvd_seq")
    np.random.seed(3)
    orc.mlsvd(g["T"], 1.0, int(g["R"]), None)
    want = np.random.rand()
    np.random.seed(3)
    tfx.mlsvd(g["T"], 1.0, int(g["R"]), None)
    assert np.random.rand() == want


def _congruence(A, B):
    """Mean over columns of the product over modes of |cos| after best column matching."""
    R = A[0].shape[1]
    C = np.ones((R, R))
    for a, b in zip(A, B):
        an = a / np.linalg.norm(a, axis=0)
        bn = b / np.linalg.norm(b, axis=0)
        C *= np.abs(an.T @ bn)
    from scipy.optimize import linear_sum_assignment
    r, c = linear_sum_assignment(-C)
    return C[r, c].min()


def _opts(g):
    o = tfx.Options()
    for k, v in zip(g["opt_names"], g["opt_values"]):
        setattr(o, str(k), eval(str(v)))
    return o


@pytest.mark.parametrize("name", ["cpd_c1_small", "cpd_L4", "cpd_refine", "cpd_smart", "cpd_smart_random",
                                  "cpd_overrank", "cpd_symm", "cpd_symm_direct"])
def test_cpd_matches_reference(name):
    g = load_golden(name)
    T, R = g["T"], int(g["R"])
    np.random.seed(int(g["seed"]))
    f, out = tfx.cpd(T, R, _opts(g))
    ref = float(g["rel_error"])
    assert abs(out.rel_error - ref) <= 1e-2 * ref
    dims = T.shape
    fref = split_x(g["factors"], dims, R)
    assert _congruence(f, fref) > 0.999
    assert _congruence(f, split_x(g["planted"], dims, R)) > 0.999


def test_reference_doctest_tensor():
    """tests/simple_tensor_cpd_options.py:17-35 of the reference."""
    g = load_golden("ref_tests_2x2x2")
    errs = []
    for seed in range(10):
        np.random.seed(seed)
        _, out = tfx.cpd(g["T"], 3)
        errs.append(out.rel_error)
    assert min(errs) < 1e-14
    o = tfx.make_options(None)
    o.initialization = [np.ones((2, 3))] * 3
    _, out = tfx.cpd(g["T"], 3, o)
    assert out.rel_error < 0.14
    o.refine = True
    _, out = tfx.cpd(g["T"], 3, o)
    assert out.rel_error < 0.14
    o.refine = False
    o.inner_method = 'cg_static'
    o.cg_maxiter = 3
    o.cg_tol = 1e-7
    _, out = tfx.cpd(g["T"], 3, o)
    assert out.rel_error < 0.14


def test_cpd_fp32_planted():
    rng = np.random.default_rng(11)
    dims, R = (60, 50, 40), 6
    W = [rng.standard_normal((d, R)) for d in dims]
    T = orc.cpd2tens(W)
    T = (T + 1e-3 * np.linalg.norm(T) / np.sqrt(T.size) * rng.standard_normal(dims)).astype(np.float32)
    np.random.seed(0)
    f, out = tfx.cpd(T, R)
    assert out.rel_error < 2e-3
    assert _congruence(f, W) > 0.999


@pytest.mark.parametrize("shape,l,n", [((512, 96, 64), 0, 50), ((50, 128, 2048), 1, 50), ((64, 64, 72), 0, 70),
                                       ((12, 40, 128), 1, 9)])
def test_ttm_f32_tiled(shape, l, n):
    """FP32 mode products on the register-tiled path (D, Q multiples of 4, Q >= 128)."""
    rng = np.random.default_rng(5)
    T = rng.standard_normal(shape).astype(np.float32)
    U = rng.standard_normal((shape[l], n)).astype(np.float32)
    out, _ = kernels.ttm(dev(T, torch.float32), list(shape), l, dev(U.T.copy(), torch.float32))
    ref = np.moveaxis(np.tensordot(U.T.astype(np.float64), T.astype(np.float64), axes=(1, l)), 0, l)
    scale = np.sqrt(shape[l]) * np.abs(U).max() * np.abs(T).max()
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=0, atol=2e-6 * scale)


def test_orthonormalize_f32_graded():
    """CGS2 keeps FP32 columns orthonormal when their norms span eight decades (a
    subspace-iteration block with signal and noise directions)."""
    rng = np.random.default_rng(6)
    D, k = 512, 60
    scales = 10.0 ** -np.linspace(0, 8, k)
    Y = (rng.standard_normal((k, D)) * scales[:, None]).astype(np.float32)
    Yd = dev(Y, torch.float32)
    kernels.orthonormalize(Yd)
    Q = Yd.double().cpu().numpy()
    np.testing.assert_allclose(Q @ Q.T, np.eye(k), atol=2e-6)
    # the leading columns span the same space as the input's leading columns
    for j in (1, 8, 20):
        P = Q[:j].T @ Q[:j]
        Yj = Y[:j].astype(np.float64)
        assert np.linalg.norm(P @ Yj.T - Yj.T) <= 1e-5 * np.linalg.norm(Yj)


@pytest.mark.parametrize("n", [60, 33])
def test_sym_eig_f32_graded(n):
    """FP32 Jacobi on a Rayleigh-Ritz sized matrix with a graded spectrum stops by
    its relative threshold (well before the sweep cap) and resolves the leading pairs."""
    rng = np.random.default_rng(7 + n)
    V0 = np.linalg.qr(rng.standard_normal((n, n)))[0]
    lam = 10.0 ** -np.linspace(0, 8, n)
    A = (V0 * lam) @ V0.T
    ev, V, sweeps = kernels.sym_eig(dev(A, torch.float32), return_sweeps=True)
    assert sweeps < 20
    ev, V = ev.double().cpu().numpy(), V.double().cpu().numpy()
    np.testing.assert_allclose(ev[:10], lam[:10], rtol=5e-5)
    # ~12 sweeps of 59 rotations per vector in FP32
    np.testing.assert_allclose(V @ V.T, np.eye(n), atol=5e-5)
    for i in range(5):
        assert abs(abs(V[i] @ V0[:, i]) - 1.0) < 1e-5


@pytest.mark.parametrize("M,K,N,tA,tB", [(60, 512, 512, False, False), (50, 60, 20480, False, False),
                                         (70, 64, 256, False, False), (60, 512, 60, False, True),
                                         (33, 20, 130, False, False), (16, 48, 96, True, False),
                                         (64, 300, 77, False, True), (1, 1000, 33, False, False)])
def test_matmul_f32(M, K, N, tA, tB):
    """FP32 device products: the wide ones on the register-tiled kernel, short
    left factors (M <= 64, K >= 32) on the K-quartered kernel (partial K
    chunks and column blocks included), the rest on the tiled GEMM."""
    rng = np.random.default_rng(8)
    A = rng.standard_normal((K, M) if tA else (M, K)).astype(np.float32)
    B = rng.standard_normal((N, K) if tB else (K, N)).astype(np.float32)
    got = kernels.matmul(dev(A, torch.float32), dev(B, torch.float32), transA=tA, transB=tB).double().cpu().numpy()
    ref = (A.T if tA else A).astype(np.float64) @ (B.T if tB else B).astype(np.float64)
    np.testing.assert_allclose(got, ref, rtol=0, atol=2e-6 * np.sqrt(K) * np.abs(ref).max())


@pytest.mark.parametrize("M,K,N,tB", [(60, 512, 512, False), (60, 512, 60, True), (7, 129, 40, False)])
def test_matmul_f64_short_left_factor(M, K, N, tB):
    """The K-quartered kernel in FP64: rounding-level agreement with NumPy."""
    rng = np.random.default_rng(9)
    A = rng.standard_normal((M, K))
    B = rng.standard_normal((N, K) if tB else (K, N))
    got = kernels.matmul(dev(A), dev(B), transB=tB).cpu().numpy()
    ref = A @ (B.T if tB else B)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13 * np.sqrt(K) * np.abs(ref).max())


@pytest.mark.parametrize("dims,R", [((257, 131, 128), 50), ((129, 129, 256), 64), ((300, 140, 100), 1)])
def test_cp_residual_tensor_core_path(dims, R):
    """Large FP32 third-order tensors take the tcgen05 residual (3xTF32 products,
    partial row and column tiles here): FP32-level agreement with FP64."""
    rng = np.random.default_rng(8)
    W = [rng.standard_normal((d, R)).astype(np.float32) for d in dims]
    M = np.einsum('ir,jr,kr->ijk', *[w.astype(np.float64) for w in W])
    T = (M + 1e-2 * rng.standard_normal(dims)).astype(np.float32)
    ref = float(np.sum((T.astype(np.float64) - M) ** 2))
    x = np.concatenate([w.flatten('F') for w in W]).astype(np.float32)
    got = float(kernels.cp_residual_sq(dev(T, torch.float32), list(dims), dev(x, torch.float32), R).cpu().numpy()[0])
    assert abs(got - ref) <= 2e-5 * ref


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cpd_truncating_mlsvd_falls_back_in_step_with_reference(precision):
    """An exact rank-2 tensor asked for rank 4: the MLSVD's energy truncation
    keeps 2 singular vectors per mode instead of the assumed 4, so the queued
    (speculative) path is discarded and the CPD reruns mode by mode.  NumPy's
    RNG afterwards is where the oracle leaves it.  'cg_static' keeps the dGN
    itself free of draws: a rank-4 fit of a rank-2 tensor is degenerate and its
    iteration count (hence the number of 'cg' cap draws) changes with the last
    bit of the input, in the reference as well.  tol_mlsvd is 1e-6: at the
    default 1e-16 the truncation of exactly-zero directions is decided below
    the Gram route's resolution (eigenvalues of T T^T carry ~1e-16 of the
    largest), where the reference's SVD still sees them as zero."""
    rng = np.random.default_rng(77)
    dims, R = (10, 9, 8), 4
    W = [rng.standard_normal((d, 2)) for d in dims]
    T = orc.cpd2tens(W)

    class O:
        inner_method = 'cg_static'
        cg_maxiter = 8
        maxiter = 30
        tol_mlsvd = 1e-6
    np.random.seed(78)
    _, out0 = orc.cpd(T, R, orc.make_options(O))
    want = np.random.rand()
    o = tfx.make_options(O)
    o.precision = precision
    np.random.seed(78)
    _, out1 = tfx.cpd(T if precision == "fp64" else T.astype(np.float32), R, o)
    assert out0.rel_error < 1e-6
    if precision == "fp64":
        assert np.random.rand() == want
        assert out1.rel_error < 1e-6
    else:
        # the TF32 Gram lifts the zero singular values to ~1e-3 of the largest,
        # so whether 'mixed' truncates is its own (precision-dependent) decision
        assert out1.rel_error < 1e-2
