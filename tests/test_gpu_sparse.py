"""Sparse (COO) device path vs the reference's golden vectors and the oracle."""
import numpy as np
import pytest

import tfx_oracle as orc
from conftest import load_golden, split_x

pytestmark = pytest.mark.gpu

tfx = pytest.importorskip("tensorfox_gb300")
torch = pytest.importorskip("torch")
from tensorfox_gb300 import sparse  # noqa: E402


def coo(dims, R, nnz, seed, noise=0.01):
    rng = np.random.default_rng(seed)
    lin = rng.choice(int(np.prod(dims)), size=nnz, replace=False)
    idxs = np.stack(np.unravel_index(lin, dims), axis=1).astype(np.int64)
    W = [rng.standard_normal((d, R)) for d in dims]
    model = np.ones((nnz, R))
    for l in range(len(dims)):
        model *= W[l][idxs[:, l]]
    return model.sum(1) + noise * rng.standard_normal(nnz), idxs, W


def dense_of(data, idxs, dims):
    T = np.zeros(dims)
    np.add.at(T, tuple(idxs.T), data)
    return T


def rm(W, dt):
    return [torch.from_numpy(np.ascontiguousarray(w)).to("cuda", dt) for w in W]


@pytest.mark.parametrize("dims,R,nnz", [((10, 9, 8), 3, 60), ((30, 20, 25), 7, 900), ((6, 5, 4, 3), 4, 200),
                                        ((40, 30, 20), 20, 3000), ((50, 40, 30), 16, 5000),
                                        ((25, 30, 35), 32, 4000)])
@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
def test_coo_mttkrp_vs_dense(dims, R, nnz, dt):
    data, idxs, W = coo(dims, R, nnz, 1)
    X = sparse.DeviceCOO(data, idxs, dims, dt)
    T = dense_of(data, idxs, dims)
    Tl = [orc.unfold(T, l + 1) for l in range(len(dims))]
    for l in range(len(dims)):
        got = sparse.coo_mttkrp(X, rm(W, dt), l).double().cpu().numpy()
        ref = orc.mttkrp(Tl, W, l)
        tol = 1e-12 if dt == torch.float64 else 1e-5
        np.testing.assert_allclose(got, ref, rtol=tol, atol=tol * np.abs(ref).max())


@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
def test_sparse_units_vs_reference(dt):
    g = load_golden("sparse_L3")
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    X = sparse.DeviceCOO(g["data"], g["idxs"], dims, dt)
    W = split_x(g["W"], dims, R)
    res = float(sparse.sparse_residual_sq(X, rm(W, dt)).cpu().numpy()[0])
    tol = 1e-12 if dt == torch.float64 else 1e-5
    assert abs(np.sqrt(res) - float(g["sparse_fastnorm"])) <= tol * float(g["sparse_fastnorm"])
    s = 0
    for l in range(3):
        G = X.gram(l).double().cpu().numpy().flatten()
        ref = g["grams"][s:s + dims[l] ** 2]
        s += dims[l] ** 2
        np.testing.assert_allclose(G, ref, rtol=tol, atol=tol * np.abs(ref).max())
    UT, s = [], 0
    for l, n in enumerate(g["UT_rows"]):
        UT.append(g["UT"][s:s + n * dims[l]].reshape(n, dims[l]))
        s += n * dims[l]
    S = sparse.sparse_ttmc(X, [torch.from_numpy(u).to("cuda", dt) for u in UT]).double().cpu().numpy()
    np.testing.assert_allclose(S, g["S"], rtol=tol, atol=tol * np.abs(g["S"]).max())


def test_coo_gram_with_shared_fibres():
    """Entries that share a fibre produce off-diagonal Gram terms; duplicates add up."""
    rng = np.random.default_rng(5)
    dims = (7, 3, 2)
    idxs = np.array([[i, j, k] for i in range(7) for j in range(3) for k in range(2) if rng.random() < 0.5])
    idxs = np.concatenate([idxs, idxs[:5]])            # duplicated coordinates
    data = rng.standard_normal(len(idxs))
    X = sparse.DeviceCOO(data, idxs, dims, torch.float64)
    T = dense_of(data, idxs, dims)
    for l in range(3):
        U = orc.unfold(T, l + 1)
        np.testing.assert_allclose(X.gram(l).cpu().numpy(), U @ U.T, rtol=1e-12, atol=1e-12)


def fibre_gram(data, idxs, d, mode):
    """T_(mode) T_(mode)^T from the entries, grouped by their exact fibre tuple."""
    others = np.delete(np.asarray(idxs), mode, axis=1)
    _, fib = np.unique(others, axis=0, return_inverse=True)
    V = np.zeros((fib.max() + 1, d))
    np.add.at(V, (fib.ravel(), np.asarray(idxs)[:, mode]), data)
    return V.T @ V


def test_coo_gram_wide_dims_no_key_wrap():
    """Order 4 with three modes of 1e7: the product of the other modes' dims
    (1e21) exceeds 2^64.  Fibre B below sits exactly 2^64 past fibre A in the
    mixed-radix order (i1 * 1e14 + i2 * 1e7 + i3), so a key formed that way in
    64 bits would merge them and add false off-diagonal terms."""
    dims = (6, 10 ** 7, 10 ** 7, 10 ** 7)
    A = (1, 2, 3)
    B = (1 + 184467, 2 + 4407370, 3 + 9551616)
    assert (B[0] - A[0]) * 10 ** 14 + (B[1] - A[1]) * 10 ** 7 + (B[2] - A[2]) == 2 ** 64
    rng = np.random.default_rng(8)
    rows = [[0] + list(A), [1] + list(A), [2] + list(B), [3] + list(B), [4] + list(A)]
    for _ in range(300):   # more fibres, some shared by several rows
        f = rng.integers(0, 10 ** 7, size=3) if rng.random() < 0.5 else np.array([7, 7, rng.integers(0, 4)])
        rows.append([int(rng.integers(0, 6))] + [int(v) for v in f])
    idxs = np.array(rows, dtype=np.int64)
    data = rng.standard_normal(len(idxs))
    want = fibre_gram(data, idxs, 6, 0)
    # what a wrapped 64-bit key would give: fibres A and B merged
    merged = idxs.copy()
    merged[2:4, 1:] = A
    wrapped = fibre_gram(data, merged, 6, 0)
    assert not np.allclose(want, wrapped)
    X = sparse.DeviceCOO(data, idxs, dims, torch.float64)
    np.testing.assert_allclose(X.gram(0).cpu().numpy(), want, rtol=1e-12, atol=1e-12)


def test_coo_encode_rejects_out_of_range():
    with pytest.raises(ValueError):
        sparse.DeviceCOO(np.ones(2), np.array([[0, 0, 0], [0, 5, 0]]), (3, 3, 3), torch.float64)


def test_sparse_cpd_vs_reference():
    g = load_golden("sparse_L3")
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    np.random.seed(41)
    f, out = tfx.cpd([g["data"], g["idxs"], np.array(dims)], R)
    ref = float(g["cpd_rel_error"])
    # same semantics (absent entries are zeros); trajectories differ by rounding only
    assert abs(out.rel_error - ref) <= 0.05 * ref + 1e-3
    assert out.stop[1] == 8


def test_reference_sparse_doctest():
    """tests/sparse_tensors.py:8-30 of the reference: an exactly low-rank sparse
    tensor (sparse factors), best of 10, dense relative error < 1e-4."""
    rng = np.random.default_rng(9)
    dims, R = [10, 10, 10, 10], 5
    W = []
    for d in dims:
        M = np.zeros((d, R))
        for _ in range(10):
            M[rng.integers(d), rng.integers(R)] = rng.standard_normal()
        W.append(M)
    T = orc.cpd2tens(W)
    idxs = np.argwhere(T != 0)
    data = T[tuple(idxs.T)]
    best = 1.0
    for seed in range(10):
        np.random.seed(seed)
        f, out = tfx.cpd([data, idxs, dims], R)
        err = np.linalg.norm(T - orc.cpd2tens(f)) / np.linalg.norm(T)
        best = min(best, err)
    assert best < 1e-4


@pytest.mark.parametrize("R", [16, 12])
def test_coo_vectorized_paths_with_unaligned_factors(R):
    """The FP32 R % 4 == 0 kernels read factor rows as 16-byte vectors; factor
    bases off a 16-byte boundary take their scalar reads, with the same result."""
    dims, nnz = (30, 25, 20), 2500
    data, idxs, W = coo(dims, R, nnz, 3)
    X = sparse.DeviceCOO(data, idxs, dims, torch.float32)
    T = dense_of(data, idxs, dims)
    Tl = [orc.unfold(T, l + 1) for l in range(len(dims))]
    al = rm(W, torch.float32)
    # the same factors at a 4-byte offset inside a larger buffer
    un = []
    for w in W:
        buf = torch.zeros(w.size + 1, dtype=torch.float32, device="cuda")
        buf[1:] = torch.from_numpy(np.ascontiguousarray(w, dtype=np.float32).ravel()).cuda()
        un.append(buf[1:].view(w.shape))
    assert all(u.data_ptr() % 16 != 0 for u in un)
    for l in range(len(dims)):
        ref = orc.mttkrp(Tl, W, l)
        for fac in (al, un):
            got = sparse.coo_mttkrp(X, fac, l).double().cpu().numpy()
            np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max())
    model = np.ones((len(data), R))
    for l in range(len(dims)):
        model *= W[l][np.asarray(idxs)[:, l]]
    want = float(np.sum((np.asarray(data) - model.sum(axis=1)) ** 2))
    for fac in (al, un):
        got = float(sparse.sparse_residual_sq(X, fac).item())
        assert abs(got - want) <= 1e-4 * want


class _Static:
    inner_method = 'cg_static'
    cg_maxiter = 10
    maxiter = 25


@pytest.mark.parametrize("dims,R,nnz", [((12, 10, 9), 3, 400), ((9, 8, 7, 6), 2, 600), ((30, 25, 20), 6, 6000)])
@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
def test_direct_coo_dgn_matches_dense_oracle(dims, R, nnz, dt):
    """dGN on the COO tensor itself (gradient and error from COO MTTKRPs, CG on
    the Gramians) against the oracle's dense dGN on sparse2dense of it, from the
    same start: the reference's objective, absent entries being zeros."""
    from tensorfox_gb300 import mttkrp_dgn
    data, idxs, _ = coo(dims, R, nnz, 4)
    T = dense_of(data, idxs, dims)
    rng = np.random.default_rng(5)
    init = [rng.standard_normal((d, R)) for d in dims]
    _, ss0, er0, _, gr0, st0 = orc.dGN(T, [w.copy() for w in init], R, orc.make_options(_Static))
    X = sparse.DeviceCOO(data, idxs, dims, dt)
    prec = 'fp64' if dt == torch.float64 else 'fp32'
    x0 = torch.from_numpy(orc.cpd2flat(init)).to("cuda", dt)
    best, ss1, er1, _, gr1, st1, mv = mttkrp_dgn.dgn_mttkrp(sparse.coo_provider(X, R), list(dims), R, x0,
                                                         tfx.make_options(_Static), prec, float(np.sum(T * T)),
                                                         float(np.mean(np.abs(T))))
    if dt == torch.float64:
        assert st1 == st0 and len(er1) == len(er0)
        np.testing.assert_allclose(er1, er0, rtol=1e-8)
        np.testing.assert_allclose(ss1, ss0, rtol=1e-6, atol=1e-12)
        np.testing.assert_allclose(gr1, gr0, rtol=1e-6)
    else:
        np.testing.assert_allclose(er1[:6], er0[:6], rtol=1e-4)
    assert mv > len(er1)


def test_direct_coo_cpd_equals_dense_uncompressed_oracle():
    """cpd(..., sparse_solver='direct') draws the reference's random start in the
    full space and runs dGN on the COO tensor: the same trajectory as the
    oracle's cpd of the dense tensor without compression (tol_mlsvd = -1)."""
    dims, R = (14, 12, 10), 3
    data, idxs, _ = coo(dims, R, 700, 6)
    T = dense_of(data, idxs, dims)

    class O(_Static):
        pass
    o = tfx.make_options(O)
    o.sparse_solver = 'direct'
    np.random.seed(3)
    f, out = tfx.cpd([data, idxs, np.array(dims)], R, o)
    after = np.random.rand()
    oo = orc.make_options(O)
    oo.tol_mlsvd = -1
    np.random.seed(3)
    f0, out0 = orc.cpd(T, R, oo)
    assert np.random.rand() == after                 # the RNG left where the reference leaves it
    np.testing.assert_allclose(out.errors[0], out0.errors[0], rtol=1e-8)
    # rel_error: the stored entries only, as the reference reports a sparse CPD
    model = np.ones((len(data), R))
    for l in range(3):
        model *= f[l][idxs[:, l]]
    want = np.linalg.norm(data - model.sum(1)) / np.linalg.norm(data)
    assert abs(out.rel_error - want) <= 1e-10 * want


@pytest.mark.parametrize("R", [8, 16, 32])
def test_coo_mttkrp_bf16_per_column_scaling_vs_fp64(R):
    """BF16 factor rows with per-column power-of-two scales (FP32 values and
    sums) against the FP64 oracle: about 3e-3 relative, within 1e-2 for every
    column even when the columns' magnitudes span twelve decades (the scales
    keep each column's own relative accuracy)."""
    import ctypes
    from tensorfox_gb300 import _lib, _dev
    dims, nnz = (40, 30, 20), 4000
    data, idxs, W = coo(dims, R, nnz, 9)
    colscale = 10.0 ** np.linspace(-6, 6, R)
    W = [w * colscale[None, :] if l == 1 else w for l, w in enumerate(W)]
    X = sparse.DeviceCOO(data, idxs, dims, torch.float32)
    flat = torch.from_numpy(orc.cpd2flat(W)).cuda().float()
    bf = torch.empty(flat.numel(), dtype=torch.bfloat16, device="cuda")
    sc = torch.empty(3 * R, dtype=torch.float32, device="cuda")
    cd = (ctypes.c_int * 3)(*dims)
    _lib.call("tfx_factors_bf16", 3, cd, R, ctypes.c_void_p(flat.data_ptr()), ctypes.c_void_p(bf.data_ptr()),
              ctypes.c_void_p(sc.data_ptr()), ctypes.c_void_p(_dev.stream()))
    offs = np.concatenate([[0], np.cumsum([R * d for d in dims])])
    ptrs = torch.tensor([bf.data_ptr() + int(offs[l]) * 2 for l in range(3)], dtype=torch.int64, device="cuda")
    T = dense_of(data, idxs, dims)
    Tl = [orc.unfold(T, l + 1) for l in range(3)]
    for l in range(3):
        rowptr, sidx, svals = X.sort_mode(l)
        out = torch.empty((dims[l], R), dtype=torch.float32, device="cuda")
        _lib.call("tfx_coo_mttkrp_bf16", ctypes.c_void_p(sidx.data_ptr()), ctypes.c_void_p(svals.data_ptr()), X.nnz,
                  ctypes.c_void_p(rowptr.data_ptr()), 3, cd, R, l, ctypes.c_void_p(ptrs.data_ptr()),
                  ctypes.c_void_p(sc.data_ptr()), ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(_dev.stream()))
        got = out.double().cpu().numpy()
        ref = orc.mttkrp(Tl, W, l)
        colerr = np.linalg.norm(got - ref, axis=0) / np.linalg.norm(ref, axis=0)
        assert colerr.max() <= 1e-2, colerr


def test_direct_coo_precision_ladder_vs_fp64_oracle():
    """precision='mixed' on the direct COO solver: BF16 gathers while the error
    falls by more than 1% an iteration, FP32 after; it ends at the FP64
    oracle's dGN error (same start, sparse2dense, FP64) within 1e-3."""
    from tensorfox_gb300 import mttkrp_dgn
    dims, R = (40, 35, 30), 8
    data, idxs, _ = coo(dims, R, 8000, 12)
    T = dense_of(data, idxs, dims)
    rng = np.random.default_rng(13)
    init = [rng.standard_normal((d, R)) for d in dims]

    class O:
        inner_method = 'cg_static'
        cg_maxiter = 10
        maxiter = 60
    _, _, er0, _, _, _ = orc.dGN(T, [w.copy() for w in init], R, orc.make_options(O))
    X = sparse.DeviceCOO(data, idxs, dims, torch.float32)
    x0 = torch.from_numpy(orc.cpd2flat(init)).cuda().float()
    _, _, er1, _, _, _, _ = mttkrp_dgn.dgn_mttkrp(sparse.coo_provider(X, R), list(dims), R, x0,
                                                  tfx.make_options(O), 'fp32', float(np.sum(T * T)),
                                                  float(np.mean(np.abs(T))), ladder=True)
    assert mttkrp_dgn.dgn_mttkrp.low_iterations >= 1
    assert abs(min(er1) - min(er0)) <= 1e-3 * min(er0)


@pytest.mark.parametrize("dims,R", [((5000, 3000, 70), 16), ((9, 8, 7, 6), 5), ((4100, 33, 2049), 64)])
@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
def test_step_update_wide_matches_one_cta_update(dims, R, dt):
    """The whole-grid step update against the one-CTA one (GaussNewton.py:284-297
    with Conversion.py:361-387 balancing): the same rounded x, the same scalars
    and the same balanced factors up to the order of the FP64 column sums."""
    import ctypes
    from tensorfox_gb300 import _dev, _lib
    rng = np.random.default_rng(11)
    n = R * sum(dims)
    x0 = torch.from_numpy(rng.standard_normal(n)).to("cuda", dt)
    y = torch.from_numpy(0.1 * rng.standard_normal(n)).cuda()
    g = torch.from_numpy(rng.standard_normal(n)).cuda()
    cd = (ctypes.c_int * len(dims))(*dims)
    lib_dt = _dev.lib_dtype("fp64" if dt == torch.float64 else "fp32")
    st = ctypes.c_void_p(_dev.stream())
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    xa, Wa, oa = x0.clone(), torch.empty_like(x0), torch.zeros(4, dtype=torch.float64, device="cuda")
    _lib.call("tfx_dgn_step_update", lib_dt, len(dims), cd, R, vp(xa), vp(Wa), vp(y), vp(g), ctypes.c_double(0.3),
              0, 0, ctypes.c_double(0.0), 0, -1, None, vp(oa), st)
    xb, Wb, ob = x0.clone(), torch.empty_like(x0), torch.zeros(4, dtype=torch.float64, device="cuda")
    nbytes = int(_lib.load().tfx_step_update_wide_scratch_bytes(len(dims), cd, R))
    scr = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    _lib.call("tfx_step_update_wide", lib_dt, len(dims), cd, R, vp(xb), vp(Wb), vp(y), vp(g), ctypes.c_double(0.3),
              vp(ob), vp(scr), nbytes, st)
    torch.cuda.synchronize()
    assert torch.equal(xa, xb)
    a, b = oa.cpu().numpy(), ob.cpu().numpy()
    np.testing.assert_allclose(b[[0, 1, 3]], a[[0, 1, 3]], rtol=1e-12)
    np.testing.assert_allclose(b[2], a[2], rtol=1e-9)      # a sum of terms of both signs
    ulp = 1e-13 if dt == torch.float64 else 2 ** -23
    np.testing.assert_allclose(Wb.double().cpu().numpy(), Wa.double().cpu().numpy(), rtol=2 * ulp, atol=0)
