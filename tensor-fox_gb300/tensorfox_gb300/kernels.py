"""Thin wrappers over the C ABI entry points, taking CUDA torch tensors.

Every function launches on the current torch stream and raises ``TfxError`` when
the library reports a failure.  Shapes and strides follow the C ABI header.
"""
import ctypes

import numpy as np
import torch

from . import _dev, _lib


def _dt(t):
    if t.dtype == torch.float64:
        return _lib.F64
    if t.dtype == torch.float32:
        return _lib.F32
    raise TypeError("tensors must be float32 or float64, got %s" % t.dtype)


def _vp(t):
    return ctypes.c_void_p(_dev.ptr(t))


def _st():
    return ctypes.c_void_p(_dev.stream())


def mode_gram(S, shape, l):
    """``S_(l) S_(l)^T`` (D x D) of a C-order tensor with the given shape."""
    P = int(np.prod(shape[:l], dtype=np.int64))
    D = int(shape[l])
    Q = int(np.prod(shape[l + 1:], dtype=np.int64))
    lib = _lib.load()
    nb = lib.tfx_mode_gram_scratch_bytes(_dt(S), P, D, Q)
    scratch = torch.empty(int(nb), dtype=torch.uint8, device=S.device)
    G = torch.empty((D, D), dtype=S.dtype, device=S.device)
    _lib.call("tfx_mode_gram", _dt(S), _vp(S), P, D, Q, _vp(G), _vp(scratch), nb, _st())
    return G


def tc_gram_supported(S, shape, l):
    """The tensor-core Gram needs FP32, Q = prod(shape[l+1:]) >= 32 with Q % 4 == 0."""
    Q = int(np.prod(shape[l + 1:], dtype=np.int64))
    return S.dtype == torch.float32 and Q >= 32 and Q % 4 == 0 and S.data_ptr() % 16 == 0


def mode_gram_tc(S, shape, l, check=True):
    """``S_(l) S_(l)^T`` on the tensor cores (tcgen05 kind::tf32, FP32 accumulation).

    ``check=False`` returns ``(G, err)`` without reading the kernel's error flag
    (a read waits for the device); the caller checks ``err`` at its next sync."""
    P = int(np.prod(shape[:l], dtype=np.int64))
    D = int(shape[l])
    Q = int(np.prod(shape[l + 1:], dtype=np.int64))
    lib = _lib.load()
    nb = int(lib.tfx_mode_gram_tc_scratch_bytes(P, D, Q))
    scratch = torch.empty(nb, dtype=torch.uint8, device=S.device)
    err = torch.zeros(1, dtype=torch.int32, device=S.device)
    G = torch.empty((D, D), dtype=torch.float32, device=S.device)
    _lib.call("tfx_mode_gram_tc", _vp(S), P, D, Q, _vp(G), _vp(scratch), nb, _vp(err), _st())
    if not check:
        return G, err
    check_gram_flag(err)
    return G


def check_gram_flag(err):
    """Raises when the tensor-core Gram's bounded wait ran out (``err`` != 0)."""
    e = int(err.item())
    if e != 0:
        raise _lib.TfxError("tensor-core Gram: bounded wait expired (code %d)" % e)


def gemm(A, B, C, M, N, K, batch, strides, alpha=1.0, beta=0.0):
    arr = (ctypes.c_longlong * 9)(*[int(s) for s in strides])
    _lib.call("tfx_gemm", _dt(A), _vp(A), _vp(B), _vp(C), int(M), int(N), int(K), int(batch), arr,
              float(alpha), float(beta), _st())
    return C


def matmul(A, B, transA=False, transB=False):
    """C = op(A) op(B) for 2-D row-major tensors (device GEMM)."""
    M = A.shape[1] if transA else A.shape[0]
    K = A.shape[0] if transA else A.shape[1]
    N = B.shape[0] if transB else B.shape[1]
    C = torch.empty((M, N), dtype=A.dtype, device=A.device)
    if (not transA and not transB and A.dtype == torch.float32 and K % 4 == 0 and N % 4 == 0 and N >= 16384):
        # a short left factor times a wide right one (enough column tiles to fill
        # the GPU): the register-tiled mode-product kernel
        A = A.contiguous()
        B = B.contiguous()
        _lib.call("tfx_ttm", _dt(B), _vp(B), 1, int(K), int(N), _vp(A), int(M), _vp(C), _st())
        return C
    sAm, sAk = (1, A.shape[1]) if transA else (A.shape[1], 1)
    sBk, sBn = (1, B.shape[1]) if transB else (B.shape[1], 1)
    A = A.contiguous()
    B = B.contiguous()
    return gemm(A, B, C, M, N, K, 1, [0, sAm, sAk, 0, sBk, sBn, 0, N, 1])


def ttm(S, shape, l, Ut, tensor_cores=False):
    """Mode-l product with U^T: out[p, j, q] = sum_i U[i, j] S[p, i, q].

    ``Ut`` is (n, D) row-major, i.e. U (D x n) column-major.  With
    ``tensor_cores`` (precision 'mixed') an FP32 product whose shape the
    tcgen05 kernel takes runs there (3xTF32, FP32 accumulation); its
    bounded-wait flag is checked with the next read of the device
    (``check_ttm_flag``)."""
    P = int(np.prod(shape[:l], dtype=np.int64))
    D = int(shape[l])
    Q = int(np.prod(shape[l + 1:], dtype=np.int64))
    n = int(Ut.shape[0])
    out = torch.empty(P * n * Q, dtype=S.dtype, device=S.device)
    Uc = Ut.contiguous()
    if (tensor_cores and S.dtype == torch.float32 and Uc.dtype == torch.float32 and S.data_ptr() % 16 == 0 and
            Uc.data_ptr() % 16 == 0 and _lib.load().tfx_ttm_tc_supported(P, D, Q, n)):
        err = torch.zeros(1, dtype=torch.int32, device=S.device)
        _lib.call("tfx_ttm_tc", _vp(S), P, D, Q, _vp(Uc), n, _vp(out), _vp(err), _st())
        _TTM_FLAGS.append(err)
    else:
        _lib.call("tfx_ttm", _dt(S), _vp(S), P, D, Q, _vp(Uc), n, _vp(out), _st())
    new_shape = list(shape)
    new_shape[l] = n
    return out.view(*new_shape), new_shape


_TTM_FLAGS = []


def check_ttm_flag():
    """Raises if a tensor-core mode product issued since the last check ran out
    of a bounded wait (one device read for all of them)."""
    flags = list(_TTM_FLAGS)
    _TTM_FLAGS.clear()
    if flags and int(torch.cat(flags).max().item()) != 0:
        raise _lib.TfxError("tensor-core mode product: a bounded wait ran out")


def orthonormalize(Y):
    """CGS2 on the columns of Y given as a (k, D) row-major tensor (= D x k column-major)."""
    k, D = Y.shape
    _lib.call("tfx_orthonormalize", _dt(Y), _vp(Y), int(D), int(k), _st())
    return Y


def sym_eig(A, max_sweeps=40, return_sweeps=False):
    """Eigenvalues (descending) and eigenvectors (rows of the returned (n, n) tensor).

    With ``return_sweeps`` the number of Jacobi sweeps taken is returned too."""
    n = A.shape[0]
    ev = torch.empty(n, dtype=A.dtype, device=A.device)
    V = torch.empty((n, n), dtype=A.dtype, device=A.device)
    sw = torch.zeros(1, dtype=torch.int32, device=A.device) if return_sweeps else None
    _lib.call("tfx_sym_eig", _dt(A), _vp(A.contiguous()), int(n), _vp(ev), _vp(V), int(max_sweeps),
              _vp(sw) if sw is not None else None, _st())
    if return_sweeps:
        return ev, V, int(sw.cpu()[0])
    return ev, V


def flip_signs(Ut):
    """Ut is (n, D) row-major = U (D x n) column-major."""
    n, D = Ut.shape
    _lib.call("tfx_flip_signs", _dt(Ut), _vp(Ut), int(D), int(n), _st())
    return Ut


def cp_residual_sq(T, dims, W_flat, R):
    """||T - [[W]]||^2 on the device (float64 scalar tensor)."""
    lib = _lib.load()
    scratch = torch.empty(int(lib.tfx_cp_residual_scratch_bytes()), dtype=torch.uint8, device=T.device)
    out = torch.empty(1, dtype=torch.float64, device=T.device)
    L = len(dims)
    cd = (ctypes.c_int * L)(*[int(d) for d in dims])
    _lib.call("tfx_cp_residual", _dt(T), _vp(T), L, cd, int(R), _vp(W_flat), _vp(out), _vp(scratch), _st())
    return out


def tensor_norms(T):
    """(sum t^2, sum |t|) as a float64 tensor of 2 entries."""
    lib = _lib.load()
    scratch = torch.empty(int(lib.tfx_cp_residual_scratch_bytes()), dtype=torch.uint8, device=T.device)
    out = torch.empty(2, dtype=torch.float64, device=T.device)
    _lib.call("tfx_tensor_norms", _dt(T), _vp(T), int(T.numel()), _vp(out), _vp(scratch), _st())
    return out


def mttkrp_tc_supported(T, dims, R, mode):
    """The tensor-core MTTKRP applies: FP32, order >= 3, R <= 64, the later dims'
    product (of the tensor the kernel reads) a multiple of 4, 16-byte aligned."""
    L = len(dims)
    if T.dtype != torch.float32 or L < 3 or R > 64 or T.data_ptr() % 16 != 0:
        return False
    if mode < L - 1:
        return int(np.prod(dims[mode + 1:], dtype=np.int64)) % 4 == 0
    return int(np.prod(dims[:L - 1], dtype=np.int64)) % 4 == 0


def last_mode_first(T, dims):
    """A copy of the tensor with its last mode moved first (the tensor-core
    MTTKRP's operand for the last mode)."""
    L = len(dims)
    return T.reshape(dims).permute(L - 1, *range(L - 1)).contiguous()


def mttkrp_tc(T, dims, W_flat, R, mode, col_major=False, T_last=None, out=None):
    """``T_(mode) KR`` on the tensor cores (tcgen05, 3xTF32, FP32 accumulation).

    ``W_flat``: the factors in the flat layout (column-major blocks).  The last
    mode reads ``T_last`` (``last_mode_first(T, dims)``, made here if absent).
    Returns (d_mode x R) row-major, or column-major with ``col_major``."""
    L = len(dims)
    dims = [int(d) for d in dims]
    offs = np.concatenate([[0], np.cumsum([R * d for d in dims])])
    base = W_flat.data_ptr()
    if mode < L - 1:
        Tk, dk, mk = T, dims, mode
        ptrs = [base + int(offs[m]) * 4 for m in range(L)]
    else:
        Tk = T_last if T_last is not None else last_mode_first(T, dims)
        dk = [dims[L - 1]] + dims[:L - 1]
        mk = 0
        ptrs = [base + int(offs[L - 1]) * 4] + [base + int(offs[m]) * 4 for m in range(L - 1)]
    lib = _lib.load()
    cd = (ctypes.c_int * L)(*dk)
    nb = int(lib.tfx_mttkrp_tc_scratch_bytes(L, cd, int(R), int(mk)))
    scratch = torch.empty(nb, dtype=torch.uint8, device=T.device)
    err = torch.zeros(1, dtype=torch.int32, device=T.device)
    if out is None:
        out = torch.empty((dims[mode], R) if not col_major else (R, dims[mode]), dtype=torch.float32, device=T.device)
    pw = (ctypes.c_void_p * L)(*ptrs)
    _lib.call("tfx_mttkrp_tc", _vp(Tk), L, cd, int(R), ctypes.cast(pw, ctypes.c_void_p), int(mk), _vp(out), 1 if col_major else 0, _vp(scratch), nb,
              _vp(err), _st())
    return out, err
