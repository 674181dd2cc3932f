"""Device plumbing: CUDA availability, streams and host<->device transfers (PyTorch)."""
import numpy as np
import torch

from . import _lib


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("tensorfox_gb300 needs a CUDA device (GB300, sm_103a); none is visible")
    _lib.load()


def device():
    return torch.device("cuda", torch.cuda.current_device())


def stream():
    return ctypes_stream(torch.cuda.current_stream())


def ctypes_stream(s):
    return int(s.cuda_stream)


def ptr(t):
    return None if t is None else int(t.data_ptr())


def torch_dtype(precision):
    return torch.float64 if precision == "fp64" else torch.float32


def lib_dtype(precision):
    return _lib.F64 if precision == "fp64" else _lib.F32


def to_device(a, dtype):
    """numpy / torch (any device) -> contiguous CUDA tensor of ``dtype``."""
    if isinstance(a, torch.Tensor):
        return a.to(device=device(), dtype=dtype).contiguous()
    arr = np.ascontiguousarray(a)
    t = torch.from_numpy(arr)
    if arr.dtype != np.float64 and arr.dtype != np.float32:
        t = t.to(torch.float64)
    return t.to(device=device(), dtype=dtype, non_blocking=False).contiguous()


def h2d(arr, dtype, dev=None):
    """NumPy array -> CUDA tensor of ``dtype`` without blocking the host: the
    values are converted on the host, staged in pinned memory and copied
    asynchronously on the current stream (a pageable copy would wait for all
    queued device work first)."""
    np_dt = np.float64 if dtype == torch.float64 else (np.float32 if dtype == torch.float32 else None)
    a = np.ascontiguousarray(arr, dtype=np_dt) if np_dt is not None else np.ascontiguousarray(arr)
    t = torch.from_numpy(a).pin_memory()
    return t.to(device=dev if dev is not None else device(), non_blocking=True)


def flat_factors(factors):
    """concat_l vec_F(W_l) as float64 numpy (GaussNewton.py:125)."""
    return np.concatenate([np.asarray(W, dtype=np.float64).flatten("F") for W in factors])


def unflat(x, dims, R):
    out, s = [], 0
    for d in dims:
        out.append(np.asarray(x[s:s + d * R], dtype=np.float64).reshape(R, d).T.copy())
        s += d * R
    return out
