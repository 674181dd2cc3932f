"""The C-ABI library builds, loads and exports every symbol declared in include/*.h (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*?[\s\*]+(tfx_[A-Za-z0-9_]+)\s*\(", src, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "tfx_dgn_solve" in names and "tfx_coo_mttkrp" in names and "tfx_mode_gram" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    from tensorfox_gb300 import _build
    path = _build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_package_fails_loudly_without_a_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numpy as np
    import tensorfox_gb300 as tfx
    with pytest.raises(RuntimeError, match="CUDA device"):
        tfx.cpd(np.ones((3, 3, 3)), 2)


def test_host_gather_copies_every_buffer():
    """tfx_host_gather is host memory work (no device call): many buffers into
    one, split over threads, at the given offsets."""
    import ctypes
    import numpy as np
    from tensorfox_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(0)
    arrs = [rng.standard_normal(int(n)).astype(np.float32) for n in rng.integers(1, 5000, size=300)]
    arrs += [rng.standard_normal(3_000_000).astype(np.float32)]          # > 8 MB in total: threaded
    sizes = np.array([a.nbytes for a in arrs], dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum((sizes + 255) // 256 * 256)[:-1]]).astype(np.int64)
    dst = np.zeros(int(offs[-1] + sizes[-1]), dtype=np.uint8)
    src = np.array([a.ctypes.data for a in arrs], dtype=np.uint64)
    lib.tfx_host_gather.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    assert lib.tfx_host_gather(src.ctypes.data, sizes.ctypes.data, offs.ctypes.data, len(arrs), dst.ctypes.data, 8) == 0
    for a, o in zip(arrs, offs):
        np.testing.assert_array_equal(dst[o:o + a.nbytes].view(np.float32), a)
