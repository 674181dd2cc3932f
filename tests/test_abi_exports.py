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
