"""Loads the reference Tensor Fox package (v1.2.1) for fixture generation only.

The reference needs Numba, matplotlib, pandas and IPython at import time; none is
installed here, so this module registers minimal stand-ins:

* ``numba.njit`` / ``numba.prange`` become identity / ``range`` (the reference's
  ``@njit`` kernels then run as plain Python with identical arithmetic);
* plotting and display modules become empty namespaces.

The pandas stand-in is removed from ``sys.modules`` again once the reference is
imported (scikit-learn, which the tensor-train path calls, probes for pandas).
It also removes the one-second ``time.sleep`` in ``Auxiliar.consistency``
(Auxiliar.py:76) and replaces ``Compression.sparse_dot_mkl_call``
(Compression.py:240-258) by the SciPy product ``(Tl @ Tl.T).toarray()``, which is
the dense matrix MKL's ``dot_product_mkl(..., dense=True)`` returns.

Only ``tests/golden/make_golden.py`` imports this file, and only in a container
where the reference source tree is mounted.  Nothing shipped or run on a GPU
machine reads the reference.
"""
import os
import sys
import types

def _ref_modules():
    """The reference's ``modules`` directory, named by TFX_REFERENCE_MODULES."""
    path = os.environ.get("TFX_REFERENCE_MODULES")
    if not path or not os.path.isdir(os.path.join(path, "TensorFox")):
        raise RuntimeError("set TFX_REFERENCE_MODULES to the reference source tree's 'modules' directory "
                           "(the one holding the TensorFox package) to regenerate the fixtures")
    return path


def _stub_modules():
    if "numba" not in sys.modules:
        numba = types.ModuleType("numba")

        def njit(*args, **kwargs):
            if len(args) == 1 and callable(args[0]) and not kwargs:
                return args[0]
            return lambda f: f

        numba.njit = njit
        numba.jit = njit
        numba.prange = range
        errors = types.ModuleType("numba.errors")
        for name in ("NumbaDeprecationWarning", "NumbaPendingDeprecationWarning",
                     "NumbaPerformanceWarning"):
            setattr(errors, name, type(name, (Warning,), {}))
        numba.errors = errors
        sys.modules["numba"] = numba
        sys.modules["numba.errors"] = errors
    for name in ("matplotlib", "matplotlib.pyplot", "IPython", "IPython.display", "pandas"):
        if name not in sys.modules:
            sys.modules[name] = types.ModuleType(name)
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    sys.modules["IPython"].display = sys.modules["IPython.display"]


_TFX = None


def load_reference():
    """Import and patch the reference package; returns the ``TensorFox`` module."""
    global _TFX
    if _TFX is not None:
        return _TFX
    ref_modules = _ref_modules()
    _stub_modules()
    if ref_modules not in sys.path:
        sys.path.insert(0, ref_modules)
    import io
    import contextlib
    with contextlib.redirect_stderr(io.StringIO()):
        import TensorFox as tfx  # noqa: E402
    import TensorFox.Auxiliar as aux
    import TensorFox.Compression as cmpr

    aux.time = types.SimpleNamespace(sleep=lambda s: None, time=__import__("time").time)

    def _dense_gram(Tl, display):
        return (Tl @ Tl.T).toarray()

    cmpr.sparse_dot_mkl_call = _dense_gram
    # the stand-ins for plotting and tables are only needed while the reference
    # imports; scikit-learn (the reference's randomized SVD of the tensor-train
    # path) probes sys.modules for a real pandas, so drop the stand-in again
    for name in ("pandas",):
        sys.modules.pop(name, None)
    _TFX = tfx
    return tfx
