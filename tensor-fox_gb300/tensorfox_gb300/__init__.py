"""Tensor Fox's damped Gauss-Newton CPD path, rebuilt on GB300 (sm_103a) CUDA kernels.

Drop-in functions (same names, arguments and return values as Tensor Fox 1.2.1):
``cpd``, ``mlsvd``, ``dGN``, ``als``, ``rank``, ``stats``, ``make_options``, ``cpd2tens``, ``cpd2unfold1``,
``unfold``, ``foldback``, ``dense2sparse``, ``sparse2dense``, ``multilin_mult``, ``multilin_mult_cpd``,
``sparse_multilin_mult``.  All computation runs in ``libtfx_gb300.so`` on the GPU.
"""
__version__ = "1.2.1+gb300"

from .options import make_options, Options  # noqa: F401
from .gauss_newton import dGN  # noqa: F401
from .als import als  # noqa: F401,E402
from .api import cpd, tricpd, consistency, Output  # noqa: F401,E402
from .compression import mlsvd, clean_compression  # noqa: F401,E402
from .batch import cpd_batch  # noqa: F401,E402
from .sweeps import rank, stats  # noqa: F401,E402
from .distributed import cpd_batch_distributed  # noqa: F401,E402
from .sparse import DeviceCOO, coo_mttkrp, sparse_residual_sq  # noqa: F401,E402
from .autograd import cp_reconstruct, cp_fit_loss, mttkrp  # noqa: F401,E402
from .conversion import (cpd2tens, cpd2unfold1, unfold, foldback, dense2sparse, sparse2dense,  # noqa: F401,E402
                         multilin_mult, multilin_mult_cpd, sparse_multilin_mult)
