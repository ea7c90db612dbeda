"""torchtt_gb300: AMEn linear solves in the tensor-train format on one NVIDIA GB300.

A drop-in for the reference's ``torchtt.solvers.amen_solve`` (ion-g-ion/torchTT,
``torchtt/solvers.py:211``) whose arithmetic runs in hand-written sm_103a CUDA kernels
(``libttgb300.so``, C ABI in ``include/ttgb300.h``).
"""
from . import errors
from .errors import GB300Error, IncompatibleTypes, InvalidArguments, RankMismatch, ShapeMismatch
from .tt import TT
from . import solvers
from .solvers import amen_solve
from .division import amen_divide
from .dmrg import dmrg_matvec
from .amen_mv import amen_mm, amen_mv
from . import custom_op  # registers torch.ops.torchtt_gb300.amen_solve

__all__ = ["TT", "amen_solve", "amen_divide", "dmrg_matvec", "amen_mv", "amen_mm", "solvers", "errors", "GB300Error", "IncompatibleTypes",
           "InvalidArguments", "RankMismatch", "ShapeMismatch"]
__version__ = "0.1.0"
