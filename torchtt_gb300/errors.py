"""Exception types of the solver boundary, with the reference's names and meaning
(torchtt/errors.py:4-29), plus the error raised when the GPU library fails."""


class ShapeMismatch(Exception):
    """Shapes of the operands do not match."""


class RankMismatch(Exception):
    """Ranks of the given cores do not match."""


class IncompatibleTypes(Exception):
    """TT-matrix / TT-vector type mismatch."""


class InvalidArguments(Exception):
    """Invalid arguments."""


class GB300Error(RuntimeError):
    """The CUDA library reported a failure (CUDA error, numerical breakdown, out of memory)."""
