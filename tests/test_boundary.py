"""Argument handling of amen_solve follows torchtt/solvers.py:259-282 (CPU-only checks)."""
import pytest
import torch

from torchtt_gb300 import TT, amen_solve, workloads as W
from torchtt_gb300.errors import IncompatibleTypes, InvalidArguments, RankMismatch, ShapeMismatch


def small():
    wl = W.small_random_system(0)
    return TT(wl["A"]), TT(wl["b"])


def test_tt_constructor_checks():
    A, b = small()
    assert A.is_ttm and not b.is_ttm
    assert A.N == [4, 5, 6] and A.M == [4, 5, 6] and A.R == [1, 2, 3, 1]
    with pytest.raises(RankMismatch):
        TT([torch.zeros(1, 3, 2), torch.zeros(3, 3, 1)])
    with pytest.raises(InvalidArguments):
        TT([torch.zeros(1, 3, 2, 2, 1)])
    with pytest.raises(InvalidArguments):
        TT([torch.zeros(2, 3, 1)])


def test_argument_errors():
    A, b = small()
    with pytest.raises(InvalidArguments):
        amen_solve([1], b)
    with pytest.raises(IncompatibleTypes):
        amen_solve(b, b)
    with pytest.raises(IncompatibleTypes):
        amen_solve(A, A)
    wrong = TT(W.laplace_ttm(3, 4))
    with pytest.raises(ShapeMismatch):
        amen_solve(wrong, b)
    rect = TT([torch.zeros(1, 4, 5, 1), torch.zeros(1, 5, 5, 1), torch.zeros(1, 6, 6, 1)])
    with pytest.raises(ShapeMismatch):
        amen_solve(rect, b)
    with pytest.raises(InvalidArguments):
        amen_solve(A, b, preconditioner="x")


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU behaviour")
def test_no_cpu_fallback():
    A, b = small()
    with pytest.raises(RuntimeError):
        amen_solve(A, b)


def test_tt_sub_on_cpu():
    """x - b concatenates cores; the difference of b with itself has norm 0 (oracle check)."""
    from oracle import amen as O
    wl = W.small_random_system(0)
    b = TT(wl["b"])
    res = [c.numpy() for c in (b - b).cores]
    assert O.tt_norm(res) < 1e-14 * O.tt_norm([c.numpy() for c in b.cores])


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU behaviour")
def test_tt_algebra_needs_gpu():
    wl = W.small_random_system(0)
    A, x, b = TT(wl["A"]), TT(wl["x"]), TT(wl["b"])
    with pytest.raises(RuntimeError):
        b.norm()
    with pytest.raises(RuntimeError):
        A @ x
    with pytest.raises(RuntimeError):
        b.round(1e-8)


def test_torch_operator_schema_and_no_cpu_fallback():
    """torch.ops.torchtt_gb300.amen_solve is registered with the documented schema and refuses
    CPU tensors (no CPU fallback)."""
    import torchtt_gb300  # noqa: F401
    from torchtt_gb300 import custom_op
    op = torch.ops.torchtt_gb300.amen_solve
    assert str(op.default._schema) == "torchtt_gb300::" + custom_op.SCHEMA
    A, b = small()
    with pytest.raises(RuntimeError, match="CUDA tensors only"):
        op(A.cores, b.cores, None)


def test_minimal_foreign_tt_argument_checks():
    """A TT class with only .cores and .is_ttm passes the argument checks (mode sizes are read from
    the cores) and is rejected with the reference's exceptions when the shapes disagree."""
    class Bare:
        def __init__(self, cores):
            self.cores = cores
            self.is_ttm = cores[0].dim() == 4
    A, b = small()
    from torchtt_gb300 import solvers as S
    assert S._rows(Bare(A.cores)) == [4, 5, 6] and S._cols(Bare(b.cores)) == [4, 5, 6]
    wrong = Bare(W.laplace_ttm(3, 4))
    with pytest.raises(ShapeMismatch):
        amen_solve(wrong, Bare(b.cores))
