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
