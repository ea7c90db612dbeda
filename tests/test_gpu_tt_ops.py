"""TT norm and TT rounding on the GPU (ttgb_tt_norm / ttgb_tt_round) against the oracle and the
reference's own rounding outputs (tests/golden/round.npz)."""
import numpy as np
import pytest
import torch

import _golden as G
from oracle import amen as O

pytestmark = pytest.mark.gpu


def _tt(cores, dev):
    from torchtt_gb300 import TT
    return TT([torch.from_numpy(np.ascontiguousarray(c)).to(dev) for c in cores])


def _np(x):
    return [c.detach().cpu().numpy() for c in x.cores]


def _flat(cores):
    return [c.reshape(c.shape[0], -1, c.shape[-1]) for c in cores]


@pytest.mark.parametrize("shape", [([7], [1, 1]), ([4, 5, 6], [1, 3, 2, 1]),
                                   ([8] * 10, [1] + [12] * 9 + [1]), ([64] * 6, [1] + [40] * 5 + [1])])
def test_norm_matches_oracle(cuda, shape):
    from torchtt_gb300 import workloads as W
    N, R = shape
    x = W.random_tt(N, R, 3, normalise=False)
    got = float(_tt([c.numpy() for c in x], cuda).norm())
    ref = O.tt_norm([c.numpy() for c in x])
    assert abs(got - ref) <= 1e-12 * ref


def test_norm_of_ttm_and_residual(cuda):
    """A TT-matrix norm, and the norm of a residual with heavy cancellation (||r|| ~ 1e-9 ||b||):
    the QR sweep keeps it accurate where a Gram-matrix sweep would lose every digit."""
    from torchtt_gb300 import workloads as W
    A = [c.numpy() for c in W.laplace_ttm(5, 7)]
    assert abs(float(_tt(A, cuda).norm()) - O.tt_norm(A)) <= 1e-12 * O.tt_norm(A)
    x = [c.numpy() for c in W.random_tt([9] * 6, [1] + [5] * 5 + [1], 4)]
    dx = [c.numpy() for c in W.random_tt([9] * 6, [1] + [3] * 5 + [1], 5)]
    y = O.tt_add(x, dx, 1.0, 1e-9)
    r = O.tt_add(y, x, 1.0, -1.0)              # = 1e-9 dx, formed with cancellation
    got = float(_tt(r, cuda).norm())
    ref = 1e-9 * O.tt_norm(dx)
    assert abs(got - ref) <= 1e-6 * ref, (got, ref)


def test_round_matches_reference(cuda):
    z = G.load("round.npz")
    for name in z["names"]:
        name = str(name)
        xin, xref = G.cores(z, name + "_in"), G.cores(z, name + "_out")
        eps, rmax = float(z[name + "_eps"]), int(z[name + "_rmax"])
        y = _tt(xin, cuda).round(eps, rmax)
        yc = _np(y)
        assert [c.shape for c in yc] == [c.shape for c in xref], name
        diff = O.tt_norm(O.tt_add(_flat(yc), _flat(xref), 1.0, -1.0))
        assert diff <= 1e-11 * O.tt_norm(xref), (name, diff)


def test_round_rank_stress(cuda):
    """Rounding of a sum of 4 random rank-16 TTs (d=16, n=32, input rank 64) at eps 1e-8:
    the ranks match the oracle's and the rounding error stays below eps."""
    from torchtt_gb300 import workloads as W
    N = [32] * 16
    parts = [[c.numpy() for c in W.random_tt(N, [1] + [16] * 15 + [1], 60 + i)] for i in range(4)]
    x = parts[0]
    for p in parts[1:]:
        x = O.tt_add(x, p)
    y = _np(_tt(x, cuda).round(1e-8))
    yo = O.tt_round(x, 1e-8)
    assert [c.shape for c in y] == [c.shape for c in yo]
    nx = O.tt_norm(x)
    assert O.tt_norm(O.tt_add(y, x, 1.0, -1.0)) <= 1e-8 * nx
    assert O.tt_norm(O.tt_add(y, yo, 1.0, -1.0)) <= 1e-10 * nx


def test_round_truncates_and_caps(cuda):
    from torchtt_gb300 import workloads as W
    b = [c.numpy() for c in W.random_tt([10] * 6, [1] + [4] * 5 + [1], 8)]
    x = O.tt_add(b, b)                              # rank 8 representation of a rank-4 tensor
    y = _tt(x, cuda).round(1e-12)
    assert max(y.R) == 4
    y2 = _tt(x, cuda).round(1e-12, 2)
    assert max(y2.R) == 2
    assert y.cores[0].device.type == "cuda"


@pytest.mark.parametrize("case", [(3, [4, 5, 6], [1, 2, 3, 1], [1, 3, 2, 1]),
                                  (6, [7] * 6, [1] + [3] * 5 + [1], [1] + [5] * 5 + [1])])
def test_matvec_matches_oracle(cuda, case):
    from torchtt_gb300 import workloads as W
    d, N, RA, RX = case
    g = np.random.Generator(np.random.PCG64(d))
    A = [g.standard_normal((RA[k], N[k], N[k], RA[k + 1])) for k in range(d)]
    x = [g.standard_normal((RX[k], N[k], RX[k + 1])) for k in range(d)]
    y = _tt(A, cuda) @ _tt(x, cuda)
    yo = O.tt_matvec(A, x)
    assert y.R == [c.shape[0] for c in yo] + [1]
    for a, b in zip(_np(y), yo):
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12 * np.abs(b).max())


def test_residual_of_reference_solution(cuda):
    """||A x_ref - b|| / ||b|| of the reference's own solution, all on the GPU, equals the
    oracle's value (the check the reference's tests apply, tests/test_solvers.py:19)."""
    z = G.load("solve_laplace_d8_n16.npz")
    A, b, x = G.cores(z, "A"), G.cores(z, "b"), G.cores(z, "x_cpp")
    At, bt, xt = _tt(A, cuda), _tt(b, cuda), _tt(x, cuda)
    got = float((At @ xt - bt).norm() / bt.norm())
    ref = O.tt_relres(A, x, b)
    assert abs(got - ref) <= 1e-3 * ref, (got, ref)
