"""AMEn matvec / matmat on the GPU (amen_mv, amen_mm) against the exact TT products and the
reference's torchtt.amen_mv / amen_mm outputs (tests/golden/amen_mv.npz)."""
import numpy as np
import pytest
import torch

import _golden as G
from oracle import amen as O

pytestmark = pytest.mark.gpu


def _tt(cores, dev):
    from torchtt_gb300 import TT
    return TT([torch.from_numpy(np.ascontiguousarray(c)).to(dev) for c in cores])


def _ttm_product(A, B):
    out = []
    for a, b in zip(A, B):
        c = np.einsum('amkA,bknB->abmnAB', a, b)
        out.append(c.reshape(a.shape[0] * b.shape[0], a.shape[1], b.shape[2], a.shape[3] * b.shape[3]))
    return out


def _flat(cores):
    return [c.reshape(c.shape[0], -1, c.shape[-1]) for c in cores]


def test_amen_mv_matches_reference(cuda):
    from torchtt_gb300 import amen_mv
    z = G.load("amen_mv.npz")
    A, b, yr = G.cores(z, "mv_A"), G.cores(z, "mv_b"), G.cores(z, "mv_y")
    y = amen_mv(_tt(A, cuda), _tt(b, cuda), eps=1e-10)
    yc = [c.cpu().numpy() for c in y.cores]
    assert O.tt_relerr(yc, O.tt_matvec(A, b)) <= 1e-11
    assert O.tt_relerr(yc, yr) <= 1e-11
    assert all(abs(a - c) <= 4 for a, c in zip(y.R, [1] + [c.shape[2] for c in yr]))


def test_amen_mm_matches_reference(cuda):
    from torchtt_gb300 import amen_mm
    z = G.load("amen_mv.npz")
    A, B, Yr = G.cores(z, "mm_A"), G.cores(z, "mm_B"), G.cores(z, "mm_Y")
    Y = amen_mm(_tt(A, cuda), _tt(B, cuda), eps=1e-10)
    Yc = [c.cpu().numpy() for c in Y.cores]
    assert Y.is_ttm and [c.shape[1:3] for c in Yc] == [c.shape[1:3] for c in Yr]
    exact = _flat(_ttm_product(A, B))
    assert O.tt_relerr(_flat(Yc), exact) <= 1e-11
    assert O.tt_relerr(_flat(Yc), _flat(Yr)) <= 1e-11


def test_amen_mv_low_rank_output(cuda):
    """A product whose exact TT has rank 3 x 6 = 18 but whose value is close to rank 6: the AMEn
    matvec reaches eps with ranks below the exact representation's."""
    from torchtt_gb300 import TT, amen_mv, workloads as W
    A = TT([c.to(cuda) for c in W.laplace_potential_ttm(10, 16)])
    x = TT([c.to(cuda) for c in W.random_tt([16] * 10, [1] + [6] * 9 + [1], 9)])
    y = amen_mv(A, x, eps=1e-8)
    exact = A @ x
    assert float((y - exact).norm() / exact.norm()) <= 1e-7
