"""DMRG matvec on the GPU (dmrg_matvec / ttgb_dmrg_matvec) against the exact TT product and the
reference's C++ dmrg_mv outputs (tests/golden/dmrg.npz)."""
import numpy as np
import pytest
import torch

import _golden as G
from oracle import amen as O

pytestmark = pytest.mark.gpu


def _tt(cores, dev):
    from torchtt_gb300 import TT
    return TT([torch.from_numpy(np.ascontiguousarray(c)).to(dev) for c in cores])


@pytest.mark.parametrize("case", [0, 1])
def test_dmrg_matches_reference(cuda, case):
    from torchtt_gb300 import dmrg_matvec
    z = G.load("dmrg.npz")
    name = str(z["names"][case])
    A, x, yr = G.cores(z, name + "_A"), G.cores(z, name + "_x"), G.cores(z, name + "_y")
    y = dmrg_matvec(_tt(A, cuda), _tt(x, cuda), eps=1e-12)
    yc = [c.cpu().numpy() for c in y.cores]
    assert O.tt_relerr(yc, O.tt_matvec(A, x)) <= 1e-11
    assert O.tt_relerr(yc, yr) <= 1e-11
    assert all(abs(a - b) <= 4 for a, b in zip(y.R, [1] + [c.shape[2] for c in yr]))


def test_dmrg_large_compresses(cuda):
    """d=12, n=32 Laplacian-plus-potential times a rank-6 TT: DMRG gives A x to 1e-10, checked by
    the GPU TT norm of the difference; its ranks stay within the exact product's 18 plus the
    kickrank and adaptive enlargement the reference also keeps."""
    from torchtt_gb300 import TT, dmrg_matvec, workloads as W
    A = TT([c.to(cuda) for c in W.laplace_potential_ttm(12, 32)])
    x = TT([c.to(cuda) for c in W.random_tt([32] * 12, [1] + [6] * 11 + [1], 5)])
    y = dmrg_matvec(A, x, eps=1e-10)
    exact = A @ x
    assert float((y - exact).norm() / exact.norm()) <= 1e-9
    assert max(y.R) <= max(exact.R) + 4 + 4
