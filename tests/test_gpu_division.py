"""Elementwise TT division on the GPU (amen_divide, TT.__truediv__) against the reference's
amen_divide outputs (tests/golden/divide.npz)."""
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
def test_amen_divide_matches_reference(cuda, case):
    from torchtt_gb300 import TT, amen_divide
    from torchtt_gb300.division import diag_ttm
    z = G.load("divide.npz")
    name = str(z["names"][case])
    a, b, xr = G.cores(z, name + "_a"), G.cores(z, name + "_b"), G.cores(z, name + "_x")
    at, bt = _tt(a, cuda), _tt(b, cuda)
    x = TT(amen_divide(at, bt, eps=1e-10))
    D = TT(diag_ttm(at.cores))
    assert float((D @ x - bt).norm() / bt.norm()) <= 1e-9
    xc = [c.cpu().numpy() for c in x.cores]
    assert O.tt_relerr(xc, xr) <= 1e-8


def test_truediv_operators(cuda):
    from torchtt_gb300 import TT
    z = G.load("divide.npz")
    a, b = G.cores(z, "d3_a"), G.cores(z, "d3_b")
    at, bt = _tt(a, cuda), _tt(b, cuda)
    full = lambda t: O.tt_full([c.cpu().numpy() for c in t.cores])
    q = bt / at
    np.testing.assert_allclose(full(q), full(bt) / full(at), rtol=1e-9, atol=1e-11 * np.abs(full(q)).max())
    inv = 2.0 / at
    np.testing.assert_allclose(full(inv), 2.0 / full(at), rtol=1e-9)
    half = bt / 2.0
    np.testing.assert_allclose(full(half), full(bt) / 2.0, rtol=1e-14)
