"""Host-side TT algebra of the boundary type (no GPU): the core concatenations of +, - and scalar
products, the dense form, and the diagonal TT-matrix built for elementwise division, each against
the dense tensors (TT.__add__/__sub__/__mul__, torchtt/_tt_base.py; diag, used by amen_divide,
torchtt/_division.py:76-398)."""
import numpy as np
import torch

from torchtt_gb300 import TT, workloads as W
from torchtt_gb300.division import diag_ttm


def dense(t):
    return t.full().numpy()


def test_add_sub_scale_against_dense():
    a = TT(W.random_tt([3, 4, 5, 2], [1, 2, 3, 2, 1], 1))
    b = TT(W.random_tt([3, 4, 5, 2], [1, 3, 1, 2, 1], 2))
    fa, fb = dense(a), dense(b)
    assert np.allclose(dense(a + b), fa + fb, atol=1e-14)
    assert np.allclose(dense(a - b), fa - fb, atol=1e-14)
    assert np.allclose(dense(2.5 * a), 2.5 * fa, atol=1e-14)
    assert np.allclose(dense(a * -1.0), -fa, atol=1e-14)
    # ranks add, as the reference's concatenation does
    assert (a + b).R == [1, 5, 4, 4, 1]
    one = TT(W.random_tt([6], [1, 1], 3))
    assert np.allclose(dense(one - one), 0.0)


def test_diag_ttm_is_the_diagonal_operator():
    a = W.random_tt([3, 4, 2], [1, 2, 2, 1], 4)
    D = TT(diag_ttm(a))
    assert D.is_ttm and list(D.M) == [3, 4, 2] and list(D.N) == [3, 4, 2]
    full_a = TT(a).full().numpy().reshape(-1)
    # dense matrix of the TT-matrix: modes (m1, n1, m2, n2, ...) -> (m1 m2 m3) x (n1 n2 n3)
    t = D.full().numpy()
    d = 3
    perm = [2 * i for i in range(d)] + [2 * i + 1 for i in range(d)]
    mat = t.transpose(perm).reshape(full_a.size, full_a.size)
    assert np.allclose(mat, np.diag(full_a), atol=1e-14)
    x = np.random.default_rng(0).standard_normal(full_a.size)
    assert np.allclose(mat @ x, full_a * x, atol=1e-13)
