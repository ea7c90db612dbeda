"""ttgb_local_product_noalloc: the local product for callers that must not allocate device memory.

Callers such as a serving loop that reserved its HBM up front, or code living inside another
framework's memory manager, cannot call cudaMalloc while they run. This entry point gives them the
local product with its scratch in a static device array. The test calls it through the C ABI twice
in a row - the second call smaller, so the array still holds the first call's intermediates - and
checks each result against the allocating entry point ttgb_local_product within the FP64 tolerance
of the other kernel tests (1e-12 relative to the output's magnitude). It also checks that a request
larger than the array is refused with a clear error. This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _call(fn, PhiL, A, PhiR, x, y):
    rl, s, r = PhiL.shape
    _, m, n, S = A.shape
    RL, _, R = PhiR.shape
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return fn(rl, s, r, m, n, S, RL, R, _ptr(PhiL), _ptr(A), _ptr(PhiR), _ptr(x), _ptr(y), 1, stream)


@pytest.mark.parametrize("shapes", [((60, 3, 64, 3, 60), (12, 2, 16, 2, 9))])
def test_noalloc_matches_allocating_entry_point(cuda, shapes):
    from torchtt_gb300 import _lib
    L = _lib.lib()
    for i, (r, s, n, S, R) in enumerate(shapes):
        g = np.random.default_rng(100 + i)
        mk = lambda *sh: torch.from_numpy(g.standard_normal(sh)).to(cuda)
        PhiL, A, PhiR, x = mk(r, s, r), mk(s, n, n, S), mk(R, S, R), mk(r, n, R)
        y_ref = torch.empty((r, n, R), dtype=torch.float64, device=cuda)
        y = torch.full((r, n, R), float("nan"), dtype=torch.float64, device=cuda)
        assert _call(L.ttgb_local_product, PhiL, A, PhiR, x, y_ref) == 0
        assert _call(L.ttgb_local_product_noalloc, PhiL, A, PhiR, x, y) == 0, L.ttgb_last_error()
        torch.cuda.synchronize()
        scale = float(y_ref.abs().max())
        assert float((y - y_ref).abs().max()) <= 1e-12 * scale


def test_noalloc_matches_on_a_sparse_laplace_core(cuda):
    """On a Kronecker-sum Laplacian core ttgb_local_product applies A from its nonzeros (the
    structured A stage) while the no-allocation variant contracts it densely: same product."""
    from torchtt_gb300 import _lib, workloads as W
    L = _lib.lib()
    A = W.laplace_potential_ttm(4, 64)[1].to(cuda)       # 3 x 64 x 64 x 3, tridiagonal blocks
    s, n, S = A.shape[0], A.shape[1], A.shape[3]
    for call, (r, R) in enumerate([(40, 48), (12, 9)]):
        g = np.random.default_rng(300 + call)
        mk = lambda *sh: torch.from_numpy(g.standard_normal(sh)).to(cuda)
        PhiL, PhiR, x = mk(r, s, r), mk(R, S, R), mk(r, n, R)
        y_ref = torch.empty((r, n, R), dtype=torch.float64, device=cuda)
        y = torch.full((r, n, R), float("nan"), dtype=torch.float64, device=cuda)
        assert _call(L.ttgb_local_product, PhiL, A, PhiR, x, y_ref) == 0
        assert _call(L.ttgb_local_product_noalloc, PhiL, A, PhiR, x, y) == 0, L.ttgb_last_error()
        torch.cuda.synchronize()
        assert float((y - y_ref).abs().max()) <= 1e-12 * float(y_ref.abs().max())


def test_noalloc_rejects_oversize(cuda):
    from torchtt_gb300 import _lib
    L = _lib.lib()
    r, s, n, S, R = 200, 3, 64, 3, 200       # needs 2 * 200*3*64*200 = 15.4 M doubles > 4 Mi
    one = torch.zeros(1, dtype=torch.float64, device=cuda)
    p = _ptr(one)
    st = L.ttgb_local_product_noalloc(r, s, r, n, n, S, R, R, p, p, p, p, p, 1, None)
    assert st == _lib.TTGB_ERR_INVALID
    assert b"more than the" in L.ttgb_last_error()
    # dimensions whose scratch size wraps around 2^64 are refused, not truncated
    big = 1 << 40
    st = L.ttgb_local_product_noalloc(big, 3, 1, big, 1, 3, 1, big, p, p, p, p, p, 1, None)
    assert st == _lib.TTGB_ERR_INVALID
    assert b"more than" in L.ttgb_last_error()
