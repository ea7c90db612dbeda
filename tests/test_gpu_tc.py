"""The low-precision engines of the local product (FP32 CUDA cores; tcgen05 tensor cores with a
3xTF32 split and FP32 accumulation in tensor memory) against the FP64 oracle. The mixed path needs
the operator to about 1e-5 relative (its inner-solve floor); 3xTF32 and FP32 give ~1e-6."""
import numpy as np
import pytest
import torch

from oracle import amen as O

pytestmark = pytest.mark.gpu

SHAPES = [(60, 3, 64, 3, 60), (52, 2, 16, 2, 50), (8, 7, 32, 7, 8), (1, 3, 64, 3, 9),
          (80, 3, 64, 3, 88), (5, 2, 12, 2, 7), (171, 2, 32, 2, 20)]


@pytest.mark.parametrize("engine", [1, 2])
@pytest.mark.parametrize("shape", SHAPES)
def test_lowp_local_product(cuda, engine, shape):
    from torchtt_gb300 import ops
    r, s, n, S, R = shape
    g = np.random.default_rng(sum(shape) + engine)
    PhiL, A = g.standard_normal((r, s, r)), g.standard_normal((s, n, n, S))
    PhiR, x = g.standard_normal((R, S, R)), g.standard_normal((r, n, R))
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    y = ops.local_product_lowp(t(PhiR), t(PhiL), t(A), t(x), engine=engine).cpu().numpy()
    ref = O.local_product(PhiR, PhiL, A, x)
    err = np.linalg.norm(y - ref) / np.linalg.norm(ref)
    assert err < 1e-5, err
    assert np.abs(y - ref).max() <= 1e-4 * np.abs(ref).max()
