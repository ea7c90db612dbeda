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


@pytest.mark.parametrize("rR", [(60, 60), (5, 7), (81, 77), (1, 9)])
def test_tc_local_product_structured_core(cuda, rR):
    """The tcgen05 engine with a sparse Kronecker-sum core (structured A stage between the two
    tensor-core GEMMs, its output written as the padded TF32 split the second GEMM's TMA reads),
    against the FP64 oracle at the engine's 1e-5."""
    from torchtt_gb300 import ops, workloads as W
    r, R = rR
    A = W.laplace_potential_ttm(4, 64)[1].numpy()       # 3 x 64 x 64 x 3
    s, n, S = A.shape[0], A.shape[1], A.shape[3]
    g = np.random.default_rng(r * 1000 + R)
    PhiL, PhiR, x = g.standard_normal((r, s, r)), g.standard_normal((R, S, R)), g.standard_normal((r, n, R))
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    y = ops.local_product_lowp(t(PhiR), t(PhiL), t(A), t(x), engine=2).cpu().numpy()
    ref = O.local_product(PhiR, PhiL, A, x)
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-5


@pytest.mark.parametrize("shape", [(60, 3, 64, 3, 60), (1, 3, 64, 3, 9), (171, 2, 32, 2, 20),
                                   (5, 2, 12, 2, 7)])
def test_double_float_local_product(cuda, shape):
    """The mixed path's FP64-class engine (double-float arithmetic on the FP32 pipe, operands split
    from their bits) against the FP64 oracle, on operands with mixed signs, exact zeros and values
    spread over 2^-20..2^20 (products stay inside the FP32 range): every entry within 1e-12 of
    the sum of the absolute values of its terms (the oracle's product of the absolute operands)."""
    from torchtt_gb300 import ops
    r, s, n, S, R = shape
    g = np.random.default_rng(sum(shape) + 31)

    def spread(*dims):
        v = g.standard_normal(dims) * np.exp2(g.integers(-20, 21, size=dims))
        v[g.random(dims) < 0.1] = 0.0
        return v

    PhiL, A, PhiR, x = spread(r, s, r), spread(s, n, n, S), spread(R, S, R), spread(r, n, R)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    y = ops.local_product_lowp(t(PhiR), t(PhiL), t(A), t(x), engine=ops.ENGINE_DF).cpu().numpy()
    ref = O.local_product(PhiR, PhiL, A, x)
    bound = O.local_product(np.abs(PhiR), np.abs(PhiL), np.abs(A), np.abs(x))
    assert np.all(np.abs(y - ref) <= 1e-12 * bound + 1e-300)
