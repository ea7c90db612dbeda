"""The batched and served workloads beside the single large solve, at reduced counts:

* parametric diffusion (A(theta) = sum_k theta_k L_k, d=10, n=32, here with rhs ranks 1-3):
  several systems served at once, each solution within 10 eps in residual and within 10 eps of the FP64
  path's solution;
* rounding stress (A = L + C C^T + I, b = a sum of 4 random TTs rounded to 1e-8 on the GPU), at
  d=6, n=12 with rank-3 terms: the rounding keeps b within its tolerance and the solve reaches eps;
* serving trace (Poisson arrivals, eps in {1e-6, 1e-8, 1e-10}; here d ~ U{8..12}, n in {16, 32},
  rhs rank ~ U{1..8}): every request meets its own eps and requests overlap on the GPU.
"""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _dev(cores, dev):
    from torchtt_gb300 import TT
    return TT([c.to(dev) for c in cores])


def test_parametric_diffusion_batch(cuda):
    from torchtt_gb300 import amen_solve, workloads as W
    from torchtt_gb300.serving import Server
    wls = [W.parametric_diffusion_d10_n32(i, rhs_rank=1 + i % 3) for i in range(4)]
    sys = [(_dev(w["A"], cuda), _dev(w["b"], cuda), w["params"]) for w in wls]
    with Server(slots=4) as srv:
        ids = [srv.submit(A, b, precision="mixed", seed=i, **p) for i, (A, b, p) in enumerate(sys)]
        res = [srv.result(i) for i in ids]
        assert srv.stats()["peak_running"] >= 2
    for (A, b, p), (x, st) in zip(sys, res):
        rr = float((A @ x - b).norm() / b.norm())
        assert rr <= 10 * p["eps"], rr
        x64 = amen_solve(A, b, precision="fp64", **p)
        assert float((x - x64).norm() / x64.norm()) <= 10 * p["eps"]


def test_rounding_stress(cuda):
    from torchtt_gb300 import amen_solve, workloads as W
    w = W.rounding_stress(0, d=6, n=12, term_rank=3)
    A, b = _dev(w["A"], cuda), _dev(w["b"], cuda)
    br = b.round(w["round_b"])
    assert max(br.R) <= 12
    nb = float(b.norm())
    assert float((br - b).norm()) <= w["round_b"] * nb
    x = amen_solve(A, br, precision="mixed", **w["params"])
    assert float((A @ x - br).norm() / br.norm()) <= 10 * w["params"]["eps"]


def test_serving_trace(cuda):
    from torchtt_gb300.trace import replay
    out = replay(6, rate=50.0, slots=4, max_d=12, ranks=(1, 8), modes=(16, 32))
    assert out["max_relres_over_eps"] <= 10.0, out
    assert out["peak_running"] >= 2
    assert out["latency_ms"]["p99"] >= out["latency_ms"]["p50"] > 0
