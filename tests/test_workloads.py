"""The seeded synthetic workloads match the benchmark definitions they stand in for: shapes, TT
ranks, operator structure, parameters, normalisation and seeding (CPU only)."""
import numpy as np

from torchtt_gb300 import workloads as W


def ranks(cores):
    return [c.shape[0] for c in cores] + [cores[-1].shape[-1]]


def test_config1_laplace_d8_n16():
    w = W.laplace_d8_n16()
    A, b, x0 = w["A"], w["b"], w["x0"]
    assert len(A) == 8 and all(c.shape[1] == c.shape[2] == 16 for c in A)
    assert ranks(A) == [1] + [2] * 7 + [1]
    assert ranks(b) == [1] + [4] * 7 + [1] and ranks(x0) == [1] + [2] * 7 + [1]
    assert w["params"] == dict(eps=1e-10, nswp=20, kickrank=4)
    assert abs(W._tt_norm_np([c.numpy() for c in b]) - 1.0) < 1e-12
    # the 1-D Laplacian block (n+1)^2 tridiag(-1, 2, -1) sits in the first core
    L = W.laplace_1d(16)
    assert np.allclose(np.diag(L), 2 * 17 ** 2) and np.allclose(np.diag(L, 1), -(17 ** 2))


def test_config2_laplace_potential_d20_n64():
    w = W.laplace_potential_d20_n64()
    A, b = w["A"], w["b"]
    assert len(A) == 20 and all(c.shape[1] == c.shape[2] == 64 for c in A)
    assert ranks(A) == [1] + [3] * 19 + [1]
    assert ranks(b) == [1] + [8] * 19 + [1] and w["x0"] is None
    assert w["params"] == dict(eps=1e-8, nswp=20, kickrank=8)
    assert abs(W._tt_norm_np([c.numpy() for c in b]) - 1.0) < 1e-12
    v = W.potential_1d(64)
    i = np.arange(64)
    assert np.allclose(np.diag(v) if v.ndim == 2 else v, 1 + 0.5 * np.cos(2 * np.pi * i / 64))


def test_config3_parametric_diffusion():
    ws = [W.parametric_diffusion_d10_n32(i) for i in range(16)]
    for w in ws:
        assert len(w["A"]) == 10 and w["A"][0].shape[1] == 32
        assert ranks(w["A"]) == [1] + [2] * 9 + [1]
        assert np.all((w["theta"] >= 0.5) & (w["theta"] <= 2.0))
        assert 1 <= w["rhs_rank"] <= 16 and ranks(w["b"])[1] == w["rhs_rank"]
        assert w["params"] == dict(eps=1e-8, nswp=40, kickrank=8)
    assert len({w["rhs_rank"] for w in ws}) > 1          # uneven ranks across the batch
    a, b = W.parametric_diffusion_d10_n32(3), W.parametric_diffusion_d10_n32(3)
    assert np.array_equal(a["theta"], b["theta"])        # seeded


def test_config4_rounding_stress_small():
    w = W.rounding_stress(0, d=6, n=12, term_rank=3)
    assert len(w["A"]) == 6 and w["A"][0].shape[1] == 12
    assert ranks(w["b"])[1] == 4 * 3                       # sum of 4 terms before rounding
    assert w["round_b"] == 1e-8


def test_config5_serving_requests_and_trace():
    for i in range(40):
        w = W.serving_request(i)
        d, n = w["d"], w["n"]
        assert 8 <= d <= 24 and n in (16, 32, 64) and 1 <= w["rhs_rank"] <= 32
        assert len(w["A"]) == d and ranks(w["A"]) == [1] + [2] * (d - 1) + [1]
        assert w["params"]["eps"] in (1e-6, 1e-8, 1e-10)
        assert w["params"]["nswp"] == 40 and w["params"]["kickrank"] == 8
    t = W.serving_trace(200, rate=4.0)
    times = np.array([a for a, _ in t])
    assert np.all(np.diff(times) > 0) and [i for _, i in t] == list(range(200))
    assert abs(times[-1] / 200 - 0.25) < 0.08               # mean inter-arrival 1 / rate
    assert W.serving_trace(5, 4.0) == W.serving_trace(5, 4.0)
