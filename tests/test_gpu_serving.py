"""Served / batched solves: several requests in flight at once on one GPU.

* every result is the same alone and in the mix (same request seed), within the solve tolerance;
* admission respects the memory budget (a budget that fits one request serialises the server);
* with room, requests overlap (peak concurrency > 1) and each reports queue/run latency.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _dev(cores, dev):
    from torchtt_gb300 import TT
    return TT([c.to(dev) for c in cores])


def requests(dev):
    from torchtt_gb300 import TT, workloads as W
    out = []
    for i in range(6):
        d, n = (5, 10) if i % 2 == 0 else (4, 12)
        A = TT([c.to(dev) for c in W.laplace_ttm(d, n, coeffs=[1.0 + 0.1 * i] * d)])
        b = TT([c.to(dev) for c in W.random_tt([n] * d, [1] + [2 + i % 3] * (d - 1) + [1], 40 + i)])
        out.append((A, b, dict(eps=1e-9, nswp=20, kickrank=4, seed=7 + i,
                               precision="mixed" if i % 3 else "fp64")))
    return out


def test_results_same_alone_and_in_mix(cuda):
    from torchtt_gb300 import amen_solve
    from torchtt_gb300.serving import Server
    reqs = requests(cuda)
    alone = [amen_solve(A, b, **kw) for A, b, kw in reqs]
    with Server(slots=4) as srv:
        ids = [srv.submit(A, b, **kw) for A, b, kw in reqs]
        mixed = [srv.result(i) for i in ids]
        st = srv.stats()
    assert st["completed"] == len(reqs)
    for (A, b, kw), xa, (xm, s) in zip(reqs, alone, mixed):
        ra = float((A @ xa - b).norm() / b.norm())
        rm = float((A @ xm - b).norm() / b.norm())
        assert rm < 1e-7 and ra < 1e-7, (ra, rm)
        assert float((xm - xa).norm() / xa.norm()) <= 10 * kw["eps"], kw
        assert s["run_ms"] > 0 and s["queue_ms"] >= 0


def test_admission_by_footprint(cuda):
    from torchtt_gb300.serving import Server
    reqs = requests(cuda)
    # a budget smaller than any request: the server admits one request at a time
    with Server(slots=4, mem_budget_bytes=1) as srv:
        ids = [srv.submit(A, b, **kw) for A, b, kw in reqs[:4]]
        for i in ids:
            srv.result(i)
        assert srv.stats()["peak_running"] == 1
    with Server(slots=4) as srv:
        ids = [srv.submit(A, b, **kw) for A, b, kw in reqs]
        for i in ids:
            srv.result(i)
        assert srv.stats()["peak_running"] >= 2


def test_invalid_request_is_rejected(cuda):
    from torchtt_gb300 import TT, workloads as W
    from torchtt_gb300.serving import Server
    A = TT([c.to(cuda) for c in W.laplace_ttm(3, 5)])
    b = TT([c.to(cuda) for c in W.random_tt([5] * 4, [1, 2, 2, 2, 1], 1)])
    with Server(slots=2) as srv:
        with pytest.raises(Exception):
            srv.submit(A, b)


def test_admission_never_overcommits_on_rank_growth(cuda):
    """Parametric diffusion systems with rank-16 right-hand sides grow their solution ranks to
    ~160 (from an initial rank of 1). Each request reserves its footprint bound, so with a budget
    just above one request's bound the requests run one at a time and the reservations never exceed
    the budget; the library's actual allocations of a request stay within its bound."""
    from torchtt_gb300 import workloads as W
    from torchtt_gb300.serving import Server, footprint, pool_usage
    wls = [W.parametric_diffusion_d10_n32(3, rhs_rank=16), W.parametric_diffusion_d10_n32(7, rhs_rank=16)]
    sys = [(_dev(w["A"], cuda), _dev(w["b"], cuda), w["params"]) for w in wls]
    fps = [footprint(A, b, precision="mixed", **p) for A, b, p in sys]
    budget = int(1.05 * max(fps))
    torch.cuda.synchronize()
    pool_usage(reset_high=True)
    base_now, _ = pool_usage()
    with Server(slots=2, mem_budget_bytes=budget) as srv:
        ids = [srv.submit(A, b, precision="mixed", seed=i, **p) for i, (A, b, p) in enumerate(sys)]
        res = [srv.result(i) for i in ids]
        mem = srv.memory()
        st = srv.stats()
    _, high = pool_usage()
    assert mem["budget"] == budget and mem["peak_in_use"] <= budget, mem
    assert st["peak_running"] == 1, st
    assert high - base_now <= max(fps), (high, base_now, fps)
    for (A, b, p), (x, _) in zip(sys, res):
        assert max(x.R) > 100      # the ranks did grow far beyond the right-hand side's
        assert float((A @ x - b).norm() / b.norm()) <= 10 * p["eps"]
