"""Replays a serving trace through the request server and reports latency and throughput.

Requests arrive by a seeded Poisson process (``workloads.serving_trace``); each draws its own d,
n, right-hand-side rank, anisotropic Laplacian and eps (``workloads.serving_request``). A request
is submitted at its arrival time with its inputs already on the device; the server admits it as a
slot and its HBM footprint allow, so requests that arrive while others run overlap on the GPU.
The report gives solves/s over the whole replay, p50/p99 of queue + run latency, and the worst
relative residual ||A x - b|| / ||b|| divided by the request's eps.

  python -m torchtt_gb300.trace --requests 200 --rate 4 --slots 8 [--precision mixed|fp64]
"""
import argparse
import json
import time

import torch

from . import TT, workloads as W
from .serving import Server


def _percentile(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    k = (len(xs) - 1) * q
    lo, hi = int(k), min(int(k) + 1, len(xs) - 1)
    return xs[lo] + (xs[hi] - xs[lo]) * (k - lo)


def replay(count, rate, slots=8, precision="mixed", engine="auto", seed=5, mem_budget_bytes=0,
           check=True, device=None, max_d=24, ranks=(1, 32), modes=(16, 32, 64), strict_eps=False):
    """Replays ``count`` requests arriving at ``rate`` per second; ``max_d``, ``ranks`` and
    ``modes`` bound the request sizes (full size: 24, (1, 32), (16, 32, 64))."""
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    trace = W.serving_trace(count, rate, seed)
    reqs = []
    for t_arr, i in trace:   # inputs prepared on the device before the clock starts
        w = W.serving_request(i, seed, max_d=max_d, ranks=ranks, modes=modes)
        A = TT([c.to(dev) for c in w["A"]])
        b = TT([c.to(dev) for c in w["b"]])
        reqs.append((t_arr, i, w, A, b))
    torch.cuda.synchronize(dev)
    ids = []
    with Server(slots=slots, mem_budget_bytes=mem_budget_bytes, device=dev) as srv:
        t0 = time.perf_counter()
        for t_arr, i, w, A, b in reqs:
            wait = t_arr - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            ids.append(srv.submit(A, b, precision=precision, engine=engine, seed=1000 + i,
                                  strict_eps=strict_eps, **w["params"]))
        results = [srv.result(r) for r in ids]
        elapsed = time.perf_counter() - t0
        peak = srv.stats()["peak_running"]
    lat = [st["queue_ms"] + st["run_ms"] for _, st in results]
    out = {"requests": count, "rate_per_s": rate, "slots": slots, "precision": precision,
           "solves_per_s": count / elapsed, "elapsed_s": elapsed,
           "latency_ms": {"p50": _percentile(lat, 0.5), "p99": _percentile(lat, 0.99),
                          "max": max(lat)},
           "queue_ms_p99": _percentile([st["queue_ms"] for _, st in results], 0.99),
           "peak_running": peak}
    if check:
        worst = 0.0
        for (x, _), (_, _, w, A, b) in zip(results, reqs):
            rr = float((A @ x - b).norm() / b.norm())
            worst = max(worst, rr / w["params"]["eps"])
        out["max_relres_over_eps"] = worst
        out["relres_pass_frac"] = sum(
            1 for (x, _), (_, _, w, A, b) in zip(results, reqs)
            if float((A @ x - b).norm() / b.norm()) <= w["params"]["eps"]) / count
        out["unconverged"] = sum(1 for _, st in results if not st.get("converged", 1))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=100)
    ap.add_argument("--rate", type=float, default=4.0)
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--engine", default="auto", choices=["auto", "tc", "fp32"])
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--max-d", type=int, default=24)
    ap.add_argument("--max-rank", type=int, default=32)
    ap.add_argument("--no-check", action="store_true")
    args = ap.parse_args()
    print(json.dumps(replay(args.requests, args.rate, args.slots, args.precision, args.engine,
                            args.seed, check=not args.no_check, max_d=args.max_d,
                            ranks=(1, args.max_rank))))


if __name__ == "__main__":
    main()
