"""Kernel timeline of one served batch: how the solves of a batch overlap on the device.

Runs one warm-up batch and one profiled batch of B mixed-precision solves of a workload (the same
A, B seeded right-hand sides) through the request server, records every kernel with the CUDA
activity tracer of ``torch.profiler``, and reports: wall time, the union of kernel-busy intervals,
the sum of kernel durations (their ratio is the mean number of kernels in flight), time spent at
each concurrency level, the gaps between consecutive kernels of one stream (launch latency and host
synchronisation), and per stream its kernel count, span and busy fraction.

  python -m torchtt_gb300.timeline [--workload laplace_potential_d20_n64] [--batch 8] [--slots 8]
"""
import argparse
import collections
import json
import os
import tempfile
import time

import torch

from . import TT, workloads as W
from .serving import Server


def _percentile(xs, q):
    return xs[int(q * (len(xs) - 1))] if xs else None


def analyse(kernels):
    """Concurrency and per-stream statistics of trace events (``ts``/``dur`` in microseconds)."""
    pts = []
    for e in kernels:
        pts.append((e["ts"], 1))
        pts.append((e["ts"] + e["dur"], -1))
    pts.sort()
    cur, last, busy = 0, pts[0][0], 0.0
    levels = collections.Counter()
    for t, dl in pts:
        if cur > 0:
            busy += t - last
        levels[min(cur, 16)] += t - last
        cur += dl
        last = t
    by_stream = collections.defaultdict(list)
    for e in kernels:
        by_stream[e.get("args", {}).get("stream", -1)].append(e)
    gaps, streams = [], {}
    for s, L in by_stream.items():
        L.sort(key=lambda e: e["ts"])
        span = L[-1]["ts"] + L[-1]["dur"] - L[0]["ts"]
        kb = sum(e["dur"] for e in L)
        gaps += [L[i + 1]["ts"] - (L[i]["ts"] + L[i]["dur"]) for i in range(len(L) - 1)]
        streams[str(s)] = {"kernels": len(L), "span_ms": span / 1e3, "kernel_ms": kb / 1e3,
                           "busy_frac": kb / max(span, 1e-9)}
    gaps.sort()
    t0 = min(e["ts"] for e in kernels)
    t1 = max(e["ts"] + e["dur"] for e in kernels)
    total = sum(e["dur"] for e in kernels)
    return {"kernels": len(kernels), "span_ms": (t1 - t0) / 1e3, "busy_ms": busy / 1e3,
            "sum_kernel_ms": total / 1e3, "mean_in_flight": total / max(busy, 1e-9),
            "ms_at_concurrency": {k: v / 1e3 for k, v in sorted(levels.items())},
            "stream_gap_us": {"p10": _percentile(gaps, 0.1), "p50": _percentile(gaps, 0.5),
                              "p90": _percentile(gaps, 0.9), "p99": _percentile(gaps, 0.99)},
            "streams": streams}


def run(workload="laplace_potential_d20_n64", batch=8, slots=8, precision="mixed", seed=1):
    from torch.profiler import ProfilerActivity, profile
    dev = torch.device("cuda", torch.cuda.current_device())
    wls = [getattr(W, workload)(seed + j) for j in range(batch)]
    p = wls[0]["params"]
    kw = dict(nswp=p.get("nswp", 22), eps=p["eps"], kickrank=p["kickrank"])
    A = TT([c.to(dev) for c in wls[0]["A"]])
    bs = [TT([c.to(dev) for c in w["b"]]) for w in wls]
    with Server(slots=slots, device=dev) as srv:
        def step():
            ids = [srv.submit(A, b, precision=precision, seed=1000 + j, **kw)
                   for j, b in enumerate(bs)]
            return [srv.result(i) for i in ids]
        step()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        step()
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t0
        with profile(activities=[ProfilerActivity.CUDA]) as prof:
            step()
            torch.cuda.synchronize(dev)
    fd, path = tempfile.mkstemp(suffix=".json")
    os.close(fd)
    try:
        prof.export_chrome_trace(path)
        with open(path) as f:
            events = json.load(f)["traceEvents"]
    finally:
        os.unlink(path)
    kernels = [e for e in events if e.get("cat") == "kernel"]
    out = {"workload": workload, "batch": batch, "slots": slots, "precision": precision,
           "wall_s_unprofiled": wall}
    out.update(analyse(kernels))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="laplace_potential_d20_n64",
                    choices=["laplace_potential_d20_n64", "laplace_d8_n16"])
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    args = ap.parse_args()
    print(json.dumps(run(args.workload, args.batch, args.slots, args.precision), indent=1))


if __name__ == "__main__":
    main()
