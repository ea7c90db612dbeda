"""Benchmark: AMEn solves/s (and per-solve latency) on one GB300.

Workload (default): the single large solve - d=20, n=64, A = Kronecker-sum Laplacian
(n+1)^2 tridiag(-1,2,-1) plus the product potential (x)_k diag(1 + 0.5 cos(2 pi i/n)) (TT rank 3),
b = random TT of rank 8 with N(0,1) cores (seeded, ||b|| = 1), x0 = ones, eps = 1e-8, kickrank 8,
nswp 20. One step = one complete solve. Synthetic seeded data; no dataset is involved.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

* gb300 arm: W warm-up solves, then K timed solves bracketed by barrier + synchronize (CUDA events
  on the solve stream), an L2 flush (256 MiB write) between solves; ``value`` = total solves / s over
  all ranks (weak scaling: every rank solves its own copy of the workload). ``e2e`` repeats the
  solve through the public API (``torchtt_gb300.amen_solve``) with CPU-resident TT cores, so host to
  device copies of A and b and the copy of x back are inside the timed region.
* reference arm: the reference's CPU algorithm (the numpy restatement in oracle/, on all host
  threads; the compiled reference cannot be built on the GPU host) on rank 0 only, same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = ("laplace_potential_d20_n64", "laplace_d8_n16")
FP64_PEAK_TFLOPS = 1.20   # measured FP64 FMA-pipe rate of this GB300 pool (profiles/fp64_fma_peak.md)


def get_workload(name, seed):
    from torchtt_gb300 import workloads as W
    if name == "laplace_potential_d20_n64":
        return W.laplace_potential_d20_n64(seed)
    if name == "laplace_d8_n16":
        return W.laplace_d8_n16(seed)
    raise SystemExit("unknown workload " + name)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def percentile(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    k = (len(xs) - 1) * q
    lo, hi = int(k), min(int(k) + 1, len(xs) - 1)
    return xs[lo] + (xs[hi] - xs[lo]) * (k - lo)


def cpu_solve_once(wl):
    """One solve of the workload with the oracle (the reference's algorithm on the CPU)."""
    from oracle import amen as O
    p = wl["params"]
    A = [c.numpy() for c in wl["A"]]
    b = [c.numpy() for c in wl["b"]]
    x0 = [c.numpy() for c in wl["x0"]] if wl.get("x0") is not None else None
    t0 = time.perf_counter()
    x, info = O.amen_solve(A, b, x0, nswp=p.get("nswp", 22), eps=p["eps"], kickrank=p["kickrank"])
    return time.perf_counter() - t0, info


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    wl = get_workload(args.workload, args.seed)
    cores = os.cpu_count() or 1
    times = []
    for i in range(args.warmup + args.steps):
        dt, info = cpu_solve_once(wl)
        if i >= args.warmup:
            times.append(dt)
    total = sum(times)
    value = len(times) / total
    line = {
        "metric": "AMEn solves/s (single large solve, FP64 CPU reference algorithm)",
        "impl": "reference", "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * total / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "eps": wl["params"]["eps"],
                   "kickrank": wl["params"]["kickrank"], "nswp": wl["params"].get("nswp", 22)},
        "latency_ms": {"p50": 1000 * percentile(times, 0.5), "p99": 1000 * percentile(times, 0.99)},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": "%d full solves of %s, numpy/OpenBLAS on all host threads"
                                   % (len(times), args.workload)},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def read_traffic(kernel_profile):
    path = os.path.join(ROOT, "profiles", kernel_profile)
    try:
        for ln in open(path):
            if ln.startswith("traffic_bytes_per_launch:"):
                return float(ln.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def run_gb300(args):
    import torch
    import torch.distributed as dist

    ws, rank, local = dist_env()
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from torchtt_gb300 import build as B
    if rank == 0:
        B.build()
    if ws > 1:
        dist.barrier()
    from torchtt_gb300 import TT, amen_solve, _lib
    from torchtt_gb300.solvers import solve_cores

    wl = get_workload(args.workload, args.seed)
    p = wl["params"]
    kw = dict(nswp=p.get("nswp", 22), eps=p["eps"], kickrank=p["kickrank"], seed=args.seed + rank)
    A_d = [c.to(dev) for c in wl["A"]]
    b_d = [c.to(dev) for c in wl["b"]]
    x0_d = [c.to(dev) for c in wl["x0"]] if wl.get("x0") is not None else None
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def solve(profile=0):
        return solve_cores(A_d, b_d, x0_d, **kw, stream=stream) if not profile else \
            _solve_profiled()

    def _solve_profiled():
        import ctypes
        L = _lib.lib()
        from torchtt_gb300.solvers import _desc
        keep = []
        dA, db = _desc(A_d, True, keep), _desc(b_d, False, keep)
        dx = _desc(x0_d, False, keep) if x0_d else None
        prm = _lib.AmenParams()
        L.ttgb_default_params(ctypes.byref(prm))
        prm.nswp, prm.eps, prm.kickrank, prm.seed, prm.profile = kw["nswp"], kw["eps"], kw["kickrank"], kw["seed"], 1
        h = _lib.c_vp()
        _lib.check(L.ttgb_amen_solve(ctypes.byref(dA), ctypes.byref(db), ctypes.byref(dx) if dx else None, None,
                                     ctypes.byref(prm), ctypes.c_void_p(stream.cuda_stream), ctypes.byref(h)))
        st = _lib.Stats()
        L.ttgb_solution_stats(h, ctypes.byref(st))
        L.ttgb_solution_free(h)
        return None, st.as_dict()

    for _ in range(args.warmup):
        solve()
    torch.cuda.synchronize()
    launches0 = _lib.lib().ttgb_launch_count()
    sampler = ClockSampler(local)
    sampler.start()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    stats = []
    last = None
    for i in range(args.steps):
        flush.fill_(float(i))            # L2 flush between solves (256 MiB > 129 MB L2)
        ev[2 * i].record(stream)
        last, st = solve()
        ev[2 * i + 1].record(stream)
        stats.append(st)
    t_end.record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    clocks = sampler.stop()
    launches = _lib.lib().ttgb_launch_count() - launches0
    elapsed_ms = t_start.elapsed_time(t_end)
    lat = [ev[2 * i].elapsed_time(ev[2 * i + 1]) for i in range(args.steps)]
    if ws > 1:
        t = torch.tensor([elapsed_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    value = ws * args.steps / (elapsed_ms / 1000.0)

    # relative residual of the last solution (TT algebra on the device)
    A_tt, b_tt = TT(A_d), TT(b_d)
    relres = float((A_tt @ TT(last) - b_tt).norm() / b_tt.norm())

    # live roofline of the dominant kernel (the FP64 contraction engine), one profiled solve
    _, pst = solve(profile=1)
    achieved = pst["contract_flops"] / (pst["contract_ms"] * 1e-3) / 1e12 if pst["contract_ms"] > 0 else None
    per_launch_flops = pst["contract_flops"] / max(1, pst["contract_launches"])
    roofline = {"bound": "fp64", "achieved": achieved, "peak": FP64_PEAK_TFLOPS, "unit": "TFLOP/s",
                "frac": (achieved / FP64_PEAK_TFLOPS) if achieved else None,
                "traffic": read_traffic("contract_f64_laplace_potential_d20_n64.md"),
                "kernel": "contract_kernel (FP64 contraction engine)",
                "launches": pst["contract_launches"], "avg_launch_us": 1000 * pst["contract_ms"] / max(1, pst["contract_launches"]),
                "flops_per_launch": per_launch_flops,
                "peak_source": "measured FP64 FMA rate (profiles/fp64_fma_peak.md); MEASURED_PEAKS.json has no FP64 entry"}

    # end to end through the public API with host-resident TT cores
    A_h, b_h = TT([c.clone() for c in wl["A"]]), TT([c.clone() for c in wl["b"]])
    x0_h = TT(wl["x0"]) if wl.get("x0") is not None else None
    h2d = sum(c.numel() * 8 for c in wl["A"]) + sum(c.numel() * 8 for c in wl["b"]) + \
        (sum(c.numel() * 8 for c in wl["x0"]) if wl.get("x0") is not None else 0)
    e2e_steps = max(1, min(args.steps, 3))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d2h = 0
    for _ in range(e2e_steps):
        xh = amen_solve(A_h, b_h, x0=x0_h, **kw)
        d2h = sum(c.numel() * 8 for c in xh.cores)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_val = ws * e2e_steps / e2e_s if ws == 1 else None
    if ws > 1:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_val = ws * e2e_steps / float(t.item())

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        dt, info = cpu_solve_once(wl)
        cpu = {"value": 1.0 / dt, "unit": "solves/s", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": "1 full solve of %s with the numpy restatement of the reference (oracle/amen.py), "
                         "numpy/OpenBLAS threads = all host cores" % args.workload}

    if rank == 0:
        st = stats[-1]
        line = {
            "metric": "AMEn solves/s (single large solve, plain FP64 GPU path)",
            "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": args.workload, "d": 20 if "d20" in args.workload else 8,
                       "eps": p["eps"], "kickrank": p["kickrank"], "nswp": p.get("nswp", 22),
                       "precision": "fp64", "l2": "256 MiB flush write between solves",
                       "parallelism": "replicas" if ws > 1 else "single"},
            "latency_ms": {"p50": percentile(lat, 0.5), "p99": percentile(lat, 0.99)},
            "solve": {"relres": relres, "sweeps": st["sweeps"], "max_rank": max(st["ranks"]),
                      "matvecs": st["matvecs"], "gmres_iterations": st["gmres_iterations"],
                      "host_syncs": st["host_syncs"]},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_val, "unit": "solves/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": e2e_steps},
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=WORKLOADS[0], choices=WORKLOADS)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
