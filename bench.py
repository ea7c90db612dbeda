"""Benchmark: AMEn solves/s and per-request p50/p99 latency on one GB300, mixed precision, batched.

Workload: the single large solve, d=20, n=64. A = Kronecker-sum Laplacian (n+1)^2 tridiag(-1,2,-1)
plus the product potential (x)_k diag(1 + 0.5 cos(2 pi i/n)) (TT rank 3); b_j = random TT of rank
8 with N(0,1) cores from seed (seed + j), ||b_j|| = 1; x0 = ones; eps 1e-8, kickrank 8, nswp 20.
Synthetic seeded data; no dataset is involved.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--batch B]
                  [--slots S]

* gb300 arm. One step = one batch of B (default 16) such solves (the same A, B right-hand sides)
  submitted together to the request server (``torchtt_gb300.serving.Server`` with S = 16 slots by
  default): each admitted solve runs the mixed-precision path (low-precision local GMRES operator
  inside FP64 iterative refinement) on its own stream and host thread, so up to S solves overlap
  on the device. With S < B a queued request is admitted as soon as a running one completes
  (continuous batching; ``--slots 8`` runs the 16 requests through 8 slots). 16 slots measured
  4.66 solves/s with p99 3.5 s, against 4.32 solves/s with p99 3.7 s for 8 slots (p50 3.2 s
  against 2.5 s). Latencies include the queueing. W untimed
  warm-up steps, then K timed steps bracketed by barrier + synchronize, CUDA events on the
  submitting stream around each step (the host waits for every result inside the step), a 256 MiB
  L2 flush write between steps. ``value`` = solves / s over all ranks (weak scaling: every rank
  serves its own batch). Beside it, measured in the same run: the plain FP64 path one solve at a
  time (the baseline the mixed/batched path is compared with), the mixed path unbatched, the FP64
  path batched, the relative residual of every solution and ||x_mixed - x_fp64|| / ||x_fp64||.
  ``e2e`` repeats batched steps with host-resident (pinned) inputs through the public API, so the
  host-to-device copies of A and every b_j and the copies of the solutions back are timed.
* reference arm: the reference's own CPU implementation (its package ``torchtt`` installed in
  baseline/_ref, with its C++ extension compiled on this host from the reference's sources by
  oracle/build_ref.py; ``torchtt.solvers.amen_solve(use_cpp=True)``, FP64, all host threads) on
  rank 0 only, one solve of the same workload per step.
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
METRIC = "AMEn solves/s & p99 latency at rel. residual 1e-8: mixed/batched vs FP64 plain"


def get_workload(name, seed):
    from torchtt_gb300 import workloads as W
    if name == "laplace_potential_d20_n64":
        return W.laplace_potential_d20_n64(seed)
    if name == "laplace_d8_n16":
        return W.laplace_d8_n16(seed)
    raise SystemExit("unknown workload " + name)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


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
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_median": statistics.median(power) if power else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(x, dist, device):
    """The largest of the ranks' values (timing is reported for the slowest rank)."""
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_seeds(seed, rank, batch):
    """Right-hand-side seeds of one rank's batch: disjoint across ranks (weak scaling)."""
    return [seed + rank * batch + j for j in range(batch)]


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


def reference_solver():
    """The reference's own CPU implementation of the path: its package ``torchtt`` from the install
    in baseline/_ref with the C++ extension ``torchttcpp`` compiled for this host from the
    reference's sources (oracle/build_ref.py). Returns ``(solve(wl) -> seconds, kind, how)``.

    ``torchtt.solvers.amen_solve(A, b, ..., use_cpp=True)`` is called when the package imports
    (its public API, which calls ``torchttcpp.amen_solve``, torchtt/solvers.py:268-285); when its
    Python dependencies are missing on this host, ``torchttcpp.amen_solve`` is called with the
    arguments that function passes. Where the reference cannot be built, the numpy restatement
    of its algorithm (oracle/amen.py) is timed instead and reported as kind "port"."""
    import torch
    torch.set_num_threads(os.cpu_count() or 1)
    try:
        from oracle import build_ref
        torchtt, cpp = build_ref.load_installed()
    except Exception as e:  # noqa: BLE001 - reported in the JSON line
        why = str(e).strip().splitlines()[0] if str(e).strip() else type(e).__name__

        def solve_port(wl):
            return cpu_solve_once(wl)[0]
        return solve_port, "port", ("the numpy restatement of the reference (oracle/amen.py); the "
                                    "compiled reference is unavailable here: %s" % why)

    def args_of(wl):
        p = wl["params"]
        return dict(nswp=p.get("nswp", 22), eps=p["eps"], kickrank=p["kickrank"])

    if torchtt is not None:
        def solve_api(wl):
            kw = args_of(wl)
            A, b = torchtt.TT(list(wl["A"])), torchtt.TT(list(wl["b"]))
            torch.manual_seed(1)
            t0 = time.perf_counter()
            torchtt.solvers.amen_solve(A, b, use_cpp=True, **kw)
            return time.perf_counter() - t0
        return solve_api, "reference", ("torchtt.solvers.amen_solve(use_cpp=True) of the reference's "
                                        "install (baseline/_ref), its C++ extension compiled on this "
                                        "host from the reference's sources")

    def solve_ext(wl):
        kw = args_of(wl)
        A, b = list(wl["A"]), list(wl["b"])
        d = len(A)
        N = [int(c.shape[2]) for c in A]
        rA = [1] + [int(c.shape[3]) for c in A]
        rb = [1] + [int(c.shape[2]) for c in b]
        torch.manual_seed(1)
        t0 = time.perf_counter()
        cpp.amen_solve(A, b, [], N, rA, rb, [1] * (d + 1), kw["nswp"], kw["eps"], 32768, 500,
                       kw["kickrank"], 0, 40, 2, False, 0)
        return time.perf_counter() - t0
    return solve_ext, "reference", ("torchttcpp.amen_solve (cpp/amen_solve.h:122) compiled on this host "
                                    "from the reference's sources, called with the arguments of "
                                    "torchtt/solvers.py:283 (the package's Python dependencies are "
                                    "not installed here)")


def workload_config(args, wl):
    p = wl["params"]
    return {"workload": args.workload, "d": len(wl["A"]), "n": int(wl["A"][0].shape[1]),
            "A_rank": int(wl["A"][0].shape[-1]), "b_rank": int(wl["b"][0].shape[-1]),
            "eps": p["eps"], "kickrank": p["kickrank"], "nswp": p.get("nswp", 22)}


def arm_config(args, wl, ws):
    """The ``config`` of the JSON line, the same for both arms."""
    cfg = workload_config(args, wl)
    cfg.update({"precision": "mixed", "engine": args.engine, "batch": args.batch,
                "server_slots": args.slots, "l2": "256 MiB flush write between steps",
                "parallelism": "replicas" if ws > 1 else "single"})
    return cfg


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    solve, kind, how = reference_solver()
    times = []
    for i in range(args.warmup + args.steps):
        wl = get_workload(args.workload, args.seed + i % args.batch)
        dt = solve(wl)
        if i >= args.warmup:
            times.append(dt)
    total = sum(times)
    value = len(times) / total
    line = {
        "metric": METRIC, "impl": "reference", "value": value, "unit": "solves/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": arm_config(args, get_workload(args.workload, args.seed), ws),
        "reference_path": "plain FP64 on the host CPU, one solve per step (the reference has no "
                          "mixed-precision or batched path); right-hand side of step i: seed "
                          "%d + i mod %d" % (args.seed, args.batch),
        "latency_ms": {"p50": 1000 * percentile(times, 0.5), "p99": 1000 * percentile(times, 0.99)},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": kind,
                         "sample": "%d full solves of %s (one per step), %s, torch intra-op threads = "
                                   "%d" % (len(times), args.workload, how, cores)},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def tt_relres_check(A_cores, x_cores, b_cores):
    """||A x - b|| / ||b|| of TT cores on the GPU, for the accuracy fields of the JSON line (a
    check on the solutions, outside every timed region): the residual's cores [A_k x_k, -b_k]
    (ranks add) are orthogonalised right to left with Householder QR (torch.linalg.qr), which keeps
    the accuracy of a norm ~1e-8 of its parts' norms."""
    import torch
    d = len(A_cores)

    def core(k):
        a, x, b = A_cores[k], x_cores[k], b_cores[k]
        s, m, _, S = a.shape
        r, _, R = x.shape
        y = torch.einsum("smnS,rnR->srmSR", a, x).reshape(s * r, m, S * R)
        if d == 1:
            return y - b
        if k == 0:
            return torch.cat([y, -b], dim=2)
        if k == d - 1:
            return torch.cat([y, b], dim=0)
        out = torch.zeros((y.shape[0] + b.shape[0], m, y.shape[2] + b.shape[2]),
                          dtype=y.dtype, device=y.device)
        out[:y.shape[0], :, :y.shape[2]] = y
        out[y.shape[0]:, :, y.shape[2]:] = b
        return out

    def norm(cores):
        cur = None
        for k in range(len(cores) - 1, -1, -1):
            c = cores[k]
            if cur is not None:
                c = torch.tensordot(c, cur, dims=([2], [0]))
            if k == 0:
                return float(torch.linalg.norm(c))
            r = c.shape[0]
            rf = torch.linalg.qr(c.reshape(r, -1).T, mode="r")[1]   # (min, r)
            cur = rf.T                                               # r x min
        return 0.0

    return norm([core(k) for k in range(d)]) / norm(list(b_cores))


def run_configs(args, dev, engine, strict):
    """The batched and served workloads beside the headline, mixed and plain FP64 through the same
    server with the same slots (so their ratio is the same-batching mixed/FP64 speed-up), within a
    wall budget (``--configs-budget-s``; a stage runs only while the budget lasts):

    * parametric diffusion (256 systems A(theta) = sum_k theta_k L_k, d=10, n=32, rhs rank U{1..16},
      eps 1e-8, nswp 40, kickrank 8): all 256 systems mixed; FP64 on every 8th system (32, rhs
      ranks across 1-16), whose mixed rate is measured in the same run for the ratio;
    * rounding stress (128 solves, d=16, n=32, A = L + C C^T + I, b = a sum of 4 random TTs rounded
      to 1e-8 before the solve): terms of rank 4 (b of rank 16, nswp 40), 8 solves - with the full
      terms of rank 16 the reference's own solve does not converge in 20 sweeps (relres 0.70,
      ranks <= 161);
    * serving trace (10,000 requests, Poisson arrivals, d U{8..24}, n in {16,32,64}, rhs rank
      U{1..32}, eps in {1e-6,1e-8,1e-10}): the first 16 requests of the seeded trace at 2
      requests/s (above capacity, so the replay measures served throughput with queueing).
    Residuals are checked after each timed run (tt_relres_check), outside the timing."""
    import torch
    from torchtt_gb300 import TT, workloads as W
    from torchtt_gb300.serving import Server

    t_start = time.perf_counter()

    def left():
        return args.configs_budget_s - (time.perf_counter() - t_start)

    def served(systems, precision, arrivals=None):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        with Server(slots=args.slots, device=dev) as srv:
            ids = []
            for i, (A, b, p) in enumerate(systems):
                if arrivals is not None:
                    wait = arrivals[i] - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(wait)
                ids.append(srv.submit(A, b, precision=precision, engine=engine, seed=7 + i,
                                      strict_eps=strict, **p))
            res = [srv.result(r) for r in ids]
        el = time.perf_counter() - t0
        lat = [st["queue_ms"] + st["run_ms"] for _, st in res]
        rr = [tt_relres_check(A.cores, x.cores, b.cores) / p["eps"]
              for (A, b, p), (x, _) in zip(systems, res)]
        return {"solves": len(systems), "solves_per_s": len(systems) / el, "elapsed_s": el,
                "latency_ms": {"p50": percentile(lat, 0.5), "p99": percentile(lat, 0.99)},
                "max_relres_over_eps": max(rr), "relres_pass_frac": sum(1 for v in rr if v <= 1.0) / len(rr),
                "max_rank": max(max(st["ranks"]) for _, st in res)}

    def pair(systems, full_count, note, arrivals=None, sample=None, sample_note=None):
        """mixed over `systems`; FP64 over `sample` (default: the same systems), and then the
        mixed rate of that sample too when it differs, so the ratio compares like with like"""
        out = {"sample": note, "full_size": full_count}
        t0 = time.perf_counter()
        out["mixed"] = served(systems, "mixed", arrivals)
        spent = time.perf_counter() - t0
        if len(systems) < full_count:
            out["extrapolated_full_s"] = {"mixed": full_count / out["mixed"]["solves_per_s"]}
        sub = systems if sample is None else sample
        if left() > 2.5 * spent * len(sub) / len(systems):
            out["fp64"] = served(sub, "fp64", None if sample is not None else arrivals)
            if sample is not None:
                out["fp64_sample"] = sample_note
                out["mixed_on_fp64_sample"] = served(sub, "mixed")
                ref = out["mixed_on_fp64_sample"]["solves_per_s"]
            else:
                ref = out["mixed"]["solves_per_s"]
            out["mixed_over_fp64"] = ref / out["fp64"]["solves_per_s"]
            out.setdefault("extrapolated_full_s", {})["fp64"] = full_count / out["fp64"]["solves_per_s"]
        else:
            out["fp64"] = "skipped: the configs budget left did not cover it"
        return out

    res = {"budget_s": args.configs_budget_s, "server_slots": args.slots, "strict_eps": strict}
    sysd = [W.parametric_diffusion_d10_n32(i) for i in range(256)]
    systems = [(TT([c.to(dev) for c in w["A"]]), TT([c.to(dev) for c in w["b"]]), w["params"]) for w in sysd]
    res["parametric_diffusion_d10_n32"] = pair(
        systems, 256, "all 256 systems", sample=systems[::8],
        sample_note="systems 0, 8, .., 248 of the 256 (rhs ranks across 1-16)")
    if left() > 0.35 * args.configs_budget_s:
        systems = []
        for i in range(8):
            w = W.rounding_stress(i, term_rank=4, nswp=40)
            A = TT([c.to(dev) for c in w["A"]])
            b = TT([c.to(dev) for c in w["b"]]).round(w["round_b"])   # rounded before the clock
            systems.append((A, b, w["params"]))
        res["rounding_stress_d16_n32"] = pair(
            systems, 128, "solves 0-7 of 128 with b = 4 rank-4 terms (rank 16) rounded to 1e-8 on "
                          "the GPU before the timed region, nswp 40")
    if left() > 0.2 * args.configs_budget_s:
        trace = W.serving_trace(16, 2.0, 5)
        systems, arrivals = [], []
        for t_arr, i in trace:
            w = W.serving_request(i, 5)
            systems.append((TT([c.to(dev) for c in w["A"]]), TT([c.to(dev) for c in w["b"]]),
                            w["params"]))
            arrivals.append(t_arr)
        res["serving_trace"] = pair(
            systems, 10000, "the first 16 requests of the seeded trace (seed 5) at 2 requests/s, "
                            "submitted at their arrival times", arrivals)
    res["elapsed_s"] = time.perf_counter() - t_start
    return res


def read_profile_value(name, key):
    """A ``key: value`` line of a committed ncu summary (per-launch DRAM traffic)."""
    try:
        for ln in open(os.path.join(ROOT, "profiles", name)):
            if ln.startswith(key + ":"):
                return float(ln.split(":", 1)[1].split()[0])
    except (OSError, ValueError):
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
    from torchtt_gb300 import TT, _lib, ops
    from torchtt_gb300.serving import Server
    from torchtt_gb300.solvers import solve_cores

    nb = args.batch
    seeds = rank_seeds(args.seed, rank, nb)
    wls = [get_workload(args.workload, s) for s in seeds]
    p = wls[0]["params"]
    kw = dict(nswp=p.get("nswp", 22), eps=p["eps"], kickrank=p["kickrank"])
    A_d = TT([c.to(dev) for c in wls[0]["A"]])
    bs_d = [TT([c.to(dev) for c in w["b"]]) for w in wls]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    engine = args.engine

    srv = Server(slots=args.slots, device=dev)

    strict = args.strict_eps

    def batch(precision, A=A_d, rhs=bs_d):
        ids = [srv.submit(A, b, precision=precision, engine=engine, seed=1000 + j,
                          strict_eps=strict, **kw) for j, b in enumerate(rhs)]
        return [srv.result(i) for i in ids]

    def single(precision, j=0, profile=False):
        return solve_cores(A_d.cores, bs_d[j].cores, precision=precision, engine=engine,
                           seed=1000 + j, profile=profile, stream=stream, strict_eps=strict, **kw)

    # ---- headline: mixed precision, batched through the server --------------------------------
    # one untimed solve of each path alone first: the contraction engine's tile autotuner times its
    # candidates on an otherwise idle GPU, and no tuning run falls inside a timed region
    single("mixed", 0)
    single("fp64", 0)
    for _ in range(args.warmup):
        batch("mixed")
    torch.cuda.synchronize()
    launches0 = _lib.lib().ttgb_launch_count()
    sampler = ClockSampler(local)
    sampler.start()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * args.steps)]
    lat, results = [], None
    for i in range(args.steps):
        flush.fill_(float(i))            # L2 flush between steps (256 MiB > 129 MB L2)
        ev[2 * i].record(stream)
        results = batch("mixed")
        ev[2 * i + 1].record(stream)
        lat.extend(st["queue_ms"] + st["run_ms"] for _, st in results)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    clocks = sampler.stop()
    launches = _lib.lib().ttgb_launch_count() - launches0
    step_ms = [ev[2 * i].elapsed_time(ev[2 * i + 1]) for i in range(args.steps)]
    elapsed_ms = sum(step_ms)
    if ws > 1:
        elapsed_ms = max_over_ranks(elapsed_ms, dist, dev)
    value = ws * nb * args.steps / (elapsed_ms / 1000.0)

    # ---- the plain FP64 path, one solve at a time (the comparison point) ------------------------
    fp64_ms, x_fp64 = [], None
    for j in range(args.fp64_solves):
        flush.fill_(0.5)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        xc, _ = single("fp64", j)
        e1.record(stream)
        torch.cuda.synchronize()
        fp64_ms.append(e0.elapsed_time(e1))
        if j == 0:
            x_fp64 = TT(xc)
    fp64_value = 1000.0 / statistics.mean(fp64_ms)

    # ---- the mixed path unbatched, and the FP64 path batched ------------------------------------
    flush.fill_(0.25)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    xm_c, mixed_stats = single("mixed", 0)
    e1.record(stream)
    torch.cuda.synchronize()
    mixed_single_ms = e0.elapsed_time(e1)
    e0.record(stream)
    fp64_batch = batch("fp64")
    e1.record(stream)
    torch.cuda.synchronize()
    fp64_batch_ms = e0.elapsed_time(e1)

    # ---- accuracy of the timed solutions (TT algebra on the device) -----------------------------
    def relres(x, b):
        return tt_relres_check(A_d.cores, x.cores, b.cores)

    res_mixed = [relres(x, b) for (x, _), b in zip(results, bs_d)]
    res_fp64 = relres(x_fp64, bs_d[0])
    res_fp64_batch = [relres(x, b) for (x, _), b in zip(fp64_batch, bs_d)]
    x_m0 = results[0][0]
    dx = float((x_m0 - x_fp64).norm() / x_fp64.norm())

    # ---- live roofline of the dominant kernels (one profiled solve of each path) ----------------
    peaks = measured_peaks()
    fp64_peak = ops.calibrate_fma("fp64")
    fp32_peak = ops.calibrate_fma("fp32")
    _, pm = single("mixed", 0, profile=True)
    _, pf = single("fp64", 0, profile=True)
    tc = engine in ("auto", "tc")
    # achieved = algorithmic FLOPs of the products (the dense a1 count 2 r n R (r s + n s S + R S),
    # as the reference computes them) / their measured device time; the FLOPs the engine's GEMM
    # launches execute (structured A stage not counted) are reported beside it
    ms = pm["lowp_ms"]
    lowp_tflops = pm["lowp_flops"] / (ms * 1e-3) / 1e12 if ms > 0 else None
    gemm_tflops = pm["lowp_gemm_flops"] / (ms * 1e-3) / 1e12 if ms > 0 else None
    if tc:
        peak = peaks.get("bf16_tflops_sustained") or 1700.0
        roofline = {
            "bound": "tensor", "achieved": lowp_tflops, "peak": peak, "unit": "TFLOP/s",
            "frac": lowp_tflops / peak if lowp_tflops else None,
            "flops": "algorithmic (dense local-product count) per product / product time",
            "gemm_tflops": gemm_tflops,
            "traffic": read_profile_value("tc_gemm_tma_d20_n64_local.md", "traffic_bytes_per_launch"),
            "traffic_source": "profiles/tc_gemm_tma_d20_n64_local.md (one ncu capture of the GEMM "
                              "launches at this workload's largest product, per launch)",
            "kernel": "low-precision local product: tc_gemm_tma_kernel (TMA-fed, warp-specialised "
                      "tcgen05.mma kind::tf32, 3xTF32 split) for its GEMMs + structured A stage + "
                      "operand split",
            "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (of measured)"
                           if "bf16_tflops_sustained" in peaks else "fallback 1.7 PF/s sustained",
            "tf32_pipe_frac": 3 * gemm_tflops / (peak / 2) if gemm_tflops else None,
        }
    else:
        roofline = {
            "bound": "fp32-fma", "achieved": lowp_tflops, "peak": fp32_peak, "unit": "TFLOP/s",
            "frac": lowp_tflops / fp32_peak if lowp_tflops else None, "traffic": None,
            "flops": "algorithmic (dense local-product count) per product / product time",
            "gemm_tflops": gemm_tflops,
            "kernel": "low-precision local product: contract_kernel<float> x3 + casts",
            "peak_source": "FP32 FMA pipe measured live (ttgb_calibrate_fma)",
        }
    roofline.update({
        "launches": pm["lowp_launches"], "ms": pm["lowp_ms"],
        "avg_launch_us": 1000 * pm["lowp_ms"] / max(1, pm["lowp_launches"]),
        "gemm_flops_per_product": pm["lowp_gemm_flops"] / max(1, pm["lowp_matvecs"]),
        "share_of_solve": pm["lowp_ms"] / max(1e-9, sum(pm["phase_ms"].values())),
    })
    fp64_tflops = pf["contract_flops"] / (pf["contract_ms"] * 1e-3) / 1e12 if pf["contract_ms"] > 0 else None
    # Krylov orthogonalisation (three Arnoldi launches per GMRES iteration) against HBM: the
    # reference's algorithmic bytes 8 N_loc (2k + 3) per iteration / the kernels' event time, and
    # the bytes the Arnoldi kernels actually move; the basis (<= 41 vectors of N_loc doubles,
    # ~125 MB at the largest local problem) is mostly L2-resident, so HBM bounds the rate
    kms = pm.get("krylov_ms", 0.0)
    hbm = peaks.get("hbm_gbs") or 6800.0
    kry = {"kernels": "arnoldi_project + arnoldi_reorth + arnoldi_finish per GMRES iteration "
                      "(mixed path)",
           "bound": "hbm", "unit": "GB/s", "peak": hbm,
           "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks
                          else "fallback 6.8 TB/s",
           "achieved": pm["krylov_bytes"] / (kms * 1e-3) / 1e9 if kms > 0 else None,
           "moved_gbs": pm["krylov_traffic_bytes"] / (kms * 1e-3) / 1e9 if kms > 0 else None,
           "moved_over_algorithmic": (pm["krylov_traffic_bytes"] / pm["krylov_bytes"]
                                      if pm.get("krylov_bytes") else None),
           "ms": kms, "launches": pm.get("krylov_launches"),
           "avg_launch_us": 1000 * kms / max(1, pm.get("krylov_launches", 0))}
    kry["frac"] = kry["achieved"] / hbm if kry["achieved"] else None
    fp64_roof = {"kernel": "contract_kernel<double> (FP64 contraction engine, plain path)",
                 "achieved": fp64_tflops, "peak": fp64_peak, "unit": "TFLOP/s",
                 "frac": fp64_tflops / fp64_peak if fp64_tflops else None,
                 "peak_source": "FP64 FMA pipe measured live (ttgb_calibrate_fma)",
                 "traffic": read_profile_value("contract_f64_laplace_potential_d20_n64.md",
                                               "traffic_bytes_per_launch"),
                 "traffic_source": "profiles/contract_f64_laplace_potential_d20_n64.md (one ncu "
                                   "capture, per launch)",
                 "launches": pf["contract_launches"],
                 "avg_launch_us": 1000 * pf["contract_ms"] / max(1, pf["contract_launches"])}

    # the mixed solve's FP64 products (true residuals, interface updates, local right-hand sides)
    # run in double-float on the FP32 pipe: ~12 FP32 operations per FP64 multiply-add (error-free
    # product, two-sum, accumulation), so the pipe's share is (flops / 2) * 12 / FP32 peak
    df_tflops = pm["contract_flops"] / (pm["contract_ms"] * 1e-3) / 1e12 if pm["contract_ms"] > 0 else None
    df_roof = {"kernel": "contract_df_kernel (double-float FP64 products of the mixed path)",
               "achieved": df_tflops, "unit": "TFLOP/s (FP64-equivalent)",
               "fp32_pipe_frac": df_tflops / 2 * 12 / fp32_peak if (df_tflops and fp32_peak) else None,
               "fp32_peak": fp32_peak, "peak_source": "FP32 FMA pipe measured live (ttgb_calibrate_fma)",
               "launches": pm["contract_launches"],
               "avg_launch_us": 1000 * pm["contract_ms"] / max(1, pm["contract_launches"])}

    # ---- end to end through the public API with host-resident inputs -----------------------------
    A_h = TT([c.clone().pin_memory() for c in wls[0]["A"]])
    bs_h = [TT([c.clone().pin_memory() for c in w["b"]]) for w in wls]
    h2d = nb * sum(c.numel() * 8 for c in A_h.cores) + sum(c.numel() * 8 for b in bs_h for c in b.cores)
    e2e_steps = args.steps
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d2h = 0
    for _ in range(e2e_steps):
        out = batch("mixed", A=A_h, rhs=bs_h)
        assert all(x.cores[0].device.type == "cpu" for x, _ in out)
        d2h = sum(c.numel() * 8 for x, _ in out for c in x.cores)
    e2e_s = time.perf_counter() - t0
    if ws > 1:
        e2e_s = max_over_ranks(e2e_s, dist, dev)
    e2e_val = ws * nb * e2e_steps / e2e_s
    srv_stats = srv.stats()
    srv.close()

    configs = run_configs(args, dev, engine, strict) if (rank == 0 and args.configs_budget_s > 0) else None

    # the cost of guaranteeing relres <= eps: one batched step with strict_eps (AMEn at eps / 4)
    strict_line = None
    if rank == 0 and not strict:
        with Server(slots=args.slots, device=dev) as srv2:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ids = [srv2.submit(A_d, b, precision="mixed", engine=engine, seed=1000 + j,
                               strict_eps=True, **kw) for j, b in enumerate(bs_d)]
            out = [srv2.result(i) for i in ids]
            el = time.perf_counter() - t0
        rr = [relres(x, b) for (x, _), b in zip(out, bs_d)]
        strict_line = {"value": nb / el, "unit": "solves/s", "relres_max": max(rr),
                       "relres_pass_frac": sum(1 for v in rr if v <= p["eps"]) / len(rr),
                       "how": "one batched step of the same 16 solves with strict_eps (AMEn run at "
                              "eps / 4 so that the true relres ends <= eps), wall clock"}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        solve_ref, kind, how = reference_solver()
        dt = solve_ref(wls[0])
        cpu = {"value": 1.0 / dt, "unit": "solves/s", "cores": os.cpu_count() or 1, "kind": kind,
               "sample": "1 full solve of %s (b seed %d): %s, threads = all host cores"
                         % (args.workload, seeds[0], how)}

    if rank == 0:
        cfg = arm_config(args, wls[0], ws)
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+tf32" if tc else "f64+f32",
            "data": "synthetic (seeded)", "config": cfg,
            "latency_ms": {"p50": percentile(lat, 0.5), "p99": percentile(lat, 0.99),
                           "requests": len(lat)},
            "fp64_plain": {"value": fp64_value, "unit": "solves/s", "ms_per_solve": statistics.mean(fp64_ms),
                           "solves": len(fp64_ms), "relres": res_fp64},
            "speedup_vs_fp64_plain": value / fp64_value,
            "speedup_vs_fp64_batched": value / (1000.0 * nb / fp64_batch_ms),
            "mixed_single": {"ms_per_solve": mixed_single_ms, "value": 1000.0 / mixed_single_ms,
                             "refinements": mixed_stats["refinements"],
                             "lowp_matvecs": mixed_stats["lowp_matvecs"], "matvecs": mixed_stats["matvecs"]},
            "fp64_batched": {"value": 1000.0 * nb / fp64_batch_ms, "unit": "solves/s", "ms_per_step": fp64_batch_ms},
            "accuracy": {"relres_max": max(res_mixed), "relres_fp64": res_fp64,
                         "relres_fp64_batched_max": max(res_fp64_batch),
                         "relres_pass_frac": sum(1 for v in res_mixed if v <= p["eps"]) / len(res_mixed),
                         "relres_pass_frac_fp64": sum(1 for v in res_fp64_batch if v <= p["eps"]) / len(res_fp64_batch),
                         "x_mixed_vs_fp64": dx, "eps": p["eps"],
                         "stopping": "strict_eps (AMEn at eps/4)" if strict
                                     else "the reference's rule (max local residual < eps)"},
            "solve": {"sweeps": mixed_stats["sweeps"], "max_rank": max(mixed_stats["ranks"]),
                      "gmres_iterations": mixed_stats["gmres_iterations"],
                      "host_syncs": mixed_stats["host_syncs"],
                      "gmres_syncs": mixed_stats.get("gmres_syncs"),
                      "gmres_overrun": mixed_stats.get("gmres_overrun"),
                      "gmres_reorth": mixed_stats.get("gmres_reorth")},
            "server": {"peak_running": srv_stats.get("peak_running"), "completed": srv_stats.get("completed")},
            "roofline": roofline,
            "fp64_contract_roofline": fp64_roof,
            "df_contract_roofline": df_roof,
            "krylov_roofline": kry,
            "phase_ms_mixed": pm["phase_ms"],
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_val, "unit": "solves/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": e2e_steps},
            "gpu_launches": int(launches),
            "clocks": clocks,
            "configs": configs,
            "strict_eps_mixed": strict_line,
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
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--slots", type=int, default=16)
    ap.add_argument("--engine", default="auto", choices=["auto", "tc", "fp32"])
    ap.add_argument("--fp64-solves", type=int, default=2)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--configs-budget-s", type=float, default=360.0,
                    help="wall budget of the batched/served workloads block (0: skip it)")
    ap.add_argument("--strict-eps", action="store_true",
                    help="solve every system to a true relres <= eps (strict_eps: AMEn at eps / 4); "
                         "default: the reference's stopping rule, with the pass fraction reported")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
