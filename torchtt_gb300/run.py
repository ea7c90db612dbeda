"""Command-line solve of a named synthetic workload (also the target of profiler runs).

  python -m torchtt_gb300.run --workload laplace_d8_n16 --solves 1 [--seed 1] [--verbose]
  python -m torchtt_gb300.run --workload parametric_diffusion_d10_n32 --solves 32 --served 8

Runs the solves one after another on cuda:0 and prints one line of statistics per solve; with
``--served K`` it submits all of them at once to a request server with K slots (for the
parametric workload, system i of the batch is the i-th index) and prints one line with the
throughput, the p50/p99 latency and the worst relative residual. It starts no helper processes,
so a profiler attached to it sees only this process's kernels.
"""
import argparse
import json
import time


def main():
    import torch

    from . import workloads as W
    from .solvers import solve_cores
    from .tt import TT

    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="laplace_d8_n16",
                    choices=["laplace_d8_n16", "laplace_potential_d20_n64", "parametric_diffusion_d10_n32"])
    ap.add_argument("--solves", type=int, default=1)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--index", type=int, default=0)
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--profile", action="store_true", help="print the stream time per sweep step")
    ap.add_argument("--engine", default="auto", choices=["auto", "fp32", "tc"],
                    help="low-precision engine of the mixed path")
    ap.add_argument("--no-check", action="store_true",
                    help="skip the relative residual (runs no kernel after the solve)")
    ap.add_argument("--served", type=int, default=0,
                    help="submit all solves at once to a server with this many slots")
    ap.add_argument("--local-product", default=None, metavar="R,S,N,S2,R2",
                    help="run only the low-precision local product (tcgen05 engine) of this shape "
                         "(r, s, n, S, R) with a Laplacian-plus-potential core, --solves times")
    args = ap.parse_args()
    if args.local_product:
        return local_product(args)
    if args.served > 0:
        return served(args)
    if args.workload == "laplace_d8_n16":
        wl = W.laplace_d8_n16(args.seed)
    elif args.workload == "laplace_potential_d20_n64":
        wl = W.laplace_potential_d20_n64(args.seed)
    else:
        wl = W.parametric_diffusion_d10_n32(args.index, args.seed)
    dev = torch.device("cuda", 0)
    A = [c.to(dev) for c in wl["A"]]
    b = [c.to(dev) for c in wl["b"]]
    x0 = [c.to(dev) for c in wl["x0"]] if wl.get("x0") is not None else None
    p = wl["params"]
    for i in range(args.solves):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        x, st = solve_cores(A, b, x0, nswp=p.get("nswp", 22), eps=p["eps"], kickrank=p["kickrank"],
                            seed=args.seed + i, verbose=args.verbose, precision=args.precision,
                            profile=args.profile, engine=args.engine)
        dt = time.perf_counter() - t0
        relres = None if args.no_check else float((TT(A) @ TT(x) - TT(b)).norm() / TT(b).norm())
        if args.profile:
            print(json.dumps({"phase_ms": {k: round(v, 2) for k, v in st["phase_ms"].items()},
                              "host_syncs": st["host_syncs"]}), flush=True)
        print(json.dumps({"solve": i, "seconds": dt, "relres": relres, "sweeps": st["sweeps"],
                          "ranks": st["ranks"], "matvecs": st["matvecs"],
                          "lowp_matvecs": st["lowp_matvecs"], "refinements": st["refinements"],
                          "gmres_iterations": st["gmres_iterations"]}), flush=True)


def local_product(args):
    """The mixed path's low-precision local product alone (a profiler target for its kernels):
    Phi_left, Phi_right and x random, the A core of the d=20 n=64 workload's operator (a middle
    core of the Laplacian plus potential, applied from its nonzeros) when n = 64 and S = 3, a
    random dense core otherwise."""
    import numpy as np
    import torch

    from . import ops, workloads as W

    r, s, n, S, R = (int(v) for v in args.local_product.split(","))
    dev = torch.device("cuda", 0)
    g = np.random.default_rng(args.seed)
    A = (W.laplace_potential_ttm(4, n)[1].numpy() if (s, S) == (3, 3)
         else g.standard_normal((s, n, n, S)))
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    PhiL, PhiR, x = t(g.standard_normal((r, s, r))), t(g.standard_normal((R, S, R))), t(g.standard_normal((r, n, R)))
    Ad = t(A)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.solves):
        y = ops.local_product_lowp(PhiR, PhiL, Ad, x, engine=2)
    torch.cuda.synchronize()
    print(json.dumps({"local_product": [r, s, n, S, R], "repeats": args.solves,
                      "ms_per_product": 1000 * (time.perf_counter() - t0) / args.solves,
                      "norm": float(y.norm())}), flush=True)


def served(args):
    import torch

    from . import workloads as W
    from .serving import Server
    from .tt import TT

    dev = torch.device("cuda", 0)
    systems = []
    for i in range(args.solves):
        if args.workload == "parametric_diffusion_d10_n32":
            wl = W.parametric_diffusion_d10_n32(args.index + i, args.seed)
        elif args.workload == "laplace_d8_n16":
            wl = W.laplace_d8_n16(args.seed + i)
        else:
            wl = W.laplace_potential_d20_n64(args.seed + i)
        systems.append((TT([c.to(dev) for c in wl["A"]]), TT([c.to(dev) for c in wl["b"]]),
                        wl["params"]))
    torch.cuda.synchronize()
    with Server(slots=args.served, device=dev) as srv:
        t0 = time.perf_counter()
        ids = [srv.submit(A, b, precision=args.precision, engine=args.engine, seed=args.seed + i,
                          eps=p["eps"], nswp=p.get("nswp", 22), kickrank=p["kickrank"])
               for i, (A, b, p) in enumerate(systems)]
        res = [srv.result(r) for r in ids]
        elapsed = time.perf_counter() - t0
    lat = sorted(st["queue_ms"] + st["run_ms"] for _, st in res)
    pick = lambda q: lat[min(len(lat) - 1, int(round(q * (len(lat) - 1))))]
    worst = None
    if not args.no_check:
        worst = max(float((A @ x - b).norm() / b.norm()) / p["eps"]
                    for (A, b, p), (x, _) in zip(systems, res))
    print(json.dumps({"workload": args.workload, "solves": args.solves, "slots": args.served,
                      "precision": args.precision, "solves_per_s": args.solves / elapsed,
                      "elapsed_s": elapsed, "latency_ms": {"p50": pick(0.5), "p99": pick(0.99)},
                      "max_rank": max(max(st["ranks"]) for _, st in res),
                      "max_relres_over_eps": worst}), flush=True)


if __name__ == "__main__":
    main()
