"""Command-line solve of a named synthetic workload (also the target of profiler runs).

  python -m torchtt_gb300.run --workload laplace_d8_n16 --solves 1 [--seed 1] [--verbose]

Runs the solves one after another on cuda:0 and prints one line of statistics per solve. It starts
no helper processes, so a profiler attached to it sees only this process's kernels.
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
    args = ap.parse_args()
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


if __name__ == "__main__":
    main()
