"""The AMEn solve as a torch operator: ``torch.ops.torchtt_gb300.amen_solve``.

Schema::

    torchtt_gb300::amen_solve(Tensor[] A, Tensor[] b, Tensor[]? x0=None, int nswp=22,
        float eps=1e-10, int rmax=32768, int max_full=500, int kickrank=4, int kick2=0,
        int local_iterations=40, int resets=2, int preconditioner=0, int precision_mode=0,
        int seed=1) -> (Tensor[] x, Tensor stats)

It takes the core lists and parameters of the reference's native entry point
``torchttcpp.amen_solve`` (``cpp/amen_solve.h:122-139``, registered with pybind at
``cpp/cpp_ext.cpp:7-12``; the mode sizes and ranks that entry point also receives are read from the
cores' shapes here) plus ``precision_mode`` (0 plain FP64, 1 mixed precision) and ``seed`` (the
counter-based RNG of the initial enrichment). It returns the solution cores (new CUDA tensors,
float64) and ``stats``, a float64 vector laid out as ``STATS_FIELDS``.

The operator has a CUDA kernel only: CPU tensors raise (there is no CPU fallback), like the rest of
the package. It is an eager operator: the solution's TT ranks depend on the data, so it has no
shape-propagation (fake) implementation for tracing.
"""
import torch

from . import solvers

STATS_FIELDS = ("sweeps", "converged", "max_res", "local_solves", "gmres_iterations", "matvecs",
                "lowp_matvecs", "refinements", "host_syncs")

SCHEMA = ("amen_solve(Tensor[] A, Tensor[] b, Tensor[]? x0=None, int nswp=22, float eps=1e-10, "
          "int rmax=32768, int max_full=500, int kickrank=4, int kick2=0, int local_iterations=40, "
          "int resets=2, int preconditioner=0, int precision_mode=0, int seed=1) "
          "-> (Tensor[] x, Tensor stats)")

_PRECISION_MODES = {0: "fp64", 1: "mixed"}


def _amen_solve_cuda(A, b, x0=None, nswp=22, eps=1e-10, rmax=32768, max_full=500, kickrank=4,
                     kick2=0, local_iterations=40, resets=2, preconditioner=0, precision_mode=0,
                     seed=1):
    if precision_mode not in _PRECISION_MODES:
        raise ValueError("precision_mode must be 0 (fp64) or 1 (mixed)")
    dev = b[0].device
    prep = lambda cs: [c.detach().to(device=dev, dtype=torch.float64).contiguous() for c in cs]
    x, st = solvers.solve_cores(prep(A), prep(b), prep(x0) if x0 else None, None, nswp=nswp,
                                eps=eps, rmax=rmax, max_full=max_full, kickrank=kickrank,
                                kick2=kick2, local_iterations=local_iterations, resets=resets,
                                preconditioner=preconditioner, seed=seed,
                                precision=_PRECISION_MODES[precision_mode])
    stats = torch.tensor([float(st[k]) for k in STATS_FIELDS], dtype=torch.float64, device=dev)
    return x, stats


def _cpu_rejected(*args, **kwargs):
    raise RuntimeError("torchtt_gb300::amen_solve runs on CUDA tensors only (no CPU fallback)")


_LIB = torch.library.Library("torchtt_gb300", "DEF")
_LIB.define(SCHEMA)
_LIB.impl("amen_solve", _amen_solve_cuda, "CUDA")
_LIB.impl("amen_solve", _cpu_rejected, "CPU")
