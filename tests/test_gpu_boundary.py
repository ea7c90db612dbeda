"""The drop-in boundary exercised from the reference's side:

* the ctypes stub of ``torchttcpp.amen_solve`` printed in INTEGRATION.md section 2, executed as
  written there, against the reference's solution of its own test system;
* a foreign TT class that has only ``.cores`` and ``.is_ttm`` (the duck typing of
  ``torchtt_gb300.amen_solve``) goes in and the same class comes out;
* the torch operator ``torch.ops.torchtt_gb300.amen_solve`` (the torch-level twin of
  ``torchttcpp.amen_solve``, cpp/cpp_ext.cpp:7-12) gives the solution of the Python entry point.
"""
import os
import re

import numpy as np
import pytest
import torch

import _golden as G
import _parity

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _integration_stub():
    """The Python block of INTEGRATION.md section 2, compiled as written."""
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    sec = text.split("## 2.", 1)[1].split("\n## ", 1)[0]
    code = re.search(r"```python\n(.*?)```", sec, re.S).group(1)
    ns = {}
    exec(compile(code, "INTEGRATION.md#2", "exec"), ns)
    return ns["torchttcpp_amen_solve"]


def test_integration_stub_runs_as_documented(cuda):
    stub = _integration_stub()
    z = G.load("solve_random_4x5x6.npz")
    A, b = G.cores(z, "A"), G.cores(z, "b")
    p = G.params(z)
    Ad = [torch.from_numpy(c).to(cuda) for c in A]
    bd = [torch.from_numpy(c).to(cuda) for c in b]
    N = [c.shape[2] for c in A]
    rA = [1] + [c.shape[3] for c in A]
    rb = [1] + [c.shape[2] for c in b]
    x = stub(Ad, bd, [], N, rA, rb, [1] * (len(A) + 1), p["nswp"], p["eps"], p["rmax"],
             p["max_full"], p["kickrank"], p["kick2"], p["local_iterations"], p["resets"], False, 0)
    xs = [c.cpu().numpy() for c in x]
    # the stub passes no z0, so the random start differs from the reference's: the bar is the
    # solve tolerance with the operator's condition number (formed densely, 120 x 120)
    _parity.check(A, b, xs, G.cores(z, "x_cpp"), p["eps"], p["kickrank"],
                  cond=_parity.dense_cond(A), label="INTEGRATION.md stub", x_ref_alt=G.cores(z, "x_py"))


class BareTT:
    """A TT class of another library: cores and the matrix flag, nothing else."""

    def __init__(self, cores):
        self.cores = list(cores)
        self.is_ttm = self.cores[0].dim() == 4


def test_foreign_tt_class_roundtrip(cuda):
    from torchtt_gb300 import TT, amen_solve, workloads as W
    wl = W.small_random_system(3)
    A = BareTT([c.to(cuda) for c in wl["A"]])
    b = BareTT([c.to(cuda) for c in wl["b"]])
    x = amen_solve(A, b, eps=1e-10, seed=2)
    assert type(x) is BareTT and not x.is_ttm
    xt = TT(x.cores)
    At, bt = TT(A.cores), TT(b.cores)
    assert float((At @ xt - bt).norm() / bt.norm()) < 1e-8
    # the same answer as the package's own TT class
    y = amen_solve(At, bt, eps=1e-10, seed=2)
    assert float((y - xt).norm() / y.norm()) <= 1e-12


@pytest.mark.parametrize("precision_mode", [0, 1])
def test_torch_operator(cuda, precision_mode):
    import torchtt_gb300  # noqa: F401  (registers the operator)
    from torchtt_gb300 import TT, custom_op
    from torchtt_gb300.solvers import solve_cores
    z = G.load("solve_laplace_d8_n16.npz")
    A = [torch.from_numpy(c).to(cuda) for c in G.cores(z, "A")]
    b = [torch.from_numpy(c).to(cuda) for c in G.cores(z, "b")]
    x0 = [torch.from_numpy(c).to(cuda) for c in G.cores(z, "x0")]
    p = G.params(z)
    x, stats = torch.ops.torchtt_gb300.amen_solve(A, b, x0, nswp=p["nswp"], eps=p["eps"],
                                                  kickrank=p["kickrank"],
                                                  precision_mode=precision_mode, seed=4)
    assert stats.dtype == torch.float64 and stats.numel() == len(custom_op.STATS_FIELDS)
    st = dict(zip(custom_op.STATS_FIELDS, stats.tolist()))
    assert st["sweeps"] >= 1 and st["converged"] == 1
    y, _ = solve_cores(A, b, x0, None, nswp=p["nswp"], eps=p["eps"], kickrank=p["kickrank"],
                       precision="mixed" if precision_mode else "fp64", seed=4)
    # the same solve twice: equal up to the order of split-K partial sums (atomics), far below the
    # solve tolerance
    assert float((TT(x) - TT(y)).norm() / TT(y).norm()) <= 10 * p["eps"]
    _parity.check(G.cores(z, "A"), G.cores(z, "b"), [c.cpu().numpy() for c in x],
                  G.cores(z, "x_cpp"), p["eps"], p["kickrank"], label="torch operator")
