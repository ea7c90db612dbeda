"""Solve-level parity of the GPU AMEn path against the reference's own solutions on identical inputs
(tests/golden/solve_*.npz: same A, b, x0 and the same initial enrichment cores z0), and the
reference's own solver tests (tests/test_solvers.py:13-65) rerun through the gb300 backend."""
import numpy as np
import pytest
import torch

import _golden as G
import _parity

pytestmark = pytest.mark.gpu


def to_dev(cores, dev):
    return [torch.from_numpy(np.ascontiguousarray(c)).to(dev) for c in cores]


def _check(z, A, b, xs, p, label, rank_tol=None):
    """Full fixtures: the solution against the reference's cores; sampled fixtures (the benchmark
    workloads at full size): residual, norm, ranks and the sampled estimate of ||x - x_ref||."""
    if G.is_sampled(z):
        _parity.check_sampled(A, b, xs, z, p["eps"], p["kickrank"], label=label, rank_tol=rank_tol)
        return
    cond = _parity.dense_cond(A) if int(np.prod([a.shape[1] for a in A])) <= 2000 else None
    _parity.check(A, b, xs, G.cores(z, "x_cpp"), p["eps"], p["kickrank"], cond=cond, label=label,
                  x_ref_alt=G.cores(z, "x_py"), rank_tol=rank_tol)


@pytest.mark.parametrize("fixture", G.solve_fixtures())
def test_solve_matches_reference(cuda, fixture):
    from torchtt_gb300 import TT, amen_solve
    z = G.load(fixture)
    A, b = G.cores(z, "A"), G.cores(z, "b")
    x0, z0 = G.cores(z, "x0"), G.cores(z, "z0")
    p = G.params(z)
    prec = {0: None, 1: "c", 2: "r"}[int(z["prec"])]
    x, st = amen_solve(TT(to_dev(A, cuda)), TT(to_dev(b, cuda)), nswp=p["nswp"],
                       x0=TT(to_dev(x0, cuda)) if x0 is not None else None, eps=p["eps"],
                       rmax=p["rmax"], max_full=p["max_full"], kickrank=p["kickrank"],
                       kick2=p["kick2"], local_iterations=p["local_iterations"], resets=p["resets"],
                       preconditioner=prec, z0=to_dev(z0, cuda), return_stats=True)
    xs = [c.cpu().numpy() for c in x.cores]
    _check(z, A, b, xs, p, fixture)
    assert st["sweeps"] >= 1 and st["local_solves"] > 0


@pytest.mark.parametrize("prec", [None, "c", "r"])
def test_reference_solver_tests(cuda, prec):
    """tests/test_solvers.py of the reference: random 4x5x6 TT-matrix, b = A x, eps 1e-10,
    relative residual < 5e-8 (nswp 40 for 'r' as in its Python variant)."""
    from torchtt_gb300 import TT, amen_solve, workloads as W
    for seed in range(3):
        wl = W.small_random_system(100 + seed)
        A, b = TT([c.to(cuda) for c in wl["A"]]), TT([c.to(cuda) for c in wl["b"]])
        xx = amen_solve(A, b, eps=1e-10, preconditioner=prec, nswp=40 if prec == "r" else 22,
                        seed=seed + 1)
        err = float((A @ xx - b).norm() / b.norm())
        assert err < 5e-8, (prec, seed, err)


def test_cpu_inputs_roundtrip(cuda):
    """CPU TT in, CPU TT out (the host-buffer path), same answer as device inputs."""
    from torchtt_gb300 import TT, amen_solve, workloads as W
    wl = W.small_random_system(7)
    A, b = TT(wl["A"]), TT(wl["b"])
    x_cpu = amen_solve(A, b, seed=3)
    assert x_cpu.cores[0].device.type == "cpu"
    x_gpu = amen_solve(A.cuda(), b.cuda(), seed=3)
    for c1, c2 in zip(x_cpu.cores, x_gpu.cores):
        assert torch.allclose(c1, c2.cpu(), rtol=0, atol=1e-12 * float(c2.abs().max()))


def test_edge_cases(cuda):
    from torchtt_gb300 import TT, amen_solve, workloads as W
    # d = 1 (a single dense local solve) and d = 2
    for d, n in ((1, 12), (2, 9)):
        A = TT([c.to(cuda) for c in W.laplace_ttm(d, n)])
        b = TT([c.to(cuda) for c in W.random_tt([n] * d, [1] + [2] * (d - 1) + [1], 5)])
        x = amen_solve(A, b, eps=1e-10)
        assert float((A @ x - b).norm() / b.norm()) < 1e-8
    # rank-1 right-hand side and an x0 of higher rank than needed
    A = TT([c.to(cuda) for c in W.laplace_ttm(4, 10)])
    b = TT([c.to(cuda) for c in W.random_tt([10] * 4, [1, 1, 1, 1, 1], 9)])
    x0 = TT([c.to(cuda) for c in W.random_tt([10] * 4, [1, 6, 6, 6, 1], 10)])
    x = amen_solve(A, b, x0=x0, eps=1e-9)
    assert float((A @ x - b).norm() / b.norm()) < 1e-7


@pytest.mark.parametrize("fixture", G.solve_fixtures())
def test_mixed_solve_matches_reference(cuda, fixture):
    """The mixed-precision path meets the same residual and solution bar against the reference's
    FP64 solution. Its ranks are held to 2 kickrank: its stopping test (max local residual < eps)
    can fire a sweep later than the FP64 path's, and a sweep grows a rank by up to kickrank (on
    the d=20 n=64 solve one extra sweep gave ranks up to 9 above the reference's, with a lower
    residual, 2.5e-8 against 3.4e-8)."""
    from torchtt_gb300 import TT, amen_solve
    z = G.load(fixture)
    A, b = G.cores(z, "A"), G.cores(z, "b")
    x0, z0 = G.cores(z, "x0"), G.cores(z, "z0")
    p = G.params(z)
    prec = {0: None, 1: "c", 2: "r"}[int(z["prec"])]
    x, st = amen_solve(TT(to_dev(A, cuda)), TT(to_dev(b, cuda)), nswp=p["nswp"],
                       x0=TT(to_dev(x0, cuda)) if x0 is not None else None, eps=p["eps"],
                       rmax=p["rmax"], max_full=p["max_full"], kickrank=p["kickrank"],
                       kick2=p["kick2"], local_iterations=p["local_iterations"], resets=p["resets"],
                       preconditioner=prec, z0=to_dev(z0, cuda), return_stats=True,
                       precision="mixed")
    xs = [c.cpu().numpy() for c in x.cores]
    _check(z, A, b, xs, p, fixture + " mixed", rank_tol=2 * p["kickrank"])


def test_mixed_equals_fp64_on_laplace(cuda):
    """Mixed and plain FP64 solves of the d=8 n=16 Laplacian agree to the solve tolerance."""
    from torchtt_gb300 import TT, amen_solve, workloads as W
    wl = W.laplace_d8_n16(3)
    A, b = TT([c.to(cuda) for c in wl["A"]]), TT([c.to(cuda) for c in wl["b"]])
    x64, s64 = amen_solve(A, b, eps=1e-10, nswp=20, kickrank=4, seed=5, return_stats=True)
    xmx, smx = amen_solve(A, b, eps=1e-10, nswp=20, kickrank=4, seed=5, return_stats=True,
                          precision="mixed")
    r64 = float((A @ x64 - b).norm() / b.norm())
    rmx = float((A @ xmx - b).norm() / b.norm())
    assert rmx <= max(1e-9, 2 * r64), (rmx, r64)
    assert float((xmx - x64).norm() / x64.norm()) <= 1e-9
    assert smx["lowp_matvecs"] > 0 and smx["refinements"] > 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_structured_a_matches_dense(cuda, precision):
    """The structured A stage (sparse Kronecker-sum cores) and the dense contraction give the same
    solve within the solve tolerance, and both match the reference's solution."""
    from torchtt_gb300 import TT, amen_solve
    z = G.load("solve_laplace_d8_n16.npz")
    A, b = G.cores(z, "A"), G.cores(z, "b")
    x0, z0 = G.cores(z, "x0"), G.cores(z, "z0")
    p = G.params(z)
    At = TT([torch.from_numpy(c).to(cuda) for c in A])
    bt = TT([torch.from_numpy(c).to(cuda) for c in b])
    kw = dict(nswp=p["nswp"], eps=p["eps"], kickrank=p["kickrank"], precision=precision,
              x0=TT([torch.from_numpy(c).to(cuda) for c in x0]),
              z0=[torch.from_numpy(c).to(cuda) for c in z0])
    xs, st = amen_solve(At, bt, return_stats=True, **kw)
    from torchtt_gb300.solvers import solve_cores
    xd, _ = solve_cores(At.cores, bt.cores, kw["x0"].cores, kw["z0"], nswp=p["nswp"], eps=p["eps"],
                        kickrank=p["kickrank"], precision=precision, a_structure=False)
    xd = TT(xd)
    assert float((xs - xd).norm() / xd.norm()) <= 10 * p["eps"]
    _parity.check(A, b, [c.cpu().numpy() for c in xs.cores], G.cores(z, "x_cpp"), p["eps"],
                  p["kickrank"], label="structured " + precision)


@pytest.mark.parametrize("fixture", ["solve_laplace_d8_n16.npz", "solve_random_4x5x6.npz"])
def test_double_float_products_match_native(cuda, fixture):
    """The mixed path's FP64 products in double-float arithmetic on the FP32 pipe (default) give
    the solution of the native-FP64 products within the solve tolerance, and the reference's. The
    two solves share z0 but not every rounding, so their difference is held to the bar of the
    parity checks: 10 eps, or cond(A) (relres_df + relres_native) where the operator can be formed
    (the random 4x5x6 system has cond 2.3e3 and relres ~3 eps at eps 1e-10). Where 1e-13 cond(A)
    exceeds eps, a setting in which the solver never picks double-float by itself, the residual
    bar is the engine's documented 50 eps instead of the reference's."""
    from torchtt_gb300 import TT
    from torchtt_gb300.solvers import solve_cores
    z = G.load(fixture)
    A, b = G.cores(z, "A"), G.cores(z, "b")
    x0, z0 = G.cores(z, "x0"), G.cores(z, "z0")
    p = G.params(z)
    dev = lambda cs: [torch.from_numpy(c).to(cuda) for c in cs] if cs is not None else None
    kw = dict(nswp=p["nswp"], eps=p["eps"], kickrank=p["kickrank"], precision="mixed",
              preconditioner=int(z["prec"]))
    xd, sd = solve_cores(dev(A), dev(b), dev(x0), dev(z0), fp64_engine="df", **kw)
    xn, sn = solve_cores(dev(A), dev(b), dev(x0), dev(z0), fp64_engine="native", **kw)
    from oracle import amen as O
    xdn, xnn = [c.cpu().numpy() for c in xd], [c.cpu().numpy() for c in xn]
    bound = 10 * p["eps"]
    if int(np.prod([a.shape[1] for a in A])) <= 2000:
        bound = max(bound, _parity.dense_cond(A) * (O.tt_relres(A, xdn, b) + O.tt_relres(A, xnn, b)))
    assert float((TT(xd) - TT(xn)).norm() / TT(xn).norm()) <= bound
    cond = _parity.dense_cond(A) if int(np.prod([a.shape[1] for a in A])) <= 2000 else None
    if cond is not None and 1e-13 * cond > p["eps"]:
        # Double-float residuals carry ~1e-13 cond(A) of error, more than eps here (cond 2.3e3 at
        # eps 1e-10 for the random 4x5x6 system): the automatic choice keeps native products below
        # eps 1e-9 for this reason, and a forced double-float solve is held to the 50 eps that the
        # engine documents for this case, with the reference's ranks.
        res = O.tt_relres(A, xdn, b)
        ranks = [c.shape[2] for c in xdn][:-1]
        ranks_ref = [c.shape[2] for c in G.cores(z, "x_cpp")][:-1]
        assert res <= 50 * p["eps"], res
        assert all(abs(a - c) <= p["kickrank"] for a, c in zip(ranks, ranks_ref)), (ranks, ranks_ref)
        return
    _parity.check(A, b, [c.cpu().numpy() for c in xd], G.cores(z, "x_cpp"), p["eps"],
                  p["kickrank"], label="double-float " + fixture, x_ref_alt=G.cores(z, "x_py"))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_strict_eps_reaches_eps(cuda, precision):
    """strict_eps (AMEn at eps / 4) takes the true relative residual of the d=20 n=64 benchmark
    solve to eps, where the reference's own rule on the same input ends at 3.4e-8; the solution
    stays within 10 eps of the reference's (sampled estimate) with ranks >= the reference's."""
    from torchtt_gb300 import TT, amen_solve
    z = G.load("solve_laplace_potential_d20_n64.npz")
    A, b, z0 = G.cores(z, "A"), G.cores(z, "b"), G.cores(z, "z0")
    p = G.params(z)
    x = amen_solve(TT(to_dev(A, cuda)), TT(to_dev(b, cuda)), nswp=p["nswp"], eps=p["eps"],
                   kickrank=p["kickrank"], z0=to_dev(z0, cuda), precision=precision, strict_eps=True)
    xs = [c.cpu().numpy() for c in x.cores]
    from oracle import amen as O
    res = O.tt_relres(A, xs, b)
    err = _parity.sampled_relerr(xs, z)
    assert res <= p["eps"], (precision, res)
    assert err <= 10 * p["eps"], (precision, err)
    assert sum(c.shape[0] for c in xs) >= int(sum(z["ref_ranks"][:-1]))
