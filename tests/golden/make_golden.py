"""Generate the golden fixtures of the AMEn path from the reference itself.

Runs where the reference tree is present (it is read from ``$TORCHTT_REFERENCE``, default
``/root/reference``): the reference's C++ extension is compiled by ``oracle/build_ref.py`` and its
Python package is imported from the tree. Writes ``tests/golden/*.npz``:

* ``kernels.npz`` - inputs and outputs of the reference's local product and the four interface
  updates (``torchtt/solvers.py:36-68,691-775``, the Python twins of ``cpp/amen_solve.h:17-98``) on
  seeded random shapes, plus a GMRES known answer (``torchtt/_iterative_solvers.py:72-158`` on a
  1-D Laplacian, the pattern of ``cpp/test_gmres.cpp:187-253``);
* ``round.npz`` - inputs and outputs of the reference's TT rounding (``TT.round``);
* ``divide.npz`` - inputs and outputs of the reference's elementwise division (``amen_divide``);
* ``dmrg.npz`` - inputs and outputs of the reference's C++ DMRG matvec (``dmrg_mv``);
* ``amen_mv.npz`` - inputs and outputs of the reference's AMEn matvec and matmat;
* ``solve_<name>.npz`` - the inputs of a whole solve (A, b, x0 cores, the initial enrichment cores z0
  that the reference drew with ``torch::randn`` after ``torch.manual_seed``), the parameters, and the
  solution cores returned by ``torchttcpp.amen_solve`` (``cpp/amen_solve.h:122``) and, for the small
  cases, by the Python path ``_amen_solve_python`` (``torchtt/solvers.py:290``).

Usage: ``python tests/golden/make_golden.py``
"""
import os
import sys
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_ref  # noqa: E402
from torchtt_gb300 import workloads as W  # noqa: E402


def _pack_cores(prefix, cores, out):
    out[prefix + "_n"] = np.array(len(cores))
    for i, c in enumerate(cores):
        out["%s_%d" % (prefix, i)] = np.ascontiguousarray(c.numpy() if torch.is_tensor(c) else c)


def kernels(torchtt):
    from torchtt import solvers as S
    from torchtt import _iterative_solvers as IS
    g = np.random.Generator(np.random.PCG64(7))
    out = {}
    cases = [(3, 5, 4, 2, 3), (7, 6, 9, 3, 2), (12, 16, 10, 2, 2), (1, 8, 5, 1, 3)]
    for ci, (r, n, R, s, S_) in enumerate(cases):
        PhiL = g.standard_normal((r, s, r))
        PhiR = g.standard_normal((R, S_, R))
        Ak = g.standard_normal((s, n, n, S_))
        x = g.standard_normal((r, n, R))
        t = lambda a: torch.from_numpy(a)
        y = S._local_product(t(PhiR), t(PhiL), t(Ak), t(x), x.shape)
        # interface updates: x core of shape r x n x R, z core rz x n x Rz
        rz, Rz = max(1, r // 2), max(1, R // 2)
        z = g.standard_normal((rz, n, Rz))
        Pf = g.standard_normal((rz, s, r))          # Phi for (z, x): rz x s x r
        Pb = g.standard_normal((Rz, S_, R))
        rb, Rb = 2, 3
        bk = g.standard_normal((rb, n, Rb))
        Pbf = g.standard_normal((rb, r))
        Pbb = g.standard_normal((Rb, R))
        fwdA = S._compute_phi_fwd_A(t(Pf), t(z), t(Ak), t(x))
        bckA = S._compute_phi_bck_A(t(Pb), t(z), t(Ak), t(x))
        fwdb = S._compute_phi_fwd_rhs(t(Pbf), t(bk), t(x))
        bckb = S._compute_phi_bck_rhs(t(Pbb), t(bk), t(x))
        for k, v in dict(PhiL=PhiL, PhiR=PhiR, A=Ak, x=x, y=y.numpy(), z=z, Pf=Pf, Pb=Pb, bk=bk,
                         Pbf=Pbf, Pbb=Pbb, fwdA=fwdA.numpy(), bckA=bckA.numpy(),
                         fwdb=fwdb.numpy(), bckb=bckb.numpy()).items():
            out["c%d_%s" % (ci, k)] = np.ascontiguousarray(v)
    out["ncases"] = np.array(len(cases))

    # GMRES known answer on the 1-D Laplacian (-1 2 -1), rhs = ones with zero ends
    n = 200
    L = 2 * np.eye(n) - np.eye(n, k=1) - np.eye(n, k=-1)

    class Op:
        def matvec(self, v):
            return torch.reshape(torch.from_numpy(L) @ torch.reshape(v, [-1, 1]), [-1, 1])
    rhs = np.ones((n, 1))
    rhs[0, 0] = rhs[-1, 0] = 0.0
    xg, flag, nit = IS.gmres_restart(Op(), torch.from_numpy(rhs), torch.zeros((n, 1), dtype=torch.float64),
                                     n, 40, 1e-10, 4)
    out["gmres_L"] = L
    out["gmres_rhs"] = rhs[:, 0]
    out["gmres_x"] = xg.numpy()[:, 0]
    out["gmres_flag"] = np.array(int(flag))
    out["gmres_nit"] = np.array(int(nit))
    np.savez_compressed(os.path.join(HERE, "kernels.npz"), **out)
    print("kernels.npz written")


def rounding(torchtt):
    """TT rounding by the reference's ``TT.round`` (torchtt/_tt_base.py:1427-1450) on inputs with
    decaying and with flat rank spectra, a rank cap, a TT-matrix and d = 1."""
    def wsum(N, r, seed, weights):
        acc = None
        for i, w in enumerate(weights):
            t = torchtt.TT(W.random_tt(N, [1] + [r] * (len(N) - 1) + [1], seed + i)) * w
            acc = t if acc is None else acc + t
        return acc
    decay = wsum([5] * 6, 6, 31, [1.0, 1e-3, 1e-6, 1e-9])
    flat = wsum([6] * 8, 16, 41, [1.0, 1.0, 1.0, 1.0])
    lap = torchtt.TT(W.laplace_ttm(4, 5))
    cases = [("decay_eps1e-7", decay, 1e-7, 2 ** 62), ("decay_rmax7", decay, 1e-12, 7),
             ("flat_eps1e-8", flat, 1e-8, 2 ** 62), ("ttm_sum", lap + lap, 1e-12, 2 ** 62),
             ("d1", torchtt.TT(W.random_tt([9], [1, 1], 51)), 1e-8, 2 ** 62)]
    out = {"names": np.array([c[0] for c in cases])}
    for name, x, eps, rmax in cases:
        y = x.round(eps, rmax)
        _pack_cores(name + "_in", x.cores, out)
        _pack_cores(name + "_out", y.cores, out)
        out[name + "_eps"] = np.array(eps)
        out[name + "_rmax"] = np.array(rmax, dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "round.npz"), **out)
    print("round.npz written")


def division(torchtt):
    """Elementwise division by the reference's amen_divide (torchtt/_division.py:76): a = 1 + a
    small random TT (no zeros), b random; the reference's own random start is not recorded (its z
    cores come from the global torch RNG), so parity is on the solution."""
    from torchtt._division import amen_divide
    out = {}
    cases = [("d3", [6, 7, 8], [1, 2, 2, 1], [1, 3, 3, 1]), ("d6", [8] * 6, [1] + [2] * 5 + [1], [1] + [3] * 5 + [1])]
    for name, N, Ra, Rb in cases:
        d = len(N)
        one = torchtt.TT([torch.ones((1, n, 1), dtype=torch.float64) for n in N])
        a = one + torchtt.TT(W.random_tt(N, Ra, 71 + d)) * 0.5
        b = torchtt.TT(W.random_tt(N, Rb, 81 + d))
        torch.manual_seed(3)
        x = amen_divide(a, b, nswp=22, eps=1e-10, verbose=False)
        _pack_cores(name + "_a", a.cores, out)
        _pack_cores(name + "_b", b.cores, out)
        _pack_cores(name + "_x", x, out)
    out["names"] = np.array([c[0] for c in cases])
    np.savez_compressed(os.path.join(HERE, "divide.npz"), **out)
    print("divide.npz written")


def dmrg(cpp):
    """The reference's C++ DMRG matvec (torchttcpp.dmrg_mv, cpp/dmrg_mv.h:23) on a Laplacian and a
    Laplacian-plus-potential operator; the random start and kicks come from the global torch RNG
    (seeded here, not replayable elsewhere), so parity is on the product."""
    out = {}
    cases = [("lap", W.laplace_ttm(5, 6), [6] * 5, [1, 3, 3, 3, 3, 1], 21),
             ("pot", W.laplace_potential_ttm(4, 8), [8] * 4, [1, 4, 4, 4, 1], 22)]
    for name, A, N, R, seed in cases:
        x = W.random_tt(N, R, seed)
        torch.manual_seed(seed)
        y = cpp.dmrg_mv(A, x, [], N, N, R, [], 20, 1e-12, 32768, 4, False)
        _pack_cores(name + "_A", A, out)
        _pack_cores(name + "_x", x, out)
        _pack_cores(name + "_y", y, out)
    out["names"] = np.array([c[0] for c in cases])
    np.savez_compressed(os.path.join(HERE, "dmrg.npz"), **out)
    print("dmrg.npz written")


def amen_products(torchtt):
    """The reference's AMEn matvec and matmat (torchtt.amen_mv / amen_mm, torchtt/_amen.py:55-125)
    on a Laplacian-plus-potential operator; their random z cores come from the global torch RNG
    (seeded here), so parity is on the product."""
    out = {}
    A = W.laplace_potential_ttm(5, 8)
    x = W.random_tt([8] * 5, [1, 3, 3, 3, 3, 1], 31)
    torch.manual_seed(31)
    y = torchtt.amen_mv(torchtt.TT(A), torchtt.TT(x), eps=1e-10)
    _pack_cores("mv_A", A, out)
    _pack_cores("mv_b", x, out)
    _pack_cores("mv_y", y.cores, out)
    B = W.laplace_ttm(4, 6)
    A2 = W.laplace_potential_ttm(4, 6)
    torch.manual_seed(32)
    Y = torchtt.amen_mm(torchtt.TT(A2), torchtt.TT(B), eps=1e-10)
    _pack_cores("mm_A", A2, out)
    _pack_cores("mm_B", B, out)
    _pack_cores("mm_Y", Y.cores, out)
    np.savez_compressed(os.path.join(HERE, "amen_mv.npz"), **out)
    print("amen_mv.npz written")


def solve_case(torchtt, cpp, wl, seed, prec=None, with_python=False, extra=None):
    A, b, x0 = wl["A"], wl["b"], wl.get("x0")
    p = dict(nswp=22, eps=1e-10, rmax=32768, max_full=500, kickrank=4, kick2=0,
             local_iterations=40, resets=2)
    p.update(wl["params"])
    if extra:
        p.update(extra)
    d = len(A)
    N = [c.shape[2] for c in A]
    rA = [1] + [c.shape[3] for c in A]
    rb = [1] + [c.shape[2] for c in b]
    x_cores = list(x0) if x0 is not None else []
    rx = ([1] + [c.shape[2] for c in x0]) if x0 is not None else [1] * (d + 1)
    precode = {None: 0, "c": 1, "r": 2}[prec]
    torch.manual_seed(seed)
    rz = [1] + [p["kickrank"] + p["kick2"]] * (d - 1) + [1]
    z0 = [torch.randn(rz[i], N[i], rz[i + 1], dtype=torch.float64) for i in range(d)]
    torch.manual_seed(seed)
    t0 = time.time()
    xr = cpp.amen_solve(A, b, x_cores, N, rA, rb, rx, p["nswp"], p["eps"], p["rmax"], p["max_full"],
                        p["kickrank"], p["kick2"], p["local_iterations"], p["resets"], False, precode)
    t_cpp = time.time() - t0
    out = {}
    _pack_cores("A", A, out)
    _pack_cores("b", b, out)
    if x0 is not None:
        _pack_cores("x0", x0, out)
    _pack_cores("z0", z0, out)
    _pack_cores("x_cpp", xr, out)
    for k, v in p.items():
        out["p_" + k] = np.array(v)
    out["prec"] = np.array(precode)
    out["seed"] = np.array(seed)
    out["t_cpp"] = np.array(t_cpp)
    out["threads"] = np.array(torch.get_num_threads())
    if with_python:
        from torchtt import solvers as S
        torch.manual_seed(seed)
        x0tt = torchtt.TT(list(x0)) if x0 is not None else None
        xp = S.amen_solve(torchtt.TT(list(A)), torchtt.TT(list(b)), nswp=p["nswp"], x0=x0tt, eps=p["eps"],
                          kickrank=p["kickrank"], preconditioner=prec, use_cpp=False)
        _pack_cores("x_py", xp.cores, out)
    name = wl["name"] + ("" if prec is None else "_prec_" + prec)
    np.savez_compressed(os.path.join(HERE, "solve_%s.npz" % name), **out)
    print("solve_%s.npz written (cpp %.2fs)" % (name, t_cpp))


def tt_entries(cores, idx):
    """Entries x(i_1, .., i_d) of a TT-vector at the rows of ``idx`` (S x d), by a batched chain of
    row-vector x core-slice products."""
    cores = [c.numpy() if torch.is_tensor(c) else np.asarray(c) for c in cores]
    v = cores[0][0, idx[:, 0], :]                                  # S x r1
    for k in range(1, len(cores)):
        sl = np.transpose(cores[k][:, idx[:, k], :], (1, 0, 2))    # S x r x R
        v = np.einsum("sr,srR->sR", v, sl)
    return v[:, 0]


def sampled_case(torchtt, cpp, wl, seed, name, nsamples=4096):
    """A whole solve at a size whose solution is too large to store (tens of MB at d = 20): the
    inputs, the parameters, the initial enrichment cores z0 that the reference draws with
    ``torch::randn`` after ``torch.manual_seed(seed)``, and a summary of the solution
    ``torchttcpp.amen_solve`` (``cpp/amen_solve.h:122``) returns:

    * its TT ranks and Frobenius norm, and its relative residual ||A x - b|| / ||b|| (oracle TT
      algebra);
    * its entries at ``nsamples`` multi-indices drawn uniformly from the full index space. For a
      second solution y of the same system, N mean_i (y(i) - x(i))^2 is an unbiased estimate of
      ||y - x||^2 (N the number of entries), so the sampled root-mean-square difference over the
      sampled root-mean-square of x estimates ||y - x|| / ||x|| without storing x."""
    from oracle import amen as O
    A, b, x0 = wl["A"], wl["b"], wl.get("x0")
    p = dict(nswp=22, eps=1e-10, rmax=32768, max_full=500, kickrank=4, kick2=0,
             local_iterations=40, resets=2)
    p.update(wl["params"])
    d = len(A)
    N = [c.shape[2] for c in A]
    rA = [1] + [c.shape[3] for c in A]
    rb = [1] + [c.shape[2] for c in b]
    torch.manual_seed(seed)
    rz = [1] + [p["kickrank"] + p["kick2"]] * (d - 1) + [1]
    z0 = [torch.randn(rz[i], N[i], rz[i + 1], dtype=torch.float64) for i in range(d)]
    torch.manual_seed(seed)
    t0 = time.time()
    xr = cpp.amen_solve(A, b, [], N, rA, rb, [1] * (d + 1), p["nswp"], p["eps"], p["rmax"],
                        p["max_full"], p["kickrank"], p["kick2"], p["local_iterations"],
                        p["resets"], False, 0)
    t_cpp = time.time() - t0
    xs = [c.numpy() for c in xr]
    An, bn = [c.numpy() for c in A], [c.numpy() for c in b]
    g = np.random.Generator(np.random.PCG64(seed + 9176))
    idx = np.stack([g.integers(0, n, size=nsamples) for n in N], axis=1).astype(np.int64)
    out = {}
    _pack_cores("A", A, out)
    _pack_cores("b", b, out)
    _pack_cores("z0", z0, out)
    for k, v in p.items():
        out["p_" + k] = np.array(v)
    out["prec"] = np.array(0)
    out["seed"] = np.array(seed)
    out["t_cpp"] = np.array(t_cpp)
    out["threads"] = np.array(torch.get_num_threads())
    out["ref_ranks"] = np.array([c.shape[0] for c in xs] + [1], dtype=np.int64)
    out["ref_norm"] = np.array(O.tt_norm(xs))
    out["ref_relres"] = np.array(O.tt_relres(An, xs, bn))
    out["sample_idx"] = idx.astype(np.uint8 if max(N) <= 256 else np.int32)
    out["sample_x"] = tt_entries(xs, idx)
    np.savez_compressed(os.path.join(HERE, "solve_%s.npz" % name), **out)
    print("solve_%s.npz written (cpp %.2fs, ranks <= %d, relres %.3e)"
          % (name, t_cpp, max(out["ref_ranks"]), float(out["ref_relres"])), flush=True)


def rounding_case(torchtt, cpp):
    """Rounding stress d=16 n=32 (A = Laplacian + C C^T + I), the right-hand side (a sum of 4
    random TTs) rounded to 1e-8 by the reference's own TT.round (torchtt/_tt_base.py:1427) before
    the solve. With the full terms of rank 16 (input rank 64) the reference's solve stops after 20
    sweeps at relres 0.70 with ranks <= 161 (AMEn grows a rank by at most kickrank per sweep, and
    this solution needs far more), so the fixture uses terms of rank 4 (input rank 16) and nswp 40,
    where it converges."""
    wl = W.rounding_stress(0, term_rank=4, nswp=40)
    bt = torchtt.TT(list(wl["b"])).round(wl["round_b"])
    wl = dict(wl, b=[c.contiguous() for c in bt.cores])
    sampled_case(torchtt, cpp, wl, 40, "rounding_stress_d16_n32_sys0_r16")


def large_solves(torchtt, cpp):
    """Sampled fixtures of the benchmark workloads at their full sizes: the d=20 n=64 solve of the
    benchmark (its first right-hand side), one system of each batch workload, and two requests of
    the serving trace."""
    sampled_case(torchtt, cpp, W.laplace_potential_d20_n64(2), 2, "laplace_potential_d20_n64")
    # parametric diffusion d=10 n=32: system 13 (rhs rank 1) and system 3 (rhs rank 15)
    for i in (13, 3):
        wl = W.parametric_diffusion_d10_n32(i)
        sampled_case(torchtt, cpp, wl, 30 + i, "parametric_diffusion_d10_n32_sys%d_r%d" % (i, wl["rhs_rank"]))
    rounding_case(torchtt, cpp)
    # serving trace requests: 44 (d=24, n=64, rank 8, eps 1e-8), 14 (d=20, n=32, rank 5, eps 1e-10)
    for i in (44, 14):
        wl = W.serving_request(i)
        sampled_case(torchtt, cpp, wl, 50 + i, "serving_req%d_d%d_n%d" % (i, wl["d"], wl["n"]))


def main():
    torch.set_num_threads(max(1, os.cpu_count() or 1))
    torchtt, cpp = build_ref.load_reference_package()
    if len(sys.argv) > 1 and sys.argv[1] == "large":
        large_solves(torchtt, cpp)
        return
    if len(sys.argv) > 1 and sys.argv[1] == "rounding":
        rounding_case(torchtt, cpp)
        return
    kernels(torchtt)
    rounding(torchtt)
    division(torchtt)
    dmrg(cpp)
    amen_products(torchtt)
    small = W.small_random_system(0)
    for prec in (None, "c", "r"):
        solve_case(torchtt, cpp, small, seed=11, prec=prec, with_python=True,
                   extra=dict(nswp=40) if prec == "r" else None)
    solve_case(torchtt, cpp, W.laplace_d8_n16(1), seed=1, with_python=False)
    # a mid-size Laplacian with a direct-solver end core and GMRES interior cores
    lap = dict(name="laplace_d5_n12", A=W.laplace_ttm(5, 12),
               b=W.random_tt([12] * 5, [1, 3, 3, 3, 3, 1], 5), x0=None,
               params=dict(eps=1e-9, nswp=20, kickrank=4))
    solve_case(torchtt, cpp, lap, seed=5, with_python=True)


if __name__ == "__main__":
    main()
