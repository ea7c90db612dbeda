"""Seeded synthetic AMEn workloads: TT-matrix operators, right-hand sides and initial guesses.

All values are float64 and are drawn with numpy ``Generator(PCG64(seed))`` so that the same seed gives
the same cores on every platform. Cores are returned as CPU ``torch.float64`` tensors in the reference's
layouts: TT-matrix cores ``r x m x n x r'`` and TT-vector cores ``r x n x r'``
(reference: ``torchtt/_tt_base.py:138-145``).

Operators:

* ``laplace_ttm``: the Kronecker sum ``sum_k I x .. x L_k x .. x I`` of 1-D operators ``L_k``, TT rank 2
  (the construction the reference's examples build with ``**`` and ``+``,
  ``examples/system_solvers.py:30-46``);
* ``laplace_potential_ttm``: that sum plus a rank-1 product potential ``V x V x .. x V``, TT rank 3;
* ``laplace_lowrank_spd_ttm``: the Kronecker sum plus ``C C^T`` for a random TT-matrix ``C`` plus the
  identity (an SPD operator of TT rank up to 2 + rank(C)^2 + 1).
"""
import math

import numpy as np
import torch


def _rng(seed):
    return np.random.Generator(np.random.PCG64(int(seed)))


def laplace_1d(n, scale=None):
    """``(n+1)^2 * tridiag(-1, 2, -1)`` (n x n), the 1-D Dirichlet finite-difference Laplacian."""
    if scale is None:
        scale = float((n + 1) ** 2)
    L = 2.0 * np.eye(n) - np.eye(n, k=1) - np.eye(n, k=-1)
    return scale * L


def potential_1d(n):
    """``diag(1 + 0.5 cos(2 pi i / n))``, i = 0..n-1."""
    i = np.arange(n)
    return np.diag(1.0 + 0.5 * np.cos(2.0 * math.pi * i / n))


def _to_torch(cores):
    return [torch.from_numpy(np.ascontiguousarray(c, dtype=np.float64)) for c in cores]


def kron_sum_cores(mats):
    """TT-matrix cores (rank 2) of ``sum_k I x .. x mats[k] x .. x I``."""
    d = len(mats)
    if d == 1:
        return [mats[0][None, :, :, None].copy()]
    cores = []
    for k, L in enumerate(mats):
        n = L.shape[0]
        I = np.eye(n)
        if k == 0:
            c = np.zeros((1, n, n, 2))
            c[0, :, :, 0] = I          # state 0: no term applied yet
            c[0, :, :, 1] = L          # state 1: the term has been applied
        elif k == d - 1:
            c = np.zeros((2, n, n, 1))
            c[0, :, :, 0] = L
            c[1, :, :, 0] = I
        else:
            c = np.zeros((2, n, n, 2))
            c[0, :, :, 0] = I
            c[0, :, :, 1] = L
            c[1, :, :, 1] = I
        cores.append(c)
    return cores


def laplace_ttm(d, n, coeffs=None):
    """Kronecker-sum Laplacian, TT rank 2; ``coeffs[k]`` scales the k-th 1-D term (default 1)."""
    if coeffs is None:
        coeffs = [1.0] * d
    return _to_torch(kron_sum_cores([float(c) * laplace_1d(n) for c in coeffs]))


def laplace_potential_ttm(d, n):
    """``sum_k L_k + V x .. x V`` with ``V = diag(1 + 0.5 cos(2 pi i/n))``, TT rank 3."""
    L = laplace_1d(n)
    V = potential_1d(n)
    I = np.eye(n)
    cores = []
    for k in range(d):
        if k == 0:
            c = np.zeros((1, n, n, 3))
            c[0, :, :, 0] = I
            c[0, :, :, 1] = L
            c[0, :, :, 2] = V
        elif k == d - 1:
            c = np.zeros((3, n, n, 1))
            c[0, :, :, 0] = L
            c[1, :, :, 0] = I
            c[2, :, :, 0] = V
        else:
            c = np.zeros((3, n, n, 3))
            c[0, :, :, 0] = I
            c[0, :, :, 1] = L
            c[1, :, :, 1] = I
            c[2, :, :, 2] = V
        cores.append(c)
    return _to_torch(cores)


def _ttm_add(a, b):
    """Sum of two TT-matrices by block concatenation of their cores."""
    d = len(a)
    out = []
    for k in range(d):
        x, y = a[k], b[k]
        if k == 0:
            out.append(np.concatenate([x, y], axis=3))
        elif k == d - 1:
            out.append(np.concatenate([x, y], axis=0))
        else:
            c = np.zeros((x.shape[0] + y.shape[0], x.shape[1], x.shape[2], x.shape[3] + y.shape[3]))
            c[:x.shape[0], :, :, :x.shape[3]] = x
            c[x.shape[0]:, :, :, x.shape[3]:] = y
            out.append(c)
    return out


def laplace_lowrank_spd_ttm(d, n, seed, rank_c=2, sigma=0.01):
    """``L + C C^T + I``: Kronecker-sum Laplacian, plus ``C C^T`` for a random TT-matrix ``C`` of rank
    ``rank_c`` with N(0, sigma^2) cores (symmetric positive semi-definite, TT rank rank_c^2), plus I."""
    g = _rng(seed)
    lap = kron_sum_cores([laplace_1d(n)] * d)
    rc = [1] + [rank_c] * (d - 1) + [1]
    C = [sigma * g.standard_normal((rc[k], n, n, rc[k + 1])) for k in range(d)]
    # (C C^T)[i,j] = sum_l C[i,l] C[j,l]: core-wise Kronecker product of C and C^T
    P = []
    for c in C:
        ct = c.transpose(0, 2, 1, 3)
        p = np.einsum("aimb,cjmd->acijbd", c, ct)
        P.append(p.reshape(c.shape[0] * c.shape[0], n, n, c.shape[3] * c.shape[3]))
    eye = [np.eye(n)[None, :, :, None] for _ in range(d)]
    return _to_torch(_ttm_add(_ttm_add(lap, P), eye))


def random_tt(N, R, seed, normalise=True):
    """Random TT-vector with iid N(0,1) cores, ranks ``R`` (len(N)+1 entries, R[0]=R[-1]=1).

    With ``normalise`` the cores are scaled equally so that the tensor has unit Frobenius norm."""
    g = _rng(seed)
    d = len(N)
    cores = [g.standard_normal((R[k], N[k], R[k + 1])) for k in range(d)]
    if normalise:
        nrm = _tt_norm_np(cores)
        f = nrm ** (-1.0 / d)
        cores = [c * f for c in cores]
    return _to_torch(cores)


def _tt_norm_np(cores):
    cur = None
    for c in cores:
        if cur is not None:
            c = np.tensordot(cur, c, axes=([1], [0]))
        _, cur = np.linalg.qr(c.reshape(-1, c.shape[2]))
    return float(abs(cur.reshape(-1)[0]))


def tt_sum(list_of_cores):
    """Sum of TT-vectors by block concatenation (ranks add)."""
    acc = [c.numpy() for c in list_of_cores[0]]
    d = len(acc)
    for other in list_of_cores[1:]:
        o = [c.numpy() for c in other]
        new = []
        for k in range(d):
            x, y = acc[k], o[k]
            if k == 0:
                new.append(np.concatenate([x, y], axis=2))
            elif k == d - 1:
                new.append(np.concatenate([x, y], axis=0))
            else:
                c = np.zeros((x.shape[0] + y.shape[0], x.shape[1], x.shape[2] + y.shape[2]))
                c[:x.shape[0], :, :x.shape[2]] = x
                c[x.shape[0]:, :, x.shape[2]:] = y
                new.append(c)
        acc = new
    return _to_torch(acc)


# ------------------------------------------------------------------------------------------------
# the named workloads
# ------------------------------------------------------------------------------------------------

def laplace_d8_n16(seed=1):
    """d=8, n=16 Kronecker-sum Laplacian (rank 2); b rank 4 N(0,1), ||b||=1; x0 rank 2 N(0,1);
    eps 1e-10, nswp 20, kickrank 4."""
    d, n = 8, 16
    A = laplace_ttm(d, n)
    b = random_tt([n] * d, [1] + [4] * (d - 1) + [1], seed)
    x0 = random_tt([n] * d, [1] + [2] * (d - 1) + [1], seed + 1000, normalise=False)
    return dict(name="laplace_d8_n16", A=A, b=b, x0=x0,
                params=dict(eps=1e-10, nswp=20, kickrank=4))


def laplace_potential_d20_n64(seed=2):
    """d=20, n=64 Laplacian plus product potential (rank 3); b rank 8 N(0,1), ||b||=1; x0 = ones;
    eps 1e-8, kickrank 8."""
    d, n = 20, 64
    A = laplace_potential_ttm(d, n)
    b = random_tt([n] * d, [1] + [8] * (d - 1) + [1], seed)
    return dict(name="laplace_potential_d20_n64", A=A, b=b, x0=None,
                params=dict(eps=1e-8, nswp=20, kickrank=8))


def parametric_diffusion_d10_n32(index, seed=3, rhs_rank=None):
    """One system of the 256-system batch: A(theta) = sum_k theta_k L_k, theta_k ~ U[0.5, 2];
    b random with rank U{1..16}; eps 1e-8, nswp 40, kickrank 8."""
    d, n = 10, 32
    g = _rng(seed * 100003 + index)
    theta = g.uniform(0.5, 2.0, size=d)
    r = int(g.integers(1, 17)) if rhs_rank is None else int(rhs_rank)
    A = laplace_ttm(d, n, coeffs=theta)
    b = random_tt([n] * d, [1] + [r] * (d - 1) + [1], seed * 100003 + index + 7)
    return dict(name="parametric_diffusion_d10_n32", A=A, b=b, x0=None, theta=theta, rhs_rank=r,
                params=dict(eps=1e-8, nswp=40, kickrank=8))


def small_random_system(seed=0, N=(4, 5, 6), RA=(1, 2, 3, 1), RX=(1, 2, 3, 1)):
    """The reference's own test system (tests/test_solvers.py:15-17): A random TT-matrix, x random,
    b = A x, all N(0,1) cores."""
    g = _rng(seed)
    d = len(N)
    A = [g.standard_normal((RA[k], N[k], N[k], RA[k + 1])) for k in range(d)]
    x = [g.standard_normal((RX[k], N[k], RX[k + 1])) for k in range(d)]
    b = []
    for a, c in zip(A, x):
        t = np.einsum("smnS,rnR->srmSR", a, c)
        b.append(t.reshape(a.shape[0] * c.shape[0], a.shape[1], a.shape[3] * c.shape[2]))
    return dict(name="random_%s" % "x".join(map(str, N)), A=_to_torch(A), b=_to_torch(b),
                x=_to_torch(x), x0=None, params=dict(eps=1e-10))


def rounding_stress(index, seed=4, d=16, n=32, term_rank=16, terms=4, kickrank=8, nswp=20):
    """One solve of the rounding batch (full size: 128 solves, d=16, n=32, 4 rank-16 terms):
    A = Laplacian + C C^T + I (C a random rank-2 TT-matrix with N(0, 0.01^2) cores, so the
    perturbation has rank 4 and A is SPD); b = the sum of ``terms`` random TTs of rank
    ``term_rank`` (N(0,1) cores), to be rounded to ``round_b`` before the solve; eps 1e-8.
    AMEn grows the solution ranks by at most ``kickrank`` per sweep, so a right-hand side of rank
    64 needs nswp * kickrank well above the rank of the solution to converge."""
    A = laplace_lowrank_spd_ttm(d, n, seed)
    parts = [random_tt([n] * d, [1] + [term_rank] * (d - 1) + [1], seed * 100003 + terms * index + i,
                       normalise=False) for i in range(terms)]
    return dict(name="rounding_stress_d%d_n%d" % (d, n), A=A, b=tt_sum(parts), x0=None,
                round_b=1e-8, params=dict(eps=1e-8, nswp=nswp, kickrank=kickrank))


def serving_request(index, seed=5, max_d=24, ranks=(1, 32), modes=(16, 32, 64)):
    """One request of the serving trace: d ~ U{8..max_d}, n in ``modes``, rhs rank ~ U{ranks}
    (N(0,1) cores, ||b|| = 1), operator = anisotropic Laplacian sum_k c_k L_k with c_k ~ U[0.1, 10],
    eps in {1e-6, 1e-8, 1e-10}; nswp 40 and kickrank 8 (as the parametric and single-solve
    workloads), the reference's other defaults. With the reference's nswp 22 and kickrank 4 the
    ranks grow by at most 4 per sweep, to 89, and most requests stop far above eps (the reference's
    own amen_solve gives relres 2.5e-4 at eps 1e-10 on request 8 of seed 5, 9.1e-11 with these
    settings). Full size: max_d 24, ranks 1..32, n in {16, 32, 64}."""
    g = _rng(seed * 1000003 + index)
    d = int(g.integers(8, max_d + 1))
    n = int(g.choice(list(modes)))
    r = int(g.integers(ranks[0], ranks[1] + 1))
    coeffs = g.uniform(0.1, 10.0, size=d)
    eps = float(g.choice([1e-6, 1e-8, 1e-10]))
    A = laplace_ttm(d, n, coeffs=coeffs)
    b = random_tt([n] * d, [1] + [r] * (d - 1) + [1], seed * 1000003 + index + 11)
    return dict(name="serving_request", A=A, b=b, x0=None, d=d, n=n, rhs_rank=r,
                params=dict(eps=eps, nswp=40, kickrank=8))


def serving_trace(count, rate, seed=5):
    """Poisson arrivals: ``count`` requests at ``rate`` per second; returns [(t_arrival, index)]
    with the request of each index given by ``serving_request(index, seed)``."""
    g = _rng(seed * 7919 + 1)
    t = np.cumsum(g.exponential(1.0 / rate, size=count))
    return [(float(t[i]), i) for i in range(count)]
