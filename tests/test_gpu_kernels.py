"""Kernel-level parity of the CUDA path (through the C ABI) against the oracle and the reference's
golden outputs. FP64 throughout: tolerance 1e-12 relative to the output's magnitude."""
import numpy as np
import pytest
import torch

import _golden as G
from oracle import amen as O

pytestmark = pytest.mark.gpu


def t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def close(a, b, tol=1e-12):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else a
    scale = max(np.abs(b).max(), 1e-300)
    assert np.abs(a - b).max() <= tol * scale, (np.abs(a - b).max(), scale)


def test_contractions_golden(cuda):
    from torchtt_gb300 import ops
    z = G.load("kernels.npz")
    for c in range(int(z["ncases"])):
        g = lambda k: t(z["c%d_%s" % (c, k)], cuda)
        close(ops.local_product(g("PhiR"), g("PhiL"), g("A"), g("x")), z["c%d_y" % c])
        close(ops.compute_phi_fwd_A(g("Pf"), g("z"), g("A"), g("x")), z["c%d_fwdA" % c])
        close(ops.compute_phi_bck_A(g("Pb"), g("z"), g("A"), g("x")), z["c%d_bckA" % c])
        close(ops.compute_phi_fwd_rhs(g("Pbf"), g("bk"), g("x")), z["c%d_fwdb" % c])
        close(ops.compute_phi_bck_rhs(g("Pbb"), g("bk"), g("x")), z["c%d_bckb" % c])


@pytest.mark.parametrize("shape", [(60, 3, 64, 3, 60), (52, 2, 16, 2, 50), (8, 7, 32, 7, 8),
                                   (1, 3, 64, 3, 9), (171, 2, 32, 2, 5)])
def test_local_product_config_shapes(cuda, shape):
    """Random operands at the local-problem shapes of the workloads (r, s, n, S, R)."""
    from torchtt_gb300 import ops
    r, s, n, S, R = shape
    g = np.random.default_rng(sum(shape))
    PhiL, A = g.standard_normal((r, s, r)), g.standard_normal((s, n, n, S))
    PhiR, x = g.standard_normal((R, S, R)), g.standard_normal((r, n, R))
    y = ops.local_product(t(PhiR, cuda), t(PhiL, cuda), t(A, cuda), t(x, cuda))
    close(y, O.local_product(PhiR, PhiL, A, x))
    # batched right-hand sides
    xb = g.standard_normal((3, r, n, R))
    yb = ops.local_product(t(PhiR, cuda), t(PhiL, cuda), t(A, cuda), t(xb, cuda))
    for i in range(3):
        close(yb[i], O.local_product(PhiR, PhiL, A, xb[i]))


@pytest.mark.parametrize("dims", [(30, 40, 3, 3, 20, 25, 16), (60, 68, 3, 3, 60, 68, 64), (8, 8, 2, 2, 50, 50, 16)])
def test_phi_updates_shapes(cuda, dims):
    from torchtt_gb300 import ops
    l, L, s, S, r, R, n = dims
    g = np.random.default_rng(l + R)
    left, right = g.standard_normal((l, n, L)), g.standard_normal((r, n, R))
    A = g.standard_normal((s, n, n, S))
    Pf, Pb = g.standard_normal((l, s, r)), g.standard_normal((L, S, R))
    close(ops.compute_phi_fwd_A(t(Pf, cuda), t(left, cuda), t(A, cuda), t(right, cuda)),
          O.compute_phi_fwd_A(Pf, left, A, right))
    close(ops.compute_phi_bck_A(t(Pb, cuda), t(left, cuda), t(A, cuda), t(right, cuda)),
          O.compute_phi_bck_A(Pb, left, A, right))
    bk = g.standard_normal((4, n, 5))
    Pbf, Pbb = g.standard_normal((4, r)), g.standard_normal((5, R))
    close(ops.compute_phi_fwd_rhs(t(Pbf, cuda), t(bk, cuda), t(right, cuda)),
          O.compute_phi_fwd_rhs(Pbf, bk, right))
    close(ops.compute_phi_bck_rhs(t(Pbb, cuda), t(bk, cuda), t(right, cuda)),
          O.compute_phi_bck_rhs(Pbb, bk, right))


@pytest.mark.parametrize("mn", [(512, 8), (4480, 70), (3840, 68), (16, 20), (70, 70), (1, 5), (5472, 179)])
def test_qr(cuda, mn):
    from torchtt_gb300 import ops
    m, n = mn
    g = np.random.default_rng(m + n)
    a = g.standard_normal((m, n)) * np.logspace(0, -9, n)[None, :]   # graded columns
    q, r = ops.qr(t(a, cuda))
    q, r = q.cpu().numpy(), r.cpu().numpy()
    k = min(m, n)
    assert q.shape == (m, k) and r.shape == (k, n)
    assert np.abs(q.T @ q - np.eye(k)).max() < 1e-12
    assert np.linalg.norm(q @ r - a) <= 1e-13 * np.linalg.norm(a)
    assert np.abs(np.tril(r, -1)).max() == 0.0


def test_qr_rank_deficient(cuda):
    """Exactly dependent and zero columns (enrichment blocks inside span(u)) keep Q orthonormal."""
    from torchtt_gb300 import ops
    g = np.random.default_rng(5)
    u = np.linalg.qr(g.standard_normal((2000, 40)))[0]
    a = np.concatenate([u, u[:, :5] @ g.standard_normal((5, 8)), np.zeros((2000, 3))], axis=1)
    q, r = ops.qr(t(a, cuda))
    q, r = q.cpu().numpy(), r.cpu().numpy()
    assert np.abs(q.T @ q - np.eye(q.shape[1])).max() < 1e-10
    assert np.linalg.norm(q @ r - a) <= 1e-12 * np.linalg.norm(a)


@pytest.mark.parametrize("mn", [(3840, 68), (512, 8), (8, 512), (70, 70), (1000, 30), (2000, 200),
                                (700, 700)])
def test_svd(cuda, mn):
    from torchtt_gb300 import ops
    m, n = mn
    g = np.random.default_rng(m * 7 + n)
    k = min(m, n)
    U0 = np.linalg.qr(g.standard_normal((m, k)))[0]
    V0 = np.linalg.qr(g.standard_normal((n, k)))[0]
    s0 = np.logspace(0, -12, k)
    a = (U0 * s0) @ V0.T
    u, s, vh = ops.svd(t(a, cuda))
    u, s, vh = u.cpu().numpy(), s.cpu().numpy(), vh.cpu().numpy()
    assert np.all(np.diff(s) <= 0)
    assert np.abs(s - s0).max() <= 1e-13
    assert np.linalg.norm((u * s) @ vh - a) <= 1e-13 * np.linalg.norm(a)
    assert np.abs(u.T @ u - np.eye(k)).max() < 1e-11
    assert np.abs(vh @ vh.T - np.eye(k)).max() < 1e-12


def test_svd_clustered_and_rank_deficient(cuda):
    """Repeated singular values, a spectrum down to 1e-14 and exact zeros in the cluster Jacobi
    range (16 <= n <= 160), where FP32 sweeps precondition the FP64 ones: the FP32 phase cannot
    resolve the clustered or tiny values and the FP64 sweeps must finish them."""
    from torchtt_gb300 import ops
    m, n = 1500, 100
    g = np.random.default_rng(11)
    s0 = np.concatenate([np.ones(20), np.logspace(-1, -14, 60), np.zeros(20)])
    U0 = np.linalg.qr(g.standard_normal((m, n)))[0]
    V0 = np.linalg.qr(g.standard_normal((n, n)))[0]
    a = (U0 * s0) @ V0.T
    u, s, vh = ops.svd(t(a, cuda))
    u, s, vh = u.cpu().numpy(), s.cpu().numpy(), vh.cpu().numpy()
    assert np.all(np.diff(s) <= 0)
    assert np.abs(s - s0).max() <= 1e-13
    assert np.linalg.norm((u * s) @ vh - a) <= 1e-13 * np.linalg.norm(a)
    assert np.abs(u[:, :80].T @ u[:, :80] - np.eye(80)).max() < 1e-11
    assert np.abs(vh @ vh.T - np.eye(n)).max() < 1e-12


def test_gmres_known_answer(cuda):
    """The reference's GMRES known answer (1-D Laplacian, restart 40, 4 cycles): the device GMRES
    (CGS2) follows the same trajectory as the reference's MGS."""
    from torchtt_gb300 import ops
    z = G.load("kernels.npz")
    L, rhs = z["gmres_L"], z["gmres_rhs"]
    n = L.shape[0]
    one = torch.ones((1, 1, 1), dtype=torch.float64, device=cuda)
    x, flag, nit = ops.local_gmres(one, t(L.reshape(1, n, n, 1), cuda), one,
                                   t(rhs.reshape(1, n, 1), cuda), iters=40, threshold=1e-10, resets=4)
    x = x.cpu().numpy().reshape(-1)
    assert flag == 0 and nit == 160
    assert np.linalg.norm(x - z["gmres_x"]) <= 1e-8 * np.linalg.norm(z["gmres_x"])


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_local_gmres_vs_oracle(cuda, prec):
    from torchtt_gb300 import ops
    g = np.random.default_rng(11 + prec)
    r, s, n, S, R = 4, 2, 6, 2, 5
    PhiL = g.standard_normal((r, s, r)) + 4 * np.eye(r)[:, None, :]
    PhiR = g.standard_normal((R, S, R)) + 4 * np.eye(R)[:, None, :]
    A = g.standard_normal((s, n, n, S)) * 0.1 + np.eye(n)[None, :, :, None]
    rhs = g.standard_normal((r, n, R))
    op = O.LocalOp(PhiL, PhiR, A, (r, n, R), prec)
    xo, fo, no = O.gmres(op.matvec, rhs.reshape(-1), np.zeros(rhs.size), 40, 1e-12, 2)
    xo = op.apply_prec(xo.reshape(r, n, R)) if prec else xo.reshape(r, n, R)
    x, flag, nit = ops.local_gmres(t(PhiL, cuda), t(A, cuda), t(PhiR, cuda), t(rhs, cuda),
                                   iters=40, threshold=1e-12, resets=2, prec=prec)
    assert flag == fo == 1
    assert abs(nit - no) <= 1
    close(x, xo, tol=1e-9)


def _kron_core(k, d, n):
    """One core of the Laplacian-plus-potential operator (rank 3, tridiagonal/diagonal blocks):
    the sparse A cores the structured A stage applies from their nonzeros."""
    from torchtt_gb300 import workloads as W
    return W.laplace_potential_ttm(d, n)[k].numpy()


@pytest.mark.parametrize("k", [0, 2, 4])
@pytest.mark.parametrize("rR", [(7, 9), (40, 36)])
def test_structured_a_stage(cuda, k, rR):
    """Local product and both interface updates with a sparse A core (structured A stage) against
    the oracle's dense contractions, FP64 and both low-precision engines."""
    from torchtt_gb300 import ops
    A = _kron_core(k, 5, 24)
    s, n, _, S = A.shape
    r, R = rR
    g = np.random.default_rng(k * 100 + r)
    PhiL, PhiR = g.standard_normal((r, s, r)), g.standard_normal((R, S, R))
    x = g.standard_normal((r, n, R))
    ref = O.local_product(PhiR, PhiL, A, x)
    close(ops.local_product(t(PhiR, cuda), t(PhiL, cuda), t(A, cuda), t(x, cuda)), ref)
    for engine in (1, 2):
        y = ops.local_product_lowp(t(PhiR, cuda), t(PhiL, cuda), t(A, cuda), t(x, cuda),
                                   engine=engine).cpu().numpy()
        assert np.linalg.norm(y - ref) <= 1e-5 * np.linalg.norm(ref), engine
    z = g.standard_normal((r + 1, n, R + 2))
    Pf = g.standard_normal((r + 1, s, r))
    close(ops.compute_phi_fwd_A(t(Pf, cuda), t(z, cuda), t(A, cuda), t(x, cuda)),
          O.compute_phi_fwd_A(Pf, z, A, x))
    Pb = g.standard_normal((R + 2, S, R))
    close(ops.compute_phi_bck_A(t(Pb, cuda), t(z, cuda), t(A, cuda), t(x, cuda)),
          O.compute_phi_bck_A(Pb, z, A, x))


def test_autotuner_records_classes_and_keeps_results(cuda):
    """The tile autotuner (times every tile shape with and without split-K on the first launch of
    a shape class, then reuses the record) gives the oracle's local product, the same as the
    occupancy heuristic, and records the classes it tuned."""
    from torchtt_gb300 import ops
    g = np.random.default_rng(77)
    r, s, n, S, R = 45, 3, 40, 3, 37
    PhiL, A = g.standard_normal((r, s, r)), g.standard_normal((s, n, n, S))
    PhiR, x = g.standard_normal((R, S, R)), g.standard_normal((r, n, R))
    ref = O.local_product(PhiR, PhiL, A, x)
    prev, _ = ops.autotune(False)
    try:
        y_off = ops.local_product(t(PhiR, cuda), t(PhiL, cuda), t(A, cuda), t(x, cuda))
        ops.autotune(True)
        _, before = ops.autotune(None)
        y_tune = ops.local_product(t(PhiR, cuda), t(PhiL, cuda), t(A, cuda), t(x, cuda))
        _, after = ops.autotune(None)
        y_rec = ops.local_product(t(PhiR, cuda), t(PhiL, cuda), t(A, cuda), t(x, cuda))
    finally:
        ops.autotune(prev)
    assert after >= before
    for y in (y_off, y_tune, y_rec):
        close(y, ref)
