"""CPU restatement (numpy, FP64) of the reference's AMEn linear solve in the TT format.

TEST INFRASTRUCTURE ONLY. This module is the parity oracle: ``tests/``, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may call it, as the checker or as
the timed CPU baseline. The shipped solver (``torchtt_gb300``) never imports it and has no CPU path.

It follows the reference's default native path, ``torchttcpp.amen_solve`` (``cpp/amen_solve.h:122-549``),
step by step, with numpy/LAPACK in place of ATen. Every function cites the reference lines it
restates. Differences from the reference, all deliberate and test-visible:

* the random enrichment cores ``z`` can be injected (``z0``) so that a run can be replayed exactly;
  otherwise they are drawn from a numpy ``Generator`` (the reference draws them from the global torch
  RNG, ``amen_solve.h:176``);
* an optional ``trace`` list records per-core statistics (local size, GMRES iterations, residuals,
  chosen rank), which the reference only prints when ``verbose``.

The restatement is pinned against the compiled reference (``oracle/build_ref.py``) by the fixtures in
``tests/golden/`` (generated by ``tests/golden/make_golden.py``).
"""
import math

import numpy as np

NO_PREC, C_PREC, R_PREC = 0, 1, 2          # cpp/define.h:10-12


# --------------------------------------------------------------------------------------------------
# contractions (cpp/amen_solve.h:17-98)
# --------------------------------------------------------------------------------------------------

def local_product(Phi_right, Phi_left, coreA, core):
    """y[l,m,L] = sum Phi_left[l,s,r] coreA[s,m,n,S] Phi_right[L,S,R] core[r,n,R].

    Restates ``local_product`` (cpp/amen_solve.h:17-27) with the same three tensordots.
    """
    t1 = np.tensordot(core, Phi_left, axes=([0], [2]))          # rnR,lsr->nRls
    t2 = np.tensordot(t1, coreA, axes=([0, 3], [2, 0]))         # nRls,smnS->RlmS
    return np.tensordot(t2, Phi_right, axes=([0, 3], [2, 1]))   # RlmS,LSR->lmL


def compute_phi_bck_A(Phi_now, core_left, core_A, core_right):
    """Phi[l,s,r] = sum Phi_now[L,S,R] core_left[l,M,L] core_A[s,M,N,S] core_right[r,N,R].

    Restates ``compute_phi_bck_A`` (cpp/amen_solve.h:38-47).
    """
    p = np.tensordot(core_left, Phi_now, axes=([2], [0]))       # lML,LSR->lMSR
    p = np.tensordot(p, core_A, axes=([1, 2], [1, 3]))          # lMSR,sMNS->lRsN
    return np.tensordot(p, core_right, axes=([1, 3], [2, 1]))   # lRsN,rNR->lsr


def compute_phi_fwd_A(Phi_now, core_left, core_A, core_right):
    """Phi_next[L,S,R] = sum Phi_now[l,s,r] core_left[l,M,L] core_A[s,M,N,S] core_right[r,N,R].

    Restates ``compute_phi_fwd_A`` (cpp/amen_solve.h:58-68).
    """
    p = np.tensordot(core_left, Phi_now, axes=([0], [0]))       # lML,lsr->MLsr
    p = np.tensordot(p, core_A, axes=([0, 2], [1, 0]))          # MLsr,sMNS->LrNS
    return np.tensordot(p, core_right, axes=([1, 2], [0, 1]))   # LrNS,rNR->LSR


def compute_phi_bck_rhs(Phi_now, core_b, core):
    """Phi[b,r] = sum Phi_now[B,R] core_b[b,n,B] core[r,n,R]  (cpp/amen_solve.h:78-83)."""
    p = np.tensordot(core_b, Phi_now, axes=([2], [0]))
    return np.tensordot(p, core, axes=([1, 2], [1, 2]))


def compute_phi_fwd_rhs(Phi_now, core_rhs, core):
    """Phi_next[B,R] = sum Phi_now[b,r] core_rhs[b,n,B] core[r,n,R]  (cpp/amen_solve.h:93-98)."""
    p = np.tensordot(Phi_now, core_rhs, axes=([0], [0]))
    return np.tensordot(p, core, axes=([0, 1], [0, 1]))


def local_rhs(Phi_b_left, core_b, Phi_b_right):
    """rhs[r,n,R] = sum Phi_b_left[b,r] core_b[b,n,B] Phi_b_right[B,R]  (cpp/amen_solve.h:303-304)."""
    t = np.tensordot(Phi_b_left, core_b, axes=([0], [0]))
    return np.tensordot(t, Phi_b_right, axes=([2], [0]))


# --------------------------------------------------------------------------------------------------
# local operator with the block-Jacobi preconditioners (cpp/matvecs.h:130-212)
# --------------------------------------------------------------------------------------------------

class LocalOp:
    """The local AMEn operator ``AMENsolveMV`` (cpp/matvecs.h:130-212)."""

    def __init__(self, Phi_left, Phi_right, coreA, shape, prec=NO_PREC):
        self.Phi_left, self.Phi_right, self.coreA = Phi_left, Phi_right, coreA
        self.shape = tuple(int(s) for s in shape)
        self.prec = prec
        if prec == C_PREC:                                        # matvecs.h:161-165
            Jl = np.tensordot(np.diagonal(Phi_left, 0, 0, 2), coreA, axes=([0], [0]))  # sd,smnS->dmnS
            Jr = np.diagonal(Phi_right, 0, 0, 2)                                      # SD
            J = np.tensordot(Jl, Jr, axes=([3], [0])).transpose(0, 3, 1, 2)           # d,D,m,n
            self.J = np.linalg.inv(J)
        elif prec == R_PREC:                                      # matvecs.h:166-174
            Jl = np.tensordot(np.diagonal(Phi_left, 0, 0, 2), coreA, axes=([0], [0]))  # dmnS
            Jt = np.tensordot(Jl, Phi_right, axes=([3], [1]))                         # dmnLR
            Jt = Jt.transpose(0, 1, 3, 2, 4)                                          # dmLnR
            sh = Jt.shape
            Jt2 = Jt.reshape(sh[0], sh[1] * sh[2], sh[3] * sh[4])
            self.J = np.linalg.inv(Jt2).reshape(sh)

    def apply_prec(self, sol):
        """matvecs.h:177-194."""
        if self.prec == C_PREC:
            s0, s1, s2 = sol.shape
            tmp = sol.transpose(0, 2, 1).reshape(s0, s2, s1, 1)
            return np.matmul(self.J, tmp).transpose(0, 2, 1, 3).reshape(s0, s1, s2)
        if self.prec == R_PREC:
            return np.einsum("rnR,rmLnR->rmL", sol, self.J)
        return sol

    def matvec(self, x, use_prec=True):
        """matvecs.h:196-212: optional preconditioner, then the three tensordots."""
        t = x.reshape(self.shape)
        if use_prec and self.prec != NO_PREC:
            t = self.apply_prec(t)
        w = np.tensordot(t, self.Phi_left, axes=([0], [2]))
        w = np.tensordot(w, self.coreA, axes=([0, 3], [2, 0]))
        w = np.tensordot(w, self.Phi_right, axes=([0, 3], [2, 1]))
        return w.reshape(-1)


# --------------------------------------------------------------------------------------------------
# restarted GMRES (cpp/gmres.h:15-161)
# --------------------------------------------------------------------------------------------------

def _givens(v1, v2):
    """gmres.h:15-18."""
    den = math.sqrt(v1 * v1 + v2 * v2)
    return v1 / den, v2 / den


def gmres_single(matvec, rhs, x0, iters, threshold):
    """One GMRES cycle with modified Gram-Schmidt and Givens rotations (gmres.h:34-144).

    Returns ``(solution, flag, nit)``.
    """
    r = rhs - matvec(x0)
    b_norm = np.linalg.norm(rhs)
    r_norm = np.linalg.norm(r)
    if not r_norm > 0:                                            # gmres.h:56-65
        return x0.copy(), 1, 0
    sn = np.zeros(iters)
    cs = np.zeros(iters)
    beta = np.zeros(iters + 1)
    H = np.zeros((iters + 1, iters))
    Q = [r / r_norm]
    beta[0] = r_norm
    flag = 0
    k = 0
    for k in range(iters):                                        # gmres.h:87-130
        q = matvec(Q[k])
        for i in range(k + 1):                                    # MGS, gmres.h:98-101
            H[i, k] = np.dot(q, Q[i])
            q = q - H[i, k] * Q[i]
        h = np.linalg.norm(q)
        q = q / h
        H[k + 1, k] = h
        Q.append(q)
        col = H[:k + 2, k].copy()                                 # apply_givens_rotation_cpu
        for i in range(k):
            temp = cs[i] * col[i] + sn[i] * col[i + 1]
            col[i + 1] = -sn[i] * col[i] + cs[i] * col[i + 1]
            col[i] = temp
        c, s = _givens(col[k], col[k + 1])
        col[k] = c * col[k] + s * col[k + 1]
        col[k + 1] = 0.0
        H[:k + 2, k] = col
        cs[k], sn[k] = c, s
        beta[k + 1] = -sn[k] * beta[k]
        beta[k] = cs[k] * beta[k]
        error = abs(beta[k + 1]) / b_norm
        if error <= threshold:
            flag = 1
            break
    k = k if k < iters else iters - 1                             # gmres.h:131
    y = np.linalg.solve(H[:k + 1, :k + 1], beta[:k + 1])
    sol = x0.copy()
    for i in range(k + 1):
        sol = sol + Q[i] * y[i]
    return sol, flag, k + 1


def gmres(matvec, rhs, x0, max_iters, threshold, resets):
    """Restarted GMRES driver (gmres.h:146-161). Returns ``(solution, flag, nit)``."""
    nit, flag = 0, 0
    xs = x0
    sol = x0
    for _ in range(resets):
        sol, flag, nowit = gmres_single(matvec, rhs, xs, max_iters, threshold)
        nit += nowit
        if flag == 1:
            break
        xs = sol.copy()
    return sol, flag, nit


# --------------------------------------------------------------------------------------------------
# orthogonalisation helpers (cpp/ortho.h:46-73)
# --------------------------------------------------------------------------------------------------

def rl_orthogonal_this(cores):
    """Right-to-left QR sweep in place (cpp/ortho.h:46-73). Returns the new rank list."""
    d = len(cores)
    ranks = [1] + [c.shape[2] for c in cores]
    for i in range(d - 1, 0, -1):
        c = cores[i]
        mat = c.reshape(c.shape[0], -1).T
        Q, R = np.linalg.qr(mat)
        r_new = R.shape[0]
        cores[i] = Q.T.reshape(r_new, c.shape[1], -1)
        ranks[i] = r_new
        p = cores[i - 1]
        cores[i - 1] = (p.reshape(-1, p.shape[2]) @ R.T).reshape(p.shape[0], p.shape[1], -1)
    return ranks


# --------------------------------------------------------------------------------------------------
# AMEn solve (cpp/amen_solve.h:122-549)
# --------------------------------------------------------------------------------------------------

def _svd(mat):
    u, s, vh = np.linalg.svd(mat, full_matrices=False)
    return u, s, vh


def amen_solve(A_cores, b_cores, x0_cores=None, nswp=22, eps=1e-10, rmax=32768, max_full=500,
               kickrank=4, kick2=0, local_iterations=40, resets=2, prec=NO_PREC, z0=None,
               rng=None, trace=None, verbose=False):
    """AMEn solve of A x = b in the TT format, restating ``amen_solve`` (cpp/amen_solve.h:122-549).

    Args mirror ``torchttcpp.amen_solve`` (cpp/amen_solve.h:122-139). ``A_cores`` are 4-D
    ``r x m x n x r'`` float64 arrays, ``b_cores`` and ``x0_cores`` 3-D ``r x n x r'``. ``z0`` optionally
    gives the initial enrichment cores (the reference draws them with ``torch::randn``,
    amen_solve.h:174-176); otherwise ``rng`` (a numpy Generator) draws them.

    Returns ``(x_cores, info)``, ``info`` holding the sweep count and the final max local residual.
    """
    A_cores = [np.asarray(c, dtype=np.float64) for c in A_cores]
    b_cores = [np.asarray(c, dtype=np.float64) for c in b_cores]
    d = len(A_cores)
    N = [c.shape[2] for c in A_cores]
    if rng is None:
        rng = np.random.default_rng(0)

    if x0_cores is None or len(x0_cores) == 0:                      # amen_solve.h:161-166
        x = [np.ones((1, N[i], 1)) for i in range(d)]
    else:
        x = [np.array(c, dtype=np.float64, copy=True) for c in x0_cores]
    rx = [1] + [c.shape[2] for c in x]

    rz = [1] + [kickrank + kick2] * (d - 1) + [1]                  # amen_solve.h:169-176
    if z0 is not None:
        z = [np.array(c, dtype=np.float64, copy=True) for c in z0]
    else:
        z = [rng.standard_normal((rz[i], N[i], rz[i + 1])) for i in range(d)]
    rz = rl_orthogonal_this(z)                                      # amen_solve.h:178

    one3 = np.ones((1, 1, 1))
    one2 = np.ones((1, 1))
    Phiz = [one3] + [None] * (d - 1) + [one3]                       # amen_solve.h:182-193
    Phiz_b = [one2] + [None] * (d - 1) + [one2]
    Phis = [one3] + [None] * (d - 1) + [one3]
    Phis_b = [one2] + [None] * (d - 1) + [one2]

    normA = np.ones(d - 1)
    normb = np.ones(d - 1)
    normx = np.ones(d - 1)
    nrmsc = 1.0
    damp = 2.0
    last = False
    swp = 0
    max_res = 0.0

    for swp in range(nswp):                                         # amen_solve.h:212
        # ---------------- backward orthogonalisation sweep (amen_solve.h:222-292)
        for k in range(d - 1, 0, -1):
            if not last:
                if swp > 0:                                         # amen_solve.h:225-236
                    czA = local_product(Phiz[k + 1], Phiz[k], A_cores[k], x[k])
                    czy = np.tensordot(Phiz_b[k], b_cores[k], axes=([0], [0]))
                    czy = np.tensordot(czy, Phiz_b[k + 1], axes=([2], [0]))
                    czy = czy * nrmsc - czA
                    _, _, vh = _svd(czy.reshape(czy.shape[0], -1))
                    temp = min(kickrank, vh.shape[0])
                    cz_new = vh[:temp, :].T
                    if k < d - 1 and kick2 > 0:
                        cz_new = np.concatenate([cz_new, rng.standard_normal((cz_new.shape[0], kick2))], 1)
                else:
                    cz_new = z[k].reshape(rz[k], -1).T
                Qz, _ = np.linalg.qr(cz_new)                        # amen_solve.h:241-244
                rz[k] = Qz.shape[1]
                z[k] = Qz.T.reshape(rz[k], N[k], rz[k + 1])

            if swp > 0:                                             # amen_solve.h:249-250
                nrmsc = nrmsc * normA[k - 1] * normx[k - 1] / normb[k - 1]

            core = x[k].reshape(rx[k], N[k] * rx[k + 1]).T          # amen_solve.h:252-267
            Q, R = np.linalg.qr(core)
            core_prev = np.tensordot(x[k - 1], R.T, axes=([2], [0]))
            rx[k] = Q.shape[1]
            current_norm = np.linalg.norm(core_prev)
            if current_norm > 0:
                core_prev = core_prev / current_norm
            else:
                current_norm = 1.0
            normx[k - 1] = normx[k - 1] * current_norm
            x[k] = Q.T.reshape(rx[k], N[k], rx[k + 1]).copy()
            x[k - 1] = core_prev.copy()

            Phis[k] = compute_phi_bck_A(Phis[k + 1], x[k], A_cores[k], x[k])   # :270-271
            Phis_b[k] = compute_phi_bck_rhs(Phis_b[k + 1], b_cores[k], x[k])

            norm = np.linalg.norm(Phis[k])                          # amen_solve.h:274-282
            norm = norm if norm > 0 else 0.0
            normA[k - 1] = norm
            Phis[k] = Phis[k] / norm
            norm = np.linalg.norm(Phis_b[k])
            norm = norm if norm > 0 else 0.0
            normb[k - 1] = norm
            Phis_b[k] = Phis_b[k] / norm
            nrmsc = nrmsc * normb[k - 1] / (normA[k - 1] * normx[k - 1])       # :285

            if not last:                                            # amen_solve.h:288-291
                Phiz[k] = compute_phi_bck_A(Phiz[k + 1], z[k], A_cores[k], x[k]) / normA[k - 1]
                Phiz_b[k] = compute_phi_bck_rhs(Phiz_b[k + 1], b_cores[k], z[k]) / normb[k - 1]

        # ---------------- forward solve sweep (amen_solve.h:296-512)
        max_res = 0.0
        max_dx = 0.0
        for k in range(d):
            previous_solution = x[k].reshape(-1)
            rhs = local_rhs(Phis_b[k], b_cores[k] * nrmsc, Phis_b[k + 1]).reshape(-1)   # :303-304
            norm_rhs = np.linalg.norm(rhs)
            real_tol = (eps / math.sqrt(d)) / damp                  # amen_solve.h:309
            shape_now = (rx[k], N[k], rx[k + 1])
            use_full = rx[k] * N[k] * rx[k + 1] < max_full          # amen_solve.h:312
            B = None
            op = None
            nit = 0
            flag = 0
            if use_full:                                            # amen_solve.h:319-330
                Bp = np.tensordot(A_cores[k], Phis[k + 1], axes=([3], [1]))   # smnLR
                Bp = np.tensordot(Phis[k], Bp, axes=([1], [0]))                # lrmnLR
                nl = rx[k] * N[k] * rx[k + 1]
                B = Bp.transpose(0, 2, 4, 1, 3, 5).reshape(nl, nl)
                solution_now = np.linalg.solve(B, rhs)
                res_old = np.linalg.norm(B @ previous_solution - rhs) / norm_rhs
                res_new = np.linalg.norm(B @ solution_now - rhs) / norm_rhs
            else:                                                   # amen_solve.h:331-365
                op = LocalOp(Phis[k], Phis[k + 1], A_cores[k], shape_now, prec)
                eps_local = real_tol * norm_rhs
                drhs = rhs - op.matvec(previous_solution, False)
                eps_local /= np.linalg.norm(drhs)
                ps = 0.0 * previous_solution
                solution_now, flag, nit = gmres(op.matvec, drhs, ps, local_iterations, eps_local, resets)
                if prec != NO_PREC:
                    solution_now = op.apply_prec(solution_now.reshape(shape_now))
                solution_now = solution_now.reshape(-1) + previous_solution
                res_old = np.linalg.norm(op.matvec(previous_solution, False) - rhs) / norm_rhs
                res_new = np.linalg.norm(op.matvec(solution_now, False) - rhs) / norm_rhs
            if verbose and res_old / res_new < damp and res_new > real_tol:
                print("WARNING: residual increase. res_old %g, res_new %g, %g" % (res_old, res_new, real_tol))

            dx = np.linalg.norm(solution_now - previous_solution) / np.linalg.norm(solution_now)  # :369
            max_dx = max(max_dx, dx)
            max_res = max(max_res, res_old)                         # amen_solve.h:375

            solution_now = solution_now.reshape(rx[k] * N[k], rx[k + 1])
            if k < d - 1:                                           # amen_solve.h:382-404
                u, s, v = _svd(solution_now)
                r = u.shape[1]
                while r > 0:
                    sol = (u[:, :r] * s[:r]) @ v[:r, :]
                    if use_full:
                        res = np.linalg.norm(B @ sol.reshape(-1) - rhs) / norm_rhs
                    else:
                        res = np.linalg.norm(op.matvec(sol.reshape(-1), False) - rhs) / norm_rhs
                    if res > (res_new if res_new > real_tol * damp else real_tol * damp):
                        break
                    r -= 1
                r += 1
                r = r if (r < u.shape[1] and r < rmax) else (u.shape[1] if u.shape[1] < rmax else rmax)
            else:                                                   # amen_solve.h:406-410
                u, v = np.linalg.qr(solution_now)
                r = u.shape[1]
                s = np.ones(r)

            u = u[:, :r]                                            # amen_solve.h:413-416
            v = (np.diag(s[:r]) @ v[:r, :]).T

            if trace is not None:
                trace.append(dict(sweep=swp, core=k, local_size=int(np.prod(shape_now)),
                                  use_full=bool(use_full), nit=int(nit), flag=int(flag),
                                  res_old=float(res_old), res_new=float(res_new), rank=int(r)))

            if not last:                                            # amen_solve.h:418-442
                tmp = (u @ v.T).reshape(rx[k], N[k], rx[k + 1])
                czA = local_product(Phiz[k + 1], Phiz[k], A_cores[k], tmp)
                czy = np.tensordot(Phiz_b[k], nrmsc * b_cores[k], axes=([0], [0]))
                czy = np.tensordot(czy, Phiz_b[k + 1], axes=([2], [0]))
                tmp = (czy - czA).reshape(rz[k] * N[k], rz[k + 1])
                uz, _, _ = _svd(tmp)
                rtmp = min(kickrank, uz.shape[1])
                tmp = uz[:, :rtmp]
                if k < d - 1 and kick2 > 0:
                    tmp = np.concatenate([tmp, rng.standard_normal((tmp.shape[0], kick2))], 1)
                qz, _ = np.linalg.qr(tmp)
                rz[k + 1] = qz.shape[1]
                z[k] = qz.reshape(rz[k], N[k], rz[k + 1]).copy()

            if k < d - 1:                                           # amen_solve.h:443-504
                if not last:
                    tmp = (u @ v.T).reshape(rx[k], N[k], rx[k + 1])
                    left_res = local_product(Phiz[k + 1], Phis[k], A_cores[k], tmp)
                    left_b = np.tensordot(Phis_b[k], b_cores[k] * nrmsc, axes=([0], [0]))
                    left_b = np.tensordot(left_b, Phiz_b[k + 1], axes=([2], [0]))
                    uk = (left_b - left_res).reshape(u.shape[0], -1)
                    uk = np.concatenate([u, uk], 1)
                    r_add = left_res.shape[2]
                    u, Rmat = np.linalg.qr(uk)
                    v = np.concatenate([v, np.zeros((rx[k + 1], r_add))], 1)
                    v = v @ Rmat.T
                r = u.shape[1]
                v = np.tensordot(v, x[k + 1], axes=([0], [0]))
                nrmsc = nrmsc * normA[k] * normx[k] / normb[k]      # amen_solve.h:465
                norm_now = np.linalg.norm(v)
                if norm_now > 0:
                    v = v / norm_now
                else:
                    norm_now = 1.0
                normx[k] = normx[k] * norm_now
                x[k] = u.reshape(rx[k], N[k], r).copy()
                x[k + 1] = v.reshape(r, N[k + 1], rx[k + 2]).copy()
                rx[k + 1] = r

                Phis[k + 1] = compute_phi_fwd_A(Phis[k], x[k], A_cores[k], x[k])   # :482-483
                Phis_b[k + 1] = compute_phi_fwd_rhs(Phis_b[k], b_cores[k], x[k])
                norm = np.linalg.norm(Phis[k + 1])                  # amen_solve.h:486-493
                norm = norm if norm > 0 else 1.0
                normA[k] = norm
                Phis[k + 1] = Phis[k + 1] / norm
                norm = np.linalg.norm(Phis_b[k + 1])
                norm = norm if norm > 0 else 1.0
                normb[k] = norm
                Phis_b[k + 1] = Phis_b[k + 1] / norm
                nrmsc = nrmsc * normb[k] / (normA[k] * normx[k])    # amen_solve.h:496
                if not last:                                        # amen_solve.h:500-503
                    Phiz[k + 1] = compute_phi_fwd_A(Phiz[k], z[k], A_cores[k], x[k]) / normA[k]
                    Phiz_b[k + 1] = compute_phi_fwd_rhs(Phiz_b[k], b_cores[k], z[k]) / normb[k]
            else:                                                   # amen_solve.h:505-508
                usv = (u * s[:r]) @ v[:r, :].T
                x[k] = usv.reshape(rx[k], N[k], rx[k + 1])
        if verbose:
            print("sweep %d ranks %s max_res %g" % (swp + 1, rx, max_res))
        if last:                                                    # amen_solve.h:522-526
            break
        if max_res < eps:
            last = True

    norm_x = math.exp(sum(math.log(v) for v in normx) / d)          # amen_solve.h:534-541
    x = [c * norm_x for c in x]
    info = dict(sweeps=(swp + 1 if swp < nswp else swp), max_res=float(max_res), ranks=list(rx))
    return x, info


# --------------------------------------------------------------------------------------------------
# TT-level helpers used by the checks (reference: torchtt/_tt_base.py)
# --------------------------------------------------------------------------------------------------

def tt_matvec(A_cores, x_cores):
    """TT-matrix @ TT-vector, core by core (torchtt/_tt_base.py:807-817): ranks multiply."""
    out = []
    for a, c in zip(A_cores, x_cores):
        t = np.einsum("smnS,rnR->srmSR", a, c)
        out.append(t.reshape(a.shape[0] * c.shape[0], a.shape[1], a.shape[3] * c.shape[2]))
    return out


def tt_add(x_cores, y_cores, alpha=1.0, beta=1.0):
    """alpha*x + beta*y by block concatenation of the cores (torchtt/_tt_base.py:413-528)."""
    d = len(x_cores)
    if d == 1:
        return [alpha * x_cores[0] + beta * y_cores[0]]
    out = []
    for k, (a, b) in enumerate(zip(x_cores, y_cores)):
        if k == 0:
            out.append(np.concatenate([alpha * a, beta * b], axis=2))
        elif k == d - 1:
            out.append(np.concatenate([a, b], axis=0))
        else:
            c = np.zeros((a.shape[0] + b.shape[0], a.shape[1], a.shape[2] + b.shape[2]))
            c[:a.shape[0], :, :a.shape[2]] = a
            c[a.shape[0]:, :, a.shape[2]:] = b
            out.append(c)
    return out


def tt_norm(cores):
    """Frobenius norm by a left-to-right QR sweep (torchtt/_tt_base.py:1021-1051); TT-matrix
    cores (4-D) are handled as r x (m n) x R."""
    cur = None
    for c in cores:
        c = c.reshape(c.shape[0], -1, c.shape[-1])
        if cur is not None:
            c = np.tensordot(cur, c, axes=([1], [0]))
        mat = c.reshape(-1, c.shape[2])
        q, cur = np.linalg.qr(mat)
    return float(np.linalg.norm(cur))


def tt_full(cores):
    """Dense tensor of a TT-vector (cpp/full.h:3-12); small cases only."""
    t = cores[0]
    for c in cores[1:]:
        t = np.tensordot(t, c, axes=([t.ndim - 1], [0]))
    return t.reshape(t.shape[1:-1])


def tt_relres(A_cores, x_cores, b_cores):
    """||A x - b|| / ||b|| computed in the TT format, as the reference's tests do
    (tests/test_solvers.py:19)."""
    r = tt_add(tt_matvec(A_cores, x_cores), b_cores, 1.0, -1.0)
    return tt_norm(r) / tt_norm(b_cores)


def tt_relerr(x_cores, y_cores):
    """||x - y|| / ||y|| in the TT format."""
    return tt_norm(tt_add(x_cores, y_cores, 1.0, -1.0)) / tt_norm(y_cores)


# --------------------------------------------------------------------------------------------------
# TT rounding (torchtt/_decomposition.py:62-113,169-228,289-324)
# --------------------------------------------------------------------------------------------------

def rank_chop(s, tol):
    """Smallest rank r >= 1 whose discarded tail sum_{k >= r} s_k^2 is below tol^2
    (restates rank_chop, torchtt/_decomposition.py:289-324)."""
    s = np.asarray(s, dtype=np.float64)
    if np.linalg.norm(s) == 0.0:
        return 1
    if tol <= 0.0:
        return s.size
    tail = np.cumsum((s ** 2)[::-1])[::-1]
    below = np.nonzero(tail < tol ** 2)[0]
    if below.size == 0:
        return s.size
    return max(int(below[0]), 1)


def tt_round(cores, eps, rmax=2 ** 62):
    """TT rounding: left-to-right QR orthogonalisation (lr_orthogonal,
    torchtt/_decomposition.py:62-113), then right-to-left truncated SVDs with threshold
    eps / sqrt(d - 1) times the norm of each core's singular values and the rank cap rmax
    (round_tt, torchtt/_decomposition.py:169-228). TT-matrix cores (4-D) are handled as
    r x (m n) x R. Returns the new cores with the input's core shapes."""
    shapes = [c.shape for c in cores]
    cs = [c.reshape(c.shape[0], -1, c.shape[-1]).copy() for c in cores]
    d = len(cs)
    if d == 1:
        return [c.copy() for c in cores]
    for i in range(d - 1):
        r, m, R = cs[i].shape
        q, rf = np.linalg.qr(cs[i].reshape(r * m, R))
        cs[i] = q.reshape(r, m, q.shape[1])
        nxt = cs[i + 1]
        cs[i + 1] = (rf @ nxt.reshape(nxt.shape[0], -1)).reshape(rf.shape[0], nxt.shape[1], nxt.shape[2])
    ep = eps / math.sqrt(d - 1)
    for i in range(d - 1, 0, -1):
        r, m, R = cs[i].shape
        u, s, vh = np.linalg.svd(cs[i].reshape(r, m * R), full_matrices=False)
        rn = min(int(rmax), rank_chop(s, np.linalg.norm(s) * ep))
        cs[i] = vh[:rn].reshape(rn, m, R)
        prev = cs[i - 1]
        cs[i - 1] = (prev.reshape(-1, r) @ (u[:, :rn] * s[:rn])).reshape(prev.shape[0], prev.shape[1], rn)
    return [c.reshape((c.shape[0],) + tuple(sh[1:-1]) + (c.shape[-1],)) for c, sh in zip(cs, shapes)]


# --------------------------------------------------------------------------------------------------
# DMRG matvec (cpp/dmrg_mv.h:23-230)
# --------------------------------------------------------------------------------------------------

def _rank_chop_cpp(s, tol):
    """rank_chop of cpp/ortho.h:16-45 (the C++ DMRG uses it): largest r with a discarded tail
    sum_{k >= r} s_k^2 >= tol^2, plus one; 1 for s = 0."""
    s = np.asarray(s)
    n = s.size
    if np.linalg.norm(s) == 0.0:
        return 1
    if tol <= 0.0:
        return n - 1
    r = n - 1
    while r > 0:
        if np.sum(s[r:] ** 2) >= tol * tol:
            break
        r -= 1
    return max(r + 1, 1)


def dmrg_matvec(A_cores, x_cores, y0_cores=None, nswp=20, eps=1e-12, rmax=32768, kickrank=4,
                rng=None):
    """y ~ A x by two-site DMRG, restating dmrg_mv (cpp/dmrg_mv.h:23-230) step by step: a
    right-to-left QR sweep with backward interfaces, then two-site blocks truncated by SVD with
    rank_chop at eps ||W|| / d^1.5 (d^0.5 in the last sweep) plus an adaptive enlargement, and
    kickrank random directions. Random numbers come from `rng` (a numpy Generator)."""
    rng = rng if rng is not None else np.random.default_rng(0)
    d = len(A_cores)
    M = [a.shape[1] for a in A_cores]
    if y0_cores is None:
        ry = [1] + [2] * (d - 1) + [1]
        y = [rng.standard_normal((ry[k], M[k], ry[k + 1])) for k in range(d)]
    else:
        y = [c.copy() for c in y0_cores]
        ry = [1] + [c.shape[2] for c in y]
    Phis = [np.ones((1, 1, 1))] + [None] * (d - 1) + [np.ones((1, 1, 1))]
    delta = np.ones(d - 1)
    delta_prev = np.ones(d - 1)
    renl = [2] * d
    last = False
    for swp in range(nswp):
        for k in range(d - 1, 0, -1):
            core = y[k].transpose(1, 2, 0).reshape(M[k] * ry[k + 1], ry[k])
            Q, R = np.linalg.qr(core)
            rnew = min(core.shape)
            y[k] = Q.T.reshape(rnew, M[k], -1)
            ry[k] = rnew
            y[k - 1] = np.tensordot(y[k - 1].reshape(-1, y[k - 1].shape[2]), R, axes=([1], [1])).reshape(-1, M[k - 1], rnew)
            Phi = np.tensordot(Phis[k + 1], x_cores[k], axes=([2], [2]))
            Phi = np.tensordot(A_cores[k], Phi, axes=([2, 3], [3, 1]))
            Phis[k] = np.tensordot(y[k], Phi, axes=([1, 2], [1, 2]))
        for k in range(d - 1):
            W_prev = np.tensordot(y[k], y[k + 1], axes=([2], [0]))
            if not last:
                W1 = np.tensordot(Phis[k], x_cores[k], axes=([2], [0]))
                W1 = np.tensordot(A_cores[k], W1, axes=([0, 2], [1, 2]))
                W2 = np.tensordot(Phis[k + 2], x_cores[k + 1], axes=([2], [2]))
                W2 = np.tensordot(A_cores[k + 1], W2, axes=([2, 3], [3, 1]))
                W = np.tensordot(W1, W2, axes=([1, 3], [0, 3])).transpose(1, 0, 2, 3)
            else:
                W = W_prev
            b = np.linalg.norm(W)
            delta[k] = np.linalg.norm(W - W_prev) / b if b > 0 else 0.0
            with np.errstate(divide="ignore", invalid="ignore"):
                ratio = delta[k] / delta_prev[k]
            if ratio >= 1 and delta[k] > eps:
                renl[k] += 1
            if ratio < 0.1 and delta[k] < eps:
                renl[k] = max(renl[k] - 1, 1)
            U, S, V = np.linalg.svd(W.reshape(W.shape[0] * W.shape[1], -1), full_matrices=False)
            r_new = _rank_chop_cpp(S, b * eps / d ** (0.5 if last else 1.5))
            if not last:
                r_new += renl[k]
            r_new = max(min(r_new, S.size, rmax), 1)
            W1 = U[:, :r_new]
            W2 = V[:r_new, :].T * S[:r_new]
            if swp < nswp - 1:
                W1, Rm = np.linalg.qr(np.concatenate([W1, rng.standard_normal((W1.shape[0], kickrank))], 1))
                W2 = np.concatenate([W2, np.zeros((W2.shape[0], kickrank))], 1)
                W2 = np.tensordot(Rm, W2, axes=([1], [1]))
                r_new = W1.shape[1]
            else:
                W2 = W2.T
            ry[k + 1] = r_new
            y[k] = W1.reshape(ry[k], M[k], r_new)
            y[k + 1] = W2.reshape(r_new, M[k + 1], ry[k + 2])
            Pn = np.tensordot(Phis[k], x_cores[k], axes=([2], [0]))
            Pn = np.tensordot(Pn, A_cores[k], axes=([1, 2], [0, 2]))
            Phis[k + 1] = np.tensordot(y[k], Pn, axes=([0, 1], [0, 2])).transpose(0, 2, 1)
        if last:
            break
        if delta.max() < eps:
            last = True
        delta_prev = delta.copy()
    return y


# --------------------------------------------------------------------------------------------------
# AMEn matvec (torchtt/_amen.py:126-410, for a TT-vector b)
# --------------------------------------------------------------------------------------------------

def _local_ab(Pl, Pr, a, b):
    """Projection of A b: out[l,M,L] = sum Pl[l,s,c] a[s,M,K,S] b[c,K,C] Pr[L,S,C]
    (_local_AB, torchtt/_amen.py:36-53, for vectors)."""
    return local_product(Pr, Pl, a, b)


def _phi_ab(fwd, Phi, a, b, core):
    """Interfaces with (A, b) (_compute_phi_bck_AB / _fwd_AB, torchtt/_amen.py:452-487)."""
    if fwd:
        return np.einsum('rac,rMR,aMKA,cKC->RAC', Phi, core, a, b, optimize=True)
    return np.einsum('RAC,rMR,aMKA,cKC->rac', Phi, core, a, b, optimize=True)


def _phi_xx(fwd, Phi, left, right):
    """Interfaces between two cores (_compute_phi_bck_x / _fwd_x, torchtt/_amen.py:416-449)."""
    if fwd:
        return np.einsum('lr,lML,rMR->LR', Phi, left, right, optimize=True)
    return np.einsum('LR,lML,rMR->lr', Phi, left, right, optimize=True)


def amen_mv(A_cores, b_cores, x0_cores=None, nswp=22, eps=1e-10, rmax=1024, kickrank=4, kick2=0,
            rng=None):
    """y ~ A b by AMEn, restating _amen_mm_python (torchtt/_amen.py:126-410) step by step for a
    TT-vector b: zeros of rank 1 as the start, random orthogonalised z, right-to-left z update /
    QR / interface refresh with the normx/normb/nrmsc bookkeeping, left-to-right projection,
    truncation (rank_chop at eps ||.|| / d^1.5, d^0.5 in the last sweep), z update and enrichment.
    Random numbers come from `rng` (a numpy Generator)."""
    rng = rng if rng is not None else np.random.default_rng(0)
    d = len(A_cores)
    M = [a.shape[1] for a in A_cores]
    if x0_cores is None:
        x = [np.zeros((1, m, 1)) for m in M]
        rx = [1] * (d + 1)
    else:
        x = [c.copy() for c in x0_cores]
        rx = [1] + [c.shape[2] for c in x]
    rz = [1] + [kickrank + kick2] * (d - 1) + [1]
    z = [rng.standard_normal((rz[k], M[k], rz[k + 1])) for k in range(d)]
    for k in range(d - 1, 0, -1):   # rl_orthogonal
        q, r = np.linalg.qr(z[k].reshape(rz[k], -1).T)
        rz[k] = q.shape[1]
        z[k] = q.T.reshape(rz[k], M[k], rz[k + 1])
        z[k - 1] = np.tensordot(z[k - 1], r.T, axes=([2], [0]))
    one2, one3 = np.ones((1, 1)), np.ones((1, 1, 1))
    Phiz = [one2] + [None] * (d - 1) + [one2]
    Phiz_rhs = [one3] + [None] * (d - 1) + [one3]
    Phis = [one2] + [None] * (d - 1) + [one2]
    Phis_rhs = [one3] + [None] * (d - 1) + [one3]
    normA, normb, normx = np.ones(d - 1), np.ones(d - 1), np.ones(d - 1)
    nrmsc = 1.0
    last = False
    for swp in range(nswp):
        for k in range(d - 1, 0, -1):
            if not last:
                if swp > 0:
                    czx = np.einsum('zr,rmR,ZR->zmZ', Phiz[k], x[k], Phiz[k + 1])
                    czAB = _local_ab(Phiz_rhs[k], Phiz_rhs[k + 1], A_cores[k], b_cores[k])
                    cz = czAB * nrmsc - czx
                    _, _, vz = np.linalg.svd(cz.reshape(cz.shape[0], -1), full_matrices=False)
                    cz = vz[:min(kickrank, vz.shape[0]), :].T
                    if k < d - 1:
                        cz = np.concatenate([cz, rng.standard_normal((cz.shape[0], kick2))], 1)
                else:
                    cz = z[k].reshape(rz[k], -1).T
                qz, _ = np.linalg.qr(cz)
                rz[k] = qz.shape[1]
                z[k] = qz.T.reshape(rz[k], M[k], rz[k + 1])
            if swp > 0:
                nrmsc = nrmsc * normA[k - 1] * normx[k - 1] / normb[k - 1]
            Q, R = np.linalg.qr(x[k].reshape(rx[k], -1).T)
            prev = np.tensordot(x[k - 1], R.T, axes=([2], [0]))
            rx[k] = Q.shape[1]
            cn = np.linalg.norm(prev)
            if cn > 0:
                prev = prev / cn
            else:
                cn = 1.0
            normx[k - 1] *= cn
            x[k] = Q.T.reshape(rx[k], M[k], rx[k + 1])
            x[k - 1] = prev
            Phis[k] = _phi_xx(False, Phis[k + 1], x[k], x[k])
            Phis_rhs[k] = _phi_ab(False, Phis_rhs[k + 1], A_cores[k], b_cores[k], x[k])
            nb = np.linalg.norm(Phis_rhs[k])
            nb = nb if nb > 0 else 1.0
            normb[k - 1] = nb
            Phis_rhs[k] = Phis_rhs[k] / nb
            nrmsc = nrmsc * normb[k - 1] / (normA[k - 1] * normx[k - 1])
            if not last:
                Phiz[k] = _phi_xx(False, Phiz[k + 1], z[k], x[k]) / normA[k - 1]
                Phiz_rhs[k] = _phi_ab(False, Phiz_rhs[k + 1], A_cores[k], b_cores[k], z[k]) / normb[k - 1]
        max_dx = 0.0
        for k in range(d):
            prev = x[k]
            sol = _local_ab(Phis_rhs[k], Phis_rhs[k + 1], A_cores[k], b_cores[k]) * nrmsc
            nsol = np.linalg.norm(sol)
            dx = np.linalg.norm(sol - prev) / nsol
            max_dx = max(dx, max_dx)
            sol = sol.reshape(rx[k] * M[k], rx[k + 1])
            if k < d - 1:
                u, s, v = np.linalg.svd(sol, full_matrices=False)
                r = rank_chop(s, nsol * eps / d ** (0.5 if last else 1.5))
                r = min(r, s.size, rmax)
            else:
                u, v = np.linalg.qr(sol)
                r = u.shape[1]
                s = np.ones(r)
            u = u[:, :r]
            v = (np.diag(s[:r]) @ v[:r, :]).T
            if not last:
                czx = np.einsum('zr,rmR,ZR->zmZ', Phiz[k], (u @ v.T).reshape(rx[k], M[k], rx[k + 1]), Phiz[k + 1])
                czAB = _local_ab(Phiz_rhs[k], Phiz_rhs[k + 1], A_cores[k], b_cores[k])
                cz = czAB * nrmsc - czx
                uz, _, _ = np.linalg.svd(cz.reshape(rz[k] * M[k], rz[k + 1]), full_matrices=False)
                cz = uz[:, :min(kickrank, uz.shape[1])]
                if k < d - 1:
                    cz = np.concatenate([cz, rng.standard_normal((cz.shape[0], kick2))], 1)
                qz, _ = np.linalg.qr(cz)
                rz[k + 1] = qz.shape[1]
                z[k] = qz.reshape(rz[k], M[k], rz[k + 1])
            if k < d - 1:
                if not last:
                    czx = np.einsum('zr,rmR,ZR->zmZ', Phis[k], (u @ v.T).reshape(rx[k], M[k], rx[k + 1]), Phiz[k + 1])
                    czAB = _local_ab(Phis_rhs[k], Phiz_rhs[k + 1], A_cores[k], b_cores[k])
                    uk = czAB * nrmsc - czx
                    u, Rm = np.linalg.qr(np.concatenate([u, uk.reshape(u.shape[0], -1)], 1))
                    v = np.concatenate([v, np.zeros((rx[k + 1], uk.shape[-1]))], 1) @ Rm.T
                r = u.shape[1]
                v = np.tensordot(v, x[k + 1], axes=([0], [0]))
                nrmsc = nrmsc * normA[k] * normx[k] / normb[k]
                nn = np.linalg.norm(v)
                if nn > 0:
                    v = v / nn
                else:
                    nn = 1.0
                normx[k] *= nn
                x[k] = u.reshape(rx[k], M[k], r)
                x[k + 1] = v.reshape(r, M[k + 1], rx[k + 2])
                rx[k + 1] = r
                Phis[k + 1] = _phi_xx(True, Phis[k], x[k], x[k])
                Phis_rhs[k + 1] = _phi_ab(True, Phis_rhs[k], A_cores[k], b_cores[k], x[k])
                nb = np.linalg.norm(Phis_rhs[k + 1])
                nb = nb if nb > 0 else 1.0
                normb[k] = nb
                Phis_rhs[k + 1] = Phis_rhs[k + 1] / nb
                nrmsc = nrmsc * normb[k] / (normA[k] * normx[k])
                if not last:
                    Phiz[k + 1] = _phi_xx(True, Phiz[k], z[k], x[k]) / normA[k]
                    Phiz_rhs[k + 1] = _phi_ab(True, Phiz_rhs[k], A_cores[k], b_cores[k], z[k]) / normb[k]
            else:
                x[k] = (u @ np.diag(s[:r]) @ v[:r, :].T).reshape(rx[k], M[k], rx[k + 1])
        if last:
            break
        if max_dx < eps:
            last = True
    f = np.exp(np.sum(np.log(normx)) / d)
    return [c * f for c in x]
