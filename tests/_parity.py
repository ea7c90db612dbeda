"""Solve-level parity criteria against the reference's solution on the same inputs.

* relative residual ||A x - b|| / ||b|| <= eps where the reference reaches eps on the same input,
  else <= 2 x the reference's own: the reference stops on its local residual
  (cpp/amen_solve.h:375,525), so its true residual can exceed eps (3.4e-8 at eps 1e-8 on the d=20
  n=64 benchmark solve; from 2e-11 to 7e-10 at eps 1e-10 on the random 4x5x6 system of
  tests/test_solvers.py, depending on the random enrichment start alone);
* ||x - x_ref|| / ||x_ref|| <= max(10 eps, cond(A) (res + res_ref)) where cond(A) is known (small
  dense cases), else <= 10 eps;
* TT ranks within +-kickrank of the reference's.
"""
import numpy as np

from oracle import amen as O


def check(A, b, x, x_ref, eps, kickrank, cond=None, label="", res_slack=1.0, x_ref_alt=None,
          rank_tol=None):
    """``x_ref_alt``: the reference's other solution of the same input (its Python path), when
    recorded; the residual bar then follows the larger of the reference's two residuals (on the
    random 4x5x6 system they are 2.2e-11 and 3.3e-10 at eps 1e-10, so "the reference reaches eps"
    holds for one of its paths only). ``res_slack`` > 1 widens the residual bar (the numpy
    restatement rounds differently from ATen along the same trajectory). ``rank_tol`` overrides
    the rank tolerance (default kickrank)."""
    A = [np.asarray(a) for a in A]
    b = [np.asarray(c) for c in b]
    x = [np.asarray(c) for c in x]
    x_ref = [np.asarray(c) for c in x_ref]
    res = O.tt_relres(A, x, b)
    res_ref = O.tt_relres(A, x_ref, b)
    if x_ref_alt is not None:
        res_ref = max(res_ref, O.tt_relres(A, [np.asarray(c) for c in x_ref_alt], b))
    err = O.tt_relerr(x, x_ref)
    bound = 10 * eps if cond is None else max(10 * eps, cond * (res + res_ref))
    ranks = [c.shape[2] for c in x][:-1]
    ranks_ref = [c.shape[2] for c in x_ref][:-1]
    msg = "%s res %.3e (ref %.3e, bar %.3e) err %.3e (bound %.3e) ranks %s ref %s" % (
        label, res, res_ref, res_slack * res_bound(eps, res_ref), err, bound, ranks, ranks_ref)
    print(msg)
    assert res <= res_slack * res_bound(eps, res_ref), msg
    assert err <= bound, msg
    tol = kickrank if rank_tol is None else rank_tol
    assert all(abs(a - c) <= tol for a, c in zip(ranks, ranks_ref)), msg
    return res, res_ref, err


def dense_cond(A_cores):
    """2-norm condition number of a small TT-matrix via its dense form."""
    d = len(A_cores)
    t = A_cores[0]
    for c in A_cores[1:]:
        t = np.tensordot(t, c, axes=([t.ndim - 1], [0]))
    t = t.reshape(t.shape[1:-1])
    M = [c.shape[1] for c in A_cores]
    N = [c.shape[2] for c in A_cores]
    perm = list(range(0, 2 * d, 2)) + list(range(1, 2 * d, 2))
    mat = t.transpose(perm).reshape(int(np.prod(M)), int(np.prod(N)))
    s = np.linalg.svd(mat, compute_uv=False)
    return float(s[0] / s[-1])


def tt_entries(cores, idx):
    """Entries x(i_1, .., i_d) of a TT-vector at the rows of ``idx`` (S x d)."""
    cores = [np.asarray(c) for c in cores]
    idx = np.asarray(idx, dtype=np.int64)
    v = cores[0][0, idx[:, 0], :]
    for k in range(1, len(cores)):
        v = np.einsum("sr,srR->sR", v, np.transpose(cores[k][:, idx[:, k], :], (1, 0, 2)))
    return v[:, 0]


def sampled_relerr(x, z):
    """Estimate of ||x - x_ref|| / ||x_ref|| from the reference's entries at uniformly drawn
    multi-indices (tests/golden/make_golden.py: sampled_case): the ratio of the sampled
    root-mean-square difference to the sampled root-mean-square of x_ref. Both means estimate
    the squared norms divided by the number of entries, without bias."""
    ref = np.asarray(z["sample_x"])
    got = tt_entries(x, z["sample_idx"])
    return float(np.sqrt(np.mean((got - ref) ** 2)) / np.sqrt(np.mean(ref ** 2)))


def res_bound(eps, res_ref):
    """Residual bar: eps where the reference reaches eps on the same input, else twice the
    reference's own residual (its stopping rule is the local residual, cpp/amen_solve.h:375,525,
    so its true residual can exceed eps)."""
    return eps if res_ref <= eps else 2.0 * res_ref


def check_sampled(A, b, x, z, eps, kickrank, label="", err_bound=None, rank_tol=None):
    """Parity of a solution against a sampled fixture of the reference's: relative residual
    (oracle TT algebra) within ``res_bound``, the TT norm within 10 eps of the reference's, the
    sampled estimate of ||x - x_ref|| / ||x_ref|| within 10 eps (or ``err_bound``), TT ranks within
    +-kickrank."""
    A = [np.asarray(a) for a in A]
    b = [np.asarray(c) for c in b]
    x = [np.asarray(c) for c in x]
    res = O.tt_relres(A, x, b)
    res_ref = float(z["ref_relres"])
    nrm, nrm_ref = O.tt_norm(x), float(z["ref_norm"])
    err = sampled_relerr(x, z)
    ranks = [c.shape[0] for c in x] + [1]
    ranks_ref = [int(r) for r in z["ref_ranks"]]
    eb = 10 * eps if err_bound is None else err_bound
    msg = "%s res %.3e (ref %.3e, bar %.3e) sampled err %.3e (bar %.3e) norm %.12e (ref %.12e) " \
          "ranks %s ref %s" % (label, res, res_ref, res_bound(eps, res_ref), err, eb, nrm, nrm_ref,
                               ranks, ranks_ref)
    print(msg)
    assert res <= res_bound(eps, res_ref), msg
    assert abs(nrm - nrm_ref) <= 10 * eps * nrm_ref, msg
    assert err <= eb, msg
    tol = kickrank if rank_tol is None else rank_tol
    assert all(abs(a - c) <= tol for a, c in zip(ranks, ranks_ref)), msg
    return res, res_ref, err
