// TT norm and TT rounding on the device (see tt_ops.cuh). Cores are row-major r x mode x R;
// a row-major (a x b) matrix is handled as the column-major (b x a) matrix on the same memory.
#include <cmath>

#include "contract.cuh"
#include "tt_ops.cuh"

namespace ttgb {

namespace {

int64_t mode_of(const TTView& x, int k) {
  return x.rows.empty() ? x.cols[k] : x.rows[k] * x.cols[k];
}

}  // namespace

int64_t rank_chop(const std::vector<double>& s, double tol) {
  double total = 0.0;
  for (double v : s) total += v * v;
  if (total == 0.0) return 1;
  const int64_t n = (int64_t)s.size();
  if (tol <= 0.0) return n;
  // tail[r] = sum_{k >= r} s_k^2, decreasing in r: the first r with tail[r] < tol^2
  double tail = 0.0;
  int64_t r = n;
  for (int64_t k = n - 1; k >= 0; --k) {
    tail += s[k] * s[k];
    if (tail < tol * tol) r = k; else break;
  }
  if (r == n) return n;   // even the smallest singular value alone is above the threshold
  return r > 0 ? r : 1;
}

std::vector<DTensor> tt_matvec(const TTView& A, const TTView& x, cudaStream_t s,
                               std::vector<int64_t>& ranks) {
  const int d = A.d;
  TTGB_REQUIRE(d >= 1 && x.d == d && !A.rows.empty() && x.rows.empty(),
               "Only TT-matrix @ TT-vector is supported here.");
  std::vector<DTensor> out(d);
  ranks.assign(d + 1, 1);
  for (int k = 0; k < d; ++k) {
    TTGB_REQUIRE(A.cols[k] == x.cols[k], "Shapes are incompatible.");
    const int64_t sa = A.ranks[k], Sa = A.ranks[k + 1], M = A.rows[k], N = A.cols[k];
    const int64_t r = x.ranks[k], R = x.ranks[k + 1];
    ranks[k + 1] = Sa * R;
    out[k] = DTensor({sa * r, M, Sa * R}, s);
    // per s: C[(m, S), (r, R)] = sum_n A[s](m, S; n) x(n; r, R), written into y[s, r, m, S, R]
    ContractDesc c;
    c.M = (int)(M * Sa); c.N = (int)(r * R); c.K = (int)N; c.batch = (int)sa;
    c.A = A.cores[k];
    c.am = Ax::two(Sa, N * Sa, 1);
    c.ak = Ax::one(Sa);
    c.a_bs = M * N * Sa;
    c.B = x.cores[k];
    c.bk = Ax::one(R);
    c.bn = Ax::two(R, N * R, 1);
    c.b_bs = 0;
    c.C = out[k].data();
    c.cm = Ax::two(Sa, Sa * R, R);
    c.cn = Ax::two(R, M * Sa * R, 1);
    c.c_bs = r * M * Sa * R;
    contract(c, s);
  }
  ranks[0] = A.ranks[0] * x.ranks[0];
  return out;
}

double tt_norm(const TTView& x, LinalgWS& ws, const RedWS& red, cudaStream_t s) {
  const int d = x.d;
  TTGB_REQUIRE(d >= 1, "empty TT");
  DBuf T, Rf, CT, out;
  out.reset(1, s);
  // CT = Cur^T (rc x R_{k+1}, column-major, ld rc), Cur = I_1 at the right end
  int64_t rc = 1;
  for (int k = d - 1; k >= 0; --k) {
    const int64_t r = x.ranks[k], n = mode_of(x, k), R = x.ranks[k + 1];
    const double* W;   // T_k as the column-major (n rc) x r matrix (ld n rc)
    if (k == d - 1) {
      W = x.cores[k];  // R = 1, Cur = [1]
      rc = 1;
    } else {
      T.ensure((size_t)rc * n * r, s);
      // T (rc x r n, column-major) = CT (rc x R) * core_k (R x r n, column-major view, ld R)
      gemm_cm(CT.p, rc, x.cores[k], R, T.p, rc, rc, r * n, R, 1.0, 0.0, s);
      W = T.p;
    }
    const int64_t m = n * rc;
    if (k == 0) {   // r = 1 and the right part is orthonormal: ||x|| = ||T_0||
      nrm2(red, W, m * r, out.p, s);
      break;
    }
    // R factor of the unfolding by TSQR (robust when it is rank deficient, as the unfoldings of
    // a residual A x - b are): an r x r upper block, rows past min(m, r) zero
    Rf.ensure((size_t)r * r, s);
    qr_r(W, m, m, r, Rf.p, ws, s);
    // Cur_new = Rf^T (r x r): CT_new = Rf (r x r, ld r)
    CT.ensure((size_t)r * r, s);
    copy(Rf.p, CT.p, r * r, s);
    rc = r;
  }
  double h = 0.0;
  TTGB_CUDA(cudaMemcpyAsync(&h, out.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  TTGB_CUDA(cudaStreamSynchronize(s));
  return h;
}

std::vector<DTensor> tt_round(const TTView& x, double eps, int64_t rmax, LinalgWS& ws,
                              const RedWS& red, cudaStream_t s, std::vector<int64_t>& ranks) {
  const int d = x.d;
  TTGB_REQUIRE(d >= 1, "empty TT");
  TTGB_REQUIRE(rmax >= 1, "rmax must be positive");
  std::vector<int64_t> mode(d);
  for (int k = 0; k < d; ++k) mode[k] = mode_of(x, k);
  ranks.assign(x.ranks.begin(), x.ranks.end());
  std::vector<DTensor> cores(d);
  for (int k = 0; k < d; ++k) {
    cores[k] = DTensor({ranks[k], mode[k], ranks[k + 1]}, s);
    copy(x.cores[k], cores[k].data(), cores[k].numel(), s);
  }
  if (d == 1) return cores;

  DBuf Xc, Q, Rf, U, S, Vh;
  // left-to-right orthogonalisation (lr_orthogonal, torchtt/_decomposition.py:62-113)
  for (int i = 0; i < d - 1; ++i) {
    const int64_t rm = ranks[i] * mode[i], R = ranks[i + 1];
    const int64_t k = std::min(rm, R);
    Xc.ensure((size_t)rm * R, s);
    transpose(cores[i].data(), R, Xc.p, rm, R, rm, s);        // column-major rm x R
    Q.ensure((size_t)rm * k, s);
    Rf.ensure((size_t)k * R, s);
    qr(Xc.p, rm, rm, R, Q.p, Rf.p, ws, red, s);
    DTensor qi({ranks[i], mode[i], k}, s);
    transpose(Q.p, rm, qi.data(), k, rm, k, s);               // row-major rm x k
    const int64_t nx = mode[i + 1] * ranks[i + 2];
    DTensor nxt({k, mode[i + 1], ranks[i + 2]}, s);
    // next (k x nx, row-major) = Rf (k x R) * core_{i+1} (R x nx, row-major)
    gemm_cm(cores[i + 1].data(), nx, Rf.p, k, nxt.data(), nx, nx, k, R, 1.0, 0.0, s, false, true);
    cores[i] = std::move(qi);
    cores[i + 1] = std::move(nxt);
    ranks[i + 1] = k;
  }

  // right-to-left truncation (round_tt, torchtt/_decomposition.py:197-226)
  const double ep = eps / std::sqrt((double)(d - 1));
  std::vector<double> hs;
  for (int i = d - 1; i > 0; --i) {
    const int64_t Ri = ranks[i], cols = mode[i] * ranks[i + 1];
    const int64_t k = std::min(cols, Ri);
    // core_i as the row-major Ri x cols matrix M; its memory is the column-major Y = M^T
    // (cols x Ri). Y = U' S Vh'  =>  M = Vh'^T S U'^T.
    U.ensure((size_t)cols * k, s);
    S.ensure((size_t)k, s);
    Vh.ensure((size_t)k * Ri, s);
    svd(cores[i].data(), cols, cols, Ri, U.p, S.p, Vh.p, ws, red, s);
    hs.resize(k);
    TTGB_CUDA(cudaMemcpyAsync(hs.data(), S.p, k * sizeof(double), cudaMemcpyDeviceToHost, s));
    TTGB_CUDA(cudaStreamSynchronize(s));
    double nrm = 0.0;
    for (double v : hs) nrm += v * v;
    nrm = std::sqrt(nrm);
    const int64_t rn = std::min(rmax, rank_chop(hs, nrm * ep));
    // core_i <- U'^T[:rn] (row-major rn x cols): the first rn columns of U' (ld cols)
    DTensor ci({rn, mode[i], ranks[i + 1]}, s);
    copy(U.p, ci.data(), rn * cols, s);
    // core_{i-1} <- core_{i-1} (rm x Ri) * Vh'^T[:, :rn] diag(S[:rn]); as column-major
    // (rn x rm) = diag(S) Vh'[:rn, :] (rn x Ri, ld k) * core_{i-1}^T (Ri x rm, ld Ri)
    const int64_t rm = ranks[i - 1] * mode[i - 1];
    DTensor cp({ranks[i - 1], mode[i - 1], rn}, s);
    gemm_cm(Vh.p, k, cores[i - 1].data(), Ri, cp.data(), rn, rn, rm, Ri, 1.0, 0.0, s);
    scale_rows_cm(cp.data(), rn, rn, rm, S.p, s);
    cores[i] = std::move(ci);
    cores[i - 1] = std::move(cp);
    ranks[i] = rn;
  }
  return cores;
}

}  // namespace ttgb
