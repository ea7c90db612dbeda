// Two-site DMRG matvec on the device (see dmrg.cuh). The sweep follows cpp/dmrg_mv.h:23-230:
// a right-to-left QR orthogonalisation of y with the backward interfaces Phi[y, A, x], then a
// left-to-right pass that forms each two-site block W = Phi_k (A_k x_k)(A_{k+1} x_{k+1}) Phi_{k+2},
// compares it with the current y_k y_{k+1}, truncates its SVD (rank_chop at eps ||W|| / d^1.5,
// d^0.5 in the last sweep, plus an adaptive enlargement), adds kickrank random directions and
// updates the forward interface. The two-site block is one local product whose right interface is
// the right half Psi of site k+1; every contraction runs on the library's engines (structured A
// stage for sparse A cores), the SVD/QR on linalg.cu.
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "blas1.cuh"
#include "contract.cuh"
#include "dmrg.cuh"
#include "linalg.cuh"
#include "sparse_a.cuh"
#include "tt_ops.cuh"

namespace ttgb {

namespace {

// Psi[m2, L, S, R] = sum_{n2, S'} A[S, m2, n2, S'] sum_{R'} Phi[L, S', R'] x[R, n2, R']
// (A: S x M2 x N2 x S2, x: R x N2 x R2, Phi: L x S2 x R2). T holds L*S2*N2*R doubles.
void right_half(const double* A, const SparseCore* sp, const double* x, const double* phi,
                int64_t S, int64_t M2, int64_t N2, int64_t S2, int64_t R, int64_t R2, int64_t L,
                double* T, double* Psi, cudaStream_t s) {
  {  // T[L, S', n2, R] = sum_{R'} Phi[(L, S'), R'] x[(R, n2), R']
    ContractDesc c;
    c.M = (int)(L * S2); c.N = (int)(R * N2); c.K = (int)R2;
    c.A = phi; c.am = Ax::one(R2); c.ak = Ax::one(1);
    c.B = x; c.bk = Ax::one(1); c.bn = Ax::one(R2);
    c.C = T; c.cm = Ax::one(N2 * R); c.cn = Ax::two(N2, 1, R);
    contract(c, s);
  }
  if (sp && sp->use) {   // key (S, m2), pairs (n2, S'), free (L, R)
    StageDims g{L, R, S2 * N2 * R, S * R, L * S * R, R, N2 * R};
    g.ke0 = M2;
    g.sk1 = R;
    sparse_stage(sp->rh, T, Psi, g, s);
    return;
  }
  ContractDesc c;   // rows (S, m2), cols (L, R), K (n2, S')
  c.M = (int)(S * M2); c.N = (int)(L * R); c.K = (int)(N2 * S2);
  c.A = A; c.am = Ax::one(N2 * S2); c.ak = Ax::one(1);
  c.B = T; c.bk = Ax::two(S2, R, N2 * R); c.bn = Ax::two(R, S2 * N2 * R, 1);
  c.C = Psi; c.cm = Ax::two(M2, R, L * S * R); c.cn = Ax::two(R, S * R, 1);
  contract(c, s);
}

__global__ void scale_cols_cm_kernel(double* X, int64_t ld, int64_t rows, int64_t cols,
                                     const double* S) {
  const int64_t total = rows * cols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % rows, j = t / rows;
    X[i + j * ld] *= S[j];
  }
}

void scale_cols_cm(double* X, int64_t ld, int64_t rows, int64_t cols, const double* S,
                   cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return;
  unsigned g = cdiv(rows * cols, 256);
  if (g > 4096) g = 4096;
  scale_cols_cm_kernel<<<g, 256, 0, s>>>(X, ld, rows, cols, S);
  TTGB_CHECK_LAUNCH();
}

}  // namespace

std::vector<DTensor> dmrg_matvec(const TTView& A, const TTView& x, const TTView& y0,
                                 const DmrgParams& p, cudaStream_t s, std::vector<int64_t>& ry,
                                 DmrgStats* stats, LinalgWS& ws, const RedWS& red) {
  const int d = A.d;
  TTGB_REQUIRE(d >= 1 && x.d == d && !A.rows.empty() && x.rows.empty(),
               "A must be a TT-matrix and x a TT-vector.");
  for (int k = 0; k < d; ++k) TTGB_REQUIRE(A.cols[k] == x.cols[k], "Shapes are incompatible.");
  TTGB_REQUIRE(p.nswp >= 1 && p.rmax >= 1 && p.kickrank >= 0, "invalid DMRG parameters");
  const std::vector<int64_t>& M = A.rows;
  const std::vector<int64_t>& N = A.cols;
  const std::vector<int64_t>& rA = A.ranks;
  const std::vector<int64_t>& rx = x.ranks;
  if (d == 1) {   // a single core: the product itself
    std::vector<int64_t> rk;
    auto out = tt_matvec(A, x, s, rk);
    ry = rk;
    if (stats) { stats->sweeps = 0; stats->max_delta = 0.0; }
    return out;
  }
  std::vector<SparseCore> sp(d);
  for (int k = 0; k < d; ++k) sp[k].build(A.cores[k], rA[k], M[k], N[k], rA[k + 1], s);

  std::vector<DTensor> y(d);
  uint64_t rng = 0;
  if (y0.d == 0) {   // random start of rank 2 (cpp/dmrg_mv.h:42-50)
    ry.assign(d + 1, 2);
    ry[0] = ry[d] = 1;
    for (int k = 0; k < d; ++k) {
      y[k] = DTensor({ry[k], M[k], ry[k + 1]}, s);
      randn(y[k].data(), y[k].numel(), p.seed, rng, s);
      rng += (uint64_t)y[k].numel();
    }
  } else {
    TTGB_REQUIRE(y0.d == d && y0.rows.empty(), "y0 must be a TT-vector of the shape of A x.");
    ry = y0.ranks;
    for (int k = 0; k < d; ++k) {
      TTGB_REQUIRE(y0.cols[k] == M[k], "y0 must be a TT-vector of the shape of A x.");
      y[k] = DTensor({ry[k], M[k], ry[k + 1]}, s);
      copy(y0.cores[k], y[k].data(), y[k].numel(), s);
    }
  }
  std::vector<DTensor> Phi(d + 1);
  Phi[0] = DTensor({1, 1, 1}, s);
  Phi[d] = DTensor({1, 1, 1}, s);
  fill(Phi[0].data(), 1.0, 1, s);
  fill(Phi[d].data(), 1.0, 1, s);

  std::vector<double> delta(d - 1, 1.0), delta_prev(d - 1, 1.0);
  std::vector<int64_t> renl(d, 2);
  DBuf wphi, w1, w2, T, Psi, scal((size_t)4, s);
  double* hscal = nullptr;
  TTGB_CUDA(cudaMallocHost((void**)&hscal, 4 * sizeof(double)));
  struct HostFree { double* p; ~HostFree() { cudaFreeHost(p); } } hf{hscal};
  std::vector<double> hs;
  bool last = false;
  int swp = 0;
  double maxdelta = 0.0;
  for (swp = 0; swp < p.nswp; ++swp) {
    // right-to-left: QR of the (M_k ry_{k+1}) x ry_k view of y_k, R absorbed into y_{k-1}
    for (int k = d - 1; k > 0; --k) {
      const int64_t m = M[k] * ry[k + 1], r = ry[k];
      const int64_t rnew = std::min(m, r);
      DTensor Q({rnew, M[k], ry[k + 1]}, s);
      DBuf R((size_t)(rnew * r), s);
      qr(y[k].data(), m, m, r, Q.data(), R.p, ws, red, s);
      const int64_t a = ry[k - 1] * M[k - 1];
      DTensor prev({ry[k - 1], M[k - 1], rnew}, s);
      // prev (a x rnew, row-major) = y_{k-1} (a x r) R^T: column-major R (rnew x r) y_{k-1}^T
      gemm_cm(R.p, rnew, y[k - 1].data(), r, prev.data(), rnew, rnew, a, r, 1.0, 0.0, s);
      y[k] = std::move(Q);
      y[k - 1] = std::move(prev);
      ry[k] = rnew;
      PhiDims pd{ry[k], ry[k + 1], rA[k], rA[k + 1], rx[k], rx[k + 1], M[k], N[k]};
      wphi.ensure(phi_A_workspace(pd), s);
      Phi[k] = DTensor({ry[k], rA[k], rx[k]}, s);
      phi_bck_A(pd, Phi[k + 1].data(), y[k].data(), A.cores[k], x.cores[k], Phi[k].data(), wphi.p, s,
                &sp[k]);
    }
    // left-to-right: two-site blocks
    maxdelta = 0.0;
    for (int k = 0; k < d - 1; ++k) {
      const int64_t p1 = ry[k] * M[k], q2 = M[k + 1] * ry[k + 2];
      DBuf Wprev((size_t)(p1 * q2), s), W((size_t)(p1 * q2), s);
      // W_prev (p1 x q2 row-major) = y_k y_{k+1}: column-major W_prev^T = y_{k+1}^T y_k^T
      gemm_cm(y[k + 1].data(), q2, y[k].data(), ry[k + 1], Wprev.p, q2, q2, p1, ry[k + 1], 1.0, 0.0, s);
      if (!last) {
        const int64_t L = ry[k + 2], S1 = rA[k + 1], S2 = rA[k + 2], R1 = rx[k + 1], R2 = rx[k + 2];
        T.ensure((size_t)(L * S2 * N[k + 1] * R1), s);
        Psi.ensure((size_t)(M[k + 1] * L * S1 * R1), s);
        right_half(A.cores[k + 1], &sp[k + 1], x.cores[k + 1], Phi[k + 2].data(), S1, M[k + 1],
                   N[k + 1], S2, R1, R2, L, T.p, Psi.p, s);
        LocalOpDims ld{ry[k], rA[k], rx[k], M[k], N[k], S1, M[k + 1] * L, R1};
        w1.ensure(local_product_w1(ld), s);
        w2.ensure(local_product_w2(ld), s);
        local_product(ld, Phi[k].data(), A.cores[k], Psi.p, x.cores[k], W.p, w1.p, w2.p, s, 1.0,
                      0.0, &sp[k]);
      } else {
        copy(Wprev.p, W.p, p1 * q2, s);
      }
      nrm2(red, W.p, p1 * q2, scal.p, s);
      sub(W.p, Wprev.p, Wprev.p, p1 * q2, s);
      nrm2(red, Wprev.p, p1 * q2, scal.p + 1, s);
      TTGB_CUDA(cudaMemcpyAsync(hscal, scal.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
      TTGB_CUDA(cudaStreamSynchronize(s));
      const double b = hscal[0];
      delta[k] = b > 0.0 ? hscal[1] / b : 0.0;
      const double ratio = delta[k] / delta_prev[k];
      if (ratio >= 1.0 && delta[k] > p.eps) renl[k] += 1;
      if (ratio < 0.1 && delta[k] < p.eps) renl[k] = std::max<int64_t>(renl[k] - 1, 1);
      maxdelta = std::max(maxdelta, delta[k]);

      // SVD of W (p1 x q2 row-major) through its column-major view W^T = U S Vh:
      // W = Vh^T S U^T, left factor Vh^T (p1 x kk), right factor S U^T (kk x q2)
      const int64_t kk = std::min(p1, q2);
      DBuf U((size_t)(q2 * kk), s), Sv((size_t)kk, s), Vh((size_t)(kk * p1), s);
      // W = F1 F2^T with a small inner dimension K: outside the last sweep F1 = Y2 (p1 x K, the
      // local product's intermediate in w2) and F2 = Psi (q2 x K), K = rA_{k+1} rx_{k+1}; in the
      // last sweep W = y_k y_{k+1}, K = ry_{k+1}. Then W = Q_L (R_L R_R^T) Q_R^T from the QRs of the
      // two tall factors and the SVD of the small K x K core: the singular triplets of W.
      const int64_t K = last ? ry[k + 1] : rA[k + 1] * rx[k + 1];
      if (K < kk) {
        DBuf Lc((size_t)(p1 * K), s), Rc;
        const double* F2cm = nullptr;   // F2 in column-major (q2 x K, ld q2)
        if (last) {
          transpose(y[k].data(), K, Lc.p, p1, K, p1, s);   // y_k (p1 x K row-major) -> column-major
          F2cm = y[k + 1].data();                         // y_{k+1} (K x q2 row-major) == F2 column-major
        } else {
          transpose(w2.p, K, Lc.p, p1, K, p1, s);         // Y2 (p1 x K row-major) -> column-major
          Rc.reset((size_t)(q2 * K), s);
          transpose(Psi.p, K, Rc.p, q2, K, q2, s);        // Psi (q2 x K row-major) -> column-major
          F2cm = Rc.p;
        }
        DBuf QL((size_t)(p1 * K), s), RL((size_t)(K * K), s), QR_((size_t)(q2 * K), s), RR((size_t)(K * K), s);
        qr(Lc.p, p1, p1, K, QL.p, RL.p, ws, red, s);
        qr(F2cm, q2, q2, K, QR_.p, RR.p, ws, red, s);
        DBuf Cc((size_t)(K * K), s), Uc((size_t)(K * K), s), Sc((size_t)K, s), Vc((size_t)(K * K), s);
        gemm_cm(RL.p, K, RR.p, K, Cc.p, K, K, K, K, 1.0, 0.0, s, false, true);   // R_L R_R^T
        svd(Cc.p, K, K, K, Uc.p, Sc.p, Vc.p, ws, red, s);
        // right singular vectors Q_R Vc^T (q2 x K) -> U[:, :K]; left Q_L Uc (p1 x K) -> Vh[:K, :]
        gemm_cm(QR_.p, q2, Vc.p, K, U.p, q2, q2, K, K, 1.0, 0.0, s, false, true);
        DBuf Lf((size_t)(p1 * K), s);
        gemm_cm(QL.p, p1, Uc.p, K, Lf.p, p1, p1, K, K, 1.0, 0.0, s);
        fill(Vh.p, 0.0, kk * p1, s);
        fill(Sv.p, 0.0, kk, s);
        transpose(Lf.p, p1, Vh.p, kk, p1, K, s);            // Vh (kk x p1, ld kk) rows 0..K-1
        copy(Sc.p, Sv.p, K, s);
        fill(U.p + q2 * K, 0.0, q2 * (kk - K), s);
      } else {
        svd(W.p, q2, q2, p1, U.p, Sv.p, Vh.p, ws, red, s);
      }
      hs.resize(kk);
      TTGB_CUDA(cudaMemcpyAsync(hs.data(), Sv.p, kk * sizeof(double), cudaMemcpyDeviceToHost, s));
      TTGB_CUDA(cudaStreamSynchronize(s));
      int64_t rn = rank_chop(hs, b * p.eps / std::pow((double)d, last ? 0.5 : 1.5));
      if (!last) rn += renl[k];
      rn = std::max<int64_t>(1, std::min({rn, kk, p.rmax}));
      // G (rn x q2 row-major) = S U^T rows: the first rn columns of U, column j scaled by S_j
      DBuf G((size_t)(rn * q2), s);
      copy(U.p, G.p, rn * q2, s);
      scale_cols_cm(G.p, q2, q2, rn, Sv.p, s);
      DTensor yk, yk1;
      if (swp < p.nswp - 1) {   // kick: QR([W1, randn]), the right factor absorbs R
        const int64_t nc = rn + p.kickrank;
        const int64_t kk2 = std::min(p1, nc);
        DBuf W1((size_t)(p1 * nc), s), Q((size_t)(p1 * kk2), s), Rm((size_t)(kk2 * nc), s);
        transpose(Vh.p, kk, W1.p, p1, rn, p1, s);   // W1 (p1 x rn col-major) = Vh[:rn, :]^T
        if (p.kickrank > 0) {
          randn(W1.p + p1 * rn, p1 * p.kickrank, p.seed, rng, s);
          rng += (uint64_t)(p1 * p.kickrank);
        }
        qr(W1.p, p1, p1, nc, Q.p, Rm.p, ws, red, s);
        yk = DTensor({ry[k], M[k], kk2}, s);
        transpose(Q.p, p1, yk.data(), kk2, p1, kk2, s);
        // y_{k+1} (kk2 x q2 row-major) = Rm[:, :rn] G: column-major G^T-view (q2 x rn) Rm^T
        yk1 = DTensor({kk2, M[k + 1], ry[k + 2]}, s);
        gemm_cm(G.p, q2, Rm.p, kk2, yk1.data(), q2, q2, kk2, rn, 1.0, 0.0, s, false, true);
        rn = kk2;
      } else {
        yk = DTensor({ry[k], M[k], rn}, s);
        copy2d(Vh.p, kk, yk.data(), rn, p1, rn, s);   // y_k (p1 x rn row-major) = Vh[:rn, :]^T
        yk1 = DTensor({rn, M[k + 1], ry[k + 2]}, s);
        copy(G.p, yk1.data(), rn * q2, s);
      }
      if (p.verbose)
        std::printf("\tcore %d: delta %g rank %lld -> %lld\n", k, delta[k], (long long)ry[k + 1],
                    (long long)rn);
      y[k] = std::move(yk);
      y[k + 1] = std::move(yk1);
      ry[k + 1] = rn;
      PhiDims pd{ry[k], ry[k + 1], rA[k], rA[k + 1], rx[k], rx[k + 1], M[k], N[k]};
      wphi.ensure(phi_A_workspace(pd), s);
      Phi[k + 1] = DTensor({ry[k + 1], rA[k + 1], rx[k + 1]}, s);
      phi_fwd_A(pd, Phi[k].data(), y[k].data(), A.cores[k], x.cores[k], Phi[k + 1].data(), wphi.p, s,
                &sp[k]);
    }
    if (last) break;
    if (maxdelta < p.eps) last = true;
    delta_prev = delta;
  }
  if (stats) {
    stats->sweeps = std::min(swp + 1, p.nswp);
    stats->max_delta = maxdelta;
  }
  TTGB_CUDA(cudaStreamSynchronize(s));
  return y;
}

}  // namespace ttgb
