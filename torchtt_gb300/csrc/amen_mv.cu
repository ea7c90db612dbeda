// AMEn matvec on the device (see amen_mv.cuh). The sweep restates _amen_mm_python
// (torchtt/_amen.py:126-410) for a TT-vector b: a right-to-left pass that updates the enrichment
// z, orthogonalises x by QR and refreshes the interfaces (x-x, x-(A,b), z-x, z-(A,b)) with the norm
// bookkeeping normx/normb/nrmsc; then a left-to-right pass in which the local solution is the
// projection of A b (one local product), truncated by SVD (rank_chop at eps ||.|| / d^1.5, d^0.5
// in the last sweep), enriched with the projected residual and moved to the next core. All
// contractions run on the library's engines (structured A stage for sparse A cores), QR/SVD on
// linalg.cu; the host reads only norms and singular values.
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "amen_mv.cuh"
#include "blas1.cuh"
#include "contract.cuh"
#include "sparse_a.cuh"
#include "tt_ops.cuh"

namespace ttgb {

namespace {

__global__ void scale_cols_kernel(double* X, int64_t ld, int64_t rows, int64_t cols,
                                  const double* S) {
  const int64_t total = rows * cols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % rows, j = t / rows;
    X[i + j * ld] *= S[j];
  }
}

class AmenMv {
 public:
  AmenMv(const TTView& A, const TTView& b, const AmenMvParams& p, cudaStream_t s, LinalgWS& ws,
         const RedWS& red)
      : A_(A), b_(b), p_(p), s_(s), ws_(ws), red_(red), d_(A.d), M_(A.rows), K_(A.cols),
        rA_(A.ranks), rb_(b.ranks) {
    sp_.resize(d_);
    for (int k = 0; k < d_; ++k) sp_[k].build(A.cores[k], rA_[k], M_[k], K_[k], rA_[k + 1], s_);
    scal_.reset(4, s_);
    TTGB_CUDA(cudaMallocHost((void**)&h_, 4 * sizeof(double)));
  }
  ~AmenMv() {
    cudaStreamSynchronize(s_);
    if (h_) cudaFreeHost(h_);
  }
  std::vector<DTensor> run(const TTView& x0, std::vector<int64_t>& ranks, AmenMvStats* st);

 private:
  const TTView& A_;
  const TTView& b_;
  AmenMvParams p_;
  cudaStream_t s_;
  LinalgWS& ws_;
  const RedWS& red_;
  int d_;
  std::vector<int64_t> M_, K_, rA_, rb_, rx_, rz_;
  std::vector<SparseCore> sp_;
  std::vector<DTensor> x_, z_, Ps_, Pr_, Pz_, Pzr_;
  DBuf scal_, w1_, w2_, wphi_, wrhs_;
  double* h_ = nullptr;
  uint64_t rng_ = 0;

  double norm(const double* v, int64_t n) {
    nrm2(red_, v, n, scal_.p, s_);
    TTGB_CUDA(cudaMemcpyAsync(h_, scal_.p, sizeof(double), cudaMemcpyDeviceToHost, s_));
    TTGB_CUDA(cudaStreamSynchronize(s_));
    return h_[0];
  }
  void scale(double* v, int64_t n, double f) { scale_copy(v, f, v, n, s_); }
  void fill_randn(double* v, int64_t n) {
    randn(v, n, p_.seed, rng_, s_);
    rng_ += (uint64_t)n;
  }

  // out[l, M, L] = sum Phi_l[l, a, c] A_k[a, M, K, A'] b_k[c, K, C'] Phi_r[L, A', C']
  void local_ab(const DTensor& pl, const DTensor& pr, int k, double* out) {
    LocalOpDims ld{pl.dim(0), rA_[k], rb_[k], M_[k], K_[k], rA_[k + 1], pr.dim(0), rb_[k + 1]};
    w1_.ensure(local_product_w1(ld), s_);
    w2_.ensure(local_product_w2(ld), s_);
    local_product(ld, pl.data(), A_.cores[k], pr.data(), b_.cores[k], out, w1_.p, w2_.p, s_, 1.0,
                  0.0, &sp_[k]);
  }
  // interfaces with (A, b): backward Phi[r, a, c] from Phi_next[R, A', C'] and core[r, M, R]
  DTensor phi_ab(bool fwd, const DTensor& phi, const double* core, int64_t r, int64_t R, int k) {
    PhiDims pd{r, R, rA_[k], rA_[k + 1], rb_[k], rb_[k + 1], M_[k], K_[k]};
    wphi_.ensure(phi_A_workspace(pd), s_);
    if (fwd) {
      DTensor out({R, rA_[k + 1], rb_[k + 1]}, s_);
      phi_fwd_A(pd, phi.data(), core, A_.cores[k], b_.cores[k], out.data(), wphi_.p, s_, &sp_[k]);
      return out;
    }
    DTensor out({r, rA_[k], rb_[k]}, s_);
    phi_bck_A(pd, phi.data(), core, A_.cores[k], b_.cores[k], out.data(), wphi_.p, s_, &sp_[k]);
    return out;
  }
  // interfaces between two cores over M_k: backward Phi[l, r], forward Phi[L, R]
  DTensor phi_xx(bool fwd, const DTensor& phi, const double* left, int64_t l, int64_t L,
                 const double* right, int64_t r, int64_t R, int k) {
    PhiRhsDims pd{l, L, r, R, M_[k]};
    wphi_.ensure(phi_rhs_workspace(pd), s_);
    if (fwd) {
      DTensor out({L, R}, s_);
      phi_fwd_rhs(pd, phi.data(), left, right, out.data(), wphi_.p, s_);
      return out;
    }
    DTensor out({l, r}, s_);
    phi_bck_rhs(pd, phi.data(), left, right, out.data(), wphi_.p, s_);
    return out;
  }
  // out[z, M, Z] = sum P1[z, r] core[r, M, R] P2[Z, R]   (P1: z x r, P2: Z x R)
  void proj(const DTensor& P1, const double* core, const DTensor& P2, int k, double* out) {
    const int64_t z = P1.dim(0), r = P1.dim(1), Z = P2.dim(0), R = P2.dim(1);
    DBuf t1((size_t)(r * z), s_), t2((size_t)(R * Z), s_);
    transpose(P1.data(), r, t1.p, z, r, z, s_);   // t1 (r x z row-major) = P1^T
    transpose(P2.data(), R, t2.p, Z, R, Z, s_);   // t2 (R x Z row-major) = P2^T
    wrhs_.ensure(local_rhs_workspace(r, M_[k], R, z, Z), s_);
    local_rhs(r, M_[k], R, z, Z, t1.p, core, t2.p, 1.0, out, wrhs_.p, s_);
  }
};

std::vector<DTensor> AmenMv::run(const TTView& x0, std::vector<int64_t>& ranks, AmenMvStats* st) {
  const int d = d_;
  const double eps = p_.eps;
  // x start: zeros of rank 1 (torchtt/_amen.py:134-137) or the given cores
  x_.resize(d);
  rx_.assign(d + 1, 1);
  if (x0.d == 0) {
    for (int k = 0; k < d; ++k) {
      x_[k] = DTensor({1, M_[k], 1}, s_);
      fill(x_[k].data(), 0.0, M_[k], s_);
    }
  } else {
    TTGB_REQUIRE(x0.d == d && x0.rows.empty(), "x0 must be a TT-vector of the shape of A b.");
    rx_ = x0.ranks;
    for (int k = 0; k < d; ++k) {
      TTGB_REQUIRE(x0.cols[k] == M_[k], "x0 must be a TT-vector of the shape of A b.");
      x_[k] = DTensor({rx_[k], M_[k], rx_[k + 1]}, s_);
      copy(x0.cores[k], x_[k].data(), x_[k].numel(), s_);
    }
  }
  // z: random of rank kickrank + kick2, right-to-left orthogonalised (_amen.py:145-151)
  rz_.assign(d + 1, p_.kickrank + p_.kick2);
  rz_[0] = rz_[d] = 1;
  z_.resize(d);
  for (int k = 0; k < d; ++k) {
    z_[k] = DTensor({rz_[k], M_[k], rz_[k + 1]}, s_);
    fill_randn(z_[k].data(), z_[k].numel());
  }
  for (int k = d - 1; k > 0; --k) {
    const int64_t m = M_[k] * rz_[k + 1], r = rz_[k], kk = std::min(m, r);
    DTensor Q({kk, M_[k], rz_[k + 1]}, s_);
    DBuf R((size_t)(kk * r), s_);
    qr(z_[k].data(), m, m, r, Q.data(), R.p, ws_, red_, s_);
    const int64_t a = rz_[k - 1] * M_[k - 1];
    DTensor prev({rz_[k - 1], M_[k - 1], kk}, s_);
    gemm_cm(R.p, kk, z_[k - 1].data(), r, prev.data(), kk, kk, a, r, 1.0, 0.0, s_);
    z_[k] = std::move(Q);
    z_[k - 1] = std::move(prev);
    rz_[k] = kk;
  }
  auto ones = [&](std::vector<int64_t> dims) {
    DTensor t(dims, s_);
    fill(t.data(), 1.0, t.numel(), s_);
    return t;
  };
  for (auto* v : {&Ps_, &Pr_, &Pz_, &Pzr_}) {
    v->clear();
    v->resize(d + 1);
  }
  Ps_[0] = ones({1, 1}); Ps_[d] = ones({1, 1});
  Pr_[0] = ones({1, 1, 1}); Pr_[d] = ones({1, 1, 1});
  Pz_[0] = ones({1, 1}); Pz_[d] = ones({1, 1});
  Pzr_[0] = ones({1, 1, 1}); Pzr_[d] = ones({1, 1, 1});
  std::vector<double> normA(std::max(d - 1, 1), 1.0), normb(std::max(d - 1, 1), 1.0),
      normx(std::max(d - 1, 1), 1.0);
  double nrmsc = 1.0;
  bool last = false;
  int swp = 0;
  double max_dx = 0.0;
  std::vector<double> hs;
  for (swp = 0; swp < p_.nswp; ++swp) {
    // ---- right to left --------------------------------------------------------------------
    for (int k = d - 1; k > 0; --k) {
      const int64_t M = M_[k];
      if (!last) {   // z update (_amen.py:195-220)
        DBuf czm;    // column-major (M rz_{k+1}) x kc directions
        const int64_t X = M * rz_[k + 1];
        int64_t kc = 0;
        if (swp > 0) {
          DBuf czx((size_t)(rz_[k] * X), s_), czab((size_t)(rz_[k] * X), s_);
          proj(Pz_[k], x_[k].data(), Pz_[k + 1], k, czx.p);
          local_ab(Pzr_[k], Pzr_[k + 1], k, czab.p);
          axpby(-1.0, czx.p, nrmsc, czab.p, rz_[k] * X, s_);   // czAB nrmsc - czx
          const int64_t kf = std::min(rz_[k], X);
          DBuf U((size_t)(X * kf), s_), S((size_t)kf, s_), Vh((size_t)(kf * rz_[k]), s_);
          svd(czab.p, X, X, rz_[k], U.p, S.p, Vh.p, ws_, red_, s_);   // right singular vectors
          const int64_t tk = std::min<int64_t>(p_.kickrank, kf);
          kc = tk + ((k < d - 1) ? p_.kick2 : 0);
          czm.reset((size_t)(X * kc), s_);
          copy(U.p, czm.p, X * tk, s_);
          if (kc > tk) fill_randn(czm.p + X * tk, X * (kc - tk));
        } else {
          kc = rz_[k];
          czm.reset((size_t)(X * kc), s_);
          copy(z_[k].data(), czm.p, X * kc, s_);
        }
        const int64_t kq = std::min(X, kc);
        DTensor Qz({kq, M, rz_[k + 1]}, s_);
        DBuf Rz((size_t)(kq * kc), s_);
        qr(czm.p, X, X, kc, Qz.data(), Rz.p, ws_, red_, s_);
        rz_[k] = kq;
        z_[k] = std::move(Qz);
      }
      if (swp > 0) nrmsc = nrmsc * normA[k - 1] * normx[k - 1] / normb[k - 1];
      // QR of x_k^T, R absorbed into x_{k-1}, normalised
      const int64_t m = M * rx_[k + 1], r = rx_[k], kk = std::min(m, r);
      DTensor Q({kk, M, rx_[k + 1]}, s_);
      DBuf R((size_t)(kk * r), s_);
      qr(x_[k].data(), m, m, r, Q.data(), R.p, ws_, red_, s_);
      const int64_t a = rx_[k - 1] * M_[k - 1];
      DTensor prev({rx_[k - 1], M_[k - 1], kk}, s_);
      gemm_cm(R.p, kk, x_[k - 1].data(), r, prev.data(), kk, kk, a, r, 1.0, 0.0, s_);
      double cn = norm(prev.data(), prev.numel());
      if (cn > 0.0) scale(prev.data(), prev.numel(), 1.0 / cn); else cn = 1.0;
      normx[k - 1] *= cn;
      rx_[k] = kk;
      x_[k] = std::move(Q);
      x_[k - 1] = std::move(prev);
      Ps_[k] = phi_xx(false, Ps_[k + 1], x_[k].data(), rx_[k], rx_[k + 1], x_[k].data(), rx_[k],
                      rx_[k + 1], k);
      Pr_[k] = phi_ab(false, Pr_[k + 1], x_[k].data(), rx_[k], rx_[k + 1], k);
      double nb = norm(Pr_[k].data(), Pr_[k].numel());
      if (!(nb > 0.0)) nb = 1.0;
      normb[k - 1] = nb;
      scale(Pr_[k].data(), Pr_[k].numel(), 1.0 / nb);
      nrmsc = nrmsc * normb[k - 1] / (normA[k - 1] * normx[k - 1]);
      if (!last) {
        Pz_[k] = phi_xx(false, Pz_[k + 1], z_[k].data(), rz_[k], rz_[k + 1], x_[k].data(), rx_[k],
                        rx_[k + 1], k);
        scale(Pz_[k].data(), Pz_[k].numel(), 1.0 / normA[k - 1]);
        Pzr_[k] = phi_ab(false, Pzr_[k + 1], z_[k].data(), rz_[k], rz_[k + 1], k);
        scale(Pzr_[k].data(), Pzr_[k].numel(), 1.0 / normb[k - 1]);
      }
    }
    // ---- left to right ----------------------------------------------------------------------
    max_dx = 0.0;
    for (int k = 0; k < d; ++k) {
      const int64_t M = M_[k], p = rx_[k] * M, q = rx_[k + 1];
      DBuf sol((size_t)(p * q), s_);
      local_ab(Pr_[k], Pr_[k + 1], k, sol.p);
      scale(sol.p, p * q, nrmsc);
      nrm2(red_, sol.p, p * q, scal_.p, s_);
      DBuf diff((size_t)(p * q), s_);
      sub(sol.p, x_[k].data(), diff.p, p * q, s_);
      nrm2(red_, diff.p, p * q, scal_.p + 1, s_);
      TTGB_CUDA(cudaMemcpyAsync(h_, scal_.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s_));
      TTGB_CUDA(cudaStreamSynchronize(s_));
      const double nsol = h_[0];
      const double dx = h_[1] / nsol;   // as the reference: NaN for a zero projection
      if (dx > max_dx) max_dx = dx;
      if (p_.verbose) std::printf("\tcore %d: dx = %g\n", k, dx);
      // truncation: u (p x r column-major), v (q x r column-major, sol = u v^T)
      int64_t r = 0;
      DBuf u, v;
      if (k < d - 1) {
        // sol (p x q row-major) = its column-major view sol^T (q x p) = U' S Vh'
        const int64_t kf = std::min(p, q);
        DBuf U((size_t)(q * kf), s_), S((size_t)kf, s_), Vh((size_t)(kf * p), s_);
        svd(sol.p, q, q, p, U.p, S.p, Vh.p, ws_, red_, s_);
        hs.resize(kf);
        TTGB_CUDA(cudaMemcpyAsync(hs.data(), S.p, kf * sizeof(double), cudaMemcpyDeviceToHost, s_));
        TTGB_CUDA(cudaStreamSynchronize(s_));
        r = rank_chop(hs, nsol * eps / std::pow((double)d, last ? 0.5 : 1.5));
        r = std::max<int64_t>(1, std::min({r, kf, p_.rmax}));
        u.reset((size_t)(p * r), s_);
        transpose(Vh.p, kf, u.p, p, r, p, s_);          // left singular vectors
        v.reset((size_t)(q * r), s_);
        copy(U.p, v.p, q * r, s_);                      // right singular vectors, scaled by S
        scale_cols_kernel<<<cdiv(q * r, 256), 256, 0, s_>>>(v.p, q, q, r, S.p);
        TTGB_CHECK_LAUNCH();
      } else {
        // last core (q = 1): the projection itself
        r = 1;
        u.reset((size_t)p, s_);
        copy(sol.p, u.p, p, s_);
        v.reset(1, s_);
        fill(v.p, 1.0, 1, s_);
      }
      if (!last) {   // z update (_amen.py:300-320)
        DBuf xn((size_t)(p * q), s_);   // u v^T as a core [rx_k, M, rx_{k+1}]
        gemm_cm(v.p, q, u.p, p, xn.p, q, q, p, r, 1.0, 0.0, s_, false, true);
        const int64_t X = rz_[k] * M, Z = rz_[k + 1];
        DBuf czx((size_t)(X * Z), s_), czab((size_t)(X * Z), s_);
        proj(Pz_[k], xn.p, Pz_[k + 1], k, czx.p);
        local_ab(Pzr_[k], Pzr_[k + 1], k, czab.p);
        axpby(-1.0, czx.p, nrmsc, czab.p, X * Z, s_);
        // left singular vectors of the (X x Z) row-major matrix: column-major view (Z x X)
        const int64_t kf = std::min(X, Z);
        DBuf U((size_t)(Z * kf), s_), S((size_t)kf, s_), Vh((size_t)(kf * X), s_);
        svd(czab.p, Z, Z, X, U.p, S.p, Vh.p, ws_, red_, s_);
        const int64_t tk = std::min<int64_t>(p_.kickrank, kf);
        const int64_t kc = tk + ((k < d - 1) ? p_.kick2 : 0);
        DBuf czm((size_t)(X * kc), s_);
        transpose(Vh.p, kf, czm.p, X, tk, X, s_);
        if (kc > tk) fill_randn(czm.p + X * tk, X * (kc - tk));
        const int64_t kq = std::min(X, kc);
        DBuf Qz((size_t)(X * kq), s_), Rz((size_t)(kq * kc), s_);
        qr(czm.p, X, X, kc, Qz.p, Rz.p, ws_, red_, s_);
        rz_[k + 1] = kq;
        DTensor zk({rz_[k], M, kq}, s_);
        transpose(Qz.p, X, zk.data(), kq, X, kq, s_);
        z_[k] = std::move(zk);
      }
      if (k < d - 1) {
        if (!last) {   // enrichment with the projected residual (_amen.py:322-337)
          DBuf xn((size_t)(p * q), s_);
          gemm_cm(v.p, q, u.p, p, xn.p, q, q, p, r, 1.0, 0.0, s_, false, true);
          const int64_t Z = Pz_[k + 1].dim(0);
          DBuf czx((size_t)(p * Z), s_), uk((size_t)(p * Z), s_);
          proj(Ps_[k], xn.p, Pz_[k + 1], k, czx.p);
          local_ab(Pr_[k], Pzr_[k + 1], k, uk.p);
          axpby(-1.0, czx.p, nrmsc, uk.p, p * Z, s_);   // uk (p x Z row-major)
          const int64_t nc = r + Z, k2 = std::min(p, nc);
          DBuf UK((size_t)(p * nc), s_);
          copy(u.p, UK.p, p * r, s_);
          transpose(uk.p, Z, UK.p + p * r, p, Z, p, s_);
          DBuf Qn((size_t)(p * k2), s_), Rm((size_t)(k2 * nc), s_);
          qr(UK.p, p, p, nc, Qn.p, Rm.p, ws_, red_, s_);
          DBuf vn((size_t)(q * k2), s_);   // [v, 0] Rm^T
          gemm_cm(v.p, q, Rm.p, k2, vn.p, q, q, k2, r, 1.0, 0.0, s_, false, true);
          u = std::move(Qn);
          v = std::move(vn);
          r = k2;
        }
        // x_{k+1} <- v^T x_{k+1}, normalised
        const int64_t Y = M_[k + 1] * rx_[k + 2];
        DTensor xn1({r, M_[k + 1], rx_[k + 2]}, s_);
        gemm_cm(x_[k + 1].data(), Y, v.p, q, xn1.data(), Y, Y, r, q, 1.0, 0.0, s_);
        nrmsc = nrmsc * normA[k] * normx[k] / normb[k];
        double nn = norm(xn1.data(), xn1.numel());
        if (nn > 0.0) scale(xn1.data(), xn1.numel(), 1.0 / nn); else nn = 1.0;
        normx[k] *= nn;
        DTensor xk({rx_[k], M, r}, s_);
        transpose(u.p, p, xk.data(), r, p, r, s_);
        x_[k] = std::move(xk);
        x_[k + 1] = std::move(xn1);
        rx_[k + 1] = r;
        Ps_[k + 1] = phi_xx(true, Ps_[k], x_[k].data(), rx_[k], rx_[k + 1], x_[k].data(), rx_[k],
                            rx_[k + 1], k);
        Pr_[k + 1] = phi_ab(true, Pr_[k], x_[k].data(), rx_[k], rx_[k + 1], k);
        double nb = norm(Pr_[k + 1].data(), Pr_[k + 1].numel());
        if (!(nb > 0.0)) nb = 1.0;
        normb[k] = nb;
        scale(Pr_[k + 1].data(), Pr_[k + 1].numel(), 1.0 / nb);
        nrmsc = nrmsc * normb[k] / (normA[k] * normx[k]);
        if (!last) {
          Pz_[k + 1] = phi_xx(true, Pz_[k], z_[k].data(), rz_[k], rz_[k + 1], x_[k].data(),
                              rx_[k], rx_[k + 1], k);
          scale(Pz_[k + 1].data(), Pz_[k + 1].numel(), 1.0 / normA[k]);
          Pzr_[k + 1] = phi_ab(true, Pzr_[k], z_[k].data(), rz_[k], rz_[k + 1], k);
          scale(Pzr_[k + 1].data(), Pzr_[k + 1].numel(), 1.0 / normb[k]);
        }
      } else {
        DTensor xk({rx_[k], M, 1}, s_);
        copy(u.p, xk.data(), p, s_);
        x_[k] = std::move(xk);
      }
    }
    if (p_.verbose) std::printf("sweep %d: max dx %g\n", swp, max_dx);
    if (last) break;
    if (max_dx < eps) last = true;
  }
  // undo the normalisation: the geometric mean of normx on every core (_amen.py:391-395)
  double lsum = 0.0;
  for (int k = 0; k < d - 1; ++k) lsum += std::log(normx[k]);
  const double f = std::exp(lsum / d);
  for (int k = 0; k < d; ++k) scale(x_[k].data(), x_[k].numel(), f);
  ranks = rx_;
  if (st) {
    st->sweeps = std::min(swp + 1, p_.nswp);
    st->max_dx = max_dx;
  }
  TTGB_CUDA(cudaStreamSynchronize(s_));
  return std::move(x_);
}

}  // namespace

std::vector<DTensor> amen_mv(const TTView& A, const TTView& b, const TTView& x0,
                             const AmenMvParams& p, cudaStream_t s, std::vector<int64_t>& ranks,
                             AmenMvStats* stats, LinalgWS& ws, const RedWS& red) {
  const int d = A.d;
  TTGB_REQUIRE(d >= 1 && b.d == d && !A.rows.empty() && b.rows.empty(),
               "A must be TT-matrix and b must be vector.");
  for (int k = 0; k < d; ++k) TTGB_REQUIRE(A.cols[k] == b.cols[k], "Dimension mismatch.");
  TTGB_REQUIRE(p.nswp >= 1 && p.rmax >= 1 && p.kickrank >= 0 && p.kick2 >= 0,
               "invalid AMEn matvec parameters");
  if (d == 1) {
    std::vector<int64_t> rk;
    auto out = tt_matvec(A, b, s, rk);
    ranks = rk;
    if (stats) { stats->sweeps = 0; stats->max_dx = 0.0; }
    return out;
  }
  AmenMv run(A, b, p, s, ws, red);
  return run.run(x0, ranks, stats);
}

}  // namespace ttgb
