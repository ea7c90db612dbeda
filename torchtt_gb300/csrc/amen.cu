// AMEn solve (plain FP64 path): the sweep orchestration of cpp/amen_solve.h:122-549 with every
// tensor in HBM and every arithmetic step a kernel of this library. The host keeps only ranks,
// the norm bookkeeping scalars (normA/normb/normx/nrmsc, amen_solve.h:195-204) and the stopping
// decisions; it reads device scalars in small batches (one synchronisation per group of norms).
#include <algorithm>
#include <cstdlib>
#include <string>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <memory>

#include "amen.cuh"
#include "blas1.cuh"
#include "contract.cuh"
#include "gmres.cuh"
#include "linalg.cuh"
#include "prec.cuh"

namespace ttgb {

namespace {

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Box-Muller on two 53-bit uniforms from a counter-based hash (splitmix64)
__global__ void randn_kernel(double* out, int64_t n, uint64_t seed, uint64_t offset) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t h1 = splitmix64(seed ^ splitmix64(offset + (uint64_t)i));
    const uint64_t h2 = splitmix64(h1 ^ 0xD1B54A32D192ED03ull);
    const double u1 = ((double)(h1 >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    const double u2 = (double)(h2 >> 11) * (1.0 / 9007199254740992.0);
    out[i] = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
  }
}

// B[(l,m,L),(r,n,R)] = sum_{s,S} Phi_l[l,s,r] A[s,m,n,S] Phi_r[L,S,R]  (amen_solve.h:322-324)
__global__ void assemble_dense_kernel(const double* __restrict__ phil, const double* __restrict__ A,
                                      const double* __restrict__ phir, int r, int s, int n, int S,
                                      int R, double* B) {
  const int64_t nl = (int64_t)r * n * R;
  const int64_t total = nl * nl;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = t / nl, col = t % nl;
    const int l = (int)(row / ((int64_t)n * R)), m = (int)((row / R) % n), L = (int)(row % R);
    const int rr = (int)(col / ((int64_t)n * R)), nn = (int)((col / R) % n), RR = (int)(col % R);
    double v = 0.0;
    for (int a = 0; a < s; ++a) {
      const double pl = phil[((int64_t)l * s + a) * r + rr];
      if (pl == 0.0) continue;
      for (int b = 0; b < S; ++b)
        v = fma(pl * A[(((int64_t)a * n + m) * n + nn) * S + b], phir[((int64_t)L * S + b) * R + RR], v);
    }
    B[t] = v;
  }
}

unsigned grid_of(int64_t n) {
  unsigned g = cdiv(n, 256);
  const unsigned cap = 8 * (unsigned)num_sms();
  if (g > cap) g = cap;
  return g ? g : 1;
}

double lp_flops(const LocalOpDims& d) { return local_product_flops(d); }

// The solve allocates its tensors stream-ordered from the device's default memory pool; keeping
// freed blocks in the pool (instead of returning them at every synchronisation) makes those
// allocations cheap.
void keep_pool_memory() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess) return;
  uint64_t thr = UINT64_MAX;
  cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
}

class AmenRun {
 public:
  AmenRun(const TTView& A, const TTView& b, const AmenParams& p, cudaStream_t s)
      : A_(A), b_(b), p_(p), s_(s) {
    keep_pool_memory();
    d_ = A.d;
    N_ = A.cols;
    rA_ = A.ranks;
    rb_ = b.ranks;
    red_partial_.reset(1024 * 128, s_);
    TTGB_CUDA(cudaMallocAsync((void**)&red_counter_, 64, s_));
    TTGB_CUDA(cudaMemsetAsync(red_counter_, 0, 64, s_));
    red_.partial = red_partial_.p;
    red_.counter = red_counter_;
    red_.cap_blocks = 1024;
    red_.cap_vec = 127;
    TTGB_CUDA(cudaMallocAsync((void**)&lws_.status, 16, s_));
    TTGB_CUDA(cudaMallocAsync((void**)&gws_.d_flag, 32, s_));
    TTGB_CUDA(cudaMemsetAsync(lws_.status, 0, 16, s_));
    TTGB_CUDA(cudaMallocHost((void**)&hbuf_, 4096));
    lws_.h_status = (int*)hbuf_;
    gws_.h_flag = (int*)(hbuf_ + 16);
    hscal_ = (double*)(hbuf_ + 64);
    dscal_.reset(kScal, s_);
    if (p.profile) {
      prof_.reset(new Profiler(s_));
      prof_lowp_.reset(new Profiler(s_));
      prof_krylov_.reset(new Profiler(s_));
      phases_.reset(new PhaseTimer(s_));
    }
  }
  ~AmenRun() {
    cudaStreamSynchronize(s_);
    if (red_counter_) cudaFreeAsync(red_counter_, s_);
    if (lws_.status) cudaFreeAsync(lws_.status, s_);
    if (gws_.d_flag) cudaFreeAsync(gws_.d_flag, s_);
    if (tc_err_) cudaFreeAsync(tc_err_, s_);
    if (hbuf_) cudaFreeHost(hbuf_);
  }

  AmenResult run(const TTView& x0, const TTView& z0);

 private:
  static constexpr int kScal = 256;
  enum Slot { kNormRhs = 0, kNormDrhs = 1, kResNew = 2, kNormX = 3, kNormPhi = 4, kNormPhiB = 5,
              kNormV = 6, kCand = 16 };

  const TTView& A_;
  const TTView& b_;
  AmenParams p_;
  cudaStream_t s_;
  int d_ = 0;
  std::vector<int64_t> N_, rA_, rb_, rx_, rz_;
  std::vector<DTensor> x_, z_, Phis_, Phis_b_, Phiz_, Phiz_b_;
  std::vector<double> normA_, normb_, normx_;
  double nrmsc_ = 1.0;
  RedWS red_;
  DBuf red_partial_;
  unsigned* red_counter_ = nullptr;
  LinalgWS lws_;
  GmresWS gws_;
  char* hbuf_ = nullptr;
  double* hscal_ = nullptr;
  DBuf dscal_;
  DBuf w1_, w2_, wp_, wphi_, wrhs_, prec_J_, prec_work_;
  AmenStats st_;
  std::unique_ptr<Profiler> prof_;
  std::unique_ptr<Profiler> prof_lowp_;
  std::unique_ptr<Profiler> prof_krylov_;
  int64_t op_count_ = 0;   // applications of the current local operator
  int64_t lowp_count_ = 0; // low-precision applications of the current local operator
  bool mixed_ = false;
  // tolerance of the sweeps: eps, or eps / 4 with strict_eps (the reference's stopping rule bounds
  // the local residuals; its true residual can end a few times above them)
  double eps_ = 0.0;
  int fp64e_ = kFp64Native;   // engine of the FP64 products (double-float on the mixed path)
  std::vector<FBuf> A32_;  // FP32 copies of the A cores (mixed path, FP32 engine)
  FBuf phil32_, phir32_, xf_, yf_, w1f_, w2f_;
  bool use_tc_ = false;    // mixed path on the tcgen05 engine
  std::vector<TcCore> tc_cores_;
  std::vector<SparseCore> spA_;   // nonzero structure of each A core (structured A stage)
  TcLocal tc_local_;
  int* tc_err_ = nullptr;
  DBuf resvec_;
  uint64_t rng_offset_ = 0;

  double* slot(int i) { return dscal_.p + i; }

  enum Phase { kPhBwdZ = 0, kPhBwdQR, kPhBwdPhi, kPhFwdSetup, kPhFwdSolve, kPhFwdSvd, kPhFwdRank,
               kPhFwdZ, kPhFwdEnrich, kPhFwdPhi, kPhOther };
  std::unique_ptr<PhaseTimer> phases_;
  void phase(int p) {
    if (phases_) phases_->mark(p);
  }

  static constexpr double kMixedOrthTol = 1e-8;

  void note_gmres(const GmresResult& gr) {
    st_.gmres_syncs += gr.syncs;
    st_.host_syncs += gr.syncs;
    st_.gmres_overrun += gr.overrun;
    st_.gmres_reorth += gr.reorth;
  }

  void read_scalars(int n) {
    TTGB_CUDA(cudaMemcpyAsync(hscal_, dscal_.p, n * sizeof(double), cudaMemcpyDeviceToHost, s_));
    TTGB_CUDA(cudaStreamSynchronize(s_));
    st_.host_syncs++;
  }

  const double* Acore(int k) const { return A_.cores[k]; }
  const double* bcore(int k) const { return b_.cores[k]; }

  void local_prod(const double* phil, int64_t rl, int64_t r, const double* phir, int64_t RL,
                  int64_t R, int k, const double* x, double* y, double alpha = 1.0,
                  double beta = 0.0, bool main_system = false) {
    LocalOpDims dm{rl, rA_[k], r, N_[k], N_[k], rA_[k + 1], RL, R};
    w1_.ensure(local_product_w1(dm), s_);
    w2_.ensure(local_product_w2(dm), s_);
    Fp64EngineScope eng(fp64e_);
    if (prof_) prof_->begin();
    local_product(dm, phil, Acore(k), phir, x, y, w1_.p, w2_.p, s_, alpha, beta, &spA_[k]);
    if (prof_) prof_->end(local_product_gemm_flops(dm, &spA_[k]), 3);
    if (main_system) { st_.matvecs++; st_.matvec_flops += lp_flops(dm); }
    else st_.other_flops += lp_flops(dm);
  }

  void lrhs(const double* phil, int64_t r, int k, const double* phir, int64_t R, double alpha,
            double* out) {
    wrhs_.ensure(local_rhs_workspace(rb_[k], N_[k], rb_[k + 1], r, R), s_);
    Fp64EngineScope eng(fp64e_);
    local_rhs(rb_[k], N_[k], rb_[k + 1], r, R, phil, bcore(k), phir, alpha, out, wrhs_.p, s_);
  }

  void phi_A(bool fwd, const DTensor& phi_in, const double* left, int64_t l, int64_t L,
             const double* right, int64_t r, int64_t R, int k, DTensor& out) {
    PhiDims pd{l, L, rA_[k], rA_[k + 1], r, R, N_[k], N_[k]};
    wphi_.ensure(phi_A_workspace(pd), s_);
    // flops of the GEMM launches; the A stage counts only when it is a GEMM (dense core)
    const double a_stage = spA_[k].use ? 0.0 : 1.0;
    const double f = 2.0 * (fwd ? (double)l * rA_[k] * r * N_[k] * L +
                                      a_stage * r * L * N_[k] * rA_[k] * N_[k] * rA_[k + 1] +
                                      (double)L * rA_[k + 1] * R * r * N_[k]
                                 : (double)l * N_[k] * rA_[k + 1] * R * L +
                                      a_stage * l * R * rA_[k] * N_[k] * N_[k] * rA_[k + 1] +
                                      (double)l * rA_[k] * r * N_[k] * R);
    Fp64EngineScope eng(fp64e_);
    if (prof_) prof_->begin();
    if (fwd) {
      out = DTensor({L, rA_[k + 1], R}, s_);
      phi_fwd_A(pd, phi_in.data(), left, Acore(k), right, out.data(), wphi_.p, s_, &spA_[k]);
    } else {
      out = DTensor({l, rA_[k], r}, s_);
      phi_bck_A(pd, phi_in.data(), left, Acore(k), right, out.data(), wphi_.p, s_, &spA_[k]);
    }
    if (prof_) prof_->end(f, 3);
    st_.phi_flops += f;
  }

  void phi_b(bool fwd, const DTensor& phi_in, const double* core, int64_t r, int64_t R, int k,
             DTensor& out) {
    PhiRhsDims pd{rb_[k], rb_[k + 1], r, R, N_[k]};
    wphi_.ensure(phi_rhs_workspace(pd), s_);
    Fp64EngineScope eng(fp64e_);
    if (fwd) {
      out = DTensor({rb_[k + 1], R}, s_);
      phi_fwd_rhs(pd, phi_in.data(), bcore(k), core, out.data(), wphi_.p, s_);
    } else {
      out = DTensor({rb_[k], r}, s_);
      phi_bck_rhs(pd, phi_in.data(), bcore(k), core, out.data(), wphi_.p, s_);
    }
  }

  // out (a x kk, row-major) = core (a x c, row-major) * R^T, R (kk x c, column-major ld kk)
  void absorb_right(const double* core, int64_t a, int64_t c, const double* R, int64_t kk,
                    double* out) {
    ContractDesc cd;
    cd.M = (int)a; cd.N = (int)kk; cd.K = (int)c;
    cd.A = core; cd.am = Ax::one(c); cd.ak = Ax::one(1);
    cd.B = R; cd.bk = Ax::one(kk); cd.bn = Ax::one(1);
    cd.C = out; cd.cm = Ax::one(kk); cd.cn = Ax::one(1);
    contract(cd, s_);
  }

  // out (k2 x Y, row-major) = sum_i V[i, j] X[i, y]; V (b x k2) column-major with given strides
  void left_apply(const double* V, int64_t vi_stride, int64_t vj_stride, int64_t bdim, int64_t k2,
                  const double* X, int64_t Y, double* out) {
    ContractDesc cd;
    cd.M = (int)k2; cd.N = (int)Y; cd.K = (int)bdim;
    cd.A = V; cd.am = Ax::one(vj_stride); cd.ak = Ax::one(vi_stride);
    cd.B = X; cd.bk = Ax::one(Y); cd.bn = Ax::one(1);
    cd.C = out; cd.cm = Ax::one(Y); cd.cn = Ax::one(1);
    contract(cd, s_);
  }

  void randn_fill(double* out, int64_t n) {
    randn(out, n, p_.seed, rng_offset_, s_);
    rng_offset_ += (uint64_t)n;
  }

  void init(const TTView& x0, const TTView& z0);
  void rl_orthogonal_z();
  void backward_step(int k, int swp, bool last);
  void forward_step(int k, int swp, bool last, double& max_res);
  void z_update_forward(int k, const double* trunc);
  void setup_lowp(LocalOperator& op, int k);
  int choose_fp64_engine();
  int rank_search_tail(const double* U, const double* SVh, int64_t a, int64_t bdim, int64_t kf,
                       const double* resvec, double norm_rhs, double thr, const LocalOperator& op,
                       int64_t nl, double* tail_buf);
  int rank_search(const double* U, const double* SVh, int64_t a, int64_t bdim, int64_t kf,
                  const double* rhs, double norm_rhs, double thr, const LocalOperator* op,
                  const double* B, int64_t nl, double* cand_buf);
};

void AmenRun::init(const TTView& x0, const TTView& z0) {
  const int d = d_;
  spA_.resize(d);
  if (p_.a_structure)
    for (int i = 0; i < d; ++i) spA_[i].build(Acore(i), rA_[i], N_[i], N_[i], rA_[i + 1], s_);
  mixed_ = p_.precision == 1;
  eps_ = p_.strict_eps ? 0.25 * p_.eps : p_.eps;
  fp64e_ = choose_fp64_engine();
  if (mixed_) {
    use_tc_ = (p_.lowp_engine == 2) || (p_.lowp_engine == 0 && tc_available());
    TTGB_REQUIRE(!use_tc_ || tc_available(), "tcgen05 engine needs an sm_100-family GPU");
    if (use_tc_) {
      tc_cores_.resize(d);
      for (int i = 0; i < d; ++i)
        if (!spA_[i].use) tc_cores_[i].build(Acore(i), rA_[i], N_[i], N_[i], rA_[i + 1], s_);
      TTGB_CUDA(cudaMallocAsync((void**)&tc_err_, sizeof(int), s_));
      TTGB_CUDA(cudaMemsetAsync(tc_err_, 0, sizeof(int), s_));
    } else {
      A32_.resize(d);
      for (int i = 0; i < d; ++i) {
        if (spA_[i].use) continue;   // the FP32 values live in the sparse structure
        const int64_t ne = rA_[i] * N_[i] * N_[i] * rA_[i + 1];
        A32_[i].reset((size_t)ne, s_);
        cast(Acore(i), A32_[i].p, ne, s_);
      }
    }
  }
  x_.resize(d);
  rx_.assign(d + 1, 1);
  if (x0.d == 0) {   // amen_solve.h:161-163
    for (int i = 0; i < d; ++i) {
      x_[i] = DTensor({1, N_[i], 1}, s_);
      fill(x_[i].data(), 1.0, N_[i], s_);
    }
  } else {
    for (int i = 0; i < d; ++i) {
      x_[i] = DTensor({x0.ranks[i], N_[i], x0.ranks[i + 1]}, s_);
      copy(x0.cores[i], x_[i].data(), x_[i].numel(), s_);
      rx_[i] = x0.ranks[i];
    }
    rx_[d] = x0.ranks[d];
  }
  rz_.assign(d + 1, p_.kickrank + p_.kick2);   // amen_solve.h:169-176
  rz_[0] = 1;
  rz_[d] = 1;
  z_.resize(d);
  for (int i = 0; i < d; ++i) {
    z_[i] = DTensor({rz_[i], N_[i], rz_[i + 1]}, s_);
    if (z0.d == d) {
      TTGB_REQUIRE(z0.ranks[i] == rz_[i] && z0.ranks[i + 1] == rz_[i + 1],
                   "z0 ranks must be [1, kickrank+kick2, ..., 1]");
      copy(z0.cores[i], z_[i].data(), z_[i].numel(), s_);
    } else {
      randn_fill(z_[i].data(), z_[i].numel());
    }
  }
  rl_orthogonal_z();   // amen_solve.h:178
  auto one3 = [&]() { DTensor t({1, 1, 1}, s_); fill(t.data(), 1.0, 1, s_); return t; };
  auto one2 = [&]() { DTensor t({1, 1}, s_); fill(t.data(), 1.0, 1, s_); return t; };
  Phis_.resize(d + 1); Phis_b_.resize(d + 1); Phiz_.resize(d + 1); Phiz_b_.resize(d + 1);
  Phis_[0] = one3(); Phis_[d] = one3(); Phiz_[0] = one3(); Phiz_[d] = one3();
  Phis_b_[0] = one2(); Phis_b_[d] = one2(); Phiz_b_[0] = one2(); Phiz_b_[d] = one2();
  normA_.assign(d > 1 ? d - 1 : 1, 1.0);
  normb_.assign(d > 1 ? d - 1 : 1, 1.0);
  normx_.assign(d > 1 ? d - 1 : 1, 1.0);
  nrmsc_ = 1.0;
}

// cpp/ortho.h:46-73 on the enrichment cores
void AmenRun::rl_orthogonal_z() {
  for (int i = d_ - 1; i > 0; --i) {
    const int64_t r = z_[i].dim(0), m = z_[i].dim(1) * z_[i].dim(2);
    const int64_t k = r < m ? r : m;
    DTensor Q({k, z_[i].dim(1), z_[i].dim(2)}, s_);
    DBuf R((size_t)(k * r), s_);
    qr(z_[i].data(), m, m, r, Q.data(), R.p, lws_, red_, s_);
    const int64_t a = z_[i - 1].dim(0) * z_[i - 1].dim(1);
    DTensor prev({z_[i - 1].dim(0), z_[i - 1].dim(1), k}, s_);
    absorb_right(z_[i - 1].data(), a, r, R.p, k, prev.data());
    z_[i] = std::move(Q);
    z_[i - 1] = std::move(prev);
    rz_[i] = k;
  }
}

void AmenRun::backward_step(int k, int swp, bool last) {
  const int64_t n = N_[k];
  phase(kPhBwdZ);
  if (!last) {   // z update, amen_solve.h:223-245
    DBuf czm;      // column-major (n * rz_{k+1}) x kc matrix of new z directions
    int64_t X = n * rz_[k + 1], kc = 0;
    if (swp > 0) {
      DBuf czA((size_t)(rz_[k] * X), s_), czy((size_t)(rz_[k] * X), s_);
      local_prod(Phiz_[k].data(), rz_[k], rx_[k], Phiz_[k + 1].data(), rz_[k + 1], rx_[k + 1], k,
                 x_[k].data(), czA.p);
      lrhs(Phiz_b_[k].data(), rz_[k], k, Phiz_b_[k + 1].data(), rz_[k + 1], nrmsc_, czy.p);
      axpby(-1.0, czA.p, 1.0, czy.p, rz_[k] * X, s_);   // czy*nrmsc - czA
      // right singular vectors of the rz_k x X matrix == left ones of its column-major view
      const int64_t kf = rz_[k] < X ? rz_[k] : X;
      const int64_t tk = p_.kickrank < kf ? p_.kickrank : kf;
      kc = tk + ((k < d_ - 1) ? p_.kick2 : 0);
      if (kc == kf && kf == rz_[k]) {
        // every singular vector is kept and nothing is appended: the new z directions span the
        // column space of czy, and only that span enters the enrichment and the z interfaces, so
        // the QR below orthonormalises czy itself (the SVD would only order a basis of the same
        // span)
        czm = std::move(czy);
      } else {
        DBuf U((size_t)(X * kf), s_), S((size_t)kf, s_), Vh((size_t)(kf * rz_[k]), s_);
        svd(czy.p, X, X, rz_[k], U.p, S.p, Vh.p, lws_, red_, s_);
        czm.reset((size_t)(X * kc), s_);
        copy(U.p, czm.p, X * tk, s_);
        if (kc > tk) randn_fill(czm.p + X * tk, X * (kc - tk));
      }
    } else {
      kc = rz_[k];
      czm.reset((size_t)(X * kc), s_);
      copy(z_[k].data(), czm.p, X * kc, s_);
    }
    const int64_t kq = X < kc ? X : kc;
    DTensor Qz({kq, n, rz_[k + 1]}, s_);
    DBuf Rz((size_t)(kq * kc), s_);
    qr(czm.p, X, X, kc, Qz.data(), Rz.p, lws_, red_, s_);
    rz_[k] = kq;
    z_[k] = std::move(Qz);
  }
  const double nrmsc_before = nrmsc_;
  const double nA0 = normA_[k - 1], nx0 = normx_[k - 1], nb0 = normb_[k - 1];

  phase(kPhBwdQR);
  // QR of x_k^T, absorb R into x_{k-1} (amen_solve.h:252-267)
  const int64_t r = rx_[k], m = n * rx_[k + 1];
  const int64_t kk = r < m ? r : m;
  DTensor Q({kk, n, rx_[k + 1]}, s_);
  DBuf R((size_t)(kk * r), s_);
  qr(x_[k].data(), m, m, r, Q.data(), R.p, lws_, red_, s_);
  const int64_t a = rx_[k - 1] * N_[k - 1];
  DTensor prev({rx_[k - 1], N_[k - 1], kk}, s_);
  absorb_right(x_[k - 1].data(), a, r, R.p, kk, prev.data());
  rx_[k] = kk;
  nrm2(red_, prev.data(), prev.numel(), slot(kNormX), s_);
  scale_dev(prev.data(), prev.numel(), nullptr, slot(kNormX), s_);
  x_[k] = std::move(Q);
  x_[k - 1] = std::move(prev);

  phase(kPhBwdPhi);
  // interfaces (amen_solve.h:270-282)
  phi_A(false, Phis_[k + 1], x_[k].data(), rx_[k], rx_[k + 1], x_[k].data(), rx_[k], rx_[k + 1], k,
        Phis_[k]);
  phi_b(false, Phis_b_[k + 1], x_[k].data(), rx_[k], rx_[k + 1], k, Phis_b_[k]);
  nrm2_multi(red_, VecSegs()
                         .norm(Phis_[k].data(), Phis_[k].numel(), slot(kNormPhi))
                         .norm(Phis_b_[k].data(), Phis_b_[k].numel(), slot(kNormPhiB)), s_);
  VecSegs scl;
  scl.scale(Phis_[k].data(), Phis_[k].numel(), slot(kNormPhi))
      .scale(Phis_b_[k].data(), Phis_b_[k].numel(), slot(kNormPhiB));
  if (!last) {   // amen_solve.h:288-291
    phi_A(false, Phiz_[k + 1], z_[k].data(), rz_[k], rz_[k + 1], x_[k].data(), rx_[k], rx_[k + 1],
          k, Phiz_[k]);
    phi_b(false, Phiz_b_[k + 1], z_[k].data(), rz_[k], rz_[k + 1], k, Phiz_b_[k]);
    scl.scale(Phiz_[k].data(), Phiz_[k].numel(), slot(kNormPhi))
        .scale(Phiz_b_[k].data(), Phiz_b_[k].numel(), slot(kNormPhiB));
  }
  scale_multi(scl, s_);
  read_scalars(8);
  double cn = hscal_[kNormX];
  if (!(cn > 0.0)) cn = 1.0;
  double nA = hscal_[kNormPhi];
  if (!(nA > 0.0)) nA = 1.0;
  double nb = hscal_[kNormPhiB];
  if (!(nb > 0.0)) nb = 1.0;
  double nr = nrmsc_before;
  if (swp > 0) nr = nr * nA0 * nx0 / nb0;   // amen_solve.h:249-250
  normx_[k - 1] = nx0 * cn;
  normA_[k - 1] = nA;
  normb_[k - 1] = nb;
  nrmsc_ = nr * nb / (nA * normx_[k - 1]);  // amen_solve.h:285
}

int AmenRun::rank_search(const double* U, const double* SVh, int64_t a, int64_t bdim, int64_t kf,
                         const double* rhs, double norm_rhs, double thr, const LocalOperator* op,
                         const double* B, int64_t nl, double* cand_buf) {
  // amen_solve.h:385-401: r from kf downwards, stop at the first candidate whose local residual
  // exceeds thr; candidates are evaluated in chunks to batch the host synchronisations.
  const int kChunk = 4;
  int64_t r = kf;
  DBuf resid((size_t)nl, s_);
  while (r > 0) {
    const int64_t nc = r < kChunk ? r : kChunk;
    for (int64_t c = 0; c < nc; ++c) {
      const int64_t rr = r - c;
      ContractDesc cd;   // cand (a x b row-major) = U[:, :rr] SVh[:rr, :]
      cd.M = (int)a; cd.N = (int)bdim; cd.K = (int)rr;
      cd.A = U; cd.am = Ax::one(1); cd.ak = Ax::one(a);
      cd.B = SVh; cd.bk = Ax::one(1); cd.bn = Ax::one(kf);
      cd.C = cand_buf; cd.cm = Ax::one(bdim); cd.cn = Ax::one(1);
      contract(cd, s_);
      if (op) {
        op->apply(cand_buf, resid.p, false, s_);
      } else {
        gemv(B, nl, cand_buf, resid.p, s_);
      }
      sub(resid.p, rhs, resid.p, nl, s_);
      nrm2(red_, resid.p, nl, slot(kCand + (int)c), s_);
    }
    read_scalars(kCand + (int)nc);
    for (int64_t c = 0; c < nc; ++c) {
      const double res = hscal_[kCand + c] / norm_rhs;
      if (res > thr) return (int)(r - c);
    }
    r -= nc;
  }
  return 0;
}

void AmenRun::forward_step(int k, int swp, bool last, double& max_res) {
  (void)swp;
  const int64_t n = N_[k];
  const int64_t rk = rx_[k], rk1 = rx_[k + 1];
  const int64_t nl = rk * n * rk1;
  const double damp = 2.0;
  const double real_tol = (eps_ / std::sqrt((double)d_)) / damp;   // amen_solve.h:309

  phase(kPhFwdSetup);
  DBuf rhs((size_t)nl, s_), sol((size_t)nl, s_), tmp((size_t)nl, s_);
  lrhs(Phis_b_[k].data(), rk, k, Phis_b_[k + 1].data(), rk1, nrmsc_, rhs.p);   // :303-304
  const double* prev = x_[k].data();
  const bool use_full = nl < p_.max_full;   // amen_solve.h:312
  st_.local_solves++;

  LocalOperator op;
  DBuf Bmat;
  double res_old = 0.0, res_new = 0.0, norm_rhs = 0.0;
  phase(kPhFwdSolve);
  if (use_full) {   // amen_solve.h:319-330
    st_.direct_solves++;
    Bmat.reset((size_t)(nl * nl), s_);
    assemble_dense_kernel<<<grid_of(nl * nl), 256, 0, s_>>>(
        Phis_[k].data(), Acore(k), Phis_[k + 1].data(), (int)rk, (int)rA_[k], (int)n,
        (int)rA_[k + 1], (int)rk1, Bmat.p);
    TTGB_CHECK_LAUNCH();
    lu_solve(Bmat.p, nl, rhs.p, sol.p, lws_, s_);
    nrm2(red_, rhs.p, nl, slot(kNormRhs), s_);
    gemv(Bmat.p, nl, prev, tmp.p, s_);
    sub(tmp.p, rhs.p, tmp.p, nl, s_);
    nrm2(red_, tmp.p, nl, slot(kNormDrhs), s_);
    gemv(Bmat.p, nl, sol.p, tmp.p, s_);
    sub(tmp.p, rhs.p, tmp.p, nl, s_);
    nrm2(red_, tmp.p, nl, slot(kResNew), s_);
    read_scalars(3);
    norm_rhs = hscal_[kNormRhs];
    res_old = hscal_[kNormDrhs] / norm_rhs;
    res_new = hscal_[kResNew] / norm_rhs;
  } else {   // amen_solve.h:331-365
    op.dims = LocalOpDims{rk, rA_[k], rk, n, n, rA_[k + 1], rk1, rk1};
    op.phi_l = Phis_[k].data();
    op.A = Acore(k);
    op.spA = &spA_[k];
    op.fp64_engine = fp64e_;
    op.phi_r = Phis_[k + 1].data();
    op.prec = p_.prec;
    w1_.ensure(local_product_w1(op.dims), s_);
    w2_.ensure(local_product_w2(op.dims), s_);
    op.w1 = w1_.p;
    op.w2 = w2_.p;
    op.prof = prof_.get();
    op.prof_krylov = prof_krylov_.get();
    op_count_ = 0;
    op.count = &op_count_;
    if (p_.prec != kNoPrec) {
      prec_J_.ensure(prec_size(p_.prec, op.dims), s_);
      prec_setup(p_.prec, op.dims, op.phi_l, op.A, op.phi_r, prec_J_.p, prec_work_, lws_.status, s_);
      wp_.ensure((size_t)nl, s_);
      op.J = prec_J_.p;
      op.wp = wp_.p;
    }
    if (mixed_) setup_lowp(op, k);
    resvec_.ensure((size_t)nl, s_);
    DBuf drhs((size_t)nl, s_);
    op.apply_fp64(prev, drhs.p, s_);
    axpby(1.0, rhs.p, -1.0, drhs.p, nl, s_);   // drhs = rhs - B x_prev
    nrm2_multi(red_, VecSegs().norm(rhs.p, nl, slot(kNormRhs)).norm(drhs.p, nl, slot(kNormDrhs)), s_);
    read_scalars(2);
    norm_rhs = hscal_[kNormRhs];
    const double nd = hscal_[kNormDrhs];
    res_old = nd / norm_rhs;   // == ||B x_prev - rhs|| / ||rhs|| (amen_solve.h:357)
    if (!mixed_) {
      const double eps_local = real_tol * norm_rhs / nd;
      GmresResult gr = gmres(op, drhs.p, sol.p, p_.local_iterations, eps_local, p_.resets, gws_, red_, s_);
      st_.gmres_iterations += gr.nit;
      note_gmres(gr);
      if (p_.prec != kNoPrec) {
        op.apply_prec(sol.p, tmp.p, s_);
        copy(tmp.p, sol.p, nl, s_);
      }
      axpby(1.0, prev, 1.0, sol.p, nl, s_);   // solution_now += previous_solution
      op.apply_fp64(sol.p, tmp.p, s_);
      sub_nrm2(red_, tmp.p, rhs.p, tmp.p, nl, slot(kResNew), s_);
      read_scalars(3);
      res_new = hscal_[kResNew] / norm_rhs;
    } else {
      // FP64 iterative refinement around a GMRES whose operator runs in low precision: every
      // outer step solves B d = rhs - B x to the low-precision floor, adds d, and recomputes the
      // true residual in FP64 (amen_solve.h:340-358 with the local solve split into steps).
      copy(prev, sol.p, nl, s_);
      const double target = real_tol * norm_rhs;
      double cur = nd;
      DBuf dx((size_t)nl, s_);
      for (int it = 0; it < p_.max_refine && cur > target; ++it) {
        double thr = target / cur;
        if (thr < p_.lowp_floor) thr = p_.lowp_floor;
        // the correction is solved to thr >= lowp_floor with a low-precision operator: a basis kept
        // orthogonal to 1e-8 (semi-orthogonality) is far inside that
        GmresResult gr = gmres(op, drhs.p, dx.p, p_.local_iterations, thr, p_.resets, gws_, red_, s_,
                               kMixedOrthTol);
        st_.gmres_iterations += gr.nit;
        note_gmres(gr);
        st_.refinements++;
        if (p_.prec != kNoPrec) {
          op.apply_prec(dx.p, tmp.p, s_);
          copy(tmp.p, dx.p, nl, s_);
        }
        axpby(1.0, dx.p, 1.0, sol.p, nl, s_);
        op.apply_fp64(sol.p, tmp.p, s_);
        sub_nrm2(red_, rhs.p, tmp.p, drhs.p, nl, slot(kResNew), s_);   // drhs = rhs - B x
        read_scalars(3);
        const double nw = hscal_[kResNew];
        const bool stalled = nw > 0.5 * cur;
        cur = nw;
        if (stalled) break;
      }
      res_new = cur / norm_rhs;
      scale_copy(drhs.p, -1.0, resvec_.p, nl, s_);   // B x - rhs for the rank search
    }
  }
  if (p_.verbose && res_old / res_new < damp && res_new > real_tol)
    std::printf("WARNING: residual increase. res_old %g, res_new %g, %g\n", res_old, res_new, real_tol);
  if (res_old > max_res) max_res = res_old;   // amen_solve.h:375

  const int64_t a = rk * n, bdim = rk1;
  if (k < d_ - 1) {
    phase(kPhFwdSvd);
    // SVD of the (r_k n) x r_{k+1} unfolding (amen_solve.h:383)
    const int64_t kf = a < bdim ? a : bdim;
    DBuf Mc((size_t)(a * bdim), s_), U((size_t)(a * kf), s_), S((size_t)kf, s_), SVh((size_t)(kf * bdim), s_);
    transpose(sol.p, bdim, Mc.p, a, bdim, a, s_);
    svd(Mc.p, a, a, bdim, U.p, S.p, SVh.p, lws_, red_, s_);
    scale_rows_cm(SVh.p, kf, kf, bdim, S.p, s_);
    phase(kPhFwdRank);
    const double thr = res_new > real_tol * damp ? res_new : real_tol * damp;
    int64_t r = (mixed_ && !use_full)
                    ? rank_search_tail(U.p, SVh.p, a, bdim, kf, resvec_.p, norm_rhs, thr, op, nl, tmp.p)
                    : rank_search(U.p, SVh.p, a, bdim, kf, rhs.p, norm_rhs, thr,
                                  use_full ? nullptr : &op, Bmat.p, nl, tmp.p);
    r += 1;   // amen_solve.h:401-403
    r = (r < kf && r < p_.rmax) ? r : (kf < p_.rmax ? kf : p_.rmax);

    // truncated solution u v^T (row-major a x b) into tmp
    {
      ContractDesc cd;
      cd.M = (int)a; cd.N = (int)bdim; cd.K = (int)r;
      cd.A = U.p; cd.am = Ax::one(1); cd.ak = Ax::one(a);
      cd.B = SVh.p; cd.bk = Ax::one(1); cd.bn = Ax::one(kf);
      cd.C = tmp.p; cd.cm = Ax::one(bdim); cd.cn = Ax::one(1);
      contract(cd, s_);
    }
    phase(kPhFwdZ);
    if (!last) z_update_forward(k, tmp.p);

    int64_t k2 = r;
    DBuf newx;            // x_k as row-major (rk, n, k2)
    DBuf vprime;          // V' (bdim x k2) column-major
    phase(kPhFwdEnrich);
    if (!last) {   // enrichment, amen_solve.h:444-460
      // width of the residual block = rows of Phiz[k+1] (the z update above may already have
      // changed rz[k+1]; the reference takes it from the tensor shape, amen_solve.h:452)
      const int64_t rzk1 = Phiz_[k + 1].dim(0);
      DBuf left_res((size_t)(a * rzk1), s_), left_b((size_t)(a * rzk1), s_);
      local_prod(Phis_[k].data(), rk, rk, Phiz_[k + 1].data(), rzk1, rk1, k, tmp.p, left_res.p);
      lrhs(Phis_b_[k].data(), rk, k, Phiz_b_[k + 1].data(), rzk1, nrmsc_, left_b.p);
      axpby(-1.0, left_res.p, 1.0, left_b.p, a * rzk1, s_);   // uk = left_b - left_res
      const int64_t nc = r + rzk1;
      k2 = a < nc ? a : nc;
      DBuf Qn((size_t)(a * k2), s_);
      vprime.reset((size_t)(bdim * k2), s_);
      if (a >= nc) {
        // The first r columns U are orthonormal (left singular vectors), so QR([U, Z]) is
        // [U, Q_z] [[I, C], [0, R_z]] with C = U^T Z and Q_z R_z = (I - U U^T) Z: the block
        // Gram-Schmidt of the rzk1 residual columns against U (applied twice, CGS2) and a small
        // QR replace a CholeskyQR3 of all r + rzk1 columns; the span, hence the TT, is the same
        // as the reference's QR of the stacked block (amen_solve.h:452-458).
        DBuf Z((size_t)(a * rzk1), s_), Cm((size_t)(r * rzk1), s_);
        transpose(left_b.p, rzk1, Z.p, a, rzk1, a, s_);                  // Z: a x rzk1, ld a
        for (int pass = 0; pass < 2; ++pass) {
          gemm_cm(U.p, a, Z.p, a, Cm.p, r, r, rzk1, a, 1.0, 0.0, s_, true, false);    // U^T Z
          gemm_cm(U.p, a, Cm.p, r, Z.p, a, a, rzk1, r, -1.0, 1.0, s_);                 // Z -= U C
        }
        DBuf Rz((size_t)(rzk1 * rzk1), s_);
        qr(Z.p, a, a, rzk1, Qn.p + a * r, Rz.p, lws_, red_, s_);
        copy(U.p, Qn.p, a * r, s_);
        // V' = SVh^T Rm[:, :r]^T = [SVh^T, 0]: V'[i, j] = SVh[j + i kf] for j < r
        fill(vprime.p, 0.0, bdim * k2, s_);
        transpose(SVh.p, kf, vprime.p, bdim, r, bdim, s_);
      } else {
        DBuf UK((size_t)(a * nc), s_), Rm((size_t)(k2 * nc), s_);
        copy(U.p, UK.p, a * r, s_);
        transpose(left_b.p, rzk1, UK.p + a * r, a, rzk1, a, s_);
        qr(UK.p, a, a, nc, Qn.p, Rm.p, lws_, red_, s_);
        // V'[i, j] = sum_{q<r} SVh[q + i kf] Rm[j + q k2]
        ContractDesc cd;
        cd.M = (int)bdim; cd.N = (int)k2; cd.K = (int)r;
        cd.A = SVh.p; cd.am = Ax::one(kf); cd.ak = Ax::one(1);
        cd.B = Rm.p; cd.bk = Ax::one(k2); cd.bn = Ax::one(1);
        cd.C = vprime.p; cd.cm = Ax::one(1); cd.cn = Ax::one(bdim);
        contract(cd, s_);
      }
      newx.reset((size_t)(a * k2), s_);
      transpose(Qn.p, a, newx.p, k2, a, k2, s_);
    } else {
      newx.reset((size_t)(a * k2), s_);
      transpose(U.p, a, newx.p, k2, a, k2, s_);
    }
    // v <- tensordot(v, x_{k+1}) (amen_solve.h:463)
    const int64_t Y = N_[k + 1] * rx_[k + 2];
    DTensor xn1({k2, N_[k + 1], rx_[k + 2]}, s_);
    if (!last) left_apply(vprime.p, 1, bdim, bdim, k2, x_[k + 1].data(), Y, xn1.data());
    else left_apply(SVh.p, kf, 1, bdim, k2, x_[k + 1].data(), Y, xn1.data());
    nrm2(red_, xn1.data(), xn1.numel(), slot(kNormV), s_);
    scale_dev(xn1.data(), xn1.numel(), nullptr, slot(kNormV), s_);
    DTensor xk({rk, n, k2}, s_);
    copy(newx.p, xk.data(), a * k2, s_);
    x_[k] = std::move(xk);
    x_[k + 1] = std::move(xn1);
    rx_[k + 1] = k2;

    phase(kPhFwdPhi);
    // next interfaces (amen_solve.h:482-503)
    phi_A(true, Phis_[k], x_[k].data(), rk, k2, x_[k].data(), rk, k2, k, Phis_[k + 1]);
    phi_b(true, Phis_b_[k], x_[k].data(), rk, k2, k, Phis_b_[k + 1]);
    nrm2_multi(red_, VecSegs()
                           .norm(Phis_[k + 1].data(), Phis_[k + 1].numel(), slot(kNormPhi))
                           .norm(Phis_b_[k + 1].data(), Phis_b_[k + 1].numel(), slot(kNormPhiB)), s_);
    VecSegs scl;
    scl.scale(Phis_[k + 1].data(), Phis_[k + 1].numel(), slot(kNormPhi))
        .scale(Phis_b_[k + 1].data(), Phis_b_[k + 1].numel(), slot(kNormPhiB));
    if (!last) {
      phi_A(true, Phiz_[k], z_[k].data(), rz_[k], rz_[k + 1], x_[k].data(), rk, k2, k, Phiz_[k + 1]);
      phi_b(true, Phiz_b_[k], z_[k].data(), rz_[k], rz_[k + 1], k, Phiz_b_[k + 1]);
      scl.scale(Phiz_[k + 1].data(), Phiz_[k + 1].numel(), slot(kNormPhi))
          .scale(Phiz_b_[k + 1].data(), Phiz_b_[k + 1].numel(), slot(kNormPhiB));
    }
    scale_multi(scl, s_);
    read_scalars(8);
    double nv = hscal_[kNormV];
    if (!(nv > 0.0)) nv = 1.0;
    double nA = hscal_[kNormPhi];
    if (!(nA > 0.0)) nA = 1.0;
    double nb = hscal_[kNormPhiB];
    if (!(nb > 0.0)) nb = 1.0;
    double nr = nrmsc_ * normA_[k] * normx_[k] / normb_[k];   // amen_solve.h:465
    normx_[k] = normx_[k] * nv;
    normA_[k] = nA;
    normb_[k] = nb;
    nrmsc_ = nr * nb / (nA * normx_[k]);                        // amen_solve.h:496
  } else {
    // last core: x_k = u s v^T = solution (amen_solve.h:406-410, 505-508)
    if (!last) z_update_forward(k, sol.p);
    DTensor xk({rk, n, rk1}, s_);
    copy(sol.p, xk.data(), nl, s_);
    x_[k] = std::move(xk);
  }
  if (!use_full) {
    st_.matvecs += op_count_;
    st_.matvec_flops += op_count_ * lp_flops(op.dims);
    st_.lowp_matvecs += lowp_count_;
    st_.lowp_flops += lowp_count_ * lp_flops(op.dims);
    op_count_ = 0;
    lowp_count_ = 0;
  }
}

// Double-float FP64 products need every operand inside the FP32 exponent range: the A and b cores
// are checked here (the interfaces and solution cores are normalised by the sweep itself).
int AmenRun::choose_fp64_engine() {
  if (p_.fp64_engine == 1) return kFp64Native;
  if (p_.fp64_engine == 2) return kFp64DoubleFloat;
  if (!mixed_) return kFp64Native;
  // Double-float products are accurate to ~1e-13 of the sum of the magnitudes of their terms, so
  // a residual with cancellation (||A|| ||x|| / ||b|| up to cond(A)) carries ~1e-13 cond(A) of
  // error: ample at eps >= 1e-9, marginal below (1e-10 on a system of condition 2e3 is within 50x).
  if (p_.eps < 1e-9) return kFp64Native;
  const int d = d_;
  DBuf nrm((size_t)(2 * d), s_);
  for (int i = 0; i < d; ++i) {
    nrm2(red_, Acore(i), rA_[i] * N_[i] * N_[i] * rA_[i + 1], nrm.p + i, s_);
    nrm2(red_, bcore(i), rb_[i] * N_[i] * rb_[i + 1], nrm.p + d + i, s_);
  }
  std::vector<double> h((size_t)(2 * d));
  TTGB_CUDA(cudaMemcpyAsync(h.data(), nrm.p, 2 * d * sizeof(double), cudaMemcpyDeviceToHost, s_));
  TTGB_CUDA(cudaStreamSynchronize(s_));
  st_.host_syncs++;
  for (double v : h)
    if (!(v < 1e30) || !std::isfinite(v)) return kFp64Native;
  return kFp64DoubleFloat;
}

// FP32 copies of the local operator for the low-precision engine (mixed path)
void AmenRun::setup_lowp(LocalOperator& op, int k) {
  const LocalOpDims& d = op.dims;
  if (use_tc_) {
    tc_local_.setup(d, Phis_[k].data(), Phis_[k + 1].data(), &tc_cores_[k], &spA_[k], tc_err_,
                    s_);
    op.lowp = true;
    op.tc = &tc_local_;
    lowp_count_ = 0;
    op.count_lowp = &lowp_count_;
    op.prof_lowp = prof_lowp_.get();
    return;
  }
  phil32_.ensure((size_t)(d.rl * d.s * d.r), s_);
  phir32_.ensure((size_t)(d.RL * d.S * d.R), s_);
  cast(Phis_[k].data(), phil32_.p, d.rl * d.s * d.r, s_);
  cast(Phis_[k + 1].data(), phir32_.p, d.RL * d.S * d.R, s_);
  const size_t nl = (size_t)(d.r * d.n * d.R);
  xf_.ensure(nl, s_);
  yf_.ensure(nl, s_);
  w1f_.ensure(local_product_w1(d), s_);
  w2f_.ensure(local_product_w2(d), s_);
  op.lowp = true;
  op.phi_l32 = phil32_.p;
  op.A32 = A32_[k].p;
  op.phi_r32 = phir32_.p;
  op.xf = xf_.p;
  op.yf = yf_.p;
  op.w1f = w1f_.p;
  op.w2f = w2f_.p;
  lowp_count_ = 0;
  op.count_lowp = &lowp_count_;
  op.prof_lowp = prof_lowp_.get();
}

// Mixed-path rank search (same rule as amen_solve.h:385-403): the candidate of rank rr leaves out
// the tail U[:, rr:] S Vh[rr:, :], so its residual is (B x - rhs) - B tail. The first term is the
// FP64 residual of the solve; the tail is small near the truncation point, so its product with the
// low-precision operator is accurate to the low-precision unit roundoff relative to ||B tail||.
int AmenRun::rank_search_tail(const double* U, const double* SVh, int64_t a, int64_t bdim,
                              int64_t kf, const double* resvec, double norm_rhs, double thr,
                              const LocalOperator& op, int64_t nl, double* tail_buf) {
  const int kChunk = 4;
  int64_t r = kf;
  DBuf y((size_t)nl, s_);
  while (r > 0) {
    const int64_t nc = r < kChunk ? r : kChunk;
    for (int64_t c = 0; c < nc; ++c) {
      const int64_t rr = r - c;
      if (rr == kf) {
        nrm2(red_, resvec, nl, slot(kCand + (int)c), s_);
        continue;
      }
      ContractDesc cd;   // tail (a x b row-major) = U[:, rr:kf] SVh[rr:kf, :]
      cd.M = (int)a; cd.N = (int)bdim; cd.K = (int)(kf - rr);
      cd.A = U + rr * a; cd.am = Ax::one(1); cd.ak = Ax::one(a);
      cd.B = SVh + rr; cd.bk = Ax::one(1); cd.bn = Ax::one(kf);
      cd.C = tail_buf; cd.cm = Ax::one(bdim); cd.cn = Ax::one(1);
      contract(cd, s_);
      op.apply(tail_buf, y.p, false, s_);
      sub(resvec, y.p, y.p, nl, s_);
      nrm2(red_, y.p, nl, slot(kCand + (int)c), s_);
    }
    read_scalars(kCand + (int)nc);
    for (int64_t c = 0; c < nc; ++c) {
      const double res = hscal_[kCand + c] / norm_rhs;
      if (res > thr) return (int)(r - c);
    }
    r -= nc;
  }
  return 0;
}

// z update after the local solve (amen_solve.h:418-442)
void AmenRun::z_update_forward(int k, const double* trunc) {
  const int64_t n = N_[k];
  const int64_t ap = rz_[k] * n, bp = rz_[k + 1];
  DBuf czA((size_t)(ap * bp), s_), czy((size_t)(ap * bp), s_);
  local_prod(Phiz_[k].data(), rz_[k], rx_[k], Phiz_[k + 1].data(), rz_[k + 1], rx_[k + 1], k, trunc,
             czA.p);
  lrhs(Phiz_b_[k].data(), rz_[k], k, Phiz_b_[k + 1].data(), rz_[k + 1], nrmsc_, czy.p);
  axpby(-1.0, czA.p, 1.0, czy.p, ap * bp, s_);
  const int64_t kf = ap < bp ? ap : bp;
  DBuf Mc((size_t)(ap * bp), s_);
  transpose(czy.p, bp, Mc.p, ap, bp, ap, s_);
  const int64_t tk = p_.kickrank < kf ? p_.kickrank : kf;
  const int64_t kc = tk + ((k < d_ - 1) ? p_.kick2 : 0);
  DBuf cz;
  if (kc == kf && kf == bp) {   // all singular vectors kept, none appended: orthonormalise Mc
    cz = std::move(Mc);
  } else {
    DBuf U((size_t)(ap * kf), s_), S((size_t)kf, s_), Vh((size_t)(kf * bp), s_);
    svd(Mc.p, ap, ap, bp, U.p, S.p, Vh.p, lws_, red_, s_);
    cz.reset((size_t)(ap * kc), s_);
    copy(U.p, cz.p, ap * tk, s_);
    if (kc > tk) randn_fill(cz.p + ap * tk, ap * (kc - tk));
  }
  const int64_t k3 = ap < kc ? ap : kc;
  DBuf qz((size_t)(ap * k3), s_), Rz((size_t)(k3 * kc), s_);
  qr(cz.p, ap, ap, kc, qz.p, Rz.p, lws_, red_, s_);
  rz_[k + 1] = k3;
  DTensor zk({rz_[k], n, k3}, s_);
  transpose(qz.p, ap, zk.data(), k3, ap, k3, s_);
  z_[k] = std::move(zk);
}

// Engine of the GEMMs of the mixed path's dense linear algebra (the CholeskyQR3 Gram and apply
// products, U = Q V', the enrichment's block Gram-Schmidt, reconstructions): double-float whenever
// the mixed path's FP64 products are double-float. Those GEMMs dominate the SM time of a solve on
// GB300's FP64 pipe; in double-float they keep ~1e-13 of the sum of magnitudes of their terms,
// Q stays orthogonal to ~1e-13 (CholeskyQR3's third pass), far below the eps >= 1e-9 where the
// double-float engine is chosen. The Cholesky factorisations, the Jacobi rotations, Gram-Schmidt
// of the Krylov basis and every norm stay native FP64. TTGB_LA_ENGINE=native keeps them native.
static int linalg_engine(int fp64_products_engine, double eps) {
  static const bool force_native = [] {
    const char* e = std::getenv("TTGB_LA_ENGINE");
    return e != nullptr && std::string(e) == "native";
  }();
  // only where the automatic choice takes double-float at all (eps >= 1e-9): a caller that forces
  // double-float products below that keeps the factorisations' GEMMs native
  return (fp64_products_engine == kFp64DoubleFloat && eps >= 1e-9 && !force_native)
             ? kFp64DoubleFloat : kFp64Native;
}

AmenResult AmenRun::run(const TTView& x0, const TTView& z0) {
  init(x0, z0);
  // every contraction issued by this solve's thread outside the scopes of the FP64 products
  Fp64EngineScope la_engine(mixed_ ? linalg_engine(fp64e_, p_.eps) : kFp64Native);
  bool last = false;
  int swp = 0;
  double max_res = 0.0;
  const auto t0 = std::chrono::steady_clock::now();
  for (swp = 0; swp < p_.nswp; ++swp) {   // amen_solve.h:212
    for (int k = d_ - 1; k > 0; --k) backward_step(k, swp, last);
    max_res = 0.0;
    for (int k = 0; k < d_; ++k) forward_step(k, swp, last, max_res);
    if (p_.verbose) {
      std::printf("Sweep %d%s: ranks [", swp + 1, last ? " (last)" : "");
      for (auto r : rx_) std::printf(" %lld", (long long)r);
      const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      std::printf(" ] max_res %g elapsed %.3f s\n", max_res, el);
    }
    if (last) break;   // amen_solve.h:522-526
    if (max_res < eps_) last = true;
  }
  phase(kPhOther);
  st_.sweeps = swp < p_.nswp ? swp + 1 : swp;
  st_.max_res = max_res;
  st_.converged = last ? 1 : 0;
  double lg = 0.0;   // amen_solve.h:534-541
  for (int i = 0; i < d_ - 1; ++i) lg += std::log(normx_[i]);
  const double norm_x = std::exp(lg / d_);
  AmenResult res;
  for (int i = 0; i < d_; ++i) {
    scale_copy(x_[i].data(), norm_x, x_[i].data(), x_[i].numel(), s_);
    res.cores.push_back(std::move(x_[i]));
  }
  res.ranks = rx_;
  TTGB_CUDA(cudaStreamSynchronize(s_));
  if (tc_err_) {
    int herr = 0;
    TTGB_CUDA(cudaMemcpy(&herr, tc_err_, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) throw Error(kTimeout, "tcgen05 GEMM: a bounded wait gave up");
  }
  if (phases_) {
    phases_->flush();
    for (int i = 0; i < PhaseTimer::kPhases && i < 12; ++i) st_.phase_ms[i] = phases_->ms[i];
  }
  if (prof_) {
    prof_->flush();
    st_.contract_ms = prof_->ms;
    st_.contract_launches = prof_->launches;
    st_.contract_flops = prof_->flops;
    prof_lowp_->flush();
    st_.lowp_ms = prof_lowp_->ms;
    st_.lowp_launches = prof_lowp_->launches;
    st_.lowp_gemm_flops = prof_lowp_->flops;
    prof_krylov_->flush();
    st_.krylov_ms = prof_krylov_->ms;
    st_.krylov_launches = prof_krylov_->launches;
    st_.krylov_bytes = prof_krylov_->flops;
    st_.krylov_traffic_bytes = prof_krylov_->aux;
  }
  res.stats = st_;
  return res;
}

}  // namespace

int64_t max_reachable_rank(const TTView& A, const TTView& x0, const AmenParams& p) {
  const int d = A.d;
  int64_t r0 = 1;
  if (x0.d == d)
    for (int k = 0; k <= d; ++k) r0 = std::max<int64_t>(r0, x0.ranks[k]);
  const double grow = (double)r0 + (double)p.nswp * (double)(p.kickrank + p.kick2);
  double best = 1.0;
  // mode-size cap of bond k (between cores k-1 and k): min(prod_{i<k} n_i, prod_{i>=k} n_i)
  for (int k = 1; k < d; ++k) {
    double left = 1.0, right = 1.0;
    for (int i = 0; i < k; ++i) left *= (double)A.cols[i];
    for (int i = k; i < d; ++i) right *= (double)A.cols[i];
    best = std::max(best, std::min(std::min(left, right), grow));
  }
  return (int64_t)std::min<double>(best, (double)p.rmax);
}

size_t footprint_bound(const TTView& A, const TTView& b, const TTView& x0, const AmenParams& p) {
  int64_t nmax = 1, smax = 1, rbmax = 1;
  for (int k = 0; k < A.d; ++k) {
    nmax = std::max<int64_t>(nmax, A.cols[k]);
    smax = std::max<int64_t>(smax, A.ranks[k + 1]);
    rbmax = std::max<int64_t>(rbmax, b.ranks[k + 1]);
  }
  const double r = (double)max_reachable_rank(A, x0, p);
  const double rz = (double)(p.kickrank + p.kick2) + 1.0;
  const double core = r * r * (double)nmax;                  // one solution core
  // per core: x, the previous x during a step, z; interfaces Phi (r s r), Phiz (rz s r), Phi_b
  // (rb r), Phiz_b (rb rz)
  const double per_core = 2.0 * core + rz * r * (double)nmax + (r * r + rz * r) * (double)smax +
                          (double)rbmax * (r + rz);
  // local working set of the largest core: Krylov basis, contraction intermediates (x s, S sides),
  // mixed-path FP32/TF32 split copies, supercore SVD/QR (matrix, U, V, Gram) and vectors
  const double nloc = core;
  const double local = (double)(p.local_iterations + 1) * nloc + 2.0 * nloc * (double)smax +
                       2.0 * nloc * (double)smax /* split copies, 2 x FP32 */ + 6.0 * nloc +
                       6.0 * r * r + 16.0 * nloc;
  return (size_t)(8.0 * ((double)A.d * per_core + local)) + ((size_t)64 << 20);
}

void randn(double* out, int64_t n, uint64_t seed, uint64_t offset, cudaStream_t s) {
  if (n <= 0) return;
  randn_kernel<<<grid_of(n), 256, 0, s>>>(out, n, seed, offset);
  TTGB_CHECK_LAUNCH();
}

static void validate(const TTView& A, const TTView& b) {
  // torchtt/solvers.py:259-266 and the rank consistency of torchtt/_tt_base.py:123-161
  TTGB_REQUIRE(A.d >= 1 && A.d == b.d, "Dimension mismatch.");
  TTGB_REQUIRE((int)A.rows.size() == A.d, "A must be TT-matrix and b must be vector.");
  for (int k = 0; k < A.d; ++k) {
    TTGB_REQUIRE(A.rows[k] == A.cols[k], "A is not quadratic.");
    TTGB_REQUIRE(A.cols[k] == b.cols[k], "Dimension mismatch.");
    TTGB_REQUIRE(A.cores[k] != nullptr && b.cores[k] != nullptr, "null core pointer");
  }
  TTGB_REQUIRE(A.ranks.front() == 1 && A.ranks.back() == 1 && b.ranks.front() == 1 &&
                   b.ranks.back() == 1,
               "Check the ranks and the mode size.");
}

AmenResult amen_solve(const TTView& A, const TTView& b, const TTView& x0, const TTView& z0,
                      const AmenParams& p, cudaStream_t stream) {
  validate(A, b);
  if (x0.d != 0) {
    TTGB_REQUIRE(x0.d == A.d && x0.ranks.front() == 1 && x0.ranks.back() == 1, "Check the ranks and the mode size.");
    for (int k = 0; k < A.d; ++k) TTGB_REQUIRE(x0.cols[k] == A.cols[k], "Dimension mismatch.");
  }
  TTGB_REQUIRE(p.nswp >= 1 && p.local_iterations >= 1 && p.resets >= 1 && p.kickrank >= 0 &&
                   p.kick2 >= 0 && p.rmax >= 1 && p.eps > 0.0,
               "invalid solver parameters");
  TTGB_REQUIRE(p.prec >= 0 && p.prec <= 2, "Invalid preconditioner.");
  AmenRun run(A, b, p, stream);
  return run.run(x0, z0);
}

}  // namespace ttgb
