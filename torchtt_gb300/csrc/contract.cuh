// FP64 tensor-contraction engine: a batched GEMM whose M, N and K indices may each be a pair of
// tensor indices with independent strides, so the permutes of the reference's tensordot chains
// (cpp/amen_solve.h:17-98, cpp/matvecs.h:196-212) are folded into addressing instead of copies.
#pragma once

#include "common.cuh"
#include "sparse_a.cuh"

namespace ttgb {

// One GEMM index i in [0, extent) split as i = i1 * e0 + i0 with address offset i1 * s1 + i0 * s0.
// A single-stride index has e0 >= extent (then only s0 is used).
struct Ax {
  int64_t e0 = 1 << 30;
  int64_t s1 = 0;
  int64_t s0 = 1;
  static Ax one(int64_t s) { Ax a; a.e0 = int64_t(1) << 40; a.s1 = 0; a.s0 = s; return a; }
  static Ax two(int64_t e0, int64_t s1, int64_t s0) { Ax a; a.e0 = e0; a.s1 = s1; a.s0 = s0; return a; }
};

// C[b](m, n) = alpha * sum_k A[b](m, k) * B[b](k, n) + beta * C[b](m, n)
template <typename T>
struct ContractDescT {
  int M = 0, N = 0, K = 0, batch = 1;
  const T* A = nullptr;
  Ax am, ak;
  int64_t a_bs = 0;
  const T* B = nullptr;
  Ax bk, bn;
  int64_t b_bs = 0;
  T* C = nullptr;
  Ax cm, cn;
  int64_t c_bs = 0;
  T alpha = T(1), beta = T(0);
  // structure flags: kTriLowerC computes only output tiles that touch m >= n (a symmetric
  // product whose upper part is not read); kTriUpperB treats B(k, n) as zero for k > n (an upper
  // triangular right factor), so a column tile sums only k < its last column.
  int tri = 0;
  // C holds zeros on entry (with beta = 0): a split-K launch then adds its partial sums into C
  // without the launch that would first scale C by beta
  bool c_zero = false;
};
constexpr int kTriLowerC = 1;
constexpr int kTriUpperB = 2;
using ContractDesc = ContractDescT<double>;
using ContractDescF = ContractDescT<float>;

// Arithmetic of the FP64 contractions issued by the calling thread: kFp64Native runs them on the
// FP64 pipe; kFp64DoubleFloat in double-float arithmetic on the FP32 pipe (~1e-13 relative, for
// operands within the FP32 exponent range). Set for a scope with Fp64EngineScope.
constexpr int kFp64Native = 0;
constexpr int kFp64DoubleFloat = 1;
struct Fp64EngineScope {
  explicit Fp64EngineScope(int engine);
  ~Fp64EngineScope();
  Fp64EngineScope(const Fp64EngineScope&) = delete;
  Fp64EngineScope& operator=(const Fp64EngineScope&) = delete;
 private:
  int prev_;
};

// Within this scope the calling thread's contractions run no tile-tuning measurements (which
// synchronise the host): a shape class that already has a record uses it, others the heuristic.
struct NoTuningScope {
  NoTuningScope();
  ~NoTuningScope();
  NoTuningScope(const NoTuningScope&) = delete;
  NoTuningScope& operator=(const NoTuningScope&) = delete;
 private:
  bool prev_;
};

// Launches the contraction on `stream`. The tile shape and split-K (C pre-scaled by beta, partial
// sums added atomically) come from the tile autotuner's record for the launch's shape class, or
// from an occupancy heuristic (deterministic requests never split K).
void contract(const ContractDesc& d, cudaStream_t stream, bool deterministic = false);
// The same engine in FP32 (CUDA-core FFMA), for the low-precision local operator.
void contract(const ContractDescF& d, cudaStream_t stream, bool deterministic = false);
// Tile autotuner switch: 1 on (default unless TTGB_AUTOTUNE=0), 0 off, other values only query.
// Returns the previous state.
int set_autotune(int mode);
// Number of shape classes with a record (including classes being tuned).
int64_t autotune_classes();

// Local AMEn product y[l,m,L] = sum Phi_left[l,s,r] A[s,m,n,S] Phi_right[L,S,R] x[r,n,R]
// (reference: local_product, cpp/amen_solve.h:17-27). `w1` needs r_l*s*n*R and `w2` r_l*m*S*R
// doubles (r_l = rows of Phi_left). `batch` independent right-hand sides x (stride x_bs) give
// batch outputs (stride y_bs).
struct LocalOpDims {
  int64_t rl, s, r;      // Phi_left: rl x s x r
  int64_t m, n, S;       // A core: s x m x n x S
  int64_t RL, R;         // Phi_right: RL x S x R
};
// `sp` (optional): the nonzero structure of A; when sp->use the A stage runs from it.
void local_product(const LocalOpDims& d, const double* phi_l, const double* A, const double* phi_r,
                   const double* x, double* y, double* w1, double* w2, cudaStream_t stream,
                   double alpha = 1.0, double beta = 0.0, const SparseCore* sp = nullptr);
void local_product(const LocalOpDims& d, const float* phi_l, const float* A, const float* phi_r,
                   const float* x, float* y, float* w1, float* w2, cudaStream_t stream,
                   float alpha = 1.0f, float beta = 0.0f, const SparseCore* sp = nullptr);
inline size_t local_product_w1(const LocalOpDims& d) { return size_t(d.rl * d.s * d.n * d.R); }
inline size_t local_product_w2(const LocalOpDims& d) { return size_t(d.rl * d.m * d.S * d.R); }

// Interface updates (reference: cpp/amen_solve.h:38-98). Shapes:
//   fwd_A: Phi[l,s,r] (rl x s x r), left[l,M,L], A[s,M,N,S], right[r,N,R] -> out[L,S,R]
//   bck_A: Phi[L,S,R], left[l,M,L], A[s,M,N,S], right[r,N,R]              -> out[l,s,r]
//   fwd_rhs: Phi[b,r], core_b[b,n,B], core[r,n,R] -> out[B,R]
//   bck_rhs: Phi[B,R], core_b[b,n,B], core[r,n,R] -> out[b,r]
struct PhiDims {
  int64_t l, L;   // left core ranks  (l x M x L)
  int64_t s, S;   // A core ranks
  int64_t r, R;   // right core ranks (r x N x R)
  int64_t M, N;   // mode sizes (rows, cols of the A core)
};
size_t phi_A_workspace(const PhiDims& d);   // doubles needed by phi_fwd_A / phi_bck_A
void phi_fwd_A(const PhiDims& d, const double* phi, const double* left, const double* A,
               const double* right, double* out, double* work, cudaStream_t stream,
               const SparseCore* sp = nullptr);
void phi_bck_A(const PhiDims& d, const double* phi, const double* left, const double* A,
               const double* right, double* out, double* work, cudaStream_t stream,
               const SparseCore* sp = nullptr);
struct PhiRhsDims {
  int64_t b, B;   // rhs core ranks (b x n x B)
  int64_t r, R;   // solution core ranks (r x n x R)
  int64_t n;
};
size_t phi_rhs_workspace(const PhiRhsDims& d);
void phi_fwd_rhs(const PhiRhsDims& d, const double* phi, const double* core_b, const double* core,
                 double* out, double* work, cudaStream_t stream);
void phi_bck_rhs(const PhiRhsDims& d, const double* phi, const double* core_b, const double* core,
                 double* out, double* work, cudaStream_t stream);
// Local right-hand side rhs[r,n,R] = alpha * sum Phi_l[b,r] core_b[b,n,B] Phi_r[B,R]
// (reference: cpp/amen_solve.h:303-304). work: b*n*R doubles... see local_rhs_workspace.
size_t local_rhs_workspace(int64_t b, int64_t n, int64_t B, int64_t r, int64_t R);
void local_rhs(int64_t b, int64_t n, int64_t B, int64_t r, int64_t R, const double* phi_l,
               const double* core_b, const double* phi_r, double alpha, double* out, double* work,
               cudaStream_t stream);

}  // namespace ttgb
