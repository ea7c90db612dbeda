// Local AMEn operator and the restarted GMRES that solves with it
// (reference: AMENsolveMV, cpp/matvecs.h:130-212; gmres / gmres_single, cpp/gmres.h:34-161).
#pragma once

#include "blas1.cuh"
#include "contract.cuh"
#include "profiler.cuh"
#include "tc_local.cuh"

namespace ttgb {

// algorithmic flops of one local product: 2 rl n R (s r) + 2 rl m S R (s n) + 2 rl m RL (S R)
inline double local_product_flops(const LocalOpDims& d) {
  return 2.0 * d.rl * d.n * d.R * (double)d.s * d.r + 2.0 * d.rl * d.m * d.S * (double)d.R * d.s * d.n +
         2.0 * d.rl * d.m * (double)d.RL * d.S * d.R;
}

// flops executed by the GEMM launches of one local product: the A stage is excluded when it runs
// from the nonzeros of a sparse core (it is then a gather, bounded by memory, not by flops)
inline double local_product_gemm_flops(const LocalOpDims& d, const SparseCore* sp) {
  if (sp && sp->use)
    return 2.0 * d.rl * d.n * d.R * (double)d.s * d.r + 2.0 * d.rl * d.m * (double)d.RL * d.S * d.R;
  return local_product_flops(d);
}

enum Prec : int { kNoPrec = 0, kCPrec = 1, kRPrec = 2 };   // cpp/define.h:10-12

// Where a kernel that produces the operator's next input vector x (r x n x R, row-major) can also
// write that vector's TF32 hi/lo split for the tcgen05 engine: element i goes to row i mod (n R),
// column i / (n R), at row pitch ld (the engine's K-major x operand). hi == nullptr: no target.
struct SplitOut {
  float* hi = nullptr;
  float* lo = nullptr;
  int64_t nR = 1;
  int64_t ld = 1;
};

// y = B x with B = Phi_left x A_k x Phi_right (the projected operator), optionally composed with
// the block-Jacobi preconditioner P: y = B (P x).
struct LocalOperator {
  LocalOpDims dims{};
  const double* phi_l = nullptr;
  const double* A = nullptr;
  const double* phi_r = nullptr;
  const SparseCore* spA = nullptr;   // nonzero structure of A (structured A stage), optional
  int fp64_engine = kFp64Native;     // arithmetic of the FP64 products (contract.cuh)
  int prec = kNoPrec;
  const double* J = nullptr;    // preconditioner blocks (see prec.cu)
  double* w1 = nullptr;         // local_product workspaces
  double* w2 = nullptr;
  double* wp = nullptr;         // preconditioned input (N_loc)
  Profiler* prof = nullptr;     // optional launch timing
  int64_t* count = nullptr;     // optional: incremented per application
  // Low-precision engine (mixed path): when lowp is set, apply() runs the contraction in FP32 on
  // FP32 copies of the operator (phi_l32, A32, phi_r32) and converts the vector in and out;
  // apply_fp64() always uses the FP64 operator (true residuals).
  bool lowp = false;
  const float* phi_l32 = nullptr;
  const float* A32 = nullptr;
  const float* phi_r32 = nullptr;
  float* xf = nullptr;          // N_loc
  float* yf = nullptr;          // N_loc
  float* w1f = nullptr;
  float* w2f = nullptr;
  TcLocal* tc = nullptr;        // when set, the low-precision engine is the tcgen05 3xTF32 GEMM
  Profiler* prof_lowp = nullptr;  // optional timing of the low-precision products
  // optional timing of the Krylov orthogonalisation of each GMRES iteration; its first figure is
  // the reference's algorithmic bytes 8 N_loc (2k + 3) of iteration k (k + 1 basis vectors), the
  // second the bytes the Arnoldi kernels read and write, 8 N_loc (2k + 7), plus 8 N_loc (k + 1)
  // for an iteration that takes the second projection
  Profiler* prof_krylov = nullptr;
  int64_t* count_lowp = nullptr;
  int64_t size() const { return dims.r * dims.n * dims.R; }
  // The split target of apply()'s input when the input goes to the tcgen05 engine unchanged
  // (mixed path, no preconditioner); otherwise an empty target.
  SplitOut input_split() const;
  // presplit: the caller has already written x's split to input_split() (see SplitOut).
  // gate (device flag, optional): on the tcgen05 engine the product's kernels do nothing when it
  // is non-zero at launch time (GMRES iterations queued past their stopping point)
  void apply(const double* x, double* y, bool use_prec, cudaStream_t s, bool presplit = false,
             const int* gate = nullptr) const;
  void apply_fp64(const double* x, double* y, cudaStream_t s) const;
  void apply_prec(const double* x, double* y, cudaStream_t s) const;
};

// Words of GmresWS::d_flag (device) / h_flag (pinned host copy).
enum GmresFlag : int {
  kGmresState = 0,        // 0 running, 1 stopped (threshold or breakdown), 2 zero start, 3 non-finite
  kGmresBreakdown = 1,    // 1 when the stop was a breakdown (H[k+1, k] = 0)
  kGmresAtIter = 2,       // iteration at which the state was set
  kGmresReorth = 3,       // iterations of the cycle that took the second projection
  kGmresReorthVecs = 4,   // basis vectors those second projections read
  kGmresFlagWords = 5
};

struct GmresWS {
  DBuf Q;        // (iters + 1) x n Krylov basis
  DBuf small;    // H, cs, sn, beta, h1, h2, scalars
  int* h_flag = nullptr;   // pinned, >= kGmresFlagWords ints
  int* d_flag = nullptr;   // device, >= kGmresFlagWords ints
  double log_rate = 0.0;   // log(threshold) / iterations of the last converged cycle (0: unknown)
};

struct GmresResult {
  int flag = 0;      // 1 when the threshold was reached (gmres.h:125-129)
  int nit = 0;       // total iterations over all restarts
  int syncs = 0;     // host reads of the stop flag
  int overrun = 0;   // iterations queued past the stopping point (their results are not used)
  int reorth = 0;    // iterations that took the second projection
};

// Restarted GMRES from x0 = 0: solves op(x) = rhs with relative threshold `threshold` on the
// residual reduction |beta_{k+1}| / ||rhs||, at most `iters` iterations per cycle and `resets`
// cycles. Each Arnoldi step is three launches over the basis: the projection h1 = V^T w; the
// update w' = w - V h1 fused with h2 = V^T w' (one read of V); and the finishing pass, which
// applies the second projection only when the first lost more than half of ||w||^2 (classical
// Gram-Schmidt with the DGKS reorthogonalisation criterion, as stable as the reference's modified
// Gram-Schmidt), normalises, and runs the Givens rotations and the convergence test on the
// device. The host reads the stop flag only from the iteration where the convergence rate of the
// previous cycle predicts the stop; iterations queued past the stop leave the solution unchanged.
// orth_tol > 0 also skips the second projection when the first leaves |V^T w'| <= orth_tol |w'|
// (measured in the same pass), i.e. it keeps the basis orthogonal to orth_tol instead of to
// rounding: for GMRES runs whose own tolerance is far above orth_tol.
GmresResult gmres(const LocalOperator& op, const double* rhs, double* sol, int iters,
                  double threshold, int resets, GmresWS& ws, const RedWS& red, cudaStream_t s,
                  double orth_tol = 0.0);

}  // namespace ttgb
