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
  // second the bytes the CGS2 kernels read and write, 8 N_loc (4k + 10)
  Profiler* prof_krylov = nullptr;
  int64_t* count_lowp = nullptr;
  int64_t size() const { return dims.r * dims.n * dims.R; }
  void apply(const double* x, double* y, bool use_prec, cudaStream_t s) const;
  void apply_fp64(const double* x, double* y, cudaStream_t s) const;
  void apply_prec(const double* x, double* y, cudaStream_t s) const;
};

struct GmresWS {
  DBuf Q;        // (iters + 1) x n Krylov basis
  DBuf small;    // H, cs, sn, beta, h1, h2, scalars
  int* h_flag = nullptr;   // pinned: converged flag, iteration count
  int* d_flag = nullptr;
};

struct GmresResult {
  int flag = 0;   // 1 when the threshold was reached (gmres.h:125-129)
  int nit = 0;    // total iterations over all restarts
};

// Restarted GMRES from x0 = 0: solves op(x) = rhs with relative threshold `threshold` on the
// residual reduction |beta_{k+1}| / ||rhs||, at most `iters` iterations per cycle and `resets`
// cycles. The orthogonalisation is classical Gram-Schmidt applied twice (CGS2), which is as
// stable as the reference's modified Gram-Schmidt and needs 3 passes over the basis instead of
// 2(k+1) dependent ones; Givens rotations and the convergence test run on the device.
GmresResult gmres(const LocalOperator& op, const double* rhs, double* sol, int iters,
                  double threshold, int resets, GmresWS& ws, const RedWS& red, cudaStream_t s);

}  // namespace ttgb
