// The local AMEn product on the tcgen05 engine (3xTF32, FP32 accumulation in tensor memory):
// y[l,m,L] = sum Phi_l[l,s,r] A[s,m,n,S] Phi_r[L,S,R] x[r,n,R] as three tensor-core GEMMs whose
// operands are all K-major:
//   W [l][R][s][n]  = x^P [(n,R), r]   . Phi_l [(l,s), r]^T       (x^P: x gathered to (n,R,r))
//   Y2[l][m][S][R]  = A'  [(m,S),(s,n)] . W_l  [R, (s,n)]^T        (batched over l; A' = A permuted)
//   y [l][m][L]     = Y2  [(l,m),(S,R)] . Phi_r [L, (S,R)]^T
// Each epilogue writes the next operand directly as a TF32 hi/lo split; the last writes FP64.
// With a sparse A core the middle GEMM is replaced by the structured A stage: W is written in
// FP32 as W[l][s][n][R] and the stage writes Y2 as the TF32 split.
#pragma once

#include "contract.cuh"
#include "tc_gemm.cuh"

namespace ttgb {

// A' [(m,S),(s,n)] split of one A core (s x m x n x S), shared by every local problem of that core
struct TcCore {
  FBuf hi, lo;
  int64_t ld = 0;   // row pitch of A' (s n rounded up to 4 floats)
  void build(const double* A, int64_t s, int64_t m, int64_t n, int64_t S, cudaStream_t st);
};

struct TcLocal {
  LocalOpDims d{};
  const TcCore* core = nullptr;
  const SparseCore* sp = nullptr;   // when sp->use, the A stage runs from the nonzeros (FP32)
  FBuf phl_h, phl_l, phr_h, phr_l, xh, xl, wh, wl, yh, yl, wf;
  int64_t ld_r = 0, ld_sn = 0, ld_SR = 0;   // padded row pitches of the K-major operands
  int* err = nullptr;   // device flag of the bounded waits
  void setup(const LocalOpDims& dims, const double* phi_l, const double* phi_r, const TcCore* c,
             const SparseCore* spa, int* errflag, cudaStream_t st);
  // presplit: xh / xl already hold x's split (written by the producer of x), so the split
  // launch is skipped. gate (device flag, optional): the GEMMs and the A stage do nothing when
  // it is non-zero at launch time.
  void apply(const double* x, double* y, cudaStream_t st, bool presplit = false,
             const int* gate = nullptr);
};

}  // namespace ttgb
