// tcgen05 (5th-generation tensor core) GEMM for the low-precision local operator of the mixed path.
//
// C[b](m, n) = sum_k A[b](m, k) B[b](n, k), with A and B K-major FP32 arrays holding TF32 values
// split in two (x = hi + lo, both TF32), so one GEMM is the three tensor-core products
// hi*hi + hi*lo + lo*hi accumulated in FP32 in tensor memory (3xTF32: ~2^-22 relative accuracy of
// the operands, FP32 accumulation). One CTA computes a 128 x BN tile (BN <= 128). The operand tiles
// are fetched by TMA (cp.async.bulk.tensor, one tensor map per operand) into a ring of
// 128-byte-swizzled shared-memory stages, consumed by one MMA-issuing thread, and the accumulator
// is read back with tcgen05.ld by four epilogue warps and written with arbitrary (two-level) output
// strides, as FP32, FP64 or a new TF32 split. Operand rows must start on 16-byte boundaries: the
// leading dimensions (and batch strides) are multiples of 4 floats, the bases 16-byte aligned; K
// and the row counts are the true extents (the copy fills zeros beyond them).
#pragma once

#include "common.cuh"

namespace ttgb {

struct TcAx {         // output index -> offset, i = i1 * e0 + i0
  int e0 = 1 << 30;
  int64_t s1 = 0, s0 = 1;
};

enum TcOut : int { kTcOutF32 = 0, kTcOutF64 = 1, kTcOutSplit = 2 };

struct TcGemm {
  int M = 0, N = 0, K = 0, batch = 1;
  const float* A_hi = nullptr;
  const float* A_lo = nullptr;
  int64_t lda = 0, a_bs = 0;      // A(m, k) at A[b*a_bs + m*lda + k]
  const float* B_hi = nullptr;
  const float* B_lo = nullptr;
  int64_t ldb = 0, b_bs = 0;      // B(n, k) at B[b*b_bs + n*ldb + k]
  int out = kTcOutF32;
  float* C32 = nullptr;           // kTcOutF32
  double* C64 = nullptr;          // kTcOutF64
  float* C_hi = nullptr;          // kTcOutSplit
  float* C_lo = nullptr;
  TcAx cm, cn;
  int64_t c_bs = 0;
  float alpha = 1.0f;
  const int* gate = nullptr;   // device flag: when non-zero at launch time the GEMM does nothing
};

// Launches the tcgen05 GEMM; `err` (device int) is set non-zero when a bounded wait gave up.
void tc_gemm(const TcGemm& g, int* err, cudaStream_t s);

// Splits x (FP64) into TF32 hi/lo with a gather: element i of the gathered sequence comes from
// x[perm(i)] where i = ((i3 * e2 + i2) * e1 + i1) * e0 + i0 -> x[i3*s3 + i2*s2 + i1*s1 + i0*s0]
// (a 4-index permutation), and is stored at (i / inner) * out_ld + i % inner: rows of `inner`
// elements with a padded pitch out_ld (inner <= 0: one contiguous row).
struct Gather4 {
  int64_t e0 = 1, e1 = 1, e2 = 1, e3 = 1;
  int64_t s0 = 1, s1 = 0, s2 = 0, s3 = 0;
};
void split_tf32(const double* x, const Gather4& g, float* hi, float* lo, cudaStream_t s,
                int64_t inner = 0, int64_t out_ld = 0);

// row pitch of a K-major tensor-core operand with K elements per row: K rounded up to 4 floats
inline int64_t tc_ld(int64_t K) { return (K + 3) & ~int64_t(3); }

// true when the device supports tcgen05 (sm_100 family)
bool tc_available();

// round an FP32 value to TF32 (round to nearest, ties away), as the tensor core reads it
__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

}  // namespace ttgb
