// Structure-aware A-core stage of the contractions. The operators of the AMEn workloads are
// Kronecker sums: their TT cores A_k[s, m, n, S] are blocks that are zero, identity, diagonal
// (potentials) or tridiagonal (1-D Laplacians), a few per cent dense. The reference contracts
// them densely (cpp/amen_solve.h:21-25,42-46,62-66); on GB300, where FP64 runs at 1/57 of the FP32
// rate, the A stage is the larger half of every local product and interface update. A core whose
// density is below 1/4 is instead applied from its nonzeros: each output element sums at most a
// handful of products, so the stage becomes a bandwidth-bound gather. Products with exact zeros
// are skipped, so results equal the dense contraction up to the order of the sums.
#pragma once

#include "common.cuh"

namespace ttgb {

// Nonzeros of one A core grouped by an output key (CSR): for each key, the nonzeros with their
// two remaining indices (a, b) and value.
struct SparseCsr {
  int64_t keys = 0, nnz = 0;
  int max_row = 0;
  DevBuf<int> rp;      // keys + 1 row pointers
  DevBuf<int> a, b;    // nnz
  DBuf val;            // nnz, FP64
  FBuf val32;          // nnz, FP32 (low-precision engines)
};

struct SparseCore {
  bool use = false;
  int64_t s = 0, M = 0, N = 0, S = 0;
  SparseCsr lp;   // key (m, S) = m*S + S, pairs (s, n): local product stage
  SparseCsr fw;   // key (N, S) = N*S + S, pairs (s, M): forward interface stage
  SparseCsr bk;   // key (s, N) = s*N + N, pairs (M, S): backward interface stage
  SparseCsr rh;   // key (s, M) = s*M + M, pairs (N, S): right half of a two-site product
  // Reads the core (device, FP64, s x M x N x S) once and sets `use` when fewer than a quarter of
  // its entries are nonzero and no key has more than kMaxRow nonzeros.
  void build(const double* A, int64_t s, int64_t M, int64_t N, int64_t S, cudaStream_t st);
  static constexpr int kMaxRow = 64;
};

// out[koff(key) + o1*so1 + o2] = sum_{j in row key} val[j] * in[o1*si1 + o2 + a[j]*pa + b[j]*pb]
// for every key < c.keys, o1 < O1, o2 < O2 (the output is overwritten), where
// koff(key) = key*sk, or (key % ke0)*sk + (key / ke0)*sk1 when ke0 > 0.
struct StageDims {
  int64_t O1, O2, si1, so1, sk, pa, pb;
  int64_t ke0 = 0, sk1 = 0;
  const int* gate = nullptr;   // device flag: when non-zero at launch time the stage does nothing
};
void sparse_stage(const SparseCsr& c, const double* in, double* out, const StageDims& g,
                  cudaStream_t s);
void sparse_stage(const SparseCsr& c, const float* in, float* out, const StageDims& g,
                  cudaStream_t s);
// FP32 input, output written as a TF32 split (hi + lo) for a following tensor-core GEMM
void sparse_stage_split(const SparseCsr& c, const float* in, float* hi, float* lo,
                        const StageDims& g, cudaStream_t s);

}  // namespace ttgb
