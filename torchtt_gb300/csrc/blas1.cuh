// Vector kernels of the AMEn path: deterministic reductions (norms, dots, multi-dots) whose result
// stays in device memory, and the element-wise updates of the local solves.
#pragma once

#include "common.cuh"

namespace ttgb {

// Scratch of the two-stage reductions. A reduction launches G blocks that write G partial sums;
// the last block to finish (atomic ticket) adds them in block order, so results are deterministic.
struct RedWS {
  double* partial = nullptr;    // cap_blocks * cap_vec doubles
  unsigned* counter = nullptr;  // one ticket counter, returned to 0 by the last block
  int cap_blocks = 0;
  int cap_vec = 0;
};

int red_blocks(int64_t n);
// grid of a reduction over n elements with nvec partial sums per block: G blocks of `chunk`
// consecutive elements (a multiple of 256), G <= ws.cap_blocks; nvec must fit ws.cap_vec
void red_launch_dims(const RedWS& ws, int64_t n, int nvec, int& G, int64_t& chunk);

// out[0] = ||x||_2 (out[1] = ||x||_2^2 if `both`)
void nrm2(const RedWS& ws, const double* x, int64_t n, double* out, cudaStream_t s);

// Up to four vectors handled by one launch: x_i of n_i elements, with a device output (norms) or
// divisor (scaling) each.
struct VecSegs {
  static constexpr int kMax = 4;
  double* x[kMax] = {nullptr, nullptr, nullptr, nullptr};
  int64_t n[kMax] = {0, 0, 0, 0};
  double* out[kMax] = {nullptr, nullptr, nullptr, nullptr};
  const double* den[kMax] = {nullptr, nullptr, nullptr, nullptr};
  int count = 0;
  VecSegs& norm(const double* v, int64_t len, double* o) {
    x[count] = const_cast<double*>(v); n[count] = len; out[count] = o; ++count;
    return *this;
  }
  VecSegs& scale(double* v, int64_t len, const double* d) {
    x[count] = v; n[count] = len; den[count] = d; ++count;
    return *this;
  }
};
// out_i = ||x_i||_2 for every segment, one launch (deterministic block-ordered sums)
void nrm2_multi(const RedWS& ws, const VecSegs& v, cudaStream_t s);
// x_i <- x_i / den_i for every segment (den_i <= 0 leaves x_i unchanged), one launch
void scale_multi(const VecSegs& v, cudaStream_t s);

// y <- a*x + b*y (host scalars)
void axpby(double a, const double* x, double b, double* y, int64_t n, cudaStream_t s);
// z <- x - y
void sub(const double* x, const double* y, double* z, int64_t n, cudaStream_t s);
// z <- x - y and out[0] = ||z||_2, one launch (z may alias x or y)
void sub_nrm2(const RedWS& ws, const double* x, const double* y, double* z, int64_t n, double* out,
              cudaStream_t s);
// x <- x * (num / den) with device scalars; den <= 0 leaves x unchanged (num may be null: 1)
void scale_dev(double* x, int64_t n, const double* num, const double* den, cudaStream_t s);
// y <- x * a (host scalar)
void scale_copy(const double* x, double a, double* y, int64_t n, cudaStream_t s);
void fill(double* x, double v, int64_t n, cudaStream_t s);
void copy(const double* x, double* y, int64_t n, cudaStream_t s);
// 2-D strided copy: dst[i*dld + j] = src[i*sld + j], i < rows, j < cols
void copy2d(const double* src, int64_t sld, double* dst, int64_t dld, int64_t rows, int64_t cols,
            cudaStream_t s);
// dst (rows x cols, row-major ld) = transpose of src (cols x rows, row-major sld)
void transpose(const double* src, int64_t sld, double* dst, int64_t dld, int64_t rows, int64_t cols,
               cudaStream_t s);
// X (rows x cols, column-major, ld): X[q + j*ld] *= S[q]  (S device)
void scale_rows_cm(double* X, int64_t ld, int64_t rows, int64_t cols, const double* S,
                   cudaStream_t s);
// precision casts
void cast(const double* x, float* y, int64_t n, cudaStream_t s);
void cast(const float* x, double* y, int64_t n, cudaStream_t s);

}  // namespace ttgb
