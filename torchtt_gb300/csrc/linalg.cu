// FP64 dense linear algebra: shifted CholeskyQR3 with a Householder fallback, one-sided Jacobi
// thin SVD, LU solve with partial pivoting.
//
// GB300 note: FP64 runs at ~1.9 FMA/clock/SM (measured), so every O(m n^2) step is expressed as a
// GEMM on the contraction engine (spread over all SMs); only O(n^3) steps on the small n x n
// factors run on few SMs: Cholesky + triangular inverse and the Jacobi of n < 16 in one thread
// block, the block Jacobi of 16 <= n <= 160 on an 8-CTA cluster, larger ones one grid-wide round
// per launch. Small QRs (the kickrank-wide blocks) run a shared-memory Householder in one block.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>

#include "contract.cuh"
#include "linalg.cuh"

namespace cg = cooperative_groups;

namespace ttgb {

namespace {

constexpr double kEps = 2.220446049250313e-16;

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ double block_sum_d(double v, double* sh) {
  v = warp_sum_d(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += sh[i];
  __syncthreads();
  return r;   // valid in all threads
}

__device__ double block_max_d(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r = fmax(r, sh[i]);
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------------------------------------
// Cholesky of the symmetric n x n matrix G (row-major, in place -> upper R with G = R^T R).
// shift_rows > 0 adds the sCholQR3 shift 11 (m n + n (n+1)) eps ||A||_F^2 with m = shift_rows
// (Fukaya, Kannan, Nakatsukasa, Yamamoto, Yanagisawa, SIAM J. Sci. Comput. 2020).
// check_identity: flag status=2 when max |G - I| > 0.1 (the third pass of CholeskyQR3 sees the
// Gram matrix of an already orthonormalised Q).
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(512) chol_kernel(double* G, int n, int64_t shift_rows,
                                                   int check_identity, int* status) {
  __shared__ double sh[32];
  __shared__ int bad;
  const int tid = threadIdx.x, nt = blockDim.x;
  if (tid == 0) bad = 0;
  __syncthreads();
  if (check_identity) {
    double mx = 0.0;
    for (int64_t t = tid; t < (int64_t)n * n; t += nt) {
      const int i = (int)(t / n), k = (int)(t % n);
      if (k < i) continue;   // the Gram matrix is formed (and read) in its upper triangle only
      const double v = G[t] - (i == k ? 1.0 : 0.0);
      mx = fmax(mx, isfinite(v) ? fabs(v) : 1e300);
    }
    mx = block_max_d(mx, sh);
    if (tid == 0 && !(mx <= 0.1)) *status = 2;
  }
  if (shift_rows > 0) {
    double tr = 0.0;
    for (int i = tid; i < n; i += nt) tr += G[(int64_t)i * n + i];
    tr = block_sum_d(tr, sh);
    const double sft = 11.0 * ((double)shift_rows * n + (double)n * (n + 1)) * kEps * tr;
    for (int i = tid; i < n; i += nt) G[(int64_t)i * n + i] += sft;
  }
  __syncthreads();
  __shared__ double piv_inv;   // pivot reciprocal, computed once per step (see chol_inv_smem)
  for (int j = 0; j < n; ++j) {
    if (tid == 0) {
      const double d = G[(int64_t)j * n + j];
      if (!(d > 0.0) || !isfinite(d)) { bad = 1; *status = 1; }
      else { const double rd = sqrt(d); G[(int64_t)j * n + j] = rd; piv_inv = 1.0 / rd; }
    }
    __syncthreads();
    if (bad) break;
    const double inv = piv_inv;
    for (int k = j + 1 + tid; k < n; k += nt) G[(int64_t)j * n + k] *= inv;
    __syncthreads();
    const int w = n - j - 1;
    for (int64_t t = tid; t < (int64_t)w * w; t += nt) {
      const int i = j + 1 + (int)(t / w), k = j + 1 + (int)(t % w);
      if (k < i) continue;
      G[(int64_t)i * n + k] = fma(-G[(int64_t)j * n + i], G[(int64_t)j * n + k], G[(int64_t)i * n + k]);
    }
    __syncthreads();
  }
  __syncthreads();
  for (int64_t t = tid; t < (int64_t)n * n; t += nt) {
    const int i = (int)(t / n), k = (int)(t % n);
    if (k < i) G[t] = 0.0;
  }
}

// Fused, shared-memory resident Cholesky + triangular inverse for n <= kCholSmemMax:
// G (row-major, global) -> R (upper, G = R^T R) written to Rout, Ri = R^{-1} written to Riout.
// Same shift / identity check semantics as chol_kernel. One block; both n x n factors live in
// shared memory, so every step is a shared-memory FP64 update plus one barrier.
constexpr int kCholSmemMax = 112;
constexpr double kNearIdentity = 1e-9;   // max |G - I| below which the first-order factor is used

// Gin is cleared after it is read (the next Gram product accumulates into it); Rout and Riout
// must not overlap it.
__global__ void __launch_bounds__(512) chol_inv_smem_kernel(double* __restrict__ Gin, int n,
                                                            int64_t shift_rows, int check_identity,
                                                            double* Rout, double* Riout, int* status) {
  extern __shared__ double sm[];
  const int ld = n + 1;   // padded rows
  double* G = sm;                 // becomes R (upper)
  double* X = sm + n * ld;        // becomes R^{-1} (upper)
  __shared__ double sh[32];
  __shared__ int bad;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int t = tid; t < n * n; t += nt) G[(t / n) * ld + (t % n)] = Gin[t];
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int t = tid; t < n * n; t += nt) Gin[t] = 0.0;   // ready for the next Gram product
  if (shift_rows == 0) {   // the second and third passes: G = I + E with E small
    double mx = 0.0;
    for (int t = tid; t < n * n; t += nt) {
      const int i = t / n, k = t % n;
      if (k < i) continue;   // the Gram matrix is formed (and read) in its upper triangle only
      const double v = G[i * ld + k] - (i == k ? 1.0 : 0.0);
      mx = fmax(mx, isfinite(v) ? fabs(v) : 1e300);
    }
    mx = block_max_d(mx, sh);   // the same value in every thread: the branches below are uniform
    if (check_identity && tid == 0 && !(mx <= 0.1)) *status = 2;
    if (mx <= kNearIdentity) {
      // First-order factor: R = I + U with U the strict upper triangle of E plus half its
      // diagonal (U + U^T = E), and R^{-1} = I - U. Both are exact to O(n max|E|^2) <= 1.2e-16
      // for max|E| <= 1e-9 and n <= 112, so the pass costs O(n^2) instead of the factorisation's
      // n^3 / 3 serial FP64 multiply-adds.
      for (int t = tid; t < n * n; t += nt) {
        const int i = t / n, k = t % n;
        const double e = (k >= i) ? G[i * ld + k] - (i == k ? 1.0 : 0.0) : 0.0;
        const double u = (k > i) ? e : (k == i ? 0.5 * e : 0.0);
        const double id = (i == k) ? 1.0 : 0.0;
        Rout[t] = id + u;
        Riout[t] = id - u;
      }
      return;
    }
  }
  if (shift_rows > 0) {
    double tr = 0.0;
    for (int i = tid; i < n; i += nt) tr += G[i * ld + i];
    tr = block_sum_d(tr, sh);
    const double sft = 11.0 * ((double)shift_rows * n + (double)n * (n + 1)) * kEps * tr;
    for (int i = tid; i < n; i += nt) G[i * ld + i] += sft;
  }
  __syncthreads();
  // right-looking Cholesky, upper triangle only. The pivot's square root and reciprocal are
  // computed once per step by one thread: FP64 sqrt and division expand to several DFMA, and 16
  // warps computing them redundantly would occupy the SM's FP64 pipe for thousands of cycles.
  __shared__ double piv_inv;
  for (int j = 0; j < n; ++j) {
    if (tid == 0) {
      const double d = G[j * ld + j];
      if (!(d > 0.0) || !isfinite(d)) { bad = 1; *status = 1; }
      else { const double rd = sqrt(d); G[j * ld + j] = rd; piv_inv = 1.0 / rd; }
    }
    __syncthreads();
    if (bad) break;
    const double inv = piv_inv;
    for (int k = j + 1 + tid; k < n; k += nt) G[j * ld + k] *= inv;
    __syncthreads();
    {   // trailing update of the upper triangle: one warp per row, lanes over columns
      const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
      for (int i = j + 1 + warp; i < n; i += nw) {
        const double gji = G[j * ld + i];
        double* gi = G + i * ld;
        const double* gj = G + j * ld;
        for (int k = i + lane; k < n; k += 32) gi[k] = fma(-gji, gj[k], gi[k]);
      }
    }
    __syncthreads();
  }
  if (bad) return;
  {
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    for (int i = warp; i < n; i += nw)
      for (int k = lane; k < n; k += 32) {
        if (k < i) G[i * ld + k] = 0.0;
        X[i * ld + k] = (k == i) ? 1.0 : 0.0;
      }
  }
  __syncthreads();
  // X = R^{-1} by column-oriented back substitution on the identity: for j = n-1..0 the row j of
  // X is final after scaling, then its multiples are removed from the rows above (one warp per row).
  {
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    for (int j = n - 1; j >= 0; --j) {
      if (tid == 0) piv_inv = 1.0 / G[j * ld + j];
      __syncthreads();
      const double inv = piv_inv;
      for (int k = j + tid; k < n; k += nt) X[j * ld + k] *= inv;
      __syncthreads();
      for (int i = warp; i < j; i += nw) {
        const double gij = G[i * ld + j];
        double* xi = X + i * ld;
        const double* xj = X + j * ld;
        for (int k = j + lane; k < n; k += 32) xi[k] = fma(-gij, xj[k], xi[k]);
      }
      __syncthreads();
    }
  }
  {
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    for (int i = warp; i < n; i += nw)
      for (int k = lane; k < n; k += 32) {
        Rout[i * n + k] = G[i * ld + k];
        Riout[i * n + k] = X[i * ld + k];
      }
  }
}

// Ri = R^{-1} for the upper-triangular row-major R (one thread per column of Ri).
__global__ void trinv_kernel(const double* __restrict__ R, double* Ri, int n) {
  for (int j = threadIdx.x + blockIdx.x * blockDim.x; j < n; j += blockDim.x * gridDim.x) {
    for (int i = n - 1; i >= 0; --i) {
      double v = (i == j) ? 1.0 : 0.0;
      if (i <= j) {
        for (int k = i + 1; k <= j; ++k) v = fma(-R[(int64_t)i * n + k], Ri[(int64_t)k * n + j], v);
        v /= R[(int64_t)i * n + i];
      }
      Ri[(int64_t)i * n + j] = (i <= j) ? v : 0.0;
    }
  }
}

// ---------------------------------------------------------------------------------------------
// Single-block Householder QR (LAPACK dgeqrf/dorgqr scheme): W (m x n col-major, ld m) is
// overwritten; outputs Q (m x k, ld m) and R (k x n, ld k), k = min(m, n).
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void householder_body(double* W, int m, int n, double* Q, double* R,
                                                 double* tau) {
  __shared__ double sh[32];
  __shared__ double refl[3];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  const int k = min(m, n);
  for (int j = 0; j < k; ++j) {
    double* col = W + (int64_t)j * m;
    double xs = 0.0;
    for (int i = j + 1 + tid; i < m; i += nt) xs = fma(col[i], col[i], xs);
    xs = block_sum_d(xs, sh);
    if (tid == 0) {   // reflector scalars once per column (FP64 sqrt/division are DFMA sequences)
      const double alpha = col[j];
      double tj = 0.0, beta = alpha, scale = 0.0;
      if (xs > 0.0) {
        beta = -copysign(sqrt(alpha * alpha + xs), alpha);
        tj = (beta - alpha) / beta;
        scale = 1.0 / (alpha - beta);
      }
      refl[0] = tj; refl[1] = beta; refl[2] = scale;
    }
    __syncthreads();
    const double tj = refl[0], beta = refl[1], scale = refl[2];
    for (int i = j + 1 + tid; i < m; i += nt) col[i] *= scale;
    __syncthreads();
    if (tid == 0) { col[j] = beta; tau[j] = tj; }
    __syncthreads();
    if (tj != 0.0) {
      for (int c = j + 1 + warp; c < n; c += nw) {
        double* cc = W + (int64_t)c * m;
        const double c0 = cc[j];   // read by every lane before lane 0 updates it
        double w = 0.0;
        for (int i = j + 1 + lane; i < m; i += 32) w = fma(col[i], cc[i], w);
        w = warp_sum_d(w) + c0;
        const double tw = tj * w;
        if (lane == 0) cc[j] -= tw;
        for (int i = j + 1 + lane; i < m; i += 32) cc[i] = fma(-tw, col[i], cc[i]);
      }
    }
    __syncthreads();
  }
  // R = upper part
  for (int64_t t = tid; t < (int64_t)k * n; t += nt) {
    const int i = (int)(t % k), c = (int)(t / k);
    R[t] = (i <= c) ? W[(int64_t)c * m + i] : 0.0;
  }
  // Q = H_0 ... H_{k-1} [I; 0]
  for (int64_t t = tid; t < (int64_t)m * k; t += nt) {
    const int i = (int)(t % m), c = (int)(t / m);
    Q[t] = (i == c) ? 1.0 : 0.0;
  }
  __syncthreads();
  for (int j = k - 1; j >= 0; --j) {
    const double tj = tau[j];
    if (tj == 0.0) continue;
    const double* col = W + (int64_t)j * m;
    for (int c = j + warp; c < k; c += nw) {
      double* qc = Q + (int64_t)c * m;
      const double q0 = qc[j];
      double w = 0.0;
      for (int i = j + 1 + lane; i < m; i += 32) w = fma(col[i], qc[i], w);
      w = warp_sum_d(w) + q0;
      const double tw = tj * w;
      if (lane == 0) qc[j] -= tw;
      for (int i = j + 1 + lane; i < m; i += 32) qc[i] = fma(-tw, col[i], qc[i]);
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(512) householder_kernel(double* W, int m, int n, double* Q,
                                                          double* R, double* tau) {
  householder_body(W, m, n, Q, R, tau);
}

// The same factorisation with W, Q and tau in shared memory (m * n + m * k + k doubles), read
// straight from A (ld lda): every step of the column sweep is a shared-memory access instead of an
// L2 round trip, which is what bounds the small QRs of the enrichment blocks (m <= 1024, n <= 16).
constexpr int kHouseholderSmemBytes = 200 * 1024;

__global__ void __launch_bounds__(512, 1) householder_smem_kernel(const double* __restrict__ A,
                                                               int64_t lda, int m, int n,
                                                               double* Qout, double* R) {
  extern __shared__ double hs[];
  const int k = min(m, n);
  double* W = hs;
  double* Q = W + (int64_t)m * n;
  double* tau = Q + (int64_t)m * k;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int64_t t = tid; t < (int64_t)m * n; t += nt) {
    const int64_t i = t % m, j = t / m;
    W[t] = A[j * lda + i];
  }
  __syncthreads();
  householder_body(W, m, n, Q, R, tau);
  __syncthreads();
  for (int64_t t = tid; t < (int64_t)m * k; t += nt) Qout[t] = Q[t];
}

// ---------------------------------------------------------------------------------------------
// Batched R-only Householder QR, one block per matrix: block b factors W + b * stride (rows x n,
// column-major, ld rows) in place and writes its R factor as the n x n column-major block
// Rout + b * n * n (upper triangle; rows >= min(rows, n) and the lower part zero). The levels of
// the TSQR reduction in qr_r are launches of this kernel.
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(512) householder_r_kernel(double* Wall, int64_t stride, int rows,
                                                            int n, double* Rout) {
  __shared__ double sh[32];
  __shared__ double refl[3];
  double* W = Wall + (int64_t)blockIdx.x * stride;
  double* R = Rout + (int64_t)blockIdx.x * n * n;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  const int k = min(rows, n);
  for (int j = 0; j < k; ++j) {
    double* col = W + (int64_t)j * rows;
    double xs = 0.0;
    for (int i = j + 1 + tid; i < rows; i += nt) xs = fma(col[i], col[i], xs);
    xs = block_sum_d(xs, sh);
    if (tid == 0) {   // reflector scalars once per column (FP64 sqrt/division are DFMA sequences)
      const double alpha = col[j];
      double tj = 0.0, beta = alpha, scale = 0.0;
      if (xs > 0.0) {
        beta = -copysign(sqrt(alpha * alpha + xs), alpha);
        tj = (beta - alpha) / beta;
        scale = 1.0 / (alpha - beta);
      }
      refl[0] = tj; refl[1] = beta; refl[2] = scale;
    }
    __syncthreads();
    const double tj = refl[0], beta = refl[1], scale = refl[2];
    for (int i = j + 1 + tid; i < rows; i += nt) col[i] *= scale;
    __syncthreads();
    if (tid == 0) col[j] = beta;
    __syncthreads();
    if (tj != 0.0) {
      for (int c = j + 1 + warp; c < n; c += nw) {
        double* cc = W + (int64_t)c * rows;
        const double c0 = cc[j];
        double w = 0.0;
        for (int i = j + 1 + lane; i < rows; i += 32) w = fma(col[i], cc[i], w);
        w = warp_sum_d(w) + c0;
        const double tw = tj * w;
        if (lane == 0) cc[j] -= tw;
        for (int i = j + 1 + lane; i < rows; i += 32) cc[i] = fma(-tw, col[i], cc[i]);
      }
    }
    __syncthreads();
  }
  for (int64_t t = tid; t < (int64_t)n * n; t += nt) {
    const int i = (int)(t % n), c = (int)(t / n);
    R[t] = (i <= c && i < k) ? W[(int64_t)c * rows + i] : 0.0;
  }
}

// Level-0 gather of TSQR: block b = rows [b*mb, b*mb + mb) of A (zero past m), column-major mb x n.
__global__ void tsqr_gather_kernel(const double* __restrict__ A, int64_t lda, int64_t m, int n,
                                   int mb, int nblk, double* W) {
  const int64_t per = (int64_t)mb * n, total = per * nblk;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / per, rem = t - b * per;
    const int64_t j = rem / mb, i = rem - j * mb;
    const int64_t row = b * mb + i;
    W[t] = (row < m) ? A[j * lda + row] : 0.0;
  }
}

// Next TSQR level: block b = [R_{2b}; R_{2b+1}] (2n x n column-major; zero when 2b+1 is missing).
__global__ void tsqr_stack_kernel(const double* __restrict__ R, int n, int nin, double* W) {
  const int nout = (nin + 1) / 2;
  const int64_t per = (int64_t)2 * n * n, total = per * nout;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / per, rem = t - b * per;
    const int64_t j = rem / (2 * n), i = rem - j * 2 * n;
    const int64_t src = 2 * b + (i >= n ? 1 : 0);
    const int64_t ii = i >= n ? i - n : i;
    W[t] = (src < nin) ? R[src * n * n + j * n + ii] : 0.0;
  }
}

// ---------------------------------------------------------------------------------------------
// One-sided (Hestenes) Jacobi SVD of the n x n column-major matrix W in one thread block, with
// the round-robin parallel ordering; rotation formulas of Demmel & Veselic (SIAM J. Matrix Anal.
// Appl. 13, 1992). On exit U (n x n) holds W_j / sigma_j, V the accumulated rotations, both with
// columns sorted by descending sigma, S the sorted singular values.
// ---------------------------------------------------------------------------------------------
// Rotation (c, s) of one-sided Jacobi for a column pair with squared norms a, b and inner product
// g (Demmel-Veselic formulas): false when the pair is orthogonal to `tol`. The tangent t of the
// angle comes from FP32 arithmetic (relative error ~1e-7: the pair is left orthogonal to ~1e-7 and
// a later sweep finishes it), and c = 1/sqrt(1 + t^2) is refined from the FP32 rsqrt to full FP64
// accuracy by two Newton steps, so (c, s) is orthogonal to rounding. On GB300 an FP64 sqrt or
// division is a sequence of DFMA on a pipe that issues one warp instruction per 16 cycles; the
// exact formula costs ~4 sqrt + 3 divisions per rotation, this one ~8 DFMA.
__device__ __forceinline__ bool jacobi_rotation(double a, double b, double g, double tol, double& c,
                                                double& s) {
  if (a == 0.0 || b == 0.0) return false;
  if (!(g * g > tol * tol * a * b)) return false;
  const double bma = b - a, g2 = 2.0 * g;
  const float fb = (float)bma, fg = (float)g2;
  float tf;
  if (fabsf(fb) >= fabsf(fg)) {   // r = 2g / (b - a), |r| <= 1: t = r / (1 + sqrt(1 + r^2))
    const float r = __fdividef(fg, fb);
    tf = __fdividef(r, 1.0f + sqrtf(fmaf(r, r, 1.0f)));
  } else {                        // zeta = (b - a) / 2g, |zeta| < 1
    const float z = __fdividef(fb, fg);
    tf = __fdividef(copysignf(1.0f, z), fabsf(z) + sqrtf(fmaf(z, z, 1.0f)));
  }
  double t;
  if (tf != 0.0f && isfinite(tf)) {
    t = (double)tf;
  } else {   // operands outside the FP32 range: the exact FP64 formula
    const double zeta = bma / g2;
    t = (fabs(zeta) > 1e150) ? 0.5 / zeta
                             : copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
  }
  const double x = fma(t, t, 1.0);
  double y = (double)rsqrtf((float)x);
  y = y * fma(-0.5 * x, y * y, 1.5);
  y = y * fma(-0.5 * x, y * y, 1.5);
  c = y;
  s = y * t;
  return true;
}

__device__ __forceinline__ double warp_sum_t(double v) { return warp_sum_d(v); }

__device__ __forceinline__ int rr_index(int p, int r, int nn) {
  return p == 0 ? 0 : ((p - 1 + r) % (nn - 1)) + 1;
}

__global__ void __launch_bounds__(512) jacobi_svd_kernel(double* Wg, double* Vg, int n, double* U,
                                                         double* S, int use_smem, int max_sweeps,
                                                         int* status, const double* Vinit) {
  extern __shared__ double smem[];
  __shared__ int nrot;
  double* W = use_smem ? smem : Wg;
  double* V = use_smem ? smem + (int64_t)n * n : Vg;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  if (use_smem) {
    for (int64_t t = tid; t < (int64_t)n * n; t += nt) W[t] = Wg[t];
  }
  for (int64_t t = tid; t < (int64_t)n * n; t += nt)
    V[t] = Vinit ? Vinit[t] : (((t % n) == (t / n)) ? 1.0 : 0.0);
  __syncthreads();
  const int nn = n + (n & 1);
  const double tol = fmax((double)n, 1.0) * kEps;
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    if (tid == 0) nrot = 0;
    __syncthreads();
    for (int r = 0; r < nn - 1; ++r) {
      for (int pi = warp; pi < nn / 2; pi += nw) {
        int p = rr_index(pi, r, nn), q = rr_index(nn - 1 - pi, r, nn);
        if (p > q) { const int t = p; p = q; q = t; }
        if (q >= n) continue;
        double* wp = W + (int64_t)p * n;
        double* wq = W + (int64_t)q * n;
        double a = 0.0, b = 0.0, g = 0.0;
        for (int i = lane; i < n; i += 32) {
          const double x = wp[i], y = wq[i];
          a = fma(x, x, a); b = fma(y, y, b); g = fma(x, y, g);
        }
        a = warp_sum_d(a); b = warp_sum_d(b); g = warp_sum_d(g);
        double c, s;
        if (!jacobi_rotation(a, b, g, tol, c, s)) continue;
        for (int i = lane; i < n; i += 32) {
          const double x = wp[i], y = wq[i];
          wp[i] = c * x - s * y;
          wq[i] = s * x + c * y;
        }
        double* vp = V + (int64_t)p * n;
        double* vq = V + (int64_t)q * n;
        for (int i = lane; i < n; i += 32) {
          const double x = vp[i], y = vq[i];
          vp[i] = c * x - s * y;
          vq[i] = s * x + c * y;
        }
        if (lane == 0) atomicAdd(&nrot, 1);
      }
      __syncthreads();
    }
    __syncthreads();
    if (nrot == 0) break;
    __syncthreads();
  }
  if (tid == 0 && sweep >= max_sweeps) *status = 3;
  // singular values, ranks by descending value (ties by index)
  double* sig = S;  // temporary: write unsorted to S via registers below
  for (int j = warp; j < n; j += nw) {
    const double* wj = W + (int64_t)j * n;
    double a = 0.0;
    for (int i = lane; i < n; i += 32) a = fma(wj[i], wj[i], a);
    a = warp_sum_d(a);
    if (lane == 0) U[(int64_t)j] = sqrt(a);   // stash sigma_j in U's first column temporarily
  }
  __syncthreads();
  // rank computation, then write sorted S (U column 0 is rewritten afterwards)
  __shared__ int rank_sh[1024];
  for (int j = tid; j < n; j += nt) {
    const double sj = U[j];
    int rk = 0;
    for (int i = 0; i < n; ++i) {
      const double si = U[i];
      rk += (si > sj) || (si == sj && i < j);
    }
    if (j < 1024) rank_sh[j] = rk;
  }
  __syncthreads();
  for (int j = tid; j < n; j += nt) sig[rank_sh[j]] = U[j];
  __syncthreads();
  // U[:, rank_j] = W_j / sigma_j ; V columns permuted into Wg (scratch) then copied back
  for (int j = warp; j < n; j += nw) {
    const int rk = rank_sh[j];
    const double sj = sig[rk];
    const double inv = sj > 0.0 ? 1.0 / sj : 0.0;
    const double* wj = W + (int64_t)j * n;
    for (int i = lane; i < n; i += 32) Vg[(int64_t)n * n + (int64_t)rk * n + i] = wj[i] * inv;
  }
  __syncthreads();
  for (int64_t t = tid; t < (int64_t)n * n; t += nt) U[t] = Vg[(int64_t)n * n + t];
  __syncthreads();
  for (int j = warp; j < n; j += nw) {
    const int rk = rank_sh[j];
    const double* vj = V + (int64_t)j * n;
    for (int i = lane; i < n; i += 32) Vg[(int64_t)n * n + (int64_t)rk * n + i] = vj[i];
  }
  __syncthreads();
  for (int64_t t = tid; t < (int64_t)n * n; t += nt) Vg[t] = Vg[(int64_t)n * n + t];
}

// ---------------------------------------------------------------------------------------------
// Block one-sided Jacobi on a thread-block cluster of kJacobiCluster CTAs for 16 <= n <=
// kJacobiBlockMaxN: the columns (padded to P = 2C blocks of nb) are treated as P blocks paired by
// the round-robin tournament; in round r the CTA i holds the blocks rr(i, r) and rr(P-1-i, r) in its
// own shared memory and rotates all their cross pairs there (nb sub-rounds of nb disjoint pairs,
// block barrier only; the pairs inside a block are rotated in the first round of each sweep), then
// pulls the two blocks of its next pair from their holders over DSMEM into its second buffer. Every
// pair of columns is visited once per sweep, as in the scalar cyclic order, with one cluster
// barrier per round (P - 1 per sweep), and every dot product reads local memory. The sweep's
// rotation count is summed in CTA 0 after a barrier and read by every CTA, so all CTAs leave the
// loop together. The value type T is the arithmetic of the sweeps; Vin (optional) gives starting
// rotations (identity when null), Vout the accumulated ones.
// ---------------------------------------------------------------------------------------------
constexpr int kJacobiCluster = 8;
constexpr int kJacobiBlockMaxN = 160;

// One rotation of a column pair with tracked squared column norms (*na, *nb): only the inner product is
// reduced; the norms follow the rotation exactly (a' = c^2 a - 2cs g + s^2 b, b' = s^2 a + 2cs g +
// c^2 b) and are recomputed from the columns once per sweep, which bounds their drift.
template <typename T>
__device__ __forceinline__ int jacobi_rotate_tracked(T* wp, T* wq, T* vp, T* vq, T* na, T* nb, int n,
                                                     T tol, int lane) {
  T g = T(0);
  for (int i = lane; i < n; i += 32) g = fma(wp[i], wq[i], g);
  g = warp_sum_t(g);
  const T a = *na, b = *nb;
  T c, s;
  if (!jacobi_rotation(a, b, g, tol, c, s)) return 0;
  for (int i = lane; i < n; i += 32) {
    const T x = wp[i], y = wq[i];
    wp[i] = c * x - s * y;
    wq[i] = s * x + c * y;
    const T u = vp[i], v = vq[i];
    vp[i] = c * u - s * v;
    vq[i] = s * u + c * v;
  }
  if (lane == 0) {
    const T cc = c * c, ss = s * s, cs2 = T(2) * c * s * g;
    const T a2 = cc * a - cs2 + ss * b, b2 = ss * a + cs2 + cc * b;
    *na = a2 > T(0) ? a2 : T(0);
    *nb = b2 > T(0) ? b2 : T(0);
  }
  return 1;
}

template <typename T>
__global__ void __cluster_dims__(kJacobiCluster, 1, 1) __launch_bounds__(256)
    jacobi_block_kernel(const T* __restrict__ Win, int n, T* Wout, T* Vout, int max_sweeps,
                        int* status, const T* __restrict__ Vin) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T* sm = reinterpret_cast<T*>(sm_raw);
  cg::cluster_group cluster = cg::this_cluster();
  constexpr int C = kJacobiCluster, P = 2 * kJacobiCluster;
  const int rank = (int)cluster.block_rank();
  const int nb = (n + P - 1) / P;
  const int64_t blk = (int64_t)nb * n;   // elements of one block of W (or of V)
  const int64_t unit = 2 * blk + nb + (nb & 1);   // W block, V block, squared column norms
  // buffer x (0/1), slot s (0/1): W block, V block, norms
  auto Wb = [&](T* base, int x, int sl) { return base + (int64_t)(x * 2 + sl) * unit; };
  auto Vb = [&](T* base, int x, int sl) { return base + (int64_t)(x * 2 + sl) * unit + blk; };
  auto Nb = [&](T* base, int x, int sl) { return base + (int64_t)(x * 2 + sl) * unit + 2 * blk; };
  __shared__ int counts[kJacobiCluster];
  __shared__ int local_cnt;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  const T tol = T(n > 1 ? n : 1) * (sizeof(T) == 8 ? T(kEps) : T(1.1920929e-7f));
  // round 0 of sweep 0: slot 0 holds block rank, slot 1 block P-1-rank
  for (int sl = 0; sl < 2; ++sl) {
    const int b = sl == 0 ? rank : P - 1 - rank;
    T* W = Wb(sm, 0, sl);
    T* V = Vb(sm, 0, sl);
    for (int64_t t = tid; t < blk; t += nt) {
      const int j = (int)(t / n), i = (int)(t - (int64_t)j * n);
      const int c = b * nb + j;
      W[t] = (c < n) ? Win[(int64_t)c * n + i] : T(0);
      V[t] = (c < n) ? (Vin ? Vin[(int64_t)c * n + i] : (i == c ? T(1) : T(0))) : T(0);
    }
  }
  int* counts0 = cluster.map_shared_rank(counts, 0);
  int x = 0, r = 0, sweep = 0, mine = 0;
  bool converged = false;
  if (tid == 0) local_cnt = 0;
  __syncthreads();
  while (true) {
    const int bA = rr_index(rank, r, P), bB = rr_index(P - 1 - rank, r, P);
    T* WA = Wb(sm, x, 0); T* VA = Vb(sm, x, 0); T* NA = Nb(sm, x, 0);
    T* WB = Wb(sm, x, 1); T* VB = Vb(sm, x, 1); T* NB = Nb(sm, x, 1);
    if (r == 0) {   // fresh column norms, then the pairs inside each block, once per sweep
      for (int c = warp; c < 2 * nb; c += nw) {
        const T* w = (c < nb ? WA : WB) + (int64_t)(c % nb) * n;
        T a = T(0);
        for (int i = lane; i < n; i += 32) a = fma(w[i], w[i], a);
        a = warp_sum_t(a);
        if (lane == 0) (c < nb ? NA : NB)[c % nb] = a;
      }
      __syncthreads();
      const int m2 = nb + (nb & 1);
      for (int t = 0; t < m2 - 1; ++t) {
        for (int task = warp; task < m2; task += nw) {   // m2/2 pairs per slot, 2 slots
          const int sl = task / (m2 / 2), pi = task % (m2 / 2);
          int p = rr_index(pi, t, m2), q = rr_index(m2 - 1 - pi, t, m2);
          if (p > q) { const int u = p; p = q; q = u; }
          if (q >= nb) continue;
          T* W = sl ? WB : WA;
          T* V = sl ? VB : VA;
          T* Nm = sl ? NB : NA;
          mine += jacobi_rotate_tracked(W + (int64_t)p * n, W + (int64_t)q * n, V + (int64_t)p * n,
                                        V + (int64_t)q * n, Nm + p, Nm + q, n, tol, lane);
        }
        __syncthreads();
      }
    }
    for (int t = 0; t < nb; ++t) {   // cross pairs (j, j + t mod nb)
      for (int j = warp; j < nb; j += nw) {
        const int k = (j + t) % nb;
        const int ga = bA * nb + j, gb = bB * nb + k;
        T *wp = WA + (int64_t)j * n, *wq = WB + (int64_t)k * n;
        T *vp = VA + (int64_t)j * n, *vq = VB + (int64_t)k * n;
        T *np = NA + j, *nq = NB + k;
        if (ga > gb) {
          T* u = wp; wp = wq; wq = u; u = vp; vp = vq; vq = u; u = np; np = nq; nq = u;
        }
        mine += jacobi_rotate_tracked(wp, wq, vp, vq, np, nq, n, tol, lane);
      }
      __syncthreads();
    }
    const bool sweep_end = (r == P - 2);
    if (sweep_end) {
      if (lane == 0 && mine) atomicAdd(&local_cnt, mine);
      mine = 0;
      __syncthreads();
      if (tid == 0) { counts0[rank] = local_cnt; local_cnt = 0; }
    }
    cluster.sync();   // every CTA finished round r (and published its count at a sweep end)
    if (sweep_end) {
      int total = 0;
      for (int c = 0; c < C; ++c) total += counts0[c];
      ++sweep;
      if (total == 0) { converged = true; break; }
      if (sweep >= max_sweeps) break;
    }
    // pull the blocks of round r+1 into buffer 1-x from their holders' buffer x
    const int rn = (r + 1) % (P - 1);
    for (int sl = 0; sl < 2; ++sl) {
      const int b = rr_index(sl == 0 ? rank : P - 1 - rank, rn, P);
      int owner = 0, oslot = 0;
      for (int c = 0; c < C; ++c) {
        if (rr_index(c, r, P) == b) { owner = c; oslot = 0; }
        if (rr_index(P - 1 - c, r, P) == b) { owner = c; oslot = 1; }
      }
      const T* srcW = cluster.map_shared_rank(Wb(sm, x, oslot), owner);
      const T* srcV = cluster.map_shared_rank(Vb(sm, x, oslot), owner);
      const T* srcN = cluster.map_shared_rank(Nb(sm, x, oslot), owner);
      T* dW = Wb(sm, 1 - x, sl);
      T* dV = Vb(sm, 1 - x, sl);
      T* dN = Nb(sm, 1 - x, sl);
      for (int64_t t = tid; t < blk; t += nt) { dW[t] = srcW[t]; dV[t] = srcV[t]; }
      for (int t = tid; t < nb; t += nt) dN[t] = srcN[t];
    }
    __syncthreads();
    x = 1 - x;
    r = rn;
  }
  if (rank == 0 && tid == 0 && !converged && status) *status = 3;
  // buffer x holds the blocks of round r
  for (int sl = 0; sl < 2; ++sl) {
    const int b = rr_index(sl == 0 ? rank : P - 1 - rank, r, P);
    const T* W = Wb(sm, x, sl);
    const T* V = Vb(sm, x, sl);
    for (int64_t t = tid; t < blk; t += nt) {
      const int j = (int)(t / n), i = (int)(t - (int64_t)j * n);
      const int c = b * nb + j;
      if (c < n) {
        Wout[(int64_t)c * n + i] = W[t];
        Vout[(int64_t)c * n + i] = V[t];
      }
    }
  }
  cluster.sync();   // no CTA leaves while another may still read its shared memory
}

// Grid-wide block Jacobi for larger n (W, V column-major n x n in global memory, L2-resident):
// one launch per round of the P-block tournament; CTA i rotates the cross pairs of the blocks
// rr(i, r) and rr(P-1-i, r) (and, in round 0, the pairs inside both), counting its rotations.
__global__ void __launch_bounds__(256) jacobi_grid_round_kernel(double* W, double* V, int n, int nb,
                                                                int P, int r, double tol,
                                                                unsigned* count) {
  const int i = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int bA = rr_index(i, r, P), bB = rr_index(P - 1 - i, r, P);
  int mine = 0;
  auto rotate = [&](int p, int q) {
    if (p > q) { const int t = p; p = q; q = t; }
    if (q >= n) return;
    double* wp = W + (int64_t)p * n;
    double* wq = W + (int64_t)q * n;
    double a = 0.0, b = 0.0, g = 0.0;
    for (int k = lane; k < n; k += 32) {
      const double x = wp[k], y = wq[k];
      a = fma(x, x, a); b = fma(y, y, b); g = fma(x, y, g);
    }
    a = warp_sum_d(a); b = warp_sum_d(b); g = warp_sum_d(g);
    double c, sn;
    if (!jacobi_rotation(a, b, g, tol, c, sn)) return;
    double* vp = V + (int64_t)p * n;
    double* vq = V + (int64_t)q * n;
    for (int k = lane; k < n; k += 32) {
      const double x = wp[k], y = wq[k];
      wp[k] = c * x - sn * y;
      wq[k] = sn * x + c * y;
      const double u = vp[k], v = vq[k];
      vp[k] = c * u - sn * v;
      vq[k] = sn * u + c * v;
    }
    ++mine;
  };
  if (r == 0) {   // pairs inside each of the two blocks
    const int m2 = nb + (nb & 1);
    for (int t = 0; t < m2 - 1; ++t) {
      for (int task = warp; task < m2; task += nw) {
        const int sl = task / (m2 / 2), pi = task % (m2 / 2);
        const int p = rr_index(pi, t, m2), q = rr_index(m2 - 1 - pi, t, m2);
        if (p >= nb || q >= nb) continue;
        const int base = (sl ? bB : bA) * nb;
        rotate(base + p, base + q);
      }
      __syncthreads();
    }
  }
  for (int t = 0; t < nb; ++t) {
    for (int j = warp; j < nb; j += nw) rotate(bA * nb + j, bB * nb + (j + t) % nb);
    __syncthreads();
  }
  if (lane == 0 && mine) atomicAdd(count, (unsigned)mine);
}

__global__ void identity_kernel(double* V, int n) {
  const int64_t total = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x)
    V[t] = (t % n == t / n) ? 1.0 : 0.0;
}

// From the rotated W (column-major n x n) and the rotations V: sigma_j = ||W_j||, descending order;
// Un[:, rank_j] = W_j / sigma_j, Vs[:, rank_j] = V_j, S[rank_j] = sigma_j. One block.
__global__ void __launch_bounds__(1024) svd_sort_kernel(const double* __restrict__ W,
                                                        const double* __restrict__ V, int n,
                                                        double* Un, double* S, double* Vs,
                                                        double* sig) {
  __shared__ int rank_sh[1024];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  for (int j = warp; j < n; j += nw) {
    double a = 0.0;
    for (int i = lane; i < n; i += 32) a = fma(W[(int64_t)j * n + i], W[(int64_t)j * n + i], a);
    a = warp_sum_d(a);
    if (lane == 0) sig[j] = sqrt(a);
  }
  __syncthreads();
  for (int j = tid; j < n; j += nt) {
    const double sj = sig[j];
    int rk = 0;
    for (int i = 0; i < n; ++i) {
      const double si = sig[i];
      rk += (si > sj) || (si == sj && i < j);
    }
    rank_sh[j] = rk;
  }
  __syncthreads();
  for (int j = tid; j < n; j += nt) S[rank_sh[j]] = sig[j];
  for (int j = warp; j < n; j += nw) {
    const int rk = rank_sh[j];
    const double inv = sig[j] > 0.0 ? 1.0 / sig[j] : 0.0;
    for (int i = lane; i < n; i += 32) {
      Un[(int64_t)rk * n + i] = W[(int64_t)j * n + i] * inv;
      Vs[(int64_t)rk * n + i] = V[(int64_t)j * n + i];
    }
  }
}

// ---------------------------------------------------------------------------------------------
// LU with partial pivoting on an n x n row-major copy, solving for one right-hand side.
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) lu_solve_kernel(double* LU, double* x, int n, int* status) {
  __shared__ double shv[32];
  __shared__ double piv_inv;
  __shared__ int shi[32];
  __shared__ int piv;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  for (int j = 0; j < n; ++j) {
    // pivot search
    double best = -1.0;
    int bi = j;
    for (int i = j + tid; i < n; i += nt) {
      const double v = fabs(LU[(int64_t)i * n + j]);
      if (v > best) { best = v; bi = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if (lane == 0) { shv[warp] = best; shi[warp] = bi; }
    __syncthreads();
    if (tid == 0) {
      double b = -1.0; int ib = j;
      for (int w = 0; w < (nt >> 5); ++w)
        if (shv[w] > b || (shv[w] == b && shi[w] < ib)) { b = shv[w]; ib = shi[w]; }
      piv = ib;
      if (!(b > 0.0)) *status = 1;
    }
    __syncthreads();
    const int p = piv;
    if (p != j) {
      for (int c = tid; c < n; c += nt) {
        const double t = LU[(int64_t)j * n + c];
        LU[(int64_t)j * n + c] = LU[(int64_t)p * n + c];
        LU[(int64_t)p * n + c] = t;
      }
      if (tid == 0) { const double t = x[j]; x[j] = x[p]; x[p] = t; }
    }
    __syncthreads();
    if (tid == 0) piv_inv = 1.0 / LU[(int64_t)j * n + j];   // one FP64 division per step
    __syncthreads();
    const double inv = piv_inv;
    const int w = n - j - 1;
    // multipliers
    for (int i = j + 1 + tid; i < n; i += nt) LU[(int64_t)i * n + j] *= inv;
    __syncthreads();
    for (int i = j + 1 + tid; i < n; i += nt) x[i] = fma(-LU[(int64_t)i * n + j], x[j], x[i]);
    for (int64_t t = tid; t < (int64_t)w * w; t += nt) {
      const int i = j + 1 + (int)(t / w), c = j + 1 + (int)(t % w);
      LU[(int64_t)i * n + c] = fma(-LU[(int64_t)i * n + j], LU[(int64_t)j * n + c], LU[(int64_t)i * n + c]);
    }
    __syncthreads();
  }
  // back substitution
  __shared__ double shs[32];
  for (int i = n - 1; i >= 0; --i) {
    double s = 0.0;
    for (int c = i + 1 + tid; c < n; c += nt) s = fma(LU[(int64_t)i * n + c], x[c], s);
    s = warp_sum_d(s);
    if (lane == 0) shs[warp] = s;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w2 = 0; w2 < (nt >> 5); ++w2) t += shs[w2];
      x[i] = (x[i] - t) / LU[(int64_t)i * n + i];
    }
    __syncthreads();
  }
}

__global__ void gemv_rm_kernel(const double* __restrict__ B, int64_t n, const double* __restrict__ x,
                               double* y) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (row >= n) return;
  double s = 0.0;
  for (int64_t c = lane; c < n; c += 32) s = fma(B[row * n + c], x[c], s);
  s = warp_sum_d(s);
  if (lane == 0) y[row] = s;
}

__global__ void copy_cm_kernel(const double* __restrict__ A, int64_t lda, double* W, int64_t m,
                               int64_t n) {
  const int64_t total = m * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % m, j = t / m;
    W[t] = A[j * lda + i];
  }
}

void read_status(LinalgWS& ws, cudaStream_t s, int* out) {
  TTGB_CUDA(cudaMemcpyAsync(ws.h_status, ws.status, sizeof(int), cudaMemcpyDeviceToHost, s));
  TTGB_CUDA(cudaStreamSynchronize(s));
  *out = *ws.h_status;
}

void householder(const double* A, int64_t lda, int64_t m, int64_t n, double* Q, double* R,
                 LinalgWS& ws, cudaStream_t s) {
  const int64_t k = m < n ? m : n;
  const size_t smem = (size_t)(m * n + m * k + k) * sizeof(double);
  if (smem <= (size_t)kHouseholderSmemBytes) {
    smem_optin((const void*)householder_smem_kernel, kHouseholderSmemBytes);
    householder_smem_kernel<<<1, 512, smem, s>>>(A, lda, (int)m, (int)n, Q, R);
    TTGB_CHECK_LAUNCH();
    return;
  }
  ws.d.ensure(m * n + k + 16, s);
  double* W = ws.d.p;
  double* tau = W + m * n;
  unsigned g = cdiv(m * n, 256);
  if (g > 4096) g = 4096;
  if (g == 0) g = 1;
  copy_cm_kernel<<<g, 256, 0, s>>>(A, lda, W, m, n);
  TTGB_CHECK_LAUNCH();
  householder_kernel<<<1, 512, 0, s>>>(W, (int)m, (int)n, Q, R, tau);
  TTGB_CHECK_LAUNCH();
}

}  // namespace

void qr_r(const double* A, int64_t lda, int64_t m, int64_t n, double* R, LinalgWS& ws,
          cudaStream_t s) {
  if (m <= 0 || n <= 0) return;
  TTGB_REQUIRE(n <= 4096, "qr_r: too many columns");
  const int mb = (int)std::max<int64_t>(2 * n, 256);
  const int64_t nblk = (m + mb - 1) / mb;
  TTGB_REQUIRE(nblk < 65536, "qr_r: too many row blocks");
  const int64_t per0 = (int64_t)mb * n;
  ws.d.ensure((size_t)(per0 * nblk + 2 * n * n * ((nblk + 1) / 2) + 16), s);
  ws.e.ensure((size_t)(n * n * nblk + 16), s);
  double* W = ws.d.p;
  double* Rb = ws.e.p;
  unsigned g = cdiv(per0 * nblk, 256);
  if (g > 8192) g = 8192;
  tsqr_gather_kernel<<<g, 256, 0, s>>>(A, lda, m, (int)n, mb, (int)nblk, W);
  TTGB_CHECK_LAUNCH();
  householder_r_kernel<<<(unsigned)nblk, 512, 0, s>>>(W, per0, mb, (int)n, Rb);
  TTGB_CHECK_LAUNCH();
  int64_t cur = nblk;
  while (cur > 1) {
    const int64_t nxt = (cur + 1) / 2;
    const int64_t per = 2 * n * n;
    unsigned g2 = cdiv(per * nxt, 256);
    if (g2 > 8192) g2 = 8192;
    tsqr_stack_kernel<<<g2, 256, 0, s>>>(Rb, (int)n, (int)cur, W);
    TTGB_CHECK_LAUNCH();
    householder_r_kernel<<<(unsigned)nxt, 512, 0, s>>>(W, per, (int)(2 * n), (int)n, Rb);
    TTGB_CHECK_LAUNCH();
    cur = nxt;
  }
  copy(Rb, R, n * n, s);
}

void gemm_cm(const double* A, int64_t lda, const double* B, int64_t ldb, double* C, int64_t ldc,
             int64_t m, int64_t n, int64_t k, double alpha, double beta, cudaStream_t s,
             bool transA, bool transB, int tri, bool c_zero) {
  ContractDesc c;
  c.M = (int)m; c.N = (int)n; c.K = (int)k;
  c.A = A;
  if (!transA) { c.am = Ax::one(1); c.ak = Ax::one(lda); }
  else { c.am = Ax::one(lda); c.ak = Ax::one(1); }
  c.B = B;
  if (!transB) { c.bk = Ax::one(1); c.bn = Ax::one(ldb); }
  else { c.bk = Ax::one(ldb); c.bn = Ax::one(1); }
  c.C = C; c.cm = Ax::one(1); c.cn = Ax::one(ldc);
  c.alpha = alpha; c.beta = beta;
  c.tri = tri;
  c.c_zero = c_zero;
  contract(c, s);
}

QRResult qr(const double* A, int64_t lda, int64_t m, int64_t n, double* Q, double* R,
            LinalgWS& ws, const RedWS& red, cudaStream_t s) {
  (void)red;
  QRResult res;
  res.k = m < n ? m : n;
  if (m <= 0 || n <= 0) return res;
  // small or wide: single-block Householder (robust, cheap at these sizes). A tall matrix with
  // few columns (m >= 1024, e.g. the kickrank-wide z blocks of 5120 rows) is not small: one
  // block's serial column sweep over m rows costs more than the GEMM passes of CholeskyQR3.
  const bool small = (double)m * n * n < 4.0e5 && m < 1024;
  if (m < n || small || n > 1024) {
    householder(A, lda, m, n, Q, R, ws, s);
    return res;
  }
  // shifted CholeskyQR3
  ws.a.ensure(5 * n * n + 16, s);
  double* Rp[3] = {ws.a.p, ws.a.p + n * n, ws.a.p + 2 * n * n};   // R of each pass (row-major)
  double* Ri = ws.a.p + 3 * n * n;   // inverse of the current factor
  double* T1 = ws.a.p + 4 * n * n;   // R_1 R_0
  if (ws.gram.p == nullptr || ws.gram.n < (size_t)(n * n)) {   // (re)allocated: clear it once
    ws.gram.ensure((size_t)(n * n), s);
    TTGB_CUDA(cudaMemsetAsync(ws.gram.p, 0, ws.gram.n * sizeof(double), s));
    ws.gram_zero = (int64_t)ws.gram.n;
  }
  double* G = ws.gram.p;             // n x n Gram matrix (row-major upper triangle)
  ws.b.ensure(m * n + 16, s);
  double* Qt = ws.b.p;
  TTGB_CUDA(cudaMemsetAsync(ws.status, 0, sizeof(int), s));
  const double* Ain = A;
  int64_t ldin = lda;
  double* outs[3] = {Q, Qt, Q};
  const bool smem_chol = n <= kCholSmemMax;
  for (int pass = 0; pass < 3; ++pass) {
    // Gram matrix: only its lower (column-major) = upper (row-major) triangle is formed and read;
    // with the shared-memory Cholesky the buffer is already zero (cleared by the previous one)
    gemm_cm(Ain, ldin, Ain, ldin, G, n, n, n, m, 1.0, 0.0, s, true, false, kTriLowerC,
            smem_chol && ws.gram_zero >= n * n);
    if (smem_chol) {
      const size_t smem = (size_t)2 * n * (n + 1) * sizeof(double);
      smem_optin((const void*)chol_inv_smem_kernel,
                 (int)(2 * kCholSmemMax * (kCholSmemMax + 1) * sizeof(double)));
      chol_inv_smem_kernel<<<1, 512, smem, s>>>(G, (int)n, pass == 0 ? m : 0, pass == 2 ? 1 : 0,
                                                Rp[pass], Ri, ws.status);
      TTGB_CHECK_LAUNCH();
      if (ws.gram_zero < n * n) ws.gram_zero = n * n;   // the kernel cleared [0, n^2)
    } else {
      chol_kernel<<<1, 512, 0, s>>>(G, (int)n, pass == 0 ? m : 0, pass == 2 ? 1 : 0, ws.status);
      TTGB_CHECK_LAUNCH();
      trinv_kernel<<<cdiv(n, 128), 128, 0, s>>>(G, Ri, (int)n);
      TTGB_CHECK_LAUNCH();
      copy(G, Rp[pass], n * n, s);
      ws.gram_zero = 0;   // G now holds R
    }
    // Q_next = Ain * R^{-1}   (Ri row-major == (Ri)^T column-major; R^{-1} upper triangular)
    gemm_cm(Ain, ldin, Ri, n, outs[pass], m, m, n, n, 1.0, 0.0, s, false, true, kTriUpperB);
    Ain = outs[pass];
    ldin = m;
  }
  int st = 0;
  read_status(ws, s, &st);
  if (st != 0) {
    householder(A, lda, m, n, Q, R, ws, s);
    return res;
  }
  // R = R_2 R_1 R_0 (row-major factors; a row-major X is the column-major X^T):
  // T1 (row-major) = R_1 R_0, and R (column-major, ld n) = R_2 T1 written directly
  gemm_cm(Rp[0], n, Rp[1], n, T1, n, n, n, n, 1.0, 0.0, s, false, false);
  gemm_cm(Rp[2], n, T1, n, R, n, n, n, n, 1.0, 0.0, s, true, true);
  return res;
}

void svd(const double* A, int64_t lda, int64_t m, int64_t n, double* U, double* S, double* Vh,
         LinalgWS& ws, const RedWS& red, cudaStream_t s) {
  if (m <= 0 || n <= 0) return;
  if (m < n) {
    // A^T = U' S V'^T  ->  A = V' S U'^T
    DBuf At((size_t)(n * m), s);
    transpose(A, lda, At.p, n, m, n, s);      // At (n x m col-major): At[j + i*n] = A[i + j*lda]
    // transpose() writes dst[r*dld + c] = src[c*sld + r] with rows=m? use explicit kernel via gemm
    DBuf Ut((size_t)(n * m), s), Vt((size_t)(m * m), s);
    svd(At.p, n, n, m, Ut.p, S, Vt.p, ws, red, s);
    // U = V' = Vt^T (m x m); Vh = U'^T (m x n)
    transpose(Vt.p, m, U, m, m, m, s);
    transpose(Ut.p, n, Vh, m, n, m, s);
    return;
  }
  // m >= n: A = Q R; one-sided Jacobi on R^T (QR-preconditioned Jacobi, Drmac & Veselic, SIAM J.
  // Matrix Anal. Appl. 29, 2008): R^T = U' S V'^T converges in far fewer sweeps than Jacobi on R.
  // Then R = V' S U'^T and A = (Q V') S U'^T.
  DBuf Qb((size_t)(m * n), s), Rb((size_t)(n * n), s);
  qr(A, lda, m, n, Qb.p, Rb.p, ws, red, s);
  TTGB_REQUIRE(n <= 1024, "SVD: too many columns");
  ws.c.ensure(3 * n * n + 16, s);
  double* W = ws.c.p;        // n x n: R^T, rotated in place
  double* Vw = W + n * n;    // 2 n x n: accumulated rotations V' (sorted) and scratch
  transpose(Rb.p, n, W, n, n, n, s);
  DBuf Up((size_t)(n * n), s);   // U' (normalised columns of the rotated R^T, sorted)
  if (n <= kJacobiBlockMaxN && n >= 2 * kJacobiCluster) {
    const int nb = (int)((n + 2 * kJacobiCluster - 1) / (2 * kJacobiCluster));
    const int64_t unit = 2 * nb * n + nb + (nb & 1);
    const size_t smem = (size_t)4 * unit * sizeof(double);
    smem_optin((const void*)jacobi_block_kernel<double>, (int)smem);
    jacobi_block_kernel<double><<<kJacobiCluster, 256, smem, s>>>(W, (int)n, W, Vw, 60, ws.status,
                                                                  nullptr);
    TTGB_CHECK_LAUNCH();
    DBuf sig((size_t)n, s);
    svd_sort_kernel<<<1, 1024, 0, s>>>(W, Vw, (int)n, Up.p, S, Vw + n * n, sig.p);
    TTGB_CHECK_LAUNCH();
    gemm_cm(Qb.p, m, Vw + n * n, n, U, m, m, n, n, 1.0, 0.0, s);   // U = Q V'
    transpose(Up.p, n, Vh, n, n, n, s);                            // Vh = U'^T
    return;
  }
  if (n > kJacobiBlockMaxN) {   // grid-wide block Jacobi, one launch per round
    const int sms = num_sms();
    const int nb = (int)std::max<int64_t>(1, (n + 2 * sms - 1) / (2 * sms));
    int P = (int)((n + nb - 1) / nb);
    P += P & 1;
    identity_kernel<<<cdiv((int64_t)n * n, 256), 256, 0, s>>>(Vw, (int)n);
    TTGB_CHECK_LAUNCH();
    DevBuf<unsigned> cnt(1, s);
    unsigned hcnt = 0;
    const double tol = std::max((double)n, 1.0) * kEps;
    int sweep = 0;
    for (; sweep < 60; ++sweep) {
      TTGB_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned), s));
      for (int r = 0; r < P - 1; ++r) {
        jacobi_grid_round_kernel<<<P / 2, 256, 0, s>>>(W, Vw, (int)n, nb, P, r, tol, cnt.p);
        TTGB_CHECK_LAUNCH();
      }
      TTGB_CUDA(cudaMemcpyAsync(&hcnt, cnt.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
      TTGB_CUDA(cudaStreamSynchronize(s));
      if (hcnt == 0) break;
    }
    if (sweep >= 60) TTGB_CUDA(cudaMemsetAsync(ws.status, 0x03, 1, s));
    DBuf sig((size_t)n, s);
    svd_sort_kernel<<<1, 1024, 0, s>>>(W, Vw, (int)n, Up.p, S, Vw + n * n, sig.p);
    TTGB_CHECK_LAUNCH();
    gemm_cm(Qb.p, m, Vw + n * n, n, U, m, m, n, n, 1.0, 0.0, s);   // U = Q V'
    transpose(Up.p, n, Vh, n, n, n, s);                            // Vh = U'^T
    return;
  }
  const size_t smem = (size_t)2 * n * n * sizeof(double);
  const int use_smem = smem <= 200 * 1024 ? 1 : 0;
  if (use_smem) smem_optin((const void*)jacobi_svd_kernel, (int)smem);
  // one warp per column pair of a round (n < 2 * kJacobiCluster here): idle warps would only
  // lengthen every block barrier of the round-robin sweep
  const int threads = (int)std::min<int64_t>(512, 32 * std::max<int64_t>(1, (n + 1) / 2));
  jacobi_svd_kernel<<<1, threads, use_smem ? smem : 0, s>>>(W, Vw, (int)n, Up.p, S, use_smem, 60,
                                                             ws.status, nullptr);
  TTGB_CHECK_LAUNCH();
  // U = Q V'
  gemm_cm(Qb.p, m, Vw, n, U, m, m, n, n, 1.0, 0.0, s);
  // Vh (n x n col-major) = U'^T
  transpose(Up.p, n, Vh, n, n, n, s);
}

void lu_solve(const double* B, int64_t n, const double* rhs, double* x, LinalgWS& ws,
              cudaStream_t s) {
  ws.e.ensure(n * n + 16, s);
  copy(B, ws.e.p, n * n, s);
  copy(rhs, x, n, s);
  lu_solve_kernel<<<1, 1024, 0, s>>>(ws.e.p, x, (int)n, ws.status);
  TTGB_CHECK_LAUNCH();
}

void gemv(const double* B, int64_t n, const double* x, double* y, cudaStream_t s) {
  if (n <= 0) return;
  gemv_rm_kernel<<<cdiv(n * 32, 256), 256, 0, s>>>(B, n, x, y);
  TTGB_CHECK_LAUNCH();
}

}  // namespace ttgb
