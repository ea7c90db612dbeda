// Block-Jacobi preconditioners of the local AMEn system (reference: AMENsolveMV::setter /
// apply_prec, cpp/matvecs.h:153-194).
//   'c' (central): for every pair (d, D) of left/right rank indices the n x n block
//        sum_{s,S} Phi_l[d,s,d] A[s,:,:,S] Phi_r[D,S,D] is inverted;
//   'r' (right):   for every left rank index d the (n R) x (n R) block
//        sum_{s} Phi_l[d,s,d] A[s,m,n,S] Phi_r[L,S,R] over ((m,L),(n,R)) is inverted.
#include "gmres.cuh"
#include "prec.cuh"

namespace ttgb {

namespace {

// Jfull[(d,D), m, n] = sum_{s,S} Phi_l[d,s,d] A[s,m,n,S] Phi_r[D,S,D]
__global__ void build_c_kernel(const double* __restrict__ phil, const double* __restrict__ A,
                               const double* __restrict__ phir, int r, int s, int n, int S, int R,
                               double* J) {
  const int64_t total = (int64_t)r * R * n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int nn = (int)(t % n);
    const int mm = (int)((t / n) % n);
    const int D = (int)((t / ((int64_t)n * n)) % R);
    const int d = (int)(t / ((int64_t)n * n * R));
    double v = 0.0;
    for (int a = 0; a < s; ++a) {
      const double pl = phil[((int64_t)d * s + a) * r + d];
      for (int b = 0; b < S; ++b)
        v = fma(pl * A[(((int64_t)a * n + mm) * n + nn) * S + b], phir[((int64_t)D * S + b) * R + D], v);
    }
    J[t] = v;
  }
}

// Jt[d, (m,L), (n,R)] = sum_{s,S} Phi_l[d,s,d] A[s,m,n,S] Phi_r[L,S,R]
__global__ void build_r_kernel(const double* __restrict__ phil, const double* __restrict__ A,
                               const double* __restrict__ phir, int r, int s, int n, int S, int R,
                               double* J) {
  const int64_t sz = (int64_t)n * R;
  const int64_t total = (int64_t)r * sz * sz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t col = t % sz, row = (t / sz) % sz;
    const int d = (int)(t / (sz * sz));
    const int mm = (int)(row / R), L = (int)(row % R);
    const int nn = (int)(col / R), Rr = (int)(col % R);
    double v = 0.0;
    for (int a = 0; a < s; ++a) {
      const double pl = phil[((int64_t)d * s + a) * r + d];
      for (int b = 0; b < S; ++b)
        v = fma(pl * A[(((int64_t)a * n + mm) * n + nn) * S + b], phir[((int64_t)L * S + b) * R + Rr], v);
    }
    J[t] = v;
  }
}

// In-place Gauss-Jordan inversion with partial pivoting of `count` sz x sz row-major blocks;
// `work` holds count * sz * sz doubles of scratch (one block per thread block).
__global__ void __launch_bounds__(256) batched_inverse_kernel(double* M, int sz, double* work,
                                                              int* status) {
  const int64_t b = blockIdx.x;
  double* A = M + b * (int64_t)sz * sz;
  double* X = work + b * (int64_t)sz * sz;   // becomes the inverse
  __shared__ int piv;
  __shared__ double shv[8];
  __shared__ int shi[8];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  for (int64_t t = tid; t < (int64_t)sz * sz; t += nt) X[t] = ((t / sz) == (t % sz)) ? 1.0 : 0.0;
  __syncthreads();
  for (int j = 0; j < sz; ++j) {
    double best = -1.0;
    int bi = j;
    for (int i = j + tid; i < sz; i += nt) {
      const double v = fabs(A[(int64_t)i * sz + j]);
      if (v > best) { best = v; bi = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if (lane == 0) { shv[warp] = best; shi[warp] = bi; }
    __syncthreads();
    if (tid == 0) {
      double bb = -1.0; int ib = j;
      for (int w = 0; w < (nt >> 5); ++w)
        if (shv[w] > bb || (shv[w] == bb && shi[w] < ib)) { bb = shv[w]; ib = shi[w]; }
      piv = ib;
      if (!(bb > 0.0)) *status = 1;
    }
    __syncthreads();
    const int p = piv;
    if (p != j) {
      for (int c = tid; c < sz; c += nt) {
        double t = A[(int64_t)j * sz + c]; A[(int64_t)j * sz + c] = A[(int64_t)p * sz + c]; A[(int64_t)p * sz + c] = t;
        t = X[(int64_t)j * sz + c]; X[(int64_t)j * sz + c] = X[(int64_t)p * sz + c]; X[(int64_t)p * sz + c] = t;
      }
    }
    __syncthreads();
    const double inv = 1.0 / A[(int64_t)j * sz + j];
    __syncthreads();
    for (int c = tid; c < sz; c += nt) {
      A[(int64_t)j * sz + c] *= inv;
      X[(int64_t)j * sz + c] *= inv;
    }
    __syncthreads();
    for (int64_t t = tid; t < (int64_t)sz * sz; t += nt) {
      const int i = (int)(t / sz), c = (int)(t % sz);
      if (i == j) continue;
      const double f = A[(int64_t)i * sz + j];
      if (f == 0.0) continue;
      if (c != j) A[(int64_t)i * sz + c] = fma(-f, A[(int64_t)j * sz + c], A[(int64_t)i * sz + c]);
      X[(int64_t)i * sz + c] = fma(-f, X[(int64_t)j * sz + c], X[(int64_t)i * sz + c]);
    }
    __syncthreads();
    for (int i = tid; i < sz; i += nt)
      if (i != j) A[(int64_t)i * sz + j] = 0.0;
    __syncthreads();
  }
  for (int64_t t = tid; t < (int64_t)sz * sz; t += nt) A[t] = X[t];
}

// 'c': y[d, m, D] = sum_n J[(d,D), m, n] x[d, n, D]
__global__ void apply_c_kernel(const double* __restrict__ J, const double* __restrict__ x, double* y,
                               int r, int n, int R) {
  const int64_t total = (int64_t)r * n * R;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int D = (int)(t % R), mm = (int)((t / R) % n), d = (int)(t / ((int64_t)R * n));
    const double* Jb = J + (((int64_t)d * R + D) * n + mm) * n;
    double v = 0.0;
    for (int nn = 0; nn < n; ++nn) v = fma(Jb[nn], x[((int64_t)d * n + nn) * R + D], v);
    y[t] = v;
  }
}

// 'r': y[d, (m,L)] = sum_{(n,R)} J[d, (m,L), (n,R)] x[d, (n,R)]  (one warp per output)
__global__ void apply_r_kernel(const double* __restrict__ J, const double* __restrict__ x, double* y,
                               int r, int n, int R) {
  const int64_t sz = (int64_t)n * R;
  const int lane = threadIdx.x & 31;
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (row >= (int64_t)r * sz) return;
  const int d = (int)(row / sz);
  const double* Jr = J + row * sz;
  const double* xd = x + (int64_t)d * sz;
  double v = 0.0;
  for (int64_t c = lane; c < sz; c += 32) v = fma(Jr[c], xd[c], v);
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) y[row] = v;
}

unsigned grid_for(int64_t n) {
  unsigned g = cdiv(n, 256);
  if (g > 8192) g = 8192;
  return g ? g : 1;
}

}  // namespace

size_t prec_size(int prec, const LocalOpDims& d) {
  if (prec == kCPrec) return (size_t)(d.r * d.R * d.n * d.n);
  if (prec == kRPrec) return (size_t)(d.r * (d.n * d.R) * (d.n * d.R));
  return 0;
}

void prec_setup(int prec, const LocalOpDims& d, const double* phi_l, const double* A,
                const double* phi_r, double* J, DBuf& work, int* status, cudaStream_t s) {
  if (prec == kCPrec) {
    const int64_t total = d.r * d.R * d.n * d.n;
    build_c_kernel<<<grid_for(total), 256, 0, s>>>(phi_l, A, phi_r, (int)d.r, (int)d.s, (int)d.n,
                                                   (int)d.S, (int)d.R, J);
    TTGB_CHECK_LAUNCH();
    work.ensure((size_t)total, s);
    batched_inverse_kernel<<<(unsigned)(d.r * d.R), 256, 0, s>>>(J, (int)d.n, work.p, status);
    TTGB_CHECK_LAUNCH();
  } else if (prec == kRPrec) {
    const int64_t sz = d.n * d.R;
    const int64_t total = d.r * sz * sz;
    TTGB_REQUIRE(total < (int64_t)1 << 31, "'r' preconditioner blocks too large");
    build_r_kernel<<<grid_for(total), 256, 0, s>>>(phi_l, A, phi_r, (int)d.r, (int)d.s, (int)d.n,
                                                   (int)d.S, (int)d.R, J);
    TTGB_CHECK_LAUNCH();
    work.ensure((size_t)total, s);
    batched_inverse_kernel<<<(unsigned)d.r, 256, 0, s>>>(J, (int)sz, work.p, status);
    TTGB_CHECK_LAUNCH();
  }
}

void LocalOperator::apply_prec(const double* x, double* y, cudaStream_t s) const {
  const LocalOpDims& d = dims;
  if (prec == kCPrec) {
    const int64_t total = d.r * d.n * d.R;
    apply_c_kernel<<<grid_for(total), 256, 0, s>>>(J, x, y, (int)d.r, (int)d.n, (int)d.R);
    TTGB_CHECK_LAUNCH();
  } else if (prec == kRPrec) {
    const int64_t rows = d.r * d.n * d.R;
    apply_r_kernel<<<cdiv(rows * 32, 256), 256, 0, s>>>(J, x, y, (int)d.r, (int)d.n, (int)d.R);
    TTGB_CHECK_LAUNCH();
  } else {
    copy(x, y, d.r * d.n * d.R, s);
  }
}

}  // namespace ttgb
