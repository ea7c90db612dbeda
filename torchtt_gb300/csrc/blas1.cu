// Vector kernels: two-stage deterministic reductions and element-wise updates (FP64).
#include <atomic>
#include <map>
#include <mutex>

#include "blas1.cuh"
#include "reduce.cuh"

namespace ttgb {

static std::atomic<int64_t> g_launches{0};
int64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void smem_optin(const void* kernel, int bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> done;
  int dev = 0;
  TTGB_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  int& cur = done[std::make_pair(kernel, dev)];
  if (cur >= bytes) return;
  TTGB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  cur = bytes;
}

namespace {

using red::RT;
using red::block_sum;

// Called by every block after writing its partials: the last block sums them in block order.
// post: 0 = plain sums, 1 = sqrt of vector 0.
__device__ void last_block_reduce(double* partial, unsigned* counter, int G, int nvec, double* out,
                                  int post) {
  if (!red::take_last_ticket(counter)) return;
  red::reduce_vectors(partial, nvec, G, [&](int v, double s) {
    out[v] = (post == 1 && v == 0) ? sqrt(s) : s;
  });
  red::reset_ticket(counter);
}

__global__ void __launch_bounds__(RT) nrm2_kernel(const double* __restrict__ x, int64_t n,
                                                   int64_t chunk, double* partial, unsigned* counter,
                                                   double* out, int post) {
  __shared__ double sh[32];
  const int64_t beg = blockIdx.x * chunk, end = min(n, beg + chunk);
  double s = 0.0;
  for (int64_t i = beg + threadIdx.x; i < end; i += blockDim.x) {
    const double v = x[i];
    s = fma(v, v, s);
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  last_block_reduce(partial, counter, gridDim.x, 1, out, post);
}

struct SegParams {
  const double* x[VecSegs::kMax];
  double* y[VecSegs::kMax];
  int64_t n[VecSegs::kMax];
  int64_t chunk[VecSegs::kMax];
  double* out[VecSegs::kMax];
  const double* den[VecSegs::kMax];
  int first_block[VecSegs::kMax + 1];   // blocks of segment i: [first_block[i], first_block[i+1])
  int count;
};

__global__ void __launch_bounds__(RT) nrm2_multi_kernel(SegParams p, double* partial,
                                                         unsigned* counter) {
  __shared__ double sh[32];
  int seg = 0;
  while (seg + 1 < p.count && (int)blockIdx.x >= p.first_block[seg + 1]) ++seg;
  const int lb = blockIdx.x - p.first_block[seg];
  const double* x = p.x[seg];
  const int64_t beg = lb * p.chunk[seg], end = min(p.n[seg], beg + p.chunk[seg]);
  double s = 0.0;
  for (int64_t i = beg + threadIdx.x; i < end; i += blockDim.x) {
    const double v = x[i];
    s = fma(v, v, s);
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  if (!red::take_last_ticket(counter)) return;
  {   // warp i sums segment i's partials (lanes over its blocks in order, then a fixed butterfly)
    const int lane = threadIdx.x & 31, i = threadIdx.x >> 5;
    if (i < p.count) {
      const volatile double* q = partial;
      double t = 0.0;
      for (int b = p.first_block[i] + lane; b < p.first_block[i + 1]; b += 32) t += q[b];
      t = red::warp_sum(t);
      if (lane == 0) *p.out[i] = sqrt(t);
    }
  }
  red::reset_ticket(counter);
}

__global__ void scale_multi_kernel(SegParams p, int64_t total) {
  __shared__ double f[VecSegs::kMax];
  if ((int)threadIdx.x < p.count) {
    const double d = *p.den[threadIdx.x];
    f[threadIdx.x] = (d > 0.0) ? 1.0 / d : 1.0;
  }
  __syncthreads();
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = t;
    int seg = 0;
    while (seg + 1 < p.count && i >= p.n[seg]) { i -= p.n[seg]; ++seg; }
    p.y[seg][i] *= f[seg];
  }
}

__global__ void axpby_kernel(double a, const double* __restrict__ x, double b, double* y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (b == 0.0) ? a * x[i] : fma(a, x[i], b * y[i]);
}

__global__ void sub_kernel(const double* __restrict__ x, const double* __restrict__ y, double* z,
                           int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    z[i] = x[i] - y[i];
}

__global__ void __launch_bounds__(RT) sub_nrm2_kernel(const double* x, const double* y, double* z,
                                                       int64_t n, int64_t chunk, double* partial,
                                                       unsigned* counter, double* out) {
  __shared__ double sh[32];
  const int64_t beg = blockIdx.x * chunk, end = min(n, beg + chunk);
  double s = 0.0;
  for (int64_t i = beg + threadIdx.x; i < end; i += blockDim.x) {
    const double v = x[i] - y[i];
    z[i] = v;
    s = fma(v, v, s);
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  last_block_reduce(partial, counter, gridDim.x, 1, out, 1);
}

__global__ void scale_dev_kernel(double* x, int64_t n, const double* num, const double* den) {
  const double d = *den;
  if (!(d > 0.0)) return;
  const double f = (num ? *num : 1.0) / d;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] *= f;
}

__global__ void scale_copy_kernel(const double* __restrict__ x, double a, double* y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i];
}

__global__ void fill_kernel(double* x, double v, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = v;
}

template <typename S, typename D>
__global__ void cast_kernel(const S* __restrict__ x, D* y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (D)x[i];
}

__global__ void copy2d_kernel(const double* __restrict__ src, int64_t sld, double* dst, int64_t dld,
                              int64_t rows, int64_t cols) {
  const int64_t total = rows * cols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / cols, j = t - (t / cols) * cols;
    dst[i * dld + j] = src[i * sld + j];
  }
}

__global__ void transpose_kernel(const double* __restrict__ src, int64_t sld, double* dst,
                                 int64_t dld, int64_t rows, int64_t cols) {
  __shared__ double tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  // src is cols x rows: src[c * sld + r]
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int64_t c = c0 + j, r = r0 + threadIdx.x;
    tile[j][threadIdx.x] = (c < cols && r < rows) ? src[c * sld + r] : 0.0;
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int64_t r = r0 + j, c = c0 + threadIdx.x;
    if (r < rows && c < cols) dst[r * dld + c] = tile[threadIdx.x][j];
  }
}

unsigned ew_grid(int64_t n) {
  unsigned g = cdiv(n, 256);
  const unsigned cap = (unsigned)num_sms() * 8;
  if (g > cap) g = cap;
  if (g == 0) g = 1;
  return g;
}

}  // namespace

int red_blocks(int64_t n) {
  int64_t g = (n + 511) / 512;
  const int64_t cap = 4 * (int64_t)num_sms();
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

void red_launch_dims(const RedWS& ws, int64_t n, int nvec, int& G, int64_t& chunk) {
  G = red_blocks(n);
  if (G > ws.cap_blocks) G = ws.cap_blocks;
  chunk = (n + G - 1) / G;
  chunk = ((chunk + 255) / 256) * 256;
  if (chunk < 256) chunk = 256;
  G = (int)((n + chunk - 1) / chunk);
  if (G < 1) G = 1;
  TTGB_REQUIRE(nvec <= ws.cap_vec, "reduction workspace too small for the number of vectors");
}

void nrm2(const RedWS& ws, const double* x, int64_t n, double* out, cudaStream_t s) {
  int G; int64_t chunk;
  red_launch_dims(ws, n, 1, G, chunk);
  nrm2_kernel<<<G, RT, 0, s>>>(x, n, chunk, ws.partial, ws.counter, out, 1);
  TTGB_CHECK_LAUNCH();
}

void nrm2_multi(const RedWS& ws, const VecSegs& v, cudaStream_t s) {
  TTGB_REQUIRE(v.count >= 1 && v.count <= VecSegs::kMax, "nrm2_multi: 1 to 4 segments");
  SegParams p{};
  p.count = v.count;
  int G = 0;
  for (int i = 0; i < v.count; ++i) {
    int g = red_blocks(v.n[i]);
    if (g > ws.cap_blocks / v.count) g = ws.cap_blocks / v.count;
    int64_t chunk = (v.n[i] + g - 1) / g;
    chunk = ((chunk + 255) / 256) * 256;
    if (chunk < 256) chunk = 256;
    g = (int)((v.n[i] + chunk - 1) / chunk);
    if (g < 1) g = 1;
    p.x[i] = v.x[i];
    p.n[i] = v.n[i];
    p.chunk[i] = chunk;
    p.out[i] = v.out[i];
    p.first_block[i] = G;
    G += g;
  }
  p.first_block[v.count] = G;
  nrm2_multi_kernel<<<G, RT, 0, s>>>(p, ws.partial, ws.counter);
  TTGB_CHECK_LAUNCH();
}

void scale_multi(const VecSegs& v, cudaStream_t s) {
  TTGB_REQUIRE(v.count >= 1 && v.count <= VecSegs::kMax, "scale_multi: 1 to 4 segments");
  SegParams p{};
  p.count = v.count;
  int64_t total = 0;
  for (int i = 0; i < v.count; ++i) {
    p.y[i] = v.x[i];
    p.n[i] = v.n[i];
    p.den[i] = v.den[i];
    total += v.n[i];
  }
  if (total <= 0) return;
  scale_multi_kernel<<<ew_grid(total), 256, 0, s>>>(p, total);
  TTGB_CHECK_LAUNCH();
}

void axpby(double a, const double* x, double b, double* y, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  axpby_kernel<<<ew_grid(n), 256, 0, s>>>(a, x, b, y, n);
  TTGB_CHECK_LAUNCH();
}

void sub(const double* x, const double* y, double* z, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  sub_kernel<<<ew_grid(n), 256, 0, s>>>(x, y, z, n);
  TTGB_CHECK_LAUNCH();
}

void sub_nrm2(const RedWS& ws, const double* x, const double* y, double* z, int64_t n, double* out,
              cudaStream_t s) {
  int G; int64_t chunk;
  red_launch_dims(ws, n, 1, G, chunk);
  sub_nrm2_kernel<<<G, RT, 0, s>>>(x, y, z, n, chunk, ws.partial, ws.counter, out);
  TTGB_CHECK_LAUNCH();
}

void scale_dev(double* x, int64_t n, const double* num, const double* den, cudaStream_t s) {
  if (n <= 0) return;
  scale_dev_kernel<<<ew_grid(n), 256, 0, s>>>(x, n, num, den);
  TTGB_CHECK_LAUNCH();
}

void scale_copy(const double* x, double a, double* y, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  scale_copy_kernel<<<ew_grid(n), 256, 0, s>>>(x, a, y, n);
  TTGB_CHECK_LAUNCH();
}

void fill(double* x, double v, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  fill_kernel<<<ew_grid(n), 256, 0, s>>>(x, v, n);
  TTGB_CHECK_LAUNCH();
}

void copy(const double* x, double* y, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  TTGB_CUDA(cudaMemcpyAsync(y, x, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
}

void cast(const double* x, float* y, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  cast_kernel<double, float><<<ew_grid(n), 256, 0, s>>>(x, y, n);
  TTGB_CHECK_LAUNCH();
}

void cast(const float* x, double* y, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  cast_kernel<float, double><<<ew_grid(n), 256, 0, s>>>(x, y, n);
  TTGB_CHECK_LAUNCH();
}

void copy2d(const double* src, int64_t sld, double* dst, int64_t dld, int64_t rows, int64_t cols,
            cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return;
  copy2d_kernel<<<ew_grid(rows * cols), 256, 0, s>>>(src, sld, dst, dld, rows, cols);
  TTGB_CHECK_LAUNCH();
}

void transpose(const double* src, int64_t sld, double* dst, int64_t dld, int64_t rows, int64_t cols,
               cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return;
  dim3 grid(cdiv(cols, 32), cdiv(rows, 32));
  TTGB_REQUIRE(grid.y < 65536, "transpose too tall");
  transpose_kernel<<<grid, dim3(32, 8), 0, s>>>(src, sld, dst, dld, rows, cols);
  TTGB_CHECK_LAUNCH();
}

namespace {
__global__ void scale_rows_cm_kernel(double* X, int64_t ld, int64_t rows, int64_t cols,
                                     const double* S) {
  const int64_t total = rows * cols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = t % rows, j = t / rows;
    X[q + j * ld] *= S[q];
  }
}
}  // namespace

void scale_rows_cm(double* X, int64_t ld, int64_t rows, int64_t cols, const double* S,
                   cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return;
  scale_rows_cm_kernel<<<ew_grid(rows * cols), 256, 0, s>>>(X, ld, rows, cols, S);
  TTGB_CHECK_LAUNCH();
}

}  // namespace ttgb
