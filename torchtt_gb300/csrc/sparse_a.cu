// Structure-aware A-core stage (see sparse_a.cuh).
#include <algorithm>
#include <array>
#include <vector>

#include "sparse_a.cuh"
#include "tc_gemm.cuh"

namespace ttgb {

namespace {

constexpr int kThreads = 256;

template <typename T, bool SPLIT>
__global__ void __launch_bounds__(kThreads)
sparse_stage_kernel(const int* __restrict__ rp, const int* __restrict__ ja,
                    const int* __restrict__ jb, const T* __restrict__ val,
                    const T* __restrict__ in, T* out, float* out_lo, StageDims g) {
  __shared__ T sv[SparseCore::kMaxRow];
  __shared__ int64_t soff[SparseCore::kMaxRow];
  if (g.gate != nullptr && *g.gate != 0) return;
  const int key = blockIdx.x;
  const int beg = rp[key];
  const int cnt = rp[key + 1] - beg;
  for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
    sv[j] = val[beg + j];
    soff[j] = (int64_t)ja[beg + j] * g.pa + (int64_t)jb[beg + j] * g.pb;
  }
  __syncthreads();
  const int64_t total = g.O1 * g.O2;
  const int64_t koff = g.ke0 > 0 ? (key % g.ke0) * g.sk + (key / g.ke0) * g.sk1 : (int64_t)key * g.sk;
  T* ob = out + koff;
  for (int64_t t = (int64_t)blockIdx.y * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.y * blockDim.x) {
    const int64_t o1 = t / g.O2, o2 = t - o1 * g.O2;
    const T* ib = in + o1 * g.si1 + o2;
    T acc = T(0);
    for (int j = 0; j < cnt; ++j) acc = fma(sv[j], ib[soff[j]], acc);
    const int64_t o = o1 * g.so1 + o2;
    if constexpr (SPLIT) {
      const float h = to_tf32((float)acc);
      ob[o] = h;
      out_lo[koff + o] = to_tf32((float)acc - h);
    } else {
      ob[o] = acc;
    }
  }
}

template <typename T, bool SPLIT>
void launch_stage(const SparseCsr& c, const T* val, const T* in, T* out, float* lo,
                  const StageDims& g, cudaStream_t s) {
  if (c.keys <= 0 || g.O1 <= 0 || g.O2 <= 0) return;
  TTGB_REQUIRE(c.keys < (int64_t(1) << 31) && c.max_row <= SparseCore::kMaxRow,
               "sparse stage: unsupported core");
  const int64_t total = g.O1 * g.O2;
  int64_t gy = (int64_t)cdiv(total, kThreads);
  const int64_t want = std::max<int64_t>(1, (int64_t)8 * num_sms() / c.keys);
  gy = std::max<int64_t>(1, std::min<int64_t>({gy, want, 65535}));
  dim3 grid((unsigned)c.keys, (unsigned)gy);
  sparse_stage_kernel<T, SPLIT><<<grid, kThreads, 0, s>>>(c.rp.p, c.a.p, c.b.p, val, in, out, lo, g);
  TTGB_CHECK_LAUNCH();
}

// entries (key, a, b, value) of one grouping, sorted by key then (a, b)
struct Entry {
  int64_t key;
  int a, b;
  double v;
};

void upload(SparseCsr& c, std::vector<Entry>& e, int64_t keys, cudaStream_t st) {
  std::sort(e.begin(), e.end(), [](const Entry& x, const Entry& y) {
    if (x.key != y.key) return x.key < y.key;
    if (x.a != y.a) return x.a < y.a;
    return x.b < y.b;
  });
  c.keys = keys;
  c.nnz = (int64_t)e.size();
  std::vector<int> rp(keys + 1, 0), a(e.size()), b(e.size());
  std::vector<double> v(e.size());
  std::vector<float> v32(e.size());
  for (size_t i = 0; i < e.size(); ++i) {
    rp[e[i].key + 1]++;
    a[i] = e[i].a;
    b[i] = e[i].b;
    v[i] = e[i].v;
    v32[i] = (float)e[i].v;
  }
  c.max_row = 0;
  for (int64_t k = 0; k < keys; ++k) {
    c.max_row = std::max(c.max_row, rp[k + 1]);
    rp[k + 1] += rp[k];
  }
  c.rp.reset(keys + 1, st);
  c.a.reset(std::max<size_t>(1, e.size()), st);
  c.b.reset(std::max<size_t>(1, e.size()), st);
  c.val.reset(std::max<size_t>(1, e.size()), st);
  c.val32.reset(std::max<size_t>(1, e.size()), st);
  TTGB_CUDA(cudaMemcpyAsync(c.rp.p, rp.data(), rp.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  if (!e.empty()) {
    TTGB_CUDA(cudaMemcpyAsync(c.a.p, a.data(), a.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    TTGB_CUDA(cudaMemcpyAsync(c.b.p, b.data(), b.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    TTGB_CUDA(cudaMemcpyAsync(c.val.p, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    TTGB_CUDA(cudaMemcpyAsync(c.val32.p, v32.data(), v32.size() * sizeof(float),
                              cudaMemcpyHostToDevice, st));
  }
  // the host vectors are released when this function returns: finish the copies first
  TTGB_CUDA(cudaStreamSynchronize(st));
}

}  // namespace

void SparseCore::build(const double* A, int64_t s_, int64_t M_, int64_t N_, int64_t S_,
                       cudaStream_t st) {
  s = s_; M = M_; N = N_; S = S_;
  use = false;
  const int64_t ne = s * M * N * S;
  if (ne <= 0 || s * N >= (int64_t(1) << 31) || M * S >= (int64_t(1) << 31)) return;
  std::vector<double> h(ne);
  TTGB_CUDA(cudaMemcpyAsync(h.data(), A, ne * sizeof(double), cudaMemcpyDeviceToHost, st));
  TTGB_CUDA(cudaStreamSynchronize(st));
  std::vector<Entry> elp, efw, ebk, erh;
  for (int64_t a = 0; a < s; ++a)
    for (int64_t m = 0; m < M; ++m)
      for (int64_t n = 0; n < N; ++n)
        for (int64_t b = 0; b < S; ++b) {
          const double v = h[((a * M + m) * N + n) * S + b];
          if (v == 0.0) continue;
          elp.push_back({m * S + b, (int)a, (int)n, v});
          efw.push_back({n * S + b, (int)a, (int)m, v});
          ebk.push_back({a * N + n, (int)m, (int)b, v});
          erh.push_back({a * M + m, (int)n, (int)b, v});
        }
  const int64_t nnz = (int64_t)elp.size();
  if (4 * nnz >= ne) return;   // dense enough for the GEMM path
  upload(lp, elp, M * S, st);
  upload(fw, efw, N * S, st);
  upload(bk, ebk, s * N, st);
  upload(rh, erh, s * M, st);
  use = lp.max_row <= kMaxRow && fw.max_row <= kMaxRow && bk.max_row <= kMaxRow &&
        rh.max_row <= kMaxRow;
}

void sparse_stage(const SparseCsr& c, const double* in, double* out, const StageDims& g,
                  cudaStream_t s) {
  launch_stage<double, false>(c, c.val.p, in, out, nullptr, g, s);
}

void sparse_stage(const SparseCsr& c, const float* in, float* out, const StageDims& g,
                  cudaStream_t s) {
  launch_stage<float, false>(c, c.val32.p, in, out, nullptr, g, s);
}

void sparse_stage_split(const SparseCsr& c, const float* in, float* hi, float* lo,
                        const StageDims& g, cudaStream_t s) {
  launch_stage<float, true>(c, c.val32.p, in, hi, lo, g, s);
}

}  // namespace ttgb
