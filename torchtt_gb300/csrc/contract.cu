// FP64 contraction engine and the AMEn contraction recipes built on it.
//
// The kernel is a shared-memory-tiled FP64 GEMM (BMxBN output tile, BK=16, 256 threads, each
// thread a (BM/16)x(BN/16) register tile). Every operand index may be a pair of tensor indices with
// their own strides (struct Ax), so the reference's tensordot permutes (cpp/amen_solve.h:17-98)
// cost no copies. FP64 FMA throughput is the bound on this path. The tile shape and split-K
// (atomic FP64 adds) of a launch come from the tile autotuner's record for its shape class, or
// from an occupancy heuristic: the largest tile whose grid covers the SMs, split-K when even the
// smallest tile leaves SMs idle. The same engine runs in double-float arithmetic on the FP32 pipe
// (contract_df_kernel) and in FP32.
#include <climits>

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <mutex>
#include <shared_mutex>
#include <type_traits>
#include <unordered_map>

#include "contract.cuh"
#include "df.cuh"

namespace ttgb {

namespace {

struct AxD {  // device copy of Ax with a 32-bit inner extent
  int e0;
  int64_t s1, s0;
};

__device__ __forceinline__ int64_t ax_off(const AxD& a, int i) {
  int i1 = i / a.e0;
  int i0 = i - i1 * a.e0;
  return (int64_t)i1 * a.s1 + (int64_t)i0 * a.s0;
}

template <typename T>
struct KParams {
  int M, N, K, batch, splitk, kchunk;
  const T* A;
  AxD am, ak;
  int64_t a_bs;
  const T* B;
  AxD bk, bn;
  int64_t b_bs;
  T* C;
  AxD cm, cn;
  int64_t c_bs;
  T alpha, beta;
  int tri;
};

constexpr int BK = 16;
constexpr int NT = 256;

template <typename T, int BM, int BN>
__global__ void __launch_bounds__(NT) contract_kernel(KParams<T> p) {
  constexpr int TM = BM / 16, TN = BN / 16;
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];

  const int tid = threadIdx.x;
  const int bz = blockIdx.z;
  const int bidx = bz / p.splitk;
  const int ks = bz - bidx * p.splitk;
  const int kbeg = ks * p.kchunk;
  int kend = min(p.K, kbeg + p.kchunk);
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  if ((p.tri & kTriLowerC) && m0 + BM <= n0) return;   // tile strictly above the diagonal
  if (p.tri & kTriUpperB) kend = min(kend, n0 + BN);   // B(k, n) = 0 for k > n

  const T* A = p.A + (int64_t)bidx * p.a_bs;
  const T* B = p.B + (int64_t)bidx * p.b_bs;

  // loader mapping: A tile BM x BK, B tile BK x BN, NT threads
  constexpr int A_ROWS_PER_PASS = NT / BK;   // threads cover (row, k) with k = tid % BK
  constexpr int B_COLS_PER_PASS = NT / BK;
  const int lk = tid % BK;
  const int lr = tid / BK;   // 0..15

  int64_t a_moff[BM / A_ROWS_PER_PASS];
  bool a_mok[BM / A_ROWS_PER_PASS];
#pragma unroll
  for (int i = 0; i < BM / A_ROWS_PER_PASS; ++i) {
    int m = m0 + lr + i * A_ROWS_PER_PASS;
    a_mok[i] = m < p.M;
    a_moff[i] = a_mok[i] ? ax_off(p.am, m) : 0;
  }
  int64_t b_noff[BN / B_COLS_PER_PASS];
  bool b_nok[BN / B_COLS_PER_PASS];
#pragma unroll
  for (int i = 0; i < BN / B_COLS_PER_PASS; ++i) {
    int n = n0 + lr + i * B_COLS_PER_PASS;
    b_nok[i] = n < p.N;
    b_noff[i] = b_nok[i] ? ax_off(p.bn, n) : 0;
  }

  const int ty = tid / 16, tx = tid % 16;
  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = T(0);

  // next K tile's operands in registers while the current one is multiplied (same sum order)
  T ra[BM / A_ROWS_PER_PASS], rb[BN / B_COLS_PER_PASS];
  auto load_tile = [&](int k0) {
    const int k = k0 + lk;
    const bool kok = k < kend;
    const int64_t a_koff = kok ? ax_off(p.ak, k) : 0;
    const int64_t b_koff = kok ? ax_off(p.bk, k) : 0;
#pragma unroll
    for (int i = 0; i < BM / A_ROWS_PER_PASS; ++i)
      ra[i] = (kok && a_mok[i]) ? __ldg(A + a_moff[i] + a_koff) : T(0);
#pragma unroll
    for (int i = 0; i < BN / B_COLS_PER_PASS; ++i)
      rb[i] = (kok && b_nok[i]) ? __ldg(B + b_noff[i] + b_koff) : T(0);
  };
  if (kbeg < kend) load_tile(kbeg);
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
    for (int i = 0; i < BM / A_ROWS_PER_PASS; ++i) As[lk][lr + i * A_ROWS_PER_PASS] = ra[i];
#pragma unroll
    for (int i = 0; i < BN / B_COLS_PER_PASS; ++i) Bs[lk][lr + i * B_COLS_PER_PASS] = rb[i];
    __syncthreads();
    if (k0 + BK < kend) load_tile(k0 + BK);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }

  T* C = p.C + (int64_t)bidx * p.c_bs;
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int m = m0 + ty + 16 * i;
    if (m >= p.M) continue;
    const int64_t cmo = ax_off(p.cm, m);
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int n = n0 + tx + 16 * j;
      if (n >= p.N) continue;
      T* c = C + cmo + ax_off(p.cn, n);
      const T v = p.alpha * acc[i][j];
      if (p.splitk > 1) {
        atomicAdd(c, v);
      } else {
        *c = (p.beta == T(0)) ? v : fma(p.beta, *c, v);
      }
    }
  }
}

// The same contraction in double-float arithmetic on the FP32 pipe: every FP64 operand is split
// into hi + lo FP32 parts (x = hi + lo to ~2^-48), a product is formed error-free from the FMA
// residual of hi*hi plus the cross terms, and the sum is kept as an unnormalised (hi, lo) FP32 pair
// with an error-free two-sum per step. About 10 FP32 operations per multiply-add: on GB300, where
// the FP32 pipe is ~60x the FP64 pipe, this is several times the FP64 rate at ~1e-13 relative
// accuracy (operands within the FP32 exponent range).
//
// The FP64 -> (hi, lo) split is df_split (df.cuh).
template <int BM, int BN>
__global__ void __launch_bounds__(NT) contract_df_kernel(KParams<double> p) {
  constexpr int TM = BM / 16, TN = BN / 16;
  __shared__ float Ah[BK][BM + 1], Al[BK][BM + 1];
  __shared__ float Bh[BK][BN + 1], Bl[BK][BN + 1];

  const int tid = threadIdx.x;
  const int bz = blockIdx.z;
  const int bidx = bz / p.splitk;
  const int ks = bz - bidx * p.splitk;
  const int kbeg = ks * p.kchunk;
  int kend = min(p.K, kbeg + p.kchunk);
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  if ((p.tri & kTriLowerC) && m0 + BM <= n0) return;
  if (p.tri & kTriUpperB) kend = min(kend, n0 + BN);

  const double* A = p.A + (int64_t)bidx * p.a_bs;
  const double* B = p.B + (int64_t)bidx * p.b_bs;
  constexpr int ROWS_PER_PASS = NT / BK;
  const int lk = tid % BK;
  const int lr = tid / BK;
  int64_t a_moff[BM / ROWS_PER_PASS];
  bool a_mok[BM / ROWS_PER_PASS];
#pragma unroll
  for (int i = 0; i < BM / ROWS_PER_PASS; ++i) {
    const int m = m0 + lr + i * ROWS_PER_PASS;
    a_mok[i] = m < p.M;
    a_moff[i] = a_mok[i] ? ax_off(p.am, m) : 0;
  }
  int64_t b_noff[BN / ROWS_PER_PASS];
  bool b_nok[BN / ROWS_PER_PASS];
#pragma unroll
  for (int i = 0; i < BN / ROWS_PER_PASS; ++i) {
    const int n = n0 + lr + i * ROWS_PER_PASS;
    b_nok[i] = n < p.N;
    b_noff[i] = b_nok[i] ? ax_off(p.bn, n) : 0;
  }
  const int ty = tid / 16, tx = tid % 16;
  float ch[TM][TN], cl[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) { ch[i][j] = 0.f; cl[i][j] = 0.f; }

  // The operands of the next K tile are loaded into registers while the current tile is
  // multiplied (the global-load latency overlaps the arithmetic); the order of the sums is the
  // same as with a load per tile.
  double ra[BM / ROWS_PER_PASS], rb[BN / ROWS_PER_PASS];
  auto load_tile = [&](int k0) {
    const int k = k0 + lk;
    const bool kok = k < kend;
    const int64_t a_koff = kok ? ax_off(p.ak, k) : 0;
    const int64_t b_koff = kok ? ax_off(p.bk, k) : 0;
#pragma unroll
    for (int i = 0; i < BM / ROWS_PER_PASS; ++i)
      ra[i] = (kok && a_mok[i]) ? __ldg(A + a_moff[i] + a_koff) : 0.0;
#pragma unroll
    for (int i = 0; i < BN / ROWS_PER_PASS; ++i)
      rb[i] = (kok && b_nok[i]) ? __ldg(B + b_noff[i] + b_koff) : 0.0;
  };
  if (kbeg < kend) load_tile(kbeg);
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
    for (int i = 0; i < BM / ROWS_PER_PASS; ++i) {
      float h, l;
      df_split(ra[i], h, l);
      Ah[lk][lr + i * ROWS_PER_PASS] = h;
      Al[lk][lr + i * ROWS_PER_PASS] = l;
    }
#pragma unroll
    for (int i = 0; i < BN / ROWS_PER_PASS; ++i) {
      float h, l;
      df_split(rb[i], h, l);
      Bh[lk][lr + i * ROWS_PER_PASS] = h;
      Bl[lk][lr + i * ROWS_PER_PASS] = l;
    }
    __syncthreads();
    if (k0 + BK < kend) load_tile(k0 + BK);
#pragma unroll 4
    for (int kk = 0; kk < BK; ++kk) {
      float ah[TM], al[TM], bh[TN], bl[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) { ah[i] = Ah[kk][ty + 16 * i]; al[i] = Al[kk][ty + 16 * i]; }
#pragma unroll
      for (int j = 0; j < TN; ++j) { bh[j] = Bh[kk][tx + 16 * j]; bl[j] = Bl[kk][tx + 16 * j]; }
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) {
          const float pr = ah[i] * bh[j];
          float e = fmaf(ah[i], bh[j], -pr);        // exact residual of the leading product
          e = fmaf(ah[i], bl[j], e);
          e = fmaf(al[i], bh[j], e);
          const float s = ch[i][j] + pr;            // two-sum of the running high part and pr
          const float bb = s - ch[i][j];
          const float err = (ch[i][j] - (s - bb)) + (pr - bb);
          ch[i][j] = s;
          cl[i][j] += err + e;
        }
    }
    // renormalise the pair once per K tile (two-sum of high and low part): the low part is summed
    // in plain FP32, so left to grow over a long K its own rounding would set the accuracy
    // (a 4928-long Gram sum: 2e-12 relative without, 3e-13 with this step)
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const float s = ch[i][j] + cl[i][j];
        const float bb = s - ch[i][j];
        cl[i][j] = (ch[i][j] - (s - bb)) + (cl[i][j] - bb);
        ch[i][j] = s;
      }
    __syncthreads();
  }

  double* C = p.C + (int64_t)bidx * p.c_bs;
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int m = m0 + ty + 16 * i;
    if (m >= p.M) continue;
    const int64_t cmo = ax_off(p.cm, m);
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int n = n0 + tx + 16 * j;
      if (n >= p.N) continue;
      double* c = C + cmo + ax_off(p.cn, n);
      const double v = p.alpha * ((double)ch[i][j] + (double)cl[i][j]);
      if (p.splitk > 1) atomicAdd(c, v);
      else *c = (p.beta == 0.0) ? v : fma(p.beta, *c, v);
    }
  }
}

// C <- beta * C over the (batched, strided) output index space
template <typename T>
__global__ void scale_output_kernel(T* C, int M, int N, int batch, AxD cm, AxD cn, int64_t c_bs,
                                    T beta) {
  const int64_t total = (int64_t)M * N * batch;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    int b = (int)(t / ((int64_t)M * N));
    int rem = (int)(t - (int64_t)b * M * N);
    int m = rem / N, n = rem - (rem / N) * N;
    T* c = C + (int64_t)b * c_bs + ax_off(cm, m) + ax_off(cn, n);
    *c = (beta == T(0)) ? T(0) : beta * *c;
  }
}

AxD to_dev(const Ax& a, int extent) {
  AxD r;
  if (a.e0 >= extent || a.e0 >= INT_MAX) {
    r.e0 = INT_MAX;
    r.s1 = 0;
  } else {
    r.e0 = (int)a.e0;
    r.s1 = a.s1;
  }
  r.s0 = a.s0;
  return r;
}

thread_local int t_fp64_engine = kFp64Native;

// ---------------------------------------------------------------------------------------------
// Tile autotuner. A launch is described by its shape class: the engine (FP64, double-float,
// FP32), power-of-two buckets of M, N, K and the batch, the triangular flags and which operand
// strides are unit, and the device. The first launch of a class with beta == 0 (the output is
// overwritten, so running it several times is harmless) and no overlap between C and its inputs
// times every candidate - the four tile shapes, each with and without split-K - with CUDA events
// on the caller's stream (best of two runs) and records the fastest; later launches of the class
// use the record. Launches that cannot be tuned (beta != 0, aliasing, a capturing stream, a
// deterministic request) and classes being tuned by another thread use the occupancy heuristic.
// ---------------------------------------------------------------------------------------------
struct TileCfg {
  int bm, bn, split;   // split: 0 no split-K, 1 split-K sized to fill the GPU
};
constexpr TileCfg kCandidates[] = {{64, 64, 0}, {64, 32, 0}, {32, 64, 0}, {32, 32, 0},
                                   {64, 64, 1}, {64, 32, 1}, {32, 64, 1}, {32, 32, 1}};
constexpr int kNumCandidates = (int)(sizeof(kCandidates) / sizeof(kCandidates[0]));

std::atomic<int> g_autotune{-1};   // -1: not read yet from TTGB_AUTOTUNE
std::shared_mutex g_tune_mu;   // readers: every launch of a recorded class; writers: tuning
std::unordered_map<uint64_t, int> g_tune_table;   // class -> candidate index (-1: being tuned)
std::atomic<int64_t> g_tune_runs{0};
std::once_flag g_table_once;
std::string g_table_path;   // TTGB_AUTOTUNE_TABLE: records read at first use, new ones appended

// Reads "class candidate" lines (hex, decimal) of a previous process into the table.
void load_table() {
  const char* e = std::getenv("TTGB_AUTOTUNE_TABLE");
  if (!e || !*e) return;
  std::unique_lock<std::shared_mutex> g(g_tune_mu);
  g_table_path = e;
  FILE* f = std::fopen(e, "r");
  if (!f) return;
  unsigned long long k = 0;
  int c = 0;
  while (std::fscanf(f, "%llx %d", &k, &c) == 2)
    if (c >= 0 && c < kNumCandidates) g_tune_table[(uint64_t)k] = c;
  std::fclose(f);
}

void append_record(uint64_t key, int c) {   // caller holds the unique lock
  if (g_table_path.empty() || c < 0) return;
  FILE* f = std::fopen(g_table_path.c_str(), "a");
  if (!f) return;
  std::fprintf(f, "%llx %d\n", (unsigned long long)key, c);
  std::fclose(f);
}

thread_local bool t_no_tuning_runs = false;   // set by NoTuningScope

bool autotune_on() {
  int v = g_autotune.load();
  if (v < 0) {
    const char* e = std::getenv("TTGB_AUTOTUNE");
    v = (e && e[0] == '0') ? 0 : 1;
    g_autotune.store(v);
  }
  return v == 1;
}

int log2_bucket(int64_t v) {
  int b = 0;
  while ((int64_t(1) << b) < v && b < 40) ++b;
  return b;
}

// largest address offset of an index of the given extent
int64_t ax_span(const Ax& a, int64_t extent) {
  if (extent <= 0) return 0;
  if (a.e0 >= extent) return (extent - 1) * a.s0;
  return (a.e0 - 1) * a.s0 + ((extent - 1) / a.e0) * a.s1;
}

template <typename T>
bool overlaps(const T* x, int64_t xs, const T* y, int64_t ys) {
  return x < y + ys + 1 && y < x + xs + 1;
}

// CTAs a split-K launch aims at, in multiples of the SM count (TTGB_SPLIT_TARGET, default 2)
double split_target() {
  static const double v = [] {
    const char* e = std::getenv("TTGB_SPLIT_TARGET");
    const double x = e ? std::atof(e) : 2.0;
    return (x > 0.0 && x <= 16.0) ? x : 2.0;
  }();
  return v;
}

template <typename T>
int heuristic_split(const ContractDescT<T>& d, int bm, int bn, int sms, bool force) {
  const int64_t t = (int64_t)cdiv(d.M, bm) * cdiv(d.N, bn) * d.batch;
  const int64_t target = (int64_t)(split_target() * sms);
  if (!force && !(t < sms && d.K >= 128)) return 1;
  int splitk = (int)((target + t - 1) / t);
  const int maxsplit = d.K / 64;
  if (splitk > maxsplit) splitk = maxsplit;
  return splitk < 1 ? 1 : splitk;
}

template <typename T>
void launch_tiles(const ContractDescT<T>& d, KParams<T> p, int bm, int bn, int splitk,
                  cudaStream_t stream) {
  int kchunk = d.K;
  if (splitk > 1) {
    kchunk = (int)cdiv(cdiv(d.K, splitk), BK) * BK;
    splitk = (int)cdiv(d.K, kchunk);
  }
  p.splitk = splitk;
  p.kchunk = kchunk;
  if (splitk > 1 && !(d.c_zero && d.beta == T(0))) {
    int64_t total = (int64_t)d.M * d.N * d.batch;
    unsigned g = cdiv(total, 256);
    if (g > 8192) g = 8192;
    scale_output_kernel<<<g, 256, 0, stream>>>(p.C, p.M, p.N, p.batch, p.cm, p.cn, p.c_bs, p.beta);
    TTGB_CHECK_LAUNCH();
  }
  dim3 grid(cdiv(d.N, bn), cdiv(d.M, bm), (unsigned)(d.batch * splitk));
  TTGB_REQUIRE(grid.y < 65536 && grid.z < 65536, "contraction grid too large");
  if constexpr (std::is_same<T, double>::value) {
    if (t_fp64_engine == kFp64DoubleFloat) {
      if (bm == 64 && bn == 64) contract_df_kernel<64, 64><<<grid, NT, 0, stream>>>(p);
      else if (bm == 64 && bn == 32) contract_df_kernel<64, 32><<<grid, NT, 0, stream>>>(p);
      else if (bm == 32 && bn == 64) contract_df_kernel<32, 64><<<grid, NT, 0, stream>>>(p);
      else contract_df_kernel<32, 32><<<grid, NT, 0, stream>>>(p);
      TTGB_CHECK_LAUNCH();
      return;
    }
  }
  if (bm == 64 && bn == 64) contract_kernel<T, 64, 64><<<grid, NT, 0, stream>>>(p);
  else if (bm == 64 && bn == 32) contract_kernel<T, 64, 32><<<grid, NT, 0, stream>>>(p);
  else if (bm == 32 && bn == 64) contract_kernel<T, 32, 64><<<grid, NT, 0, stream>>>(p);
  else contract_kernel<T, 32, 32><<<grid, NT, 0, stream>>>(p);
  TTGB_CHECK_LAUNCH();
}

template <typename T>
uint64_t tune_key(const ContractDescT<T>& d) {
  const int eng = std::is_same<T, float>::value ? 2 : (t_fp64_engine == kFp64DoubleFloat ? 1 : 0);
  const int units = (d.am.s0 == 1) | ((d.ak.s0 == 1) << 1) | ((d.bk.s0 == 1) << 2) |
                    ((d.bn.s0 == 1) << 3) | ((d.cm.s0 == 1) << 4);
  uint64_t k = (uint64_t)eng;
  k = k * 64 + (uint64_t)log2_bucket(d.M);
  k = k * 64 + (uint64_t)log2_bucket(d.N);
  k = k * 64 + (uint64_t)log2_bucket(d.K);
  k = k * 64 + (uint64_t)log2_bucket(d.batch);
  k = k * 4 + (uint64_t)(d.tri & 3);
  k = k * 32 + (uint64_t)units;
  k = k * 1024 + (uint64_t)(num_sms() & 1023);   // the GPU model, through its SM count
  return k;
}

// Returns the candidate index to use, tuning the class first when this launch may be repeated.
// -1: use the heuristic. A tuned launch has already written C (tuned = true).
template <typename T>
int tuned_choice(const ContractDescT<T>& d, const KParams<T>& p, cudaStream_t stream,
                 bool& tuned) {
  tuned = false;
  if (d.beta != T(0)) return -1;
  const int64_t sa = (d.batch - 1) * d.a_bs + ax_span(d.am, d.M) + ax_span(d.ak, d.K);
  const int64_t sb = (d.batch - 1) * d.b_bs + ax_span(d.bk, d.K) + ax_span(d.bn, d.N);
  const int64_t sc = (d.batch - 1) * d.c_bs + ax_span(d.cm, d.M) + ax_span(d.cn, d.N);
  if (overlaps<T>(d.C, sc, d.A, sa) || overlaps<T>(d.C, sc, d.B, sb)) return -1;
  std::call_once(g_table_once, load_table);
  const uint64_t key = tune_key(d);
  {
    std::shared_lock<std::shared_mutex> g(g_tune_mu);
    auto it = g_tune_table.find(key);
    if (it != g_tune_table.end()) return it->second;
  }
  {
    std::unique_lock<std::shared_mutex> g(g_tune_mu);
    auto it = g_tune_table.find(key);
    if (it != g_tune_table.end()) return it->second;
    if (t_no_tuning_runs) return -1;   // a caller that must not block: heuristic tile
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
      return -1;
    g_tune_table[key] = -1;   // being tuned: other threads use the heuristic meanwhile
  }
  const int sms = num_sms();
  struct Events {   // destroyed on every exit, also when a launch check throws
    cudaEvent_t e[2] = {nullptr, nullptr};
    ~Events() {
      if (e[0]) cudaEventDestroy(e[0]);
      if (e[1]) cudaEventDestroy(e[1]);
    }
  } evs;
  cudaEvent_t* ev = evs.e;
  TTGB_CUDA(cudaEventCreate(&ev[0]));
  TTGB_CUDA(cudaEventCreate(&ev[1]));
  int best = -1;
  float best_ms = 0.f;
  for (int rep = 0; rep < 2; ++rep) {
    for (int c = 0; c < kNumCandidates; ++c) {
      const TileCfg& t = kCandidates[c];
      const int split = t.split ? heuristic_split(d, t.bm, t.bn, sms, true) : 1;
      if (t.split && split == 1) continue;   // the same launch as the unsplit candidate
      TTGB_CUDA(cudaEventRecord(ev[0], stream));
      launch_tiles(d, p, t.bm, t.bn, split, stream);
      TTGB_CUDA(cudaEventRecord(ev[1], stream));
      TTGB_CUDA(cudaEventSynchronize(ev[1]));
      float ms = 0.f;
      TTGB_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
      if (rep == 1 && (best < 0 || ms < best_ms)) { best = c; best_ms = ms; }
    }
  }
  g_tune_runs.fetch_add(1);
  {
    std::unique_lock<std::shared_mutex> g(g_tune_mu);
    g_tune_table[key] = best;
    append_record(key, best);
  }
  tuned = true;
  return best;
}

template <typename T>
void launch_contract(const ContractDescT<T>& d, cudaStream_t stream, bool deterministic) {
  if (d.M <= 0 || d.N <= 0 || d.batch <= 0) return;
  // the tuning runs write C before the chosen tile runs again: those launches may not assume C = 0
  ContractDescT<T> dz = d;
  dz.c_zero = false;
  KParams<T> p;
  p.M = d.M; p.N = d.N; p.K = d.K; p.batch = d.batch;
  p.A = d.A; p.am = to_dev(d.am, d.M); p.ak = to_dev(d.ak, d.K); p.a_bs = d.a_bs;
  p.B = d.B; p.bk = to_dev(d.bk, d.K); p.bn = to_dev(d.bn, d.N); p.b_bs = d.b_bs;
  p.C = d.C; p.cm = to_dev(d.cm, d.M); p.cn = to_dev(d.cn, d.N); p.c_bs = d.c_bs;
  p.alpha = d.alpha; p.beta = d.beta;
  p.tri = d.tri;
  if (d.K <= 0) {  // empty sum: C = beta * C
    scale_output_kernel<<<cdiv((int64_t)d.M * d.N * d.batch, 256) > 4096 ? 4096 : cdiv((int64_t)d.M * d.N * d.batch, 256), 256, 0, stream>>>(
        p.C, p.M, p.N, p.batch, p.cm, p.cn, p.c_bs, p.beta);
    TTGB_CHECK_LAUNCH();
    return;
  }
  const int sms = num_sms();
  if (!deterministic && autotune_on()) {
    bool tuned = false;
    const int c = tuned_choice(dz, p, stream, tuned);
    // after tuning, C holds the last candidate's result: the chosen tile runs once more, so the
    // first launch of a class gives what every later launch of the class computes
    if (c >= 0) {
      const TileCfg& t = kCandidates[c];
      launch_tiles(tuned ? dz : d, p, t.bm, t.bn,
                   t.split ? heuristic_split(d, t.bm, t.bn, sms, true) : 1, stream);
      return;
    }
  }
  // occupancy heuristic: the largest tile whose grid still gives two CTAs per SM, split-K when
  // even 32 x 32 tiles leave SMs idle
  auto tiles = [&](int bm, int bn) { return (int64_t)cdiv(d.M, bm) * cdiv(d.N, bn) * d.batch; };
  int bm = 64, bn = 64;
  const int64_t target = 2 * (int64_t)sms;
  if (tiles(64, 64) < target) {
    if (d.M >= d.N) { bm = 64; bn = 32; } else { bm = 32; bn = 64; }
    if (tiles(bm, bn) < target) { bm = 32; bn = 32; }
  }
  launch_tiles(d, p, bm, bn, deterministic ? 1 : heuristic_split(d, bm, bn, sms, false), stream);
}

}  // namespace

int set_autotune(int mode) {
  const int prev = autotune_on() ? 1 : 0;
  if (mode == 0 || mode == 1) g_autotune.store(mode);
  return prev;
}

int64_t autotune_classes() {
  std::shared_lock<std::shared_mutex> g(g_tune_mu);
  return (int64_t)g_tune_table.size();
}

NoTuningScope::NoTuningScope() : prev_(t_no_tuning_runs) { t_no_tuning_runs = true; }
NoTuningScope::~NoTuningScope() { t_no_tuning_runs = prev_; }

Fp64EngineScope::Fp64EngineScope(int engine) : prev_(t_fp64_engine) { t_fp64_engine = engine; }
Fp64EngineScope::~Fp64EngineScope() { t_fp64_engine = prev_; }

void contract(const ContractDesc& d, cudaStream_t stream, bool deterministic) {
  launch_contract<double>(d, stream, deterministic);
}

void contract(const ContractDescF& d, cudaStream_t stream, bool deterministic) {
  launch_contract<float>(d, stream, deterministic);
}

// --------------------------------------------------------------------------------------------
// AMEn contraction recipes
// --------------------------------------------------------------------------------------------

template <typename T>
static void local_product_t(const LocalOpDims& d, const T* phi_l, const T* A, const T* phi_r,
                            const T* x, T* y, T* w1, T* w2, cudaStream_t stream, T alpha, T beta,
                            const SparseCore* sp) {
  // step 1: W[(l,s),(n,R)] = sum_r Phi_l[(l,s), r] X[r, (n,R)]
  {
    ContractDescT<T> c;
    c.M = (int)(d.rl * d.s); c.N = (int)(d.n * d.R); c.K = (int)d.r;
    c.A = phi_l; c.am = Ax::one(d.r); c.ak = Ax::one(1);
    c.B = x; c.bk = Ax::one(d.n * d.R); c.bn = Ax::one(1);
    c.C = w1; c.cm = Ax::one(d.n * d.R); c.cn = Ax::one(1);
    contract(c, stream);
  }
  // step 2 (batched over l): Y2_l[(m,S), R] = sum_{(s,n)} A[s,m,n,S] W_l[(s,n), R]
  if (sp && sp->use) {
    // from the nonzeros: Y2[l,(m,S),R] = sum A[s,m,n,S] W[l,s,n,R]
    const StageDims g{d.rl, d.R, d.s * d.n * d.R, d.m * d.S * d.R, d.R, d.n * d.R, d.R};
    sparse_stage(sp->lp, w1, w2, g, stream);
  } else {
    ContractDescT<T> c;
    c.M = (int)(d.m * d.S); c.N = (int)d.R; c.K = (int)(d.s * d.n); c.batch = (int)d.rl;
    c.A = A; c.am = Ax::two(d.S, d.n * d.S, 1); c.ak = Ax::two(d.n, d.m * d.n * d.S, d.S);
    c.B = w1; c.bk = Ax::one(d.R); c.bn = Ax::one(1); c.b_bs = d.s * d.n * d.R;
    c.C = w2; c.cm = Ax::one(d.R); c.cn = Ax::one(1); c.c_bs = d.m * d.S * d.R;
    contract(c, stream);
  }
  // step 3: y[(l,m), L] = alpha * sum_{(S,R)} Y2[(l,m),(S,R)] Phi_r[L,(S,R)] + beta * y
  {
    ContractDescT<T> c;
    c.M = (int)(d.rl * d.m); c.N = (int)d.RL; c.K = (int)(d.S * d.R);
    c.A = w2; c.am = Ax::one(d.S * d.R); c.ak = Ax::one(1);
    c.B = phi_r; c.bk = Ax::one(1); c.bn = Ax::one(d.S * d.R);
    c.C = y; c.cm = Ax::one(d.RL); c.cn = Ax::one(1);
    c.alpha = alpha; c.beta = beta;
    contract(c, stream);
  }
}

void local_product(const LocalOpDims& d, const double* phi_l, const double* A, const double* phi_r,
                   const double* x, double* y, double* w1, double* w2, cudaStream_t stream,
                   double alpha, double beta, const SparseCore* sp) {
  local_product_t<double>(d, phi_l, A, phi_r, x, y, w1, w2, stream, alpha, beta, sp);
}

void local_product(const LocalOpDims& d, const float* phi_l, const float* A, const float* phi_r,
                   const float* x, float* y, float* w1, float* w2, cudaStream_t stream,
                   float alpha, float beta, const SparseCore* sp) {
  local_product_t<float>(d, phi_l, A, phi_r, x, y, w1, w2, stream, alpha, beta, sp);
}

size_t phi_A_workspace(const PhiDims& d) {
  size_t fwd = size_t(d.s * d.r * d.M * d.L + d.r * d.L * d.N * d.S);
  size_t bck = size_t(d.l * d.M * d.S * d.R + d.l * d.s * d.N * d.R);
  return fwd > bck ? fwd : bck;
}

void phi_fwd_A(const PhiDims& d, const double* phi, const double* left, const double* A,
               const double* right, double* out, double* work, cudaStream_t stream,
               const SparseCore* sp) {
  double* T1 = work;                              // [s, r, M, L]
  double* T2 = work + d.s * d.r * d.M * d.L;      // [r, L, N, S]
  {  // T1[(s,r),(M,L)] = sum_l Phi[l,(s,r)] left[l,(M,L)]
    ContractDesc c;
    c.M = (int)(d.s * d.r); c.N = (int)(d.M * d.L); c.K = (int)d.l;
    c.A = phi; c.am = Ax::one(1); c.ak = Ax::one(d.s * d.r);
    c.B = left; c.bk = Ax::one(d.M * d.L); c.bn = Ax::one(1);
    c.C = T1; c.cm = Ax::one(d.M * d.L); c.cn = Ax::one(1);
    contract(c, stream);
  }
  if (sp && sp->use) {
    // from the nonzeros, into the key-major layout T2'[N,S,r,L]
    const StageDims g{d.r, d.L, d.M * d.L, d.L, d.r * d.L, d.r * d.M * d.L, d.L};
    sparse_stage(sp->fw, T1, T2, g, stream);
    // out[L,S,R] = sum_{(r,N)} T2'[N,S,r,L] right[r,N,R]   (batched over S)
    ContractDesc c;
    c.M = (int)d.L; c.N = (int)d.R; c.K = (int)(d.r * d.N); c.batch = (int)d.S;
    c.A = T2; c.am = Ax::one(1); c.ak = Ax::two(d.N, d.L, d.S * d.r * d.L); c.a_bs = d.r * d.L;
    c.B = right; c.bk = Ax::one(d.R); c.bn = Ax::one(1);
    c.C = out; c.cm = Ax::one(d.S * d.R); c.cn = Ax::one(1); c.c_bs = d.R;
    contract(c, stream);
    return;
  }
  {  // T2[(r,L),(N,S)] = sum_{(s,M)} T1[s,r,M,L] A[s,M,N,S]
    ContractDesc c;
    c.M = (int)(d.r * d.L); c.N = (int)(d.N * d.S); c.K = (int)(d.s * d.M);
    c.A = T1; c.am = Ax::two(d.L, d.M * d.L, 1); c.ak = Ax::two(d.M, d.r * d.M * d.L, d.L);
    c.B = A; c.bk = Ax::two(d.M, d.M * d.N * d.S, d.N * d.S); c.bn = Ax::one(1);
    c.C = T2; c.cm = Ax::one(d.N * d.S); c.cn = Ax::one(1);
    contract(c, stream);
  }
  {  // out[L,S,R] = sum_{(r,N)} T2[r,L,N,S] right[r,N,R]   (batched over S)
    ContractDesc c;
    c.M = (int)d.L; c.N = (int)d.R; c.K = (int)(d.r * d.N); c.batch = (int)d.S;
    c.A = T2; c.am = Ax::one(d.N * d.S); c.ak = Ax::two(d.N, d.L * d.N * d.S, d.S); c.a_bs = 1;
    c.B = right; c.bk = Ax::one(d.R); c.bn = Ax::one(1);
    c.C = out; c.cm = Ax::one(d.S * d.R); c.cn = Ax::one(1); c.c_bs = d.R;
    contract(c, stream);
  }
}

void phi_bck_A(const PhiDims& d, const double* phi, const double* left, const double* A,
               const double* right, double* out, double* work, cudaStream_t stream,
               const SparseCore* sp) {
  double* T1 = work;                              // [l, M, S, R]
  double* T2 = work + d.l * d.M * d.S * d.R;      // [l, s, N, R]
  {  // T1[(l,M),(S,R)] = sum_L left[(l,M), L] Phi[L,(S,R)]
    ContractDesc c;
    c.M = (int)(d.l * d.M); c.N = (int)(d.S * d.R); c.K = (int)d.L;
    c.A = left; c.am = Ax::one(d.L); c.ak = Ax::one(1);
    c.B = phi; c.bk = Ax::one(d.S * d.R); c.bn = Ax::one(1);
    c.C = T1; c.cm = Ax::one(d.S * d.R); c.cn = Ax::one(1);
    contract(c, stream);
  }
  if (sp && sp->use) {   // from the nonzeros: key (s,N), free (l, R)
    const StageDims g{d.l, d.R, d.M * d.S * d.R, d.s * d.N * d.R, d.R, d.S * d.R, d.R};
    sparse_stage(sp->bk, T1, T2, g, stream);
  } else {  // T2[l,s,N,R] = sum_{(M,S)} T1[l,M,S,R] A[s,M,N,S]; rows (l,R), cols (s,N)
    ContractDesc c;
    c.M = (int)(d.l * d.R); c.N = (int)(d.s * d.N); c.K = (int)(d.M * d.S);
    c.A = T1; c.am = Ax::two(d.R, d.M * d.S * d.R, 1); c.ak = Ax::two(d.S, d.S * d.R, d.R);
    c.B = A; c.bk = Ax::two(d.S, d.N * d.S, 1); c.bn = Ax::two(d.N, d.M * d.N * d.S, d.S);
    c.C = T2; c.cm = Ax::two(d.R, d.s * d.N * d.R, 1); c.cn = Ax::two(d.N, d.N * d.R, d.R);
    contract(c, stream);
  }
  {  // out[(l,s), r] = sum_{(N,R)} T2[(l,s),(N,R)] right[r,(N,R)]
    ContractDesc c;
    c.M = (int)(d.l * d.s); c.N = (int)d.r; c.K = (int)(d.N * d.R);
    c.A = T2; c.am = Ax::one(d.N * d.R); c.ak = Ax::one(1);
    c.B = right; c.bk = Ax::one(1); c.bn = Ax::one(d.N * d.R);
    c.C = out; c.cm = Ax::one(d.r); c.cn = Ax::one(1);
    contract(c, stream);
  }
}

size_t phi_rhs_workspace(const PhiRhsDims& d) {
  size_t f = size_t(d.n * d.B * d.r), b = size_t(d.b * d.n * d.R);
  return f > b ? f : b;
}

void phi_fwd_rhs(const PhiRhsDims& d, const double* phi, const double* core_b, const double* core,
                 double* out, double* work, cudaStream_t stream) {
  {  // T[(n,B), r] = sum_b core_b[b,(n,B)] Phi[b, r]
    ContractDesc c;
    c.M = (int)(d.n * d.B); c.N = (int)d.r; c.K = (int)d.b;
    c.A = core_b; c.am = Ax::one(1); c.ak = Ax::one(d.n * d.B);
    c.B = phi; c.bk = Ax::one(d.r); c.bn = Ax::one(1);
    c.C = work; c.cm = Ax::one(d.r); c.cn = Ax::one(1);
    contract(c, stream);
  }
  {  // out[B, R] = sum_{(r,n)} T[n,B,r] core[r,n,R]
    ContractDesc c;
    c.M = (int)d.B; c.N = (int)d.R; c.K = (int)(d.r * d.n);
    c.A = work; c.am = Ax::one(d.r); c.ak = Ax::two(d.n, 1, d.B * d.r);
    c.B = core; c.bk = Ax::one(d.R); c.bn = Ax::one(1);
    c.C = out; c.cm = Ax::one(d.R); c.cn = Ax::one(1);
    contract(c, stream);
  }
}

void phi_bck_rhs(const PhiRhsDims& d, const double* phi, const double* core_b, const double* core,
                 double* out, double* work, cudaStream_t stream) {
  {  // T[(b,n), R] = sum_B core_b[(b,n), B] Phi[B, R]
    ContractDesc c;
    c.M = (int)(d.b * d.n); c.N = (int)d.R; c.K = (int)d.B;
    c.A = core_b; c.am = Ax::one(d.B); c.ak = Ax::one(1);
    c.B = phi; c.bk = Ax::one(d.R); c.bn = Ax::one(1);
    c.C = work; c.cm = Ax::one(d.R); c.cn = Ax::one(1);
    contract(c, stream);
  }
  {  // out[b, r] = sum_{(n,R)} T[b,(n,R)] core[r,(n,R)]
    ContractDesc c;
    c.M = (int)d.b; c.N = (int)d.r; c.K = (int)(d.n * d.R);
    c.A = work; c.am = Ax::one(d.n * d.R); c.ak = Ax::one(1);
    c.B = core; c.bk = Ax::one(1); c.bn = Ax::one(d.n * d.R);
    c.C = out; c.cm = Ax::one(d.r); c.cn = Ax::one(1);
    contract(c, stream);
  }
}

size_t local_rhs_workspace(int64_t b, int64_t n, int64_t B, int64_t r, int64_t R) {
  (void)B; (void)r;
  return size_t(b * n * R);
}

void local_rhs(int64_t b, int64_t n, int64_t B, int64_t r, int64_t R, const double* phi_l,
               const double* core_b, const double* phi_r, double alpha, double* out, double* work,
               cudaStream_t stream) {
  {  // T[(b,n), R] = sum_B core_b[(b,n),B] Phi_r[B,R]
    ContractDesc c;
    c.M = (int)(b * n); c.N = (int)R; c.K = (int)B;
    c.A = core_b; c.am = Ax::one(B); c.ak = Ax::one(1);
    c.B = phi_r; c.bk = Ax::one(R); c.bn = Ax::one(1);
    c.C = work; c.cm = Ax::one(R); c.cn = Ax::one(1);
    contract(c, stream);
  }
  {  // out[r, (n,R)] = alpha * sum_b Phi_l[b, r] T[b, (n,R)]
    ContractDesc c;
    c.M = (int)r; c.N = (int)(n * R); c.K = (int)b;
    c.A = phi_l; c.am = Ax::one(1); c.ak = Ax::one(r);
    c.B = work; c.bk = Ax::one(n * R); c.bn = Ax::one(1);
    c.C = out; c.cm = Ax::one(n * R); c.cn = Ax::one(1);
    c.alpha = alpha;
    contract(c, stream);
  }
}

}  // namespace ttgb
