// tcgen05 3xTF32 GEMM (see tc_gemm.cuh). Hand-written PTX: tcgen05.alloc / mma / commit / ld /
// dealloc, mbarrier completion tracking with bounded waits, 128-byte swizzled K-major operands.
#include <atomic>

#include "tc_gemm.cuh"

namespace ttgb {

namespace {

constexpr int kBM = 128;       // rows per tile (MMA M)
constexpr int kBK = 32;        // TF32 elements per K chunk = one 128-byte swizzle row
constexpr int kThreads = 128;  // four warps: one TMEM lane quarter each in the epilogue
constexpr int kWaitIters = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor (tcgen05): K-major, 128-byte swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4)        // start address >> 4
         | ((uint64_t)0 << 16)                      // leading byte offset (unused for swizzled K-major)
         | ((uint64_t)(1024 >> 4) << 32)            // stride byte offset: 8 rows x 128 B
         | ((uint64_t)1 << 46)                      // descriptor version
         | ((uint64_t)2 << 61);                     // 128-byte swizzle
}

// Instruction descriptor: kind::tf32, D = F32, A = B = TF32, both K-major, M = 128, N = n.
__device__ __forceinline__ uint32_t idesc_tf32(int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int i = 0; i < kWaitIters; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ int64_t tc_off(const TcAx& a, int i) {
  const int i1 = i / a.e0;
  const int i0 = i - i1 * a.e0;
  return (int64_t)i1 * a.s1 + (int64_t)i0 * a.s0;
}

// Asynchronous copies global -> shared (cp.async): the issuing thread does not wait, so every
// element of a K chunk is in flight at once; a source size below the copy size zero-fills.
__device__ __forceinline__ void cp_async4(uint32_t dst, const float* src, int bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async16(uint32_t dst, const float* src, int bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(bytes)
               : "memory");
}

// Stage rows [row0, row0 + rows) x K chunk [k0, k0 + 32) of a K-major matrix into the 128-byte
// swizzled tile (16-byte granule c of row r at granule c ^ (r & 7)). VEC: 16-byte copies (rows
// and the matrix 16-byte aligned); otherwise 4-byte copies.
template <bool VEC>
__device__ __forceinline__ void stage_async(const float* __restrict__ src, int64_t ld,
                                            int nrows_valid, int row0, int rows, int K, int k0,
                                            float* dst) {
  if constexpr (VEC) {
    for (int c = threadIdx.x; c < rows * 8; c += kThreads) {
      const int r = c >> 3, ch = c & 7;
      const int gr = row0 + r, k = k0 + ch * 4;
      int bytes = 0;
      const float* p = src;
      if (gr < nrows_valid && k < K) {
        bytes = (K - k >= 4 ? 4 : K - k) * 4;
        p = src + (int64_t)gr * ld + k;
      }
      cp_async16(smem_u32(dst + r * kBK + ((ch ^ (r & 7)) << 2)), p, bytes);
    }
  } else {
    for (int c = threadIdx.x; c < rows * kBK; c += kThreads) {
      const int r = c >> 5, kk = c & 31;
      const int gr = row0 + r, k = k0 + kk;
      const bool ok = gr < nrows_valid && k < K;
      cp_async4(smem_u32(dst + r * kBK + (((kk >> 2) ^ (r & 7)) << 2) + (kk & 3)),
                ok ? src + (int64_t)gr * ld + k : src, ok ? 4 : 0);
    }
  }
}

// K loop with two shared-memory stages: the copies of chunk k+1 are issued before the MMAs of
// chunk k, and a stage is refilled only after the MMAs that read it have committed (mbarrier).
template <int BN, bool VEC>
__global__ void __launch_bounds__(kThreads) tc_gemm_kernel(TcGemm g, int* err) {
  extern __shared__ uint8_t smraw[];
  uint8_t* smbase = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  constexpr int kStage = 2 * kBM * kBK + 2 * BN * kBK;   // floats per stage: A hi/lo, B hi/lo
  float* const stage0 = reinterpret_cast<float*>(smbase);
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh;
  constexpr uint32_t kCols = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int bz = blockIdx.z, m0 = blockIdx.y * kBM, n0 = blockIdx.x * BN;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_sh)),
                 "n"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[1])));
    asm volatile("fence.mbarrier_init.release.cluster;");
    abort_sh = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_sh;
  const uint32_t bar[2] = {smem_u32(&mbar[0]), smem_u32(&mbar[1])};

  const float* Ah = g.A_hi + (int64_t)bz * g.a_bs;
  const float* Al = g.A_lo + (int64_t)bz * g.a_bs;
  const float* Bh = g.B_hi + (int64_t)bz * g.b_bs;
  const float* Bl = g.B_lo + (int64_t)bz * g.b_bs;
  const uint32_t idesc = idesc_tf32(BN);
  const int nk = (g.K + kBK - 1) / kBK;

  auto issue = [&](int kc, int st) {
    const int k0 = kc * kBK;
    float* sAh = stage0 + st * kStage;
    float* sAl = sAh + kBM * kBK;
    float* sBh = sAl + kBM * kBK;
    float* sBl = sBh + BN * kBK;
    stage_async<VEC>(Ah, g.lda, g.M, m0, kBM, g.K, k0, sAh);
    stage_async<VEC>(Al, g.lda, g.M, m0, kBM, g.K, k0, sAl);
    stage_async<VEC>(Bh, g.ldb, g.N, n0, BN, g.K, k0, sBh);
    stage_async<VEC>(Bl, g.ldb, g.N, n0, BN, g.K, k0, sBl);
    asm volatile("cp.async.commit_group;" ::: "memory");
  };

  uint32_t phase[2] = {0u, 0u};
  bool pending[2] = {false, false};   // a commit on this barrier has not been waited for
  bool ok = true;
  issue(0, 0);
  for (int kc = 0; kc < nk; ++kc) {
    const int st = kc & 1;
    if (kc + 1 < nk) {
      if (pending[st ^ 1]) {   // the MMAs of chunk kc-1 read stage st^1: wait before refilling it
        if (!mbar_wait(bar[st ^ 1], phase[st ^ 1])) abort_sh = 1;
        phase[st ^ 1] ^= 1u;
        pending[st ^ 1] = false;
      }
      issue(kc + 1, st ^ 1);
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // copies -> async proxy
    __syncthreads();
    if (abort_sh) { ok = false; break; }
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const float* sAh = stage0 + st * kStage;
      const uint32_t ah = smem_u32(sAh), al = smem_u32(sAh + kBM * kBK);
      const uint32_t bh = smem_u32(sAh + 2 * kBM * kBK), bl = smem_u32(sAh + 2 * kBM * kBK + BN * kBK);
#pragma unroll
      for (int kk = 0; kk < kBK / 8; ++kk) {   // K = 8 TF32 (32 bytes) per instruction
        const uint32_t o = kk * 32;
        mma_tf32(tmem, desc_sw128(ah + o), desc_sw128(bh + o), idesc, (kc | kk) != 0 ? 1u : 0u);
        mma_tf32(tmem, desc_sw128(ah + o), desc_sw128(bl + o), idesc, 1u);
        mma_tf32(tmem, desc_sw128(al + o), desc_sw128(bh + o), idesc, 1u);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar[st])
                   : "memory");
    }
    pending[st] = true;
  }
  if (ok) {   // the last commit covers every MMA issued before it
    const int st = (nk - 1) & 1;
    if (!mbar_wait(bar[st], phase[st])) abort_sh = 1;
    pending[0] = pending[1] = false;
    __syncthreads();
    if (abort_sh) ok = false;
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (ok) {
    const int row = m0 + warp * 32 + lane;
    const bool row_ok = row < g.M;
    const int64_t roff = row_ok ? (int64_t)bz * g.c_bs + tc_off(g.cm, row) : 0;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 16) {
      uint32_t v[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
          "%11, %12, %13, %14, %15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
            "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
            "=r"(v[14]), "=r"(v[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row_ok) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = n0 + c0 + j;
          if (col >= g.N) break;
          const float x = __uint_as_float(v[j]) * g.alpha;
          const int64_t o = roff + tc_off(g.cn, col);
          if (g.out == kTcOutF32) {
            g.C32[o] = x;
          } else if (g.out == kTcOutF64) {
            g.C64[o] = (double)x;
          } else {
            const float h = to_tf32(x);
            g.C_hi[o] = h;
            g.C_lo[o] = to_tf32(x - h);
          }
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(err, 1);
    // give MMAs still in flight a bounded chance to finish before their accumulator is released
    for (int b = 0; b < 2; ++b)
      if (pending[b]) mbar_wait(bar[b], phase[b]);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(kCols));
  }
}

__global__ void split_tf32_kernel(const double* __restrict__ x, Gather4 g, float* hi, float* lo) {
  const int64_t total = g.e0 * g.e1 * g.e2 * g.e3;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i0 = i % g.e0, t = i / g.e0;
    const int64_t i1 = t % g.e1, t2 = t / g.e1;
    const int64_t i2 = t2 % g.e2, i3 = t2 / g.e2;
    const float v = (float)x[i3 * g.s3 + i2 * g.s2 + i1 * g.s1 + i0 * g.s0];
    const float h = to_tf32(v);
    hi[i] = h;
    lo[i] = to_tf32(v - h);
  }
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

template <int BN>
void launch(const TcGemm& g, int* err, cudaStream_t s) {
  const size_t smem = (size_t)2 * (2 * kBM * kBK + 2 * BN * kBK) * sizeof(float) + 1024;
  dim3 grid(cdiv(g.N, BN), cdiv(g.M, kBM), (unsigned)g.batch);
  TTGB_REQUIRE(grid.y < 65536 && grid.z < 65536, "tc_gemm grid too large");
  // 16-byte copies when every row of both operands starts on a 16-byte boundary
  const bool vec = aligned16(g.A_hi) && aligned16(g.A_lo) && aligned16(g.B_hi) && aligned16(g.B_lo) &&
                   g.lda % 4 == 0 && g.ldb % 4 == 0 && g.a_bs % 4 == 0 && g.b_bs % 4 == 0;
  if (vec) {
    smem_optin((const void*)tc_gemm_kernel<BN, true>, (int)smem);
    tc_gemm_kernel<BN, true><<<grid, kThreads, smem, s>>>(g, err);
  } else {
    smem_optin((const void*)tc_gemm_kernel<BN, false>, (int)smem);
    tc_gemm_kernel<BN, false><<<grid, kThreads, smem, s>>>(g, err);
  }
  TTGB_CHECK_LAUNCH();
}

}  // namespace

void tc_gemm(const TcGemm& g, int* err, cudaStream_t s) {
  if (g.M <= 0 || g.N <= 0 || g.batch <= 0) return;
  TTGB_REQUIRE(g.K > 0, "tc_gemm: empty K");
  if (g.N <= 32) launch<32>(g, err, s);
  else if (g.N <= 64) launch<64>(g, err, s);
  else if (g.N <= 128) launch<128>(g, err, s);
  else launch<256>(g, err, s);
}

void split_tf32(const double* x, const Gather4& g, float* hi, float* lo, cudaStream_t s) {
  const int64_t total = g.e0 * g.e1 * g.e2 * g.e3;
  if (total <= 0) return;
  unsigned grid = cdiv(total, 256);
  const unsigned cap = 8 * (unsigned)num_sms();
  if (grid > cap) grid = cap;
  split_tf32_kernel<<<grid, 256, 0, s>>>(x, g, hi, lo);
  TTGB_CHECK_LAUNCH();
}

bool tc_available() {
  int dev = 0, major = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess) return false;
  return major == 10;
}

}  // namespace ttgb
