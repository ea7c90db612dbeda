// tcgen05 3xTF32 GEMM fed by TMA (see tc_gemm.cuh). Hand-written PTX: cp.async.bulk.tensor (TMA)
// loads into 128-byte-swizzled shared memory with mbarrier transaction counts, tcgen05.alloc /
// mma / commit / ld / dealloc, and bounded mbarrier waits.
//
// One CTA computes one 128 x BN output tile with three warp roles:
//   warp 0  producer: one thread streams the K chunks (32 TF32 = one 128-byte swizzle row) of the
//           four operand tiles (A hi/lo, B hi/lo) through a ring of shared-memory stages, each
//           stage one TMA load per operand completing on the stage's "full" barrier;
//   warp 1  MMA issuer: one thread waits for a full stage, issues the 3 x (32 / 8) tcgen05.mma of
//           the chunk (hi*hi, hi*lo, lo*hi) into the tensor-memory accumulator, and commits them to
//           the stage's "empty" barrier so the producer refills it as soon as the tensor core has
//           read it; after the last chunk it commits to the "accumulator full" barrier;
//   warps 2-5 epilogue: wait for the accumulator, read it with tcgen05.ld (warp w reads TMEM lanes
//           32 (w % 4) .. +31, the rows its lanes own) and write the tile with arbitrary output
//           strides as FP32, FP64 or a new TF32 split.
// Copies, tensor-core work and the other CTAs' epilogues overlap with no block-wide barrier in the
// K loop. Every wait is bounded: a wait that gives up sets the error flag, the CTA stops issuing,
// drains (again bounded) the copies and MMAs it has in flight, frees its tensor memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "tc_gemm.cuh"

namespace ttgb {

namespace {

constexpr int kBM = 128;        // rows per tile (MMA M)
constexpr int kBK = 32;         // TF32 elements per K chunk = one 128-byte swizzle row
constexpr int kThreads = 192;   // 6 warps: producer, MMA, 4 epilogue
constexpr int kMaxStages = 6;
constexpr int kWaitIters = 1 << 22;
constexpr int kStageBudget = 200 * 1024;   // shared memory for the operand ring

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor (tcgen05): K-major, 128-byte swizzle, 8-row groups 1024 B apart
// (the layout a TMA load with CU_TENSOR_MAP_SWIZZLE_128B writes for a box of 128-byte rows).
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

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

// TMA tile load of a 3-D tensor map (K, rows, batch) into shared memory, completing on `bar`
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            int z, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

__device__ __forceinline__ int64_t tc_off(const TcAx& a, int i) {
  const int i1 = i / a.e0;
  const int i0 = i - i1 * a.e0;
  return (int64_t)i1 * a.s1 + (int64_t)i0 * a.s0;
}

struct TmaParams {
  CUtensorMap a_hi, a_lo, b_hi, b_lo;   // 64-byte aligned inside the kernel parameters
  int M, N, K, stages;
  int a_batched, b_batched;             // 0: the operand is shared by every batch entry
  int out;
  float alpha;
  float* C32;
  double* C64;
  float* C_hi;
  float* C_lo;
  TcAx cm, cn;
  int64_t c_bs;
  const int* gate;   // when non-zero at launch time every CTA returns before any set-up
};

template <int BN>
__global__ void __launch_bounds__(kThreads, 1) tc_gemm_tma_kernel(const __grid_constant__ TmaParams P,
                                                                  int* err) {
  extern __shared__ uint8_t smraw[];
  // a gated launch (a GMRES iteration queued past its stopping point) leaves before any barrier,
  // allocation or copy; the flag is set by an earlier kernel on this stream, so every thread of
  // every CTA reads the same value
  if (P.gate != nullptr && *P.gate != 0) return;
  uint8_t* ring = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  constexpr int kABytes = kBM * 128;   // one 128-row operand tile of a chunk (hi or lo)
  constexpr int kBBytes = BN * 128;
  constexpr int kStageBytes = 2 * kABytes + 2 * kBBytes;
  constexpr uint32_t kCols = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));
  __shared__ __align__(8) uint64_t full[kMaxStages], empty[kMaxStages], accf;
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh, issued_sh, consumed_sh;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int bz = blockIdx.z, m0 = blockIdx.y * kBM, n0 = blockIdx.x * BN;
  const int stages = P.stages;
  const int nk = (P.K + kBK - 1) / kBK;

  if (tid == 0) {
    for (int s = 0; s < stages; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[s])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[s])));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&accf)));
    asm volatile("fence.mbarrier_init.release.cluster;");
    abort_sh = 0;
    issued_sh = 0;
    consumed_sh = 0;
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_sh)),
                 "n"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_sh;

  if (warp == 0) {
    if (lane == 0) {   // ---- producer -------------------------------------------------------
      const int za = P.a_batched ? bz : 0, zb = P.b_batched ? bz : 0;
      for (int kc = 0; kc < nk; ++kc) {
        const int s = kc % stages;
        const uint32_t round = (uint32_t)(kc / stages);
        if (!mbar_wait(smem_u32(&empty[s]), (round & 1u) ^ 1u)) {
          atomicExch(&abort_sh, 1);
          break;
        }
        if (*(volatile int*)&abort_sh) break;
        uint8_t* st = ring + (size_t)s * kStageBytes;
        const uint32_t fb = smem_u32(&full[s]);
        mbar_expect_tx(fb, (uint32_t)kStageBytes);
        const int k0 = kc * kBK;
        tma_load_3d(smem_u32(st), &P.a_hi, k0, m0, za, fb);
        tma_load_3d(smem_u32(st + kABytes), &P.a_lo, k0, m0, za, fb);
        tma_load_3d(smem_u32(st + 2 * kABytes), &P.b_hi, k0, n0, zb, fb);
        tma_load_3d(smem_u32(st + 2 * kABytes + kBBytes), &P.b_lo, k0, n0, zb, fb);
        *(volatile int*)&issued_sh = kc + 1;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {   // ---- MMA issuer -----------------------------------------------------
      const uint32_t idesc = idesc_tf32(BN);
      for (int kc = 0; kc < nk; ++kc) {
        const int s = kc % stages;
        const uint32_t round = (uint32_t)(kc / stages);
        if (!mbar_wait(smem_u32(&full[s]), round & 1u)) {
          atomicExch(&abort_sh, 1);
          break;
        }
        *(volatile int*)&consumed_sh = kc + 1;
        if (*(volatile int*)&abort_sh) break;
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint8_t* st = ring + (size_t)s * kStageBytes;
        const uint32_t ah = smem_u32(st), al = smem_u32(st + kABytes);
        const uint32_t bh = smem_u32(st + 2 * kABytes), bl = smem_u32(st + 2 * kABytes + kBBytes);
#pragma unroll
        for (int kk = 0; kk < kBK / 8; ++kk) {   // K = 8 TF32 (32 bytes) per instruction
          const uint32_t o = kk * 32;
          mma_tf32(tmem, desc_sw128(ah + o), desc_sw128(bh + o), idesc, (kc | kk) != 0 ? 1u : 0u);
          mma_tf32(tmem, desc_sw128(ah + o), desc_sw128(bl + o), idesc, 1u);
          mma_tf32(tmem, desc_sw128(al + o), desc_sw128(bh + o), idesc, 1u);
        }
        // the stage is free once the tensor core has read it
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(&empty[s]))
                     : "memory");
      }
      // every MMA issued so far (none when aborted early) completes before this arrives
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&accf))
                   : "memory");
    }
  } else {   // ---- epilogue (warps 2-5) -------------------------------------------------------
    // warp-uniform outcome: the tcgen05.ld below is .sync.aligned
    const bool ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&accf), 0u) ? 1 : 0) != 0;
    if (!ok && lane == 0) atomicExch(&abort_sh, 1);
    asm volatile("tcgen05.fence::after_thread_sync;");
    const int q = warp & 3;   // TMEM lane quarter this warp may access
    const int row = m0 + q * 32 + lane;
    const bool row_ok = ok && row < P.M && !*(volatile int*)&abort_sh;
    const int64_t roff = row_ok ? (int64_t)bz * P.c_bs + tc_off(P.cm, row) : 0;
#pragma unroll 1
    for (int c0 = 0; c0 < BN && ok; c0 += 16) {
      uint32_t v[16];
      const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0;
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
          if (col >= P.N) break;
          const float x = __uint_as_float(v[j]) * P.alpha;
          const int64_t o = roff + tc_off(P.cn, col);
          if (P.out == kTcOutF32) {
            P.C32[o] = x;
          } else if (P.out == kTcOutF64) {
            P.C64[o] = (double)x;
          } else {
            const float h = to_tf32(x);
            P.C_hi[o] = h;
            P.C_lo[o] = to_tf32(x - h);
          }
        }
      }
    }
  }

  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (abort_sh && tid == 0) {
    atomicExch(err, 1);
    // drain: TMA loads issued but not consumed, then the MMAs (bounded waits)
    const int issued = issued_sh;
    for (int kc = consumed_sh; kc < issued; ++kc)
      mbar_wait(smem_u32(&full[kc % stages]), (uint32_t)((kc / stages) & 1));
    mbar_wait(smem_u32(&accf), 0u);
  }
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(kCols));
  }
}

__global__ void split_tf32_kernel(const double* __restrict__ x, Gather4 g, int64_t inner,
                                  int64_t out_ld, float* hi, float* lo) {
  const int64_t total = g.e0 * g.e1 * g.e2 * g.e3;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i0 = i % g.e0, t = i / g.e0;
    const int64_t i1 = t % g.e1, t2 = t / g.e1;
    const int64_t i2 = t2 % g.e2, i3 = t2 / g.e2;
    const float v = (float)x[i3 * g.s3 + i2 * g.s2 + i1 * g.s1 + i0 * g.s0];
    const float h = to_tf32(v);
    const int64_t o = (i / inner) * out_ld + (i % inner);
    hi[o] = h;
    lo[o] = to_tf32(v - h);
  }
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  TTGB_REQUIRE(fn != nullptr, "cuTensorMapEncodeTiled is not available from the driver");
  return fn;
}

// Tensor map of a K-major FP32 operand: element (row, k) of batch entry z at
// base[z * bs + row * ld + k]; box = 32 K-elements (128 bytes, the swizzle row) x box_rows rows.
// K and the rows are the true extents: the copy fills zeros past them.
void make_map(CUtensorMap* map, const float* base, int64_t K, int64_t rows, int64_t batch,
              int64_t ld, int64_t bs, int box_rows) {
  TTGB_REQUIRE(aligned16(base) && ld % 4 == 0 && (batch == 1 || bs % 4 == 0),
               "tc_gemm: operands need 16-byte aligned rows (leading dimension a multiple of 4)");
  TTGB_REQUIRE(ld >= K && K >= 1 && rows >= 1, "tc_gemm: bad operand extents");
  const cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)batch};
  const cuuint64_t strides[2] = {(cuuint64_t)ld * 4, (cuuint64_t)(batch == 1 ? rows * ld : bs) * 4};
  const cuuint32_t box[3] = {(cuuint32_t)kBK, (cuuint32_t)box_rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = encode_fn()(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims,
                                 strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                 CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  TTGB_REQUIRE(r == CUDA_SUCCESS, "tc_gemm: cuTensorMapEncodeTiled rejected an operand");
}

template <int BN>
void launch(const TcGemm& g, int* err, cudaStream_t s) {
  TmaParams P;
  const int64_t a_rows = g.M, b_rows = g.N;
  const bool a_b = g.batch > 1 && g.a_bs != 0, b_b = g.batch > 1 && g.b_bs != 0;
  make_map(&P.a_hi, g.A_hi, g.K, a_rows, a_b ? g.batch : 1, g.lda, g.a_bs, kBM);
  make_map(&P.a_lo, g.A_lo, g.K, a_rows, a_b ? g.batch : 1, g.lda, g.a_bs, kBM);
  make_map(&P.b_hi, g.B_hi, g.K, b_rows, b_b ? g.batch : 1, g.ldb, g.b_bs, BN);
  make_map(&P.b_lo, g.B_lo, g.K, b_rows, b_b ? g.batch : 1, g.ldb, g.b_bs, BN);
  P.M = g.M; P.N = g.N; P.K = g.K;
  P.a_batched = a_b ? 1 : 0;
  P.b_batched = b_b ? 1 : 0;
  P.out = g.out; P.alpha = g.alpha;
  P.gate = g.gate;
  P.C32 = g.C32; P.C64 = g.C64; P.C_hi = g.C_hi; P.C_lo = g.C_lo;
  P.cm = g.cm; P.cn = g.cn; P.c_bs = g.c_bs;
  constexpr int kStageBytes = 2 * kBM * 128 + 2 * BN * 128;
  const int nk = (g.K + kBK - 1) / kBK;
  int stages = kStageBudget / kStageBytes;
  if (stages > kMaxStages) stages = kMaxStages;
  if (stages > nk) stages = nk;
  if (stages < 1) stages = 1;
  P.stages = stages;
  const size_t smem = (size_t)stages * kStageBytes + 1024;
  dim3 grid(cdiv(g.N, BN), cdiv(g.M, kBM), (unsigned)g.batch);
  TTGB_REQUIRE(grid.y < 65536 && grid.z < 65536, "tc_gemm grid too large");
  smem_optin((const void*)tc_gemm_tma_kernel<BN>, (int)smem);
  tc_gemm_tma_kernel<BN><<<grid, kThreads, smem, s>>>(P, err);
  TTGB_CHECK_LAUNCH();
}

}  // namespace

void tc_gemm(const TcGemm& g, int* err, cudaStream_t s) {
  if (g.M <= 0 || g.N <= 0 || g.batch <= 0) return;
  TTGB_REQUIRE(g.K > 0, "tc_gemm: empty K");
  if (g.N <= 32) launch<32>(g, err, s);
  else if (g.N <= 64) launch<64>(g, err, s);
  else launch<128>(g, err, s);
}

void split_tf32(const double* x, const Gather4& g, float* hi, float* lo, cudaStream_t s,
                int64_t inner, int64_t out_ld) {
  const int64_t total = g.e0 * g.e1 * g.e2 * g.e3;
  if (total <= 0) return;
  if (inner <= 0) inner = total;
  if (out_ld <= 0) out_ld = inner;
  unsigned grid = cdiv(total, 256);
  const unsigned cap = 8 * (unsigned)num_sms();
  if (grid > cap) grid = cap;
  split_tf32_kernel<<<grid, 256, 0, s>>>(x, g, inner, out_ld, hi, lo);
  TTGB_CHECK_LAUNCH();
}

bool tc_available() {
  int dev = 0, major = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess) return false;
  return major == 10;
}

}  // namespace ttgb
