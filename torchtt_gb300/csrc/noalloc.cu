// ttgb_local_product_noalloc: the local AMEn product with its scratch in a fixed device array.
//
// Some callers must not allocate device memory while they run. One example is a serving loop that
// reserved its HBM up front and admits solves by footprint: a cudaMalloc there can fail, or take
// memory that a resident solve was promised. Another is code running inside another framework
// whose memory manager owns every device allocation. cudaMalloc may also synchronise the device,
// which latency-bound callers avoid. For these callers this entry point computes the same product
// as ttgb_local_product, but it never allocates: the two contraction intermediates live in one
// file-scope __device__ array of kNoAllocScratchDoubles doubles (32 MiB). Every GPU that loads the
// library holds that array until the process exits.
//
// The array is shared by all calls and keeps the last call's contents. Nothing in it needs to
// start at zero: each call overwrites the parts it reads (the first GEMM writes all of the first
// intermediate, the second all of the second). Calls that overlap on the GPU (different streams,
// or different host threads) race on the array and give wrong results; the caller must order them.
// The product is always the dense contraction (the structured A stage of ttgb_local_product,
// which applies sparse A cores from their nonzeros, keeps its index tables in allocated memory).
// The array's device address is looked up once per device and kept for the process: after a
// cudaDeviceReset the cached address is stale, so this entry point does not support device resets.
#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/ttgb300.h"
#include "contract.cuh"

namespace ttgb {
void set_last_error(const std::string& msg);   // capi.cu: the message ttgb_last_error() returns
}

namespace {

constexpr size_t kNoAllocScratchDoubles = size_t(4) << 20;   // 4 Mi doubles = 32 MiB

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kMaxDevices] = {nullptr};

void fail(const char* msg) { ttgb::set_last_error(msg); }

// Device address of the scratch array on the current device. In host code the array's name is only
// a host-side stand-in, so the address is looked up once per device with that device current.
cudaError_t scratch_on_current_device(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (g_noalloc_ptr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" int ttgb_local_product_noalloc(int64_t rl, int64_t s, int64_t r, int64_t m, int64_t n,
                                          int64_t S, int64_t RL, int64_t R, const double* phi_l,
                                          const double* A, const double* phi_r, const double* x,
                                          double* y, int32_t nrhs, void* stream) {
  char msg[256];
  if (!(rl > 0 && s > 0 && r > 0 && m > 0 && n > 0 && S > 0 && RL > 0 && R > 0 && nrhs > 0) ||
      !(phi_l && A && phi_r && x && y)) {
    fail("ttgb_local_product_noalloc: non-positive dimension or null pointer");
    return TTGB_ERR_INVALID;
  }
  const ttgb::LocalOpDims d{rl, s, r, m, n, S, RL, R};
  // scratch sizes rl*s*n*R and rl*m*S*R with overflow checks: a wrapped product could pass the
  // size test below and let the kernels write past the static array
  uint64_t w1 = 0, w2 = 0, wsum = 0;
  const bool wrapped =
      __builtin_mul_overflow((uint64_t)rl, (uint64_t)s, &w1) || __builtin_mul_overflow(w1, (uint64_t)n, &w1) ||
      __builtin_mul_overflow(w1, (uint64_t)R, &w1) || __builtin_mul_overflow((uint64_t)rl, (uint64_t)m, &w2) ||
      __builtin_mul_overflow(w2, (uint64_t)S, &w2) || __builtin_mul_overflow(w2, (uint64_t)R, &w2) ||
      __builtin_add_overflow(w1, w2, &wsum);
  if (wrapped || wsum > kNoAllocScratchDoubles) {
    snprintf(msg, sizeof(msg),
             "ttgb_local_product_noalloc: this product needs %s doubles of scratch "
             "(rl*s*n*R + rl*m*S*R), more than the %zu (32 MiB) the entry point holds; "
             "use ttgb_local_product", wrapped ? "more than 2^64" : std::to_string(wsum).c_str(),
             kNoAllocScratchDoubles);
    fail(msg);
    return TTGB_ERR_INVALID;
  }
  double* base = nullptr;
  cudaError_t e = scratch_on_current_device(&base);
  if (e != cudaSuccess) {
    snprintf(msg, sizeof(msg), "ttgb_local_product_noalloc: cudaGetSymbolAddress failed: %s",
             cudaGetErrorString(e));
    fail(msg);
    return TTGB_ERR_CUDA;
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  try {
    // no tile-tuning runs here: they time candidates with events and synchronise the host
    ttgb::NoTuningScope no_tuning;
    for (int32_t i = 0; i < nrhs; ++i)
      ttgb::local_product(d, phi_l, A, phi_r, x + (int64_t)i * r * n * R,
                          y + (int64_t)i * rl * m * RL, base, base + w1, st);
  } catch (const ttgb::Error& err) {
    snprintf(msg, sizeof(msg), "ttgb_local_product_noalloc: %s", err.what());
    fail(msg);
    return err.status;
  } catch (const std::exception& err) {
    snprintf(msg, sizeof(msg), "ttgb_local_product_noalloc: %s", err.what());
    fail(msg);
    return TTGB_ERR_INTERNAL;
  } catch (...) {
    fail("ttgb_local_product_noalloc: unknown error");
    return TTGB_ERR_INTERNAL;
  }
  return TTGB_OK;
}
