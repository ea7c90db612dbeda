// Shared definitions of the GB300 AMEn library: error handling, stream-ordered device buffers and
// small launch helpers. Everything here is internal; the public surface is include/ttgb300.h.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace ttgb {

// Status codes returned through the C-ABI (mirrored in include/ttgb300.h).
enum Status : int {
  kOk = 0,
  kInvalidArgument = 1,   // bad shapes / ranks / null pointers (reference: torchtt/errors.py)
  kCudaError = 2,         // a CUDA runtime call failed
  kNumericalError = 3,    // NaN/Inf or a breakdown the solver could not recover from
  kNotConverged = 4,      // informational: nswp sweeps ran without reaching eps
  kOutOfMemory = 5,
  kTimeout = 6,           // a bounded device wait gave up
  kInternal = 7,
};

struct Error : std::runtime_error {
  int status;
  Error(int st, const std::string& msg) : std::runtime_error(msg), status(st) {}
};

[[noreturn]] inline void throw_cuda(cudaError_t e, const char* what, const char* file, int line) {
  char buf[512];
  std::snprintf(buf, sizeof(buf), "CUDA error %d (%s) in %s at %s:%d", (int)e, cudaGetErrorString(e),
                what, file, line);
  throw Error(e == cudaErrorMemoryAllocation ? kOutOfMemory : kCudaError, buf);
}

#define TTGB_CUDA(x)                                                  \
  do {                                                                \
    cudaError_t e_ = (x);                                             \
    if (e_ != cudaSuccess) ::ttgb::throw_cuda(e_, #x, __FILE__, __LINE__); \
  } while (0)

// Every kernel launch of the library is followed by TTGB_CHECK_LAUNCH(), which also counts it.
int64_t launch_count();
// measured FMA-pipe peak in TFLOP/s (0: FP64, 1: FP32), see calibrate.cu
double calibrate_fma(int dtype);
void count_launch();
#define TTGB_CHECK_LAUNCH()                 \
  do {                                      \
    ::ttgb::count_launch();                 \
    TTGB_CUDA(cudaGetLastError());          \
  } while (0)

#define TTGB_REQUIRE(cond, msg)                                        \
  do {                                                                 \
    if (!(cond)) throw ::ttgb::Error(::ttgb::kInvalidArgument, (msg)); \
  } while (0)

inline int num_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 152;
  }
  return sms;
}

inline unsigned cdiv(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

// Raises a kernel's dynamic shared-memory limit to `bytes` on the current device, calling the
// runtime only when the cached limit for that (kernel, device) is lower.
void smem_optin(const void* kernel, int bytes);

// A stream-ordered device buffer (cudaMallocAsync / cudaFreeAsync from the device's default
// memory pool, whose release threshold the solver raises so that freed blocks are reused).
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;

  DevBuf() = default;
  DevBuf(size_t count, cudaStream_t stream) { reset(count, stream); }
  ~DevBuf() { release(); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n), s(o.s) { o.p = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p; n = o.n; s = o.s;
      o.p = nullptr; o.n = 0;
    }
    return *this;
  }
  void reset(size_t count, cudaStream_t stream) {
    release();
    s = stream;
    n = count;
    if (count) TTGB_CUDA(cudaMallocAsync((void**)&p, count * sizeof(T), stream));
  }
  // grow-only reuse: keeps the allocation when it is already large enough
  void ensure(size_t count, cudaStream_t stream) {
    if (count > n || p == nullptr) reset(count < 16 ? 16 : count, stream);
  }
  void release() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    n = 0;
  }
  T* get() const { return p; }
};
using DBuf = DevBuf<double>;
using FBuf = DevBuf<float>;

// A dense tensor in device memory: buffer plus its dims (row-major, last dim fastest).
struct DTensor {
  DBuf buf;
  std::vector<int64_t> dims;
  DTensor() = default;
  DTensor(std::vector<int64_t> d, cudaStream_t s) : dims(std::move(d)) { buf.reset(numel(), s); }
  int64_t numel() const {
    int64_t n = 1;
    for (auto v : dims) n *= v;
    return n;
  }
  double* data() const { return buf.p; }
  int64_t dim(int i) const { return dims[i]; }
};

}  // namespace ttgb
