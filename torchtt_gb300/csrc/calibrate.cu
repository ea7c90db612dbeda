// Peak rates of this GPU's FP64 and FP32 FMA pipes, measured with independent FMA chains. They
// are the denominators of the CUDA-core contraction rooflines (the FP64 engine of the plain path,
// the FP32 engine of the mixed path); the tensor-pipe and HBM peaks are measured separately.
#include <algorithm>

#include "../../include/ttgb300.h"
#include "common.cuh"

namespace ttgb {

namespace {

constexpr int kChains = 8;

template <typename T>
__global__ void __launch_bounds__(256) fma_chains_kernel(T* out, int iters, T a, T c) {
  T x[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) x[i] = (T)(threadIdx.x + i) * (T)1e-3;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < kChains; ++i) x[i] = fma(x[i], a, c);
  }
  T sum = 0;
#pragma unroll
  for (int i = 0; i < kChains; ++i) sum += x[i];
  if (sum == (T)-1) out[0] = sum;   // never true for these inputs; keeps the chains live
}

template <typename T>
double measure(int iters) {
  const int blocks = 8 * num_sms(), threads = 256;
  cudaStream_t s;
  TTGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  T* out = nullptr;
  cudaEvent_t e0, e1;
  TTGB_CUDA(cudaMallocAsync((void**)&out, sizeof(T), s));
  TTGB_CUDA(cudaEventCreate(&e0));
  TTGB_CUDA(cudaEventCreate(&e1));
  double best = 0.0;
  for (int rep = 0; rep < 4; ++rep) {   // the first repetition is the warm-up
    TTGB_CUDA(cudaEventRecord(e0, s));
    fma_chains_kernel<T><<<blocks, threads, 0, s>>>(out, iters, (T)0.999999, (T)1e-6);
    TTGB_CHECK_LAUNCH();
    TTGB_CUDA(cudaEventRecord(e1, s));
    TTGB_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    TTGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    const double flops = 2.0 * kChains * (double)iters * blocks * threads;
    if (rep > 0 && ms > 0.f) best = std::max(best, flops / (ms * 1e-3) / 1e12);
  }
  cudaFreeAsync(out, s);
  cudaStreamSynchronize(s);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  return best;
}

}  // namespace

double calibrate_fma(int dtype) {
  // about 50 ms per launch at the expected rates (1.2 TF/s FP64, 69 TF/s FP32)
  return dtype == 0 ? measure<double>(12000) : measure<float>(700000);
}

}  // namespace ttgb
