// Optional CUDA-event timing of the contraction launches of a solve (AmenParams::profile).
// Pairs of events bracket each local product / interface update on the solve's stream; the pool is
// drained (one synchronisation) when full and at the end of the solve.
#pragma once

#include <vector>

#include "common.cuh"

namespace ttgb {

struct Profiler {
  cudaStream_t s = nullptr;
  std::vector<cudaEvent_t> pool;
  std::vector<double> pending_flops;
  std::vector<double> pending_aux;
  std::vector<int> pending_launches;
  size_t used = 0;
  double ms = 0.0;
  int64_t launches = 0;
  double flops = 0.0;   // the first work figure of every bracket (flops or bytes)
  double aux = 0.0;     // an optional second figure

  explicit Profiler(cudaStream_t st, size_t pairs = 2048) : s(st) {
    pool.resize(2 * pairs);
    for (auto& e : pool) TTGB_CUDA(cudaEventCreate(&e));
  }
  ~Profiler() {
    for (auto& e : pool) cudaEventDestroy(e);
  }
  Profiler(const Profiler&) = delete;
  Profiler& operator=(const Profiler&) = delete;

  void begin() {
    if (used + 2 > pool.size()) flush();
    TTGB_CUDA(cudaEventRecord(pool[used], s));
  }
  void end(double f, int nlaunch, double f2 = 0.0) {
    TTGB_CUDA(cudaEventRecord(pool[used + 1], s));
    pending_flops.push_back(f);
    pending_aux.push_back(f2);
    pending_launches.push_back(nlaunch);
    used += 2;
  }
  void flush() {
    if (used == 0) return;
    TTGB_CUDA(cudaEventSynchronize(pool[used - 1]));
    for (size_t i = 0; i < used; i += 2) {
      float t = 0.f;
      TTGB_CUDA(cudaEventElapsedTime(&t, pool[i], pool[i + 1]));
      ms += t;
    }
    for (double f : pending_flops) flops += f;
    for (double f : pending_aux) aux += f;
    for (int l : pending_launches) launches += l;
    pending_flops.clear();
    pending_aux.clear();
    pending_launches.clear();
    used = 0;
  }
};

// Attribution of a solve's stream time to its steps: an event is recorded at every phase change;
// the time between consecutive events (device work plus any idle gap the host leaves) is charged
// to the phase that was active.
struct PhaseTimer {
  static constexpr int kPhases = 12;
  cudaStream_t s = nullptr;
  std::vector<cudaEvent_t> ev;
  std::vector<int> ph;
  double ms[kPhases] = {0};
  int current = -1;

  explicit PhaseTimer(cudaStream_t st) : s(st) {}
  ~PhaseTimer() {
    for (auto& e : ev) cudaEventDestroy(e);
  }
  PhaseTimer(const PhaseTimer&) = delete;
  PhaseTimer& operator=(const PhaseTimer&) = delete;

  void mark(int phase) {
    if (ev.size() >= 8192) flush();
    cudaEvent_t e;
    TTGB_CUDA(cudaEventCreate(&e));
    TTGB_CUDA(cudaEventRecord(e, s));
    ev.push_back(e);
    ph.push_back(phase);
    current = phase;
  }
  void flush() {
    if (ev.empty()) return;
    TTGB_CUDA(cudaEventSynchronize(ev.back()));
    for (size_t i = 0; i + 1 < ev.size(); ++i) {
      float t = 0.f;
      TTGB_CUDA(cudaEventElapsedTime(&t, ev[i], ev[i + 1]));
      if (ph[i] >= 0 && ph[i] < kPhases) ms[ph[i]] += t;
    }
    cudaEvent_t last = ev.back();
    const int lastph = ph.back();
    for (size_t i = 0; i + 1 < ev.size(); ++i) cudaEventDestroy(ev[i]);
    ev.clear();
    ph.clear();
    ev.push_back(last);
    ph.push_back(lastph);
  }
};

}  // namespace ttgb
