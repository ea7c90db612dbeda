// Request server for batched / served AMEn solves (declared in include/ttgb300.h).
//
// `slots` host worker threads each own a non-blocking CUDA stream and run one solve at a time,
// so up to `slots` solves overlap on the GPU. Admission is FIFO and by footprint: the head
// request starts when a worker is free and its footprint fits in what the running requests leave
// of the budget (a request larger than the whole budget runs alone). The footprint is an upper
// bound (footprint_bound: every buffer at the largest rank the solve can reach), so the ranks a
// running solve grows to never take the budget past what admission reserved.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>

#include "../../include/ttgb300.h"
#include "amen.cuh"
#include "solution.cuh"

using namespace ttgb;


namespace ttgb {
void set_last_error(const std::string& msg);
}

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t id = 0;
  TTView A, b, x0;
  AmenParams p;
  size_t footprint = 0;
  Clock::time_point t_submit, t_start, t_end;
  bool done = false;
  int status = TTGB_OK;
  std::string error;
  std::unique_ptr<ttgb_solution> sol;
};

TTView copy_view(const ttgb_tt* t, bool matrix) {
  TTView v;
  if (!t || t->d <= 0) return v;
  TTGB_REQUIRE(t->cols && t->ranks && t->cores, "TT descriptor with null arrays");
  v.d = t->d;
  v.cols.assign(t->cols, t->cols + t->d);
  v.ranks.assign(t->ranks, t->ranks + t->d + 1);
  if (matrix) {
    TTGB_REQUIRE(t->rows != nullptr, "A must be TT-matrix and b must be vector.");
    v.rows.assign(t->rows, t->rows + t->d);
  }
  v.cores.assign(t->cores, t->cores + t->d);
  return v;
}

}  // namespace

struct ttgb_server {
  int device = 0;
  int slots = 1;
  size_t budget = 0;
  size_t in_use = 0;
  size_t peak_in_use = 0;
  int running = 0;
  int peak = 0;
  int64_t next_id = 1;
  int64_t submitted = 0, completed = 0;
  bool stopping = false;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Request>> queue;
  std::map<int64_t, std::shared_ptr<Request>> table;
  std::vector<std::thread> workers;

  void worker() {
    cudaSetDevice(device);
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) st = nullptr;
    for (;;) {
      std::shared_ptr<Request> req;
      {
        std::unique_lock<std::mutex> lock(mu);
        cv_work.wait(lock, [&] {
          if (stopping && queue.empty()) return true;
          if (queue.empty()) return false;
          const size_t fp = queue.front()->footprint;
          return running == 0 || in_use + fp <= budget;
        });
        if (queue.empty()) break;
        req = queue.front();
        queue.pop_front();
        in_use += req->footprint;
        peak_in_use = std::max(peak_in_use, in_use);
        ++running;
        peak = std::max(peak, running);
        req->t_start = Clock::now();
      }
      try {
        if (!st) throw Error(kCudaError, "could not create a stream for the worker");
        auto sol = std::make_unique<ttgb_solution>();
        TTView z0;
        sol->res = amen_solve(req->A, req->b, req->x0, z0, req->p, st);
        // the solve synchronised its stream; the result outlives this worker's stream, so its
        // buffers are released on the legacy default stream from now on
        for (auto& c : sol->res.cores) c.buf.s = nullptr;
        req->sol = std::move(sol);
        req->status = TTGB_OK;
      } catch (const Error& e) {
        req->status = e.status;
        req->error = e.what();
      } catch (const std::exception& e) {
        req->status = TTGB_ERR_INTERNAL;
        req->error = e.what();
      }
      {
        std::lock_guard<std::mutex> lock(mu);
        req->t_end = Clock::now();
        req->done = true;
        in_use -= req->footprint;
        --running;
        ++completed;
      }
      cv_done.notify_all();
      cv_work.notify_all();
    }
    if (st) cudaStreamDestroy(st);
  }
};

extern "C" {

int ttgb_server_create(int32_t slots, int64_t mem_budget_bytes, ttgb_server** out) {
  try {
    TTGB_REQUIRE(out && slots >= 1 && slots <= 256, "slots must be in [1, 256]");
    auto* s = new ttgb_server;
    TTGB_CUDA(cudaGetDevice(&s->device));
    s->slots = slots;
    if (mem_budget_bytes <= 0) {
      size_t fr = 0, tot = 0;
      TTGB_CUDA(cudaMemGetInfo(&fr, &tot));
      s->budget = (size_t)(0.8 * (double)fr);
    } else {
      s->budget = (size_t)mem_budget_bytes;
    }
    for (int i = 0; i < slots; ++i) s->workers.emplace_back([s] { s->worker(); });
    *out = s;
    return TTGB_OK;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.status;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return TTGB_ERR_INTERNAL;
  }
}

int ttgb_server_submit(ttgb_server* srv, const ttgb_tt* A, const ttgb_tt* b, const ttgb_tt* x0,
                       const ttgb_amen_params* params, int64_t* id) {
  try {
    TTGB_REQUIRE(srv && A && b && params && id, "null argument");
    auto req = std::make_shared<Request>();
    req->A = copy_view(A, true);
    req->b = copy_view(b, false);
    req->x0 = copy_view(x0, false);
    TTGB_REQUIRE(req->A.d >= 1 && req->A.d == req->b.d, "Dimension mismatch.");
    req->p = params_from_c(params);
    const AmenParams& p = req->p;
    req->footprint = footprint_bound(req->A, req->b, req->x0, p);
    std::lock_guard<std::mutex> lock(srv->mu);
    TTGB_REQUIRE(!srv->stopping, "server is shutting down");
    req->id = srv->next_id++;
    req->t_submit = Clock::now();
    srv->queue.push_back(req);
    srv->table[req->id] = req;
    ++srv->submitted;
    *id = req->id;
    srv->cv_work.notify_one();
    return TTGB_OK;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.status;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return TTGB_ERR_INTERNAL;
  }
}

int ttgb_server_wait(ttgb_server* srv, int64_t id, double timeout_s, ttgb_solution** out,
                     double* queue_ms, double* run_ms) {
  if (!srv) return TTGB_ERR_INVALID;
  std::unique_lock<std::mutex> lock(srv->mu);
  auto it = srv->table.find(id);
  if (it == srv->table.end()) {
    set_last_error("unknown request id");
    return TTGB_ERR_INVALID;
  }
  std::shared_ptr<Request> req = it->second;
  auto pred = [&] { return req->done; };
  if (timeout_s < 0) {
    srv->cv_done.wait(lock, pred);
  } else if (!srv->cv_done.wait_for(lock, std::chrono::duration<double>(timeout_s), pred)) {
    set_last_error("request still running");
    return TTGB_ERR_TIMEOUT;
  }
  srv->table.erase(id);
  if (queue_ms) *queue_ms = std::chrono::duration<double, std::milli>(req->t_start - req->t_submit).count();
  if (run_ms) *run_ms = std::chrono::duration<double, std::milli>(req->t_end - req->t_start).count();
  if (req->status != TTGB_OK) {
    set_last_error(req->error);
    return req->status;
  }
  if (out) *out = req->sol.release();
  return TTGB_OK;
}

int ttgb_server_stats(const ttgb_server* srv, int64_t* submitted, int64_t* completed,
                      int32_t* running, int32_t* peak_running) {
  if (!srv) return TTGB_ERR_INVALID;
  auto* s = const_cast<ttgb_server*>(srv);
  std::lock_guard<std::mutex> lock(s->mu);
  if (submitted) *submitted = s->submitted;
  if (completed) *completed = s->completed;
  if (running) *running = s->running;
  if (peak_running) *peak_running = s->peak;
  return TTGB_OK;
}

int ttgb_server_memory(const ttgb_server* srv, int64_t* budget, int64_t* in_use,
                       int64_t* peak_in_use) {
  if (!srv) return TTGB_ERR_INVALID;
  auto* s = const_cast<ttgb_server*>(srv);
  std::lock_guard<std::mutex> lock(s->mu);
  if (budget) *budget = (int64_t)s->budget;
  if (in_use) *in_use = (int64_t)s->in_use;
  if (peak_in_use) *peak_in_use = (int64_t)s->peak_in_use;
  return TTGB_OK;
}

void ttgb_server_destroy(ttgb_server* srv) {
  if (!srv) return;
  {
    std::lock_guard<std::mutex> lock(srv->mu);
    srv->stopping = true;
  }
  srv->cv_work.notify_all();
  for (auto& t : srv->workers) t.join();
  delete srv;
}

}  // extern "C"
