// extern "C" surface of the library (declared in include/ttgb300.h). Every entry point converts
// exceptions into status codes and keeps the message in a thread-local buffer.
#include <cstring>
#include <memory>
#include <string>

#include "../../include/ttgb300.h"
#include "amen.cuh"
#include "solution.cuh"
#include "blas1.cuh"
#include "contract.cuh"
#include "gmres.cuh"
#include "linalg.cuh"
#include "prec.cuh"
#include "tc_gemm.cuh"
#include "tc_local.cuh"
#include "tt_ops.cuh"
#include "dmrg.cuh"
#include "amen_mv.cuh"

using namespace ttgb;


namespace {

thread_local std::string g_last_error;

template <typename F>
int guarded(F&& f) {
  try {
    f();
    return TTGB_OK;
  } catch (const Error& e) {
    g_last_error = e.what();
    return e.status;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return TTGB_ERR_INTERNAL;
  } catch (...) {
    g_last_error = "unknown error";
    return TTGB_ERR_INTERNAL;
  }
}

TTView view_of(const ttgb_tt* t, bool matrix) {
  TTView v;
  if (!t || t->d <= 0) return v;
  TTGB_REQUIRE(t->cols && t->ranks && t->cores, "TT descriptor with null arrays");
  v.d = t->d;
  v.cols.assign(t->cols, t->cols + t->d);
  v.ranks.assign(t->ranks, t->ranks + t->d + 1);
  if (matrix) {
    TTGB_REQUIRE(t->rows != nullptr, "A must be TT-matrix and b must be vector.");
    v.rows.assign(t->rows, t->rows + t->d);
  } else {
    TTGB_REQUIRE(t->rows == nullptr, "A must be TT-matrix and b must be vector.");
  }
  v.cores.assign(t->cores, t->cores + t->d);
  for (int k = 0; k < t->d; ++k) {
    TTGB_REQUIRE(v.ranks[k] >= 1 && v.cols[k] >= 1, "Check the ranks and the mode size.");
    TTGB_REQUIRE(v.cores[k] != nullptr, "null core pointer");
  }
  TTGB_REQUIRE(v.ranks[t->d] >= 1, "Check the ranks and the mode size.");
  return v;
}

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

struct Scratch {   // per-call workspace of the kernel-level entry points
  cudaStream_t s;
  DBuf partial;
  unsigned* counter = nullptr;
  RedWS red;
  LinalgWS lws;
  char* hbuf = nullptr;
  explicit Scratch(cudaStream_t st) : s(st) {
    partial.reset(1024 * 128, s);
    TTGB_CUDA(cudaMallocAsync((void**)&counter, 64, s));
    TTGB_CUDA(cudaMemsetAsync(counter, 0, 64, s));
    red.partial = partial.p;
    red.counter = counter;
    red.cap_blocks = 1024;
    red.cap_vec = 127;
    TTGB_CUDA(cudaMallocAsync((void**)&lws.status, 16, s));
    TTGB_CUDA(cudaMemsetAsync(lws.status, 0, 16, s));
    hbuf = pinned_scratch();
    lws.h_status = (int*)hbuf;
  }
  ~Scratch() {
    cudaStreamSynchronize(s);
    if (counter) cudaFreeAsync(counter, s);
    if (lws.status) cudaFreeAsync(lws.status, s);
  }
  // one small pinned host buffer per host thread, kept for the thread's lifetime
  static char* pinned_scratch() {
    struct Holder {
      char* p = nullptr;
      ~Holder() { if (p) cudaFreeHost(p); }
    };
    static thread_local Holder h;
    if (!h.p) TTGB_CUDA(cudaMallocHost((void**)&h.p, 256));
    return h.p;
  }
};

}  // namespace

namespace ttgb {
void set_last_error(const std::string& msg) { g_last_error = msg; }

AmenParams params_from_c(const ttgb_amen_params* params) {
  TTGB_REQUIRE(params != nullptr, "null parameters");
  AmenParams p;
  p.nswp = params->nswp;
  p.eps = params->eps;
  p.rmax = params->rmax;
  p.max_full = params->max_full;
  p.kickrank = params->kickrank;
  p.kick2 = params->kick2;
  p.local_iterations = params->local_iterations;
  p.resets = params->resets;
  p.verbose = params->verbose;
  p.prec = params->preconditioner;
  p.seed = params->seed;
  p.profile = params->profile;
  TTGB_REQUIRE(params->precision == TTGB_PRECISION_FP64 || params->precision == TTGB_PRECISION_MIXED,
               "invalid precision mode");
  p.precision = params->precision;
  TTGB_REQUIRE(params->lowp_engine >= 0 && params->lowp_engine <= 2, "invalid low-precision engine");
  p.lowp_engine = params->lowp_engine;
  TTGB_REQUIRE(params->a_structure == 0 || params->a_structure == 1, "invalid a_structure");
  p.a_structure = params->a_structure;
  TTGB_REQUIRE(params->fp64_engine >= 0 && params->fp64_engine <= 2, "invalid fp64_engine");
  p.fp64_engine = params->fp64_engine;
  TTGB_REQUIRE(params->strict_eps == 0 || params->strict_eps == 1, "invalid strict_eps");
  p.strict_eps = params->strict_eps;
  return p;
}
}  // namespace ttgb

extern "C" {

void ttgb_default_params(ttgb_amen_params* p) {
  if (!p) return;
  p->nswp = 22;
  p->eps = 1e-10;
  p->rmax = 32768;
  p->max_full = 500;
  p->kickrank = 4;
  p->kick2 = 0;
  p->local_iterations = 40;
  p->resets = 2;
  p->verbose = 0;
  p->preconditioner = TTGB_PREC_NONE;
  p->seed = 1;
  p->profile = 0;
  p->precision = TTGB_PRECISION_FP64;
  p->lowp_engine = 0;
  p->a_structure = 1;
  p->fp64_engine = 0;
  p->strict_eps = 0;
}

int ttgb_amen_solve(const ttgb_tt* A, const ttgb_tt* b, const ttgb_tt* x0, const ttgb_tt* z0,
                    const ttgb_amen_params* params, void* stream, ttgb_solution** out) {
  return guarded([&] {
    TTGB_REQUIRE(A && b && params && out, "A, b, params and out must not be NULL");
    TTView Av = view_of(A, true), bv = view_of(b, false);
    TTView xv = view_of(x0, false), zv = view_of(z0, false);
    const AmenParams p = params_from_c(params);
    auto* sol = new ttgb_solution;
    try {
      sol->res = amen_solve(Av, bv, xv, zv, p, as_stream(stream));
    } catch (...) {
      delete sol;
      throw;
    }
    *out = sol;
  });
}

int ttgb_solution_dims(const ttgb_solution* sol, int32_t* d, int64_t* ranks) {
  return guarded([&] {
    TTGB_REQUIRE(sol != nullptr, "null solution");
    if (d) *d = (int32_t)sol->res.cores.size();
    if (ranks)
      for (size_t i = 0; i < sol->res.ranks.size(); ++i) ranks[i] = sol->res.ranks[i];
  });
}

int ttgb_solution_stats(const ttgb_solution* sol, ttgb_stats* st) {
  return guarded([&] {
    TTGB_REQUIRE(sol && st, "null argument");
    const AmenStats& a = sol->res.stats;
    st->sweeps = a.sweeps;
    st->converged = a.converged;
    st->max_res = a.max_res;
    st->local_solves = a.local_solves;
    st->direct_solves = a.direct_solves;
    st->gmres_iterations = a.gmres_iterations;
    st->matvecs = a.matvecs;
    st->matvec_flops = a.matvec_flops;
    st->phi_flops = a.phi_flops;
    st->other_flops = a.other_flops;
    st->host_syncs = a.host_syncs;
    st->contract_ms = a.contract_ms;
    st->contract_launches = a.contract_launches;
    st->contract_flops = a.contract_flops;
    st->lowp_matvecs = a.lowp_matvecs;
    st->lowp_flops = a.lowp_flops;
    st->refinements = a.refinements;
    for (int i = 0; i < 12; ++i) st->phase_ms[i] = a.phase_ms[i];
    st->lowp_ms = a.lowp_ms;
    st->lowp_launches = a.lowp_launches;
    st->lowp_gemm_flops = a.lowp_gemm_flops;
    st->krylov_ms = a.krylov_ms;
    st->krylov_launches = a.krylov_launches;
    st->krylov_bytes = a.krylov_bytes;
    st->krylov_traffic_bytes = a.krylov_traffic_bytes;
    st->gmres_syncs = a.gmres_syncs;
    st->gmres_overrun = a.gmres_overrun;
    st->gmres_reorth = a.gmres_reorth;
  });
}

const double* ttgb_solution_core(const ttgb_solution* sol, int32_t k) {
  if (!sol || k < 0 || k >= (int32_t)sol->res.cores.size()) return nullptr;
  return sol->res.cores[k].data();
}

int ttgb_solution_copy_core(const ttgb_solution* sol, int32_t k, double* dst, int32_t dst_is_host,
                            void* stream) {
  return guarded([&] {
    TTGB_REQUIRE(sol && dst && k >= 0 && k < (int32_t)sol->res.cores.size(), "bad core index");
    const DTensor& c = sol->res.cores[k];
    TTGB_CUDA(cudaMemcpyAsync(dst, c.data(), c.numel() * sizeof(double),
                              dst_is_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                              as_stream(stream)));
    if (dst_is_host) TTGB_CUDA(cudaStreamSynchronize(as_stream(stream)));
  });
}

void ttgb_solution_free(ttgb_solution* sol) { delete sol; }

int ttgb_tt_matvec(const ttgb_tt* A, const ttgb_tt* x, void* stream, ttgb_solution** out) {
  return guarded([&] {
    TTGB_REQUIRE(A && x && out && A->d > 0 && A->d == x->d, "bad TT matvec arguments");
    TTGB_REQUIRE(A->rows != nullptr && x->rows == nullptr,
                 "Only TT-matrix @ TT-vector is supported here.");
    const TTView va = view_of(A, true), vx = view_of(x, false);
    cudaStream_t s = as_stream(stream);
    std::unique_ptr<ttgb_solution> sol(new ttgb_solution());
    sol->res.cores = tt_matvec(va, vx, s, sol->res.ranks);
    TTGB_CUDA(cudaStreamSynchronize(s));
    *out = sol.release();
  });
}

int ttgb_dmrg_matvec(const ttgb_tt* A, const ttgb_tt* x, const ttgb_tt* y0, int32_t nswp,
                     double eps, int64_t rmax, int32_t kickrank, uint64_t seed, int32_t verbose,
                     void* stream, ttgb_solution** out) {
  return guarded([&] {
    TTGB_REQUIRE(A && x && out && A->d > 0 && A->d == x->d, "bad DMRG arguments");
    TTGB_REQUIRE(A->rows != nullptr && x->rows == nullptr,
                 "A must be a TT-matrix and x a TT-vector.");
    const TTView va = view_of(A, true), vx = view_of(x, false), vy = view_of(y0, false);
    DmrgParams p;
    p.nswp = nswp; p.eps = eps; p.rmax = rmax; p.kickrank = kickrank; p.seed = seed;
    p.verbose = verbose;
    Scratch sc(as_stream(stream));
    std::unique_ptr<ttgb_solution> sol(new ttgb_solution());
    DmrgStats st;
    sol->res.cores = dmrg_matvec(va, vx, vy, p, sc.s, sol->res.ranks, &st, sc.lws, sc.red);
    sol->res.stats.sweeps = st.sweeps;
    sol->res.stats.max_res = st.max_delta;
    *out = sol.release();
  });
}

int ttgb_amen_mv(const ttgb_tt* A, const ttgb_tt* b, const ttgb_tt* x0, int32_t nswp, double eps,
                 int64_t rmax, int32_t kickrank, int32_t kick2, uint64_t seed, int32_t verbose,
                 void* stream, ttgb_solution** out) {
  return guarded([&] {
    TTGB_REQUIRE(A && b && out && A->d > 0 && A->d == b->d, "bad AMEn matvec arguments");
    TTGB_REQUIRE(A->rows != nullptr && b->rows == nullptr,
                 "A must be TT-matrix and b must be vector.");
    const TTView va = view_of(A, true), vb = view_of(b, false), vx = view_of(x0, false);
    AmenMvParams p;
    p.nswp = nswp; p.eps = eps; p.rmax = rmax; p.kickrank = kickrank; p.kick2 = kick2;
    p.seed = seed; p.verbose = verbose;
    Scratch sc(as_stream(stream));
    std::unique_ptr<ttgb_solution> sol(new ttgb_solution());
    AmenMvStats st;
    sol->res.cores = amen_mv(va, vb, vx, p, sc.s, sol->res.ranks, &st, sc.lws, sc.red);
    sol->res.stats.sweeps = st.sweeps;
    sol->res.stats.max_res = st.max_dx;
    *out = sol.release();
  });
}

int ttgb_tt_norm(const ttgb_tt* x, double* out, void* stream) {
  return guarded([&] {
    TTGB_REQUIRE(x != nullptr && x->d > 0 && out != nullptr, "bad TT norm arguments");
    const TTView v = view_of(x, x->rows != nullptr);
    Scratch sc(as_stream(stream));
    *out = tt_norm(v, sc.lws, sc.red, sc.s);
  });
}

int ttgb_tt_round(const ttgb_tt* x, double eps, int64_t rmax, void* stream, ttgb_solution** out) {
  return guarded([&] {
    TTGB_REQUIRE(x != nullptr && x->d > 0 && out != nullptr, "bad TT round arguments");
    TTGB_REQUIRE(rmax >= 1, "rmax must be positive");
    const TTView v = view_of(x, x->rows != nullptr);
    Scratch sc(as_stream(stream));
    std::unique_ptr<ttgb_solution> sol(new ttgb_solution());
    sol->res.cores = tt_round(v, eps, rmax, sc.lws, sc.red, sc.s, sol->res.ranks);
    TTGB_CUDA(cudaStreamSynchronize(sc.s));
    *out = sol.release();
  });
}

int ttgb_local_product(int64_t rl, int64_t s, int64_t r, int64_t m, int64_t n, int64_t S,
                       int64_t RL, int64_t R, const double* phi_l, const double* A,
                       const double* phi_r, const double* x, double* y, int32_t nrhs,
                       void* stream) {
  return guarded([&] {
    TTGB_REQUIRE(rl > 0 && s > 0 && r > 0 && m > 0 && n > 0 && S > 0 && RL > 0 && R > 0 && nrhs > 0,
                 "non-positive dimension");
    TTGB_REQUIRE(phi_l && A && phi_r && x && y, "null pointer");
    cudaStream_t st = as_stream(stream);
    LocalOpDims d{rl, s, r, m, n, S, RL, R};
    DBuf w1(local_product_w1(d), st), w2(local_product_w2(d), st);
    SparseCore sp;   // the solver's structured A stage when A is sparse enough
    sp.build(A, s, m, n, S, st);
    for (int32_t i = 0; i < nrhs; ++i)
      local_product(d, phi_l, A, phi_r, x + (int64_t)i * r * n * R, y + (int64_t)i * rl * m * RL,
                    w1.p, w2.p, st, 1.0, 0.0, &sp);
  });
}

int ttgb_local_product_lowp(int64_t rl, int64_t s, int64_t r, int64_t m, int64_t n, int64_t S,
                            int64_t RL, int64_t R, const double* phi_l, const double* A,
                            const double* phi_r, const double* x, double* y, int32_t engine,
                            void* stream) {
  return guarded([&] {
    TTGB_REQUIRE(rl > 0 && s > 0 && r > 0 && m > 0 && n > 0 && S > 0 && RL > 0 && R > 0,
                 "non-positive dimension");
    TTGB_REQUIRE(phi_l && A && phi_r && x && y, "null pointer");
    TTGB_REQUIRE(engine == TTGB_ENGINE_FP32 || engine == TTGB_ENGINE_TC ||
                     engine == TTGB_ENGINE_DF, "unknown engine");
    cudaStream_t st = as_stream(stream);
    LocalOpDims d{rl, s, r, m, n, S, RL, R};
    if (engine == TTGB_ENGINE_DF) {
      Fp64EngineScope eng(kFp64DoubleFloat);
      DBuf w1(local_product_w1(d), st), w2(local_product_w2(d), st);
      SparseCore sp;
      sp.build(A, s, m, n, S, st);
      local_product(d, phi_l, A, phi_r, x, y, w1.p, w2.p, st, 1.0, 0.0, &sp);
    } else if (engine == TTGB_ENGINE_TC) {
      TTGB_REQUIRE(tc_available(), "tcgen05 engine needs an sm_100-family GPU");
      int* err = nullptr;
      TTGB_CUDA(cudaMallocAsync((void**)&err, sizeof(int), st));
      TTGB_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
      {
        SparseCore sp;
        sp.build(A, s, m, n, S, st);
        TcCore core;
        if (!sp.use) core.build(A, s, m, n, S, st);
        TcLocal tl;
        tl.setup(d, phi_l, phi_r, &core, &sp, err, st);
        tl.apply(x, y, st);
        int herr = 0;
        TTGB_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
        TTGB_CUDA(cudaStreamSynchronize(st));
        cudaFreeAsync(err, st);
        if (herr) throw Error(kTimeout, "tcgen05 GEMM: a bounded wait gave up");
      }
    } else {
      const size_t nx = (size_t)(r * n * R), ny = (size_t)(rl * m * RL);
      FBuf pl((size_t)(rl * s * r), st), a32((size_t)(s * m * n * S), st), pr((size_t)(RL * S * R), st);
      FBuf xf(nx, st), yf(ny, st), w1(local_product_w1(d), st), w2(local_product_w2(d), st);
      cast(phi_l, pl.p, rl * s * r, st);
      cast(A, a32.p, s * m * n * S, st);
      cast(phi_r, pr.p, RL * S * R, st);
      cast(x, xf.p, (int64_t)nx, st);
      SparseCore sp;
      sp.build(A, s, m, n, S, st);
      local_product(d, pl.p, a32.p, pr.p, xf.p, yf.p, w1.p, w2.p, st, 1.0f, 0.0f, &sp);
      cast(yf.p, y, (int64_t)ny, st);
    }
  });
}

static int phi_A_entry(bool fwd, int64_t l, int64_t L, int64_t s, int64_t S, int64_t r, int64_t R,
                       int64_t M, int64_t N, const double* phi, const double* left, const double* A,
                       const double* right, double* out, void* stream) {
  return guarded([&] {
    TTGB_REQUIRE(l > 0 && L > 0 && s > 0 && S > 0 && r > 0 && R > 0 && M > 0 && N > 0,
                 "non-positive dimension");
    TTGB_REQUIRE(phi && left && A && right && out, "null pointer");
    cudaStream_t st = as_stream(stream);
    PhiDims d{l, L, s, S, r, R, M, N};
    DBuf w(phi_A_workspace(d), st);
    SparseCore sp;
    sp.build(A, s, M, N, S, st);
    if (fwd) phi_fwd_A(d, phi, left, A, right, out, w.p, st, &sp);
    else phi_bck_A(d, phi, left, A, right, out, w.p, st, &sp);
  });
}

int ttgb_phi_fwd_A(int64_t l, int64_t L, int64_t s, int64_t S, int64_t r, int64_t R, int64_t M,
                   int64_t N, const double* phi, const double* left, const double* A,
                   const double* right, double* out, void* stream) {
  return phi_A_entry(true, l, L, s, S, r, R, M, N, phi, left, A, right, out, stream);
}

int ttgb_phi_bck_A(int64_t l, int64_t L, int64_t s, int64_t S, int64_t r, int64_t R, int64_t M,
                   int64_t N, const double* phi, const double* left, const double* A,
                   const double* right, double* out, void* stream) {
  return phi_A_entry(false, l, L, s, S, r, R, M, N, phi, left, A, right, out, stream);
}

static int phi_rhs_entry(bool fwd, int64_t b, int64_t B, int64_t r, int64_t R, int64_t n,
                         const double* phi, const double* core_b, const double* core, double* out,
                         void* stream) {
  return guarded([&] {
    TTGB_REQUIRE(b > 0 && B > 0 && r > 0 && R > 0 && n > 0, "non-positive dimension");
    TTGB_REQUIRE(phi && core_b && core && out, "null pointer");
    cudaStream_t st = as_stream(stream);
    PhiRhsDims d{b, B, r, R, n};
    DBuf w(phi_rhs_workspace(d), st);
    if (fwd) phi_fwd_rhs(d, phi, core_b, core, out, w.p, st);
    else phi_bck_rhs(d, phi, core_b, core, out, w.p, st);
  });
}

int ttgb_phi_fwd_rhs(int64_t b, int64_t B, int64_t r, int64_t R, int64_t n, const double* phi,
                     const double* core_b, const double* core, double* out, void* stream) {
  return phi_rhs_entry(true, b, B, r, R, n, phi, core_b, core, out, stream);
}

int ttgb_phi_bck_rhs(int64_t b, int64_t B, int64_t r, int64_t R, int64_t n, const double* phi,
                     const double* core_b, const double* core, double* out, void* stream) {
  return phi_rhs_entry(false, b, B, r, R, n, phi, core_b, core, out, stream);
}

int ttgb_qr(const double* a, int64_t lda, int64_t m, int64_t n, double* q, double* r,
            void* stream) {
  return guarded([&] {
    TTGB_REQUIRE(m > 0 && n > 0 && lda >= m && a && q && r, "bad QR arguments");
    Scratch sc(as_stream(stream));
    qr(a, lda, m, n, q, r, sc.lws, sc.red, sc.s);
    TTGB_CUDA(cudaStreamSynchronize(sc.s));
  });
}

int ttgb_svd(const double* a, int64_t lda, int64_t m, int64_t n, double* u, double* s, double* vh,
             void* stream) {
  return guarded([&] {
    TTGB_REQUIRE(m > 0 && n > 0 && lda >= m && a && u && s && vh, "bad SVD arguments");
    Scratch sc(as_stream(stream));
    svd(a, lda, m, n, u, s, vh, sc.lws, sc.red, sc.s);
    TTGB_CUDA(cudaStreamSynchronize(sc.s));
  });
}

int ttgb_local_gmres(int64_t r, int64_t s, int64_t n, int64_t S, int64_t R, const double* phi_l,
                     const double* A, const double* phi_r, const double* rhs, double* x,
                     int32_t iters, double threshold, int32_t resets, int32_t prec,
                     int32_t* flag, int32_t* nit, void* stream) {
  return guarded([&] {
    TTGB_REQUIRE(r > 0 && s > 0 && n > 0 && S > 0 && R > 0 && iters > 0 && resets > 0,
                 "bad GMRES arguments");
    TTGB_REQUIRE(prec >= 0 && prec <= 2, "Invalid preconditioner.");
    Scratch sc(as_stream(stream));
    LocalOperator op;
    op.dims = LocalOpDims{r, s, r, n, n, S, R, R};
    op.phi_l = phi_l;
    op.A = A;
    op.phi_r = phi_r;
    op.prec = prec;
    DBuf w1(local_product_w1(op.dims), sc.s), w2(local_product_w2(op.dims), sc.s);
    op.w1 = w1.p;
    op.w2 = w2.p;
    DBuf J, pw, wp, tmp;
    if (prec) {
      J.reset(prec_size(prec, op.dims), sc.s);
      prec_setup(prec, op.dims, phi_l, A, phi_r, J.p, pw, sc.lws.status, sc.s);
      wp.reset((size_t)op.size(), sc.s);
      op.J = J.p;
      op.wp = wp.p;
    }
    GmresWS gws;
    TTGB_CUDA(cudaMallocAsync((void**)&gws.d_flag, 32, sc.s));
    gws.h_flag = (int*)(sc.hbuf + 64);
    GmresResult g;
    try {
      g = gmres(op, rhs, x, iters, threshold, resets, gws, sc.red, sc.s);
    } catch (...) {
      cudaFreeAsync(gws.d_flag, sc.s);
      throw;
    }
    if (prec) {
      tmp.reset((size_t)op.size(), sc.s);
      op.apply_prec(x, tmp.p, sc.s);
      copy(tmp.p, x, op.size(), sc.s);
    }
    cudaFreeAsync(gws.d_flag, sc.s);
    TTGB_CUDA(cudaStreamSynchronize(sc.s));
    if (flag) *flag = g.flag;
    if (nit) *nit = g.nit;
  });
}

const char* ttgb_last_error(void) { return g_last_error.c_str(); }

int64_t ttgb_launch_count(void) { return launch_count(); }

int ttgb_autotune(int32_t mode) { return set_autotune(mode); }

int64_t ttgb_autotune_classes(void) { return autotune_classes(); }

int ttgb_calibrate_fma(int32_t dtype, double* tflops) {
  return guarded([&] {
    TTGB_REQUIRE(tflops != nullptr && (dtype == 0 || dtype == 1), "invalid calibration request");
    *tflops = calibrate_fma(dtype);
  });
}

int ttgb_footprint(const ttgb_tt* A, const ttgb_tt* b, const ttgb_tt* x0,
                   const ttgb_amen_params* params, int64_t* bytes) {
  return guarded([&] {
    TTGB_REQUIRE(A && b && params && bytes, "null argument");
    const TTView vA = view_of(A, true), vb = view_of(b, false), vx = view_of(x0, false);
    TTGB_REQUIRE(vA.d >= 1 && vA.d == vb.d, "Dimension mismatch.");
    *bytes = (int64_t)footprint_bound(vA, vb, vx, params_from_c(params));
  });
}

int ttgb_pool_usage(int64_t* used_now, int64_t* used_high, int32_t reset_high) {
  return guarded([&] {
    int dev = 0;
    TTGB_CUDA(cudaGetDevice(&dev));
    cudaMemPool_t pool;
    TTGB_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
    unsigned long long cur = 0, high = 0;   // the attributes are 64-bit unsigned
    TTGB_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &cur));
    TTGB_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &high));
    if (used_now) *used_now = (int64_t)cur;
    if (used_high) *used_high = (int64_t)high;
    if (reset_high) {
      unsigned long long zero = 0;
      TTGB_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &zero));
    }
  });
}

int32_t ttgb_version(void) { return 103; }

}  // extern "C"
