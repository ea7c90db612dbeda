/*
 * ttgb300.h - C ABI of the GB300-native AMEn solver for linear systems in the tensor-train format.
 *
 * This is the drop-in boundary for torchTT's AMEn path. It replaces the reference's native entry
 * point `torchttcpp.amen_solve` (cpp/amen_solve.h:122-139, registered at cpp/cpp_ext.cpp:26) and,
 * for kernel-level parity, the contraction helpers of cpp/amen_solve.h:17-98.
 *
 * Conventions
 *   - All core pointers are DEVICE pointers to contiguous row-major float64 arrays in the
 *     reference's layouts: TT-matrix cores r x m x n x r', TT-vector cores r x n x r'
 *     (torchtt/_tt_base.py:138-145). Inputs are borrowed; nothing is written through them.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream). All work is ordered on it.
 *   - Every function returns a status code (TTGB_OK = 0); ttgb_last_error() returns the message of
 *     the last failure on the calling thread. No function throws or aborts.
 *   - Solutions are library-owned until ttgb_solution_free().
 *   - There is no CPU fallback: without a CUDA device every entry point returns TTGB_ERR_CUDA.
 */
#ifndef TTGB300_H
#define TTGB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TTGB_OK 0
#define TTGB_ERR_INVALID 1      /* shape / rank / argument errors (torchtt/errors.py:4-29) */
#define TTGB_ERR_CUDA 2         /* a CUDA runtime call failed */
#define TTGB_ERR_NUMERICAL 3    /* NaN/Inf or an unrecoverable breakdown */
#define TTGB_NOT_CONVERGED 4    /* informational, not returned as an error */
#define TTGB_ERR_OOM 5
#define TTGB_ERR_TIMEOUT 6
#define TTGB_ERR_INTERNAL 7

#define TTGB_PREC_NONE 0        /* preconditioner=None  (torchtt/solvers.py:275-282) */
#define TTGB_PREC_C 1           /* preconditioner='c'   (cpp/matvecs.h:161-165) */
#define TTGB_PREC_R 2           /* preconditioner='r'   (cpp/matvecs.h:166-174) */

/* A TT-matrix (rows != NULL) or TT-vector (rows == NULL) of d cores. */
typedef struct ttgb_tt {
  int32_t d;
  const int64_t* rows;          /* M_k, d entries (TT-matrix only) */
  const int64_t* cols;          /* N_k, d entries */
  const int64_t* ranks;         /* d + 1 entries, ranks[0] = ranks[d] = 1 */
  const double* const* cores;   /* d device pointers */
} ttgb_tt;

/* Parameters of torchttcpp.amen_solve (cpp/amen_solve.h:130-139), same meaning and defaults
 * (torchtt/solvers.py:211): nswp 22, eps 1e-10, rmax 32768, max_full 500, kickrank 4, kick2 0,
 * local_iterations 40, resets 2, verbose 0, preconditioner TTGB_PREC_NONE. `seed` drives the
 * counter-based RNG of the enrichment cores when no z0 is given. */
typedef struct ttgb_amen_params {
  int32_t nswp;
  double eps;
  int64_t rmax;
  int64_t max_full;
  int32_t kickrank;
  int32_t kick2;
  int32_t local_iterations;
  int32_t resets;
  int32_t verbose;
  int32_t preconditioner;
  uint64_t seed;
  int32_t profile;              /* 1: time the contraction launches with CUDA events (stats) */
  int32_t precision;            /* TTGB_PRECISION_FP64 (default) or TTGB_PRECISION_MIXED */
  int32_t lowp_engine;          /* MIXED only: 0 auto (TTGB_ENGINE_TC when available),
                                   TTGB_ENGINE_FP32 or TTGB_ENGINE_TC */
  int32_t a_structure;          /* 1 (default): A cores with density < 1/4 (Kronecker-sum
                                   operators) are applied from their nonzeros; 0: always dense */
  int32_t fp64_engine;          /* FP64 products of local matvecs, interfaces and local rhs:
                                   0 auto (double-float arithmetic on the FP32 pipe on the MIXED
                                   path when eps >= 1e-9 and A and b fit the FP32 exponent range,
                                   ~1e-13 relative; native FP64 otherwise), 1 native FP64,
                                   2 double-float.
                                   On the MIXED path with double-float products the GEMMs
                                   of the QR/SVD (CholeskyQR Gram and apply products) run in
                                   double-float too; the factorisations themselves (Cholesky,
                                   Jacobi rotations) always run in native FP64. */
  int32_t strict_eps;           /* 0 (default): the reference's tolerance and stopping rule,
                                   which bound the local residuals (its true residual can end a
                                   few times above eps); 1: the sweeps solve, truncate and stop
                                   at eps / 4, so that the true relative residual ends at or
                                   below eps (at the cost of higher ranks and more sweeps) */
} ttgb_amen_params;

/* Precision modes. FP64: the reference's arithmetic. MIXED: the local GMRES applies the projected
 * operator with a low-precision contraction engine inside FP64 iterative refinement (true
 * residuals, orthogonalisation, QR/SVD and the interfaces stay FP64); the analogue of the
 * reference's Python-only use_single_precision (torchtt/solvers.py:469-496). */
#define TTGB_PRECISION_FP64 0
#define TTGB_PRECISION_MIXED 1

/* Per-solve statistics. */
typedef struct ttgb_stats {
  int32_t sweeps;
  int32_t converged;            /* 1 when the max local residual fell below eps (last sweep run) */
  double max_res;               /* max local residual of the final sweep (amen_solve.h:375) */
  int64_t local_solves;
  int64_t direct_solves;
  int64_t gmres_iterations;
  int64_t matvecs;              /* local products of the projected system */
  double matvec_flops;          /* algorithmic flops of those products: 2 r n R (r s + n s S + R S) */
  double phi_flops;             /* algorithmic flops of the interface updates */
  double other_flops;           /* enrichment / z products */
  int64_t host_syncs;
  double contract_ms;           /* profile only: device time of the contraction kernels */
  int64_t contract_launches;    /* profile only: number of contraction kernel launches */
  double contract_flops;        /* profile only: flops of those GEMM launches (an A stage applied
                                   from the nonzeros of a sparse core is not counted) */
  int64_t lowp_matvecs;         /* mixed: low-precision local products */
  double lowp_flops;            /* mixed: their algorithmic flops */
  int64_t refinements;          /* mixed: FP64 refinement steps */
  double phase_ms[12];          /* profile only: stream time per sweep step - backward z, backward
                                   QR, backward interfaces, forward setup, local solve, SVD, rank
                                   search, forward z, enrichment, forward interfaces, other */
  double lowp_ms;               /* profile + mixed: device time of the low-precision products */
  int64_t lowp_launches;        /* profile + mixed: kernel launches of those products */
  double lowp_gemm_flops;       /* profile + mixed: flops of their GEMM launches */
  double krylov_ms;             /* profile: device time of the GMRES orthogonalisation kernels */
  int64_t krylov_launches;      /* profile: their launches */
  double krylov_bytes;          /* profile: algorithmic bytes of those iterations, 8 N_loc (2k + 3)
                                   for iteration k (the reference's MGS reads k + 1 vectors twice
                                   and writes one) */
  double krylov_traffic_bytes;  /* profile: bytes the Arnoldi kernels read and write: 8 N_loc (2k + 7)
                                   for iteration k, plus 8 N_loc (k + 1) when it takes the second
                                   projection */
  int64_t gmres_syncs;          /* host reads of the GMRES stop flag (also counted in host_syncs) */
  int64_t gmres_overrun;        /* GMRES iterations queued past their cycle's stopping point */
  int64_t gmres_reorth;         /* GMRES iterations that took the second projection */
} ttgb_stats;

typedef struct ttgb_solution ttgb_solution;   /* opaque, library-owned result */

/* Fills `p` with the reference defaults. */
void ttgb_default_params(ttgb_amen_params* p);

/* AMEn solve of A x = b (replaces torchttcpp.amen_solve, cpp/amen_solve.h:122-549).
 * x0 may be NULL or have d == 0 (start from the all-ones tensor, amen_solve.h:161-163).
 * z0 may be NULL (enrichment cores drawn from the seeded RNG) or give the d initial enrichment
 * cores of ranks [1, kickrank+kick2, ..., 1] (the reference draws them with torch::randn,
 * amen_solve.h:174-176). On success *out receives the solution. */
int ttgb_amen_solve(const ttgb_tt* A, const ttgb_tt* b, const ttgb_tt* x0, const ttgb_tt* z0,
                    const ttgb_amen_params* params, void* stream, ttgb_solution** out);

/* Solution accessors. ranks must hold d + 1 entries. */
int ttgb_solution_dims(const ttgb_solution* sol, int32_t* d, int64_t* ranks);
int ttgb_solution_stats(const ttgb_solution* sol, ttgb_stats* stats);
/* Device pointer of core k (r_k x n_k x r_{k+1}, row-major), valid until ttgb_solution_free. */
const double* ttgb_solution_core(const ttgb_solution* sol, int32_t k);
/* Copies core k to dst (host memory when dst_is_host != 0, else device memory). */
int ttgb_solution_copy_core(const ttgb_solution* sol, int32_t k, double* dst, int32_t dst_is_host,
                            void* stream);
void ttgb_solution_free(ttgb_solution* sol);

/* ---- batched / served solves ------------------------------------------------------------------
 * A server runs up to `slots` solves at once on the current device, each on its own stream and
 * host thread, so their kernels overlap on the GPU (continuous batching: a request is admitted as
 * soon as a slot is free and its estimated HBM footprint - cores, interfaces and Krylov basis at an
 * estimated final rank - fits in `mem_budget_bytes`; 0 means 80% of the free device memory).
 * Requests are FIFO. The input cores of a request must stay valid until it completes. A request's
 * result does not depend on what else is in flight (per-request RNG seed, per-request stream). */
typedef struct ttgb_server ttgb_server;
int ttgb_server_create(int32_t slots, int64_t mem_budget_bytes, ttgb_server** out);
/* Queues A x = b (same arguments as ttgb_amen_solve without z0/stream); *id identifies it. */
int ttgb_server_submit(ttgb_server* srv, const ttgb_tt* A, const ttgb_tt* b, const ttgb_tt* x0,
                       const ttgb_amen_params* params, int64_t* id);
/* Waits up to timeout_s (< 0: forever) for request id. On completion returns the request's status
 * (TTGB_OK and *out = its solution, owned by the caller; or the error of the solve) and its times:
 * queue_ms (submit to start) and run_ms (start to end). Returns TTGB_ERR_TIMEOUT if still running. */
int ttgb_server_wait(ttgb_server* srv, int64_t id, double timeout_s, ttgb_solution** out,
                     double* queue_ms, double* run_ms);
/* Server counters: requests submitted, completed, running now, peak concurrently running. */
int ttgb_server_stats(const ttgb_server* srv, int64_t* submitted, int64_t* completed,
                      int32_t* running, int32_t* peak_running);
/* Admission accounting: the server's budget, the bytes reserved by the running requests now and
 * the most reserved at once so far. Each request reserves its ttgb_footprint bound. */
int ttgb_server_memory(const ttgb_server* srv, int64_t* budget, int64_t* in_use,
                       int64_t* peak_in_use);
/* Finishes queued and running requests, then frees the server. */
void ttgb_server_destroy(ttgb_server* srv);
/* Upper bound of the device bytes one solve of A x = b with these parameters allocates (the
 * server's admission unit): every core, interface and local workspace at the largest TT rank the
 * solve can reach, rank(x0) + nswp (kickrank + kick2), capped by rmax and by the mode sizes.
 * x0 may be NULL. (no reference counterpart: the reference has no admission) */
int ttgb_footprint(const ttgb_tt* A, const ttgb_tt* b, const ttgb_tt* x0,
                   const ttgb_amen_params* params, int64_t* bytes);
/* Bytes the library's stream-ordered allocations hold in the current device's default memory
 * pool now and at most since the last reset (reset_high != 0 resets the high-water mark). */
int ttgb_pool_usage(int64_t* used_now, int64_t* used_high, int32_t reset_high);

/* ---- TT-level operations (FP64, device cores; a TT-matrix when x->rows is set) ---- */

/* y = A x for a TT-matrix A and a TT-vector x (ranks multiply); the result is a library-owned
   ttgb_solution. (replaces TT.__matmul__, torchtt/_tt_base.py:807-817) */
int ttgb_tt_matvec(const ttgb_tt* A, const ttgb_tt* x, void* stream, ttgb_solution** out);
/* y ~ A x by two-site DMRG to relative accuracy eps (replaces dmrg_mv, cpp/dmrg_mv.h:23-230,
   torchttcpp.dmrg_mv / torchtt dmrg_matvec, torchtt/_dmrg.py:22-45). y0 may be NULL (random start
   of rank 2 from `seed`); the result is a library-owned ttgb_solution. */
int ttgb_dmrg_matvec(const ttgb_tt* A, const ttgb_tt* x, const ttgb_tt* y0, int32_t nswp,
                     double eps, int64_t rmax, int32_t kickrank, uint64_t seed, int32_t verbose,
                     void* stream, ttgb_solution** out);
/* y ~ A b by AMEn (the projection of A b onto the sweep's interfaces with residual enrichment) to
   relative accuracy eps (replaces torchtt.amen_mv / _amen_mm_python, torchtt/_amen.py:55-101,
   126-410). x0 may be NULL (zeros of rank 1); the result is a library-owned ttgb_solution. */
int ttgb_amen_mv(const ttgb_tt* A, const ttgb_tt* b, const ttgb_tt* x0, int32_t nswp, double eps,
                 int64_t rmax, int32_t kickrank, int32_t kick2, uint64_t seed, int32_t verbose,
                 void* stream, ttgb_solution** out);
/* ||x||_F by a QR sweep (replaces TT.norm, torchtt/_tt_base.py:1021-1051). */
int ttgb_tt_norm(const ttgb_tt* x, double* out, void* stream);
/* TT rounding to relative accuracy eps with rank cap rmax; the result is a library-owned
   ttgb_solution (read with ttgb_solution_dims / _copy_core, free with ttgb_solution_free; a
   TT-matrix core comes back as r x (m n) x R). (replaces TT.round / round_tt,
   torchtt/_tt_base.py:1427-1450, torchtt/_decomposition.py:169-228; round_this,
   cpp/compression.h:3-42) */
int ttgb_tt_round(const ttgb_tt* x, double eps, int64_t rmax, void* stream, ttgb_solution** out);

/* ---- kernel-level entry points (FP64, device pointers, workspace allocated internally) ---- */

/* y[l,m,L] = sum Phi_l[l,s,r] A[s,m,n,S] Phi_r[L,S,R] x[r,n,R]
 * (replaces local_product, cpp/amen_solve.h:17-27, and AMENsolveMV::matvec, cpp/matvecs.h:196-212).
 * nrhs > 1 applies the operator to nrhs stacked inputs x (stride r*n*R) into y (stride rl*m*RL). */
int ttgb_local_product(int64_t rl, int64_t s, int64_t r, int64_t m, int64_t n, int64_t S,
                       int64_t RL, int64_t R, const double* phi_l, const double* A,
                       const double* phi_r, const double* x, double* y, int32_t nrhs, void* stream);

/* The local product with a low-precision engine (the operator of the mixed path's inner GMRES):
 * FP64 in and out, contraction in TTGB_ENGINE_FP32 (CUDA-core FFMA) or TTGB_ENGINE_TC
 * (tcgen05 tensor cores, 3xTF32 with FP32 accumulation in tensor memory); TTGB_ENGINE_DF is the
 * mixed path's FP64-class engine for its residual products (double-float arithmetic on the FP32
 * pipe, ~1e-13 relative for operands within the FP32 exponent range). Same shapes as
 * ttgb_local_product with one right-hand side. No counterpart in the reference (its only mixed mode
 * is the FP32 GMRES of torchtt/solvers.py:469-496). */
#define TTGB_ENGINE_FP32 1
#define TTGB_ENGINE_TC 2
#define TTGB_ENGINE_DF 3
int ttgb_local_product_lowp(int64_t rl, int64_t s, int64_t r, int64_t m, int64_t n, int64_t S,
                            int64_t RL, int64_t R, const double* phi_l, const double* A,
                            const double* phi_r, const double* x, double* y, int32_t engine,
                            void* stream);

/* The same product as ttgb_local_product for callers that must not allocate device memory while
 * they run (a serving loop that reserved its HBM up front and admits work by footprint, code inside
 * another framework's memory manager, latency-bound code that cannot take cudaMalloc's implicit
 * synchronisation). No counterpart in the reference. It calls no cudaMalloc/cudaFree: its two
 * contraction intermediates live in one static device array of 4 Mi doubles (32 MiB) that every
 * GPU loading the library holds until process exit, so rl*s*n*R + rl*m*S*R must not exceed
 * 4194304 (larger requests return TTGB_ERR_INVALID with a message in ttgb_last_error()). The first
 * call on a device looks up the array's device address (cudaGetSymbolAddress) with that device
 * current; make that first call before any stream capture. All calls share the array: calls that
 * overlap on the GPU race and must be ordered by the caller. It always contracts A densely (no
 * structured A stage), runs no tile-tuning measurements (so it never blocks the host), and does
 * not support cudaDeviceReset (the array's address is cached per device for the process). */
int ttgb_local_product_noalloc(int64_t rl, int64_t s, int64_t r, int64_t m, int64_t n, int64_t S,
                               int64_t RL, int64_t R, const double* phi_l, const double* A,
                               const double* phi_r, const double* x, double* y, int32_t nrhs,
                               void* stream);

/* Interface updates (replace compute_phi_fwd_A / compute_phi_bck_A / compute_phi_fwd_rhs /
 * compute_phi_bck_rhs, cpp/amen_solve.h:58-68, 38-47, 93-98, 78-83).
 *   fwd_A: phi[l,s,r], left[l,M,L], A[s,M,N,S], right[r,N,R] -> out[L,S,R]
 *   bck_A: phi[L,S,R], left[l,M,L], A[s,M,N,S], right[r,N,R] -> out[l,s,r]        */
int ttgb_phi_fwd_A(int64_t l, int64_t L, int64_t s, int64_t S, int64_t r, int64_t R, int64_t M,
                   int64_t N, const double* phi, const double* left, const double* A,
                   const double* right, double* out, void* stream);
int ttgb_phi_bck_A(int64_t l, int64_t L, int64_t s, int64_t S, int64_t r, int64_t R, int64_t M,
                   int64_t N, const double* phi, const double* left, const double* A,
                   const double* right, double* out, void* stream);
/*   fwd_rhs: phi[b,r], core_b[b,n,B], core[r,n,R] -> out[B,R]
 *   bck_rhs: phi[B,R], core_b[b,n,B], core[r,n,R] -> out[b,r]                        */
int ttgb_phi_fwd_rhs(int64_t b, int64_t B, int64_t r, int64_t R, int64_t n, const double* phi,
                     const double* core_b, const double* core, double* out, void* stream);
int ttgb_phi_bck_rhs(int64_t b, int64_t B, int64_t r, int64_t R, int64_t n, const double* phi,
                     const double* core_b, const double* core, double* out, void* stream);

/* Thin QR of the column-major m x n matrix a (lda): q (m x k), r (k x n), k = min(m, n)
 * (replaces at::linalg_qr at cpp/amen_solve.h:242,254,437,454 and cpp/ortho.h:59). */
int ttgb_qr(const double* a, int64_t lda, int64_t m, int64_t n, double* q, double* r, void* stream);
/* Thin SVD of the column-major m x n matrix a: u (m x k), s (k, descending), vh (k x n)
 * (replaces at::linalg_svd(.., false) at cpp/amen_solve.h:231,383,430). */
int ttgb_svd(const double* a, int64_t lda, int64_t m, int64_t n, double* u, double* s, double* vh,
             void* stream);

/* Solves the local system Phi_l x A x Phi_r (x) = rhs with the restarted GMRES of the AMEn local
 * step (replaces gmres, cpp/gmres.h:146-161, on AMENsolveMV): x starts at 0, `threshold` is the
 * relative residual target, at most `iters` iterations per cycle and `resets` cycles. The
 * preconditioned variable is mapped back when `prec` != 0. Returns flag/iteration count. */
int ttgb_local_gmres(int64_t r, int64_t s, int64_t n, int64_t S, int64_t R, const double* phi_l,
                     const double* A, const double* phi_r, const double* rhs, double* x,
                     int32_t iters, double threshold, int32_t resets, int32_t prec,
                     int32_t* flag, int32_t* nit, void* stream);

/* Number of kernels this library has launched in the process so far. */
int64_t ttgb_launch_count(void);

/* Measured peak of this GPU's FMA pipe in TFLOP/s (dtype 0: FP64, 1: FP32): independent FMA
   chains on every SM, best of three timed launches (about 50 ms each). */
int ttgb_calibrate_fma(int32_t dtype, double* tflops);

/* Tile autotuner of the contraction engine (no counterpart in the reference): the first launch of
   each shape class (engine, power-of-two buckets of M, N, K and batch, triangular flags, unit
   strides, device) that overwrites its output times every tile shape with and without split-K on
   the caller's stream and keeps the fastest for the process. mode 1 turns it on (the default
   unless the environment sets TTGB_AUTOTUNE=0), 0 off (occupancy heuristic), any other value only
   queries; returns the previous state. ttgb_autotune_classes gives the number of recorded classes.
   When the environment sets TTGB_AUTOTUNE_TABLE to a file path, the records of earlier processes
   are read from it at the first contraction and every new record is appended ("class candidate"
   lines), so a restarted server or a profiler run reuses the tuned tiles without timing them. */
int ttgb_autotune(int32_t mode);
int64_t ttgb_autotune_classes(void);

/* Message of the last error on this thread. */
const char* ttgb_last_error(void);
/* ABI version: 100 * major + minor. */
int32_t ttgb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* TTGB300_H */
