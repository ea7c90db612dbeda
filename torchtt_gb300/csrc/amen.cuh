// AMEn solve in the TT format, orchestrated on the host with all tensors device resident
// (reference: amen_solve, cpp/amen_solve.h:122-549).
#pragma once

#include <vector>

#include "common.cuh"

namespace ttgb {

struct AmenParams {
  int nswp = 22;
  double eps = 1e-10;
  int64_t rmax = 32768;
  int64_t max_full = 500;
  int kickrank = 4;
  int kick2 = 0;
  int local_iterations = 40;
  int resets = 2;
  int verbose = 0;
  int prec = 0;
  uint64_t seed = 1;
  int profile = 0;   // time every local product / interface update with CUDA events
  // 0: plain FP64 (the reference's arithmetic); 1: mixed - the local GMRES applies the operator
  // with a low-precision contraction engine inside FP64 iterative refinement, and the rank search
  // evaluates candidates as res - B tail (FP64 residual, low-precision product of the small tail).
  int precision = 0;
  int max_refine = 4;          // refinement steps per local solve (mixed)
  int lowp_engine = 0;         // mixed: 0 auto (tcgen05 when available), 1 FP32 CUDA cores, 2 tcgen05
  double lowp_floor = 1e-5;    // relative target of one low-precision inner solve (mixed)
  int a_structure = 1;         // 1: apply A cores of density < 1/4 from their nonzeros
  // FP64 contractions of the local products, interfaces and local right-hand sides: 0 auto
  // (double-float on the mixed path when A and b lie within the FP32 exponent range, native FP64
  // otherwise), 1 native FP64, 2 double-float. QR/SVD always run in native FP64.
  int fp64_engine = 0;
  // 1: the sweeps solve, truncate and stop at eps / 4, so that the true relative residual ends at
  // or below eps (the reference's rule bounds only the local residuals)
  int strict_eps = 0;
};

// A TT-matrix or TT-vector given by device pointers (borrowed).
struct TTView {
  int d = 0;
  std::vector<int64_t> rows;    // M_k (TT-matrix only)
  std::vector<int64_t> cols;    // N_k
  std::vector<int64_t> ranks;   // d + 1
  std::vector<const double*> cores;
};

struct AmenStats {
  int sweeps = 0;
  double max_res = 0.0;
  int64_t local_solves = 0;
  int64_t gmres_iterations = 0;
  int64_t matvecs = 0;            // local products of the main system
  double matvec_flops = 0.0;      // algorithmic FP64 flops of those products
  double phi_flops = 0.0;         // interface updates (x and z)
  double other_flops = 0.0;       // z / enrichment products
  int64_t direct_solves = 0;
  int64_t host_syncs = 0;
  int converged = 0;
  int64_t lowp_matvecs = 0;       // low-precision local products (mixed path)
  double lowp_flops = 0.0;        // their algorithmic flops
  int64_t refinements = 0;        // FP64 refinement steps (mixed path)
  // profile only: stream time per step of the sweep: backward z, backward QR, backward
  // interfaces, forward setup, local solve, SVD, rank search, forward z, enrichment, forward
  // interfaces, other
  double phase_ms[12] = {0};
  // profile only: CUDA-event time of the low-precision local products (mixed path)
  double lowp_ms = 0.0;
  int64_t lowp_launches = 0;
  double lowp_gemm_flops = 0.0;   // flops of their GEMM launches
  // profile only: CUDA-event time of the GMRES orthogonalisation kernels, the reference's
  // algorithmic bytes of those iterations (8 N_loc (2k + 3)) and the bytes the kernels move
  double krylov_ms = 0.0;
  int64_t krylov_launches = 0;
  double krylov_bytes = 0.0;
  double krylov_traffic_bytes = 0.0;
  int64_t gmres_syncs = 0;
  int64_t gmres_overrun = 0;
  int64_t gmres_reorth = 0;
  // filled when AmenParams::profile is set: CUDA-event time of the contraction launches and the
  // flops of their GEMMs (an A stage run from the nonzeros of a sparse core is not counted)
  double contract_ms = 0.0;
  int64_t contract_launches = 0;
  double contract_flops = 0.0;
};

struct AmenResult {
  std::vector<DTensor> cores;
  std::vector<int64_t> ranks;
  AmenStats stats;
};

// Solves A x = b. `x0` may have d == 0 (start from the all-ones tensor, amen_solve.h:161-166);
// `z0` may have d == 0 (draw the enrichment cores from a counter-based RNG seeded by p.seed).
AmenResult amen_solve(const TTView& A, const TTView& b, const TTView& x0, const TTView& z0,
                      const AmenParams& p, cudaStream_t stream);

// Upper bound of the device bytes one solve allocates: cores of x and z, the four kinds of
// interface and the local working set (Krylov basis, contraction intermediates, dense linear
// algebra) at the largest TT rank the solve can reach. An AMEn sweep raises a rank by at most
// kickrank + kick2 (the enrichment columns appended to the truncated supercore), so after nswp
// sweeps a rank is at most rank(x0) + nswp (kickrank + kick2), capped by rmax and by the products
// of the mode sizes on either side of the bond.
int64_t max_reachable_rank(const TTView& A, const TTView& x0, const AmenParams& p);
size_t footprint_bound(const TTView& A, const TTView& b, const TTView& x0, const AmenParams& p);

// device RNG: out[i] ~ N(0,1) from (seed, offset + i)
void randn(double* out, int64_t n, uint64_t seed, uint64_t offset, cudaStream_t s);

}  // namespace ttgb
