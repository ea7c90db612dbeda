// TT matvec y ~ A b by AMEn on the device (reference: amen_mv / _amen_mm_python,
// torchtt/_amen.py:55-101,126-410): the sweep of the AMEn solver in which the local "solve" is the
// projection of A b onto the current interfaces, with residual-based enrichment z.
#pragma once

#include <vector>

#include "amen.cuh"
#include "linalg.cuh"

namespace ttgb {

struct AmenMvParams {
  int nswp = 22;
  double eps = 1e-10;
  int64_t rmax = 1024;
  int kickrank = 4;
  int kick2 = 0;
  uint64_t seed = 1;   // counter-based RNG of the initial z and of the kick2 columns
  int verbose = 0;
};

struct AmenMvStats {
  int sweeps = 0;
  double max_dx = 0.0;   // largest relative core update of the last sweep
};

// A: TT-matrix (rows M_k, cols N_k), b: TT-vector over N_k, x0: optional start over M_k (d == 0:
// zeros of rank 1, as the reference). Returns the cores of y (r x M_k x r') and its ranks.
std::vector<DTensor> amen_mv(const TTView& A, const TTView& b, const TTView& x0,
                             const AmenMvParams& p, cudaStream_t s, std::vector<int64_t>& ranks,
                             AmenMvStats* stats, LinalgWS& ws, const RedWS& red);

}  // namespace ttgb
