// Fast TT matvec y ~ A x by two-site DMRG on the device (reference: dmrg_mv,
// cpp/dmrg_mv.h:23-230; dmrg_matvec, torchtt/_dmrg.py:22-45).
#pragma once

#include <vector>

#include "amen.cuh"
#include "linalg.cuh"

namespace ttgb {

struct DmrgParams {
  int nswp = 20;
  double eps = 1e-12;
  int64_t rmax = 32768;
  int kickrank = 4;
  uint64_t seed = 1;     // counter-based RNG of the random start and the rank kicks
  int verbose = 0;
};

struct DmrgStats {
  int sweeps = 0;
  double max_delta = 0.0;   // largest relative change of a two-site block in the last sweep
};

// A: TT-matrix (rows M_k, cols N_k), x: TT-vector over N_k, y0: optional start over M_k (d == 0:
// random cores of rank 2). Returns the cores of y (r x M_k x r') and its ranks (d + 1).
std::vector<DTensor> dmrg_matvec(const TTView& A, const TTView& x, const TTView& y0,
                                 const DmrgParams& p, cudaStream_t s, std::vector<int64_t>& ranks,
                                 DmrgStats* stats, LinalgWS& ws, const RedWS& red);

}  // namespace ttgb
