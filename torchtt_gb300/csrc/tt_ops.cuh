// TT-level operations around the solve: the Frobenius norm (true residuals ||A x - b||) and TT
// rounding (inputs such as sums of TTs are rounded before a solve). Both run on the QR/SVD kernels
// of linalg.cu and the FP64 GEMM; the host only reads the singular values to choose ranks.
#pragma once

#include <vector>

#include "amen.cuh"
#include "linalg.cuh"

namespace ttgb {

// ||x||_F of a TT-vector (rows empty) or TT-matrix (rows set; a core is r x (m n) x R).
// Right-to-left QR sweep: T_k = x_k x_3 Cur, QR of T_k^T (r x (n rc) unfolding), Cur <- R^T;
// ||x|| = ||T_0||. (reference: TT.norm, torchtt/_tt_base.py:1021-1051, a left-to-right sweep)
double tt_norm(const TTView& x, LinalgWS& ws, const RedWS& red, cudaStream_t s);

// TT rounding: left-to-right QR orthogonalisation, then right-to-left truncated SVDs with the
// relative threshold eps / sqrt(d - 1) on each unfolding and the rank cap rmax (reference:
// round_tt and rank_chop, torchtt/_decomposition.py:169-228,289-324; round_this,
// cpp/compression.h:3-42). Returns the new cores (r x mode x R row-major) and ranks (d + 1).
std::vector<DTensor> tt_round(const TTView& x, double eps, int64_t rmax, LinalgWS& ws,
                              const RedWS& red, cudaStream_t s, std::vector<int64_t>& ranks);

// y = A x for a TT-matrix A and a TT-vector x, core by core: y_k[(s r), m, (S R)] =
// sum_n A_k[s, m, n, S] x_k[r, n, R] (reference: TT.__matmul__, torchtt/_tt_base.py:807-817).
// One batched contraction per core (batch over s); ranks multiply.
std::vector<DTensor> tt_matvec(const TTView& A, const TTView& x, cudaStream_t s,
                               std::vector<int64_t>& ranks);

// Smallest rank r >= 1 with sum_{k >= r} s_k^2 < tol^2 (all of s when no such r; 1 when s = 0).
// (reference: rank_chop, torchtt/_decomposition.py:289-324)
int64_t rank_chop(const std::vector<double>& s, double tol);

}  // namespace ttgb
