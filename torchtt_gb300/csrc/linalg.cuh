// FP64 dense linear algebra of the AMEn path: QR, thin SVD, LU solve (reference: at::linalg_qr,
// at::linalg_svd, at::linalg_solve at cpp/amen_solve.h:231,242,254,326,383,407,430,437,454 and
// cpp/ortho.h:59). Matrices are column-major with an explicit leading dimension unless stated.
#pragma once

#include "blas1.cuh"
#include "common.cuh"

namespace ttgb {

// Device workspace shared by the dense kernels of one stream; grown on demand.
struct LinalgWS {
  DBuf a, b, c, d, e;
  int* status = nullptr;      // device status word of the last factorisation (0 = ok)
  int* h_status = nullptr;    // pinned host mirror
  // Gram matrices of CholeskyQR3. The shared-memory Cholesky kernel clears the Gram matrix it has
  // read, so the next Gram product (split-K, atomic partial sums) starts from zeros without a
  // zeroing launch; the first gram_zero elements are known to be zero.
  DBuf gram;
  int64_t gram_zero = 0;
};

struct QRResult {
  int64_t k = 0;   // number of columns of Q / rows of R = min(m, n)
};

// Thin QR of the m x n column-major matrix A (lda): Q (m x k, ldq = m), R (k x n, ldr = k),
// k = min(m, n). A is not modified. Tall matrices use shifted CholeskyQR3 (three Gram/Cholesky
// passes built on the contraction engine), checked for orthogonality; small, wide or degenerate
// ones use a single-block Householder QR.
QRResult qr(const double* A, int64_t lda, int64_t m, int64_t n, double* Q, double* R,
            LinalgWS& ws, const RedWS& red, cudaStream_t s);

// R factor only (n x n column-major, ld n; rows past min(m, n) zero) of the m x n column-major A,
// by a TSQR reduction of single-block Householder QRs (blocks of max(2n, 256) rows, then pairs of
// stacked R factors): backward stable for any rank, every level one batched launch.
void qr_r(const double* A, int64_t lda, int64_t m, int64_t n, double* R, LinalgWS& ws,
          cudaStream_t s);

// Thin SVD A = U diag(S) Vh of the m x n column-major matrix A (lda): U (m x k, ld m),
// S (k), Vh (k x n, ld k), k = min(m, n), singular values in descending order.
// (reference: at::linalg_svd(A, full_matrices=false))
void svd(const double* A, int64_t lda, int64_t m, int64_t n, double* U, double* S, double* Vh,
         LinalgWS& ws, const RedWS& red, cudaStream_t s);

// Solves B x = rhs for the dense n x n row-major matrix B with partial pivoting (B is not
// modified). (reference: at::linalg_solve, cpp/amen_solve.h:326)
void lu_solve(const double* B, int64_t n, const double* rhs, double* x, LinalgWS& ws,
              cudaStream_t s);

// y = B x for the n x n row-major B
void gemv(const double* B, int64_t n, const double* x, double* y, cudaStream_t s);

// C (m x n col-major, ldc) = A (m x k col-major, lda) * B (k x n col-major, ldb)  [FP64];
// `tri`: structure flags of the contraction engine (kTriLowerC, kTriUpperB)
void gemm_cm(const double* A, int64_t lda, const double* B, int64_t ldb, double* C, int64_t ldc,
             int64_t m, int64_t n, int64_t k, double alpha, double beta, cudaStream_t s,
             bool transA = false, bool transB = false, int tri = 0, bool c_zero = false);

}  // namespace ttgb
