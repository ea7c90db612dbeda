// Block-Jacobi preconditioners of the local system (reference: cpp/matvecs.h:153-194).
#pragma once

#include "contract.cuh"

namespace ttgb {

// number of doubles of the preconditioner blocks J for `prec` (0 for none)
size_t prec_size(int prec, const LocalOpDims& d);
// builds and inverts the blocks into J (prec_size doubles); `work` is grown as needed
void prec_setup(int prec, const LocalOpDims& d, const double* phi_l, const double* A,
                const double* phi_r, double* J, DBuf& work, int* status, cudaStream_t s);

}  // namespace ttgb
