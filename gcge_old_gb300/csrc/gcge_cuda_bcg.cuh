// Device-resident block CG (W step of GCG); see gcge_cuda_bcg.cu.
#pragma once
#include "gcge_cuda_common.cuh"

namespace gcge {

// Per-column scalars of the block CG, all device arrays of length >= len,
// except nu_host which is mapped pinned host memory of at least 4 ints (the
// active count after each step of a batch).
struct BcgScalars {
  double* rho1;
  double* rho2;
  double* err;
  double* lerr;
  double* ptw;
  double* rnew;
  int* unl;
  int* nu;
  volatile int* nu_host;
};

// Solves A x_c = rhs_c for the len columns (rhs is overwritten by the
// residual).  The diagonal fast path is not used here: A is the stiffness.
// Returns the reference's final niter, or -1 on a CUDA error.
template <typename T>
int bcg_run(const int* rp, const int* ci, const T* val, int n, const ColList<T>& RHS,
            const ColList<T>& X, const ColList<T>& P, const ColList<T>& W, int len, int max_it,
            double rate, const BcgScalars& s, double* partial, cudaStream_t st, int* launches);

}  // namespace gcge
