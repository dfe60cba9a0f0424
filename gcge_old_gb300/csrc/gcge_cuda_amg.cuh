// Internal access to an AMG hierarchy (gcge_cuda_amg.cu) for the multilevel
// eigensolver (gcge_cuda_pase.cu): the level operators, transfers and the
// Galerkin product, as plain device CSR views.
#pragma once
#include <cuda_runtime.h>

#include "../../include/gcge_cuda.h"

namespace gcge {
namespace amg {

// rows x cols device CSR with FP64 values (a view: the hierarchy owns it,
// except where a function says the caller does)
struct View {
  int rows = 0, cols = 0, nnz = 0;
  int* rp = nullptr;
  int* ci = nullptr;
  double* v = nullptr;
};

int levels(const GCGE_CUDA_AMG* a);
View op(const GCGE_CUDA_AMG* a, int l);        // A_l
View prolong(const GCGE_CUDA_AMG* a, int l);   // P_l: level l + 1 -> level l
View restrict_to(const GCGE_CUDA_AMG* a, int l);  // R_l = P_l^T: level l -> level l + 1
// C = R M P, rows sorted by column; the caller owns C (free_view).  0 or an
// error code (recorded).
int galerkin(const View& R, const View& M, const View& P, View* C, cudaStream_t st);
// the n x n identity
int identity(int n, View* I, cudaStream_t st);
void free_view(View& v);
// AMG-PCG steps and residual target of GCGE_CUDA_AMGPCG (returns the old ones)
void set_pcg(GCGE_CUDA_AMG* a, int max_it, double rate, int* old_max_it, double* old_rate);

}  // namespace amg
}  // namespace gcge
