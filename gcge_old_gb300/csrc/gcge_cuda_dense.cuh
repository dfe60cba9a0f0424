// Small dense kernels of the GCG iteration; see gcge_cuda_dense.cu.
#pragma once
#include "gcge_cuda_common.cuh"

struct IntList {
  int v[GCGE_MAXCOLS];
};

namespace gcge {

// C = alpha op(A) op(B) + beta C (column-major); symA reads A as a symmetric
// matrix from its upper triangle (ta ignored).
void dgemm_small(bool ta, bool tb, bool symA, int m, int n, int k, double alpha, const double* A,
                 int lda, const double* B, int ldb, double beta, double* C, int ldc,
                 cudaStream_t st);
size_t jacobi_smem_bytes(int nrows);
// Eigenpairs il..iu (1-based, ascending) of the symmetric nrows x nrows
// matrix a (upper triangle).  work: jacobi_work_doubles(nrows) doubles.
size_t jacobi_work_doubles(int nrows);
void jacobi_eig(int nrows, const double* a, int lda, double* eval, double* evec, int lde, int il,
                int iu, double* work, int* status, cudaStream_t st);
void sub_mgs(double* V, int ldV, int nrows, int start, int end, double tol, int* end_out,
             cudaStream_t st);
// work: 2 k^2 doubles of device scratch, used when they do not fit in shared memory
void chol_drop(int k, const double* G, int ldg, double tol, double* T, int* kept, int* nk,
               double* work, cudaStream_t st);
void gather_cols(const double* src, int lds, int r0, int rows, const IntList& idx, int ncols,
                 double* dst, int ldd, cudaStream_t st);
void set_diag(double* M, int ld, const double* d, int k, cudaStream_t st);
void add_diag(double* M, int ld, double s, int k, cudaStream_t st);
void sqrt_div(const double* r2, const double* x2, double* out, int k, cudaStream_t st);

}  // namespace gcge
