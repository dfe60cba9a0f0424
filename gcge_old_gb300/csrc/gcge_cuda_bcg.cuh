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
  double* acol;  // row-interleaved path: alpha of each column (32 doubles)
  int* mask;     // row-interleaved path: 1 for the active columns (32 ints)
  float* bcol;   // row-interleaved path: beta of each active column for the next p (32 floats)
  float* acolf;  // row-interleaved path: acol rounded to float (32 floats)
};

// Solves A x_c = rhs_c for the len columns (rhs is overwritten by the
// residual).  The diagonal fast path is not used here: A is the stiffness.
// Returns the reference's final niter, or -1 on a CUDA error.
// M (optional): the matrix rp / ci describe (val: its values or their FP32
// copy), whose heavy rows are then multiplied chunk-wise.
template <typename T>
int bcg_run(const int* rp, const int* ci, const T* val, int n, const ColList<T>& RHS,
            const ColList<T>& X, const ColList<T>& P, const ColList<T>& W, int len, int max_it,
            double rate, const BcgScalars& s, double* partial, cudaStream_t st, int* launches,
            const GcgeDevCsr* M = nullptr);

// The same FP32 block CG with the four vectors stored row-interleaved: R, X,
// P, W are n x KW float arrays (element (r, c) at r*KW + c, KW = len rounded
// up to a multiple of 4, rows 16-byte aligned) for len <= 16, so the SpMM
// gathers one contiguous KW-float row per nonzero and every vector kernel
// streams whole rows.  Same steps, scalars and reductions (same order) as
// bcg_run<float>; s.acol and s.mask must be set.  Returns niter or -1.
// M (optional): the matrix whose heavy-row chunks (GcgeDevCsr::nheavy) rp / ci
// / val describe; its heavy rows are then multiplied chunk-wise.
int bcg_run_rows_f32(const int* rp, const int* ci, const float* val, int n, float* R, float* X,
                     float* P, float* W, int len, int max_it, double rate, const BcgScalars& s,
                     double* partial, cudaStream_t st, int* launches,
                     const GcgeDevCsr* M = nullptr);
inline int bcg_rows_width(int len) { return (len + 3) / 4 * 4; }
// Y = A X on row-interleaved n x bcg_rows_width(k) blocks (k <= 32).
void spmm_rows_f32(const int* rp, const int* ci, const float* val, int n, const float* X,
                   float* Y, int k, cudaStream_t st, const GcgeDevCsr* M = nullptr);
// Rr (n x KW rows) <- FP64 columns R[0:len] (zero-padded); Y[c] = Xr[:, c].
void cols_to_rows_f32(const ColList<double>& R, int len, float* Rr, int n, cudaStream_t st);
void rows_to_cols_f64(const float* Xr, int len, const ColList<double>& Y, int n,
                      cudaStream_t st);

}  // namespace gcge
