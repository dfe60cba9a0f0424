// Shared definitions for the GB300 GCG eigensolver kernels.
//
// Multivectors are arrays of device column pointers, the device analogue of
// the reference's default "void**" multivector (src/gcge_ops.c:52-398): a
// column swap is a pointer swap, and a kernel receives the columns it works
// on as a ColList passed by value in its parameter block.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define GCGE_MAXCOLS 256

template <typename T>
struct ColList {
  T* p[GCGE_MAXCOLS];
};

struct DblList {
  double v[GCGE_MAXCOLS];
};

struct GcgeDevCsr {
  int n = 0, nnz = 0;
  int* rp = nullptr;
  int* ci = nullptr;
  double* v = nullptr;
  float* v32 = nullptr;   // FP32 copy for the mixed-precision inner solve
  double* diag = nullptr; // set when the matrix is diagonal (rp[i] = i, ci[i] = i)
  float* diag32 = nullptr;
  // Rows of more than gcge::kHeavyRow entries ("heavy", e.g. the hubs of a
  // power-law graph), cut into chunks of up to gcge::kHeavyChunk entries that a
  // warp each multiplies before the thread-per-row kernels run; those kernels
  // then read the heavy rows' products (hb64, or the chunk sums of cb32)
  // instead of walking them.
  int nheavy = 0, nchunk = 0;
  int* hidx = nullptr;     // per row: index among the heavy rows, or -1
  int* hch = nullptr;      // nheavy + 1: heavy row h owns chunks hch[h] .. hch[h+1]-1
  int* chb = nullptr;      // per chunk: first entry
  int* che = nullptr;      // per chunk: one past the last entry
  double* hb64 = nullptr;  // nheavy x GCGE_MAXCOLS products of columns, [h * k + c]
                           // (FP64, or FP32 entries for the FP32 column block CG)
  double* cb64 = nullptr;  // nchunk x kHeavyGroup chunk partials (likewise)
  float* cb32 = nullptr;   // nchunk x KW chunk partials (FP32 row-interleaved), [q * KW + c]
};


// Definition of the opaque GCGE_CUDA_MAT of include/gcge_cuda.h.
struct GCGE_CUDA_MAT_ {
  GcgeDevCsr m;
};

// ---------------------------------------------------------------- launchers
// All kernels run on the given stream; sizes are checked by the callers.
namespace gcge {

constexpr int kRowBlocks = 2 * 152;  // row-split blocks for reductions (2 per SM)

// Uneven rows (gcge_cuda_heavy.cu).
constexpr int kHeavyRow = 64, kHeavyChunk = 256, kHeavyGroup = 64;
// Builds the heavy-row chunks of M from its host row pointers; 0 or a cudaError_t.
int heavy_setup(GcgeDevCsr& M, const int* h_rp);
void heavy_free(GcgeDevCsr& M);
// hb[h * k + c] = (M X_c)[heavy row h] for c < k, with M's values val (M.v, or
// an FP32 copy for T = float); hb is M.hb64 viewed as T entries.
template <typename T>
void heavy_cols(const GcgeDevCsr& M, const T* val, const ColList<T>& X, int k, cudaStream_t st);
void heavy_cols_f64(const GcgeDevCsr& M, const ColList<double>& X, int k, cudaStream_t st);
// hb[h * kmax + id] = (M P_{unl[id]})[heavy row h] for the active ids id < *nu
// (a block CG's active list, read on the device), kmax >= *nu.
template <typename T>
void heavy_cols_active(const GcgeDevCsr& M, const T* val, const ColList<T>& P, const int* unl,
                       const int* nu, int kmax, cudaStream_t st);
// M.cb32[q * KW + c] = chunk q's share of (M X)[its row][c] for the row-interleaved
// n x KW block X with M's FP32 values val (a heavy row's product is the sum of
// its chunks hch[h] .. hch[h+1]-1, in that order); skipped on the device when
// nu != null and *nu == 0.
void heavy_rows_f32(const GcgeDevCsr& M, const float* val, const float* X, int KW, const int* nu,
                    cudaStream_t st);

// Y[:,j] = A X[:,j] for j < k.
void spmm_f64(const GcgeDevCsr& A, const ColList<double>& X, const ColList<double>& Y, int k,
              cudaStream_t st);
// Y[:,j] = A X[:,j] in FP32 on the FP32 copy of A.
void spmm_f32(const GcgeDevCsr& A, const ColList<float>& X, const ColList<float>& Y, int k,
              cudaStream_t st);
// B X, or a copy when B is the identity (B == nullptr).
void apply_b_f64(const GcgeDevCsr* B, const ColList<double>& X, const ColList<double>& Y, int k,
                 int n, cudaStream_t st);

// G[i + j*ldg] = V_i . W_j  (i < k1, j < k2).  sym: k1 == k2 and only the
// upper triangle is formed, then mirrored.  partial: scratch of
// kRowBlocks*k1*k2 doubles.
void gram_f64(const ColList<double>& V, int k1, const ColList<double>& W, int k2, int n,
              double* G, int ldg, bool sym, double* partial, cudaStream_t st);
// Y_j = beta*Y_j + sum_i X_i C[i + j*ldc]; Y must not alias X.
void lincomb_f64(const ColList<double>& X, int k1, const double* C, int ldc,
                 const ColList<double>& Y, int k2, double beta, int n, cudaStream_t st);
// The same product with FP64 accuracy on the tcgen05 bf16 tensor cores
// (error-free digit splitting, gcge_cuda_ozaki.cu); scratch of
// lincomb_oz_scratch_bytes(k1, k2).
size_t lincomb_oz_scratch_bytes(int k1, int k2);
// 1 when a tensor-core kernel gave up waiting on its MMAs (its outputs were
// set to NaN); reset clears the flag.  -1 when the flag cannot be read.
int oz_tc_status(bool reset);
void lincomb_oz(const ColList<double>& X, int k1, const double* C, int ldc,
                const ColList<double>& Y, int k2, double beta, int n, void* scratch,
                cudaStream_t st, bool balance = false, bool negate = false);
// G = V^T W with FP64 accuracy on the bf16 tensor cores; partial holds
// gram_oz_partial_doubles(k1, k2) doubles.
size_t gram_oz_partial_doubles(int k1, int k2);
// wdiag (optional): W's rows are scaled by wdiag[r] first (G = V^T diag(d) W,
// the B-Gram of a diagonal B).
void gram_oz(const ColList<double>& V, int k1, const ColList<double>& W, int k2, int n, double* G,
             int ldg, bool sym, double* partial, cudaStream_t st, const double* wdiag = nullptr);
// Digit planes (gcge_cuda_ozaki.cu): the FP64-accurate digits of a block of
// columns cut once, for Gram products that multiply the same columns again.
// A plane set of ldp columns takes planes_bytes(n, ldp) bytes (16-byte
// aligned base).
size_t planes_bytes(int n, int ldp);
// columns of X (rows weighted by d when given) -> plane columns c0 .. c0 + k - 1
void cut_planes(const ColList<double>& X, int k, int n, uint8_t* planes, int ldp, int c0,
                cudaStream_t st, const double* d = nullptr);
// gram_oz with V = plane columns voff .. voff + k1 - 1 of a set of ldv and
// W = plane columns woff .. woff + k2 - 1 of a set of ldw (not symmetric);
// partial: gram_oz_partial_doubles(k1, k2) doubles.
void gram_oz_planes(const uint8_t* vpl, int ldv, int voff, int k1, const uint8_t* wpl, int ldw,
                    int woff, int k2, int n, double* G, int ldg, double* partial,
                    cudaStream_t st);
// G[i + j*ldg] = sum_b partial[b*k1*k2 + i + j*k1] (fixed order); sym mirrors
// the upper triangle.
void gram_reduce_partials(int k1, int k2, int nblk, bool sym, const double* partial, double* G,
                          int ldg, cudaStream_t st);
// Y_j = a X_j + b Y_j
void axpby_f64(double a, const ColList<double>& X, double b, const ColList<double>& Y, int k, int n,
               cudaStream_t st);
// Y_j = s_j * Y_j with device scalars s (s_j == 0 allowed)
void scale_cols_f64(const ColList<double>& Y, const double* s, int k, int n, cudaStream_t st);
// per-column squared norms into out[j] (device), via partial.
void colnorm2_f64(const ColList<double>& X, int k, int n, double* out, double* partial,
                  cudaStream_t st);
// res_j = ||A x_j - lam_j B x_j||^2 and xn_j = ||x_j||^2 (device outputs).
void residual_f64(const GcgeDevCsr& A, const GcgeDevCsr* B, const ColList<double>& X,
                  const double* lam, int k, double* rnorm2, double* xnorm2, double* partial,
                  cudaStream_t st);
void convert_f64_to_f32(const ColList<double>& X, const ColList<float>& Y, int k, int n,
                        cudaStream_t st);
void convert_f32_to_f64(const ColList<float>& X, const ColList<double>& Y, int k, int n,
                        cudaStream_t st);

}  // namespace gcge
