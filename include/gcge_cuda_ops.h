/* GCGE_OPS plugin surface of the CUDA app.
 *
 * The reference core (src/gcge_*.c) reaches vectors only through the
 * function-pointer table struct GCGE_OPS (src/gcge_ops.h:29-150), which an
 * app fills: the CSR app with per-vector host callbacks
 * (app/csr/gcge_app_csr.c:70-84), the SLEPc app with block handles
 * (app/slepc/gcge_app_slepc.c:497-527).  GCGE_CUDA_SetOps fills the same
 * table with callbacks that run on one GPU, so the unmodified core can solve
 * on device vectors: a caller builds the core as before and replaces
 * GCGE_CSR_SetOps by GCGE_CUDA_SetOps (see gcge_app_cuda.c for the
 * GCGE_SOLVER set-up, the analogue of GCGE_CSR_Solver_Init).
 *
 * GCGE_CUDA_OPS below declares the table with the reference's field order and
 * types (GCGE_INT = int, GCGE_DOUBLE = double, as the reference's
 * gcge_config.h sets them); a GCGE_OPS* can be passed wherever a
 * GCGE_CUDA_OPS* is expected and back.
 *
 * Handles: a matrix is a GCGE_CUDA_MAT* (include/gcge_cuda.h); a vector is an
 * opaque device vector handle; a multivector ("void **" in the table) is an
 * opaque block handle holding one device column per vector (the SLEPc app's
 * BV pattern), so the core never indexes it; GetVecFromMultiVec hands out a
 * view of one column.  MultiVecSwap exchanges column buffers, not data.
 *
 * Dense arrays stay on the host, as the core expects: MultiVecInnerProd
 * writes a host array, MultiVecLinearComb reads one, and each scalar inner
 * product returns to the host.  This path is for drop-in use of the
 * reference core; the device-resident solver of include/gcge_cuda.h
 * (GCGE_CUDA_SOLVER_Solve) keeps those blocks on the GPU and is the fast path.
 *
 * Errors: the callbacks return void, as the table's signatures demand.  The
 * first failure (a CUDA error, an allocation failure, a bad range) is kept in
 * a sticky flag that GCGE_CUDA_OpsGetError reads; later callbacks do nothing
 * until GCGE_CUDA_OpsClearError. */
#ifndef GCGE_CUDA_OPS_H_
#define GCGE_CUDA_OPS_H_

#include "gcge_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct GCGE_CUDA_OPS_ GCGE_CUDA_OPS;
struct GCGE_CUDA_OPS_ {
  void* ops;
  void (*VecSetRandomValue)(void* vec, GCGE_CUDA_OPS* ops);
  void (*MatDotVec)(void* mat, void* x, void* r, GCGE_CUDA_OPS* ops);
  void (*MatTransposeDotVec)(void* mat, void* x, void* r, GCGE_CUDA_OPS* ops);
  void (*VecAxpby)(double a, void* x, double b, void* y, GCGE_CUDA_OPS* ops);
  void (*VecInnerProd)(void* x, void* y, double* value_ip, GCGE_CUDA_OPS* ops);
  void (*VecLocalInnerProd)(void* x, void* y, double* value_ip, GCGE_CUDA_OPS* ops);
  void (*VecCreateByVec)(void** des_vec, void* src_vec, GCGE_CUDA_OPS* ops);
  void (*VecCreateByMat)(void** vec, void* mat, GCGE_CUDA_OPS* ops);
  void (*VecDestroy)(void** vec, GCGE_CUDA_OPS* ops);
  void (*GetVecFromMultiVec)(void** V, int j, void** x, GCGE_CUDA_OPS* ops);
  void (*RestoreVecForMultiVec)(void** V, int j, void** x, GCGE_CUDA_OPS* ops);
  void (*MultiGridCreate)(void*** A_array, void*** B_array, void*** P_array, int* num_levels,
                          void* A, void* B, GCGE_CUDA_OPS* ops);
  void (*MultiGridDestroy)(void*** A_array, void*** B_array, void*** P_array, int* num_levels,
                           GCGE_CUDA_OPS* ops);
  void (*VecFromItoJ)(void** P_array, int level_i, int level_j, void* vec_i, void* vec_j,
                      void** vec_tmp, GCGE_CUDA_OPS* ops);
  void (*MultiVecFromItoJ)(void** P_array, int level_i, int level_j, void** multi_vec_i,
                           void** multi_vec_j, void*** multi_vec_tmp, int* start, int* end,
                           GCGE_CUDA_OPS* ops);
  void (*LinearSolver)(void* Matrix, void* b, void* x, GCGE_CUDA_OPS* ops);
  void* linear_solver_workspace;
  void (*MultiLinearSolver)(void* Matrix, void** b, void** x, int* start, int* end,
                            GCGE_CUDA_OPS* ops);
  void (*Orthonormalization)(void** V, int start, int* end, void* B, double orth_zero_tol,
                             void** work);
  void (*DenseMatCreate)(void** densemat, int nrows, int ncols);
  void (*DenseMatDestroy)(void** mat);
  void (*MultiVecCreateByVec)(void*** multi_vec, int n_vec, void* vec, GCGE_CUDA_OPS* ops);
  void (*MultiVecCreateByMat)(void*** multi_vec, int n_vec, void* mat, GCGE_CUDA_OPS* ops);
  void (*MultiVecCreateByMultiVec)(void*** multi_vec, int n_vec, void** init_vec,
                                   GCGE_CUDA_OPS* ops);
  void (*MultiVecDestroy)(void*** multi_vec, int n_vec, GCGE_CUDA_OPS* ops);
  void (*MultiVecSetRandomValue)(void** multi_vec, int start, int n_vec, GCGE_CUDA_OPS* ops);
  void (*MatDotMultiVec)(void* mat, void** x, void** y, int* start, int* end, GCGE_CUDA_OPS* ops);
  void (*MatTransposeDotMultiVec)(void* mat, void** x, void** y, int* start, int* end,
                                  GCGE_CUDA_OPS* ops);
  void (*MultiVecAxpby)(double a, void** x, double b, void** y, int* start, int* end,
                        GCGE_CUDA_OPS* ops);
  void (*MultiVecAxpbyColumn)(double a, void** x, int col_x, double b, void** y, int col_y,
                              GCGE_CUDA_OPS* ops);
  void (*MultiVecLinearComb)(void** x, void** y, int* start, int* end, double* a, int lda,
                             int if_Vec, double alpha, double beta, GCGE_CUDA_OPS* ops);
  void (*MultiVecInnerProd)(void** V, void** W, double* a, char* is_sym, int* start, int* end,
                            int lda, int if_Vec, GCGE_CUDA_OPS* ops);
  void (*MultiVecInnerProdLocal)(void** V, void** W, double* a, char* is_sym, int* start,
                                 int* end, int lda, int if_Vec, GCGE_CUDA_OPS* ops);
  void (*MultiVecSwap)(void** V_1, void** V_2, int* start, int* end, GCGE_CUDA_OPS* ops);
  void (*MultiVecPrint)(void** x, int n, GCGE_CUDA_OPS* ops);
  void (*SetDirichletBoundary)(void** Vecs, int nev, void* A, void* B);
  void (*DenseMatEigenSolver)(double* a, int lda, int nrows, double* eval, double* evec, int lde,
                              int il, int iu, int* iwork, double* dwork);
  void (*DenseMatDotDenseMat)(char* transa, char* transb, int* nrows, int* ncols, int* mid,
                              double* alpha, double* a, int* lda, double* b, int* ldb,
                              double* beta, double* c, int* ldc);
  void (*DenseSymMatDotDenseMat)(char* side, char* uplo, int* nrows, int* ncols, double* alpha,
                                 double* a, int* lda, double* b, int* ldb, double* beta,
                                 double* c, int* ldc);
  double (*ArrayDotArray)(double* x, double* y, int length);
  double (*ArrayNorm)(double* x, int length);
  void (*ArrayAXPBY)(double a, double* x, double b, double* y, int length);
  void (*ArrayCopy)(double* x, double* y, int length);
  void (*ArrayScale)(double alpha, double* a, int length);
};

/* Fills the vector, multivector and matrix callbacks of `ops` (a GCGE_OPS*,
 * laid out as GCGE_CUDA_OPS): the 8 callbacks GCGE_OPS_Setup requires
 * (src/gcge_ops.c:827-874) and the block operations a block backend
 * overrides (GetVecFromMultiVec / RestoreVecForMultiVec, MultiVecCreateBy*,
 * MultiVecDestroy, MultiVecSetRandomValue, MatDotMultiVec, MultiVecAxpby,
 * MultiVecAxpbyColumn, MultiVecLinearComb, MultiVecInnerProd(Local),
 * MultiVecSwap, MultiVecPrint) and DenseMatEigenSolver (the projected
 * eigenproblem solved on the device).  The dense host BLAS entries, the
 * linear-solver hooks and the multigrid entries are left as they are (the
 * core's defaults).  Replaces GCGE_CSR_SetOps (app/csr/gcge_app_csr.c:70-84). */
int GCGE_CUDA_SetOps(void* ops);

/* Multivector handles for the caller's eigenvector block (the reference app
 * allocates its evec the same way, app/csr/gcge_app_csr.c:105-111): n_vec
 * device columns of A's size, zero-filled. */
int GCGE_CUDA_MultiVecCreate(void*** multi_vec, int n_vec, const GCGE_CUDA_MAT* A);
int GCGE_CUDA_MultiVecDestroy(void*** multi_vec);
/* Columns start .. start+k-1 from / to a column-major host block h (ldh >= n). */
int GCGE_CUDA_MultiVecSetFromHost(void** multi_vec, int start, int k, const double* h, int ldh);
int GCGE_CUDA_MultiVecGetToHost(void** multi_vec, int start, int k, double* h, int ldh);

/* The sticky status of the table's callbacks: GCGE_CUDA_OK, or the code of
 * the first failure since the last clear (its message: GCGE_CUDA_GetLastErrorMessage
 * of the failing thread). */
int GCGE_CUDA_OpsGetError(void);
void GCGE_CUDA_OpsClearError(void);

#ifdef __cplusplus
}
#endif

#endif /* GCGE_CUDA_OPS_H_ */
