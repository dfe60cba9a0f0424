/*
 * gcge_cuda.h — C ABI of the GB300-native GCG eigensolver.
 *
 * A CUDA-backed app that sits beside the reference's CSR app (app/csr/):
 * it solves A x = lambda B x for the nev smallest eigenpairs of sparse
 * symmetric A and SPD B (B = NULL means the identity) with the GCG
 * iteration, entirely on one GPU.  Every entry point returns an int status
 * (0 = success, see GCGE_CUDA_ERR_*); the reference's callbacks return void
 * and exit() on fatal errors (src/gcge_eigsol.c:904-905), which a library
 * must not do.
 *
 * Plain C types only: host arrays are host pointers, "device" arrays are
 * CUDA device pointers, multivectors are arrays of column pointers (the
 * shape of the reference's default "void**" multivector, src/gcge_ops.c).
 */
#ifndef GCGE_CUDA_H_
#define GCGE_CUDA_H_

#ifdef __cplusplus
extern "C" {
#endif

#define GCGE_CUDA_OK 0
#define GCGE_CUDA_ERR_ARG 1
#define GCGE_CUDA_ERR_CUDA 2
#define GCGE_CUDA_ERR_ALLOC 3
#define GCGE_CUDA_ERR_STATE 4
#define GCGE_CUDA_ERR_NUMERIC 5
#define GCGE_CUDA_ERR_IO 6 /* file missing, unreadable or malformed */

/* Layout-compatible with the reference's CSR_MAT (app/csr/gcge_app_csr.h:27-41):
 * 0-based int32 row pointers and column indices, double entries, so a
 * CSR_MAT* can be passed where a GCGE_CUDA_CSR_HOST* is expected. */
typedef struct GCGE_CUDA_CSR_HOST_ {
  int N_Rows;
  int N_Columns;
  int N_Entries;
  int* KCol;
  int* RowPtr;
  double* Entries;
} GCGE_CUDA_CSR_HOST;

typedef struct GCGE_CUDA_MAT_ GCGE_CUDA_MAT;       /* device CSR matrix */
typedef struct GCGE_CUDA_SOLVER_ GCGE_CUDA_SOLVER; /* solver state */

/* Counters of the last Solve (see GCGE_CUDA_SOLVER_GetStats). */
typedef struct GCGE_CUDA_STATS_ {
  int num_iter;            /* GCG iterations, as para->num_iter counts them */
  int num_conv_continuous; /* leading converged pairs */
  int bcg_steps;           /* block-CG steps over all W computations */
  long long kernel_launches;
  double seconds;          /* wall time of Solve, host clock */
  double t_x_orth, t_rr_mat, t_rr_eig, t_x_axpy, t_p, t_w_line, t_w_orth, t_conv;
  int w_orth_passes;       /* block Gram-Schmidt passes of the W orthogonalisation */
} GCGE_CUDA_STATS;

/* ---------------------------------------------------------------- errors */
const char* GCGE_CUDA_GetErrorString(int code);
/* Message of the last failing call in this thread. */
const char* GCGE_CUDA_GetLastErrorMessage(void);

/* ---------------------------------------------------------------- matrices */
/* Copy a host CSR matrix to the device (replaces CSR_MAT for the solver;
 * the reference's equivalents are CSR_ReadMatFile + the CSR_MAT struct). */
int GCGE_CUDA_MatCreateFromCSR(GCGE_CUDA_MAT** mat, const GCGE_CUDA_CSR_HOST* csr);
/* rowptr/col/val are host arrays when on_device == 0, device arrays otherwise
 * (then they are copied too, the caller keeps ownership).  Rows of more than 64
 * entries are cut into chunks here that products multiply warp by warp into
 * scratch owned by the matrix: products with such a matrix must not run
 * concurrently on different streams. */
int GCGE_CUDA_MatCreate(GCGE_CUDA_MAT** mat, int n, const int* rowptr, const int* col,
                        const double* val, int on_device);
int GCGE_CUDA_MatDestroy(GCGE_CUDA_MAT** mat);
/* Rows (= columns) and stored entries of a device matrix. */
int GCGE_CUDA_MatGetSize(const GCGE_CUDA_MAT* mat, int* n, int* nnz);

/* ---------------------------------------------------------------- eigenvector adjoint
 * For eigenvector losses: with g_k = dL/dx_k (device columns, G[k] = NULL for
 * columns the loss does not touch) solves, for each requested k,
 *   (A - lambda_k B) mu_k = g_k - B x_k (x_k^T g_k),  mu_k B-orthogonal to x_k,
 * writing mu_k to MU[k] (device column of length n), and gx[k] = g_k^T x_k
 * (host array, may be NULL).  X holds the nev B-orthonormal eigenvectors and
 * eval (host) their eigenvalues, all simple; B = NULL is the identity.  mu_k
 * is the sum of its components on the other computed pairs,
 * x_j (x_j^T g_k) / (lambda_j - lambda_k), and a part in the B-orthogonal
 * complement of X found by a Jacobi-preconditioned projected CG (positive
 * definite there when lambda_k < lambda_{nev+1}), run until every column's
 * residual is below tol times its initial value (at most max_it steps;
 * GCGE_CUDA_ERR_NUMERIC if a column does not get there).  The gradient then is
 *   dL/dA_ij = -mu_k[i] x_k[j],
 *   dL/dB_ij = lambda_k mu_k[i] x_k[j] - 1/2 (g_k^T x_k) x_k[i] x_k[j],
 * which GCGE_CUDA_EigGradCSR2 assembles over a CSR pattern. */
int GCGE_CUDA_EigvecAdjointSolve(const GCGE_CUDA_MAT* A, const GCGE_CUDA_MAT* B, double* const* X,
                                 const double* eval, int nev, double* const* G, double* const* MU,
                                 double* gx, int max_it, double tol, int* iters);
/* grad[e] = sum_k (a[k] x_k[i] + b[k] mu_k[i]) x_k[j] over the stored entries
 * e = (i, j) of M (device output of M's nnz doubles); MU may be NULL (then b
 * is ignored) and MU[k] may be NULL for columns without an eigenvector term. */
int GCGE_CUDA_EigGradCSR2(const GCGE_CUDA_MAT* M, double* const* X, double* const* MU,
                          const double* a, const double* b, int k, double* grad);

/* ---------------------------------------------------------------- matrix files
 * Text: the reference's CSR file (CSR_ReadMatFile, app/csr/gcge_app_csr.c:185-236):
 * nrow, ncol, nnz, rowptr[nrow+1], col[nnz], val[nnz], whitespace separated,
 * 0-based; written with 17 significant digits, so it reads back bit-exact.
 * Binary: PETSc's Mat binary format (what the reference's PETSc app loads,
 * the test/data files ending in .petsc.bin): big-endian int32 classid 1211216, rows, cols, nnz,
 * row lengths, col, then big-endian float64 val; 32-bit indices.
 * CSR_ReadFile picks the format from the first four bytes, checks the
 * structure (row pointers 0..nnz without decrease, columns in range) and
 * fills csr with malloc'd arrays that CSR_Free releases.  Errors:
 * GCGE_CUDA_ERR_IO with the reason in GCGE_CUDA_GetLastErrorMessage. */
int GCGE_CUDA_CSR_ReadFile(const char* path, GCGE_CUDA_CSR_HOST* csr);
int GCGE_CUDA_CSR_WriteText(const char* path, const GCGE_CUDA_CSR_HOST* csr);
int GCGE_CUDA_CSR_WriteBinary(const char* path, const GCGE_CUDA_CSR_HOST* csr);
int GCGE_CUDA_CSR_Free(GCGE_CUDA_CSR_HOST* csr);
/* CSR_ReadFile + MatCreateFromCSR (square matrices). */
int GCGE_CUDA_MatCreateFromFile(GCGE_CUDA_MAT** mat, const char* path);

/* ---------------------------------------------------------------- solver
 * Mirrors GCGE_SOLVER (src/gcge_solver.h:42-60): Create, Set*, Setup,
 * Solve, Get*, Free.  Parameter names and defaults follow GCGE_PARA
 * (src/gcge_para.c:25-113) and its -gcge_* command-line flags
 * (src/gcge_para.c:128-407).  Extra flag: -gcge_precision fp64|mixed. */
int GCGE_CUDA_SOLVER_Create(GCGE_CUDA_SOLVER** solver);
int GCGE_CUDA_SOLVER_SetMatA(GCGE_CUDA_SOLVER* solver, GCGE_CUDA_MAT* A);
int GCGE_CUDA_SOLVER_SetMatB(GCGE_CUDA_SOLVER* solver, GCGE_CUDA_MAT* B);
int GCGE_CUDA_SOLVER_SetNumEigen(GCGE_CUDA_SOLVER* solver, int nev);
/* Host arrays of nev doubles / n*nev doubles (column-major) that receive the
 * result; evec also carries the initial block when num_init_evec >= nev
 * (src/gcge_eigsol.c:134,219-242). */
int GCGE_CUDA_SOLVER_SetEigenvalues(GCGE_CUDA_SOLVER* solver, double* eval);
int GCGE_CUDA_SOLVER_SetEigenvectors(GCGE_CUDA_SOLVER* solver, double* evec);
/* Same as SetEigenvectors with a DEVICE array of n*nev doubles (column j at
 * evec + j*n): the initial block is read from and the result written to
 * device memory, so a caller that keeps its data in HBM pays no transfer. */
int GCGE_CUDA_SOLVER_SetEigenvectorsDevice(GCGE_CUDA_SOLVER* solver, double* evec);
/* A block linear solver for the W step in place of the built-in block CG
 * (GCGE_OPS.MultiLinearSolver, src/gcge_ops.h:77, called at src/gcge_xpw.c:178-191):
 * on entry x[j] holds the initial guess and rhs[j] the right-hand side of
 * A x[j] = rhs[j] (device columns of length n, j < k, FP64 in both precision
 * modes); on return x[j] holds the approximate solution; rhs may be overwritten.
 * stream is the solver's cudaStream_t (all earlier work is queued on it); the
 * callback returns 0 on success.  fn = NULL restores the built-in block CG. */
typedef int (*GCGE_CUDA_MULTI_LINEAR_SOLVER)(void* ctx, const GCGE_CUDA_MAT* A,
                                             double* const* rhs, double* const* x, int k,
                                             int n, void* stream);
int GCGE_CUDA_SOLVER_SetMultiLinearSolver(GCGE_CUDA_SOLVER* solver,
                                          GCGE_CUDA_MULTI_LINEAR_SOLVER fn, void* ctx);
/* A stock GCGE_CUDA_MULTI_LINEAR_SOLVER: block CG preconditioned by the diagonal of A
 * (per column: z = D^-1 r, p = z + beta p), on the GPU; ctx points to a
 * GCGE_CUDA_PCG_PARAM (NULL: 20 steps, rate 1e-2).  A column stops once
 * ||r|| < rate ||r_0||, as the built-in block CG does. */
typedef struct GCGE_CUDA_PCG_PARAM_ {
  int max_it;
  double rate;
} GCGE_CUDA_PCG_PARAM;
int GCGE_CUDA_JacobiPCG(void* ctx, const GCGE_CUDA_MAT* A, double* const* rhs, double* const* x,
                        int k, int n, void* stream);
/* A stock GCGE_CUDA_MULTI_LINEAR_SOLVER with a polynomial preconditioner, the
 * GPU counterpart of the hypre app's preconditioned W-step solver
 * (app/hypre/gcge_app_hypre.c:305-331): per column, CG preconditioned by
 * `degree` steps of the Chebyshev semi-iteration in diag(A)^-1 A on
 * [lower_frac b, b] (b the Gershgorin bound of diag(A)^-1 A; degree 0: the
 * diagonal alone), stopping at ||r|| < rate ||r_0|| or max_it steps.  The step
 * scalars stay on the device; the host reads the active-column count every
 * 4 steps.  ctx points to a GCGE_CUDA_CHEB_PARAM (NULL: 20 steps, rate 1e-2,
 * degree 4, lower_frac 0.05).  rhs is overwritten. */
typedef struct GCGE_CUDA_CHEB_PARAM_ {
  int max_it;
  double rate;
  int degree;
  double lower_frac;
} GCGE_CUDA_CHEB_PARAM;
int GCGE_CUDA_ChebyshevPCG(void* ctx, const GCGE_CUDA_MAT* A, double* const* rhs,
                           double* const* x, int k, int n, void* stream);

/* ---------------------------------------------------------------- algebraic multigrid
 * A smoothed-aggregation AMG hierarchy of a device matrix, built on the GPU,
 * and the W-step solver that uses it.  The reference reaches an AMG through
 * its hypre app: BoomerAMG-preconditioned solvers behind MultiLinearSolver
 * (app/hypre/gcge_app_hypre.c:305-331, called at src/gcge_xpw.c:178-191) and
 * the BoomerAMG hierarchy its multilevel eigensolver builds
 * (pase/src/pase_mg.c:101-131).  Set-up: aggregation by a distance-2 maximal
 * independent set of the strength graph, prolongation P = (I - w D^-1 A) T,
 * Galerkin operators P^T A P, dense inverse of the coarsest level.  Solve:
 * Chebyshev-smoothed V-cycles in FP32 on row-interleaved blocks.  The
 * hierarchy keeps pointers to A's arrays: A must outlive it. */
typedef struct GCGE_CUDA_AMG_ GCGE_CUDA_AMG;
typedef struct GCGE_CUDA_AMG_PARAM_ {
  int max_levels;     /* hierarchy depth cap, 1..16 (default 10) */
  int coarse_size;    /* stop coarsening at this many rows or fewer, 1..512 (default 256) */
  double strength;    /* aggregation graph: |a_ij| >= strength sqrt(a_ii a_jj) (default 0) */
  int smooth_p;       /* 1 smoothed prolongation (default), 0 plain aggregation */
  int cheb_degree;    /* Chebyshev smoother degree, pre and post, 1..16 (default 3) */
  double cheb_ratio;  /* smoother interval [lambda_max / ratio, lambda_max] (default 30) */
  int pcg_max_it;     /* AMG-PCG steps per call (default 20) */
  double pcg_rate;    /* a column stops at ||r|| < pcg_rate ||r_0|| (default 1e-2) */
} GCGE_CUDA_AMG_PARAM;
void GCGE_CUDA_AMG_DefaultParam(GCGE_CUDA_AMG_PARAM* prm);
/* Builds the hierarchy of A (symmetric, positive diagonal); prm NULL: defaults. */
int GCGE_CUDA_AMG_Create(GCGE_CUDA_AMG** amg, const GCGE_CUDA_MAT* A,
                         const GCGE_CUDA_AMG_PARAM* prm);
int GCGE_CUDA_AMG_Destroy(GCGE_CUDA_AMG** amg);
int GCGE_CUDA_AMG_GetNumLevels(const GCGE_CUDA_AMG* amg, int* nlev);
/* Level l: rows, nonzeros of A_l and of P_l (0 on the coarsest level), and the
 * lambda_max(D^-1 A_l) bound of its smoother; NULL outputs are skipped. */
int GCGE_CUDA_AMG_GetLevelInfo(const GCGE_CUDA_AMG* amg, int l, int* n, int* nnz_a, int* nnz_p,
                               double* lmax);
/* Copies A_l (which = 0), P_l (1) or R_l = P_l^T (2) into host CSR arrays
 * sized from GetLevelInfo (rows + 1 row pointers). */
int GCGE_CUDA_AMG_GetLevelCSR(const GCGE_CUDA_AMG* amg, int l, int which, int* rowptr, int* col,
                              double* val);
/* The aggregate of every row of level l < nlev - 1, into host agg[n_l]. */
int GCGE_CUDA_AMG_GetAggregates(const GCGE_CUDA_AMG* amg, int l, int* agg);
/* One V-cycle x = M^-1 b for k <= 32 FP64 device columns, asynchronous on stream. */
int GCGE_CUDA_AMG_Apply(GCGE_CUDA_AMG* amg, double* const* b, double* const* x, int k,
                        void* stream);
/* A stock GCGE_CUDA_MULTI_LINEAR_SOLVER: per column, CG on A x = rhs
 * preconditioned by one V-cycle, stopping at ||r|| < pcg_rate ||r_0|| or after
 * pcg_max_it steps; ctx is a GCGE_CUDA_AMG built on this A.  The residual of
 * the start x is formed in FP64 (skipped when x is zero), the FP32 correction
 * is added to x; rhs is overwritten.  k <= 256, run 32 columns at a time.  A
 * hierarchy keeps its work blocks inside: it serves one call at a time (calls
 * on different streams must not overlap on the GPU). */
int GCGE_CUDA_AMGPCG(void* ctx, const GCGE_CUDA_MAT* A, double* const* rhs, double* const* x,
                     int k, int n, void* stream);
/* AMG-PCG steps of the last GCGE_CUDA_AMGPCG call on this hierarchy. */
int GCGE_CUDA_AMG_GetLastSteps(const GCGE_CUDA_AMG* amg, int* steps);
/* GCGE_CUDA_EigvecAdjointSolve with the projected CG preconditioned by one
 * V-cycle of amg (a hierarchy of A, n rows on its finest level) in place of
 * diag(A), with the flexible direction update -z^T U / p^T U that the FP32
 * V-cycle calls for; amg NULL: the Jacobi-preconditioned solve. */
int GCGE_CUDA_EigvecAdjointSolveAMG(const GCGE_CUDA_MAT* A, const GCGE_CUDA_MAT* B,
                                    double* const* X, const double* eval, int nev,
                                    double* const* G, double* const* MU, double* gx, int max_it,
                                    double tol, int* iters, GCGE_CUDA_AMG* amg);

/* ---------------------------------------------------------------- multilevel eigensolver
 * The multilevel correction method of the reference's PASE add-on
 * (PASE_EigenSolver, pase/src/pase_solver.c:17-82; two-grid cycle :596-627)
 * on one GPU, over the AMG hierarchy of A: B is carried down by Galerkin
 * products, the GCG solver finds nev + more_nev pairs on the auxiliary level,
 * and each cycle on the finest level smooths the vectors with AMG-PCG on
 * A u = lambda B u and solves the auxiliary problem on (coarse space + current
 * vectors) with the GCG solver.  The auxiliary level is fixed (the reference
 * also searches it at run time); converged pairs are not locked. */
typedef struct GCGE_CUDA_PASE_PARAM_ {
  int more_nev;       /* pairs carried beyond nev (default 10, the reference's more_nev) */
  int aux_level;      /* AMG level of the auxiliary coarse space, >= 1 (default 1) */
  int max_cycles;     /* two-grid cycles on the finest level (default 60) */
  int smooth_steps;   /* AMG-PCG steps per smoothing (default 2) */
  int aux_max_it;     /* GCG iterations per auxiliary solve (default 3, the reference's
                         max_direct_count_each_level) */
  int initial_max_it; /* GCG iterations of the initial solve on the auxiliary level (default 300) */
  double tol;         /* every wanted pair: ||A u - lambda B u|| / (|lambda| ||u||) < tol (default 1e-10) */
  double initial_tol; /* ev_tol of the initial solve (default 1e-8, the reference's initial_rtol) */
  double aux_tol;     /* ev_tol of the auxiliary solves (default 1e-12) */
} GCGE_CUDA_PASE_PARAM;
typedef struct GCGE_CUDA_PASE_STATS_ {
  int cycles, initial_gcg_iterations, aux_gcg_iterations, smoothing_steps;
  double max_residual, seconds;
  double t_initial, t_smooth, t_aux_build, t_aux_solve, t_prolong, t_check;
} GCGE_CUDA_PASE_STATS;
void GCGE_CUDA_PASE_DefaultParam(GCGE_CUDA_PASE_PARAM* prm);
/* The nev smallest pairs of A x = lambda B x (B NULL: identity); amg is the
 * hierarchy of A (its AMG-PCG settings are used for the smoothing and
 * restored).  eval: host array of nev; evec: DEVICE n x nev column-major
 * (B-orthonormal columns).  GCGE_CUDA_ERR_NUMERIC (with the pairs so far) when
 * max_cycles end above tol.  stats may be NULL. */
int GCGE_CUDA_PASE_Solve(const GCGE_CUDA_MAT* A, const GCGE_CUDA_MAT* B, GCGE_CUDA_AMG* amg,
                         int nev, const GCGE_CUDA_PASE_PARAM* prm, double* eval, double* evec,
                         GCGE_CUDA_PASE_STATS* stats);
/* The CUDA stream (cudaStream_t) the solver runs on, for event timing. */
int GCGE_CUDA_SOLVER_GetStream(GCGE_CUDA_SOLVER* solver, void** stream);
int GCGE_CUDA_SOLVER_SetFromCommandLine(GCGE_CUDA_SOLVER* solver, int argc, char** argv);
int GCGE_CUDA_SOLVER_SetParamInt(GCGE_CUDA_SOLVER* solver, const char* name, int value);
int GCGE_CUDA_SOLVER_SetParamDouble(GCGE_CUDA_SOLVER* solver, const char* name, double value);
int GCGE_CUDA_SOLVER_Setup(GCGE_CUDA_SOLVER* solver);
int GCGE_CUDA_SOLVER_Solve(GCGE_CUDA_SOLVER* solver);
int GCGE_CUDA_SOLVER_GetEigenvalues(GCGE_CUDA_SOLVER* solver, double** eval);
int GCGE_CUDA_SOLVER_GetEigenvectors(GCGE_CUDA_SOLVER* solver, double** evec);
/* para->res: the convergence criterion value per pair (src/gcge_eigsol.c:722). */
int GCGE_CUDA_SOLVER_GetResiduals(GCGE_CUDA_SOLVER* solver, double* res);
int GCGE_CUDA_SOLVER_GetStats(GCGE_CUDA_SOLVER* solver, GCGE_CUDA_STATS* stats);
int GCGE_CUDA_SOLVER_Free(GCGE_CUDA_SOLVER** solver);

/* Mirrors GCGE_CSR_Solver_Init (app/csr/gcge_app_csr.c:92-124): creates the
 * solver for host CSR matrices A and B (B may be NULL), allocates eval/evec,
 * reads -gcge_* flags and runs Setup.  NULL on failure. */
GCGE_CUDA_SOLVER* GCGE_CUDA_Solver_Init(const GCGE_CUDA_CSR_HOST* A, const GCGE_CUDA_CSR_HOST* B,
                                        int num_eigenvalues, int argc, char* argv[]);
/* Frees the solver and the eval/evec arrays Solver_Init allocated
 * (GCGE_SOLVER_Free_All, src/gcge_solver.c:75-82). */
int GCGE_CUDA_SOLVER_Free_All(GCGE_CUDA_SOLVER** solver);

/* ---------------------------------------------------------------- eigenvalue adjoint
 * grad[e] = sum_j coef[j] * x[j][row(e)] * x[j][col(e)] for every stored entry e of M
 * (grad: DEVICE array of nnz doubles, in M's CSR order; x: k device columns of length n;
 * coef: host array of k doubles; synchronous).  For B-normalised eigenpairs
 * (lambda_j, x_j) of A x = lambda B x and a loss L(lambda), dL/dA over A's pattern is this
 * with coef = dL/dlambda, and dL/dB over B's pattern with coef = -lambda dL/dlambda.
 * The reference has no derivatives; this is the adjoint of the eigenvalues it computes. */
int GCGE_CUDA_EigGradCSR(const GCGE_CUDA_MAT* M, double* const* x, const double* coef, int k,
                         double* grad);

/* ---------------------------------------------------------------- multivector ops
 * Device kernels in the shape of the GCGE_OPS multivector callbacks
 * (src/gcge_ops.h:76-127).  Columns are device pointers of length n; the
 * column-pointer arrays themselves are host arrays.  Synchronous. */
/* y[j] = A x[j], j < k   (MatDotMultiVec, src/gcge_ops.h:95) */
int GCGE_CUDA_MatDotMultiVec(const GCGE_CUDA_MAT* A, double* const* x, double* const* y, int k);
/* Asynchronous y[j] = A x[j] on the given cudaStream_t (NULL = legacy
 * default stream); no synchronisation, for pipelines and timing. */
int GCGE_CUDA_MatDotMultiVecAsync(const GCGE_CUDA_MAT* A, double* const* x, double* const* y,
                                  int k, void* stream);
/* FP32 variant on the FP32 copy of A (made on first use), float columns;
 * the SpMM of the mixed-precision inner solve. */
int GCGE_CUDA_MatDotMultiVecF32Async(GCGE_CUDA_MAT* A, float* const* x, float* const* y, int k,
                                     void* stream);
/* FP32 y = A x on row-interleaved blocks: x and y are device arrays of
 * n x round_up(k, 4) floats (element (r, c) at r*round_up(k,4) + c, 16-byte
 * aligned), k <= 32.  The operator of the mixed-precision block CG
 * (GCGE_BCG, src/gcge_cg.c:429-445, on FP32 copies), whose gathers read one
 * contiguous row per nonzero; asynchronous on the given cudaStream_t. */
int GCGE_CUDA_MatDotRowsF32Async(GCGE_CUDA_MAT* A, const float* x, float* y, int k, void* stream);
/* a[i + j*lda] = V[i] . W[j] into a HOST array; sym != 0 forms the upper
 * triangle and mirrors it (MultiVecInnerProd, src/gcge_ops.h:113-114). */
int GCGE_CUDA_MultiVecInnerProd(double* const* V, int k1, double* const* W, int k2, int n,
                                double* a, int lda, int sym);
/* The same inner products with FP64 accuracy on the tcgen05 bf16 tensor
 * cores: per-64-row column scaling, 7 balanced base-256 digits per value,
 * exact FP32 level sums in tensor memory, 64-bit fixed-point combination. */
int GCGE_CUDA_MultiVecInnerProdOzaki(double* const* V, int k1, double* const* W, int k2, int n,
                                     double* a, int lda, int sym);
/* a[i + j*lda] = sum_r V[i][r] d[r] W[j][r] (d = wdiag, a DEVICE array of n
 * entries, or NULL for the identity) into a HOST array, with the columns of V
 * first cut into digit planes (7 digit bytes per value and one exponent per
 * 64-row chunk), the form in which the solver multiplies the same basis
 * columns by several blocks in one GCG iteration; same accuracy as
 * GCGE_CUDA_MultiVecInnerProdOzaki (MultiVecInnerProd, src/gcge_ops.h:113-114,
 * with the B-inner product of a diagonal B folded in). */
int GCGE_CUDA_MultiVecInnerProdPlanes(double* const* V, int k1, double* const* W, int k2, int n,
                                      const double* wdiag, double* a, int lda);
/* Digit planes, for a caller that multiplies the same block of columns by
 * several others (the solver does: the basis [X, P] against each block
 * Gram-Schmidt pass and the Rayleigh-Ritz block of one GCG iteration).  A
 * plane set of ldp columns over n rows takes GCGE_CUDA_PlanesBytes(n, ldp)
 * bytes of device memory (16-byte aligned); GCGE_CUDA_PlanesCut writes the
 * columns X[0..k) (rows weighted by the device array wdiag when it is not
 * NULL) as plane columns c0 .. c0+k-1; GCGE_CUDA_PlanesGram writes
 * a[i + j*lda] = V_i . W_j (a DEVICE array) for V = plane columns
 * voff .. voff+k1-1 of one set and W = plane columns woff .. woff+k2-1 of
 * another, with FP64 accuracy (the digit scheme of
 * GCGE_CUDA_MultiVecInnerProdOzaki), using `partial`
 * (GCGE_CUDA_PlanesGramScratchDoubles(k1, k2) device doubles).  Both run
 * asynchronously on the given cudaStream_t.  No counterpart in the reference
 * (its MultiVecInnerProd, src/gcge_ops.h:113-114, is one call per product). */
size_t GCGE_CUDA_PlanesBytes(int n, int ldp);
size_t GCGE_CUDA_PlanesGramScratchDoubles(int k1, int k2);
int GCGE_CUDA_PlanesCut(double* const* X, int k, int n, const double* wdiag, void* planes,
                        int ldp, int c0, void* stream);
int GCGE_CUDA_PlanesGram(const void* vplanes, int ldv, int voff, int k1, const void* wplanes,
                         int ldw, int woff, int k2, int n, double* a, int lda, double* partial,
                         void* stream);
/* Allocation-free FP64 inner products (no counterpart in the reference):
 * the same a[i + j*lda] = V[i] . W[j] as GCGE_CUDA_MultiVecInnerProd, for
 * callers that must not allocate device memory (a fixed memory budget owned
 * by the host application, or loops where an allocation could stall or fail
 * mid-solve).  It calls no cudaMalloc/cudaFree: its reduction scratch is a
 * fixed device array of GCGE_CUDA_NOALLOC_MAX_OUTPUTS x 304 doubles
 * (9.5 MiB), so k1 * k2 above GCGE_CUDA_NOALLOC_MAX_OUTPUTS is rejected with
 * GCGE_CUDA_ERR_ARG.  `a` is a DEVICE array; the call is asynchronous on the
 * given cudaStream_t (NULL = legacy default stream).  The first call on each
 * device looks up the scratch array's address; make that first call before
 * any stream capture begins.  The address is kept per device for the life of
 * the process: after cudaDeviceReset on a device, this entry point must not
 * be called on that device again.  All calls share the one scratch array
 * (each overwrites what it reads), so calls that overlap on the GPU race.  A
 * CUDA error left pending by earlier work is reported (and left pending for
 * the caller's own check) instead of launching. */
#define GCGE_CUDA_NOALLOC_MAX_OUTPUTS 4096
int GCGE_CUDA_MultiVecInnerProdNoAlloc(double* const* V, int k1, double* const* W, int k2, int n,
                                       double* a, int lda, int sym, void* stream);
/* y[j] = sum_i x[i] a[i + j*lda] + beta y[j], a a HOST array
 * (MultiVecLinearComb, src/gcge_ops.h:109-111). */
int GCGE_CUDA_MultiVecLinearComb(double* const* x, int k1, double* const* y, int k2, int n,
                                 const double* a, int lda, double beta);
/* The same linear combination with FP64 accuracy computed on the tcgen05
 * bf16 tensor cores (per-row scaling, 7 balanced base-256 digits per value,
 * exact FP32 level sums in tensor memory, 64-bit fixed-point combination);
 * the solver's default for its X, P and W updates on GB300, where FP64 FMA
 * runs at ~1 TFLOP/s against ~2 PFLOP/s of bf16 MMA.  The columns of x are
 * balanced by powers of two first, so columns of very different magnitude
 * keep their accuracy. */
int GCGE_CUDA_MultiVecLinearCombOzaki(double* const* x, int k1, double* const* y, int k2, int n,
                                      const double* a, int lda, double beta);
/* y[j] = alpha x[j] + beta y[j] (MultiVecAxpby, src/gcge_ops.h:98-99) */
int GCGE_CUDA_MultiVecAxpby(double alpha, double* const* x, double beta, double* const* y, int k,
                            int n);
/* Eigenpairs il..iu (1-based, ascending) of the symmetric nrows x nrows HOST
 * matrix a (upper triangle), computed on the device
 * (DenseMatEigenSolver, src/gcge_ops.h:134-137). */
int GCGE_CUDA_DenseMatEigenSolver(const double* a, int lda, int nrows, double* eval,
                                  double* evec, int lde, int il, int iu);
/* Block CG (GCGE_BCG, src/gcge_cg.c:302-501) on A x_j = rhs_j for k device
 * columns; rhs is overwritten with the residual.  fp32 != 0 runs it in
 * single precision on FP32 copies.  *steps receives the final niter. */
int GCGE_CUDA_BlockCG(const GCGE_CUDA_MAT* A, double* const* rhs, double* const* x, int k, int n,
                      int max_it, double rate, int fp32, int* steps);

#ifdef __cplusplus
}
#endif
#endif /* GCGE_CUDA_H_ */
