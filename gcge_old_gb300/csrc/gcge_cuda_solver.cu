// GCG eigensolver driver on one GPU, behind the C ABI of include/gcge_cuda.h.
//
// The control flow is that of GCGE_Solve (src/gcge_eigsol.c:65-646) with the
// default parameters of GCGE_PARA_Create (src/gcge_para.c:25-113): X from the
// initial block, Rayleigh-Ritz on X, one [X, W] step, then the loop
// P -> X swap -> W (block CG) -> W orthonormalisation -> Rayleigh-Ritz -> X
// -> convergence check with soft locking.  Every O(n) operation runs as a
// CUDA kernel on device-resident columns; the projected (ldm x ldm) matrices
// stay in device memory too.  The host keeps the integer bookkeeping
// (dimensions, the unlock list) and reads back nev eigenvalues, residual
// norms and a few counts per iteration, which is the only host<->device
// traffic inside Solve.
//
// Differences from the reference, all basis choices inside spans that
// Rayleigh-Ritz is invariant to:
//  * W is B-orthonormalised against V by block CGS passes as in
//    GCGE_StableMultiOrthonormalization (src/gcge_orthogonal.c:1909-2019), but
//    its self-orthonormalisation is CholQR2 (Cholesky of the B-Gram with
//    zero-column dropping, twice) instead of the recursive MGS of
//    GCGE_MultiOrthonormalization (:2087-2263);
//  * the initial block is B-orthonormalised by the same CholQR2 instead of
//    GCGE_Orthonormalization (:112-308): both are QR factorisations with the
//    same triangular structure;
//  * the P coefficients are orthonormalised by CGS x max_reorth_time plus a
//    two-pass Gram-Schmidt with dropping; the reference's dgemm there uses the
//    leading dimension as the row count (:2338, :2386), which also updates
//    rows above the soft-locked block; here only the block's own rows move;
//  * the projected eigenproblem is solved by cyclic Jacobi, not dsyevx.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <string>
#include <vector>

#include "../../include/gcge_cuda.h"
#include "gcge_cuda_bcg.cuh"
#include "gcge_cuda_common.cuh"
#include "gcge_cuda_dense.cuh"

// ------------------------------------------------------------------ errors
static thread_local char g_errmsg[512] = "";

static int set_err(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_errmsg, sizeof(g_errmsg), fmt, ap);
  va_end(ap);
  return code;
}

#define CU(x)                                                                            \
  do {                                                                                   \
    cudaError_t e_ = (x);                                                                \
    if (e_ != cudaSuccess)                                                               \
      return set_err(GCGE_CUDA_ERR_CUDA, "%s failed: %s (%s:%d)", #x, cudaGetErrorString(e_), \
                     __FILE__, __LINE__);                                                \
  } while (0)

#define CHK(x)                      \
  do {                              \
    int r_ = (x);                   \
    if (r_ != GCGE_CUDA_OK) return r_; \
  } while (0)

extern "C" const char* GCGE_CUDA_GetErrorString(int code) {
  switch (code) {
    case GCGE_CUDA_OK: return "ok";
    case GCGE_CUDA_ERR_ARG: return "invalid argument";
    case GCGE_CUDA_ERR_CUDA: return "CUDA error";
    case GCGE_CUDA_ERR_ALLOC: return "allocation failed";
    case GCGE_CUDA_ERR_STATE: return "invalid solver state";
    case GCGE_CUDA_ERR_NUMERIC: return "numerical failure";
    case GCGE_CUDA_ERR_IO: return "file error";
  }
  return "unknown error";
}
extern "C" const char* GCGE_CUDA_GetLastErrorMessage(void) { return g_errmsg; }

// Records a message for GCGE_CUDA_GetLastErrorMessage from the library's
// other translation units; returns code.
int gcge_record_error(int code, const char* msg) { return set_err(code, "%s", msg); }

// ------------------------------------------------------------------ matrices

// Rejects malformed CSR input before any kernel reads it: row pointers must
// start at 0 and be non-decreasing, column indices must lie in [0, n).
static int csr_validate(int n, const int* rp, const int* ci) {
  if (rp[0] != 0) return set_err(GCGE_CUDA_ERR_ARG, "CSR: RowPtr[0] must be 0");
  for (int i = 0; i < n; i++)
    if (rp[i + 1] < rp[i]) return set_err(GCGE_CUDA_ERR_ARG, "CSR: RowPtr decreases at row %d", i);
  const int nnz = rp[n];
  for (int k = 0; k < nnz; k++)
    if (ci[k] < 0 || ci[k] >= n)
      return set_err(GCGE_CUDA_ERR_ARG, "CSR: column index %d out of range at entry %d", ci[k], k);
  return GCGE_CUDA_OK;
}

static int mat_finish(GCGE_CUDA_MAT_* M, const int* h_rp, const int* h_ci) {
  // detect a diagonal matrix (rp[i] = i, ci[i] = i) for the B fast path
  const int n = M->m.n;
  bool diag = (M->m.nnz == n);
  if (diag && h_rp && h_ci) {
    for (int i = 0; i < n && diag; i++) diag = (h_rp[i] == i && h_ci[i] == i);
  } else {
    diag = false;
  }
  if (diag) M->m.diag = M->m.v;
  if (h_rp) {
    const int e = gcge::heavy_setup(M->m, h_rp);
    if (e) return set_err(GCGE_CUDA_ERR_ALLOC, "heavy-row chunks: %s",
                          cudaGetErrorString((cudaError_t)e));
  }
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_MatCreate(GCGE_CUDA_MAT** mat, int n, const int* rowptr, const int* col,
                                   const double* val, int on_device) {
  if (!mat || n <= 0 || !rowptr || !col || !val)
    return set_err(GCGE_CUDA_ERR_ARG, "MatCreate: bad arguments");
  GCGE_CUDA_MAT_* M = new GCGE_CUDA_MAT_();
  M->m.n = n;
  std::vector<int> hrp, hci;
  const int* rp_h = rowptr;
  const int* ci_h = col;
  int nnz;
  if (on_device) {
    int last = 0;
    CU(cudaMemcpy(&last, rowptr + n, sizeof(int), cudaMemcpyDeviceToHost));
    nnz = last;
    hrp.resize(n + 1);
    hci.resize(nnz);
    CU(cudaMemcpy(hrp.data(), rowptr, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(hci.data(), col, sizeof(int) * nnz, cudaMemcpyDeviceToHost));
    rp_h = hrp.data();
    ci_h = hci.data();
  } else {
    nnz = rowptr[n];
  }
  if (nnz < 0) {
    delete M;
    return set_err(GCGE_CUDA_ERR_ARG, "MatCreate: negative nnz");
  }
  {
    const int rc = csr_validate(n, rp_h, ci_h);
    if (rc != GCGE_CUDA_OK) {
      delete M;
      return rc;
    }
  }
  M->m.nnz = nnz;
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  CU(cudaMalloc(&M->m.rp, sizeof(int) * (n + 1)));
  CU(cudaMalloc(&M->m.ci, sizeof(int) * (nnz > 0 ? nnz : 1)));
  CU(cudaMalloc(&M->m.v, sizeof(double) * (nnz > 0 ? nnz : 1)));
  CU(cudaMemcpy(M->m.rp, rowptr, sizeof(int) * (n + 1), kind));
  if (nnz > 0) {
    CU(cudaMemcpy(M->m.ci, col, sizeof(int) * nnz, kind));
    CU(cudaMemcpy(M->m.v, val, sizeof(double) * nnz, kind));
  }
  const int rc = mat_finish(M, rp_h, ci_h);
  if (rc) {
    GCGE_CUDA_MAT* tmp = M;
    GCGE_CUDA_MatDestroy(&tmp);
    return rc;
  }
  *mat = M;
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_MatCreateFromCSR(GCGE_CUDA_MAT** mat, const GCGE_CUDA_CSR_HOST* csr) {
  if (!csr || csr->N_Rows != csr->N_Columns)
    return set_err(GCGE_CUDA_ERR_ARG, "MatCreateFromCSR: matrix must be square");
  return GCGE_CUDA_MatCreate(mat, csr->N_Rows, csr->RowPtr, csr->KCol, csr->Entries, 0);
}

extern "C" int GCGE_CUDA_MatGetSize(const GCGE_CUDA_MAT* mat, int* n, int* nnz) {
  if (!mat) return set_err(GCGE_CUDA_ERR_ARG, "MatGetSize: null matrix");
  if (n) *n = mat->m.n;
  if (nnz) *nnz = mat->m.nnz;
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_MatDestroy(GCGE_CUDA_MAT** mat) {
  if (!mat || !*mat) return GCGE_CUDA_OK;
  GcgeDevCsr& m = (*mat)->m;
  gcge::heavy_free(m);
  cudaFree(m.rp);
  cudaFree(m.ci);
  cudaFree(m.v);
  if (m.v32) cudaFree(m.v32);
  delete *mat;
  *mat = nullptr;
  return GCGE_CUDA_OK;
}

static __global__ void k_to_f32(const double* __restrict__ a, float* __restrict__ b, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

static int mat_ensure_f32(GcgeDevCsr& m, cudaStream_t st) {
  if (m.v32) return GCGE_CUDA_OK;
  CU(cudaMalloc(&m.v32, sizeof(float) * (m.nnz > 0 ? m.nnz : 1)));
  if (m.nnz > 0) k_to_f32<<<(m.nnz + 255) / 256, 256, 0, st>>>(m.v, m.v32, m.nnz);
  CU(cudaGetLastError());
  return GCGE_CUDA_OK;
}

// ------------------------------------------------------------------ parameters
struct Para {
  int nev = 1;
  int ev_max_it = 30;
  int block_size = 0;
  int num_init_evec = 0;
  int cg_max_it = 20;
  int max_reorth_time = 3;
  double ev_tol = 1e-8;
  double cg_rate = 1e-2;
  double orth_zero_tol = 1e-14;
  double reorth_tol = 0.75;
  double scbgs_reorth_tol = 1e-16;
  double multi_tol_for_lock = 1e-6;
  int precision = 0;  // 0: all FP64, 1: FP32 block CG
  // tall-skinny products: 0 FP64 FMA, 1 Ozaki on bf16 tensor cores; 2 / 3:
  // Ozaki only for the linear combinations / only for the Gram blocks
  int gemm = 1;
  int print_level = 0;
  // shift (GCGE_PARA use_shift / if_shift / shift, src/gcge_para.h:90-92):
  // use_shift = 1 recomputes if_shift = 1 and shift from the Ritz values after
  // every convergence check; if_shift = 1 with shift set gives a fixed shift.
  // The block CG then solves (A + shift B) w = (lambda + shift) B x.
  int use_shift = 0;
  int if_shift = 0;
  double shift = 0.0;
  int eval_type = 0;  // 0 "sa" (smallest algebraic), 1 "sm" (smallest magnitude)
  // convergence criterion (GCGE_PARA conv_type, src/gcge_eigsol.c:713-721):
  // 0 "R" divides the residual by max(1, |lambda|), 1 "O" by
  // (conv_omega_norm + |lambda|), 2 "A" leaves it absolute
  int conv_type = 0;
  double conv_omega_norm = 0.0;
  // W block of the FP64 block CG: 0 the reference's in-place iterate w0 + e,
  // 1 the correction e alone (what the mixed form always hands over)
  int w_form = 0;
  // reports on stdout in the reference's format (GCGE_PrintFinalInfo,
  // src/gcge_para.c:577-699); off unless asked for
  int print_result = 0, print_conv = 0, print_final_part_time = 0, print_eval = 0,
      print_para = 0;
};

// ------------------------------------------------------------------ solver


struct GCGE_CUDA_SOLVER_ {
  Para para;
  GCGE_CUDA_MAT_* A = nullptr;
  GCGE_CUDA_MAT_* B = nullptr;
  double* eval_user = nullptr;  // host, nev
  double* evec_user = nullptr;  // host, n x nev
  double* evec_dev = nullptr;   // device, n x nev (alternative to evec_user)
  bool owns_user = false;
  GCGE_CUDA_MAT_* ownA = nullptr;
  GCGE_CUDA_MAT_* ownB = nullptr;
  bool setup_done = false;

  int n = 0, ldn = 0, nev = 0, bs = 0, max_dim_x = 0, V_size = 0, V_tmp_size = 0, mx = 0;
  cudaStream_t st = nullptr;
  double* pool = nullptr;  // all FP64 columns
  float* pool32 = nullptr; // FP32 columns of the mixed block CG
  std::vector<double*> V, V_tmp, CG_p, evec;
  std::vector<float*> f_rhs, f_x, f_p, f_w;
  double *sub_mat = nullptr, *sub_evec = nullptr, *sub_tmp = nullptr, *sub_tmp2 = nullptr;
  double *d_eval = nullptr, *d_small = nullptr, *partial = nullptr, *jac_work = nullptr;
  void* oz_scratch = nullptr;
  // digit planes of V[0:plane_n] (gcge::cut_planes), cut in w_orth and used
  // by its Gram passes and the Rayleigh-Ritz Gram of the same iteration;
  // plane_n = 0 outside that window
  uint8_t* planes = nullptr;
  uint8_t* wplanes = nullptr;  // the other operand's planes (bs columns)
  int plane_n = 0;
  std::vector<double*> plane_src;
  size_t partial_len = 0;
  int* d_int = nullptr;
  gcge::BcgScalars bcg{};
  // A + shift B on the union of the two patterns (built by Setup when a shift
  // is enabled): ash_av / ash_bv hold A's / B's value per union entry
  GcgeDevCsr ash{};
  double *ash_av = nullptr, *ash_bv = nullptr;
  double ash_sigma = 0.0;
  bool ash_valid = false;
  int if_shift_run = 0;   // the shift state of the running Solve
  double shift_run = 0.0;
  GCGE_CUDA_MULTI_LINEAR_SOLVER mls = nullptr;  // user W-step solver
  void* mls_ctx = nullptr;
  double* bcg_mem = nullptr;
  int* bcg_int = nullptr;
  int* h_pinned_int = nullptr;

  std::vector<double> eval, res;
  std::vector<int> unlock;
  int dim_x = 0, dim_xp = 0, dim_xpw = 0, last_dim_x = 0, last_dim_xpw = 0, unconv_bs = 0;
  int num_soft_locked = 0, num_iter = 0, num_unlock = 0, num_conv_continuous = 0;
  GCGE_CUDA_STATS stats{};
  long long launches = 0;
};

typedef GCGE_CUDA_SOLVER_ Solver;

static ColList<double> cols(const std::vector<double*>& v, int s, int e) {
  ColList<double> c;
  for (int i = 0; i < e - s; i++) c.p[i] = v[s + i];
  return c;
}
static ColList<float> colsf(const std::vector<float*>& v, int s, int e) {
  ColList<float> c;
  for (int i = 0; i < e - s; i++) c.p[i] = v[s + i];
  return c;
}
static void swap_cols(std::vector<double*>& a, int sa, int ea, std::vector<double*>& b, int sb) {
  for (int i = 0; i < ea - sa; i++) std::swap(a[sa + i], b[sb + i]);
}

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

extern "C" int GCGE_CUDA_SOLVER_Create(GCGE_CUDA_SOLVER** solver) {
  if (!solver) return set_err(GCGE_CUDA_ERR_ARG, "Create: null");
  *solver = new Solver();
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_SOLVER_SetMatA(GCGE_CUDA_SOLVER* s, GCGE_CUDA_MAT* A) {
  if (!s) return set_err(GCGE_CUDA_ERR_ARG, "SetMatA: null solver");
  s->A = A;
  return GCGE_CUDA_OK;
}
extern "C" int GCGE_CUDA_SOLVER_SetMatB(GCGE_CUDA_SOLVER* s, GCGE_CUDA_MAT* B) {
  if (!s) return set_err(GCGE_CUDA_ERR_ARG, "SetMatB: null solver");
  s->B = B;
  return GCGE_CUDA_OK;
}
extern "C" int GCGE_CUDA_SOLVER_SetNumEigen(GCGE_CUDA_SOLVER* s, int nev) {
  if (!s || nev <= 0) return set_err(GCGE_CUDA_ERR_ARG, "SetNumEigen: bad nev");
  s->para.nev = nev;
  return GCGE_CUDA_OK;
}
extern "C" int GCGE_CUDA_SOLVER_SetEigenvalues(GCGE_CUDA_SOLVER* s, double* eval) {
  if (!s) return set_err(GCGE_CUDA_ERR_ARG, "SetEigenvalues: null solver");
  s->eval_user = eval;
  return GCGE_CUDA_OK;
}
extern "C" int GCGE_CUDA_SOLVER_SetEigenvectors(GCGE_CUDA_SOLVER* s, double* evec) {
  if (!s) return set_err(GCGE_CUDA_ERR_ARG, "SetEigenvectors: null solver");
  s->evec_user = evec;
  s->evec_dev = nullptr;
  return GCGE_CUDA_OK;
}
extern "C" int GCGE_CUDA_SOLVER_SetEigenvectorsDevice(GCGE_CUDA_SOLVER* s, double* evec) {
  if (!s) return set_err(GCGE_CUDA_ERR_ARG, "SetEigenvectorsDevice: null solver");
  s->evec_dev = evec;
  s->evec_user = nullptr;
  return GCGE_CUDA_OK;
}
extern "C" int GCGE_CUDA_SOLVER_SetMultiLinearSolver(GCGE_CUDA_SOLVER* solver,
                                                     GCGE_CUDA_MULTI_LINEAR_SOLVER fn,
                                                     void* ctx) {
  if (!solver) return set_err(GCGE_CUDA_ERR_ARG, "SetMultiLinearSolver: no solver");
  solver->mls = fn;
  solver->mls_ctx = fn ? ctx : nullptr;
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_SOLVER_GetStream(GCGE_CUDA_SOLVER* s, void** stream) {
  if (!s || !stream) return set_err(GCGE_CUDA_ERR_ARG, "GetStream: null");
  if (!s->setup_done) return set_err(GCGE_CUDA_ERR_STATE, "GetStream: call Setup first");
  *stream = (void*)s->st;
  return GCGE_CUDA_OK;
}

static int set_param(Para& p, const char* name, double v) {
  std::string k(name);
  if (k.rfind("-gcge_", 0) == 0) k = k.substr(6);
  if (k == "nev") p.nev = (int)v;
  else if (k == "ev_max_it") p.ev_max_it = (int)v;
  else if (k == "block_size") p.block_size = (int)v;
  else if (k == "num_init_evec") p.num_init_evec = (int)v;
  else if (k == "cg_max_it") p.cg_max_it = (int)v;
  else if (k == "max_reorth_time") p.max_reorth_time = (int)v;
  else if (k == "ev_tol") p.ev_tol = v;
  else if (k == "cg_rate") p.cg_rate = v;
  else if (k == "orth_zero_tol") p.orth_zero_tol = v;
  else if (k == "reorth_tol") p.reorth_tol = v;
  else if (k == "scbgs_reorth_tol") p.scbgs_reorth_tol = v;
  else if (k == "multi_tol_for_lock") p.multi_tol_for_lock = v;
  else if (k == "print_level") p.print_level = (int)v;
  else if (k == "precision") p.precision = (int)v;
  else if (k == "gemm") p.gemm = (int)v;
  else if (k == "use_shift") p.use_shift = (int)v;
  else if (k == "if_shift") p.if_shift = (int)v;
  else if (k == "shift") p.shift = v;
  else if (k == "conv_type") {
    if (v != 0.0 && v != 1.0 && v != 2.0)
      return set_err(GCGE_CUDA_ERR_ARG, "conv_type: 0 (R), 1 (O) or 2 (A)");
    p.conv_type = (int)v;
  }
  else if (k == "conv_omega_norm") p.conv_omega_norm = v;
  else if (k == "w_form") {
    if (v != 0.0 && v != 1.0) return set_err(GCGE_CUDA_ERR_ARG, "w_form: 0 (reference) or 1 (correction)");
    p.w_form = (int)v;
  }
  else if (k == "print_result") p.print_result = (int)v;
  else if (k == "print_conv") p.print_conv = (int)v;
  else if (k == "print_final_part_time") p.print_final_part_time = (int)v;
  else if (k == "print_eval") p.print_eval = (int)v;
  else if (k == "print_para") p.print_para = (int)v;
  else if (k == "eval_type") {
    if (v != 0.0 && v != 1.0) return set_err(GCGE_CUDA_ERR_ARG, "eval_type: 0 (sa) or 1 (sm)");
    p.eval_type = (int)v;
  }
  else return set_err(GCGE_CUDA_ERR_ARG, "unknown parameter %s", name);
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_SOLVER_SetParamInt(GCGE_CUDA_SOLVER* s, const char* name, int v) {
  if (!s || !name) return set_err(GCGE_CUDA_ERR_ARG, "SetParamInt: null");
  if (s->setup_done) return set_err(GCGE_CUDA_ERR_STATE, "parameters are fixed after Setup");
  return set_param(s->para, name, (double)v);
}
extern "C" int GCGE_CUDA_SOLVER_SetParamDouble(GCGE_CUDA_SOLVER* s, const char* name, double v) {
  if (!s || !name) return set_err(GCGE_CUDA_ERR_ARG, "SetParamDouble: null");
  if (s->setup_done) return set_err(GCGE_CUDA_ERR_STATE, "parameters are fixed after Setup");
  return set_param(s->para, name, v);
}

// The flags of GCGE_PARA_SetFromCommandLine (src/gcge_para.c:128-407).  A
// -gcge_* flag is either honoured, accepted because it has no effect on one
// GPU (MPI layout options) or none in the reference either (opt_rr_eig_partly
// is overwritten with 1 by GCGE_ComputeSubspaceMatrix, src/gcge_rayleighritz.c:175;
// multi_tol feeds only the unused GCGE_CheckEvalMultiplicity), accepted only
// with the value whose behaviour this solver implements, or rejected with
// GCGE_CUDA_ERR_ARG: no flag is dropped silently.  -gcge_cg_rate is read as a
// real number (the reference reads it with atoi, :287, which turns 1e-2 into 0).
// Arguments that do not start with -gcge_ are skipped, as there.
static void print_usage() {
  printf("GCGE CUDA solver flags (values in brackets: the only value accepted):\n"
         "  -gcge_nev <i> -gcge_ev_max_it <i> -gcge_block_size <i> -gcge_num_init_evec <i>\n"
         "  -gcge_ev_tol <d> -gcge_conv_type R|O|A -gcge_conv_omega_norm <d> -gcge_eval_type sa|sm\n"
         "  -gcge_cg_max_it <i> -gcge_cg_rate <d> -gcge_max_reorth_time <i> -gcge_orth_zero_tol <d>\n"
         "  -gcge_reorth_tol <d> -gcge_scbgs_reorth_tol <d> -gcge_multi_tol_for_lock <d>\n"
         "  -gcge_use_shift <i> -gcge_print_result|print_conv|print_final_part_time|print_eval|"
         "print_para <i>\n"
         "  -gcge_orth_type [B] -gcge_w_orth_type [multi] -gcge_p_orth_type [multi] "
         "-gcge_x_orth_type [bgs]\n"
         "  -gcge_if_use_bcg [1] -gcge_if_use_cg [1] -gcge_use_bcg_continuous [0] -gcge_if_lobgcg [0]\n"
         "  -gcge_x_orth_block_size [0] -gcge_w_orth_block_size [0] -gcge_max_direct_orth_length [1]\n"
         "  -gcge_scbgs_wself_max_reorth_time [1]\n"
         "  no effect here: -gcge_opt_bcast -gcge_opt_allgatherv -gcge_min_nev_each_proc "
         "-gcge_partition_type -gcge_opt_rr_eig_partly -gcge_multi_tol -gcge_print_cg_error "
         "-gcge_print_part_time -gcge_print_orth_zero -gcge_print_split\n"
         "  this solver: -gcge_precision fp64|mixed -gcge_gemm ozaki|fp64 -gcge_w_form "
         "reference|correction -gcge_print_level <i>\n");
}

extern "C" int GCGE_CUDA_SOLVER_SetFromCommandLine(GCGE_CUDA_SOLVER* s, int argc, char** argv) {
  if (!s) return set_err(GCGE_CUDA_ERR_ARG, "SetFromCommandLine: null solver");
  if (s->setup_done)
    return set_err(GCGE_CUDA_ERR_STATE, "SetFromCommandLine: parameters are fixed after Setup");
  if (argc > 0 && !argv) return set_err(GCGE_CUDA_ERR_ARG, "SetFromCommandLine: null argv");
  static const char* ints[] = {"-gcge_nev", "-gcge_ev_max_it", "-gcge_block_size",
                               "-gcge_num_init_evec", "-gcge_cg_max_it", "-gcge_max_reorth_time",
                               "-gcge_print_level", "-gcge_use_shift", "-gcge_print_result",
                               "-gcge_print_conv", "-gcge_print_final_part_time",
                               "-gcge_print_eval", "-gcge_print_para"};
  static const char* dbls[] = {"-gcge_ev_tol", "-gcge_cg_rate", "-gcge_orth_zero_tol",
                               "-gcge_reorth_tol", "-gcge_scbgs_reorth_tol",
                               "-gcge_multi_tol_for_lock", "-gcge_conv_omega_norm"};
  static const char* no_effect[] = {"-gcge_opt_bcast", "-gcge_opt_allgatherv",
                                    "-gcge_min_nev_each_proc", "-gcge_partition_type",
                                    "-gcge_opt_rr_eig_partly", "-gcge_multi_tol",
                                    "-gcge_print_cg_error", "-gcge_print_part_time",
                                    "-gcge_print_orth_zero", "-gcge_print_split"};
  static const struct { const char* flag; const char* value; bool num; } fixed[] = {
      {"-gcge_orth_type", "B", false},        {"-gcge_w_orth_type", "multi", false},
      {"-gcge_p_orth_type", "multi", false},  {"-gcge_x_orth_type", "bgs", false},
      {"-gcge_if_use_bcg", "1", true},        {"-gcge_if_use_cg", "1", true},
      {"-gcge_use_bcg_continuous", "0", true}, {"-gcge_if_lobgcg", "0", true},
      {"-gcge_x_orth_block_size", "0", true}, {"-gcge_w_orth_block_size", "0", true},
      {"-gcge_max_direct_orth_length", "1", true},
      {"-gcge_scbgs_wself_max_reorth_time", "1", true}};
  Para p = s->para;  // committed only when every flag is valid
  for (int i = 0; i < argc; i++) {
    const char* a = argv[i];
    if (!a || strncmp(a, "-gcge_", 6) != 0) continue;
    if (!strcmp(a, "-gcge_help")) {
      print_usage();
      break;
    }
    if (i + 1 >= argc || !argv[i + 1])
      return set_err(GCGE_CUDA_ERR_ARG, "%s: missing value", a);
    const char* v = argv[++i];
    bool hit = false;
    for (const char* f : ints)
      if (!strcmp(a, f)) {
        CHK(set_param(p, f, (double)atoi(v)));
        hit = true;
      }
    for (const char* f : dbls)
      if (!strcmp(a, f)) {
        CHK(set_param(p, f, atof(v)));
        hit = true;
      }
    for (const char* f : no_effect)
      if (!strcmp(a, f)) hit = true;
    for (const auto& f : fixed)
      if (!strcmp(a, f.flag)) {
        const bool ok = f.num ? atoi(v) == atoi(f.value) : !strcmp(v, f.value);
        if (!ok)
          return set_err(GCGE_CUDA_ERR_ARG, "%s %s is not supported by the CUDA solver (only %s)",
                         a, v, f.value);
        hit = true;
      }
    if (!strcmp(a, "-gcge_gemm")) {
      if (!strcmp(v, "ozaki") || !strcmp(v, "1")) p.gemm = 1;
      else if (!strcmp(v, "fp64") || !strcmp(v, "0")) p.gemm = 0;
      else return set_err(GCGE_CUDA_ERR_ARG, "-gcge_gemm: fp64 or ozaki");
      hit = true;
    }
    if (!strcmp(a, "-gcge_eval_type")) {  // src/gcge_para.c:184-187
      if (!strcmp(v, "sa")) p.eval_type = 0;
      else if (!strcmp(v, "sm")) p.eval_type = 1;
      else return set_err(GCGE_CUDA_ERR_ARG, "-gcge_eval_type: sa or sm");
      hit = true;
    }
    if (!strcmp(a, "-gcge_conv_type")) {  // src/gcge_para.c:179-182, used at src/gcge_eigsol.c:713-721
      if (!strcmp(v, "R")) p.conv_type = 0;
      else if (!strcmp(v, "O")) p.conv_type = 1;
      else if (!strcmp(v, "A")) p.conv_type = 2;
      else return set_err(GCGE_CUDA_ERR_ARG, "-gcge_conv_type: R, O or A");
      hit = true;
    }
    if (!strcmp(a, "-gcge_precision")) {
      if (!strcmp(v, "mixed") || !strcmp(v, "1")) p.precision = 1;
      else if (!strcmp(v, "fp64") || !strcmp(v, "0")) p.precision = 0;
      else return set_err(GCGE_CUDA_ERR_ARG, "-gcge_precision: fp64 or mixed");
      hit = true;
    }
    if (!strcmp(a, "-gcge_w_form")) {
      if (!strcmp(v, "reference") || !strcmp(v, "0")) p.w_form = 0;
      else if (!strcmp(v, "correction") || !strcmp(v, "1")) p.w_form = 1;
      else return set_err(GCGE_CUDA_ERR_ARG, "-gcge_w_form: reference or correction");
      hit = true;
    }
    if (!hit) return set_err(GCGE_CUDA_ERR_ARG, "unknown flag %s", a);
  }
  s->para = p;
  return GCGE_CUDA_OK;
}

static void free_ws(Solver* s) {
  if (s->pool) cudaFree(s->pool);
  if (s->pool32) cudaFree(s->pool32);
  cudaFree(s->sub_mat);
  cudaFree(s->sub_evec);
  cudaFree(s->sub_tmp);
  cudaFree(s->sub_tmp2);
  cudaFree(s->d_eval);
  cudaFree(s->d_small);
  cudaFree(s->partial);
  cudaFree(s->jac_work);
  cudaFree(s->oz_scratch);
  s->oz_scratch = nullptr;
  cudaFree(s->planes);
  cudaFree(s->wplanes);
  s->planes = s->wplanes = nullptr;
  s->plane_n = 0;
  cudaFree(s->d_int);
  cudaFree(s->bcg_mem);
  cudaFree(s->bcg_int);
  if (s->h_pinned_int) cudaFreeHost(s->h_pinned_int);
  gcge::heavy_free(s->ash);
  cudaFree(s->ash.rp);
  cudaFree(s->ash.ci);
  cudaFree(s->ash.v);
  cudaFree(s->ash.v32);
  cudaFree(s->ash_av);
  cudaFree(s->ash_bv);
  s->ash = GcgeDevCsr{};
  s->ash_av = s->ash_bv = nullptr;
  s->ash_valid = false;
  if (s->st) cudaStreamDestroy(s->st);
  s->pool = nullptr;
  s->pool32 = nullptr;
  s->sub_mat = s->sub_evec = s->sub_tmp = s->sub_tmp2 = nullptr;
  s->d_eval = s->d_small = s->partial = s->jac_work = s->bcg_mem = nullptr;
  s->d_int = s->bcg_int = s->h_pinned_int = nullptr;
  s->st = nullptr;
}

// The operator of the shifted block CG (src/gcge_cg.c:348-360, 420-432 apply
// A p + shift B p): one CSR matrix on the union of A's and B's patterns (B =
// NULL is the identity), with A's and B's values kept per entry so that a new
// shift costs one pass over the values.  Built once on the host from the
// device copies.
static int build_shift_op(Solver* s) {
  const GcgeDevCsr& A = s->A->m;
  const int n = A.n;
  std::vector<int> arp(n + 1), aci(A.nnz), brp, bci;
  std::vector<double> av(A.nnz), bv;
  CU(cudaMemcpy(arp.data(), A.rp, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
  CU(cudaMemcpy(aci.data(), A.ci, sizeof(int) * A.nnz, cudaMemcpyDeviceToHost));
  CU(cudaMemcpy(av.data(), A.v, sizeof(double) * A.nnz, cudaMemcpyDeviceToHost));
  if (s->B) {
    const GcgeDevCsr& B = s->B->m;
    brp.resize(n + 1);
    bci.resize(B.nnz);
    bv.resize(B.nnz);
    CU(cudaMemcpy(brp.data(), B.rp, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(bci.data(), B.ci, sizeof(int) * B.nnz, cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(bv.data(), B.v, sizeof(double) * B.nnz, cudaMemcpyDeviceToHost));
  } else {
    brp.resize(n + 1);
    bci.resize(n);
    bv.assign(n, 1.0);
    for (int i = 0; i <= n; i++) brp[i] = i;
    for (int i = 0; i < n; i++) bci[i] = i;
  }
  std::vector<int> urp(n + 1, 0), uci;
  std::vector<double> ua, ub;
  uci.reserve((size_t)A.nnz + n);
  ua.reserve((size_t)A.nnz + n);
  ub.reserve((size_t)A.nnz + n);
  std::vector<std::pair<int, int>> row;  // (column, A entry e >= 0 or B entry -1-e)
  for (int i = 0; i < n; i++) {
    row.clear();
    for (int e = arp[i]; e < arp[i + 1]; e++) row.push_back({aci[e], e});
    for (int e = brp[i]; e < brp[i + 1]; e++) row.push_back({bci[e], -1 - e});
    std::stable_sort(row.begin(), row.end(),
                     [](const std::pair<int, int>& x, const std::pair<int, int>& y) {
                       return x.first < y.first;
                     });
    for (size_t k = 0; k < row.size(); k++) {
      if (k == 0 || row[k].first != row[k - 1].first) {
        uci.push_back(row[k].first);
        ua.push_back(0.0);
        ub.push_back(0.0);
      }
      if (row[k].second >= 0) ua.back() += av[row[k].second];
      else ub.back() += bv[-1 - row[k].second];
    }
    urp[i + 1] = (int)uci.size();
  }
  const size_t nz = uci.size();
  GcgeDevCsr& M = s->ash;
  M.n = n;
  M.nnz = (int)nz;
  CU(cudaMalloc(&M.rp, sizeof(int) * (n + 1)));
  CU(cudaMalloc(&M.ci, sizeof(int) * nz));
  CU(cudaMalloc(&M.v, sizeof(double) * nz));
  CU(cudaMalloc(&s->ash_av, sizeof(double) * nz));
  CU(cudaMalloc(&s->ash_bv, sizeof(double) * nz));
  if (s->para.precision == 1) CU(cudaMalloc(&M.v32, sizeof(float) * nz));
  CU(cudaMemcpy(M.rp, urp.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(M.ci, uci.data(), sizeof(int) * nz, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(s->ash_av, ua.data(), sizeof(double) * nz, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(s->ash_bv, ub.data(), sizeof(double) * nz, cudaMemcpyHostToDevice));
  {
    const int e = gcge::heavy_setup(M, urp.data());
    if (e) return set_err(GCGE_CUDA_ERR_ALLOC, "heavy-row chunks of the shifted operator");
  }
  s->ash_valid = false;
  return GCGE_CUDA_OK;
}

static __global__ void k_shift_values(const double* __restrict__ av, const double* __restrict__ bv,
                                      double sigma, double* __restrict__ v,
                                      float* __restrict__ v32, int nnz) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += gridDim.x * blockDim.x) {
    const double x = fma(sigma, bv[e], av[e]);
    v[e] = x;
    if (v32) v32[e] = (float)x;
  }
}

// GCGE_SOLVER_Setup = PARA_Setup + OPS_Setup + WORKSPACE_Setup
// (src/gcge_solver.c:83-88, src/gcge_para.c:414-448, src/gcge_workspace.c:61-139).
extern "C" int GCGE_CUDA_SOLVER_Setup(GCGE_CUDA_SOLVER* s) {
  if (!s || !s->A) return set_err(GCGE_CUDA_ERR_STATE, "Setup: matrix A not set");
  if (s->setup_done) free_ws(s);
  Para& p = s->para;
  const int nev = p.nev;
  if (nev <= 0) return set_err(GCGE_CUDA_ERR_ARG, "Setup: nev must be positive");
  if (p.block_size == 0) {
    p.block_size = nev < 10 ? nev : 10;
    p.block_size = (nev / 5 > p.block_size) ? nev / 5 : p.block_size;
  } else if (p.block_size > nev) {
    p.block_size = nev;
  }
  const double eps = 2.220446049250313e-16;
  // the reference adds DBL_EPSILON once in PARA_Setup (:447-448)
  static const double add = eps;
  s->n = s->A->m.n;
  if (s->B && s->B->m.n != s->n) return set_err(GCGE_CUDA_ERR_ARG, "Setup: B size differs from A");
  if (nev + 20 + 2 * p.block_size > GCGE_MAXCOLS)
    return set_err(GCGE_CUDA_ERR_ARG, "Setup: nev + 20 + 2*block_size must be <= %d", GCGE_MAXCOLS);
  if (nev > s->n) return set_err(GCGE_CUDA_ERR_ARG, "Setup: nev larger than the matrix");
  s->nev = nev;
  s->bs = p.block_size;
  s->max_dim_x = nev + 20;
  s->V_size = s->max_dim_x + 2 * s->bs;
  s->V_tmp_size = s->max_dim_x - nev + s->bs;
  s->mx = s->max_dim_x + 2 * s->bs;
  s->ldn = (s->n + 31) / 32 * 32;  // 256-byte aligned columns
  CU(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking));
  const int ncols = s->V_size + s->V_tmp_size + s->bs + nev;
  CU(cudaMalloc(&s->pool, sizeof(double) * (size_t)s->ldn * ncols));
  CU(cudaMemsetAsync(s->pool, 0, sizeof(double) * (size_t)s->ldn * ncols, s->st));
  double* q = s->pool;
  auto take = [&](std::vector<double*>& v, int k) {
    v.resize(k);
    for (int i = 0; i < k; i++, q += s->ldn) v[i] = q;
  };
  take(s->V, s->V_size);
  take(s->V_tmp, s->V_tmp_size);
  take(s->CG_p, s->bs);
  take(s->evec, nev);
  if (p.precision == 1) {
    CHK(mat_ensure_f32(s->A->m, s->st));
    // four column blocks of the block CG, wide enough for the row-interleaved
    // layout (block size rounded up to 4)
    const size_t f32n = (size_t)s->ldn * 4 * gcge::bcg_rows_width(s->bs);
    CU(cudaMalloc(&s->pool32, sizeof(float) * f32n));
    CU(cudaMemsetAsync(s->pool32, 0, sizeof(float) * f32n, s->st));
    float* f = s->pool32;
    auto takef = [&](std::vector<float*>& v) {
      v.resize(s->bs);
      for (int i = 0; i < s->bs; i++, f += s->ldn) v[i] = f;
    };
    takef(s->f_rhs);
    takef(s->f_x);
    takef(s->f_p);
    takef(s->f_w);
  }
  const size_t mm = (size_t)s->mx * s->mx;
  CU(cudaMalloc(&s->sub_mat, sizeof(double) * mm));
  CU(cudaMalloc(&s->sub_evec, sizeof(double) * mm));
  CU(cudaMalloc(&s->sub_tmp, sizeof(double) * mm));
  CU(cudaMalloc(&s->sub_tmp2, sizeof(double) * mm));
  CU(cudaMemsetAsync(s->sub_mat, 0, sizeof(double) * mm, s->st));
  CU(cudaMemsetAsync(s->sub_evec, 0, sizeof(double) * mm, s->st));
  CU(cudaMalloc(&s->d_eval, sizeof(double) * s->mx));
  CU(cudaMemsetAsync(s->d_eval, 0, sizeof(double) * s->mx, s->st));
  CU(cudaMalloc(&s->d_small, sizeof(double) * 8 * GCGE_MAXCOLS));
  CU(cudaMalloc(&s->d_int, sizeof(int) * 4 * GCGE_MAXCOLS));
  CU(cudaMalloc(&s->jac_work, sizeof(double) * gcge::jacobi_work_doubles(s->mx)));
  CU(cudaMalloc(&s->oz_scratch, gcge::lincomb_oz_scratch_bytes(s->mx, s->mx)));
  if (s->para.gemm == 1 || s->para.gemm == 3) {
    CU(cudaMalloc(&s->planes, gcge::planes_bytes(s->n, s->mx)));
    CU(cudaMalloc(&s->wplanes, gcge::planes_bytes(s->n, s->bs)));
    s->plane_src.assign(s->mx, nullptr);
  }
  s->plane_n = 0;
  // partial sums: Gram tiles (<= 4 x 4 tiles of 64 x 64 per row block) or
  // per-column partials of the row-split reductions
  const int tiles = ((s->mx + 63) / 64) * ((s->mx + 63) / 64);
  s->partial_len = (size_t)gcge::kRowBlocks * tiles * 64 * 64;
  const size_t colpart = (size_t)gcge::kRowBlocks * 2 * GCGE_MAXCOLS * 2;
  if (s->partial_len < colpart) s->partial_len = colpart;
  CU(cudaMalloc(&s->partial, sizeof(double) * s->partial_len));
  // block-CG scalars
  CU(cudaMalloc(&s->bcg_mem, sizeof(double) * 8 * GCGE_MAXCOLS));
  CU(cudaMemsetAsync(s->bcg_mem, 0, sizeof(double) * 8 * GCGE_MAXCOLS, s->st));
  CU(cudaMalloc(&s->bcg_int, sizeof(int) * (2 * GCGE_MAXCOLS + 1)));
  CU(cudaMemsetAsync(s->bcg_int, 0, sizeof(int) * (2 * GCGE_MAXCOLS + 1), s->st));
  CU(cudaHostAlloc(&s->h_pinned_int, sizeof(int) * 16, cudaHostAllocMapped));
  int* dev_alias = nullptr;
  CU(cudaHostGetDevicePointer((void**)&dev_alias, s->h_pinned_int, 0));
  if (dev_alias != s->h_pinned_int)
    return set_err(GCGE_CUDA_ERR_STATE, "Setup: mapped host memory needs unified addressing");
  s->bcg.rho1 = s->bcg_mem;
  s->bcg.rho2 = s->bcg_mem + GCGE_MAXCOLS;
  s->bcg.err = s->bcg_mem + 2 * GCGE_MAXCOLS;
  s->bcg.lerr = s->bcg_mem + 3 * GCGE_MAXCOLS;
  s->bcg.ptw = s->bcg_mem + 4 * GCGE_MAXCOLS;
  s->bcg.rnew = s->bcg_mem + 5 * GCGE_MAXCOLS;
  s->bcg.unl = s->bcg_int;
  s->bcg.nu = s->bcg_int + GCGE_MAXCOLS;
  s->bcg.nu_host = s->h_pinned_int;
  s->bcg.acol = s->bcg_mem + 6 * GCGE_MAXCOLS;
  s->bcg.bcol = reinterpret_cast<float*>(s->bcg_mem + 7 * GCGE_MAXCOLS);
  s->bcg.acolf = s->bcg.bcol + 64;  // 32 floats after the betas, still inside the slot
  s->bcg.mask = s->bcg_int + GCGE_MAXCOLS + 1;
  CU(cudaStreamSynchronize(s->st));
  if (p.use_shift == 1 || p.if_shift == 1) CHK(build_shift_op(s));
  (void)add;
  s->setup_done = true;
  return GCGE_CUDA_OK;
}

// ------------------------------------------------------------------ steps
#define KL(x)                 \
  do {                        \
    x;                        \
    s->launches++;            \
  } while (0)

static int sync(Solver* s) {
  CU(cudaStreamSynchronize(s->st));
  CU(cudaGetLastError());
  return GCGE_CUDA_OK;
}

static const GcgeDevCsr* Bptr(Solver* s) { return s->B ? &s->B->m : nullptr; }

// max |a - b| and max |b| over k columns (debug comparison of two products)
static __global__ void k_maxdiff(ColList<double> A, ColList<double> B, int k, int n,
                                 unsigned long long* out) {
  const int row = blockIdx.x * 256 + threadIdx.x;
  const int c = blockIdx.y;
  if (row >= n || c >= k) return;
  const double d = fabs(A.p[c][row] - B.p[c][row]);
  const double v = fabs(B.p[c][row]);
  atomicMax(out, (unsigned long long)__double_as_longlong(d));
  atomicMax(out + 1, (unsigned long long)__double_as_longlong(v));
}

// Products with at most this many outputs (k1 k2; the CholQR2 Gram and
// W R^-1 of a 10-column block) run on the FP64 FMA units: their FP64 work is
// below the fixed per-chunk cost of the tensor-core pipelines, and plain FP64
// is the reference's own arithmetic.
constexpr int kSmallProduct = 256;

// Tall-skinny Y = X C (+ beta Y) with the configured arithmetic.  With the
// environment variable GCGE_CUDA_CHECK_GEMM set, every tensor-core product is
// recomputed in FP64 and the largest difference is printed (diagnostics).
static void lincomb(Solver* s, const ColList<double>& X, int k1, const double* C, int ldc,
                    const ColList<double>& Y, int k2, double beta, bool balance = false) {
  if ((s->para.gemm == 1 || s->para.gemm == 2) && k1 > 0 && k1 * k2 > kSmallProduct) {
    static const bool check = getenv("GCGE_CUDA_CHECK_GEMM") != nullptr;
    if (check && beta == 0.0 && k2 <= (int)s->evec.size()) {
      // FP64 result into evec-sized debug columns
      static double* dbg = nullptr;
      static unsigned long long* dmx = nullptr;
      if (!dbg) {
        cudaMalloc(&dbg, sizeof(double) * (size_t)s->ldn * GCGE_MAXCOLS);
        cudaMalloc(&dmx, 16);
      }
      ColList<double> D;
      for (int j = 0; j < k2; j++) D.p[j] = dbg + (size_t)j * s->ldn;
      gcge::lincomb_f64(X, k1, C, ldc, D, k2, 0.0, s->n, s->st);
      gcge::lincomb_oz(X, k1, C, ldc, Y, k2, beta, s->n, s->oz_scratch, s->st, balance);
      cudaMemsetAsync(dmx, 0, 16, s->st);
      k_maxdiff<<<dim3((s->n + 255) / 256, k2), 256, 0, s->st>>>(Y, D, k2, s->n, dmx);
      unsigned long long h[2];
      cudaMemcpyAsync(h, dmx, 16, cudaMemcpyDeviceToHost, s->st);
      cudaStreamSynchronize(s->st);
      double d, v;
      memcpy(&d, &h[0], 8);
      memcpy(&v, &h[1], 8);
      fprintf(stderr, "[gemm-check] iter %d k1 %d k2 %d ldc %d maxdiff %.3e maxval %.3e\n",
              s->num_iter, k1, k2, ldc, d, v);
      return;
    }
    gcge::lincomb_oz(X, k1, C, ldc, Y, k2, beta, s->n, s->oz_scratch, s->st, balance);
  } else {
    gcge::lincomb_f64(X, k1, C, ldc, Y, k2, beta, s->n, s->st);
  }
}

// Tall-skinny G = V^T W with the configured arithmetic.
static void gram(Solver* s, const ColList<double>& V, int k1, const ColList<double>& W, int k2,
                 double* G, int ldg, bool sym) {
  if ((s->para.gemm == 1 || s->para.gemm == 3) && k1 * k2 > kSmallProduct)
    gcge::gram_oz(V, k1, W, k2, s->n, G, ldg, sym, s->partial, s->st);
  else
    gcge::gram_f64(V, k1, W, k2, s->n, G, ldg, sym, s->partial, s->st);
}

// Digit planes of V[0:k] (the columns from plane_n on are cut; those before
// were cut in this window from the same buffers).  Returns false when the
// configuration has no planes.
static bool planes_cover(Solver* s, int k) {
  if (!s->planes || k <= 0) return false;
  if (k > s->plane_n) {
    gcge::cut_planes(cols(s->V, s->plane_n, k), k - s->plane_n, s->n, s->planes, s->mx,
                     s->plane_n, s->st);
    s->launches++;
    for (int i = s->plane_n; i < k; i++) s->plane_src[i] = s->V[i];
    s->plane_n = k;
  }
  return true;
}

// true when the planes hold V[start:end] as it is now
static bool planes_valid(const Solver* s, int start, int end) {
  if (!s->planes || end > s->plane_n) return false;
  for (int i = start; i < end; i++)
    if (s->plane_src[i] != s->V[i]) return false;
  return true;
}

// Y_j = s_j X_j (host scalars), used for the W initial guess / rhs scaling.
static __global__ void k_scale_copy(ColList<double> X, ColList<double> Y, DblList sc, int k,
                                    int n) {
  const int row = blockIdx.x * 256 + threadIdx.x;
  const int c = blockIdx.y;
  if (row >= n || c >= k) return;
  const double f = sc.v[c];
  Y.p[c][row] = (f == 1.0) ? X.p[c][row] : f * X.p[c][row];
}

static DblList scalars(const std::vector<double>& v) {
  DblList c;
  for (size_t i = 0; i < v.size(); i++) c.v[i] = v[i];
  return c;
}

static __global__ void k_frob(const double* __restrict__ G, int m, int k, double* out) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int e = threadIdx.x; e < m * k; e += blockDim.x) s = fma(G[e], G[e], s);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sqrt(sh[0]);
}

// X_c[i] <- pseudo-random in [-1, 1): splitmix64 of (row, column, seed)
static __global__ void k_fill_random(ColList<double> X, int n, unsigned seed) {
  const int c = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    unsigned long long z = ((unsigned long long)c << 32 | (unsigned)i) +
                           0x9E3779B97F4A7C15ull * (seed + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    X.p[c][i] = (double)(z >> 11) * 0x1.0p-52 - 1.0;
  }
}

// V[start:*end] <- B-orthonormal, dropping dependent columns.  CholQR with
// dropping, applied twice.  The scratch columns are T[0:k] (swapped with V).
static int cholqr2(Solver* s, std::vector<double*>& V, int start, int* end,
                   std::vector<double*>& T) {
  for (int pass = 0; pass < 2; pass++) {
    const int k = *end - start;
    if (k <= 0) return GCGE_CUDA_OK;
    if (k > (int)T.size()) return set_err(GCGE_CUDA_ERR_STATE, "cholqr2: block too wide");
    ColList<double> W = cols(V, start, *end);
    ColList<double> BW = cols(T, 0, k);
    KL(gcge::apply_b_f64(Bptr(s), W, BW, k, s->n, s->st));
    KL(gram(s, W, k, BW, k, s->sub_tmp2, k, true));
    int* kept = s->d_int;
    int* nk = s->d_int + GCGE_MAXCOLS;
    KL(gcge::chol_drop(k, s->sub_tmp2, k, s->para.orth_zero_tol, s->sub_tmp, kept, nk,
                       s->jac_work, s->st));
    int h[GCGE_MAXCOLS + 1];
    CU(cudaMemcpyAsync(h, s->d_int, sizeof(int) * (GCGE_MAXCOLS + 1), cudaMemcpyDeviceToHost, s->st));
    CHK(sync(s));
    const int m = h[GCGE_MAXCOLS];
    ColList<double> Wk;
    for (int j = 0; j < m; j++) Wk.p[j] = V[start + h[j]];
    ColList<double> out = cols(T, 0, m);
    // the columns of W can differ by orders of magnitude (R^{-1} undoes it):
    // balance them before the fixed-point splitting
    KL(lincomb(s, Wk, m, s->sub_tmp, k, out, m, 0.0, true));
    // W <- V_tmp[0:m]; the kept old W buffers become V_tmp[0:m] and the
    // dropped ones are parked beyond the new end, so the pool stays a
    // permutation of the same buffers
    std::vector<double*> oldW(V.begin() + start, V.begin() + *end);
    std::vector<char> used(k, 0);
    for (int j = 0; j < m; j++) used[h[j]] = 1;
    for (int j = 0; j < m; j++) V[start + j] = T[j];
    int t = 0, d = start + m;
    for (int j = 0; j < k; j++) {
      if (used[j]) T[t++] = oldW[j];
      else V[d++] = oldW[j];
    }
    *end = start + m;
  }
  return GCGE_CUDA_OK;
}

// GCGE_StableMultiOrthonormalization (src/gcge_orthogonal.c:1909-2019):
// block CGS of V[start:*end] against V[0:start] with re-orthogonalisation
// until ||V1^T B V2||_F <= scbgs_reorth_tol, then self-orthonormalisation.
// On the tensor-core path a diagonal B is folded into the Gram and the update
// W <- W - V1 G is one product with beta = 1.
static int w_orth(Solver* s, int start, int* end) {
  const Para& p = s->para;
  const bool oz = (p.gemm == 1 || p.gemm == 3);
  const bool ozl = (p.gemm == 1 || p.gemm == 2);
  const double* bdiag = s->B ? s->B->m.diag : nullptr;
  // [X, P] is fixed during the orthogonalisation and the Rayleigh-Ritz step
  // that follows: its digit planes are cut once here
  s->plane_n = 0;
  const bool pl = oz && start > 0 && *end - start <= s->bs && planes_cover(s, start);
  if (start > 0) {
    double vi = 1.0;
    int it = 0;
    while (vi > p.scbgs_reorth_tol + 2.220446049250313e-16) {
      it++;
      const int l2 = *end - start;
      if (l2 <= 0) break;
      ColList<double> W = cols(s->V, start, *end);
      ColList<double> T = cols(s->V_tmp, 0, l2);
      ColList<double> V1 = cols(s->V, 0, start);
      if (pl) {
        // W's planes (B W, or W weighted by a diagonal B), then the plane Gram
        if (bdiag || !s->B) {
          KL(gcge::cut_planes(W, l2, s->n, s->wplanes, s->bs, 0, s->st, bdiag));
        } else {
          KL(gcge::apply_b_f64(Bptr(s), W, T, l2, s->n, s->st));
          KL(gcge::cut_planes(T, l2, s->n, s->wplanes, s->bs, 0, s->st));
        }
        KL(gcge::gram_oz_planes(s->planes, s->mx, 0, start, s->wplanes, s->bs, 0, l2, s->n,
                                s->sub_tmp2, start, s->partial, s->st));
      } else if (oz && (bdiag || !s->B)) {
        KL(gcge::gram_oz(V1, start, W, l2, s->n, s->sub_tmp2, start, false, s->partial, s->st,
                         bdiag));
      } else {
        KL(gcge::apply_b_f64(Bptr(s), W, T, l2, s->n, s->st));
        KL(gram(s, V1, start, T, l2, s->sub_tmp2, start, false));
      }
      if (ozl) {
        // W <- W - V1 G
        KL(gcge::lincomb_oz(V1, start, s->sub_tmp2, start, W, l2, 1.0, s->n, s->oz_scratch, s->st,
                            false, true));
      } else {
        KL(lincomb(s, V1, start, s->sub_tmp2, start, T, l2, 0.0));
        KL(gcge::axpby_f64(-1.0, T, 1.0, W, l2, s->n, s->st));
      }
      // ||G||_F is an absolute measure (W is not normalised yet), so the update
      // of the last pass is kept even when ||G||_F is below the tolerance
      KL((k_frob<<<1, 256, 0, s->st>>>(s->sub_tmp2, start, l2, s->d_small)));
      double h = 0.0;
      CU(cudaMemcpyAsync(&h, s->d_small, sizeof(double), cudaMemcpyDeviceToHost, s->st));
      CHK(sync(s));
      vi = h;
      s->stats.w_orth_passes++;
      if (it >= p.max_reorth_time) break;
    }
  }
  CHK(cholqr2(s, s->V, start, end, s->V_tmp));
  // the orthonormal W joins the planes for the Rayleigh-Ritz Gram
  if (pl) planes_cover(s, *end);
  return GCGE_CUDA_OK;
}

// GCGE_ComputeSubspaceMatrixVTAW (src/gcge_rayleighritz.c:40-90); A W goes
// to evec[0:w_length] as scratch, as in the reference.
static __global__ void k_mirror_upper(double* __restrict__ G, int ld, int k) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= k * k) return;
  const int i = e % k, j = e / k;
  if (i > j) G[i + (size_t)j * ld] = G[j + (size_t)i * ld];
}

static int vtaw(Solver* s, int start_W, int start_V, int end_V, double* smat) {
  const int wl = end_V - start_W, xpl = end_V - wl;
  ColList<double> W = cols(s->V, start_W, end_V);
  ColList<double> AW = cols(s->evec, 0, wl);
  KL(gcge::spmm_f64(s->A->m, W, AW, wl, s->st));
  CU(cudaMemsetAsync(smat, 0, sizeof(double) * (size_t)end_V * wl, s->st));
  // one Gram [V[start_V:xpl], W]^T (A W), then the W^T A W block is made
  // symmetric from its upper triangle (the "sym" product of the reference)
  ColList<double> VV = cols(s->V, start_V, end_V);
  if (planes_valid(s, start_V, end_V) && wl <= s->bs) {
    KL(gcge::cut_planes(AW, wl, s->n, s->wplanes, s->bs, 0, s->st));
    KL(gcge::gram_oz_planes(s->planes, s->mx, start_V, end_V - start_V, s->wplanes, s->bs, 0, wl,
                            s->n, smat + start_V, end_V, s->partial, s->st));
  } else
    KL(gram(s, VV, end_V - start_V, AW, wl, smat + start_V, end_V, false));
  KL((k_mirror_upper<<<(wl * wl + 127) / 128, 128, 0, s->st>>>(smat + xpl, end_V, wl)));
  return GCGE_CUDA_OK;
}

// GCGE_ComputeSubspaceMatrix (src/gcge_rayleighritz.c:121-190).
static int compute_subspace_matrix(Solver* s) {
  const int dim_xp = s->dim_xp, ldm = s->dim_xpw;
  if (dim_xp != 0) {
    const int lde = s->last_dim_xpw, dim_x = s->dim_x, dim_p = dim_xp - dim_x;
    const double* pp = s->sub_evec + (size_t)dim_x * lde;
    if (dim_p > 0)
      KL(gcge::dgemm_small(false, false, true, lde, dim_p, lde, 1.0, s->sub_mat, lde, pp, lde, 0.0,
                           s->sub_tmp, lde, s->st));
    CU(cudaMemsetAsync(s->sub_mat, 0, sizeof(double) * (size_t)ldm * ldm, s->st));
    if (dim_p > 0)
      KL(gcge::dgemm_small(true, false, false, dim_p, dim_p, lde, 1.0, pp, lde, s->sub_tmp, lde,
                           0.0, s->sub_mat + (size_t)dim_x * ldm + dim_x, ldm, s->st));
    KL(gcge::set_diag(s->sub_mat, ldm, s->d_eval, dim_x, s->st));
  }
  CHK(vtaw(s, dim_xp, s->num_soft_locked, ldm, s->sub_mat + (size_t)dim_xp * ldm));
  s->plane_n = 0;  // the X and P updates change the basis next
  if (s->if_shift_run == 1) KL(gcge::add_diag(s->sub_mat, ldm, s->shift_run, ldm, s->st));  // :181-189
  return GCGE_CUDA_OK;
}

// GCGE_SortByMagnitude (src/gcge_rayleighritz.c:842-874): quicksort of
// a[left..right] by |a| with the first element as pivot, carrying idx.  Kept
// as the reference's partition scheme so that ties order the same way.
static void sort_by_magnitude(double* a, int* idx, int left, int right) {
  if (left > right) return;
  int i = left, j = right;
  const int pidx = idx[left];
  const double piv = a[left], pm = fabs(a[left]);
  while (i != j) {
    while (fabs(a[j]) >= pm && j > i) j--;
    if (j > i) {
      idx[i] = idx[j];
      a[i++] = a[j];
    }
    while (fabs(a[i]) <= pm && j > i) i++;
    if (j > i) {
      idx[j] = idx[i];
      a[j--] = a[i];
    }
  }
  a[i] = piv;
  idx[i] = pidx;
  sort_by_magnitude(a, idx, left, i - 1);
  sort_by_magnitude(a, idx, i + 1, right);
}

// GCGE_ComputeSubspaceEigenpairs (src/gcge_rayleighritz.c:507-805), serial
// branch.  eval_type "sm" computes all pairs and moves the smallest |lambda|
// first (:748-769); a shift is taken off the Ritz values and the diagonal
// afterwards (:771-783).
static int compute_subspace_eigenpairs(Solver* s) {
  const int ldm = s->dim_xpw;
  const int sl = s->unlock[0];
  s->num_soft_locked = sl;
  const bool sm = s->para.eval_type == 1;
  const int iu_sa = (s->max_dim_x < ldm) ? s->max_dim_x : ldm;
  const int iu = sm ? ldm : iu_sa;
  const int nw = s->dim_xpw - s->dim_xp;
  if (sl > 0 && nw > 0)
    CU(cudaMemset2DAsync(s->sub_mat + (size_t)s->dim_xp * ldm, sizeof(double) * ldm, 0,
                         sizeof(double) * sl, nw, s->st));
  const int nrows = ldm - sl;
  KL(gcge::jacobi_eig(nrows, s->sub_mat + (size_t)sl * ldm + sl, ldm, s->d_eval + sl,
                      s->sub_evec + (size_t)sl * ldm + sl, ldm, 1, iu - sl, s->jac_work,
                      s->d_int + 2 * GCGE_MAXCOLS, s->st));
  CU(cudaMemcpyAsync(s->eval.data(), s->d_eval, sizeof(double) * s->mx, cudaMemcpyDeviceToHost,
                     s->st));
  int status = 0;
  CU(cudaMemcpyAsync(&status, s->d_int + 2 * GCGE_MAXCOLS, sizeof(int), cudaMemcpyDeviceToHost,
                     s->st));
  CHK(sync(s));
  if (status < 0) return set_err(GCGE_CUDA_ERR_NUMERIC, "subspace Jacobi did not converge");
  if (sm) {
    std::vector<int> ord(nrows);
    for (int i = 0; i < nrows; i++) ord[i] = i;
    sort_by_magnitude(s->eval.data() + sl, ord.data(), 0, nrows - 1);
    const int len = iu_sa - sl;
    if (len > 0) {
      IntList idx;
      for (int i = 0; i < len; i++) idx.v[i] = ord[i];
      double* blk = s->sub_evec + (size_t)sl * ldm;
      KL(gcge::gather_cols(blk, ldm, sl, nrows, idx, len, s->sub_tmp, ldm, s->st));
      CU(cudaMemcpy2DAsync(blk + sl, sizeof(double) * ldm, s->sub_tmp, sizeof(double) * ldm,
                           sizeof(double) * nrows, len, cudaMemcpyDeviceToDevice, s->st));
    }
  }
  if (s->if_shift_run == 1) {
    for (int i = sl; i < iu; i++) s->eval[i] -= s->shift_run;
    KL(gcge::add_diag(s->sub_mat, ldm, -s->shift_run, ldm, s->st));
  }
  if (sm || s->if_shift_run == 1) {
    CU(cudaMemcpyAsync(s->d_eval + sl, s->eval.data() + sl, sizeof(double) * (iu - sl),
                       cudaMemcpyHostToDevice, s->st));
    CHK(sync(s));
  }
  return GCGE_CUDA_OK;
}

// GCGE_ComputeX (src/gcge_xpw.c:47-76).
static int compute_x(Solver* s, int size_x, int size_v) {
  const int sx = s->num_soft_locked;
  if (size_x - sx <= 0) return GCGE_CUDA_OK;
  KL(lincomb(s, cols(s->V, sx, size_v), size_v - sx, s->sub_evec + (size_t)sx * size_v + sx,
             size_v, cols(s->evec, sx, size_x), size_x - sx, 0.0));
  return GCGE_CUDA_OK;
}

// GCGE_ComputeW + GCGE_BCG (src/gcge_xpw.c:118-260, src/gcge_cg.c:302-501).
static int compute_w(Solver* s) {
  const int ws = s->dim_xp, wl = s->unconv_bs;
  if (wl <= 0) return GCGE_CUDA_OK;
  ColList<double> X, Wc, R = cols(s->V_tmp, 0, wl);
  std::vector<double> rs(wl), wsc(wl);
  // the reference adds para->shift to lambda here whether or not if_shift is
  // set (src/gcge_xpw.c:158,166)
  const double sh = s->shift_run;
  for (int i = 0; i < wl; i++) {
    const int xi = s->unlock[i];
    X.p[i] = s->V[xi];
    Wc.p[i] = s->V[ws + i];
    const double lam = s->eval[xi];
    if (fabs(lam) <= 1.0) {
      rs[i] = lam + sh;
      wsc[i] = 1.0;
    } else {
      rs[i] = 1.0;
      wsc[i] = 1.0 / (lam + sh);
    }
  }
  // the block-CG operator: A, or A + shift B
  const GcgeDevCsr* Aop = &s->A->m;
  if (s->if_shift_run == 1) {
    if (!s->ash.rp) return set_err(GCGE_CUDA_ERR_STATE, "shift active without a shifted operator");
    if (!s->ash_valid || s->ash_sigma != sh) {
      KL((k_shift_values<<<4 * 152, 256, 0, s->st>>>(s->ash_av, s->ash_bv, sh, s->ash.v,
                                                      s->ash.v32, s->ash.nnz)));
      s->ash_sigma = sh;
      s->ash_valid = true;
    }
    Aop = &s->ash;
  }
  KL(gcge::apply_b_f64(Bptr(s), X, R, wl, s->n, s->st));
  dim3 g((s->n + 255) / 256, wl);
  KL((k_scale_copy<<<g, 256, 0, s->st>>>(R, R, scalars(rs), wl, s->n)));
  KL((k_scale_copy<<<g, 256, 0, s->st>>>(X, Wc, scalars(wsc), wl, s->n)));
  int launches = 0, steps;
  if (s->mls) {
    // a user block solver replaces the block CG (GCGE_OPS.MultiLinearSolver);
    // in the correction form (mixed precision, or w_form 1) it gets
    // rhs - A w0 and a zero start, and its solution e is the W block
    if (s->para.precision == 1 || s->para.w_form == 1) {
      ColList<double> AW = cols(s->evec, 0, wl);
      KL(gcge::spmm_f64(*Aop, Wc, AW, wl, s->st));
      KL(gcge::axpby_f64(-1.0, AW, 1.0, R, wl, s->n, s->st));
      for (int i = 0; i < wl; i++) CU(cudaMemsetAsync(Wc.p[i], 0, sizeof(double) * s->n, s->st));
    }
    const int rc = s->mls(s->mls_ctx, s->A, R.p, Wc.p, wl, s->n, (void*)s->st);
    if (rc != 0) return set_err(GCGE_CUDA_ERR_NUMERIC, "user linear solver returned %d", rc);
    return GCGE_CUDA_OK;
  }
  if (s->para.precision == 0) {
    if (s->para.w_form == 1) {
      // the correction form (see the mixed branch below) in FP64
      ColList<double> AW = cols(s->evec, 0, wl);
      KL(gcge::spmm_f64(*Aop, Wc, AW, wl, s->st));
      KL(gcge::axpby_f64(-1.0, AW, 1.0, R, wl, s->n, s->st));
      for (int i = 0; i < wl; i++) CU(cudaMemsetAsync(Wc.p[i], 0, sizeof(double) * s->n, s->st));
    }
    steps = gcge::bcg_run<double>(Aop->rp, Aop->ci, Aop->v, s->n, R, Wc,
                                  cols(s->CG_p, 0, wl), cols(s->evec, 0, wl), wl,
                                  s->para.cg_max_it, s->para.cg_rate, s->bcg, s->partial, s->st,
                                  &launches, Aop);
  } else {
    // Iterative-refinement form: the FP32 block CG solves A e = rhs - A w0
    // from e0 = 0 (the reference's CG iterates shifted by w0: same residuals,
    // same stopping rule), and the W block is e itself.  w0 is x scaled, and
    // x is a column of the basis W is orthogonalised against, so [X, P, e]
    // spans the subspace of [X, P, w0 + e].  Near convergence e is as small as
    // the eigen-residual: handing w0 + e to the orthogonalisation would
    // leave it to cancel w0 (rounding ~1e-16 |w0|) under an absolute stopping
    // test, and the renormalised remainder of a converged-looking column then
    // kept a coupling of (|w0| / |e|) 1e-16 to X (1e-5 on hub-localised
    // eigenvectors of a power-law graph, where the solve broke down).
    ColList<double> AW = cols(s->evec, 0, wl);
    KL(gcge::spmm_f64(*Aop, Wc, AW, wl, s->st));
    KL(gcge::axpby_f64(-1.0, AW, 1.0, R, wl, s->n, s->st));
    if (wl <= 32) {
      // row-interleaved FP32 vectors: one contiguous row per SpMM gather
      const size_t blk = (size_t)s->ldn * gcge::bcg_rows_width(wl);
      float* Rr = s->pool32;
      float* Xr = Rr + blk;
      float* Pr = Xr + blk;
      float* Wr = Pr + blk;
      KL(gcge::cols_to_rows_f32(R, wl, Rr, s->n, s->st));
      CU(cudaMemsetAsync(Xr, 0, sizeof(float) * blk, s->st));
      steps = gcge::bcg_run_rows_f32(Aop->rp, Aop->ci, Aop->v32, s->n, Rr, Xr, Pr, Wr,
                                     wl, s->para.cg_max_it, s->para.cg_rate, s->bcg, s->partial,
                                     s->st, &launches, Aop);
      KL(gcge::rows_to_cols_f64(Xr, wl, Wc, s->n, s->st));
    } else {
      ColList<float> fr = colsf(s->f_rhs, 0, wl), fx = colsf(s->f_x, 0, wl);
      KL(gcge::convert_f64_to_f32(R, fr, wl, s->n, s->st));
      for (int i = 0; i < wl; i++)
        CU(cudaMemsetAsync(fx.p[i], 0, sizeof(float) * s->n, s->st));
      steps = gcge::bcg_run<float>(Aop->rp, Aop->ci, Aop->v32, s->n, fr, fx,
                                   colsf(s->f_p, 0, wl), colsf(s->f_w, 0, wl), wl,
                                   s->para.cg_max_it, s->para.cg_rate, s->bcg, s->partial, s->st,
                                   &launches, Aop);
      KL(gcge::convert_f32_to_f64(fx, Wc, wl, s->n, s->st));
    }
  }
  s->launches += launches;
  if (steps < 0) return set_err(GCGE_CUDA_ERR_CUDA, "block CG: %s", cudaGetErrorString(cudaGetLastError()));
  s->stats.bcg_steps += steps;
  return GCGE_CUDA_OK;
}

// GCGE_ComputeP (src/gcge_xpw.c:329-478) with the P coefficients
// orthonormalised by GCGE_StableMultiOrthonormalizationInSubspace semantics.
static int compute_p(Solver* s) {
  double* coef = s->sub_evec;
  const int ldc = s->dim_xpw;
  int p_start = s->dim_x, p_ncols = s->unconv_bs;
  const int xx_nrows = s->last_dim_x;
  double* px = coef + (size_t)p_start * ldc;
  CU(cudaMemsetAsync(px, 0, sizeof(double) * (size_t)p_ncols * ldc, s->st));
  IntList idx;
  for (int c = 0; c < p_ncols; c++) idx.v[c] = s->unlock[c];
  KL(gcge::gather_cols(coef, ldc, xx_nrows, ldc - xx_nrows, idx, p_ncols, px + xx_nrows, ldc,
                       s->st));
  const int os = s->num_soft_locked;
  const int ol = ldc - os;
  p_start -= os;
  int p_end = p_start + p_ncols;
  double* Vc = coef + (size_t)os * ldc + os;
  if (p_start != 0) {
    for (int rc = 0; rc < s->para.max_reorth_time; rc++) {
      const int olen = p_end - p_start;
      KL(gcge::dgemm_small(true, false, false, p_start, olen, ol, 1.0, Vc, ldc,
                           Vc + (size_t)p_start * ldc, ldc, 0.0, s->sub_tmp, p_start, s->st));
      KL(gcge::dgemm_small(false, false, false, ol, olen, p_start, -1.0, Vc, ldc, s->sub_tmp,
                           p_start, 1.0, Vc + (size_t)p_start * ldc, ldc, s->st));
    }
  }
  KL(gcge::sub_mgs(Vc, ldc, ol, p_start, p_end, s->para.orth_zero_tol + 2.220446049250313e-16,
                   s->d_int + 3 * GCGE_MAXCOLS, s->st));
  int pe = 0;
  CU(cudaMemcpyAsync(&pe, s->d_int + 3 * GCGE_MAXCOLS, sizeof(int), cudaMemcpyDeviceToHost, s->st));
  CHK(sync(s));
  p_end = pe;
  p_ncols = p_end - p_start;
  p_end += os;
  const int nev = s->nev;
  const int pe_tmp = p_end - nev;
  if (pe_tmp > s->V_tmp_size) return set_err(GCGE_CUDA_ERR_STATE, "compute_p: V_tmp too small");
  KL(lincomb(s, cols(s->V, os, ldc), ldc - os, coef + (size_t)nev * ldc + os, ldc,
             cols(s->V_tmp, 0, pe_tmp), pe_tmp, 0.0));
  swap_cols(s->V, nev, p_end, s->V_tmp, 0);
  s->dim_xp = p_end;
  return GCGE_CUDA_OK;
}

// GCGE_CheckConvergence (src/gcge_eigsol.c:663-887) with the "R", "O" and
// absolute criteria (:704-721).  The residuals are computed on the device in
// chunks; the lock logic runs here.
static int check_convergence(Solver* s) {
  const int nev = s->nev;
  std::vector<int>& unlock = s->unlock;
  int max_conv_idx = unlock[0] - 1, start = unlock[0], flag = 0, nu = 0;
  int ncc = unlock[0];
  double* res = s->res.data();
  const double* eval = s->eval.data();
  const Para& p = s->para;
  const double ev_tol = p.ev_tol;
  unlock[0] = -1;
  const int chunk = 16;
  std::vector<double> r2(chunk), x2(chunk);
  bool stop = false;
  double max_res = 0.0, min_res = 0.0;
  int max_ind = 0, min_ind = 0;
  for (int c0 = start; c0 < nev && !stop; c0 += chunk) {
    const int k = (nev - c0 < chunk) ? nev - c0 : chunk;
    KL(gcge::residual_f64(s->A->m, Bptr(s), cols(s->evec, c0, c0 + k), s->d_eval + c0, k,
                          s->d_small, s->d_small + GCGE_MAXCOLS, s->partial, s->st));
    CU(cudaMemcpyAsync(r2.data(), s->d_small, sizeof(double) * k, cudaMemcpyDeviceToHost, s->st));
    CU(cudaMemcpyAsync(x2.data(), s->d_small + GCGE_MAXCOLS, sizeof(double) * k,
                       cudaMemcpyDeviceToHost, s->st));
    CHK(sync(s));
    for (int idx = c0; idx < c0 + k; idx++) {
      const double rn = sqrt(r2[idx - c0]), en = sqrt(x2[idx - c0]);
      double r = rn / en;
      const double ab = r;
      if (p.conv_type == 0) r /= (1.0 > fabs(eval[idx]) ? 1.0 : fabs(eval[idx]));
      else if (p.conv_type == 1) r /= (p.conv_omega_norm + fabs(eval[idx]));
      res[idx] = r;
      if (r < ev_tol && ab < 1e-2) {
        if (idx > 0) {
          if (res[idx - 1] < ev_tol) {
            max_conv_idx = idx;
            if (flag == 0) ncc = idx + 1;
          } else {
            const double me = fabs(eval[idx] - eval[idx - 1]) / fabs(eval[idx - 1]);
            if (me < p.multi_tol_for_lock) unlock[nu++] = idx;
            else max_conv_idx = idx;
          }
        } else {
          max_conv_idx = 0;
          ncc = 1;
        }
      } else {
        flag = 1;
        if (idx > 0 && res[idx - 1] < ev_tol) {
          int mmi = idx;
          for (int i = idx; i > 0; i--) {
            const double me = fabs(eval[i] - eval[i - 1]) / fabs(eval[i - 1]);
            if (me < p.multi_tol_for_lock) mmi = i - 1;
            else break;
          }
          for (int i = mmi; i <= idx; i++) unlock[nu++] = i;
        } else {
          unlock[nu++] = idx;
        }
      }
      if (idx == start) {
        max_res = min_res = r;
      } else {
        if (r > max_res) { max_res = r; max_ind = idx; }
        if (r < min_res) { min_res = r; min_ind = idx; }
      }
      if (idx - max_conv_idx > 9) {
        stop = true;
        break;
      }
    }
  }
  if (ncc < nev && nu < p.block_size) {
    if (nu > 0 && unlock[nu - 1] < nev - 1) {
      for (int i = nu; i < p.block_size; i++) {
        unlock[i] = unlock[i - 1] + 1;
        nu++;
        if (unlock[i] > nev - 2) break;
      }
    }
  }
  if (ncc < nev && unlock[0] < ncc) ncc = unlock[0];
  if (p.use_shift == 1) {  // src/gcge_eigsol.c:827-831
    s->if_shift_run = 1;
    s->shift_run = (eval[s->dim_x - 1] - 100.0 * eval[0]) / 99.0;
  }
  if (nu > p.block_size) nu = p.block_size;
  s->num_unlock = nu;
  s->num_conv_continuous = ncc;
  s->unconv_bs = nu;
  s->num_iter++;
  if (p.print_level > 0)
    fprintf(stderr, "[gcge-cuda] iter %d conv %d unconv_bs %d res[0]=%.3e\n", s->num_iter, ncc, nu,
            res[0]);
  // per-iteration report in the layout of GCGE_PrintIterationInfo
  // (src/gcge_para.c:461-514), whose iteration label is the count before this check
  const int it = s->num_iter - 1;
  if (p.print_conv == 1)
    printf("num_conv_continuous(%3d) = %3d; max_res(%3d) = %e; min_res(%3d) = %e;\n", it, ncc, it,
           max_res, it, min_res);
  if (p.print_eval == 1) {
    const char* ct = p.conv_type == 0 ? "relative_res" : p.conv_type == 1 ? "omega_res" : "abosolute_res";
    for (int i = 0; i < nev; i++) {
      printf("eval(%d,%3d) = %20.15e ; %s(%d,%3d) =  %20.15e ;", it, i + 1, eval[i], ct, it, i + 1,
             res[i]);
      if (res[i] < ev_tol) printf(" (converged)\n");
      else if (i == max_ind) printf(" (max)\n");
      else if (i == min_ind) printf(" (min)\n");
      else printf("\n");
    }
  }
  if (p.print_conv == 1 || p.print_eval == 1) fflush(stdout);
  return GCGE_CUDA_OK;
}

// Final report in the layout of GCGE_PrintFinalInfo (src/gcge_para.c:577-699):
// the eigenvalue / residual table, the iteration summary and the phase times
// (seconds of wall time here; the reference's are CPU user time).  The P step
// is timed as one phase (its orthonormalisation runs inside it): p_orth
// reads 0 and p_axpy holds the whole P step.
static void print_final_info(const Solver* s) {
  const Para& p = s->para;
  const GCGE_CUDA_STATS& t = s->stats;
  const double total = t.t_x_orth + t.t_x_axpy + t.t_p + t.t_w_line + t.t_w_orth + t.t_rr_mat +
                       t.t_rr_eig + t.t_conv;
  if (p.print_result) {
    printf("\nFinal eigenvalues and residual information:\n");
    printf("\n            eigenvalue           ");
    if (p.conv_type == 0) printf("relative residual\n\n");
    else if (p.conv_type == 1) printf("omega residual\n\n");
    else printf("abosolute residual\n\n");
    for (int i = 0; i < s->nev; i++) {
      printf("%5d  %20.15e  %20.15e ", i + 1, s->eval[i], s->res[i]);
      printf(s->res[i] < p.ev_tol ? " (converged)\n" : "\n");
    }
  }
  if (p.print_conv == 1) {
    printf("\nTotal gcg iteration: %d, total time: %.2lf. ", s->num_iter, total);
    if (s->num_conv_continuous == s->nev) printf("All %d eigenpairs converged! ", s->nev);
    else printf("%d converged, %d unconverged. ", s->num_conv_continuous, s->nev - s->num_conv_continuous);
  }
  if (p.print_final_part_time == 1) {
    printf("Use 1 process. block_size: %d", s->bs);
    printf("\nDetail time in total gcg iteration:\n"
           "Section Name        x_orth       x_axpy       p_orth       p_axpy   check_conv\n"
           "Section Time  %12.2lf %12.2lf %12.2lf %12.2lf %12.2lf\n",
           t.t_x_orth, t.t_x_axpy, 0.0, t.t_p, t.t_conv);
    if (total >= 1e-10)
      printf("Section Ratio %11.2lf%% %11.2lf%% %11.2lf%% %11.2lf%% %11.2lf%%\n", 100 * t.t_x_orth / total,
             100 * t.t_x_axpy / total, 0.0, 100 * t.t_p / total, 100 * t.t_conv / total);
    printf("Section Name        w_lsol       w_orth       rr_eig       rr_mat\n"
           "Section Time  %12.2lf %12.2lf %12.2lf %12.2lf\n",
           t.t_w_line, t.t_w_orth, t.t_rr_eig, t.t_rr_mat);
    if (total < 1e-10) printf("Total time is less than 1e-10, the percentege is not presented.\n");
    else
      printf("Section Ratio %11.2lf%% %11.2lf%% %11.2lf%% %11.2lf%%\n\n", 100 * t.t_w_line / total,
             100 * t.t_w_orth / total, 100 * t.t_rr_eig / total, 100 * t.t_rr_mat / total);
  }
  fflush(stdout);
}

static void print_para_info(const Solver* s) {
  const Para& p = s->para;
  static const char* ct[] = {"R", "O", "A"};
  printf("GCGE CUDA parameters: nev %d, block_size %d, ev_max_it %d, ev_tol %g, conv_type %s "
         "(omega norm %g), eval_type %s, cg_max_it %d, cg_rate %g, max_reorth_time %d, "
         "orth_zero_tol %g, scbgs_reorth_tol %g, multi_tol_for_lock %g, use_shift %d, "
         "precision %s, w_form %s, products %s\n",
         s->nev, s->bs, p.ev_max_it, p.ev_tol, ct[p.conv_type], p.conv_omega_norm,
         p.eval_type ? "sm" : "sa", p.cg_max_it, p.cg_rate, p.max_reorth_time, p.orth_zero_tol,
         p.scbgs_reorth_tol, p.multi_tol_for_lock, p.use_shift, p.precision ? "mixed" : "fp64",
         p.w_form ? "correction" : "reference", p.gemm ? "ozaki" : "fp64");
  fflush(stdout);
}

static int omega_norm(Solver* s) {
  const int nev = s->nev;
  double acc = 0.0;
  std::vector<double> r2(16), x2(16);
  for (int c0 = 0; c0 < nev; c0 += 16) {
    const int k = nev - c0 < 16 ? nev - c0 : 16;
    // d_eval is zero here: the residual kernel returns ||A x||^2 and ||x||^2
    KL(gcge::residual_f64(s->A->m, Bptr(s), cols(s->evec, c0, c0 + k), s->d_eval, k, s->d_small,
                          s->d_small + GCGE_MAXCOLS, s->partial, s->st));
    CU(cudaMemcpyAsync(r2.data(), s->d_small, sizeof(double) * k, cudaMemcpyDeviceToHost, s->st));
    CU(cudaMemcpyAsync(x2.data(), s->d_small + GCGE_MAXCOLS, sizeof(double) * k,
                       cudaMemcpyDeviceToHost, s->st));
    CHK(sync(s));
    for (int i = 0; i < k; i++) acc += r2[i] / x2[i];
  }
  s->para.conv_omega_norm = sqrt(acc / nev);
  return GCGE_CUDA_OK;
}

struct Timer {
  Solver* s;
  double* acc;
  double t0;
  Timer(Solver* s_, double* a) : s(s_), acc(a), t0(now_s()) {}
  void stop() {
    cudaStreamSynchronize(s->st);
    *acc += now_s() - t0;
  }
};

#define PHASE(field, call)                        \
  do {                                            \
    Timer tm_(s, &s->stats.field);                \
    int rc_ = (call);                             \
    tm_.stop();                                   \
    if (rc_ != GCGE_CUDA_OK) return rc_;          \
  } while (0)

// GCGE_Solve (src/gcge_eigsol.c:65-646).
extern "C" int GCGE_CUDA_SOLVER_Solve(GCGE_CUDA_SOLVER* s) {
  if (!s || !s->setup_done) return set_err(GCGE_CUDA_ERR_STATE, "Solve: call Setup first");
  if (!s->eval_user || (!s->evec_user && !s->evec_dev))
    return set_err(GCGE_CUDA_ERR_STATE, "Solve: eigenvalue/eigenvector arrays not set");
  Para& p = s->para;
  const int nev = s->nev, n = s->n;
  if (p.num_init_evec < 0) return set_err(GCGE_CUDA_ERR_ARG, "Solve: num_init_evec < 0");
  // the first num_init_evec columns of evec are the given start; the rest are
  // pseudo-random, as the reference fills them (src/gcge_eigsol.c:134-140)
  const int n_given = p.num_init_evec < nev ? p.num_init_evec : nev;
  const double t_start = now_s();
  if (p.print_para) print_para_info(s);
  memset(&s->stats, 0, sizeof(s->stats));
  s->launches = 0;
  s->eval.assign(s->mx, 0.0);
  s->res.assign(nev, 1.0);
  s->unlock.assign(s->max_dim_x + 1, 0);
  for (int i = 0; i < s->max_dim_x; i++) s->unlock[i] = i;
  s->dim_x = nev;
  s->dim_xp = 0;
  s->dim_xpw = nev;
  s->last_dim_x = 0;
  s->last_dim_xpw = 0;
  s->unconv_bs = nev < s->bs ? nev : s->bs;
  s->num_soft_locked = 0;
  s->num_iter = 0;
  s->num_conv_continuous = 0;
  s->if_shift_run = p.if_shift;
  s->shift_run = p.shift;
  CU(cudaMemsetAsync(s->d_eval, 0, sizeof(double) * s->mx, s->st));
  CU(cudaMemsetAsync(s->sub_mat, 0, sizeof(double) * (size_t)s->mx * s->mx, s->st));
  CU(cudaMemsetAsync(s->sub_evec, 0, sizeof(double) * (size_t)s->mx * s->mx, s->st));
  for (int j = 0; j < n_given; j++) {
    if (s->evec_dev)
      CU(cudaMemcpyAsync(s->evec[j], s->evec_dev + (size_t)j * n, sizeof(double) * n,
                         cudaMemcpyDeviceToDevice, s->st));
    else
      CU(cudaMemcpyAsync(s->evec[j], s->evec_user + (size_t)j * n, sizeof(double) * n,
                         cudaMemcpyHostToDevice, s->st));
  }
  if (n_given < nev) {
    dim3 g((n + 255) / 256, nev - n_given);
    KL((k_fill_random<<<g, 256, 0, s->st>>>(cols(s->evec, n_given, nev), n, 0u)));
  }
  // "O" criterion from a random start: ||A||_Omega = ||A Omega||_F / ||Omega||_F
  // over the normalised random block (src/gcge_eigsol.c:141-177); with a given
  // start the caller's conv_omega_norm stays
  if (p.conv_type == 1 && n_given == 0) CHK(omega_norm(s));
  // initial B-orthonormalisation of the given block (:219-242)
  {
    Timer tm(s, &s->stats.t_x_orth);
    // V is free before the first Rayleigh-Ritz step: its first nev columns
    // are the scratch block of the initial CholQR2
    std::vector<double*> scratch(s->V.begin(), s->V.begin() + nev);
    int dx = nev;
    int rc = cholqr2(s, s->evec, 0, &dx, scratch);
    // a block that loses columns (dependent or zero columns) is completed with
    // pseudo-random columns and orthonormalised again, as the reference does
    // for a short initial block (src/gcge_eigsol.c:134-217)
    for (int attempt = 1; rc == GCGE_CUDA_OK && dx < nev && attempt <= 8; attempt++) {
      dim3 g((n + 255) / 256, nev - dx);
      KL((k_fill_random<<<g, 256, 0, s->st>>>(cols(s->evec, dx, nev), n, (unsigned)attempt)));
      dx = nev;
      rc = cholqr2(s, s->evec, 0, &dx, scratch);
    }
    for (int j = 0; j < nev; j++) s->V[j] = scratch[j];
    tm.stop();
    if (rc) return rc;
    if (dx < nev) return set_err(GCGE_CUDA_ERR_NUMERIC, "initial block: %d independent columns", dx);
    s->dim_x = dx;
  }
  for (int j = 0; j < nev; j++)
    CU(cudaMemcpyAsync(s->V[j], s->evec[j], sizeof(double) * n, cudaMemcpyDeviceToDevice, s->st));
  s->dim_xpw = s->dim_x;
  s->last_dim_x = s->dim_x;
  s->dim_xp = 0;
  PHASE(t_rr_mat, compute_subspace_matrix(s));
  PHASE(t_rr_eig, compute_subspace_eigenpairs(s));
  PHASE(t_x_axpy, compute_x(s, nev, s->dim_xpw));
  PHASE(t_conv, check_convergence(s));
  if (s->num_conv_continuous < nev) {
    const int sl = s->num_soft_locked;
    swap_cols(s->V, sl, nev, s->evec, sl);
    s->dim_xp = s->dim_x;
    PHASE(t_w_line, compute_w(s));
    s->last_dim_xpw = s->dim_xpw;
    s->dim_xpw = s->dim_xp + s->unconv_bs;
    PHASE(t_w_orth, w_orth(s, s->dim_x, &s->dim_xpw));
    s->dim_xp = nev;
    PHASE(t_rr_mat, compute_subspace_matrix(s));
    PHASE(t_rr_eig, compute_subspace_eigenpairs(s));
    PHASE(t_x_axpy, compute_x(s, nev, s->dim_xpw));
    PHASE(t_conv, check_convergence(s));
  }
  while (s->num_conv_continuous < nev && s->num_iter < p.ev_max_it) {
    PHASE(t_p, compute_p(s));
    const int sl = s->num_soft_locked;
    swap_cols(s->V, sl, nev, s->evec, sl);
    PHASE(t_w_line, compute_w(s));
    s->last_dim_xpw = s->dim_xpw;
    s->dim_xpw = s->dim_xp + s->unconv_bs;
    PHASE(t_w_orth, w_orth(s, s->dim_xp, &s->dim_xpw));
    PHASE(t_rr_mat, compute_subspace_matrix(s));
    PHASE(t_rr_eig, compute_subspace_eigenpairs(s));
    s->last_dim_x = s->dim_x;
    // the reference sets dim_x = max_dim_x (src/gcge_eigsol.c:561) even when
    // the subspace has fewer Ritz vectors (dim_xpw < nev + 20 when
    // 2 * block_size < 20); its guard columns then come from stale
    // coefficients and show up as spurious zero eigenvalues.  Only the Ritz
    // vectors that exist are kept here.
    s->dim_x = s->max_dim_x < s->dim_xpw ? s->max_dim_x : s->dim_xpw;
    PHASE(t_x_axpy, compute_x(s, nev, s->dim_xpw));
    PHASE(t_conv, check_convergence(s));
  }
  // output (:636-642)
  memcpy(s->eval_user, s->eval.data(), sizeof(double) * nev);
  const int sl = s->num_soft_locked;
  for (int j = 0; j < nev; j++) {
    const double* src = (j < sl) ? s->V[j] : s->evec[j];
    if (s->evec_dev)
      CU(cudaMemcpyAsync(s->evec_dev + (size_t)j * n, src, sizeof(double) * n,
                         cudaMemcpyDeviceToDevice, s->st));
    else
      CU(cudaMemcpyAsync(s->evec_user + (size_t)j * n, src, sizeof(double) * n,
                         cudaMemcpyDeviceToHost, s->st));
  }
  CHK(sync(s));
  s->stats.num_iter = s->num_iter;
  s->stats.num_conv_continuous = s->num_conv_continuous;
  s->stats.kernel_launches = s->launches;
  s->stats.seconds = now_s() - t_start;
  if (p.print_result || p.print_conv || p.print_final_part_time) print_final_info(s);
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_SOLVER_GetEigenvalues(GCGE_CUDA_SOLVER* s, double** eval) {
  if (!s || !eval) return set_err(GCGE_CUDA_ERR_ARG, "GetEigenvalues: null");
  *eval = s->eval_user;
  return GCGE_CUDA_OK;
}
extern "C" int GCGE_CUDA_SOLVER_GetEigenvectors(GCGE_CUDA_SOLVER* s, double** evec) {
  if (!s || !evec) return set_err(GCGE_CUDA_ERR_ARG, "GetEigenvectors: null");
  *evec = s->evec_user;
  return GCGE_CUDA_OK;
}
extern "C" int GCGE_CUDA_SOLVER_GetResiduals(GCGE_CUDA_SOLVER* s, double* res) {
  if (!s || !res) return set_err(GCGE_CUDA_ERR_ARG, "GetResiduals: null");
  if ((int)s->res.size() < s->nev) return set_err(GCGE_CUDA_ERR_STATE, "GetResiduals: no solve yet");
  memcpy(res, s->res.data(), sizeof(double) * s->nev);
  return GCGE_CUDA_OK;
}
extern "C" int GCGE_CUDA_SOLVER_GetStats(GCGE_CUDA_SOLVER* s, GCGE_CUDA_STATS* st) {
  if (!s || !st) return set_err(GCGE_CUDA_ERR_ARG, "GetStats: null");
  *st = s->stats;
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_SOLVER_Free(GCGE_CUDA_SOLVER** solver) {
  if (!solver || !*solver) return GCGE_CUDA_OK;
  Solver* s = *solver;
  free_ws(s);
  if (s->ownA) GCGE_CUDA_MatDestroy((GCGE_CUDA_MAT**)&s->ownA);
  if (s->ownB) GCGE_CUDA_MatDestroy((GCGE_CUDA_MAT**)&s->ownB);
  delete s;
  *solver = nullptr;
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_SOLVER_Free_All(GCGE_CUDA_SOLVER** solver) {
  if (!solver || !*solver) return GCGE_CUDA_OK;
  Solver* s = *solver;
  if (s->owns_user) {
    free(s->eval_user);
    free(s->evec_user);
  }
  return GCGE_CUDA_SOLVER_Free(solver);
}

extern "C" GCGE_CUDA_SOLVER* GCGE_CUDA_Solver_Init(const GCGE_CUDA_CSR_HOST* A,
                                                   const GCGE_CUDA_CSR_HOST* B,
                                                   int num_eigenvalues, int argc, char* argv[]) {
  GCGE_CUDA_SOLVER* s = nullptr;
  if (GCGE_CUDA_SOLVER_Create(&s)) return nullptr;
  GCGE_CUDA_MAT *dA = nullptr, *dB = nullptr;
  if (GCGE_CUDA_MatCreateFromCSR(&dA, A)) {
    GCGE_CUDA_SOLVER_Free(&s);
    return nullptr;
  }
  s->ownA = dA;
  if (B) {
    if (GCGE_CUDA_MatCreateFromCSR(&dB, B)) {
      GCGE_CUDA_SOLVER_Free(&s);
      return nullptr;
    }
    s->ownB = dB;
  }
  if (num_eigenvalues != -1) s->para.nev = num_eigenvalues;
  if (GCGE_CUDA_SOLVER_SetFromCommandLine(s, argc, argv)) {
    GCGE_CUDA_SOLVER_Free(&s);
    return nullptr;
  }
  const int nev = s->para.nev;
  s->eval_user = (double*)calloc(nev, sizeof(double));
  s->evec_user = (double*)calloc((size_t)nev * A->N_Rows, sizeof(double));
  s->owns_user = true;
  s->A = dA;
  s->B = dB;
  if (GCGE_CUDA_SOLVER_Setup(s)) {
    GCGE_CUDA_SOLVER_Free_All(&s);
    return nullptr;
  }
  return s;
}
