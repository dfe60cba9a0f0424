// GCGE_CUDA_PASE_Solve: a multilevel correction eigensolver on the device,
// the GPU counterpart of the reference's PASE add-on (pase/src/pase_solver.c,
// PASE_EigenSolver at :17-82, PASE_Mg_solve at :443-503, the two-grid cycle
// PASE_Mg_cycle at :596-627), on the AMG hierarchy of gcge_cuda_amg.cu in
// place of the BoomerAMG hierarchy the reference converts from hypre
// (pase/src/pase_mg.c:101-131).
//
// The method (the reference's, restated on device data):
//   * B_l = P_l^T B_{l-1} P_l down to the auxiliary level H (MatPtAP in
//     pase_mg.c);
//   * initial pairs: the GCG solver on (A_H, B_H) for pase_nev = nev + more_nev
//     pairs (PASE_Direct_solve, :666-696), prolonged to the finest level;
//   * per cycle on the finest level:
//       smoothing: a few AMG-preconditioned CG steps on A u_i = lambda_i B u_i
//       from u_i (PASE_Mg_smoothing, :1114-1187, which runs multigrid-
//       preconditioned block CG the same way);
//       auxiliary problem on V_H + span(U): A_aux = [A_H, R A U; (R A U)^T,
//       U^T A U], B_aux likewise (PASE_Aux_matrix_set_by_pase_matrix,
//       :741-808), solved by the GCG solver from [0; e_i]
//       (PASE_Mg_set_pase_aux_vector, :811-852; PASE_Aux_direct_solve,
//       :902-946);
//       prolongation u_i = P y_H,i + U alpha_i
//       (PASE_Mg_prolong_from_pase_aux_vector, :1071-1112);
//       convergence of the first nev pairs by their residual
//       (PASE_Mg_error_estimate, :1189-1312).
// Device design: the auxiliary matrices are explicit device CSR matrices of
// n_H + pase_nev rows whose last pase_nev rows are dense (the heavy-row path of
// the SpMM takes them), built once and refilled in place each cycle; the
// auxiliary solver is set up once and re-solved from the new start.  Every
// vector operation runs on the GPU; the host sequences the cycle and reads the
// pase_nev eigenvalues and residual norms once per cycle.
// Differences from the reference (documented simplifications): a fixed
// auxiliary level instead of its run-time search over levels
// (PASE_Mg_get_new_aux_coarse_level, :522-570), no locking of converged pairs
// between cycles (every pair is recomputed), one smoothing between auxiliary
// solves (its post-smoothing and the next pre-smoothing are consecutive).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <vector>

#include "../../include/gcge_cuda.h"
#include "gcge_cuda_amg.cuh"
#include "gcge_cuda_common.cuh"

int gcge_record_error(int code, const char* msg);

namespace {

using gcge::amg::View;

#define PASE_CU(call)                                                                     \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      char b_[256];                                                                       \
      snprintf(b_, sizeof b_, "PASE: %s (%s:%d)", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return gcge_record_error(GCGE_CUDA_ERR_CUDA, b_);                                   \
    }                                                                                     \
  } while (0)

#define PASE_CHK(expr)          \
  do {                          \
    const int rc_ = (expr);     \
    if (rc_ != GCGE_CUDA_OK) return rc_; \
  } while (0)

GcgeDevCsr csr_of(const View& v) {
  GcgeDevCsr m;
  m.n = v.rows;
  m.nnz = v.nnz;
  m.rp = v.rp;
  m.ci = v.ci;
  m.v = v.v;
  return m;
}

ColList<double> cols(double* base, size_t ld, int k) {
  ColList<double> c;
  for (int j = 0; j < k; j++) c.p[j] = base + (size_t)j * ld;
  return c;
}

// auxiliary row pointers: rows r < nH hold A_H's row r then the k border
// entries; the k last rows are dense (nH + k entries)
__global__ void k_aux_rowptr(int nH, int k, const int* __restrict__ rpH, int* __restrict__ rp) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = nH + k;
  if (r > n) return;
  if (r <= nH)
    rp[r] = rpH[r] + r * k;
  else
    rp[r] = rpH[nH] + nH * k + (r - nH) * (nH + k);
}

// auxiliary values (and, with ci != null, columns): AHh is nH x k (column j at
// AHh + j * nH), Ahh is k x k (column-major, ld k)
__global__ void k_aux_fill_sparse(int nH, int k, const int* __restrict__ rpH,
                                  const int* __restrict__ ciH, const double* __restrict__ vH,
                                  const double* __restrict__ AHh, const int* __restrict__ rp,
                                  int* __restrict__ ci, double* __restrict__ v) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nH) return;
  int o = rp[r];
  for (int e = rpH[r]; e < rpH[r + 1]; e++, o++) {
    if (ci) ci[o] = ciH[e];
    v[o] = vH[e];
  }
  for (int j = 0; j < k; j++, o++) {
    if (ci) ci[o] = nH + j;
    v[o] = AHh[(size_t)j * nH + r];
  }
}

__global__ void k_aux_fill_dense(int nH, int k, const double* __restrict__ AHh,
                                 const double* __restrict__ Ahh, const int* __restrict__ rp,
                                 int* __restrict__ ci, double* __restrict__ v) {
  const int i = blockIdx.y;  // dense row nH + i
  const int w = nH + k;
  const size_t o = (size_t)rp[nH + i];
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < w; c += gridDim.x * blockDim.x) {
    if (ci) ci[o + c] = c;
    v[o + c] = c < nH ? AHh[(size_t)i * nH + c] : Ahh[(size_t)(c - nH) * k + i];
  }
}

__global__ void k_to32(size_t n, const double* __restrict__ a, float* __restrict__ b) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

// Y = [0; I] (n_aux x k, column-major ld n_aux): the current vectors as the start
__global__ void k_aux_start(int nH, int k, double* __restrict__ Y) {
  const int j = blockIdx.y;
  const int n = nH + k;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    Y[(size_t)j * n + r] = (r == nH + j) ? 1.0 : 0.0;
}

// columns scaled by host-given factors
__global__ void k_scale_cols(ColList<double> X, DblList s, int k, int n) {
  const int j = blockIdx.y;
  if (j >= k) return;
  const double a = s.v[j];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    X.p[j][i] *= a;
}

int grid_of(long long n) { return (int)std::min<long long>((n + 255) / 256, 4 * 152); }

// Y_c = R X_c for the restriction R (rows of a few hundred entries: an
// aggregate's smoothed support): one warp per (row, group of RW columns), the
// lanes striding over the row's entries, then a shuffle tree per column (a
// fixed order).  Thread-per-row gathers serialise a whole row per thread.
constexpr int RW = 8;
__global__ void k_restrict_warp(int nr, const int* __restrict__ rp, const int* __restrict__ ci,
                                const double* __restrict__ v, ColList<double> X, ColList<double> Y,
                                int k) {
  const int row = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= nr) return;  // whole warps leave together
  const int c0 = blockIdx.y * RW;
  const int nc = min(RW, k - c0);
  double s[RW];
#pragma unroll
  for (int c = 0; c < RW; c++) s[c] = 0.0;
  const int e1 = rp[row + 1];
  for (int e = rp[row] + lane; e < e1; e += 32) {
    const int j = ci[e];
    const double a = v[e];
#pragma unroll
    for (int c = 0; c < RW; c++)
      if (c < nc) s[c] = fma(a, X.p[c0 + c][j], s[c]);
  }
#pragma unroll
  for (int c = 0; c < RW; c++) {
    double t = s[c];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0 && c < nc) Y.p[c0 + c][row] = t;
  }
}

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Pase {
  cudaStream_t st = nullptr;
  int n = 0, nH = 0, k = 0, H = 1;
  std::vector<View> Bchain;     // B_1 .. B_H (owned)
  View Bid;                     // identity (owned) when B is the identity
  GCGE_CUDA_MAT* AH = nullptr;  // level-H operators for the initial solve
  GCGE_CUDA_MAT* BH = nullptr;
  GCGE_CUDA_MAT* auxA = nullptr;
  GCGE_CUDA_MAT* auxB = nullptr;
  GCGE_CUDA_SOLVER* aux = nullptr;
  double* U = nullptr;      // n x k current vectors
  double* Z = nullptr;      // n x k (prolonged, then the new U)
  double* AU = nullptr;     // n x k
  double* BU = nullptr;     // n x k
  double* rhs = nullptr;    // n x 32 smoothing right-hand sides
  std::vector<double*> lvl; // per level 1 .. H - 1: n_l x k transfers
  double* RH = nullptr;     // nH x k restricted block (A, then B)
  double* RH2 = nullptr;
  double* hh = nullptr;     // k x k Gram
  uint8_t* upl = nullptr;   // digit planes of U (k columns), cut once per cycle
  uint8_t* mpl = nullptr;   // digit planes of A U, then of B U
  double* Yaux = nullptr;   // n_aux x k
  double* partial = nullptr;
  size_t partial_len = 0;
  double* dlam = nullptr;   // k eigenvalues on the device
  double* rn = nullptr;     // k residual norms^2, then k norms^2
  void* lcs = nullptr;      // scratch of the tensor-core linear combination
  std::vector<double> lam;

  ~Pase() {
    if (aux) GCGE_CUDA_SOLVER_Free(&aux);
    GCGE_CUDA_MatDestroy(&auxA);
    GCGE_CUDA_MatDestroy(&auxB);
    GCGE_CUDA_MatDestroy(&AH);
    GCGE_CUDA_MatDestroy(&BH);
    for (auto& b : Bchain) gcge::amg::free_view(b);
    gcge::amg::free_view(Bid);
    for (double* p : {U, Z, AU, BU, rhs, RH, RH2, hh, Yaux, partial, dlam, rn}) cudaFree(p);
    cudaFree(lcs);
    cudaFree(upl);
    cudaFree(mpl);
    for (double* p : lvl) cudaFree(p);
    if (st) cudaStreamDestroy(st);
  }
};

template <typename T>
int dalloc(T** p, size_t count) {
  *p = nullptr;
  if (cudaMalloc(p, sizeof(T) * (count > 0 ? count : 1)) != cudaSuccess) {
    cudaGetLastError();
    return gcge_record_error(GCGE_CUDA_ERR_ALLOC, "PASE: device allocation failed");
  }
  return GCGE_CUDA_OK;
}

// a GCGE_CUDA_MAT copy of a device view (the solver's matrix type)
int mat_from_view(const View& v, GCGE_CUDA_MAT** out) {
  return GCGE_CUDA_MatCreate(out, v.rows, v.rp, v.ci, v.v, 1);
}

// X_0 = P_0 P_1 ... P_{H-1} X_H (k columns; X_H with leading dimension ldh)
int prolong_chain(Pase& s, const GCGE_CUDA_AMG* amg, const double* XH, size_t ldh, double* X0) {
  const double* src = XH;
  size_t lds = ldh;
  for (int l = s.H - 1; l >= 0; l--) {
    const View P = gcge::amg::prolong(amg, l);
    double* dst = l == 0 ? X0 : s.lvl[l - 1];
    gcge::spmm_f64(csr_of(P), cols(const_cast<double*>(src), lds, s.k), cols(dst, P.rows, s.k), s.k,
                   s.st);
    src = dst;
    lds = P.rows;
  }
  PASE_CU(cudaGetLastError());
  return GCGE_CUDA_OK;
}

// XH = R_{H-1} ... R_0 X0 into dst (nH x k)
int restrict_chain(Pase& s, const GCGE_CUDA_AMG* amg, const double* X0, double* dst) {
  const double* src = X0;
  size_t lds = s.n;
  for (int l = 0; l < s.H; l++) {
    const View R = gcge::amg::restrict_to(amg, l);
    double* out = l == s.H - 1 ? dst : s.lvl[l];
    const dim3 g((unsigned)(((size_t)R.rows * 32 + 255) / 256), (unsigned)((s.k + RW - 1) / RW));
    k_restrict_warp<<<g, 256, 0, s.st>>>(R.rows, R.rp, R.ci, R.v,
                                         cols(const_cast<double*>(src), lds, s.k),
                                         cols(out, R.rows, s.k), s.k);
    src = out;
    lds = R.rows;
  }
  PASE_CU(cudaGetLastError());
  return GCGE_CUDA_OK;
}

int set_params(GCGE_CUDA_SOLVER* so, int nev, double tol, int max_it) {
  PASE_CHK(GCGE_CUDA_SOLVER_SetNumEigen(so, nev));
  PASE_CHK(GCGE_CUDA_SOLVER_SetParamDouble(so, "ev_tol", tol));
  PASE_CHK(GCGE_CUDA_SOLVER_SetParamInt(so, "ev_max_it", max_it));
  PASE_CHK(GCGE_CUDA_SOLVER_SetParamInt(so, "precision", 0));
  return GCGE_CUDA_OK;
}

}  // namespace

extern "C" void GCGE_CUDA_PASE_DefaultParam(GCGE_CUDA_PASE_PARAM* p) {
  if (!p) return;
  p->more_nev = 10;
  p->aux_level = 1;
  p->max_cycles = 60;
  p->smooth_steps = 2;
  p->aux_max_it = 3;
  p->initial_max_it = 300;
  p->tol = 1e-10;
  p->initial_tol = 1e-8;
  p->aux_tol = 1e-12;
}

extern "C" int GCGE_CUDA_PASE_Solve(const GCGE_CUDA_MAT* A, const GCGE_CUDA_MAT* B,
                                    GCGE_CUDA_AMG* amg, int nev, const GCGE_CUDA_PASE_PARAM* prm,
                                    double* eval, double* evec, GCGE_CUDA_PASE_STATS* stats) {
  GCGE_CUDA_PASE_PARAM p;
  GCGE_CUDA_PASE_DefaultParam(&p);
  if (prm) p = *prm;
  if (!A || !amg || nev < 1 || !eval || !evec)
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "PASE_Solve: bad arguments");
  const int nlev = gcge::amg::levels(amg);
  const View A0 = gcge::amg::op(amg, 0);
  if (A0.rp != A->m.rp || A0.rows != A->m.n)
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "PASE_Solve: the hierarchy was not built on A");
  if (B && B->m.n != A->m.n) return gcge_record_error(GCGE_CUDA_ERR_ARG, "PASE_Solve: B size");
  if (p.aux_level < 1 || p.aux_level >= nlev || p.more_nev < 0 || p.max_cycles < 1 ||
      p.smooth_steps < 1 || p.aux_max_it < 1 || p.initial_max_it < 1 || !(p.tol > 0.0) ||
      !(p.initial_tol > 0.0) || !(p.aux_tol > 0.0))
    return gcge_record_error(GCGE_CUDA_ERR_ARG,
                             "PASE_Solve: parameter out of range (1 <= aux_level < number of "
                             "levels, counts >= 1, tolerances > 0)");
  const double t_start = now();
  Pase s;
  s.n = A->m.n;
  s.H = p.aux_level;
  s.nH = gcge::amg::op(amg, s.H).rows;
  s.k = nev + p.more_nev;
  if (s.k > GCGE_MAXCOLS - 32 || 2 * s.k > s.nH)
    return gcge_record_error(GCGE_CUDA_ERR_ARG,
                             "PASE_Solve: nev + more_nev must stay below 224 and below half the "
                             "auxiliary level's size");
  const int k = s.k, n = s.n, nH = s.nH;
  PASE_CU(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
  GCGE_CUDA_PASE_STATS S = {};
  double t0 = now();

  // ---------------------------------------------------------------- B hierarchy
  View Bl;
  if (B) {
    Bl.rows = Bl.cols = B->m.n;
    Bl.nnz = B->m.nnz;
    Bl.rp = B->m.rp;
    Bl.ci = B->m.ci;
    Bl.v = B->m.v;
  } else {
    PASE_CHK(gcge::amg::identity(n, &s.Bid, s.st));
    Bl = s.Bid;
  }
  for (int l = 0; l < s.H; l++) {
    View C;
    PASE_CHK(gcge::amg::galerkin(gcge::amg::restrict_to(amg, l), Bl, gcge::amg::prolong(amg, l), &C,
                                 s.st));
    s.Bchain.push_back(C);
    Bl = C;
  }
  const View AHv = gcge::amg::op(amg, s.H);
  const View BHv = s.Bchain.back();
  PASE_CHK(mat_from_view(AHv, &s.AH));
  PASE_CHK(mat_from_view(BHv, &s.BH));

  // ---------------------------------------------------------------- work space
  PASE_CHK(dalloc(&s.U, (size_t)n * k));
  PASE_CHK(dalloc(&s.Z, (size_t)n * k));
  PASE_CHK(dalloc(&s.AU, (size_t)n * k));
  PASE_CHK(dalloc(&s.BU, (size_t)n * k));
  PASE_CHK(dalloc(&s.rhs, (size_t)n * 32));
  for (int l = 1; l < s.H; l++) {
    double* t = nullptr;
    PASE_CHK(dalloc(&t, (size_t)gcge::amg::op(amg, l).rows * k));
    s.lvl.push_back(t);
  }
  s.lvl.push_back(nullptr);  // unused slot (restrict_chain writes level H to dst)
  const int naux = nH + k;
  PASE_CHK(dalloc(&s.RH, (size_t)nH * k));
  PASE_CHK(dalloc(&s.RH2, (size_t)nH * k));
  PASE_CHK(dalloc(&s.hh, (size_t)k * k));
  PASE_CHK(dalloc(&s.Yaux, (size_t)naux * k));
  s.partial_len = std::max(gcge::gram_oz_partial_doubles(k, k),
                           (size_t)(2 * k + 2) * gcge::kRowBlocks + 4 * k + 64);
  PASE_CHK(dalloc(&s.partial, s.partial_len));
  PASE_CHK(dalloc(&s.dlam, (size_t)k));
  PASE_CHK(dalloc(&s.rn, (size_t)2 * k));
  PASE_CU(cudaMalloc(&s.lcs, gcge::lincomb_oz_scratch_bytes(k, k)));
  PASE_CU(cudaMalloc(&s.upl, gcge::planes_bytes(n, k)));
  PASE_CU(cudaMalloc(&s.mpl, gcge::planes_bytes(n, k)));
  s.lam.assign(k, 0.0);

  // ---------------------------------------------------------------- initial pairs on level H
  {
    GCGE_CUDA_SOLVER* so = nullptr;
    PASE_CHK(GCGE_CUDA_SOLVER_Create(&so));
    int rc = GCGE_CUDA_SOLVER_SetMatA(so, s.AH);
    if (!rc) rc = GCGE_CUDA_SOLVER_SetMatB(so, s.BH);
    if (!rc) rc = set_params(so, k, p.initial_tol, p.initial_max_it);
    if (!rc) rc = GCGE_CUDA_SOLVER_SetEigenvalues(so, s.lam.data());
    if (!rc) rc = GCGE_CUDA_SOLVER_SetEigenvectorsDevice(so, s.RH);
    if (!rc) rc = GCGE_CUDA_SOLVER_Setup(so);
    if (!rc) rc = GCGE_CUDA_SOLVER_Solve(so);
    GCGE_CUDA_STATS st0;
    if (!rc) rc = GCGE_CUDA_SOLVER_GetStats(so, &st0);
    GCGE_CUDA_SOLVER_Free(&so);
    if (rc) return rc;
    S.initial_gcg_iterations = st0.num_iter;
  }
  PASE_CHK(prolong_chain(s, amg, s.RH, nH, s.U));
  PASE_CU(cudaStreamSynchronize(s.st));
  S.t_initial = now() - t0;

  // ---------------------------------------------------------------- auxiliary matrices + solver
  {
    // the staging arrays are freed however this block is left
    struct Staging {
      int* rp = nullptr;
      int* ci = nullptr;
      double* v = nullptr;
      void release() {
        cudaFree(rp);
        cudaFree(ci);
        cudaFree(v);
        rp = ci = nullptr;
        v = nullptr;
      }
      ~Staging() { release(); }
    } sg;
    int nnzH = 0;
    PASE_CU(cudaMemcpy(&nnzH, AHv.rp + nH, sizeof(int), cudaMemcpyDeviceToHost));
    int nnzBH = 0;
    PASE_CU(cudaMemcpy(&nnzBH, BHv.rp + nH, sizeof(int), cudaMemcpyDeviceToHost));
    for (int which = 0; which < 2; which++) {
      const View& M = which == 0 ? AHv : BHv;
      const long long nnz = (long long)(which == 0 ? nnzH : nnzBH) + 2ll * nH * k + (long long)k * k;
      if (nnz > 2000000000ll)
        return gcge_record_error(GCGE_CUDA_ERR_ARG, "PASE_Solve: auxiliary matrix too large");
      PASE_CHK(dalloc(&sg.rp, (size_t)naux + 1));
      PASE_CHK(dalloc(&sg.ci, (size_t)nnz));
      PASE_CHK(dalloc(&sg.v, (size_t)nnz));
      k_aux_rowptr<<<(naux + 256) / 256, 256, 0, s.st>>>(nH, k, M.rp, sg.rp);
      PASE_CU(cudaMemsetAsync(s.RH, 0, sizeof(double) * nH * k, s.st));
      PASE_CU(cudaMemsetAsync(s.hh, 0, sizeof(double) * k * k, s.st));
      k_aux_fill_sparse<<<(nH + 255) / 256, 256, 0, s.st>>>(nH, k, M.rp, M.ci, M.v, s.RH, sg.rp,
                                                            sg.ci, sg.v);
      k_aux_fill_dense<<<dim3(grid_of(naux), k), 256, 0, s.st>>>(nH, k, s.RH, s.hh, sg.rp, sg.ci,
                                                                 sg.v);
      PASE_CU(cudaGetLastError());
      PASE_CU(cudaStreamSynchronize(s.st));
      const int rc =
          GCGE_CUDA_MatCreate(which == 0 ? &s.auxA : &s.auxB, naux, sg.rp, sg.ci, sg.v, 1);
      sg.release();
      if (rc) return rc;
    }
    PASE_CHK(GCGE_CUDA_SOLVER_Create(&s.aux));
    PASE_CHK(GCGE_CUDA_SOLVER_SetMatA(s.aux, s.auxA));
    PASE_CHK(GCGE_CUDA_SOLVER_SetMatB(s.aux, s.auxB));
    PASE_CHK(set_params(s.aux, k, p.aux_tol, p.aux_max_it));
    PASE_CHK(GCGE_CUDA_SOLVER_SetParamInt(s.aux, "num_init_evec", k));
    PASE_CHK(GCGE_CUDA_SOLVER_SetEigenvalues(s.aux, s.lam.data()));
    PASE_CHK(GCGE_CUDA_SOLVER_SetEigenvectorsDevice(s.aux, s.Yaux));
    PASE_CHK(GCGE_CUDA_SOLVER_Setup(s.aux));
  }

  // ---------------------------------------------------------------- cycles
  // the smoothing runs AMG-PCG for exactly smooth_steps steps; the hierarchy's
  // own settings come back however this function returns
  struct PcgRestore {
    GCGE_CUDA_AMG* amg;
    int it = 0;
    double rate = 0.0;
    ~PcgRestore() { gcge::amg::set_pcg(amg, it, rate, nullptr, nullptr); }
  } restore{amg};
  gcge::amg::set_pcg(amg, p.smooth_steps, 1e-12, &restore.it, &restore.rate);
  int rc = GCGE_CUDA_OK;
  const GcgeDevCsr* Bm = B ? &B->m : nullptr;
  double maxres = 0.0;
  for (int cyc = 0; cyc < p.max_cycles && rc == GCGE_CUDA_OK; cyc++) {
    // smoothing: AMG-PCG on A u_i = lambda_i B u_i from u_i, 32 columns at a time
    t0 = now();
    for (int c0 = 0; c0 < k && rc == GCGE_CUDA_OK; c0 += 32) {
      const int kc = std::min(32, k - c0);
      ColList<double> X = cols(s.U + (size_t)c0 * n, n, kc), Rh = cols(s.rhs, n, kc);
      gcge::apply_b_f64(Bm, X, Rh, kc, n, s.st);
      DblList sc;
      for (int j = 0; j < kc; j++) sc.v[j] = s.lam[c0 + j];
      k_scale_cols<<<dim3(grid_of(n), kc), 256, 0, s.st>>>(Rh, sc, kc, n);
      rc = GCGE_CUDA_AMGPCG(amg, A, Rh.p, X.p, kc, n, s.st);
      S.smoothing_steps += p.smooth_steps;
    }
    if (rc) break;
    if (cudaStreamSynchronize(s.st) != cudaSuccess) {
      rc = gcge_record_error(GCGE_CUDA_ERR_CUDA, "PASE: smoothing failed");
      break;
    }
    S.t_smooth += now() - t0;
    // auxiliary matrices: [A_H, R A U; (R A U)^T, U^T A U] and the same with B
    t0 = now();
    const ColList<double> Uc = cols(s.U, n, k), AUc = cols(s.AU, n, k), BUc = cols(s.BU, n, k);
    gcge::spmm_f64(A->m, Uc, AUc, k, s.st);
    gcge::apply_b_f64(Bm, Uc, BUc, k, n, s.st);
    // U^T (M U) from digit planes: U's cut once for both products
    gcge::cut_planes(Uc, k, n, s.upl, k, 0, s.st);
    for (int which = 0; which < 2 && rc == GCGE_CUDA_OK; which++) {
      const double* MU = which == 0 ? s.AU : s.BU;
      rc = restrict_chain(s, amg, MU, s.RH);
      if (rc) break;
      gcge::cut_planes(cols(const_cast<double*>(MU), n, k), k, n, s.mpl, k, 0, s.st);
      gcge::gram_oz_planes(s.upl, k, 0, k, s.mpl, k, 0, k, n, s.hh, k, s.partial, s.st);
      GCGE_CUDA_MAT* aux = which == 0 ? s.auxA : s.auxB;
      const View& M = which == 0 ? AHv : BHv;
      GcgeDevCsr& am = aux->m;
      k_aux_fill_sparse<<<(nH + 255) / 256, 256, 0, s.st>>>(nH, k, M.rp, M.ci, M.v, s.RH, am.rp,
                                                            nullptr, am.v);
      k_aux_fill_dense<<<dim3(grid_of(naux), k), 256, 0, s.st>>>(nH, k, s.RH, s.hh, am.rp, nullptr,
                                                                 am.v);
      if (am.v32)
        k_to32<<<(unsigned)((am.nnz + 255) / 256), 256, 0, s.st>>>((size_t)am.nnz, am.v, am.v32);
    }
    if (rc) break;
    k_aux_start<<<dim3(grid_of(naux), k), 256, 0, s.st>>>(nH, k, s.Yaux);
    if (cudaStreamSynchronize(s.st) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
      rc = gcge_record_error(GCGE_CUDA_ERR_CUDA, "PASE: auxiliary assembly failed");
      break;
    }
    S.t_aux_build += now() - t0;
    // auxiliary eigenproblem
    t0 = now();
    rc = GCGE_CUDA_SOLVER_Solve(s.aux);
    if (rc) break;
    {
      GCGE_CUDA_STATS sa;
      GCGE_CUDA_SOLVER_GetStats(s.aux, &sa);
      S.aux_gcg_iterations += sa.num_iter;
    }
    S.t_aux_solve += now() - t0;
    // u_i = P y_H,i + U alpha_i
    t0 = now();
    rc = prolong_chain(s, amg, s.Yaux, naux, s.Z);
    if (rc) break;
    gcge::lincomb_oz(Uc, k, s.Yaux + nH, naux, cols(s.Z, n, k), k, 1.0, n, s.lcs, s.st);
    std::swap(s.U, s.Z);
    PASE_CU(cudaMemcpyAsync(s.dlam, s.lam.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s.st));
    if (cudaStreamSynchronize(s.st) != cudaSuccess) {
      rc = gcge_record_error(GCGE_CUDA_ERR_CUDA, "PASE: prolongation failed");
      break;
    }
    S.t_prolong += now() - t0;
    // convergence of the first nev pairs: ||A u - lambda B u|| / (|lambda| ||u||)
    t0 = now();
    gcge::residual_f64(A->m, Bm, cols(s.U, n, nev), s.dlam, nev, s.rn, s.rn + k, s.partial, s.st);
    std::vector<double> hr(2 * k);
    PASE_CU(cudaMemcpyAsync(hr.data(), s.rn, sizeof(double) * 2 * k, cudaMemcpyDeviceToHost, s.st));
    PASE_CU(cudaStreamSynchronize(s.st));
    maxres = 0.0;
    for (int i = 0; i < nev; i++) {
      const double r = sqrt(hr[i]) / (fabs(s.lam[i]) * sqrt(hr[k + i]));
      maxres = std::max(maxres, std::isfinite(r) ? r : INFINITY);
    }
    S.t_check += now() - t0;
    S.cycles = cyc + 1;
    if (maxres < p.tol) break;
  }
  if (rc) return rc;
  for (int i = 0; i < nev; i++) eval[i] = s.lam[i];
  PASE_CU(cudaMemcpyAsync(evec, s.U, sizeof(double) * n * nev, cudaMemcpyDeviceToDevice, s.st));
  PASE_CU(cudaStreamSynchronize(s.st));
  S.max_residual = maxres;
  S.seconds = now() - t_start;
  if (stats) *stats = S;
  if (!(maxres < p.tol))
    return gcge_record_error(GCGE_CUDA_ERR_NUMERIC,
                             "PASE_Solve: the pairs did not reach the tolerance within max_cycles");
  return GCGE_CUDA_OK;
}
