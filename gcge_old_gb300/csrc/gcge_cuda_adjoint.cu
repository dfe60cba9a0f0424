// Adjoint of the eigenvectors of A x = lambda B x (B-normalised, simple
// eigenvalues), for losses that depend on the eigenvectors.
//
// For a loss L with g_k = dL/dx_k, differentiating A x_k = lambda_k B x_k and
// x_k^T B x_k = 1 gives
//   dL = -mu_k^T dA x_k + lambda_k mu_k^T dB x_k - 1/2 (g_k^T x_k) x_k^T dB x_k,
// where mu_k is B-orthogonal to x_k and solves
//   (A - lambda_k B) mu_k = g_k - B x_k (x_k^T g_k).
// A - lambda_k B is singular on x_k and indefinite below lambda_k, so mu_k is
// split over the nev computed pairs X and their B-orthogonal complement:
//   mu_k = sum_{j != k} x_j (x_j^T g_k) / (lambda_j - lambda_k) + m_k,
// with m_k = Q m_k, Q = I - X X^T B, from the projected system
//   Q^T (A - lambda_k B) Q m_k = Q^T g_k,
// which is positive definite on range(Q) when lambda_k < lambda_{nev+1}.  It is
// solved by conjugate gradients on range(Q), preconditioned by Q D^-1 Q^T with
// D = diag(A), all requested columns at once (one SpMM per step), with the step
// scalars kept on the device and the residuals read back every few steps.
// GCGE_CUDA_EigvecAdjointSolveAMG preconditions by Q M^-1 Q^T instead, M^-1 one
// V-cycle of an AMG hierarchy of A: for v in range(Q), v^T (A - lambda_k B) v
// lies between (1 - lambda_k / lambda_{nev+1}) v^T A v and v^T A v, so a
// preconditioner of A serves the shifted system.  The V-cycle runs in FP32, which makes it a
// slightly nonlinear operator; those solves take the flexible direction update
// beta = -z_new^T U / p^T U (U the projected operator times p), which keeps
// successive directions conjugate whatever the preconditioner.
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/gcge_cuda.h"
#include "gcge_cuda_common.cuh"

int gcge_record_error(int code, const char* msg);

namespace {

constexpr int kDotBlocks = 2 * 152;
constexpr int kCheckEvery = 8;

std::mutex g_mu;
double* g_buf = nullptr;
size_t g_len = 0;

int buffer(size_t len, double** out) {
  if (len > g_len) {
    if (g_buf) cudaFree(g_buf);
    g_buf = nullptr;
    g_len = 0;
    if (cudaMalloc(&g_buf, sizeof(double) * len) != cudaSuccess) return GCGE_CUDA_ERR_ALLOC;
    g_len = len;
  }
  *out = g_buf;
  return GCGE_CUDA_OK;
}

// partial[c * gridDim.x + b] = this block's share of X_c . Y_c
__global__ void k_dots(ColList<double> X, ColList<double> Y, int n, double* __restrict__ partial) {
  __shared__ double sh[256];
  const int c = blockIdx.y;
  const double* __restrict__ x = X.p[c];
  const double* __restrict__ y = Y.p[c];
  double s = 0.0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    s = fma(x[r], y[r], s);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(size_t)c * gridDim.x + blockIdx.x] = sh[0];
}

// out[c] = sum of the partials of column c, in a fixed order (one warp a column)
__global__ void k_dots_sum(const double* __restrict__ partial, int m, double* __restrict__ out) {
  const int c = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < kDotBlocks; b += 32) s += partial[(size_t)c * kDotBlocks + b];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (threadIdx.x == 0 && c < m) out[c] = s;
}

void dots(const ColList<double>& X, const ColList<double>& Y, int m, int n, double* partial,
          double* out, cudaStream_t st) {
  k_dots<<<dim3(kDotBlocks, m), 256, 0, st>>>(X, Y, n, partial);
  k_dots_sum<<<m, 32, 0, st>>>(partial, m, out);
}

// partial[(j + k1 * c) * gridDim.x + b] = block b's share of X_j . U_c: one
// block row per (j, c) pair, so a k1 x m Gram with m small keeps every SM busy
__global__ void k_pair_dots(ColList<double> X, int k1, ColList<double> U, int n,
                            double* __restrict__ partial) {
  __shared__ double sh[256];
  const int pr = blockIdx.y, j = pr % k1, c = pr / k1;
  const double* __restrict__ x = X.p[j];
  const double* __restrict__ u = U.p[c];
  double s = 0.0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    s = fma(x[r], u[r], s);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(size_t)pr * gridDim.x + blockIdx.x] = sh[0];
}

// G[j + c * k1] = X_j . U_c (j < k1, c < m), fixed summation order
void pair_gram(const ColList<double>& X, int k1, const ColList<double>& U, int m, int n,
               double* partial, double* G, cudaStream_t st) {
  k_pair_dots<<<dim3(kDotBlocks, k1 * m), 256, 0, st>>>(X, k1, U, n, partial);
  k_dots_sum<<<k1 * m, 32, 0, st>>>(partial, k1 * m, G);
}

__global__ void k_diag_inv(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                           const double* __restrict__ v, double* __restrict__ dinv) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double d = 0.0;
  for (int e = rp[r]; e < rp[r + 1]; e++)
    if (ci[e] == r) d += v[e];
  dinv[r] = (d > 0.0) ? 1.0 / d : 1.0;
}

// Y_c <- Y_c - sum_j W_j G[j + c * ldg]  (j < k, c < m); G is small (k x m)
__global__ void k_sub_lincomb(ColList<double> Y, ColList<double> W, const double* __restrict__ G,
                              int ldg, int k, int m, int n) {
  extern __shared__ double g[];
  for (int t = threadIdx.x; t < k * m; t += blockDim.x) g[t] = G[(t % k) + (size_t)(t / k) * ldg];
  __syncthreads();
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    double w[8];
    for (int j0 = 0; j0 < k; j0 += 8) {
      const int jn = min(8, k - j0);
#pragma unroll
      for (int j = 0; j < 8; j++) w[j] = (j < jn) ? W.p[j0 + j][r] : 0.0;
      for (int c = 0; c < m; c++) {
        double s = 0.0;
#pragma unroll
        for (int j = 0; j < 8; j++)
          if (j < jn) s = fma(w[j], g[j0 + j + c * k], s);
        Y.p[c][r] -= s;
      }
    }
  }
}

// U_c <- U_c - lambda_c V_c
__global__ void k_shift_sub(ColList<double> U, ColList<double> V, DblList lam, int n) {
  const int c = blockIdx.y;
  const double l = lam.v[c];
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    U.p[c][r] = fma(-l, V.p[c][r], U.p[c][r]);
}

// Z_c <- D^-1 R_c
__global__ void k_precond(ColList<double> R, ColList<double> Z, const double* __restrict__ dinv,
                          int n) {
  const int c = blockIdx.y;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    Z.p[c][r] = dinv[r] * R.p[c][r];
}

// alpha = rz / pu; MU += alpha P; R -= alpha U  (active columns)
__global__ void k_step(ColList<double> MU, ColList<double> R, ColList<double> P, ColList<double> U,
                       const double* __restrict__ rz, const double* __restrict__ pu,
                       const int* __restrict__ active, int n) {
  const int c = blockIdx.y;
  if (!active[c]) return;
  __shared__ double a_s;  // one division per block
  if (threadIdx.x == 0) a_s = (pu[c] != 0.0) ? rz[c] / pu[c] : 0.0;
  __syncthreads();
  const double a = a_s;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    MU.p[c][r] = fma(a, P.p[c][r], MU.p[c][r]);
    R.p[c][r] = fma(-a, U.p[c][r], R.p[c][r]);
  }
}

// beta = sign num / den (rz_new / rz_old, or -z_new^T U / p^T U for the
// flexible update); P = Z + beta P  (active columns)
__global__ void k_direction(ColList<double> Z, ColList<double> P, const double* __restrict__ num,
                            const double* __restrict__ den, double sign,
                            const int* __restrict__ active, int n) {
  const int c = blockIdx.y;
  if (!active[c]) return;
  __shared__ double b_s;  // one division per block
  if (threadIdx.x == 0) b_s = (den[c] != 0.0) ? sign * num[c] / den[c] : 0.0;
  __syncthreads();
  const double b = b_s;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    P.p[c][r] = fma(b, P.p[c][r], Z.p[c][r]);
}

__global__ void k_copy_cols(ColList<double> X, ColList<double> Y, int n) {
  const int c = blockIdx.y;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    Y.p[c][r] = X.p[c][r];
}

// grad[e] = sum_k (a_k X_k[i] + b_k MU_k[i]) X_k[j] over the stored entries e = (i, j)
__global__ void k_grad2(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                        ColList<double> X, ColList<double> MU, DblList a, DblList b, int k,
                        int has_mu, double* __restrict__ grad) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  for (int e = __ldg(rp + r); e < __ldg(rp + r + 1); e++) {
    const int col = __ldg(ci + e);
    double s = 0.0;
    for (int j = 0; j < k; j++) {
      double w = a.v[j] * X.p[j][r];
      if (has_mu && MU.p[j]) w = fma(b.v[j], MU.p[j][r], w);
      s = fma(w, X.p[j][col], s);
    }
    grad[e] = s;
  }
}

int finish(cudaStream_t st) {
  cudaError_t e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return gcge_record_error(GCGE_CUDA_ERR_CUDA, cudaGetErrorString(e));
  return GCGE_CUDA_OK;
}

}  // namespace

extern "C" int GCGE_CUDA_EigvecAdjointSolveAMG(const GCGE_CUDA_MAT* A, const GCGE_CUDA_MAT* B,
                                               double* const* X, const double* eval, int nev,
                                               double* const* G, double* const* MU, double* gx,
                                               int max_it, double tol, int* iters,
                                               GCGE_CUDA_AMG* amg) {
  if (!A || !X || !eval || !G || !MU || nev <= 0 || nev > GCGE_MAXCOLS || max_it < 0)
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "EigvecAdjointSolve: bad argument");
  const int n = A->m.n;
  if (B && B->m.n != n) return gcge_record_error(GCGE_CUDA_ERR_ARG, "EigvecAdjointSolve: B size");
  if (amg) {
    int n0 = -1;
    if (GCGE_CUDA_AMG_GetLevelInfo(amg, 0, &n0, nullptr, nullptr, nullptr) != GCGE_CUDA_OK ||
        n0 != n)
      return gcge_record_error(GCGE_CUDA_ERR_ARG,
                               "EigvecAdjointSolveAMG: the hierarchy's finest level is not n rows");
  }
  std::vector<int> ks;  // requested columns
  for (int k = 0; k < nev; k++)
    if (G[k]) {
      if (!MU[k]) return gcge_record_error(GCGE_CUDA_ERR_ARG, "EigvecAdjointSolve: MU[k] missing");
      ks.push_back(k);
    }
  if (iters) *iters = 0;
  const int m = (int)ks.size();
  if (m == 0 || n == 0) return GCGE_CUDA_OK;
  for (int a = 0; a < m; a++)
    for (int j = 0; j < nev; j++)
      if (j != ks[a] && !(fabs(eval[j] - eval[ks[a]]) > 1e-14 * fabs(eval[ks[a]])))
        return gcge_record_error(GCGE_CUDA_ERR_NUMERIC,
                                 "EigvecAdjointSolve: repeated eigenvalue, the adjoint is undefined");
  if ((size_t)nev * m * sizeof(double) > 200 * 1024)
    return gcge_record_error(GCGE_CUDA_ERR_ARG,
                             "EigvecAdjointSolve: nev x requested columns above 25600");
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t st = 0;
  const size_t ld = ((size_t)n + 31) / 32 * 32;
  // columns: BX (nev), R, Z, P, U, V (m each); dinv; small arrays
  const size_t small = (size_t)kDotBlocks * GCGE_MAXCOLS + 4 * (size_t)GCGE_MAXCOLS * GCGE_MAXCOLS +
                       8 * GCGE_MAXCOLS;
  double* buf;
  if (buffer(ld * ((size_t)nev + 5 * m + 1) + small, &buf))
    return gcge_record_error(GCGE_CUDA_ERR_ALLOC, "EigvecAdjointSolve: device memory");
  ColList<double> Xl, BX, R, Z, P, U, V, Gl, Ml;
  double* q = buf;
  for (int j = 0; j < nev; j++, q += ld) {
    Xl.p[j] = X[j];
    BX.p[j] = q;
  }
  for (int a = 0; a < m; a++) {
    R.p[a] = q;
    Z.p[a] = q + ld;
    P.p[a] = q + 2 * ld;
    U.p[a] = q + 3 * ld;
    V.p[a] = q + 4 * ld;
    q += 5 * ld;
    Gl.p[a] = G[ks[a]];
    Ml.p[a] = MU[ks[a]];
  }
  double* dinv = q;
  q += ld;
  double* partial = q;
  q += (size_t)kDotBlocks * GCGE_MAXCOLS;
  double* Gm = q;  // nev x m, ld nev
  q += (size_t)GCGE_MAXCOLS * GCGE_MAXCOLS;
  double* Cm = q;  // nev x m
  q += (size_t)GCGE_MAXCOLS * GCGE_MAXCOLS;
  double* rz = q;
  double* rz2 = q + GCGE_MAXCOLS;
  double* pu = q + 2 * GCGE_MAXCOLS;
  double* rr = q + 3 * GCGE_MAXCOLS;
  int* active = reinterpret_cast<int*>(q + 4 * GCGE_MAXCOLS);
  // Gram partials: kDotBlocks per (column of X, column of U) pair
  double* gp = nullptr;
  if (cudaMalloc(&gp, sizeof(double) * kDotBlocks * (size_t)nev * m) != cudaSuccess)
    return gcge_record_error(GCGE_CUDA_ERR_ALLOC, "EigvecAdjointSolve: device memory");
  struct Free {
    double* p;
    ~Free() { cudaFree(p); }
  } free_gp{gp};

  const GcgeDevCsr* Bm = B ? &B->m : nullptr;
  const dim3 gcol((unsigned)std::min<size_t>((n + 255) / 256, 4 * 152), m);
  const int nb_rows = (int)std::min<size_t>((n + 255) / 256, 4 * 152);
  DblList lam;
  for (int a = 0; a < m; a++) lam.v[a] = eval[ks[a]];

  k_diag_inv<<<(n + 255) / 256, 256, 0, st>>>(n, A->m.rp, A->m.ci, A->m.v, dinv);
  gcge::apply_b_f64(Bm, Xl, BX, nev, n, st);
  // x_j^T g_k (nev x m) to the host: the coefficients over the computed pairs
  pair_gram(Xl, nev, Gl, m, n, gp, Gm, st);
  std::vector<double> hg((size_t)nev * m), hc((size_t)nev * m, 0.0);
  if (cudaMemcpyAsync(hg.data(), Gm, sizeof(double) * nev * m, cudaMemcpyDeviceToHost, st) !=
      cudaSuccess)
    return finish(st);
  if (int r = finish(st)) return r;
  for (int a = 0; a < m; a++) {
    const int k = ks[a];
    if (gx) gx[k] = hg[k + (size_t)a * nev];
    for (int j = 0; j < nev; j++)
      if (j != k) hc[j + (size_t)a * nev] = hg[j + (size_t)a * nev] / (eval[j] - eval[k]);
  }
  cudaMemcpyAsync(Cm, hc.data(), sizeof(double) * nev * m, cudaMemcpyHostToDevice, st);
  // MU = X C; R = Q^T G = G - BX (X^T G)
  gcge::lincomb_f64(Xl, nev, Cm, nev, Ml, m, 0.0, n, st);
  k_copy_cols<<<gcol, 256, 0, st>>>(Gl, R, n);
  const size_t shm = sizeof(double) * nev * m;
  if (shm > 48 * 1024)
    cudaFuncSetAttribute(k_sub_lincomb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  k_sub_lincomb<<<nb_rows, 256, shm, st>>>(R, BX, Gm, nev, nev, m, n);
  // Z = Q M^-1 R = M^-1 R - X (BX^T M^-1 R), M = D or one V-cycle; P = Z
  auto precond = [&]() -> int {
    if (amg) {
      for (int c0 = 0; c0 < m; c0 += 32) {
        const int r = GCGE_CUDA_AMG_Apply(amg, &R.p[c0], &Z.p[c0], std::min(32, m - c0), st);
        if (r != GCGE_CUDA_OK) return r;
      }
    } else {
      k_precond<<<gcol, 256, 0, st>>>(R, Z, dinv, n);
    }
    pair_gram(BX, nev, Z, m, n, gp, Gm, st);
    k_sub_lincomb<<<nb_rows, 256, shm, st>>>(Z, Xl, Gm, nev, nev, m, n);
    return GCGE_CUDA_OK;
  };
  int rc = precond();
  if (rc) return rc;
  k_copy_cols<<<gcol, 256, 0, st>>>(Z, P, n);
  dots(R, Z, m, n, partial, rz, st);
  dots(R, R, m, n, partial, rr, st);
  std::vector<double> r0(m), rn(m);
  std::vector<int> act(m, 1);
  cudaMemcpyAsync(rn.data(), rr, sizeof(double) * m, cudaMemcpyDeviceToHost, st);
  if ((rc = finish(st))) return rc;
  int live = 0;
  for (int a = 0; a < m; a++) {
    r0[a] = sqrt(rn[a]);
    act[a] = r0[a] > 0.0;
    live += act[a];
  }
  cudaMemcpyAsync(active, act.data(), sizeof(int) * m, cudaMemcpyHostToDevice, st);
  int it = 0;
  while (live > 0 && it < max_it) {
    // U = Q^T (A - lambda B) P
    gcge::spmm_f64(A->m, P, U, m, st);
    if (Bm) {
      gcge::apply_b_f64(Bm, P, V, m, n, st);
      k_shift_sub<<<gcol, 256, 0, st>>>(U, V, lam, n);
    } else {
      k_shift_sub<<<gcol, 256, 0, st>>>(U, P, lam, n);
    }
    pair_gram(Xl, nev, U, m, n, gp, Gm, st);
    k_sub_lincomb<<<nb_rows, 256, shm, st>>>(U, BX, Gm, nev, nev, m, n);
    dots(P, U, m, n, partial, pu, st);
    k_step<<<gcol, 256, 0, st>>>(Ml, R, P, U, rz, pu, active, n);
    if ((rc = precond())) return rc;
    dots(R, Z, m, n, partial, rz2, st);
    if (amg) {
      dots(Z, U, m, n, partial, rr, st);
      k_direction<<<gcol, 256, 0, st>>>(Z, P, rr, pu, -1.0, active, n);
    } else {
      k_direction<<<gcol, 256, 0, st>>>(Z, P, rz2, rz, 1.0, active, n);
    }
    std::swap(rz, rz2);
    it++;
    if (it % kCheckEvery == 0 || it == max_it) {
      dots(R, R, m, n, partial, rr, st);
      cudaMemcpyAsync(rn.data(), rr, sizeof(double) * m, cudaMemcpyDeviceToHost, st);
      if ((rc = finish(st))) return rc;
      live = 0;
      for (int a = 0; a < m; a++) {
        if (act[a] && !(sqrt(rn[a]) > tol * r0[a])) act[a] = 0;
        live += act[a];
      }
      cudaMemcpyAsync(active, act.data(), sizeof(int) * m, cudaMemcpyHostToDevice, st);
    }
  }
  if (iters) *iters = it;
  if ((rc = finish(st))) return rc;
  if (live > 0) {
    char msg[160];
    snprintf(msg, sizeof(msg),
             "EigvecAdjointSolve: %d column(s) above the tolerance after %d steps", live, it);
    return gcge_record_error(GCGE_CUDA_ERR_NUMERIC, msg);
  }
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_EigvecAdjointSolve(const GCGE_CUDA_MAT* A, const GCGE_CUDA_MAT* B,
                                            double* const* X, const double* eval, int nev,
                                            double* const* G, double* const* MU, double* gx,
                                            int max_it, double tol, int* iters) {
  return GCGE_CUDA_EigvecAdjointSolveAMG(A, B, X, eval, nev, G, MU, gx, max_it, tol, iters,
                                         nullptr);
}

extern "C" int GCGE_CUDA_EigGradCSR2(const GCGE_CUDA_MAT* M, double* const* X, double* const* MU,
                                     const double* a, const double* b, int k, double* grad) {
  if (!M || !X || !a || !grad || k <= 0 || k > GCGE_MAXCOLS || (MU && !b))
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "EigGradCSR2: bad argument");
  std::lock_guard<std::mutex> lk(g_mu);
  ColList<double> Xl, Ml;
  DblList al, bl;
  for (int j = 0; j < k; j++) {
    Xl.p[j] = X[j];
    Ml.p[j] = MU ? MU[j] : nullptr;
    al.v[j] = a[j];
    bl.v[j] = MU ? b[j] : 0.0;
  }
  if (M->m.n > 0)
    k_grad2<<<(M->m.n + 255) / 256, 256>>>(M->m.n, M->m.rp, M->m.ci, Xl, Ml, al, bl, k,
                                           MU ? 1 : 0, grad);
  return finish(0);
}
