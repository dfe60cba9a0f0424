// GCGE_CUDA_ChebyshevPCG: a stock W-step solver for the MultiLinearSolver hook
// (GCGE_OPS.MultiLinearSolver, src/gcge_ops.h:77, called at src/gcge_xpw.c:178-191),
// the GPU counterpart of the hypre app's preconditioned solver there
// (app/hypre/gcge_app_hypre.c:305-331).
//
// Per column: conjugate gradients on A x = rhs, preconditioned by a Chebyshev
// polynomial in D^-1 A (D = diag(A)) of the given degree: z = p(D^-1 A) D^-1 r
// is `degree` steps of the Chebyshev semi-iteration for A z = r from z = 0 on
// the interval [lower_frac b, b], b the Gershgorin bound of D^-1 A (so every
// eigenvalue of D^-1 A lies in (0, b] and p stays positive there: the
// preconditioner is SPD for SPD A).  Degree 0 is the diagonal preconditioner.
// A column stops once ||r|| < rate ||r_0|| or after max_it steps, as the
// reference's block CG does (src/gcge_cg.c:488).
//
// Everything per column lives on the device: the inner products reduce in a
// fixed order into device arrays, the step scalars (alpha, beta) are formed
// in the update kernels, and a converged column is frozen by its flag.  The
// host reads the number of active columns every kCheck steps (one stream
// synchronisation per kCheck steps instead of one per reduction).
#include <cmath>
#include <mutex>
#include <vector>

#include "../../include/gcge_cuda.h"
#include "gcge_cuda_common.cuh"

int gcge_record_error(int code, const char* msg);

namespace {

constexpr int kBlocks = 2 * 152;  // row blocks of the reductions
constexpr int kCheck = 4;

std::mutex g_pcg_mu;
double* g_pcg_buf = nullptr;
size_t g_pcg_len = 0;

double* pcg_scratch(size_t len) {
  if (len > g_pcg_len) {
    if (g_pcg_buf) cudaFree(g_pcg_buf);
    g_pcg_buf = nullptr;
    g_pcg_len = 0;
    if (cudaMalloc(&g_pcg_buf, sizeof(double) * len) != cudaSuccess) return nullptr;
    g_pcg_len = len;
  }
  return g_pcg_buf;
}

// dinv = 1 / a_ii; gb[block] = max over the block's rows of sum_j |a_ij| / a_ii
__global__ void k_cheb_diag(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                            const double* __restrict__ v, double* __restrict__ dinv,
                            double* __restrict__ gb) {
  __shared__ double sm[256];
  double m = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double d = 0.0, s = 0.0;
    for (int e = rp[i]; e < rp[i + 1]; e++) {
      s += fabs(v[e]);
      if (ci[e] == i) d = v[e];
    }
    const double di = d > 0.0 ? 1.0 / d : 0.0;
    dinv[i] = di;
    m = fmax(m, s * di);
  }
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) gb[blockIdx.x] = sm[0];
}

__global__ void k_cheb_maxb(const double* __restrict__ gb, int nb, double* out) {
  double m = 0.0;
  for (int b = 0; b < nb; b++) m = fmax(m, gb[b]);
  *out = m;
}

// partial[b * k + j] = sum over block b's rows of X_j . Y_j
__global__ void k_cheb_dot(ColList<double> X, ColList<double> Y, int n, double* __restrict__ partial,
                           int k) {
  __shared__ double sm[256];
  const int j = blockIdx.y;
  const double* x = X.p[j];
  const double* y = Y.p[j];
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    s = fma(x[i], y[i], s);
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(size_t)blockIdx.x * k + j] = sm[0];
}

// out[j] = sum_b partial[b * k + j], block order fixed
__global__ void k_cheb_sum(const double* __restrict__ partial, int nb, int k,
                           double* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k) return;
  double s = 0.0;
  for (int b = 0; b < nb; b++) s += partial[(size_t)b * k + j];
  out[j] = s;
}

// r = rhs - w
__global__ void k_cheb_resid(ColList<double> R, ColList<double> W, int n) {
  const int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    R.p[j][i] -= W.p[j][i];
}

// first Chebyshev step: d = c D^-1 r, z = d (active columns)
__global__ void k_cheb_first(ColList<double> R, ColList<double> Dd, ColList<double> Z,
                             const double* __restrict__ dinv, double c, int n,
                             const int* __restrict__ act) {
  const int j = blockIdx.y;
  if (!act[j]) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double d = c * dinv[i] * R.p[j][i];
    Dd.p[j][i] = d;
    Z.p[j][i] = d;
  }
}

// later steps: d = c1 d + c2 D^-1 (r - t), z += d (t = A z)
__global__ void k_cheb_step(ColList<double> R, ColList<double> T, ColList<double> Dd,
                            ColList<double> Z, const double* __restrict__ dinv, double c1,
                            double c2, int n, const int* __restrict__ act) {
  const int j = blockIdx.y;
  if (!act[j]) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double d = c1 * Dd.p[j][i] + c2 * dinv[i] * (R.p[j][i] - T.p[j][i]);
    Dd.p[j][i] = d;
    Z.p[j][i] += d;
  }
}

// x += alpha p, r -= alpha w with alpha = rz / pw per active column
__global__ void k_cheb_update(ColList<double> X, ColList<double> R, ColList<double> P,
                              ColList<double> W, const double* __restrict__ rz,
                              const double* __restrict__ pw, int n, const int* __restrict__ act) {
  const int j = blockIdx.y;
  if (!act[j] || pw[j] == 0.0) return;
  const double a = rz[j] / pw[j];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    X.p[j][i] = fma(a, P.p[j][i], X.p[j][i]);
    R.p[j][i] = fma(-a, W.p[j][i], R.p[j][i]);
  }
}

// p = z + beta p with beta = rznew / rz (beta = 0 on the first step)
__global__ void k_cheb_dir(ColList<double> Z, ColList<double> P, const double* __restrict__ rznew,
                           const double* __restrict__ rz, int first, int n,
                           const int* __restrict__ act) {
  const int j = blockIdx.y;
  if (!act[j]) return;
  const double b = (first || rz[j] == 0.0) ? 0.0 : rznew[j] / rz[j];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    P.p[j][i] = fma(b, P.p[j][i], Z.p[j][i]);
}

// the column flags after a step: active while ||r|| >= rate ||r_0||; also
// rz <- rznew (for the next beta) and the count of active columns
__global__ void k_cheb_flags(const double* __restrict__ rr, const double* __restrict__ r0,
                             double rate, int* __restrict__ act, int k, int* __restrict__ count,
                             int set_r0, double* __restrict__ r0w) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int c = 0;
  for (int j = 0; j < k; j++) {
    const double nr = sqrt(rr[j]);
    if (set_r0) {
      r0w[j] = nr;
      act[j] = nr > 0.0 ? 1 : 0;
    } else if (act[j] && !(nr >= rate * r0[j])) {
      act[j] = 0;
    }
    c += act[j];
  }
  *count = c;
}

__global__ void k_copy_d(const double* __restrict__ a, double* __restrict__ b, int k) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < k) b[j] = a[j];
}

int grid_rows(int n) {
  const int b = (n + 255) / 256;
  return b < 256 ? (b < 1 ? 1 : b) : 256;
}

}  // namespace

extern "C" int GCGE_CUDA_ChebyshevPCG(void* ctx, const GCGE_CUDA_MAT* A, double* const* rhs,
                                      double* const* x, int k, int n, void* stream) {
  if (!A || !rhs || !x || k <= 0 || k > GCGE_MAXCOLS || n != A->m.n)
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "ChebyshevPCG: bad arguments");
  const GCGE_CUDA_CHEB_PARAM* prm = static_cast<const GCGE_CUDA_CHEB_PARAM*>(ctx);
  const int max_it = prm ? prm->max_it : 20;
  const double rate = prm ? prm->rate : 1e-2;
  const int degree = prm ? prm->degree : 4;
  const double lower = prm ? prm->lower_frac : 0.05;
  if (max_it < 0 || degree < 0 || degree > 64 || !(lower >= 0.0 && lower < 1.0))
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "ChebyshevPCG: bad parameters");
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(g_pcg_mu);
  const size_t ld = ((size_t)n + 31) / 32 * 32;
  // columns: Z, P, W, T (A z inside the polynomial), Dd (its step); dinv; scalars
  const size_t nsc = 6 * (size_t)GCGE_MAXCOLS + 2 * GCGE_MAXCOLS;
  const size_t need = 5 * (size_t)k * ld + ld + (size_t)kBlocks * k + kBlocks + nsc + 8;
  double* buf = pcg_scratch(need);
  if (!buf) return gcge_record_error(GCGE_CUDA_ERR_ALLOC, "ChebyshevPCG: scratch allocation failed");
  ColList<double> R, X, Z, P, W, T, Dd;
  for (int j = 0; j < k; j++) {
    R.p[j] = rhs[j];
    X.p[j] = x[j];
    Z.p[j] = buf + (size_t)j * ld;
    P.p[j] = buf + (size_t)(k + j) * ld;
    W.p[j] = buf + (size_t)(2 * k + j) * ld;
    T.p[j] = buf + (size_t)(3 * k + j) * ld;
    Dd.p[j] = buf + (size_t)(4 * k + j) * ld;
  }
  double* dinv = buf + 5 * (size_t)k * ld;
  double* partial = dinv + ld;
  double* gb = partial + (size_t)kBlocks * k;
  double* rz = gb + kBlocks;
  double* rznew = rz + GCGE_MAXCOLS;
  double* pw = rznew + GCGE_MAXCOLS;
  double* rr = pw + GCGE_MAXCOLS;
  double* r0 = rr + GCGE_MAXCOLS;
  double* bmax = r0 + GCGE_MAXCOLS;
  int* act = reinterpret_cast<int*>(bmax + 8);
  int* count = act + GCGE_MAXCOLS;
  const GcgeDevCsr& M = A->m;
  const dim3 g2(grid_rows(n), k);
  auto dot = [&](const ColList<double>& a, const ColList<double>& b, double* out) {
    k_cheb_dot<<<dim3(kBlocks, k), 256, 0, st>>>(a, b, n, partial, k);
    k_cheb_sum<<<(k + 127) / 128, 128, 0, st>>>(partial, kBlocks, k, out);
  };
  // Gershgorin bound of D^-1 A and D^-1 (one read to the host per call)
  k_cheb_diag<<<kBlocks, 256, 0, st>>>(n, M.rp, M.ci, M.v, dinv, gb);
  k_cheb_maxb<<<1, 1, 0, st>>>(gb, kBlocks, bmax);
  double b = 0.0;
  if (cudaMemcpyAsync(&b, bmax, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return gcge_record_error(GCGE_CUDA_ERR_CUDA, "ChebyshevPCG: set-up failed");
  if (!(b > 0.0) || !std::isfinite(b))
    return gcge_record_error(GCGE_CUDA_ERR_NUMERIC, "ChebyshevPCG: A has a non-positive diagonal");
  // Chebyshev semi-iteration scalars on [lower b, b]
  const double lo = lower * b, theta = 0.5 * (b + lo), delta = 0.5 * (b - lo);
  std::vector<double> c1(degree + 1, 0.0), c2(degree + 1, 0.0);
  {
    const double sigma = theta / delta;
    double rho = 1.0 / sigma;
    for (int s = 1; s < degree; s++) {
      const double rn = 1.0 / (2.0 * sigma - rho);
      c1[s] = rn * rho;
      c2[s] = 2.0 * rn / delta;
      rho = rn;
    }
  }
  // z = p(D^-1 A) D^-1 r on the active columns
  auto precondition = [&]() {
    k_cheb_first<<<g2, 256, 0, st>>>(R, Dd, Z, dinv, degree > 0 ? 1.0 / theta : 1.0, n, act);
    for (int s = 1; s < degree; s++) {
      gcge::spmm_f64(M, Z, T, k, st);
      k_cheb_step<<<g2, 256, 0, st>>>(R, T, Dd, Z, dinv, c1[s], c2[s], n, act);
    }
  };
  // r = rhs - A x, r_0, flags
  gcge::spmm_f64(M, X, W, k, st);
  k_cheb_resid<<<g2, 256, 0, st>>>(R, W, n);
  dot(R, R, rr);
  k_cheb_flags<<<1, 1, 0, st>>>(rr, r0, rate, act, k, count, 1, r0);
  precondition();
  dot(R, Z, rz);
  k_cheb_dir<<<g2, 256, 0, st>>>(Z, P, rz, rz, 1, n, act);
  int* h_count = nullptr;
  if (cudaHostAlloc(&h_count, sizeof(int), cudaHostAllocDefault) != cudaSuccess)
    return gcge_record_error(GCGE_CUDA_ERR_ALLOC, "ChebyshevPCG: pinned allocation failed");
  int rc = GCGE_CUDA_OK;
  for (int it = 0; it < max_it; it++) {
    gcge::spmm_f64(M, P, W, k, st);
    dot(P, W, pw);
    k_cheb_update<<<g2, 256, 0, st>>>(X, R, P, W, rz, pw, n, act);
    dot(R, R, rr);
    k_cheb_flags<<<1, 1, 0, st>>>(rr, r0, rate, act, k, count, 0, nullptr);
    if (it + 1 == max_it) break;
    precondition();
    dot(R, Z, rznew);
    k_cheb_dir<<<g2, 256, 0, st>>>(Z, P, rznew, rz, 0, n, act);
    k_copy_d<<<(k + 127) / 128, 128, 0, st>>>(rznew, rz, k);
    if ((it + 1) % kCheck == 0) {
      if (cudaMemcpyAsync(h_count, count, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess) {
        rc = gcge_record_error(GCGE_CUDA_ERR_CUDA, "ChebyshevPCG: step failed");
        break;
      }
      if (*h_count == 0) break;
    }
  }
  if (rc == GCGE_CUDA_OK &&
      (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess))
    rc = gcge_record_error(GCGE_CUDA_ERR_CUDA, "ChebyshevPCG: kernels failed");
  cudaFreeHost(h_count);
  return rc;
}
