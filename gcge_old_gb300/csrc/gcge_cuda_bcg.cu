// Block conjugate gradient for the W step of GCG, device resident.
//
// Follows GCGE_BCG (src/gcge_cg.c:302-501): per-column CG on A w = rhs with
// per-column lock-out once ||r_k|| < rate * ||r_0|| or ||r_k|| < 1e-15.  The
// reference's scalar bookkeeping is kept exactly, including that once a
// column has locked out the scalars are addressed by the compacted index in
// some places (alpha, rho update: :451,465,474) and by the column index in
// others (beta: :411).  All scalars and the active list live in device
// memory; a one-thread control kernel updates them after every reduction, so
// the host only reads the active count.
//
// T = double for the all-FP64 solve, T = float for the mixed-precision solve
// (FP32 copies of A and of the vectors; scalars and reductions in FP64).
#include "gcge_cuda_common.cuh"
#include "gcge_cuda_bcg.cuh"

namespace gcge {
namespace {

constexpr int kT = 256;
constexpr int kBatch = 4;  // steps launched per host synchronisation

__device__ inline double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += sh[w];
  return s;
}

// r_c = rhs_c - A x_c  and  partial ||r_c||^2, for every column c < len.
template <typename T, int KC>
__global__ void __launch_bounds__(kT) k_bcg_init(int n, const int* __restrict__ rp,
                                                 const int* __restrict__ ci,
                                                 const T* __restrict__ val, ColList<T> X,
                                                 ColList<T> R, int len,
                                                 double* __restrict__ partial) {
  __shared__ double sh[32];
  const int c0 = blockIdx.y * KC;
  const int kc = min(KC, len - c0);
  T acc2[KC];
#pragma unroll
  for (int c = 0; c < KC; c++) acc2[c] = T(0);
  for (int r = blockIdx.x * kT + threadIdx.x; r < n; r += gridDim.x * kT) {
    T ax[KC];
#pragma unroll
    for (int c = 0; c < KC; c++) ax[c] = T(0);
    for (int j = __ldg(rp + r); j < __ldg(rp + r + 1); j++) {
      const int col = __ldg(ci + j);
      const T a = __ldg(val + j);
#pragma unroll
      for (int c = 0; c < KC; c++)
        if (c < kc) ax[c] = fma(a, X.p[c0 + c][col], ax[c]);
    }
#pragma unroll
    for (int c = 0; c < KC; c++)
      if (c < kc) {
        T* rr = R.p[c0 + c] + r;
        const T v = *rr - ax[c];
        *rr = v;
        acc2[c] = fma(v, v, acc2[c]);
      }
  }
  for (int c = 0; c < kc; c++) {
    const double s = block_sum((double)acc2[c], sh);
    if (threadIdx.x == 0) partial[(size_t)(c0 + c) * gridDim.x + blockIdx.x] = s;
  }
}

// out[c] = sum_b partial[c*nblk + b] for c < k (or c < *active when given).
__global__ void k_reduce(const double* __restrict__ partial, int nblk, int k,
                         const int* __restrict__ active, double* __restrict__ out) {
  __shared__ double sh[32];
  const int c = blockIdx.x;
  if (c >= k) return;
  if (active && c >= *active) return;
  double s = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += partial[(size_t)c * nblk + b];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) out[c] = s;
}

// :392-410 initial residual norms and the first active list.
__global__ void k_ctrl_init(BcgScalars s, int len) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int nu = 0;
  for (int idx = 0; idx < len; idx++) {
    s.err[idx] = sqrt(s.rho2[idx]);
    s.lerr[idx] = s.err[idx];
    if (s.err[idx] >= 1e-15) s.unl[nu++] = idx;
  }
  *s.nu = nu;
  *s.nu_host = nu;
}

// :414-427 p = r (first step) or p = r + beta p with beta = rho2[idx]/rho1[idx].
template <typename T>
__global__ void k_bcg_p(int n, ColList<T> R, ColList<T> P, BcgScalars s, int first) {
  const int id = blockIdx.y;
  if (id >= *s.nu) return;
  const int idx = s.unl[id];
  const T* r = R.p[idx];
  T* p = P.p[idx];
  if (first) {
    for (int i = blockIdx.x * kT + threadIdx.x; i < n; i += gridDim.x * kT) p[i] = r[i];
  } else {
    const T beta = (T)(s.rho2[idx] / s.rho1[idx]);
    for (int i = blockIdx.x * kT + threadIdx.x; i < n; i += gridDim.x * kT)
      p[i] = r[i] + beta * p[i];
  }
}

// :429-445 w = A p and partial p.w for the active ids (KC per pass).
template <typename T, int KC>
__global__ void __launch_bounds__(kT) k_bcg_ap(int n, const int* __restrict__ rp,
                                               const int* __restrict__ ci,
                                               const T* __restrict__ val, ColList<T> P,
                                               ColList<T> W, BcgScalars s,
                                               double* __restrict__ partial) {
  __shared__ double sh[32];
  const int nu = *s.nu;
  const int c0 = blockIdx.y * KC;
  if (c0 >= nu) return;
  const int kc = min(KC, nu - c0);
  int ix[KC];  // column of each active id (pointers read from the parameter block)
#pragma unroll
  for (int c = 0; c < KC; c++) ix[c] = (c < kc) ? s.unl[c0 + c] : s.unl[c0];
  T dot[KC];
#pragma unroll
  for (int c = 0; c < KC; c++) dot[c] = T(0);
  for (int r = blockIdx.x * kT + threadIdx.x; r < n; r += gridDim.x * kT) {
    T ap[KC];
#pragma unroll
    for (int c = 0; c < KC; c++) ap[c] = T(0);
    for (int j = __ldg(rp + r); j < __ldg(rp + r + 1); j++) {
      const int col = __ldg(ci + j);
      const T a = __ldg(val + j);
#pragma unroll
      for (int c = 0; c < KC; c++)
        if (c < kc) ap[c] = fma(a, P.p[ix[c]][col], ap[c]);
    }
#pragma unroll
    for (int c = 0; c < KC; c++)
      if (c < kc) {
        W.p[ix[c]][r] = ap[c];
        dot[c] = fma(P.p[ix[c]][r], ap[c], dot[c]);
      }
  }
  for (int c = 0; c < kc; c++) {
    const double v = block_sum((double)dot[c], sh);
    if (threadIdx.x == 0) partial[(size_t)(c0 + c) * gridDim.x + blockIdx.x] = v;
  }
}

// :448-476 alpha = rho2[id]/ptw[id]; x += alpha p; r -= alpha w; partial r.r
template <typename T>
__global__ void k_bcg_update(int n, ColList<T> X, ColList<T> R, ColList<T> P, ColList<T> W,
                             BcgScalars s, double* __restrict__ partial) {
  __shared__ double sh[32];
  const int id = blockIdx.y;
  if (id >= *s.nu) return;
  const int idx = s.unl[id];
  const T alpha = (T)(s.rho2[id] / s.ptw[id]);
  T* x = X.p[idx];
  T* r = R.p[idx];
  const T* p = P.p[idx];
  const T* w = W.p[idx];
  T acc = T(0);
  for (int i = blockIdx.x * kT + threadIdx.x; i < n; i += gridDim.x * kT) {
    x[i] = fma(alpha, p[i], x[i]);
    const T rv = fma(-alpha, w[i], r[i]);
    r[i] = rv;
    acc = fma(rv, rv, acc);
  }
  const double v = block_sum((double)acc, sh);
  if (threadIdx.x == 0) partial[(size_t)id * gridDim.x + blockIdx.x] = v;
}

// :465-495 rho1 <- rho2, rho2 <- r.r, error update and the new active list;
// the active count also goes to host slot `slot` (one per step of a batch).
__global__ void k_ctrl_step(BcgScalars s, double rate, int slot) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int nu = *s.nu;
  for (int id = 0; id < nu; id++) {
    s.rho1[id] = s.rho2[id];
    s.rho2[id] = s.rnew[id];
  }
  for (int id = 0; id < nu; id++) s.lerr[s.unl[id]] = sqrt(fabs(s.rho2[id]));
  int m = 0;
  for (int id = 0; id < nu; id++) {
    const int idx = s.unl[id];
    if (s.lerr[idx] >= rate * s.err[idx] && s.lerr[idx] >= 1e-15) s.unl[m++] = idx;
  }
  *s.nu = m;
  s.nu_host[slot] = m;
}

inline int nblocks(int n) {
  int b = (n + kT - 1) / kT;
  return b < kRowBlocks ? (b < 1 ? 1 : b) : kRowBlocks;
}

}  // namespace

template <typename T>
int bcg_run(const int* rp, const int* ci, const T* val, int n, const ColList<T>& RHS,
            const ColList<T>& X, const ColList<T>& P, const ColList<T>& W, int len, int max_it,
            double rate, const BcgScalars& s, double* partial, cudaStream_t st,
            int* launches) {
  if (len <= 0) return 0;
  const int nb = nblocks(n);
  int nl = 0;
  // FP64: one pass over A for up to 16 columns; FP32: passes of 8 columns
  // (the 16-column FP32 pass, at 80 registers, left too few warps per SM)
  constexpr int KW = sizeof(T) == 8 ? 16 : 8;
  if (len <= 8)
    k_bcg_init<T, 8><<<dim3(nb, 1), kT, 0, st>>>(n, rp, ci, val, X, RHS, len, partial);
  else
    k_bcg_init<T, KW><<<dim3(nb, (len + KW - 1) / KW), kT, 0, st>>>(n, rp, ci, val, X, RHS,
                                                                      len, partial);
  k_reduce<<<len, 256, 0, st>>>(partial, nb, len, nullptr, s.rho2);
  k_ctrl_init<<<1, 1, 0, st>>>(s, len);
  nl += 3;
  if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
  int niter = 1;
  int nu = s.nu_host[0];
  // Steps are launched kBatch at a time between host synchronisations.  Every
  // kernel of a step reads the active count on the device and does nothing
  // once it is 0, so the steps past convergence are empty; step j of a batch
  // leaves the active count in host slot j, from which the host counts the
  // steps that ran (the reference's niter).
  while (nu > 0 && niter < max_it) {
    const int batch = (max_it - niter) < kBatch ? (max_it - niter) : kBatch;
    for (int j = 0; j < batch; j++) {
      k_bcg_p<T><<<dim3(nb, len), kT, 0, st>>>(n, RHS, P, s, niter + j == 1 ? 1 : 0);
      if (len <= 8)
        k_bcg_ap<T, 8><<<dim3(nb, 1), kT, 0, st>>>(n, rp, ci, val, P, W, s, partial);
      else
        k_bcg_ap<T, KW><<<dim3(nb, (len + KW - 1) / KW), kT, 0, st>>>(n, rp, ci, val, P, W, s,
                                                                       partial);
      k_reduce<<<len, 256, 0, st>>>(partial, nb, len, s.nu, s.ptw);
      k_bcg_update<T><<<dim3(nb, len), kT, 0, st>>>(n, X, RHS, P, W, s, partial);
      k_reduce<<<len, 256, 0, st>>>(partial, nb, len, s.nu, s.rnew);
      k_ctrl_step<<<1, 1, 0, st>>>(s, rate, j);
      nl += 6;
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    for (int j = 0; j < batch; j++) {
      niter++;  // step j ran: the count before it was > 0
      nu = s.nu_host[j];
      if (nu == 0) break;
    }
  }
  if (launches) *launches += nl;
  return niter;
}

template int bcg_run<double>(const int*, const int*, const double*, int, const ColList<double>&,
                             const ColList<double>&, const ColList<double>&,
                             const ColList<double>&, int, int, double, const BcgScalars&, double*,
                             cudaStream_t, int*);
template int bcg_run<float>(const int*, const int*, const float*, int, const ColList<float>&,
                            const ColList<float>&, const ColList<float>&, const ColList<float>&,
                            int, int, double, const BcgScalars&, double*, cudaStream_t, int*);

}  // namespace gcge
