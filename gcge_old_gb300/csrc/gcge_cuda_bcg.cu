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
// 256-thread blocks of the fused A p kernel resident per SM at block widths <= 12
// (five measured no faster: the kernel then spills)
constexpr int kApBlocks12 = 4;
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
                                                 double* __restrict__ partial,
                                                 const int* __restrict__ hidx,
                                                 const T* __restrict__ hb) {
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
    const int h = hidx ? __ldg(hidx + r) : -1;
    if (h >= 0) {  // a heavy row: its products were formed chunk by chunk
#pragma unroll
      for (int c = 0; c < KC; c++)
        if (c < kc) ax[c] = hb[(size_t)h * len + c0 + c];
    } else {
      for (int j = __ldg(rp + r); j < __ldg(rp + r + 1); j++) {
        const int col = __ldg(ci + j);
        const T a = __ldg(val + j);
#pragma unroll
        for (int c = 0; c < KC; c++)
          if (c < kc) ax[c] = fma(a, X.p[c0 + c][col], ax[c]);
      }
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
    // one division per block (not per thread: FP64 divisions are costly on GB300)
    __shared__ T beta_s;
    if (threadIdx.x == 0) beta_s = (T)(s.rho2[idx] / s.rho1[idx]);
    __syncthreads();
    const T beta = beta_s;
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
                                               double* __restrict__ partial,
                                               const int* __restrict__ hidx,
                                               const T* __restrict__ hb, int kmax) {
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
    const int h = hidx ? __ldg(hidx + r) : -1;
    if (h >= 0) {  // a heavy row: products of the active ids, formed chunk by chunk
#pragma unroll
      for (int c = 0; c < KC; c++)
        if (c < kc) ap[c] = hb[(size_t)h * kmax + c0 + c];
    } else {
      for (int j = __ldg(rp + r); j < __ldg(rp + r + 1); j++) {
        const int col = __ldg(ci + j);
        const T a = __ldg(val + j);
#pragma unroll
        for (int c = 0; c < KC; c++)
          if (c < kc) ap[c] = fma(a, P.p[ix[c]][col], ap[c]);
      }
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
  __shared__ T alpha_s;  // one division per block
  if (threadIdx.x == 0) alpha_s = (T)(s.rho2[id] / s.ptw[id]);
  __syncthreads();
  const T alpha = alpha_s;
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
            int* launches, const GcgeDevCsr* M) {
  if (len <= 0) return 0;
  const int nb = nblocks(n);
  int nl = 0;
  // heavy rows: products of the long rows formed chunk-wise first (with the
  // values val, FP64 or the FP32 copy)
  const bool hv = M && M->nheavy > 0;
  const int* hidx = hv ? M->hidx : nullptr;
  const T* hb = hv ? reinterpret_cast<const T*>(M->hb64) : nullptr;
  const int hl = hv ? 2 * ((len + kHeavyGroup - 1) / kHeavyGroup) : 0;  // its launches
  if (hv) heavy_cols<T>(*M, val, X, len, st);
  // FP64: one pass over A for up to 16 columns; FP32: passes of 8 columns
  // (the 16-column FP32 pass, at 80 registers, left too few warps per SM)
  constexpr int KW = sizeof(T) == 8 ? 16 : 8;
  if (len <= 8)
    k_bcg_init<T, 8><<<dim3(nb, 1), kT, 0, st>>>(n, rp, ci, val, X, RHS, len, partial, hidx, hb);
  else
    k_bcg_init<T, KW><<<dim3(nb, (len + KW - 1) / KW), kT, 0, st>>>(n, rp, ci, val, X, RHS,
                                                                      len, partial, hidx, hb);
  k_reduce<<<len, 256, 0, st>>>(partial, nb, len, nullptr, s.rho2);
  k_ctrl_init<<<1, 1, 0, st>>>(s, len);
  nl += 3 + hl;
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
      if (hv) heavy_cols_active<T>(*M, val, P, s.unl, s.nu, len, st);
      if (len <= 8)
        k_bcg_ap<T, 8><<<dim3(nb, 1), kT, 0, st>>>(n, rp, ci, val, P, W, s, partial, hidx, hb,
                                                    len);
      else
        k_bcg_ap<T, KW><<<dim3(nb, (len + KW - 1) / KW), kT, 0, st>>>(n, rp, ci, val, P, W, s,
                                                                       partial, hidx, hb, len);
      k_reduce<<<len, 256, 0, st>>>(partial, nb, len, s.nu, s.ptw);
      k_bcg_update<T><<<dim3(nb, len), kT, 0, st>>>(n, X, RHS, P, W, s, partial);
      k_reduce<<<len, 256, 0, st>>>(partial, nb, len, s.nu, s.rnew);
      k_ctrl_step<<<1, 1, 0, st>>>(s, rate, j);
      nl += 6 + hl;
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
                             cudaStream_t, int*, const GcgeDevCsr*);
template int bcg_run<float>(const int*, const int*, const float*, int, const ColList<float>&,
                            const ColList<float>&, const ColList<float>&, const ColList<float>&,
                            int, int, double, const BcgScalars&, double*, cudaStream_t, int*,
                            const GcgeDevCsr*);

}  // namespace gcge

// ---------------------------------------------------------------- row-interleaved FP32 block CG
namespace gcge {
namespace {

// per-column block sums in the order of block_sum, into partial[c*nblk + b]
template <int KW>
__device__ __forceinline__ void block_sum_cols(const float* acc, int len, double* sh,
                                               double* __restrict__ partial) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < KW; c++) {
    double v = (double)acc[c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[wid * 32 + c] = v;
  }
  __syncthreads();
  if ((int)threadIdx.x < len) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w * 32 + threadIdx.x];
    partial[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = t;
  }
}

template <int KW>
__device__ __forceinline__ void load_row(const float* __restrict__ base, size_t r, float* v) {
  const float4* p = reinterpret_cast<const float4*>(base + r * KW);
#pragma unroll
  for (int q = 0; q < KW / 4; q++) {
    const float4 t = __ldg(p + q);
    v[4 * q] = t.x;
    v[4 * q + 1] = t.y;
    v[4 * q + 2] = t.z;
    v[4 * q + 3] = t.w;
  }
}
template <int KW>
__device__ __forceinline__ void store_row(float* base, size_t r, const float* v) {
  float4* p = reinterpret_cast<float4*>(base + r * KW);
#pragma unroll
  for (int q = 0; q < KW / 4; q++) p[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
}

// acc = (A X)[r] for the row-interleaved block X (acc zeroed here).  With
// G > 1 the entries are taken in groups of G: first the group's column
// indices and values, then its G row gathers, then the FMAs in entry order, so
// G gathers are in flight per thread and the sums are the same as one entry
// at a time.  G is chosen per kernel to stay inside its register budget.
template <int KW, int G>
__device__ __forceinline__ void row_gather(const int* __restrict__ rp, const int* __restrict__ ci,
                                           const float* __restrict__ val,
                                           const float* __restrict__ X, int r, float* acc) {
#pragma unroll
  for (int c = 0; c < KW; c++) acc[c] = 0.f;
  const int e = __ldg(rp + r + 1);
  int j = __ldg(rp + r);
  if (G > 1) {
    for (; j + G <= e; j += G) {
      int col[G];
      float a[G];
#pragma unroll
      for (int u = 0; u < G; u++) {
        col[u] = __ldg(ci + j + u);
        a[u] = __ldg(val + j + u);
      }
      float xv[G][KW];
#pragma unroll
      for (int u = 0; u < G; u++) load_row<KW>(X, col[u], xv[u]);
#pragma unroll
      for (int u = 0; u < G; u++)
#pragma unroll
        for (int c = 0; c < KW; c++) acc[c] = fmaf(a[u], xv[u][c], acc[c]);
    }
  }
  for (; j < e; j++) {
    const int col = __ldg(ci + j);
    const float a = __ldg(val + j);
    float xv[KW];
    load_row<KW>(X, col, xv);
#pragma unroll
    for (int c = 0; c < KW; c++) acc[c] = fmaf(a, xv[c], acc[c]);
  }
}

// v = the product of heavy row h: its chunk partials in chunk order
template <int KW>
__device__ __forceinline__ void heavy_row_sum(const int* __restrict__ hch,
                                              const float* __restrict__ cb, int h, float* v) {
#pragma unroll
  for (int c = 0; c < KW; c++) v[c] = 0.f;
  for (int q = __ldg(hch + h); q < __ldg(hch + h + 1); q++) {
    float t[KW];
    load_row<KW>(cb, q, t);
#pragma unroll
    for (int c = 0; c < KW; c++) v[c] += t[c];
  }
}

// r = rhs - A x and partial ||r_c||^2 (c < len)
template <int KW>
__global__ void __launch_bounds__(kT) k_rows_init(int n, const int* __restrict__ rp,
                                                  const int* __restrict__ ci,
                                                  const float* __restrict__ val,
                                                  const float* __restrict__ X, float* __restrict__ R, int len,
                                                  double* __restrict__ partial,
                                                  const int* __restrict__ hidx,
                                                  const int* __restrict__ hch,
                                                  const float* __restrict__ hb) {
  __shared__ double sh[(kT / 32) * 32];
  float acc2[KW];
#pragma unroll
  for (int c = 0; c < KW; c++) acc2[c] = 0.f;
  for (int r = blockIdx.x * kT + threadIdx.x; r < n; r += gridDim.x * kT) {
    float ax[KW];
#pragma unroll
    for (int c = 0; c < KW; c++) ax[c] = 0.f;
    const int h = hidx ? __ldg(hidx + r) : -1;
    if (h >= 0) {
      heavy_row_sum<KW>(hch, hb, h, ax);
    } else {
      for (int j = __ldg(rp + r); j < __ldg(rp + r + 1); j++) {
        const int col = __ldg(ci + j);
        const float a = __ldg(val + j);
        float xv[KW];
        load_row<KW>(X, col, xv);
#pragma unroll
        for (int c = 0; c < KW; c++) ax[c] = fmaf(a, xv[c], ax[c]);
      }
    }
    float rv[KW];
    load_row<KW>(R, r, rv);
#pragma unroll
    for (int c = 0; c < KW; c++) {
      rv[c] = rv[c] - ax[c];
      acc2[c] = fmaf(rv[c], rv[c], acc2[c]);
    }
    store_row<KW>(R, r, rv);
  }
  block_sum_cols<KW>(acc2, len, sh, partial);
}

// p = r (first step) or p = r + beta p, beta = rho2[c] / rho1[c], for the active columns
template <int KW>
__global__ void __launch_bounds__(kT) k_rows_p(int n, const float* __restrict__ R, float* __restrict__ P,
                                               BcgScalars s, int first) {
  if (*s.nu == 0) return;
  float beta[KW];
  bool on[KW];
#pragma unroll
  for (int c = 0; c < KW; c++) {
    on[c] = s.mask[c] != 0;
    beta[c] = (on[c] && !first) ? s.bcol[c] : 0.f;
  }
  for (int r = blockIdx.x * kT + threadIdx.x; r < n; r += gridDim.x * kT) {
    float rv[KW], pv[KW];
    load_row<KW>(R, r, rv);
    load_row<KW>(P, r, pv);
#pragma unroll
    for (int c = 0; c < KW; c++)
      if (on[c]) pv[c] = first ? rv[c] : rv[c] + beta[c] * pv[c];
    store_row<KW>(P, r, pv);
  }
}

// w = A p and partial p.w for the active columns
template <int KW>
__global__ void __launch_bounds__(kT, KW <= 12 ? kApBlocks12 : 1) k_rows_ap(int n, const int* __restrict__ rp,
                                                const int* __restrict__ ci,
                                                const float* __restrict__ val,
                                                const float* __restrict__ P, float* __restrict__ W, int len,
                                                BcgScalars s, double* __restrict__ partial,
                                                const int* __restrict__ hidx,
                                                const int* __restrict__ hch,
                                                const float* __restrict__ hb) {
  __shared__ double sh[(kT / 32) * 32];
  if (*s.nu == 0) return;
  bool on[KW];
#pragma unroll
  for (int c = 0; c < KW; c++) on[c] = s.mask[c] != 0;
  float dot[KW];
#pragma unroll
  for (int c = 0; c < KW; c++) dot[c] = 0.f;
  for (int r = blockIdx.x * kT + threadIdx.x; r < n; r += gridDim.x * kT) {
    float ap[KW];
#pragma unroll
    for (int c = 0; c < KW; c++) ap[c] = 0.f;
    const int h = hidx ? __ldg(hidx + r) : -1;
    if (h >= 0) {
      heavy_row_sum<KW>(hch, hb, h, ap);
    } else {
      for (int j = __ldg(rp + r); j < __ldg(rp + r + 1); j++) {
        const int col = __ldg(ci + j);
        const float a = __ldg(val + j);
        float pv[KW];
        load_row<KW>(P, col, pv);
#pragma unroll
        for (int c = 0; c < KW; c++) ap[c] = fmaf(a, pv[c], ap[c]);
      }
    }
    store_row<KW>(W, r, ap);
    float pr[KW];
    load_row<KW>(P, r, pr);
#pragma unroll
    for (int c = 0; c < KW; c++)
      if (on[c]) dot[c] = fmaf(pr[c], ap[c], dot[c]);
  }
  block_sum_cols<KW>(dot, len, sh, partial);
}

// x += alpha p, r -= alpha w and partial r.r for the active columns.  The
// blocks are walked as flat float4 arrays (n * KW/4 of them): consecutive
// threads take consecutive float4s, so every load instruction of a warp reads
// 512 contiguous bytes (a thread per 48-byte row touched twice the sectors it
// used and its 4 streams thrashed L1).  The thread count of the grid is a
// multiple of G = KW/4, so a thread keeps one group of 4 columns (4q..4q+3)
// for all its float4s.  Block partials per column: the threads of a group in
// thread order, a warp per column, fixed shuffle tree.
template <int KW>
__global__ void __launch_bounds__(kT, 4) k_rows_update(int n, float* __restrict__ X,
                                                       float* __restrict__ R,
                                                       const float* __restrict__ P,
                                                       const float* __restrict__ W, int len,
                                                       BcgScalars s, double* __restrict__ partial) {
  constexpr int G = KW / 4;
  __shared__ double sacc[4][kT];
  if (*s.nu == 0) return;
  const int f0 = blockIdx.x * kT + threadIdx.x;  // < gridDim.x * kT, which fits an int
  const int q = f0 % G;
  bool on[4];
  float alpha[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    on[j] = s.mask[4 * q + j] != 0;
    alpha[j] = on[j] ? s.acolf[4 * q + j] : 0.f;
  }
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  const long long n4 = (long long)n * G, stride = (long long)gridDim.x * kT;
  float4* X4 = reinterpret_cast<float4*>(X);
  float4* R4 = reinterpret_cast<float4*>(R);
  const float4* P4 = reinterpret_cast<const float4*>(P);
  const float4* W4 = reinterpret_cast<const float4*>(W);
  for (long long f = f0; f < n4; f += stride) {  // f % G == q: stride is a multiple of G
    float4 x = X4[f], r = R4[f];
    const float4 p = __ldg(P4 + f), w = __ldg(W4 + f);
    if (on[0]) { x.x = fmaf(alpha[0], p.x, x.x); r.x = fmaf(-alpha[0], w.x, r.x); acc[0] = fmaf(r.x, r.x, acc[0]); }
    if (on[1]) { x.y = fmaf(alpha[1], p.y, x.y); r.y = fmaf(-alpha[1], w.y, r.y); acc[1] = fmaf(r.y, r.y, acc[1]); }
    if (on[2]) { x.z = fmaf(alpha[2], p.z, x.z); r.z = fmaf(-alpha[2], w.z, r.z); acc[2] = fmaf(r.z, r.z, acc[2]); }
    if (on[3]) { x.w = fmaf(alpha[3], p.w, x.w); r.w = fmaf(-alpha[3], w.w, r.w); acc[3] = fmaf(r.w, r.w, acc[3]); }
    X4[f] = x;
    R4[f] = r;
  }
#pragma unroll
  for (int j = 0; j < 4; j++) sacc[j][threadIdx.x] = (double)acc[j];
  __syncthreads();
  // thread t of this block has group (blockIdx.x * kT + t) % G
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int b0 = (blockIdx.x * kT) % G;
  for (int c = wid; c < len; c += kT / 32) {
    const int g = c >> 2, j = c & 3;
    const int t0 = (g - b0 + G) % G;  // first thread of group g
    double v = 0.0;
    for (int t = t0 + G * lane; t < kT; t += 32 * G) v += sacc[j][t];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) partial[(size_t)c * gridDim.x + blockIdx.x] = v;
  }
}

// column sums of the per-block partials: warp w adds column w (lanes take
// blocks lane, lane + 32, ...; then a fixed shuffle tree), so the order is
// fixed.  Launched with 1024 threads (32 warps, one per column).
__device__ __forceinline__ void reduce_cols(const double* __restrict__ partial, int nblk, int len,
                                            double* out /* shared, 32 */) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (w < len) {
    double v = 0.0;
    for (int b = lane; b < nblk; b += 32) v += partial[(size_t)w * nblk + b];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) out[w] = v;
  }
  __syncthreads();
}

// initial rho2 (by column), err, lerr, active list and mask
__global__ void k_rows_init_ctrl(const double* __restrict__ partial, int nblk, int len,
                                 BcgScalars s) {
  __shared__ double rr[32];
  reduce_cols(partial, nblk, len, rr);
  if (threadIdx.x != 0) return;
  int nu = 0;
  for (int c = 0; c < 32; c++) s.mask[c] = 0;
  for (int idx = 0; idx < len; idx++) {
    s.rho2[idx] = rr[idx];
    s.err[idx] = sqrt(s.rho2[idx]);
    s.lerr[idx] = s.err[idx];
    if (s.err[idx] >= 1e-15) {
      s.unl[nu++] = idx;
      s.mask[idx] = 1;
    }
  }
  *s.nu = nu;
  s.nu_host[0] = nu;
}

// ptw[id] = p.w of column unl[id]; alpha of that column = rho2[id] / ptw[id]
__global__ void k_rows_alpha(const double* __restrict__ partial, int nblk, int len,
                             BcgScalars s) {
  __shared__ double pw[32];
  const int nu = *s.nu;
  if (nu == 0) return;
  reduce_cols(partial, nblk, len, pw);
  if (threadIdx.x != 0) return;
  for (int id = 0; id < nu; id++) {
    const int c = s.unl[id];
    s.ptw[id] = pw[c];
    s.acol[c] = s.rho2[id] / s.ptw[id];
    s.acolf[c] = (float)s.acol[c];  // once here instead of in every thread of k_rows_update
  }
}

// rnew[id] = r.r of column unl[id]; then the step control of k_ctrl_step and the mask
__global__ void k_rows_step(const double* __restrict__ partial, int nblk, int len, BcgScalars s,
                            double rate, int slot) {
  __shared__ double rr[32];
  const int nu = *s.nu;
  if (nu == 0) {
    if (threadIdx.x == 0) s.nu_host[slot] = 0;
    return;
  }
  reduce_cols(partial, nblk, len, rr);
  if (threadIdx.x != 0) return;
  for (int id = 0; id < nu; id++) s.rnew[id] = rr[s.unl[id]];
  for (int id = 0; id < nu; id++) {
    s.rho1[id] = s.rho2[id];
    s.rho2[id] = s.rnew[id];
  }
  for (int id = 0; id < nu; id++) s.lerr[s.unl[id]] = sqrt(fabs(s.rho2[id]));
  for (int c = 0; c < 32; c++) s.mask[c] = 0;
  int m = 0;
  for (int id = 0; id < nu; id++) {
    const int idx = s.unl[id];
    if (s.lerr[idx] >= rate * s.err[idx] && s.lerr[idx] >= 1e-15) {
      s.unl[m++] = idx;
      s.mask[idx] = 1;
    }
  }
  // beta of the next p step, once here instead of in every thread of k_rows_p;
  // indexed by column as the reference indexes it (rho arrays by active id)
  for (int c = 0; c < 32; c++) s.bcol[c] = s.mask[c] ? (float)(s.rho2[c] / s.rho1[c]) : 0.f;
  *s.nu = m;
  s.nu_host[slot] = m;
}

// y = A x on row-interleaved blocks (the operator of the mixed block CG)
template <int KW>
__global__ void __launch_bounds__(kT, KW <= 12 ? 6 : (KW <= 16 ? 4 : 2))
    k_rows_spmm(int n, const int* __restrict__ rp,
                                                  const int* __restrict__ ci,
                                                  const float* __restrict__ val,
                                                  const float* __restrict__ X, float* Y,
                                                  const int* __restrict__ hidx,
                                                  const int* __restrict__ hch,
                                                  const float* __restrict__ hb) {
  const int r = blockIdx.x * kT + threadIdx.x;
  if (r >= n) return;
  float acc[KW];
  const int h = hidx ? __ldg(hidx + r) : -1;
  if (h >= 0)
    heavy_row_sum<KW>(hch, hb, h, acc);
  else
    row_gather<KW, 1>(rp, ci, val, X, r, acc);
  store_row<KW>(Y, r, acc);
}

template <int KW>
__global__ void k_cols_to_rows(ColList<double> R, int len, float* __restrict__ Rr, int n) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  float v[KW];
#pragma unroll
  for (int c = 0; c < KW; c++) v[c] = c < len ? (float)R.p[c][r] : 0.f;
  store_row<KW>(Rr, r, v);
}

template <int KW>
__global__ void k_rows_to_cols(const float* __restrict__ Xr, int len, ColList<double> Y, int n) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  float v[KW];
  load_row<KW>(Xr, r, v);
#pragma unroll
  for (int c = 0; c < KW; c++)
    if (c < len) Y.p[c][r] = (double)v[c];
}

template <int KW>
int rows_run(const int* rp, const int* ci, const float* val, int n, float* R, float* X, float* P,
             float* W, int len, int max_it, double rate, const BcgScalars& s, double* partial,
             cudaStream_t st, int* launches, const GcgeDevCsr* M) {
  const bool hv = M && M->nheavy > 0;
  const int* hidx = hv ? M->hidx : nullptr;
  // four CTAs of 8 warps per SM for the row-streaming kernels (two from 20
  // columns up, where the update kernel holds over 100 registers a thread);
  // the latency-bound A p kernel gets kApBlocks12 up to 12 columns
  const int nb = min((n + kT - 1) / kT, (KW <= 16 ? 4 : 2) * 152);
  const int nba = KW <= 12 ? min((n + kT - 1) / kT, kApBlocks12 * 152) : nb;
  // the update kernel: flat float4s, four CTAs per SM (its loop is unrolled
  // into 56-64 registers; at six CTAs it spilled), a multiple of KW/4 CTAs
  const long long n4 = (long long)n * (KW / 4);
  int nbu = (int)((n4 + kT - 1) / kT);
  if (nbu > 4 * 152) nbu = 4 * 152;
  nbu = nbu / (KW / 4) * (KW / 4);
  if (nbu < KW / 4) nbu = KW / 4;
  int nl = 0;
  if (hv) heavy_rows_f32(*M, val, X, KW, nullptr, st);
  k_rows_init<KW><<<nb, kT, 0, st>>>(n, rp, ci, val, X, R, len, partial, hidx,
                                     hv ? M->hch : nullptr, hv ? M->cb32 : nullptr);
  k_rows_init_ctrl<<<1, 1024, 0, st>>>(partial, nb, len, s);
  nl += 2;
  if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
  int niter = 1;
  int nu = s.nu_host[0];
  while (nu > 0 && niter < max_it) {
    const int batch = (max_it - niter) < kBatch ? (max_it - niter) : kBatch;
    for (int j = 0; j < batch; j++) {
      k_rows_p<KW><<<nb, kT, 0, st>>>(n, R, P, s, niter + j == 1 ? 1 : 0);
      if (hv) heavy_rows_f32(*M, val, P, KW, s.nu, st);
      k_rows_ap<KW><<<nba, kT, 0, st>>>(n, rp, ci, val, P, W, len, s, partial, hidx,
                                        hv ? M->hch : nullptr, hv ? M->cb32 : nullptr);
      k_rows_alpha<<<1, 1024, 0, st>>>(partial, nba, len, s);
      k_rows_update<KW><<<nbu, kT, 0, st>>>(n, X, R, P, W, len, s, partial);
      k_rows_step<<<1, 1024, 0, st>>>(partial, nbu, len, s, rate, j);
      nl += 5;
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    for (int j = 0; j < batch; j++) {
      niter++;
      nu = s.nu_host[j];
      if (nu == 0) break;
    }
  }
  if (launches) *launches += nl;
  return niter;
}

}  // namespace

int bcg_run_rows_f32(const int* rp, const int* ci, const float* val, int n, float* R, float* X,
                     float* P, float* W, int len, int max_it, double rate, const BcgScalars& s,
                     double* partial, cudaStream_t st, int* launches, const GcgeDevCsr* M) {
  if (len <= 0) return 0;
  switch (bcg_rows_width(len)) {
    case 4: return rows_run<4>(rp, ci, val, n, R, X, P, W, len, max_it, rate, s, partial, st, launches, M);
    case 8: return rows_run<8>(rp, ci, val, n, R, X, P, W, len, max_it, rate, s, partial, st, launches, M);
    case 12: return rows_run<12>(rp, ci, val, n, R, X, P, W, len, max_it, rate, s, partial, st, launches, M);
    case 16: return rows_run<16>(rp, ci, val, n, R, X, P, W, len, max_it, rate, s, partial, st, launches, M);
    case 20: return rows_run<20>(rp, ci, val, n, R, X, P, W, len, max_it, rate, s, partial, st, launches, M);
    case 24: return rows_run<24>(rp, ci, val, n, R, X, P, W, len, max_it, rate, s, partial, st, launches, M);
    case 28: return rows_run<28>(rp, ci, val, n, R, X, P, W, len, max_it, rate, s, partial, st, launches, M);
    case 32: return rows_run<32>(rp, ci, val, n, R, X, P, W, len, max_it, rate, s, partial, st, launches, M);
  }
  return -1;
}

void spmm_rows_f32(const int* rp, const int* ci, const float* val, int n, const float* X,
                   float* Y, int k, cudaStream_t st, const GcgeDevCsr* M) {
  const int g = (n + kT - 1) / kT;
  const bool hv = M && M->nheavy > 0;
  if (hv) heavy_rows_f32(*M, val, X, bcg_rows_width(k), nullptr, st);
  const int* hidx = hv ? M->hidx : nullptr;
  const int* hch = hv ? M->hch : nullptr;
  const float* hb = hv ? M->cb32 : nullptr;
  switch (bcg_rows_width(k)) {
    case 4: k_rows_spmm<4><<<g, kT, 0, st>>>(n, rp, ci, val, X, Y, hidx, hch, hb); break;
    case 8: k_rows_spmm<8><<<g, kT, 0, st>>>(n, rp, ci, val, X, Y, hidx, hch, hb); break;
    case 12: k_rows_spmm<12><<<g, kT, 0, st>>>(n, rp, ci, val, X, Y, hidx, hch, hb); break;
    case 16: k_rows_spmm<16><<<g, kT, 0, st>>>(n, rp, ci, val, X, Y, hidx, hch, hb); break;
    case 20: k_rows_spmm<20><<<g, kT, 0, st>>>(n, rp, ci, val, X, Y, hidx, hch, hb); break;
    case 24: k_rows_spmm<24><<<g, kT, 0, st>>>(n, rp, ci, val, X, Y, hidx, hch, hb); break;
    case 28: k_rows_spmm<28><<<g, kT, 0, st>>>(n, rp, ci, val, X, Y, hidx, hch, hb); break;
    case 32: k_rows_spmm<32><<<g, kT, 0, st>>>(n, rp, ci, val, X, Y, hidx, hch, hb); break;
  }
}

void cols_to_rows_f32(const ColList<double>& R, int len, float* Rr, int n, cudaStream_t st) {
  const int g = (n + 255) / 256;
  switch (bcg_rows_width(len)) {
    case 4: k_cols_to_rows<4><<<g, 256, 0, st>>>(R, len, Rr, n); break;
    case 8: k_cols_to_rows<8><<<g, 256, 0, st>>>(R, len, Rr, n); break;
    case 12: k_cols_to_rows<12><<<g, 256, 0, st>>>(R, len, Rr, n); break;
    case 16: k_cols_to_rows<16><<<g, 256, 0, st>>>(R, len, Rr, n); break;
    case 20: k_cols_to_rows<20><<<g, 256, 0, st>>>(R, len, Rr, n); break;
    case 24: k_cols_to_rows<24><<<g, 256, 0, st>>>(R, len, Rr, n); break;
    case 28: k_cols_to_rows<28><<<g, 256, 0, st>>>(R, len, Rr, n); break;
    case 32: k_cols_to_rows<32><<<g, 256, 0, st>>>(R, len, Rr, n); break;
  }
}

void rows_to_cols_f64(const float* Xr, int len, const ColList<double>& Y, int n,
                      cudaStream_t st) {
  const int g = (n + 255) / 256;
  switch (bcg_rows_width(len)) {
    case 4: k_rows_to_cols<4><<<g, 256, 0, st>>>(Xr, len, Y, n); break;
    case 8: k_rows_to_cols<8><<<g, 256, 0, st>>>(Xr, len, Y, n); break;
    case 12: k_rows_to_cols<12><<<g, 256, 0, st>>>(Xr, len, Y, n); break;
    case 16: k_rows_to_cols<16><<<g, 256, 0, st>>>(Xr, len, Y, n); break;
    case 20: k_rows_to_cols<20><<<g, 256, 0, st>>>(Xr, len, Y, n); break;
    case 24: k_rows_to_cols<24><<<g, 256, 0, st>>>(Xr, len, Y, n); break;
    case 28: k_rows_to_cols<28><<<g, 256, 0, st>>>(Xr, len, Y, n); break;
    case 32: k_rows_to_cols<32><<<g, 256, 0, st>>>(Xr, len, Y, n); break;
  }
}

}  // namespace gcge
