// Large-vector kernels of the GB300 GCG eigensolver: CSR SpMM, tall-skinny
// Gram products and linear combinations, residual norms and column updates.
//
// Layout: every vector is one contiguous length-n column (256-byte aligned
// allocation); multivectors are ColLists of column pointers.  Reductions are
// deterministic: each block writes a partial sum, a second kernel adds the
// partials in a fixed order.
#include "gcge_cuda_common.cuh"

namespace gcge {

namespace {

constexpr int kThreads = 256;

inline int row_blocks(int n) {
  int b = (n + kThreads - 1) / kThreads;
  return b < kRowBlocks ? (b < 1 ? 1 : b) : kRowBlocks;
}

// ---------------------------------------------------------------- SpMM
// Thread per row, KC columns per pass so A's row is read once per pass.
// Reference: CSR_MatDotVec (app/csr/gcge_app_csr.c:297-323) column by column
// through GCGE_Default_MatDotMultiVec (src/gcge_ops.c:115-129).
template <typename T, int KC>
__global__ void __launch_bounds__(kThreads) k_spmm(int n, const int* __restrict__ rp,
                                                   const int* __restrict__ ci,
                                                   const T* __restrict__ val, ColList<T> X,
                                                   ColList<T> Y, int k,
                                                   const int* __restrict__ hidx,
                                                   const T* __restrict__ hb) {
  const int row = blockIdx.x * kThreads + threadIdx.x;
  if (row >= n) return;
  const int c0 = blockIdx.y * KC;
  const int kc = min(KC, k - c0);
  if (hidx) {  // a heavy row: its products were formed chunk by chunk
    const int h = __ldg(hidx + row);
    if (h >= 0) {
#pragma unroll
      for (int c = 0; c < KC; c++)
        if (c < kc) Y.p[c0 + c][row] = hb[(size_t)h * k + c0 + c];
      return;
    }
  }
  T acc[KC];
#pragma unroll
  for (int c = 0; c < KC; c++) acc[c] = T(0);
  const int s = __ldg(rp + row), e = __ldg(rp + row + 1);
  for (int j = s; j < e; j++) {
    const int col = __ldg(ci + j);
    const T a = __ldg(val + j);
#pragma unroll
    for (int c = 0; c < KC; c++)
      if (c < kc) acc[c] = fma(a, __ldg(X.p[c0 + c] + col), acc[c]);
  }
#pragma unroll
  for (int c = 0; c < KC; c++)
    if (c < kc) Y.p[c0 + c][row] = acc[c];
}

template <typename T>
__global__ void k_diag_mul(int n, const T* __restrict__ d, ColList<T> X, ColList<T> Y, int k) {
  const int row = blockIdx.x * kThreads + threadIdx.x;
  if (row >= n) return;
  const T dv = d[row];
  for (int c = 0; c < k; c++) Y.p[c][row] = dv * X.p[c][row];
}

// ---------------------------------------------------------------- Gram
// 64 x 64 output tile per block, 4 x 4 register tile per thread, rows
// staged 32 at a time in shared memory; grid.x splits the rows.
constexpr int GT = 64, GR = 32;

__global__ void __launch_bounds__(kThreads) k_gram(ColList<double> V, int k1, ColList<double> W,
                                                   int k2, int n, int tiles_j, int sym,
                                                   double* __restrict__ partial) {
  __shared__ double Vs[GR][GT];
  __shared__ double Ws[GR][GT];
  const int tile = blockIdx.y;
  const int ti = tile / tiles_j, tj = tile % tiles_j;
  if (sym && ti > tj) return;
  const int t = threadIdx.x, tx = t % 16, ty = t / 16;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = 0.0;
  const int i0 = ti * GT, j0 = tj * GT;
  const int nchunks = (n + GR - 1) / GR;
  for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const int r0 = ch * GR;
#pragma unroll
    for (int e = 0; e < (GR * GT) / kThreads; e++) {
      const int idx = e * kThreads + t;
      const int rr = idx % GR, cc = idx / GR;
      const int r = r0 + rr;
      double v = 0.0, w = 0.0;
      if (r < n) {
        if (i0 + cc < k1) v = V.p[i0 + cc][r];
        if (j0 + cc < k2) w = W.p[j0 + cc][r];
      }
      Vs[rr][cc] = v;
      Ws[rr][cc] = w;
    }
    __syncthreads();
#pragma unroll 8
    for (int rr = 0; rr < GR; rr++) {
      double a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        a[q] = Vs[rr][tx * 4 + q];
        b[q] = Ws[rr][ty * 4 + q];
      }
#pragma unroll
      for (int p = 0; p < 4; p++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[p][q] = fma(a[p], b[q], acc[p][q]);
    }
    __syncthreads();
  }
  double* out = partial + ((size_t)blockIdx.x * gridDim.y + tile) * (GT * GT);
#pragma unroll
  for (int p = 0; p < 4; p++)
#pragma unroll
    for (int q = 0; q < 4; q++) out[(tx * 4 + p) * GT + ty * 4 + q] = acc[p][q];
}

// Gram for narrow blocks (k1 * k2 <= 4096): every thread owns up to 16 of
// the k1 x k2 outputs, rows are staged GR at a time, so no FMA is spent on
// padding when k2 is a block-size-wide W block (10..25 columns).
constexpr int GF_MAX = 16;
__global__ void __launch_bounds__(kThreads) k_gram_flex(ColList<double> V, int k1,
                                                        ColList<double> W, int k2, int n,
                                                        int sym, double* __restrict__ partial) {
  extern __shared__ double gsm[];  // [GR][k1] then [GR][k2]
  double* Vs = gsm;
  double* Ws = gsm + GR * k1;
  const int t = threadIdx.x;
  const int nout = k1 * k2;
  double acc[GF_MAX];
  int oi[GF_MAX], oj[GF_MAX];
#pragma unroll
  for (int q = 0; q < GF_MAX; q++) {
    acc[q] = 0.0;
    const int o = t + q * kThreads;
    oi[q] = (o < nout) ? o % k1 : 0;
    oj[q] = (o < nout) ? o / k1 : 0;
  }
  const int nchunks = (n + GR - 1) / GR;
  for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const int r0 = ch * GR;
    for (int e = t; e < GR * (k1 + k2); e += kThreads) {
      const int rr = e % GR, c = e / GR;
      const int r = r0 + rr;
      if (c < k1) Vs[rr * k1 + c] = (r < n) ? V.p[c][r] : 0.0;
      else Ws[rr * k2 + (c - k1)] = (r < n) ? W.p[c - k1][r] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < GF_MAX; q++) {
      if (t + q * kThreads >= nout) break;
      if (sym && oi[q] > oj[q]) continue;
      double a = acc[q];
      for (int rr = 0; rr < GR; rr++) a = fma(Vs[rr * k1 + oi[q]], Ws[rr * k2 + oj[q]], a);
      acc[q] = a;
    }
    __syncthreads();
  }
  double* out = partial + (size_t)blockIdx.x * nout;
#pragma unroll
  for (int q = 0; q < GF_MAX; q++) {
    const int o = t + q * kThreads;
    if (o < nout) out[o] = acc[q];
  }
}

__global__ void k_gram_flex_reduce(int k1, int k2, int nblk, int sym,
                                   const double* __restrict__ partial, double* __restrict__ G,
                                   int ldg) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  const int nout = k1 * k2;
  if (o >= nout) return;
  const int i = o % k1, j = o / k1;
  if (sym && i > j) return;
  double s = 0.0;
  for (int b = 0; b < nblk; b++) s += partial[(size_t)b * nout + o];
  G[i + (size_t)j * ldg] = s;
  if (sym && i < j) G[j + (size_t)i * ldg] = s;
}

// G[i + j*ldg] = sum over row blocks of the partial tiles (fixed order).
__global__ void k_gram_reduce(int k1, int k2, int tiles_j, int nblk, int sym,
                              const double* __restrict__ partial, double* __restrict__ G,
                              int ldg) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= k1 * k2) return;
  const int i = e % k1, j = e / k1;
  if (sym && i > j) return;
  const int ti = i / GT, tj = j / GT;
  const int tile = ti * tiles_j + tj;
  const int ntiles = ((k1 + GT - 1) / GT) * tiles_j;
  const int off = (i % GT) * GT + (j % GT);
  double s = 0.0;
  for (int b = 0; b < nblk; b++) s += partial[((size_t)b * ntiles + tile) * (GT * GT) + off];
  G[i + (size_t)j * ldg] = s;
  if (sym && i < j) G[j + (size_t)i * ldg] = s;
}

// ---------------------------------------------------------------- LinComb
// Thread per row, 32 output columns per block column, coefficients in
// shared memory.  Reference: GCGE_Default_MultiVecLinearComb
// (src/gcge_ops.c:190-221).
constexpr int LT = 128;

template <int LJ>
__global__ void __launch_bounds__(LT) k_lincomb(ColList<double> X, int k1,
                                                const double* __restrict__ C, int ldc,
                                                ColList<double> Y, int k2, double beta, int n) {
  extern __shared__ double Cs[];  // [k1][LJ]
  const int j0 = blockIdx.y * LJ;
  const int kj = min(LJ, k2 - j0);
  for (int e = threadIdx.x; e < k1 * LJ; e += LT) {
    const int i = e / LJ, j = e % LJ;
    Cs[e] = (j < kj) ? C[i + (size_t)(j0 + j) * ldc] : 0.0;
  }
  __syncthreads();
  const int row = blockIdx.x * LT + threadIdx.x;
  if (row >= n) return;
  double acc[LJ];
#pragma unroll
  for (int j = 0; j < LJ; j++) acc[j] = 0.0;
  for (int i = 0; i < k1; i++) {
    const double x = __ldg(X.p[i] + row);
    const double* c = Cs + i * LJ;
#pragma unroll
    for (int j = 0; j < LJ; j++) acc[j] = fma(x, c[j], acc[j]);
  }
#pragma unroll
  for (int j = 0; j < LJ; j++)
    if (j < kj) {
      double* y = Y.p[j0 + j] + row;
      *y = (beta == 0.0) ? acc[j] : fma(beta, *y, acc[j]);
    }
}

// ---------------------------------------------------------------- column ops
__global__ void k_axpby(double a, ColList<double> X, double b, ColList<double> Y, int k, int n) {
  const int row = blockIdx.x * kThreads + threadIdx.x;
  if (row >= n) return;
  const int c = blockIdx.y;
  if (c >= k) return;
  double* y = Y.p[c] + row;
  // same special cases as CSR_VecAxpby (app/csr/gcge_app_csr.c:330-365)
  if (a == 0.0) *y = b * *y;
  else if (b == 0.0) *y = (a == 1.0) ? X.p[c][row] : a * X.p[c][row];
  else *y = a * X.p[c][row] + b * *y;
}

__global__ void k_scale_cols(ColList<double> Y, const double* __restrict__ s, int k, int n) {
  const int row = blockIdx.x * kThreads + threadIdx.x;
  if (row >= n) return;
  const int c = blockIdx.y;
  if (c >= k) return;
  Y.p[c][row] *= s[c];
}

template <typename S, typename D>
__global__ void k_convert(ColList<S> X, ColList<D> Y, int k, int n) {
  const int row = blockIdx.x * kThreads + threadIdx.x;
  if (row >= n) return;
  const int c = blockIdx.y;
  if (c >= k) return;
  Y.p[c][row] = (D)X.p[c][row];
}

// Block-level sum of one value per thread into out (thread 0 returns it).
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

__global__ void k_colnorm2(ColList<double> X, int k, int n, double* __restrict__ partial) {
  __shared__ double sh[32];
  const int c = blockIdx.y;
  double s = 0.0;
  for (int r = blockIdx.x * kThreads + threadIdx.x; r < n; r += gridDim.x * kThreads) {
    const double v = X.p[c][r];
    s = fma(v, v, s);
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partial[(size_t)c * gridDim.x + blockIdx.x] = s;
}

// out[c] = sum_b partial[c*nblk + b]
__global__ void k_reduce_rows(const double* __restrict__ partial, int nblk, int k,
                              double* __restrict__ out) {
  __shared__ double sh[32];
  const int c = blockIdx.x;
  if (c >= k) return;
  double s = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += partial[(size_t)c * nblk + b];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) out[c] = s;
}

// ||A x - lam B x||^2 and ||x||^2 per column (GCGE_CheckConvergence,
// src/gcge_eigsol.c:689-707), RC columns per block: a thread walks its rows of
// A and B once for the block's columns, so the matrices are read k / RC times
// instead of k times (each column's sums keep the order they had column by
// column).
constexpr int RC = 4;
__global__ void __launch_bounds__(kThreads) k_residual(int n, const int* __restrict__ arp,
                                                       const int* __restrict__ aci,
                                                       const double* __restrict__ av,
                                                       const int* __restrict__ brp,
                                                       const int* __restrict__ bci,
                                                       const double* __restrict__ bv,
                                                       ColList<double> X,
                                                       const double* __restrict__ lam,
                                                       double* __restrict__ partial,
                                                       const int* __restrict__ ahidx,
                                                       const double* __restrict__ ahb,
                                                       const int* __restrict__ bhidx,
                                                       const double* __restrict__ bhb, int k) {
  __shared__ double sh[32];
  const int c0 = blockIdx.y * RC;
  const int kc = min(RC, k - c0);
  const double* x[RC];
  double l[RC], rs[RC], xs[RC];
#pragma unroll
  for (int q = 0; q < RC; q++) {
    x[q] = X.p[c0 + (q < kc ? q : 0)];
    l[q] = lam[c0 + (q < kc ? q : 0)];
    rs[q] = 0.0;
    xs[q] = 0.0;
  }
  for (int r = blockIdx.x * kThreads + threadIdx.x; r < n; r += gridDim.x * kThreads) {
    double ax[RC], bx[RC];
#pragma unroll
    for (int q = 0; q < RC; q++) ax[q] = 0.0;
    const int ha = ahidx ? __ldg(ahidx + r) : -1;
    if (ha >= 0) {
#pragma unroll
      for (int q = 0; q < RC; q++)
        if (q < kc) ax[q] = ahb[(size_t)ha * k + c0 + q];
    } else {
      for (int j = __ldg(arp + r); j < __ldg(arp + r + 1); j++) {
        const double a = __ldg(av + j);
        const int cj = __ldg(aci + j);
#pragma unroll
        for (int q = 0; q < RC; q++)
          if (q < kc) ax[q] = fma(a, x[q][cj], ax[q]);
      }
    }
    const int hb_ = bhidx ? __ldg(bhidx + r) : -1;
    if (hb_ >= 0) {
#pragma unroll
      for (int q = 0; q < RC; q++)
        if (q < kc) bx[q] = bhb[(size_t)hb_ * k + c0 + q];
    } else if (brp) {
#pragma unroll
      for (int q = 0; q < RC; q++) bx[q] = 0.0;
      for (int j = __ldg(brp + r); j < __ldg(brp + r + 1); j++) {
        const double b = __ldg(bv + j);
        const int cj = __ldg(bci + j);
#pragma unroll
        for (int q = 0; q < RC; q++)
          if (q < kc) bx[q] = fma(b, x[q][cj], bx[q]);
      }
    } else {
#pragma unroll
      for (int q = 0; q < RC; q++) bx[q] = q < kc ? x[q][r] : 0.0;
    }
#pragma unroll
    for (int q = 0; q < RC; q++) {
      if (q < kc) {
        const double rr = ax[q] - l[q] * bx[q];
        rs[q] = fma(rr, rr, rs[q]);
        xs[q] = fma(x[q][r], x[q][r], xs[q]);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < RC; q++) {
    const double s1 = block_sum(rs[q], sh);
    const double s2 = block_sum(xs[q], sh);
    if (threadIdx.x == 0 && q < kc) {
      partial[(size_t)(2 * (c0 + q)) * gridDim.x + blockIdx.x] = s1;
      partial[(size_t)(2 * (c0 + q) + 1) * gridDim.x + blockIdx.x] = s2;
    }
  }
}

__global__ void k_split_pairs(const double* __restrict__ pr, int k, double* __restrict__ r2,
                              double* __restrict__ x2) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  r2[c] = pr[2 * c];
  x2[c] = pr[2 * c + 1];
}

}  // namespace

// ---------------------------------------------------------------- launchers
// Y[:, j] = A X[:, j]: 8 columns per pass (a 16-column pass halves the
// CTAs per row range and measured slower on GB300).
void spmm_f64(const GcgeDevCsr& A, const ColList<double>& X, const ColList<double>& Y, int k,
              cudaStream_t st) {
  if (k <= 0 || A.n <= 0) return;
  constexpr int KC = 8;
  dim3 g((A.n + kThreads - 1) / kThreads, (k + KC - 1) / KC);
  heavy_cols_f64(A, X, k, st);
  k_spmm<double, KC><<<g, kThreads, 0, st>>>(A.n, A.rp, A.ci, A.v, X, Y, k,
                                             A.nheavy ? A.hidx : nullptr, A.hb64);
}

void spmm_f32(const GcgeDevCsr& A, const ColList<float>& X, const ColList<float>& Y, int k,
              cudaStream_t st) {
  if (k <= 0 || A.n <= 0) return;
  constexpr int KC = 8;
  dim3 g((A.n + kThreads - 1) / kThreads, (k + KC - 1) / KC);
  k_spmm<float, KC><<<g, kThreads, 0, st>>>(A.n, A.rp, A.ci, A.v32, X, Y, k, nullptr, nullptr);
}

void apply_b_f64(const GcgeDevCsr* B, const ColList<double>& X, const ColList<double>& Y, int k,
                 int n, cudaStream_t st) {
  if (k <= 0) return;
  if (!B) {
    for (int c = 0; c < k; c++)
      cudaMemcpyAsync(Y.p[c], X.p[c], sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
    return;
  }
  if (B->diag) {
    dim3 g((n + kThreads - 1) / kThreads);
    k_diag_mul<double><<<g, kThreads, 0, st>>>(n, B->diag, X, Y, k);
    return;
  }
  spmm_f64(*B, X, Y, k, st);
}

void gram_f64(const ColList<double>& V, int k1, const ColList<double>& W, int k2, int n,
              double* G, int ldg, bool sym, double* partial, cudaStream_t st) {
  if (k1 <= 0 || k2 <= 0) return;
  if (k1 * k2 <= GF_MAX * kThreads) {
    const int nchunks = (n + GR - 1) / GR;
    const int nblk = nchunks < kRowBlocks ? (nchunks < 1 ? 1 : nchunks) : kRowBlocks;
    const size_t sm = sizeof(double) * GR * (k1 + k2);
    if (sm > 48 * 1024)
      cudaFuncSetAttribute(k_gram_flex, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_gram_flex<<<nblk, kThreads, sm, st>>>(V, k1, W, k2, n, sym ? 1 : 0, partial);
    const int tot = k1 * k2;
    k_gram_flex_reduce<<<(tot + 255) / 256, 256, 0, st>>>(k1, k2, nblk, sym ? 1 : 0, partial, G,
                                                          ldg);
    return;
  }
  const int ti = (k1 + GT - 1) / GT, tj = (k2 + GT - 1) / GT;
  const int nchunks = (n + GR - 1) / GR;
  const int nblk = nchunks < kRowBlocks ? (nchunks < 1 ? 1 : nchunks) : kRowBlocks;
  dim3 g(nblk, ti * tj);
  k_gram<<<g, kThreads, 0, st>>>(V, k1, W, k2, n, tj, sym ? 1 : 0, partial);
  const int tot = k1 * k2;
  k_gram_reduce<<<(tot + 255) / 256, 256, 0, st>>>(k1, k2, tj, nblk, sym ? 1 : 0, partial, G, ldg);
}

void gram_reduce_partials(int k1, int k2, int nblk, bool sym, const double* partial, double* G,
                          int ldg, cudaStream_t st) {
  const int tot = k1 * k2;
  k_gram_flex_reduce<<<(tot + 255) / 256, 256, 0, st>>>(k1, k2, nblk, sym ? 1 : 0, partial, G, ldg);
}

void lincomb_f64(const ColList<double>& X, int k1, const double* C, int ldc,
                 const ColList<double>& Y, int k2, double beta, int n, cudaStream_t st) {
  if (k2 <= 0 || n <= 0) return;
  if (k1 <= 0) {
    // empty sum: Y = beta*Y
    ColList<double> Z = Y;
    dim3 g((n + kThreads - 1) / kThreads, k2);
    k_axpby<<<g, kThreads, 0, st>>>(0.0, Z, beta, Y, k2, n);
    return;
  }
  auto launch = [&](auto kern, int lj) {
    dim3 g((n + LT - 1) / LT, (k2 + lj - 1) / lj);
    const size_t sm = sizeof(double) * k1 * lj;
    if (sm > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kern<<<g, LT, sm, st>>>(X, k1, C, ldc, Y, k2, beta, n);
  };
  if (k2 <= 8) launch(k_lincomb<8>, 8);
  else if (k2 <= 16) launch(k_lincomb<16>, 16);
  else launch(k_lincomb<32>, 32);
}

void axpby_f64(double a, const ColList<double>& X, double b, const ColList<double>& Y, int k, int n,
               cudaStream_t st) {
  if (k <= 0) return;
  dim3 g((n + kThreads - 1) / kThreads, k);
  k_axpby<<<g, kThreads, 0, st>>>(a, X, b, Y, k, n);
}

void scale_cols_f64(const ColList<double>& Y, const double* s, int k, int n, cudaStream_t st) {
  if (k <= 0) return;
  dim3 g((n + kThreads - 1) / kThreads, k);
  k_scale_cols<<<g, kThreads, 0, st>>>(Y, s, k, n);
}

void colnorm2_f64(const ColList<double>& X, int k, int n, double* out, double* partial,
                  cudaStream_t st) {
  if (k <= 0) return;
  const int nb = row_blocks(n);
  k_colnorm2<<<dim3(nb, k), kThreads, 0, st>>>(X, k, n, partial);
  k_reduce_rows<<<k, 256, 0, st>>>(partial, nb, k, out);
}

void residual_f64(const GcgeDevCsr& A, const GcgeDevCsr* B, const ColList<double>& X,
                  const double* lam, int k, double* rnorm2, double* xnorm2, double* partial,
                  cudaStream_t st) {
  if (k <= 0) return;
  const int n = A.n;
  const int nb = row_blocks(n);
  heavy_cols_f64(A, X, k, st);
  const bool bh = B && B->nheavy;
  if (bh) heavy_cols_f64(*B, X, k, st);
  k_residual<<<dim3(nb, (k + RC - 1) / RC), kThreads, 0, st>>>(n, A.rp, A.ci, A.v, B ? B->rp : nullptr,
                                                B ? B->ci : nullptr, B ? B->v : nullptr, X, lam,
                                                partial, A.nheavy ? A.hidx : nullptr, A.hb64,
                                                bh ? B->hidx : nullptr, bh ? B->hb64 : nullptr, k);
  // partial holds 2k rows of nb entries: reduce into a scratch pair array
  double* pr = partial + (size_t)2 * k * nb;
  k_reduce_rows<<<2 * k, 256, 0, st>>>(partial, nb, 2 * k, pr);
  k_split_pairs<<<(k + 127) / 128, 128, 0, st>>>(pr, k, rnorm2, xnorm2);
}

void convert_f64_to_f32(const ColList<double>& X, const ColList<float>& Y, int k, int n,
                        cudaStream_t st) {
  if (k <= 0) return;
  dim3 g((n + kThreads - 1) / kThreads, k);
  k_convert<double, float><<<g, kThreads, 0, st>>>(X, Y, k, n);
}

void convert_f32_to_f64(const ColList<float>& X, const ColList<double>& Y, int k, int n,
                        cudaStream_t st) {
  if (k <= 0) return;
  dim3 g((n + kThreads - 1) / kThreads, k);
  k_convert<float, double><<<g, kThreads, 0, st>>>(X, Y, k, n);
}


}  // namespace gcge
