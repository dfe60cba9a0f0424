// Uneven rows.  The row kernels run a thread per row, which is the fastest
// schedule for the short, similar rows of a stencil; on a power-law graph a few
// rows hold tens of thousands of entries and one thread walking such a row
// stalls its whole launch.  Rows of more than kHeavyRow entries are therefore
// cut at matrix creation into chunks of up to kHeavyChunk entries; before a
// row kernel runs, one warp per chunk multiplies its chunk (lanes stride the
// entries, then a fixed xor-shuffle tree); the chunks of each heavy row are
// then added in chunk order (by a second pass for FP64 columns, by the row
// kernel itself for the FP32 row-interleaved blocks), and the row kernel takes
// those rows' products instead of walking them.  Every sum has a fixed order, so the
// products are deterministic.
#include <vector>

#include "gcge_cuda_common.cuh"

namespace gcge {

namespace {

constexpr int kWarpsPerBlock = 8;

// Column form (T = double: FP64 columns and values; T = float: the FP32
// columns of the mixed block CG with the FP32 copy of the values).
template <typename T>
__global__ void k_heavy_cols(int nchunk, const int* __restrict__ chb, const int* __restrict__ che,
                             const int* __restrict__ ci, const T* __restrict__ v,
                             ColList<T> X, int cbase, int ncols, T* __restrict__ cb) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nchunk) return;
  const int g0 = blockIdx.y * 8;
  const int kc = min(8, ncols - g0);
  if (kc <= 0) return;
  T acc[8];
#pragma unroll
  for (int c = 0; c < 8; c++) acc[c] = T(0);
  const int e = __ldg(che + warp);
  for (int j = __ldg(chb + warp) + lane; j < e; j += 32) {
    const int col = __ldg(ci + j);
    const T a = __ldg(v + j);
#pragma unroll
    for (int c = 0; c < 8; c++)
      if (c < kc) acc[c] = fma(a, __ldg(X.p[cbase + g0 + c] + col), acc[c]);
  }
#pragma unroll
  for (int c = 0; c < 8; c++)
    for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
  if (lane == 0)
    for (int c = 0; c < kc; c++) cb[(size_t)warp * kHeavyGroup + g0 + c] = acc[c];
}

// the same over the active columns of a block CG: column g of this pass is
// P.p[unl[cbase + g]] for cbase + g < *nu (the active count, on the device)
template <typename T>
__global__ void k_heavy_cols_active(int nchunk, const int* __restrict__ chb,
                                    const int* __restrict__ che, const int* __restrict__ ci,
                                    const T* __restrict__ v, ColList<T> P,
                                    const int* __restrict__ unl, const int* __restrict__ nu,
                                    int cbase, T* __restrict__ cb) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nchunk) return;
  const int g0 = blockIdx.y * 8;
  const int kc = min(8, *nu - cbase - g0);
  if (kc <= 0) return;
  const T* col[8];
#pragma unroll
  for (int c = 0; c < 8; c++) col[c] = P.p[unl[cbase + g0 + (c < kc ? c : 0)]];
  T acc[8];
#pragma unroll
  for (int c = 0; c < 8; c++) acc[c] = T(0);
  const int e = __ldg(che + warp);
  for (int j = __ldg(chb + warp) + lane; j < e; j += 32) {
    const int cj = __ldg(ci + j);
    const T a = __ldg(v + j);
#pragma unroll
    for (int c = 0; c < 8; c++)
      if (c < kc) acc[c] = fma(a, col[c][cj], acc[c]);
  }
#pragma unroll
  for (int c = 0; c < 8; c++)
    for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
  if (lane == 0)
    for (int c = 0; c < kc; c++) cb[(size_t)warp * kHeavyGroup + g0 + c] = acc[c];
}

template <typename T>
__global__ void k_heavy_sum_active(int nheavy, const int* __restrict__ hch,
                                   const T* __restrict__ cb, int ncols, int cbase,
                                   const int* __restrict__ nu, int ldh, T* __restrict__ hb) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nheavy * ncols) return;
  const int h = t / ncols, c = t % ncols;
  if (cbase + c >= *nu) return;
  T s = T(0);
  for (int q = __ldg(hch + h); q < __ldg(hch + h + 1); q++) s += cb[(size_t)q * kHeavyGroup + c];
  hb[(size_t)h * ldh + cbase + c] = s;
}

template <typename T>
__global__ void k_heavy_sum_cols(int nheavy, const int* __restrict__ hch,
                                 const T* __restrict__ cb, int ncols, int cbase, int ldh,
                                 T* __restrict__ hb) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nheavy * ncols) return;
  const int h = t / ncols, c = t % ncols;
  T s = T(0);
  for (int q = __ldg(hch + h); q < __ldg(hch + h + 1); q++) s += cb[(size_t)q * kHeavyGroup + c];
  hb[(size_t)h * ldh + cbase + c] = s;
}

template <int KW>
__global__ void k_heavy_rows(int nchunk, const int* __restrict__ chb, const int* __restrict__ che,
                             const int* __restrict__ ci, const float* __restrict__ v,
                             const float* __restrict__ X, float* __restrict__ cb,
                             const int* __restrict__ nu) {
  if (nu && *nu == 0) return;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nchunk) return;
  float acc[KW];
#pragma unroll
  for (int c = 0; c < KW; c++) acc[c] = 0.f;
  const int e = __ldg(che + warp);
  for (int j = __ldg(chb + warp) + lane; j < e; j += 32) {
    const int col = __ldg(ci + j);
    const float a = __ldg(v + j);
    const float4* p = reinterpret_cast<const float4*>(X + (size_t)col * KW);
#pragma unroll
    for (int q = 0; q < KW / 4; q++) {
      const float4 t = __ldg(p + q);
      acc[4 * q] = fmaf(a, t.x, acc[4 * q]);
      acc[4 * q + 1] = fmaf(a, t.y, acc[4 * q + 1]);
      acc[4 * q + 2] = fmaf(a, t.z, acc[4 * q + 2]);
      acc[4 * q + 3] = fmaf(a, t.w, acc[4 * q + 3]);
    }
  }
#pragma unroll
  for (int c = 0; c < KW; c++)
    for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < KW; c++) cb[(size_t)warp * KW + c] = acc[c];
  }
}

template <int KW>
void heavy_rows_kw(const GcgeDevCsr& M, const float* val, const float* X, const int* nu,
                   cudaStream_t st) {
  const int threads = 32 * kWarpsPerBlock;
  k_heavy_rows<KW><<<(M.nchunk + kWarpsPerBlock - 1) / kWarpsPerBlock, threads, 0, st>>>(
      M.nchunk, M.chb, M.che, M.ci, val, X, M.cb32, nu);
}

}  // namespace

int heavy_setup(GcgeDevCsr& M, const int* h_rp) {
  const int n = M.n;
  std::vector<int> hidx(n, -1), hch(1, 0), chb, che;
  int nheavy = 0;
  for (int r = 0; r < n; r++) {
    const int b = h_rp[r], e = h_rp[r + 1];
    if (e - b <= kHeavyRow) continue;
    hidx[r] = nheavy++;
    for (int s = b; s < e; s += kHeavyChunk) {
      chb.push_back(s);
      che.push_back(s + kHeavyChunk < e ? s + kHeavyChunk : e);
    }
    hch.push_back((int)chb.size());
  }
  if (nheavy == 0) return 0;
  const int nchunk = (int)chb.size();
  cudaError_t err = cudaSuccess;
  auto alloc = [&](void** p, size_t bytes) {
    if (err == cudaSuccess) err = cudaMalloc(p, bytes);
  };
  alloc((void**)&M.hidx, sizeof(int) * n);
  alloc((void**)&M.hch, sizeof(int) * (nheavy + 1));
  alloc((void**)&M.chb, sizeof(int) * nchunk);
  alloc((void**)&M.che, sizeof(int) * nchunk);
  alloc((void**)&M.hb64, sizeof(double) * nheavy * (size_t)GCGE_MAXCOLS);
  alloc((void**)&M.cb64, sizeof(double) * nchunk * (size_t)kHeavyGroup);
  alloc((void**)&M.cb32, sizeof(float) * nchunk * (size_t)32);
  if (err == cudaSuccess)
    err = cudaMemcpy(M.hidx, hidx.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
  if (err == cudaSuccess)
    err = cudaMemcpy(M.hch, hch.data(), sizeof(int) * (nheavy + 1), cudaMemcpyHostToDevice);
  if (err == cudaSuccess)
    err = cudaMemcpy(M.chb, chb.data(), sizeof(int) * nchunk, cudaMemcpyHostToDevice);
  if (err == cudaSuccess)
    err = cudaMemcpy(M.che, che.data(), sizeof(int) * nchunk, cudaMemcpyHostToDevice);
  if (err != cudaSuccess) {
    heavy_free(M);
    return (int)err;
  }
  M.nheavy = nheavy;
  M.nchunk = nchunk;
  return 0;
}

void heavy_free(GcgeDevCsr& M) {
  cudaFree(M.hidx);
  cudaFree(M.hch);
  cudaFree(M.chb);
  cudaFree(M.che);
  cudaFree(M.hb64);
  cudaFree(M.cb64);
  cudaFree(M.cb32);
  M.hidx = M.hch = M.chb = M.che = nullptr;
  M.hb64 = M.cb64 = nullptr;
  M.cb32 = nullptr;
  M.nheavy = M.nchunk = 0;
}

template <typename T>
void heavy_cols(const GcgeDevCsr& M, const T* val, const ColList<T>& X, int k, cudaStream_t st) {
  if (M.nheavy == 0 || k <= 0) return;
  const int threads = 32 * kWarpsPerBlock;
  const int nbx = (M.nchunk + kWarpsPerBlock - 1) / kWarpsPerBlock;
  T* cb = reinterpret_cast<T*>(M.cb64);  // T = float: the same buffers at float entries
  T* hb = reinterpret_cast<T*>(M.hb64);
  for (int cbase = 0; cbase < k; cbase += kHeavyGroup) {
    const int ncols = k - cbase < kHeavyGroup ? k - cbase : kHeavyGroup;
    k_heavy_cols<T><<<dim3(nbx, (ncols + 7) / 8), threads, 0, st>>>(M.nchunk, M.chb, M.che,
                                                                    M.ci, val, X, cbase, ncols,
                                                                    cb);
    k_heavy_sum_cols<T><<<(M.nheavy * ncols + 255) / 256, 256, 0, st>>>(M.nheavy, M.hch, cb,
                                                                        ncols, cbase, k, hb);
  }
}

template <typename T>
void heavy_cols_active(const GcgeDevCsr& M, const T* val, const ColList<T>& P, const int* unl,
                       const int* nu, int kmax, cudaStream_t st) {
  if (M.nheavy == 0 || kmax <= 0) return;
  const int threads = 32 * kWarpsPerBlock;
  const int nbx = (M.nchunk + kWarpsPerBlock - 1) / kWarpsPerBlock;
  T* cb = reinterpret_cast<T*>(M.cb64);
  T* hb = reinterpret_cast<T*>(M.hb64);
  for (int cbase = 0; cbase < kmax; cbase += kHeavyGroup) {
    const int ncols = kmax - cbase < kHeavyGroup ? kmax - cbase : kHeavyGroup;
    k_heavy_cols_active<T><<<dim3(nbx, (ncols + 7) / 8), threads, 0, st>>>(
        M.nchunk, M.chb, M.che, M.ci, val, P, unl, nu, cbase, cb);
    k_heavy_sum_active<T><<<(M.nheavy * ncols + 255) / 256, 256, 0, st>>>(
        M.nheavy, M.hch, cb, ncols, cbase, nu, kmax, hb);
  }
}

template void heavy_cols<double>(const GcgeDevCsr&, const double*, const ColList<double>&, int,
                                 cudaStream_t);
template void heavy_cols<float>(const GcgeDevCsr&, const float*, const ColList<float>&, int,
                                cudaStream_t);
template void heavy_cols_active<double>(const GcgeDevCsr&, const double*, const ColList<double>&,
                                        const int*, const int*, int, cudaStream_t);
template void heavy_cols_active<float>(const GcgeDevCsr&, const float*, const ColList<float>&,
                                       const int*, const int*, int, cudaStream_t);

void heavy_cols_f64(const GcgeDevCsr& M, const ColList<double>& X, int k, cudaStream_t st) {
  heavy_cols<double>(M, M.v, X, k, st);
}

void heavy_rows_f32(const GcgeDevCsr& M, const float* val, const float* X, int KW, const int* nu,
                    cudaStream_t st) {
  if (M.nheavy == 0) return;
  switch (KW) {
    case 4: heavy_rows_kw<4>(M, val, X, nu, st); break;
    case 8: heavy_rows_kw<8>(M, val, X, nu, st); break;
    case 12: heavy_rows_kw<12>(M, val, X, nu, st); break;
    case 16: heavy_rows_kw<16>(M, val, X, nu, st); break;
    case 20: heavy_rows_kw<20>(M, val, X, nu, st); break;
    case 24: heavy_rows_kw<24>(M, val, X, nu, st); break;
    case 28: heavy_rows_kw<28>(M, val, X, nu, st); break;
    case 32: heavy_rows_kw<32>(M, val, X, nu, st); break;
  }
}

}  // namespace gcge
