// FP64-accurate tall-skinny linear combination Y = X C (+ beta Y) on the
// bf16 tensor cores (mma.sync.m16n8k16, FP32 accumulate), by error-free
// splitting (the Ozaki scheme).
//
// Why: on GB300 FP64 FMA runs at ~1 TFLOP/s while bf16 MMA runs at ~600
// TFLOP/s (measured), so the X/P/W updates of GCG (n x k1 times k1 x k2,
// k1 <= 200) are the solve's bottleneck in FP64.
//
// Scheme.  Each row r of X is scaled by 2^{e_r} (e_r: smallest power of two
// above the row's largest |x|) and each column j of C by 2^{t_j}; the scaled
// values in (-1, 1) are cut into S = 8 signed 7-bit integer slices
// (x / 2^e = sum_a s_a 2^{-7a}, 56 bits, truncation error < 2^{-56}).  Every
// slice is exactly a bf16.  The products P_ab = X_a C_b of slices are
// integers bounded by k * 127^2; for k <= 128 a level L = a + b (up to 8
// pairs) sums below 2^24, so one FP32 MMA accumulator per level is exact.
// Levels L = 2..10 are kept (43 of the 64 slice products); the first dropped
// level contributes below 6 * 127^2 * 2^{-77} < 2^{-60} of the scale.  The levels are combined exactly in a 64-bit fixed-point integer
// T = sum_L acc_L 2^{54-7L}, and Y = T 2^{e_r + t_j - 54}.  The error is
// about k * 2^{-55} relative to sum_i |x_ri| |c_ij|, the bound of an FP64
// dot product.  k1 > 128 is processed in blocks of 128 that add into T.
#include <cuda_bf16.h>
#include <stdint.h>

#include "gcge_cuda_common.cuh"

namespace gcge {
namespace {

constexpr int OZ_S = 8;           // slices per value
constexpr int OZ_KC = 32;         // k columns per shared-memory stage
constexpr int OZ_KB = 128;        // k columns per exact accumulation block
constexpr int OZ_LD = OZ_KC + 8;  // bf16 stride of a staged row (20 words: conflict-free)
constexpr int OZ_T = 256;         // 8 warps per CTA
constexpr int OZ_NL = 9;          // levels L = 2..10

// Scaled 56-bit magnitude of x for the group exponent e (|x| < 2^e).
__device__ __forceinline__ uint64_t oz_m56(double x, int e, bool* neg) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  *neg = (b >> 63) != 0;
  const int ex = (int)((b >> 52) & 0x7FF);
  if (ex == 0 || ex == 0x7FF) return 0;  // zero/subnormal (negligible) or non-finite (flagged)
  const uint64_t mant = (b & ((1ull << 52) - 1)) | (1ull << 52);
  const int sh = (ex - 1023) + 4 - e;
  if (sh >= 0) return mant << sh;  // sh <= 3 since |x| < 2^e
  if (sh <= -64) return 0;
  return mant >> (-sh);
}

// exponent e with |x| < 2^e (0 for zero/subnormal); non-finite -> 4096
__device__ __forceinline__ int oz_exp(double x) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7FF);
  if (ex == 0x7FF) return 4096;
  if (ex == 0) return -2000;
  return ex - 1023 + 1;
}

__device__ __forceinline__ __nv_bfloat16 oz_slice(uint64_t m, int a, bool neg) {
  const int v = (int)((m >> (56 - 7 * a)) & 127u);
  return __float2bfloat16_rn(neg ? -(float)v : (float)v);
}

// exponent of x scaled by 2^d (sentinels kept)
__device__ __forceinline__ int oz_exp_shift(double x, int d) {
  const int e = oz_exp(x);
  return (e >= 4096 || e <= -2000) ? e : e + d;
}

// Column balancing of X: xe[i] = max exponent of the finite entries of
// column i (-2000 for a zero column; consumers read that as 0).  Grid:
// (row blocks, k1); xe must be preset to -2000.
__global__ void k_oz_colexp(ColList<double> X, int k1, int n, int* __restrict__ xe) {
  __shared__ int emax;
  const int i = blockIdx.y;
  if (threadIdx.x == 0) emax = -2000;
  __syncthreads();
  int e = -2000;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const int ex = oz_exp(X.p[i][r]);
    if (ex < 4096) e = max(e, ex);  // non-finite rows are flagged by the row exponent
  }
  atomicMax(&emax, e);
  __syncthreads();
  if (threadIdx.x == 0) atomicMax(xe + i, emax);
}

__global__ void k_fill_int(int* __restrict__ a, int v, int k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) a[i] = v;
}

__device__ __forceinline__ int oz_bal(const int* xe, int i) {
  if (!xe) return 0;
  const int d = xe[i];
  return d <= -2000 ? 0 : d;
}

// C (k1 x k2, ldc) -> slices Cg[s][j][i] (k2p x k1p, zero padded), texp[j].
// With balancing, row i of C is taken as C[i][j] * 2^{xe[i]} (exactly).
__global__ void k_oz_split_c(const double* __restrict__ C, int ldc, int k1, int k2, int k1p,
                             int k2p, const int* __restrict__ xe, int negate,
                             __nv_bfloat16* __restrict__ Cg, int* __restrict__ texp) {
  __shared__ int emax;
  const int j = blockIdx.x;
  if (threadIdx.x == 0) emax = -2000;
  __syncthreads();
  int e = -2000;
  if (j < k2)
    for (int i = threadIdx.x; i < k1; i += blockDim.x)
      e = max(e, oz_exp_shift(C[i + (size_t)j * ldc], oz_bal(xe, i)));
  atomicMax(&emax, e);
  __syncthreads();
  const int t = emax;
  if (threadIdx.x == 0) texp[j] = t;
  for (int i = threadIdx.x; i < k1p; i += blockDim.x) {
    const double c = (j < k2 && i < k1) ? C[i + (size_t)j * ldc] : 0.0;
    bool neg = false;
    const int d = (i < k1) ? oz_bal(xe, i) : 0;
    const uint64_t m = (t >= 4096) ? 0 : oz_m56(c, t - d, &neg);
    if (negate) neg = !neg;
#pragma unroll
    for (int a = 1; a <= OZ_S; a++)
      Cg[((size_t)(a - 1) * k2p + j) * k1p + i] = oz_slice(m, a, neg);
  }
}

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

template <int TM, int TN>
struct OzSmem {
  __nv_bfloat16 xs[OZ_S][TM][OZ_LD];  // X slices, [slice][row][k]
  __nv_bfloat16 cs[OZ_S][TN][OZ_LD];  // C slices, [slice][col][k]
  int rexp[TM];
};

// CTA: WM x WN warps, warp tile 16 rows x (8*NT) columns;
// CTA tile TM = 16*WM rows x TN = 8*NT*WN columns.
template <int WM, int WN, int NT>
__global__ void __launch_bounds__(OZ_T, 1)
    k_lincomb_oz(ColList<double> X, int k1, int k1p, const __nv_bfloat16* __restrict__ Cg,
                 const int* __restrict__ texp, int k2, int k2p, ColList<double> Y, double beta,
                 int n, const int* __restrict__ xe) {
  constexpr int TM = 16 * WM, TN = 8 * NT * WN;
  static_assert(WM * WN * 32 == OZ_T, "8 warps");
  extern __shared__ __align__(16) unsigned char smraw[];
  OzSmem<TM, TN>& sm = *reinterpret_cast<OzSmem<TM, TN>*>(smraw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp % WM, wn = warp / WM;
  const int g = lane >> 2, tq = lane & 3;
  const int r0 = blockIdx.x * TM;
  const int j0 = blockIdx.y * TN;

  // row exponents (OZ_T / TM threads per row), loads issued in batches of 8
  {
    constexpr int PARTS = OZ_T / TM;
    const int rr = tid % TM, part = tid / TM;
    int e = -2000;
    const int r = r0 + rr;
    if (r < n) {
      for (int i0 = part; i0 < k1; i0 += 8 * PARTS) {
        double v[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const int i = i0 + q * PARTS;
          v[q] = (i < k1) ? __ldg(X.p[i] + r) : 0.0;
        }
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const int i = i0 + q * PARTS;
          if (i < k1) e = max(e, oz_exp_shift(v[q], -oz_bal(xe, i)));
        }
      }
    }
    if (part == 0) sm.rexp[rr] = -2000;
    __syncthreads();
    atomicMax(&sm.rexp[rr], e);
    __syncthreads();
  }

  int64_t T[NT][4];  // [n-tile][fragment element] fixed-point accumulators
#pragma unroll
  for (int a = 0; a < NT; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) T[a][b] = 0;

  for (int kb = 0; kb < k1p; kb += OZ_KB) {
    float acc[OZ_NL][NT][4];
#pragma unroll
    for (int l = 0; l < OZ_NL; l++)
#pragma unroll
      for (int a = 0; a < NT; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[l][a][b] = 0.f;
    const int kend = min(kb + OZ_KB, k1p);
    for (int kc = kb; kc < kend; kc += OZ_KC) {
      __syncthreads();
      // split the X chunk rows [r0, r0+TM) x cols [kc, kc+32) into slices;
      // all of a thread's loads are issued before any is used
      {
        constexpr int PER = TM * OZ_KC / OZ_T;
        double xv[PER];
#pragma unroll
        for (int q = 0; q < PER; q++) {
          const int e = tid + q * OZ_T;
          const int rr = e % TM, cc = e / TM;
          const int r = r0 + rr, i = kc + cc;
          xv[q] = (r < n && i < k1) ? __ldg(X.p[i] + r) : 0.0;
        }
#pragma unroll
        for (int q = 0; q < PER; q++) {
          const int e = tid + q * OZ_T;
          const int rr = e % TM, cc = e / TM;
          const int i = kc + cc;
          const int ex = sm.rexp[rr];
          bool neg = false;
          const int d = (i < k1) ? oz_bal(xe, i) : 0;  // column i is taken as X * 2^{-d}
          const uint64_t m = (ex >= 4096) ? 0 : oz_m56(xv[q], ex + d, &neg);
#pragma unroll
          for (int a = 1; a <= OZ_S; a++) sm.xs[a - 1][rr][cc] = oz_slice(m, a, neg);
        }
      }
      // stage the C slices [slice][j0..j0+TN)[kc..kc+32) (16-byte copies)
      for (int e = tid; e < OZ_S * TN * (OZ_KC / 8); e += OZ_T) {
        const int q = e % (OZ_KC / 8);
        const int jj = (e / (OZ_KC / 8)) % TN;
        const int s = e / ((OZ_KC / 8) * TN);
        const uint4 v = *reinterpret_cast<const uint4*>(Cg + ((size_t)s * k2p + j0 + jj) * k1p +
                                                        kc + q * 8);
        *reinterpret_cast<uint4*>(&sm.cs[s][jj][q * 8]) = v;
      }
      __syncthreads();
#pragma unroll
      for (int ks = 0; ks < OZ_KC; ks += 16) {
        uint32_t af[OZ_S][4];
#pragma unroll
        for (int a = 0; a < OZ_S; a++) {
          const __nv_bfloat16* base = &sm.xs[a][wm * 16][ks];
          af[a][0] = *reinterpret_cast<const uint32_t*>(base + g * OZ_LD + tq * 2);
          af[a][1] = *reinterpret_cast<const uint32_t*>(base + (g + 8) * OZ_LD + tq * 2);
          af[a][2] = *reinterpret_cast<const uint32_t*>(base + g * OZ_LD + tq * 2 + 8);
          af[a][3] = *reinterpret_cast<const uint32_t*>(base + (g + 8) * OZ_LD + tq * 2 + 8);
        }
#pragma unroll
        for (int b = 0; b < OZ_S; b++) {
#pragma unroll
          for (int nt = 0; nt < NT; nt++) {
            const __nv_bfloat16* bb = &sm.cs[b][wn * (8 * NT) + nt * 8 + g][ks];
            const uint32_t b0 = *reinterpret_cast<const uint32_t*>(bb + tq * 2);
            const uint32_t b1 = *reinterpret_cast<const uint32_t*>(bb + tq * 2 + 8);
#pragma unroll
            for (int a = 0; a < OZ_S; a++)
              if (a + b <= OZ_NL - 1)  // slices a+1, b+1: level (a+1)+(b+1) <= 10
                mma_bf16(acc[a + b][nt], af[a], b0, b1);
          }
        }
      }
    }
    // fold the exact level sums into the fixed-point accumulators
#pragma unroll
    for (int l = 0; l < OZ_NL; l++) {
      const int L = l + 2;
      const int sh = 54 - 7 * L;
#pragma unroll
      for (int nt = 0; nt < NT; nt++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const int64_t v = (int64_t)__float2int_rn(acc[l][nt][q]);
          T[nt][q] += (sh >= 0) ? v * ((int64_t)1 << sh) : (v >> (-sh));
        }
    }
  }
  __syncthreads();
  // stage the results as doubles [col][row] for coalesced column writes
  double* ys = reinterpret_cast<double*>(smraw);  // TN x TM doubles
#pragma unroll
  for (int nt = 0; nt < NT; nt++)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int rr = wm * 16 + g + ((q >= 2) ? 8 : 0);
      const int jj = wn * (8 * NT) + nt * 8 + tq * 2 + (q & 1);
      const int j = j0 + jj;
      const int re = sm.rexp[rr];
      double y;
      if (j >= k2) {
        y = 0.0;
      } else {
        const int te = texp[j];
        if (re >= 4096 || te >= 4096) y = __longlong_as_double(0x7ff8000000000000ll);  // NaN in
        else if (re <= -2000 || te <= -2000) y = 0.0;
        else y = scalbn((double)T[nt][q], re + te - 54);
      }
      ys[jj * TM + rr] = y;
    }
  __syncthreads();
  for (int e = tid; e < TN * TM; e += OZ_T) {
    const int rr = e % TM, jj = e / TM;
    const int r = r0 + rr, j = j0 + jj;
    if (r < n && j < k2) {
      double* yp = Y.p[j] + r;
      const double v = ys[jj * TM + rr];
      *yp = (beta == 0.0) ? v : fma(beta, *yp, v);
    }
  }
}

template <int WM, int WN, int NT>
void launch_oz(const ColList<double>& X, int k1, int k1p, const __nv_bfloat16* Cg,
               const int* texp, const ColList<double>& Y, int k2, int k2p, double beta, int n,
               const int* xe, cudaStream_t st) {
  constexpr int TM = 16 * WM, TN = 8 * NT * WN;
  const size_t sm = sizeof(OzSmem<TM, TN>) > (size_t)TN * TM * 8 ? sizeof(OzSmem<TM, TN>)
                                                                  : (size_t)TN * TM * 8;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_lincomb_oz<WM, WN, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
    attr = true;
  }
  dim3 grid((n + TM - 1) / TM, (k2 + TN - 1) / TN);
  k_lincomb_oz<WM, WN, NT><<<grid, OZ_T, sm, st>>>(X, k1, k1p, Cg, texp, k2, k2p, Y, beta, n, xe);
}

// ---------------------------------------------------------------- Gram
// G = V^T W (k1 x k2) over n rows with FP64 accuracy.  Rows are processed in
// chunks of OG_R = 32; within a chunk every column of V and of W gets its own
// power-of-two scale, the 8 x 8 slice products of a level are summed exactly
// in FP32 by the MMAs (32 * 8 * 127^2 < 2^24), the levels are combined in a
// 64-bit fixed-point integer and the chunk's exact value is added to an FP64
// per-CTA partial sum.  A CTA owns a group of GM columns of V x GN columns of
// W; warp w owns m-tile w of its group.  A warp reads one column's 32 rows of
// a chunk with one coalesced load (lane = row), finds the column's scale by
// a warp max and writes the 8 slices, so each value is read from HBM once.
constexpr int OG_R = 32;
constexpr int OG_LD = OG_R + 8;  // 20 words per staged column: conflict-free fragments

template <int GM, int GN>
struct OgSmem {
  __nv_bfloat16 vs[OZ_S][GM][OG_LD];  // [slice][col of V][row]
  __nv_bfloat16 ws[OZ_S][GN][OG_LD];  // [slice][col of W][row]
  int cexp[GM + GN];
  double gsum[GM][GN];  // FP64 partial sums of this CTA
};

template <int GM, int GN>
__global__ void __launch_bounds__(OZ_T, (GM <= 96 ? 2 : 1))
    k_gram_oz(ColList<double> V, int k1, ColList<double> W, int k2, int n, int groups_n,
              const double* __restrict__ wdiag, double* __restrict__ partial) {
  constexpr int MT = GM / 16, NTN = GN / 8;
  extern __shared__ __align__(16) unsigned char smraw[];
  OgSmem<GM, GN>& sm = *reinterpret_cast<OgSmem<GM, GN>*>(smraw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, tq = lane & 3;
  const int gi = blockIdx.y / groups_n, gj = blockIdx.y % groups_n;
  const int i0 = gi * GM, j0 = gj * GN;
  const int mi = min(GM, k1 - i0), nj = min(GN, k2 - j0);
  for (int e = tid; e < GM * GN; e += OZ_T) (&sm.gsum[0][0])[e] = 0.0;
  const int nchunks = (n + OG_R - 1) / OG_R;
  const int mt = warp;
  const bool active = mt < MT && mt * 16 < mi;
  const int ntiles = (nj + 7) / 8;
  for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const int r = ch * OG_R + lane;
    __syncthreads();
    // one warp per column (lane = row): all of the warp's loads are issued
    // first, then each column is scaled by its chunk maximum and sliced
    constexpr int CPW = (GM + GN + 7) / 8;  // columns per warp
    double cv[CPW];
#pragma unroll
    for (int q = 0; q < CPW; q++) {
      const int c = warp + 8 * q;
      const bool isv = c < GM;
      const int cc = isv ? c : c - GM;
      const bool valid = c < GM + GN && (isv ? (cc < mi) : (cc < nj));
      double v = 0.0;
      if (valid && r < n) {
        if (isv) v = __ldg(V.p[i0 + cc] + r);
        else v = wdiag ? __ldg(wdiag + r) * __ldg(W.p[j0 + cc] + r) : __ldg(W.p[j0 + cc] + r);
      }
      cv[q] = v;
    }
#pragma unroll
    for (int q = 0; q < CPW; q++) {
      const int c = warp + 8 * q;
      if (c >= GM + GN) break;
      const bool isv = c < GM;
      const int cc = isv ? c : c - GM;
      const double v = cv[q];
      int e = oz_exp(v);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
      if (lane == 0) sm.cexp[c] = e;
      bool neg = false;
      const uint64_t m = (e >= 4096) ? 0 : oz_m56(v, e, &neg);
#pragma unroll
      for (int a = 1; a <= OZ_S; a++) {
        const __nv_bfloat16 sv = oz_slice(m, a, neg);
        if (isv) sm.vs[a - 1][cc][lane] = sv;
        else sm.ws[a - 1][cc][lane] = sv;
      }
    }
    __syncthreads();
    if (active) {
      float acc[OZ_NL][NTN][4];
#pragma unroll
      for (int l = 0; l < OZ_NL; l++)
#pragma unroll
        for (int a = 0; a < NTN; a++)
#pragma unroll
          for (int b = 0; b < 4; b++) acc[l][a][b] = 0.f;
#pragma unroll
      for (int ks = 0; ks < OG_R; ks += 16) {
        uint32_t af[OZ_S][4];
#pragma unroll
        for (int a = 0; a < OZ_S; a++) {
          // A = V^T: row m = column of V, k = row of the chunk
          const __nv_bfloat16* base = &sm.vs[a][mt * 16][ks];
          af[a][0] = *reinterpret_cast<const uint32_t*>(base + g * OG_LD + tq * 2);
          af[a][1] = *reinterpret_cast<const uint32_t*>(base + (g + 8) * OG_LD + tq * 2);
          af[a][2] = *reinterpret_cast<const uint32_t*>(base + g * OG_LD + tq * 2 + 8);
          af[a][3] = *reinterpret_cast<const uint32_t*>(base + (g + 8) * OG_LD + tq * 2 + 8);
        }
#pragma unroll
        for (int b = 0; b < OZ_S; b++) {
#pragma unroll
          for (int nt = 0; nt < NTN; nt++) {
            if (nt < ntiles) {
              const __nv_bfloat16* bb = &sm.ws[b][nt * 8 + g][ks];
              const uint32_t b0 = *reinterpret_cast<const uint32_t*>(bb + tq * 2);
              const uint32_t b1 = *reinterpret_cast<const uint32_t*>(bb + tq * 2 + 8);
#pragma unroll
              for (int a = 0; a < OZ_S; a++)
                if (a + b <= OZ_NL - 1) mma_bf16(acc[a + b][nt], af[a], b0, b1);
            }
          }
        }
      }
      // exact chunk value -> FP64 partial sums
#pragma unroll
      for (int nt = 0; nt < NTN; nt++) {
        if (nt >= ntiles) continue;
#pragma unroll
        for (int q = 0; q < 4; q++) {
          int64_t T = 0;
#pragma unroll
          for (int l = 0; l < OZ_NL; l++) {
            const int sh = 54 - 7 * (l + 2);
            const int64_t v = (int64_t)__float2int_rn(acc[l][nt][q]);
            T += (sh >= 0) ? v * ((int64_t)1 << sh) : (v >> (-sh));
          }
          const int ii = mt * 16 + g + ((q >= 2) ? 8 : 0);
          const int jj = nt * 8 + tq * 2 + (q & 1);
          if (ii < mi && jj < nj) {
            const int ea = sm.cexp[ii], eb = sm.cexp[GM + jj];
            double v;
            if (ea >= 4096 || eb >= 4096) v = __longlong_as_double(0x7ff8000000000000ll);
            else if (ea <= -2000 || eb <= -2000) v = 0.0;
            else v = scalbn((double)T, ea + eb - 54);
            sm.gsum[ii][jj] += v;
          }
        }
      }
    }
  }
  __syncthreads();
  // partial layout [block][o], o = i + j*k1 (the flex-Gram reduction layout)
  double* out = partial + (size_t)blockIdx.x * k1 * k2;
  for (int e = tid; e < mi * nj; e += OZ_T) {
    const int ii = e % mi, jj = e / mi;
    out[(i0 + ii) + (size_t)(j0 + jj) * k1] = sm.gsum[ii][jj];
  }
}

template <int GM, int GN>
int launch_gram_oz(const ColList<double>& V, int k1, const ColList<double>& W, int k2, int n,
                   const double* wdiag, double* partial, cudaStream_t st) {
  const int groups_m = (k1 + GM - 1) / GM, groups_n = (k2 + GN - 1) / GN;
  const int nchunks = (n + OG_R - 1) / OG_R;
  const int per_sm = GM <= 96 ? 2 : 1;
  const int nblk = nchunks < 152 * per_sm ? nchunks : 152 * per_sm;
  const size_t sm = sizeof(OgSmem<GM, GN>);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_gram_oz<GM, GN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    attr = true;
  }
  k_gram_oz<GM, GN><<<dim3(nblk, groups_m * groups_n), OZ_T, sm, st>>>(V, k1, W, k2, n, groups_n,
                                                                       wdiag, partial);
  return nblk;
}

}  // namespace

size_t lincomb_oz_scratch_bytes(int k1, int k2) {
  const int k1p = (k1 + OZ_KC - 1) / OZ_KC * OZ_KC;
  const int k2p = (k2 + 63) / 64 * 64;
  return sizeof(__nv_bfloat16) * (size_t)OZ_S * k1p * k2p + sizeof(int) * (size_t)(k2p + k1p) +
         256;
}

// Y_j = beta Y_j + sum_i X_i C[i + j*ldc], FP64 accuracy on bf16 tensor cores.
// scratch: lincomb_oz_scratch_bytes(k1, k2) bytes, 16-byte aligned.  balance:
// scale the columns of X by powers of two (and the rows of C inversely)
// first, for blocks whose columns differ widely in magnitude (the product is
// unchanged: the scaling is exact).
void lincomb_oz(const ColList<double>& X, int k1, const double* C, int ldc,
                const ColList<double>& Y, int k2, double beta, int n, void* scratch,
                cudaStream_t st, bool balance, bool negate) {
  if (k2 <= 0 || n <= 0) return;
  const int k1p = (k1 + OZ_KC - 1) / OZ_KC * OZ_KC;
  const int k2p = (k2 + 63) / 64 * 64;  // C slices padded to the widest CTA tile
  __nv_bfloat16* Cg = reinterpret_cast<__nv_bfloat16*>(scratch);
  int* texp = reinterpret_cast<int*>(Cg + (size_t)OZ_S * k1p * k2p);
  int* xe = balance ? texp + k2p : nullptr;
  if (balance) {
    k_fill_int<<<(k1 + 127) / 128, 128, 0, st>>>(xe, -2000, k1);
    const int nb = (n + 255) / 256 < 64 ? (n + 255) / 256 : 64;
    k_oz_colexp<<<dim3(nb, k1), 256, 0, st>>>(X, k1, n, xe);
  }
  k_oz_split_c<<<k2p, 128, 0, st>>>(C, ldc, k1, k2, k1p, k2p, xe, negate ? 1 : 0, Cg, texp);
  if (k2 <= 16) launch_oz<8, 1, 2>(X, k1, k1p, Cg, texp, Y, k2, k2p, beta, n, xe, st);
  else if (k2 <= 32) launch_oz<8, 1, 4>(X, k1, k1p, Cg, texp, Y, k2, k2p, beta, n, xe, st);
  else launch_oz<4, 2, 4>(X, k1, k1p, Cg, texp, Y, k2, k2p, beta, n, xe, st);
}

size_t gram_oz_partial_doubles(int k1, int k2) {
  return (size_t)304 * k1 * k2;
}

// G = V^T W (k1 x k2) into partial (gram_oz_partial_doubles) then G (ldg);
// sym: only the upper triangle is kept and mirrored.
void gram_oz(const ColList<double>& V, int k1, const ColList<double>& W, int k2, int n, double* G,
             int ldg, bool sym, double* partial, cudaStream_t st, const double* wdiag) {
  if (k1 <= 0 || k2 <= 0 || n <= 0) return;
  int nblk;
  if (k1 <= 96 && k2 <= 16) nblk = launch_gram_oz<96, 16>(V, k1, W, k2, n, wdiag, partial, st);
  else nblk = launch_gram_oz<128, 32>(V, k1, W, k2, n, wdiag, partial, st);
  gram_reduce_partials(k1, k2, nblk, sym, partial, G, ldg, st);
}

}  // namespace gcge
