// FP64-accurate tall-skinny products on the GB300 tensor cores (tcgen05,
// bf16 operands in shared memory, FP32 accumulators in tensor memory) by
// error-free splitting into integer digits (the Ozaki scheme):
//   * k_lincomb_tc: Y = X C (+ beta Y), the X/P/W updates of GCG
//     (n x k1 times k1 x k2, k1 <= 256, k2 <= 256);
//   * k_gram_tc: G = V^T diag(d) W, the inner products of the orthogonalisation
//     and of the Rayleigh-Ritz projection.
//
// Why: on GB300 FP64 FMA runs at ~1 TFLOP/s while the bf16 tensor cores run
// at ~2 PFLOP/s (measured), so in FP64 these products, not the memory
// traffic, bound the GCG iteration.
//
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "gcge_cuda_common.cuh"
#include "gcge_cuda_tc.cuh"

namespace gcge {
namespace {

// exponent e with |x| < 2^e (0 for zero/subnormal); non-finite -> 4096
__device__ __forceinline__ int oz_exp(double x) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7FF);
  if (ex == 0x7FF) return 4096;
  if (ex == 0) return -2000;
  return ex - 1023 + 1;
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

// ---------------------------------------------------------------- tcgen05 linear combination
// Y = X C on the 5th-generation tensor cores.  Digits: every value, scaled by
// its group's power of two into (-1, 1), is cut into D8_S = 7 balanced
// base-256 digits (m = trunc(x 2^{55-E}) = sum_a d_a 256^{7-a}, the top digit
// in [-128, 128], the others in [-128, 127]); each digit is exactly a bf16.
// A product of two digits is an integer of magnitude <= 2^14; a level
// L = a + b holds at most 7 of them, so a level summed over K <= 128 stays
// below 7 * 2^21 < 2^24 and its FP32 tensor-memory accumulator is exact.
// Levels L = 2..9 (34 digit products) are kept; the first dropped level is
// below 5 * 2^14 * 2^{2-80} < 2^{-61} of the scale, the digit truncation
// 2^{-55}.  Levels combine in a 64-bit integer T = sum_L acc_L 2^{57-8L}
// (|T| < 2^62; levels 8 and 9 rounded to the integer unit), and
// y = T 2^{e_r + t_j - 55}.
//
// One CTA: 128 rows (MMA M, TMEM lane = row) x up to 64 output columns (MMA
// N).  Per k step of 16: all 256 threads slice their 8 values into shared
// memory (K-major core-matrix layout, no swizzle), one thread issues the 34
// MMAs (kind::f16, bf16 x bf16 -> FP32) into the 8 level accumulators in
// tensor memory and commits them to the stage's mbarrier; stages rotate
// through TC_STAGES buffers.  The epilogue reads the levels with
// tcgen05.ld, combines them in registers and writes Y column-coalesced.
constexpr int D8_S = 7;
constexpr int D8_NL = 8;
constexpr int TC_M = 128;
constexpr int TC_KS = 16;
constexpr int TC_NMAX = 64;
constexpr int TC_STAGES = 3;
constexpr int TC_T = 512;
constexpr int TC_ABYTES = D8_S * TC_M * TC_KS * 2;  // 28672
constexpr int TC_WAIT = 1 << 26;                    // mbarrier polls before giving up

__device__ int g_oz_tc_status = 0;  // 1: an mbarrier wait gave up (outputs set to NaN)

__device__ __forceinline__ uint32_t d8_pack(float lo, float hi) {
  return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}

// The 7 digits of x / 2^E (|x| < 2^E) as exact FP32 values, most significant
// first.  Zero, subnormal and non-finite x give zero digits.
__device__ __forceinline__ void d8_digits(double x, int E, float* f) {
  const long long b = __double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7FF);
  long long m = 0;
  if (ex != 0 && ex != 0x7FF) {
    const unsigned long long mant = ((unsigned long long)b & ((1ull << 52) - 1)) | (1ull << 52);
    const int sh = ex - 1020 - E;  // <= 2 because |x| < 2^E
    const unsigned long long mm =
        sh >= 0 ? (mant << sh) : (sh > -64 ? (mant >> (-sh)) : 0ull);
    m = b < 0 ? -(long long)mm : (long long)mm;
  }
  const long long u = m + 0x808080808080ll;  // bytes 0..5 of u are the low digits + 128
  const int hi = (int)(u >> 32);
  const unsigned lo = (unsigned)u;
  f[0] = __int_as_float(0x4B000000 + (hi >> 16) + 256) - 8388864.0f;
  f[1] = __int_as_float(__byte_perm((unsigned)hi, 0x4B000000u, 0x7651)) - 8388736.0f;
  f[2] = __int_as_float(__byte_perm((unsigned)hi, 0x4B000000u, 0x7650)) - 8388736.0f;
  f[3] = __int_as_float(__byte_perm(lo, 0x4B000000u, 0x7653)) - 8388736.0f;
  f[4] = __int_as_float(__byte_perm(lo, 0x4B000000u, 0x7652)) - 8388736.0f;
  f[5] = __int_as_float(__byte_perm(lo, 0x4B000000u, 0x7651)) - 8388736.0f;
  f[6] = __int_as_float(__byte_perm(lo, 0x4B000000u, 0x7650)) - 8388736.0f;
}

// exponent e with |x| < 2^e from the high 32 bits of x (sentinels as oz_exp)
__device__ __forceinline__ int oz_exp_hi(int hi) {
  const int ex = (hi >> 20) & 0x7FF;
  if (ex == 0x7FF) return 4096;
  if (ex == 0) return -2000;
  return ex - 1023 + 1;
}

// high 32 bits of p[i] (the sign, exponent and top of the mantissa)
__device__ __forceinline__ int ld_hi(const double* p) {
  return __ldg(reinterpret_cast<const int*>(p) + 1);
}

// 4 values -> 7 digit rows of 8 bytes at dst + a*dstride (half of a
// core-matrix row), value q scaled by 2^{-E[q]}
__device__ __forceinline__ void d8_slice4(const double* v, const int* E, uint8_t* dst,
                                          int dstride) {
  float f[4][D8_S];
#pragma unroll
  for (int q = 0; q < 4; q++) d8_digits(v[q], E[q], f[q]);
#pragma unroll
  for (int a = 0; a < D8_S; a++) {
    uint2 w;
    w.x = d8_pack(f[0][a], f[1][a]);
    w.y = d8_pack(f[2][a], f[3][a]);
    *reinterpret_cast<uint2*>(dst + a * dstride) = w;
  }
}

// T 2^s rounded to the nearest double (ties to even), by integer operations.
__device__ __forceinline__ double d8_to_double(long long T, int s) {
  if (T == 0) return 0.0;
  const unsigned long long sgn = T < 0 ? (1ull << 63) : 0ull;
  const unsigned long long mag = T < 0 ? (unsigned long long)(-T) : (unsigned long long)T;
  const int lz = __clzll((long long)mag);
  const unsigned long long nrm = mag << lz;  // top bit at 63
  unsigned long long mant = nrm >> 11;       // 53 bits
  const unsigned long long rem = nrm & 0x7FFull;
  int e2 = 63 - lz;  // value = nrm 2^{e2 - 63} 2^s
  if (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) {
    mant += 1ull;
    if (mant == (1ull << 53)) {
      mant >>= 1;
      e2 += 1;
    }
  }
  const int be = e2 + s + 1023;
  if (be >= 1 && be <= 2046)
    return __longlong_as_double((long long)(sgn | ((unsigned long long)be << 52) |
                                            (mant & ((1ull << 52) - 1))));
  return scalbn(T < 0 ? -(double)mag : (double)mag, s);  // out of the normal range
}

__host__ __device__ __forceinline__ int tc_round16(int v) { return (v + 15) / 16 * 16; }

// width (MMA N) of output-column tile nt
__host__ __device__ __forceinline__ int tc_tile_n(int k2, int nt) {
  const int rem = k2 - nt * TC_NMAX;
  return rem >= TC_NMAX ? TC_NMAX : tc_round16(rem);
}

// C (k1 x k2, ldc; k1 <= 128) -> B operand images Cg and column exponents
// texp.  Layout: tile nt (TC_NMAX columns) at byte nt*TC_NMAX*k1p*14, inside it
// stage ks (16 values of i) at ks*7*N*32: the K-major core-matrix image of a
// 7N x 16 matrix whose row (a, j) = a*N + j is digit a of column j (so one
// descriptor spans several digits of the tile).  Grid: one CTA per
// padded column.  Row i of C is taken as C[i][j] 2^{xe[i]} (balancing), and
// negated when negate is set.
__global__ void k_d8_split_c(const double* __restrict__ C, int ldc, int k1, int k2, int k1p,
                             const int* __restrict__ xe, int negate, uint8_t* __restrict__ Cg,
                             int* __restrict__ texp) {
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
  if (threadIdx.x == 0 && j < k2) texp[j] = t;
  const int nt = j / TC_NMAX, jj = j % TC_NMAX;
  const int N = tc_tile_n(k2, nt);
  uint8_t* tile = Cg + (size_t)nt * TC_NMAX * k1p * (D8_S * 2);
  for (int i = threadIdx.x; i < k1p; i += blockDim.x) {
    double c = (j < k2 && i < k1 && t < 4096) ? C[i + (size_t)j * ldc] : 0.0;
    if (negate) c = -c;
    const int d = (i < k1) ? oz_bal(xe, i) : 0;
    float f[D8_S];
    d8_digits(c, t - d, f);
    const int ks = i / TC_KS, kk = i % TC_KS;
    const size_t off = (size_t)ks * (D8_S * N * 32) + (size_t)(kk >> 3) * (D8_S * N * 16) +
                       (size_t)(jj >> 3) * 128 + (jj & 7) * 16 + (kk & 7) * 2;
#pragma unroll
    for (int a = 0; a < D8_S; a++) {
      const unsigned short h = (unsigned short)(__float_as_uint(f[a]) >> 16);
      *reinterpret_cast<unsigned short*>(tile + off + (size_t)a * (N * 16)) = h;
    }
  }
}

__device__ __forceinline__ void d8_fill_nan(ColList<double> Y, int j0, int N, int k2, int n,
                                            int r0) {
  for (int e = threadIdx.x; e < N * TC_M; e += TC_T) {
    const int rr = e % TC_M, jj = e / TC_M;
    if (r0 + rr < n && j0 + jj < k2)
      Y.p[j0 + jj][r0 + rr] = __longlong_as_double(0x7ff8000000000000ll);
  }
}

// Issues the 34 digit products of one K step of 16.  A digit a (1..7) is
// multiplied by B digits b = 1..min(7, 9-a) in MMAs whose N spans several
// digits (at most 256 columns each), with D offset so that product (a, b)
// accumulates on level a + b, i.e. TMEM columns (a+b-2)*Nw of the 8*Nw level
// block: 7 MMAs per step for Nw <= 32 instead of one per product.  first: the
// step opens the accumulation (level blocks 2..8 are first written by a = 1,
// level 9 by (a, b) = (2, 7), issued on its own then).  A digit a is the
// 128 x 16 tile at abase + (a-1)*astride (core matrices 2048 bytes apart
// along K); the B image is the 7Nw x 16 matrix described at k_d8_split_c.
template <bool F16 = false>
__device__ __forceinline__ void d8_issue(uint32_t tacc, uint32_t abase, uint32_t astride,
                                         uint32_t bbase, int Nw, bool first) {
  const int maxd = 256 / Nw;
#pragma unroll
  for (int a = 1; a <= D8_S; a++) {
    const uint64_t ad = gcge::tc::smem_desc(abase + (a - 1) * astride, TC_M * 16, 128);
    const int bmax = (9 - a) < D8_S ? (9 - a) : D8_S;
    int b0 = 1;
    while (b0 <= bmax) {
      int cnt = (bmax - b0 + 1) < maxd ? (bmax - b0 + 1) : maxd;
      if (first && a == 2 && b0 + cnt - 1 == D8_S && cnt > 1) cnt -= 1;
      const uint32_t accum = (first && (a == 1 || (a == 2 && b0 == D8_S))) ? 0u : 1u;
      const uint64_t bd = gcge::tc::smem_desc(bbase + (b0 - 1) * Nw * 16, D8_S * Nw * 16, 128);
      gcge::tc::mma_bf16(tacc + (uint32_t)((a + b0 - 2) * Nw), ad, bd,
                         F16 ? gcge::tc::idesc_f16(TC_M, cnt * Nw)
                             : gcge::tc::idesc_bf16(TC_M, cnt * Nw),
                         accum);
      b0 += cnt;
    }
  }
}

// Y[:, j] = beta Y[:, j] + sum_i X[:, i] C[i][j] for k1 <= 128.  Grid:
// (row tiles of 128, output-column tiles of 64), 512 threads.  Dynamic
// shared memory: tc_lincomb_smem(N of tile 0).
__global__ void __launch_bounds__(TC_T, 2)
    k_lincomb_tc(ColList<double> X, int k1, int k1p, const uint8_t* __restrict__ Cg,
                 const int* __restrict__ texp, int k2, ColList<double> Y, double beta, int n,
                 const int* __restrict__ xe) {
  extern __shared__ __align__(1024) uint8_t smtc[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nt = blockIdx.y, j0 = nt * TC_NMAX;
  const int N = tc_tile_n(k2, nt);
  const int BB = D8_S * N * 32;                          // B bytes per stage
  const int SB = (TC_ABYTES + BB + 1023) / 1024 * 1024;  // stage stride
  uint8_t* base = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smtc) + 1023) & ~(uintptr_t)1023);
  int* rexp = reinterpret_cast<int*>(base + TC_STAGES * SB);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(rexp + TC_M);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + TC_STAGES);
  const int r0 = blockIdx.x * TC_M;
  const uint8_t* Ct = Cg + (size_t)j0 * k1p * (D8_S * 2);
  const uint32_t ncols = N <= 16 ? 128u : (N <= 32 ? 256u : 512u);

  if (warp == 0) gcge::tc::tmem_alloc(tslot, ncols);
  if (tid == 0)
    for (int s = 0; s < TC_STAGES; s++) gcge::tc::mbar_init(&mbar[s], 1);
  if (tid < TC_M) rexp[tid] = -2000;
  gcge::tc::fence_before();
  __syncthreads();
  gcge::tc::fence_after();
  // row exponents: four threads per row, the high words of all (<= 32) of a
  // thread's values loaded at once
  {
    const int rr = tid & (TC_M - 1), part = tid >> 7;
    const int r = r0 + rr;
    int e = -2000;
    if (r < n) {
      int hv[32];
#pragma unroll
      for (int q = 0; q < 32; q++) {
        const int i = part + 4 * q;
        hv[q] = (i < k1) ? ld_hi(X.p[i] + r) : 0;
      }
      if (!xe) {
        int fmax = 0, bad = 0;
#pragma unroll
        for (int q = 0; q < 32; q++) {
          const int f = (hv[q] >> 20) & 0x7FF;
          bad |= f == 0x7FF;
          fmax = max(fmax, f);
        }
        e = bad ? 4096 : (fmax == 0 ? -2000 : fmax - 1022);
      } else {
#pragma unroll
        for (int q = 0; q < 32; q++) {
          const int i = part + 4 * q;
          if (i < k1) {
            const int ex = oz_exp_hi(hv[q]);
            e = max(e, (ex >= 4096 || ex <= -2000) ? ex : ex - oz_bal(xe, i));
          }
        }
      }
    }
    atomicMax(&rexp[rr], e);
  }
  __syncthreads();
  const uint32_t tmem = *tslot;

  // slicing role: row srr, values k = 16 s + 4 kq + q (q < 4); the two
  // threads of a lane pair fill the two halves of one 16-byte core-matrix row
  const int srr = (tid >> 1) & (TC_M - 1), kq = ((tid >> 8) << 1) | (tid & 1);
  const int sr = r0 + srr;
  const int myexp = rexp[srr];
  const int doff = (kq >> 1) * 2048 + (srr >> 3) * 128 + (srr & 7) * 16 + (kq & 1) * 8;
  const int nks = k1p / TC_KS;
  bool ok = true;
  double vn[4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int i = 4 * kq + q;
    vn[q] = (sr < n && i < k1) ? __ldg(X.p[i] + sr) : 0.0;
  }
  for (int s = 0; s < nks; s++) {
    const int buf = s % TC_STAGES;
    double v[4];
#pragma unroll
    for (int q = 0; q < 4; q++) v[q] = vn[q];
    if (s + 1 < nks) {
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int i = (s + 1) * TC_KS + 4 * kq + q;
        vn[q] = (sr < n && i < k1) ? __ldg(X.p[i] + sr) : 0.0;
      }
    }
    uint8_t* As = base + buf * SB;
    uint8_t* Bs = As + TC_ABYTES;
    if (s >= TC_STAGES) {
      // the MMAs of stage s - TC_STAGES read this buffer
      if (!gcge::tc::mbar_wait_warp(&mbar[buf], ((s / TC_STAGES) - 1) & 1, TC_WAIT)) ok = false;
    }
    {
      int E[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int i = s * TC_KS + 4 * kq + q;
        E[q] = (myexp >= 4096) ? 4096 : myexp + ((i < k1) ? oz_bal(xe, i) : 0);
        if (myexp >= 4096) v[q] = 0.0;
      }
      d8_slice4(v, E, As + doff, TC_M * TC_KS * 2);
    }
    // B operand of this stage: one contiguous block of BB bytes
    {
      const uint4* src = reinterpret_cast<const uint4*>(Ct + (size_t)s * BB);
      uint4* dst = reinterpret_cast<uint4*>(Bs);
      for (int e = tid; e < BB / 16; e += TC_T) dst[e] = __ldg(src + e);
    }
    gcge::tc::fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      gcge::tc::fence_after();
      d8_issue(tmem, gcge::tc::smem_u32(As), TC_M * TC_KS * 2, gcge::tc::smem_u32(Bs), N, s == 0);
      gcge::tc::commit(&mbar[buf]);
    }
  }
  // wait for the last stage (its commit covers every earlier MMA)
  {
    const int s = nks - 1;
    if (!gcge::tc::mbar_wait_warp(&mbar[s % TC_STAGES], (s / TC_STAGES) & 1, TC_WAIT)) ok = false;
  }
  gcge::tc::fence_after();
  const int anybad = __syncthreads_or(ok ? 0 : 1);
  if (anybad) {
    if (tid == 0) atomicExch(&g_oz_tc_status, 1);
    d8_fill_nan(Y, j0, N, k2, n, r0);
  } else {
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31, column quarter w / 4
    const int q4 = warp & 3, cg = warp >> 2;
    const int row = r0 + 32 * q4 + lane;
    const int re = rexp[32 * q4 + lane];
    const int quarter = N / 4;
    for (int c0 = cg * quarter; c0 < (cg + 1) * quarter; c0 += 4) {
      uint32_t acc[D8_NL][4];
#pragma unroll
      for (int l = 0; l < D8_NL; l++)
        gcge::tc::tmem_ld4(tmem + ((uint32_t)(32 * q4) << 16) + (uint32_t)(l * N + c0), acc[l]);
      gcge::tc::tmem_wait_ld();
#pragma unroll
      for (int jj = 0; jj < 4; jj++) {
        const int j = j0 + c0 + jj;
        if (j >= k2 || row >= n) continue;
        long long T = 0;
#pragma unroll
        for (int l = 0; l < D8_NL; l++) {
          const long long v = (long long)__float2int_rn(__uint_as_float(acc[l][jj]));
          const int sh = 57 - 8 * (l + 2);  // levels 8, 9 rounded to the nearest unit
          T += sh >= 0 ? (v << sh) : ((v + (1ll << (-sh - 1))) >> (-sh));
        }
        const int te = __ldg(texp + j);
        double y;
        if (re >= 4096 || te >= 4096) y = __longlong_as_double(0x7ff8000000000000ll);
        else if (re <= -2000 || te <= -2000) y = 0.0;
        else y = d8_to_double(T, re + te - 55);
        double* yp = Y.p[j] + row;
        *yp = (beta == 0.0) ? y : fma(beta, *yp, y);
      }
    }
  }
  gcge::tc::fence_before();
  __syncthreads();
  if (warp == 0) {
    gcge::tc::fence_after();
    gcge::tc::tmem_dealloc(tmem, ncols);
  }
}

size_t tc_lincomb_smem(int N) {
  const int SB = (TC_ABYTES + D8_S * N * 32 + 1023) / 1024 * 1024;
  return (size_t)TC_STAGES * SB + 1024 /* alignment */ + TC_M * 4 + TC_STAGES * 8 + 16;
}
// ---------------------------------------------------------------- tcgen05 Gram
// G = V^T diag(wd) W (wd NULL: identity) with FP64 accuracy.  One CTA per SM
// owns up to GC_MI columns of V (MMA M, TMEM lane = column of V) and 16
// columns of W (MMA N) over a contiguous run of 64-row chunks.  Its warps have
// fixed roles and hand work over through mbarriers (no block-wide barrier in
// the loop):
//  * producer/MMA warp: streams each chunk's columns (and the diagonal) into
//    a ring of raw FP64 buffers in shared memory with cp.async.bulk, and for
//    every 16-row stage issues the skewed digit MMAs into the chunk's 8 level
//    accumulators in tensor memory (two accumulator sets alternate);
//  * 12 slicer warps: per chunk the column scales (largest exponent over the
//    chunk's 64 rows, a W column taken with the diagonal; a warp max of the
//    raw exponent fields), then per stage the 7 balanced base-256 digits of
//    every value into a double-buffered stage in shared memory;
//  * 4 fold warps (one per TMEM lane quadrant): per chunk, the exact level
//    sums (FP32, below 2^24 for 64 rows) combined in 32-bit pairs into a
//    64-bit fixed-point value, added to a 64-bit accumulator per output that
//    is rounded into an FP64 partial sum only when the chunk exponent changes
//    (or the integer sum would overflow).
// Each CTA writes its FP64 partial Gram; a second kernel adds the partials in
// a fixed order.
constexpr int GC_K = 64;                 // rows per exact chunk
constexpr int GC_ST = GC_K / TC_KS;      // stages per chunk (4)
constexpr int GC_N = 16;                 // W columns per CTA
constexpr int GC_MI = 96;                // V columns per CTA
constexpr int GC_SW = 12;                // slicer warps
constexpr int GC_FW = 4;                 // fold warps
constexpr int GC_THREADS = (GC_SW + GC_FW + 1) * 32;
constexpr int GC_PW = GC_SW + GC_FW;     // producer/MMA warp
constexpr int GC_RAWLD = GC_K * 8 + 16;  // bytes per raw column (padded: conflict-free reads)
constexpr int GC_MAXRAW = 3;
constexpr int GC_CE = TC_M + GC_N;       // exponent slots: V columns, then W columns
constexpr int GC_SB = (TC_ABYTES + D8_S * GC_N * 32 + 1023) / 1024 * 1024;  // stage bytes
constexpr int GC_FOLDB = TC_M * GC_N * 20;  // fold state: FP64 sum, 64-bit value, exponent
constexpr int GC_FIXED = 1024 + 3 * GC_CE * 4 + (8 + GC_MAXRAW) * 8 + 16;
constexpr int GC_SMEM_CAP = 227 * 1024;

__host__ __device__ __forceinline__ int gc_nraw(int rawcols) {
  const int room = GC_SMEM_CAP - 2 * GC_SB - GC_FOLDB - GC_FIXED;
  const int k = room / (rawcols * GC_RAWLD);
  return k < GC_MAXRAW ? k : GC_MAXRAW;
}
size_t gc_smem(int rawcols) {
  return (size_t)2 * GC_SB + GC_FOLDB + GC_FIXED + (size_t)gc_nraw(rawcols) * rawcols * GC_RAWLD;
}

// A quad: 4 consecutive rows of one column of a 16-row stage.  A tile of
// ncolt columns has 4 * ncolt quads per stage; quad u is half h = u & 1 of
// the core-matrix row of column (u >> 1) % ncolt in K slab g = (u >> 1) /
// ncolt (rows 8 g + 4 h .. +3), so a lane pair fills one 16-byte row.
struct GcQuad {
  int col, roff, g, h;
};
__device__ __forceinline__ GcQuad gc_quad(int u, int ncolt) {
  GcQuad q;
  q.h = u & 1;
  const int rest = u >> 1;
  q.col = rest % ncolt;
  q.g = rest / ncolt;
  q.roff = q.g * 8 + q.h * 4;
  return q;
}

__device__ __forceinline__ void gc_flush(long long* gT, int* gE, double* gS) {
  if (*gT != 0) *gS += d8_to_double(*gT, *gE - 48);
  *gT = 0;
  *gE = -1000000;
}

template <bool BULK>
__global__ void __launch_bounds__(GC_THREADS, 1)
    k_gram_tc(ColList<double> V, int k1, ColList<double> W, int k2, int n, int ntn,
              const double* __restrict__ wd, double* __restrict__ partial, int nchunks,
              int nraw) {
  extern __shared__ __align__(1024) uint8_t smgc[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int mt = blockIdx.y / ntn, nt = blockIdx.y % ntn;
  const int i0 = mt * GC_MI, j0 = nt * GC_N;
  const int mi = min(GC_MI, k1 - i0), nj = min(GC_N, k2 - j0);
  const int ncolt = mi + nj;
  const int rawcols = ncolt + (wd ? 1 : 0);
  const int RC = rawcols * GC_RAWLD;
  constexpr uint32_t ncols = 2 * D8_NL * GC_N;  // two sets of 8 levels (256)
  uint8_t* base = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smgc) + 1023) & ~(uintptr_t)1023);
  double* gS = reinterpret_cast<double*>(base + 2 * GC_SB);
  long long* gT = reinterpret_cast<long long*>(gS + TC_M * GC_N);
  int* gE = reinterpret_cast<int*>(gT + TC_M * GC_N);
  uint8_t* rawbase = reinterpret_cast<uint8_t*>(gE + TC_M * GC_N);
  int* cex = reinterpret_cast<int*>(rawbase + nraw * RC);
  uint64_t* mfull = reinterpret_cast<uint64_t*>(cex + 3 * GC_CE);  // stage digits ready (2)
  uint64_t* mempty = mfull + 2;   // stage MMAs done (2)
  uint64_t* maccf = mfull + 4;    // chunk accumulators complete (2)
  uint64_t* macce = mfull + 6;    // chunk accumulators folded (2)
  uint64_t* mraw = mfull + 8;     // raw chunk arrived (nraw)
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mraw + GC_MAXRAW);
  // this CTA's chunks: a contiguous run (consecutive reads of every column)
  const int cbase = nchunks / (int)gridDim.x, crem = nchunks % (int)gridDim.x;
  const int nch = cbase + ((int)blockIdx.x < crem ? 1 : 0);
  const int cfirst = (int)blockIdx.x * cbase + min((int)blockIdx.x, crem);
  auto colptr = [&](int col) -> const double* {
    return col < mi ? V.p[i0 + col] : (col < ncolt ? W.p[j0 + col - mi] : wd);
  };

  if (warp == 0) gcge::tc::tmem_alloc(tslot, ncols);
  if (tid == 0) {
    for (int b = 0; b < 2; b++) {
      gcge::tc::mbar_init(&mfull[b], GC_SW);
      gcge::tc::mbar_init(&mempty[b], 1);
      gcge::tc::mbar_init(&maccf[b], 1);
      gcge::tc::mbar_init(&macce[b], GC_FW);
    }
    for (int b = 0; b < nraw; b++) gcge::tc::mbar_init(&mraw[b], 1);
  }
  for (int e = tid; e < TC_M * GC_N; e += GC_THREADS) {
    gS[e] = 0.0;
    gT[e] = 0;
    gE[e] = -1000000;
  }
  gcge::tc::fence_before();
  __syncthreads();
  gcge::tc::fence_after();
  const uint32_t tmem = *tslot;
  bool ok = true;

  if (warp == GC_PW) {
    // ------------------------------------------------ producer / MMA warp
    auto issue_raw = [&](int cc) {
      const int row0 = (cfirst + cc) * GC_K;
      const int valid = min(GC_K, n - row0);
      const int rows = BULK ? (valid & ~1) : 0;
      uint64_t* mb = &mraw[cc % nraw];
      if (lane == 0) gcge::tc::mbar_arrive_expect_tx(mb, (uint32_t)(rawcols * rows * 8));
      __syncwarp();
      if (rows > 0) {
        uint8_t* dst = rawbase + (cc % nraw) * RC;
        for (int col = lane; col < rawcols; col += 32)
          gcge::tc::bulk_g2s(dst + col * GC_RAWLD, colptr(col) + row0, (uint32_t)(rows * 8), mb);
      }
    };
    for (int cc = 0; cc < nraw && cc < nch; cc++) issue_raw(cc);
    for (int c = 0; c < nch; c++) {
      const int tb = c & 1;
      if (c >= 2 && !gcge::tc::mbar_wait_warp(&macce[tb], ((c >> 1) - 1) & 1, TC_WAIT)) ok = false;
      for (int st = 0; st < GC_ST; st++) {
        const int g = c * GC_ST + st, buf = g & 1;
        if (!gcge::tc::mbar_wait_warp(&mfull[buf], (g >> 1) & 1, TC_WAIT)) ok = false;
        if (lane == 0) {
          gcge::tc::fence_after();
          uint8_t* As = base + buf * GC_SB;
          d8_issue(tmem + (uint32_t)(tb * D8_NL * GC_N), gcge::tc::smem_u32(As),
                   TC_M * TC_KS * 2, gcge::tc::smem_u32(As + TC_ABYTES), GC_N, st == 0);
          gcge::tc::commit(&mempty[buf]);
          if (st == GC_ST - 1) gcge::tc::commit(&maccf[tb]);
        }
        __syncwarp();
      }
      // every slicer has cut chunk c: its raw buffer can be refilled
      if (c + nraw < nch) issue_raw(c + nraw);
    }
  } else if (warp >= GC_SW) {
    // ------------------------------------------------ fold warps
    const int q4 = warp - GC_SW;
    const int i = 32 * q4 + lane;
    for (int c = 0; c < nch; c++) {
      const int tb = c & 1;
      if (!gcge::tc::mbar_wait_warp(&maccf[tb], (c >> 1) & 1, TC_WAIT)) ok = false;
      gcge::tc::fence_after();
      if (32 * q4 < mi) {
        const int* ce = cex + (c % 3) * GC_CE;
        const int ea = ce[i];
        const uint32_t tacc = tmem + (uint32_t)(tb * D8_NL * GC_N) + ((uint32_t)(32 * q4) << 16);
#pragma unroll
        for (int c0 = 0; c0 < GC_N; c0 += 4) {
          uint32_t acc[D8_NL][4];
#pragma unroll
          for (int l = 0; l < D8_NL; l++)
            gcge::tc::tmem_ld4(tacc + (uint32_t)(l * GC_N + c0), acc[l]);
          gcge::tc::tmem_wait_ld();
#pragma unroll
          for (int jj = 0; jj < 4; jj++) {
            const int j = c0 + jj;
            if (i >= mi || j >= nj) continue;
            const int eb = ce[TC_M + j];
            const int o = j * TC_M + i;
            if (ea >= 4096 || eb >= 4096) {
              gS[o] = __longlong_as_double(0x7ff8000000000000ll);
            } else if (ea > -2000 && eb > -2000) {
              int lv[D8_NL];
#pragma unroll
              for (int l = 0; l < D8_NL; l++) lv[l] = __float2int_rn(__uint_as_float(acc[l][jj]));
              // level pairs (L, L+1) in 32 bits: |acc_L| <= 7 * 2^14 * 64 < 2^23
              const int p0 = lv[0] * 256 + lv[1], p1 = lv[2] * 256 + lv[3];
              const int p2 = lv[4] * 256 + lv[5], p3 = lv[6] * 256 + lv[7];
              const long long T = ((long long)p0 << 26) + ((long long)p1 << 10) +
                                  (long long)((p2 + 32) >> 6) +
                                  (long long)((p3 + (1 << 21)) >> 22);  // sum_L acc_L 2^{50-8L}
              const int E = ea + eb;
              const long long t = gT[o], r = t + T;
              if (gE[o] != E || ((t ^ r) & (T ^ r)) < 0) {
                gc_flush(gT + o, gE + o, gS + o);
                gT[o] = T;
                gE[o] = E;
              } else {
                gT[o] = r;
              }
            }
          }
        }
      }
      gcge::tc::fence_before();
      __syncwarp();
      if (lane == 0) gcge::tc::mbar_arrive(&macce[tb]);
    }
  } else {
    // ------------------------------------------------ slicer warps
    const int nquads = 4 * ncolt;
    const int st0 = warp * 32 + lane;  // first quad of this thread
    const GcQuad uq = gc_quad(st0 < nquads ? st0 : 0, ncolt);
    for (int c = 0; c < nch; c++) {
      const int cb = cfirst + c;
      const int row0 = cb * GC_K;
      const int valid = min(GC_K, n - row0);
      const int rb = c % nraw;
      double* raw = reinterpret_cast<double*>(rawbase + rb * RC);
      if (!gcge::tc::mbar_wait_warp(&mraw[rb], (c / nraw) & 1, TC_WAIT)) ok = false;
      const int rfill = BULK ? (valid & ~1) : 0;
      if (rfill < GC_K) {  // rows the bulk copy did not bring: tail row, zero padding
        const int nr = GC_K - rfill;
        for (int e = st0; e < rawcols * nr; e += GC_SW * 32) {
          const int col = e / nr, rr = rfill + e % nr;
          raw[col * (GC_RAWLD / 8) + rr] = rr < valid ? __ldg(colptr(col) + row0 + rr) : 0.0;
        }
        gcge::tc::named_sync(1, GC_SW * 32);
      }
      // chunk exponents: warp per column, lane = rows 2 lane, 2 lane + 1
      int* ce = cex + (c % 3) * GC_CE;
      for (int col = warp; col < ncolt; col += GC_SW) {
        const double2 v2 =
            *reinterpret_cast<const double2*>(raw + col * (GC_RAWLD / 8) + 2 * lane);
        int f0 = (__double2hiint(v2.x) >> 20) & 0x7FF, f1 = (__double2hiint(v2.y) >> 20) & 0x7FF;
        int bad = (f0 == 0x7FF) | (f1 == 0x7FF);
        if (wd && col >= mi) {
          const double2 w2 =
              *reinterpret_cast<const double2*>(raw + ncolt * (GC_RAWLD / 8) + 2 * lane);
          const int g0 = (__double2hiint(w2.x) >> 20) & 0x7FF,
                    g1 = (__double2hiint(w2.y) >> 20) & 0x7FF;
          bad |= (g0 == 0x7FF) | (g1 == 0x7FF);
          // product fields (a product at the bottom of the range still gets >= 1)
          f0 = (f0 == 0 || g0 == 0) ? 0 : max(f0 + g0 - 1022, 1);
          f1 = (f1 == 0 || g1 == 0) ? 0 : max(f1 + g1 - 1022, 1);
        }
        const int fmax = __reduce_max_sync(0xffffffffu, max(f0, f1));
        const int anybad = __reduce_or_sync(0xffffffffu, bad);
        if (lane == 0)
          ce[col < mi ? col : TC_M + col - mi] = anybad ? 4096 : (fmax == 0 ? -2000 : fmax - 1022);
      }
      gcge::tc::named_sync(1, GC_SW * 32);
      for (int st = 0; st < GC_ST; st++) {
        const int g = c * GC_ST + st, buf = g & 1;
        if (g >= 2 && !gcge::tc::mbar_wait_warp(&mempty[buf], ((g >> 1) - 1) & 1, TC_WAIT))
          ok = false;
        uint8_t* As = base + buf * GC_SB;
        uint8_t* Bs = As + TC_ABYTES;
        for (int u = st0; u < nquads; u += GC_SW * 32) {
          const GcQuad q = (u == st0) ? uq : gc_quad(u, ncolt);
          const bool isv = q.col < mi;
          const double* src = raw + q.col * (GC_RAWLD / 8) + st * TC_KS + q.roff;
          const double2 a01 = *reinterpret_cast<const double2*>(src);
          const double2 a23 = *reinterpret_cast<const double2*>(src + 2);
          double v[4] = {a01.x, a01.y, a23.x, a23.y};
          if (wd && !isv) {
            const double* ws = raw + ncolt * (GC_RAWLD / 8) + st * TC_KS + q.roff;
            const double2 w01 = *reinterpret_cast<const double2*>(ws);
            const double2 w23 = *reinterpret_cast<const double2*>(ws + 2);
            v[0] *= w01.x;
            v[1] *= w01.y;
            v[2] *= w23.x;
            v[3] *= w23.y;
          }
          const int E0 = ce[isv ? q.col : TC_M + q.col - mi];
          int E[4];
#pragma unroll
          for (int t = 0; t < 4; t++) {
            E[t] = E0;
            if (E0 >= 4096) v[t] = 0.0;
          }
          const int cc = isv ? q.col : q.col - mi;
          uint8_t* dst = (isv ? As + q.g * (TC_M / 8 * 128) : Bs + q.g * (D8_S * GC_N * 16)) +
                         (cc >> 3) * 128 + (cc & 7) * 16 + q.h * 8;
          d8_slice4(v, E, dst, isv ? TC_M * TC_KS * 2 : GC_N * 16);
        }
        gcge::tc::fence_proxy_async();
        __syncwarp();
        if (lane == 0) gcge::tc::mbar_arrive(&mfull[buf]);
      }
    }
  }
  const int anybad = __syncthreads_or(ok ? 0 : 1);
  if (anybad && tid == 0) atomicExch(&g_oz_tc_status, 1);
  // partial layout [block][o], o = i + j*k1 (the flex-Gram reduction layout)
  double* out = partial + (size_t)blockIdx.x * k1 * k2;
  for (int e = tid; e < mi * nj; e += GC_THREADS) {
    const int ii = e % mi, jj = e / mi;
    const int o = jj * TC_M + ii;
    gc_flush(gT + o, gE + o, gS + o);
    out[(i0 + ii) + (size_t)(j0 + jj) * k1] =
        anybad ? __longlong_as_double(0x7ff8000000000000ll) : gS[o];
  }
  gcge::tc::fence_before();
  __syncthreads();
  if (warp == 0) {
    gcge::tc::fence_after();
    gcge::tc::tmem_dealloc(tmem, ncols);
  }
}

// Returns the CTAs along the rows (the partial blocks to add).
template <bool BULK>
int gram_tc_all(const ColList<double>& V, int k1, const ColList<double>& W, int k2, int n,
                const double* wd, double* partial, cudaStream_t st) {
  const int ntm = (k1 + GC_MI - 1) / GC_MI, ntn = (k2 + GC_N - 1) / GC_N;
  const int nchunks = (n + GC_K - 1) / GC_K;
  const int rawcols = (k1 < GC_MI ? k1 : GC_MI) + (k2 < GC_N ? k2 : GC_N) + (wd ? 1 : 0);
  const int nraw = gc_nraw(rawcols);
  const int nblk = nchunks < 152 ? nchunks : 152;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_gram_tc<BULK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         GC_SMEM_CAP);
    attr = true;
  }
  k_gram_tc<BULK><<<dim3(nblk, ntm * ntn), GC_THREADS, gc_smem(rawcols), st>>>(
      V, k1, W, k2, n, ntn, wd, partial, nchunks, nraw);
  return nblk;
}

// ---------------------------------------------------------------- digit planes
// The Gram blocks of one GCG iteration (the block Gram-Schmidt passes of the W
// orthogonalisation and the Rayleigh-Ritz projection) all multiply the same
// basis columns [X, P] (and W once it is orthonormal), so those columns are
// cut into digits once, into "digit planes": per column and 64-row chunk a
// record of PL_REC bytes,
//   bytes 0..3    the chunk exponent E (|x| < 2^E over the chunk; -2000 for
//                 an all-zero chunk, 4096 when the chunk holds a NaN or Inf),
//   bytes 16..    4 stages of 16 rows, each stage 7 digit rows of 16 bytes:
//                 digit a (0 = most significant) of row r is byte a of
//                 u = m + 0x0080808080808080, m = trunc(x 2^{55-E}),
//                 i.e. the balanced base-256 digit plus 128.
// Seven digit bytes hold m only while m <= 0x007F7F7F7F7F7F7F (the top digit
// then stays in [-128, 127]); a chunk whose largest value is within 0.4 % of
// 2^E is cut with E + 1 instead (54 bits of it kept).  Rows past n are zero.
// The Gram kernel turns a byte b into the f16 value (1024 + b) - 1152 = b - 128
// with one byte permute and one half2 subtraction per two digits.
// Layout of a plane set: chunk-major, the records of chunk q for columns
// 0 .. ldp-1 side by side at planes + (q * ldp + c) * PL_REC, so the records of
// a run of columns for one chunk are one contiguous block (one bulk copy).
constexpr int PL_K = 64;              // rows per record (the Gram's chunk)
constexpr int PL_HDR = 16;            // header bytes
constexpr int PL_STB = D8_S * TC_KS;  // bytes per 16-row stage (112)
constexpr int PL_REC = PL_HDR + (PL_K / TC_KS) * PL_STB;  // 464
constexpr long long PL_MAXM = 0x007F7F7F7F7F7F7Fll;
constexpr int PL_WARPS = 8;

// m = trunc(x 2^{55-E}) for |x| < 2^{E+1} (zero, subnormal and non-finite: 0)
__device__ __forceinline__ long long d8_mant(double x, int E) {
  const long long b = __double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7FF);
  if (ex == 0 || ex == 0x7FF) return 0;
  const unsigned long long mant = ((unsigned long long)b & ((1ull << 52) - 1)) | (1ull << 52);
  const int sh = ex - 1020 - E;
  const unsigned long long mm = sh >= 0 ? (mant << sh) : (sh > -64 ? (mant >> (-sh)) : 0ull);
  return b < 0 ? -(long long)mm : (long long)mm;
}

// One warp per (column, chunk): lane l holds rows 2l, 2l+1 of the chunk.  The
// record is assembled in shared memory and written as 29 16-byte stores.
// Grid: (chunk groups, columns), PL_WARPS warps per block; column y of X goes
// to plane column c0 + y.  d (optional): the rows are weighted first,
// x[r] * d[r] rounded to FP64 (the B-inner product of a diagonal B).
__global__ void __launch_bounds__(PL_WARPS * 32)
    k_cut_planes(ColList<double> X, const double* __restrict__ d, int n, int nchunks,
                 uint8_t* __restrict__ planes, int ldp, int c0) {
  __shared__ __align__(16) uint8_t rec[PL_WARPS][PL_REC];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double* x = X.p[blockIdx.y];
  uint8_t* out = planes + (size_t)(c0 + (int)blockIdx.y) * PL_REC;
  const size_t qstride = (size_t)ldp * PL_REC;
  uint8_t* sb = rec[warp];
  const bool vec = ((uintptr_t)x & 15) == 0 && ((uintptr_t)d & 15) == 0;
  for (int q = blockIdx.x * PL_WARPS + warp; q < nchunks; q += gridDim.x * PL_WARPS) {
    const int r = q * PL_K + 2 * lane;
    double v0 = 0.0, v1 = 0.0;
    if (vec && r + 1 < n) {
      const double2 t = __ldg(reinterpret_cast<const double2*>(x + r));
      v0 = t.x;
      v1 = t.y;
      if (d) {
        const double2 w = __ldg(reinterpret_cast<const double2*>(d + r));
        v0 *= w.x;
        v1 *= w.y;
      }
    } else {
      if (r < n) v0 = __ldg(x + r) * (d ? __ldg(d + r) : 1.0);
      if (r + 1 < n) v1 = __ldg(x + r + 1) * (d ? __ldg(d + r + 1) : 1.0);
    }
    const int f0 = (__double2hiint(v0) >> 20) & 0x7FF, f1 = (__double2hiint(v1) >> 20) & 0x7FF;
    const int fmax = __reduce_max_sync(0xffffffffu, max(f0 == 0x7FF ? 0 : f0, f1 == 0x7FF ? 0 : f1));
    const int bad = __reduce_or_sync(0xffffffffu, (f0 == 0x7FF) | (f1 == 0x7FF));
    int E = bad ? 4096 : (fmax == 0 ? -2000 : fmax - 1022);
    long long m0 = 0, m1 = 0;
    if (E > -2000 && E < 4096) {
      m0 = d8_mant(v0, E);
      m1 = d8_mant(v1, E);
      if (__any_sync(0xffffffffu, m0 > PL_MAXM || m1 > PL_MAXM)) {
        E += 1;
        m0 = d8_mant(v0, E);
        m1 = d8_mant(v1, E);
      }
    }
    const unsigned long long u0 = (unsigned long long)(m0 + 0x0080808080808080ll);
    const unsigned long long u1 = (unsigned long long)(m1 + 0x0080808080808080ll);
    // rows 2l, 2l+1: stage l / 8, rows 2 (l % 8), 2 (l % 8) + 1 of it
    uint8_t* dst = sb + PL_HDR + (lane >> 3) * PL_STB + 2 * (lane & 7);
#pragma unroll
    for (int a = 0; a < D8_S; a++) {
      const int sh = 8 * (D8_S - 1 - a);
      const unsigned short w = (unsigned short)(((u0 >> sh) & 0xFF) | (((u1 >> sh) & 0xFF) << 8));
      *reinterpret_cast<unsigned short*>(dst + a * TC_KS) = w;
    }
    if (lane < 4) reinterpret_cast<int*>(sb)[lane] = lane == 0 ? E : 0;
    __syncwarp();
    if (lane < PL_REC / 16)
      reinterpret_cast<uint4*>(out + (size_t)q * qstride)[lane] = reinterpret_cast<const uint4*>(sb)[lane];
    __syncwarp();
  }
}

// Two biased digit bytes (the low half first) -> two f16 digits in one word.
__device__ __forceinline__ uint32_t pl_f16x2(uint32_t word, uint32_t sel) {
  const uint32_t h = __byte_perm(word, 0x64u, sel);
  const __half2 v = __hsub2(*reinterpret_cast<const __half2*>(&h), __float2half2_rn(1152.0f));
  return *reinterpret_cast<const uint32_t*>(&v);
}

// G = V^T W with both operands given as digit planes: V = plane columns
// voff .. voff + k1 - 1 of a set of ldv columns, W = plane columns
// woff .. woff + k2 - 1 of a set of ldw columns (a diagonal weight is folded
// into W's planes when they are cut).  One CTA per SM owns up to GC_MI columns
// of V (MMA M, TMEM lane) and GC_N columns of W (MMA N) over a contiguous run
// of 64-row chunks.  Per chunk one bulk copy brings V's records and one W's
// (the chunk-major plane layout makes each a contiguous block) into a ring of
// raw buffers.  Roles:
//  * warp 0, one thread: issues the bulk copies and, per 16-row stage once the
//    stage is converted, the stage's skewed MMAs into the chunk's level
//    accumulators in tensor memory (two sets alternate), committing them to
//    the stage buffer's "empty" barrier;
//  * 11 converter warps: per stage they turn the digit bytes of both operands
//    into f16 digits (32-byte swizzled K-major operand layout) in a ring of
//    GP_NS stage buffers and arrive on the buffer's "full" barrier; they run
//    ahead of the MMAs by up to GP_NS stages, so conversion and MMA execution
//    overlap;
//  * 8 fold warps (two per TMEM lane quadrant, 8 W columns each): per chunk
//    the exact level sums into a 64-bit fixed-point accumulator per output,
//    rounded into an FP64 partial only when the chunk exponent changes; each
//    fold thread keeps its 8 outputs' state in registers and writes them at
//    the end.
constexpr int GP_CW = 11;                       // converter warps (warps 1 .. 11)
constexpr int GP_FW = 8;                        // fold warps (warps 12 .. 19)
constexpr int GP_THREADS = (1 + GP_CW + GP_FW) * 32;
constexpr int GP_NS = 3;                        // stage buffers
constexpr int GP_FIXED = 1024 + 3 * GC_CE * 4 + (2 * GP_NS + 4 + GC_MAXRAW) * 8 + 16;

__host__ __device__ __forceinline__ int gp_nraw(int mi, int nj) {
  const int room = GC_SMEM_CAP - GP_NS * GC_SB - GP_FIXED;
  const int k = room / ((mi + nj) * PL_REC);
  return k < GC_MAXRAW ? k : GC_MAXRAW;
}
size_t gp_smem(int mi, int nj) {
  return (size_t)GP_NS * GC_SB + GP_FIXED + (size_t)gp_nraw(mi, nj) * (mi + nj) * PL_REC;
}

// the digit bytes of rows 4q .. 4q+3 of a record's stage -> 7 f16 digit pairs
// (8 bytes each) at dst + a * dstride
__device__ __forceinline__ void pl_quad(const uint8_t* rec, int st, int q, uint8_t* dst,
                                        int dstride) {
  const uint8_t* src = rec + PL_HDR + st * PL_STB + q * 4;
#pragma unroll
  for (int a = 0; a < D8_S; a++) {
    const uint32_t w = *reinterpret_cast<const uint32_t*>(src + a * TC_KS);
    uint2 o;
    o.x = pl_f16x2(w, 0x4140);
    o.y = pl_f16x2(w, 0x4342);
    *reinterpret_cast<uint2*>(dst + a * dstride) = o;
  }
}

// The skewed MMAs of one 16-row stage on operands in the 32-byte swizzled
// K-major layout: digit a of A (TC_M rows) at abase + (a - 1) * TC_M * 32,
// digit b of B (GC_N rows) at bbase + (b - 1) * GC_N * 32.  Level L = a + b
// accumulates at TMEM column (L - 2) * GC_N; FIRST (the chunk's first stage)
// starts every level afresh.  Shapes and offsets are compile-time; the
// descriptors are the base descriptors plus start-address increments (the
// 14-bit address field does not carry: shared addresses are below 256 KB).
template <bool FIRST>
__device__ __forceinline__ void gp_issue(uint32_t tacc, uint32_t abase, uint32_t bbase) {
  const uint64_t ad0 = gcge::tc::smem_desc_sw32(abase, 256);
  const uint64_t bd0 = gcge::tc::smem_desc_sw32(bbase, 256);
#pragma unroll
  for (int a = 1; a <= D8_S; a++) {
    const uint64_t ad = ad0 + (uint64_t)(((a - 1) * TC_M * 32) >> 4);
    const int bmax = (9 - a) < D8_S ? (9 - a) : D8_S;
    // levels a + 1 .. a + bmax; on the first stage level 2 (a = 1) and level
    // 9 (a = 2, b = 7) are written first by a = 1 / a = 2 and must start fresh
    if (FIRST && a == 2) {
      gcge::tc::mma_bf16(tacc + (uint32_t)((a - 1) * GC_N), ad, bd0,
                         gcge::tc::idesc_f16(TC_M, (bmax - 1) * GC_N), 1u);
      gcge::tc::mma_bf16(tacc + (uint32_t)((a + D8_S - 2) * GC_N), ad,
                         bd0 + (uint64_t)(((D8_S - 1) * GC_N * 32) >> 4),
                         gcge::tc::idesc_f16(TC_M, GC_N), 0u);
    } else {
      gcge::tc::mma_bf16(tacc + (uint32_t)((a - 1) * GC_N), ad, bd0,
                         gcge::tc::idesc_f16(TC_M, bmax * GC_N), (FIRST && a == 1) ? 0u : 1u);
    }
  }
}

// the fold state of one output: FP64 sum, 64-bit fixed-point value, exponent
__device__ __forceinline__ void gp_flush(long long& T, int& E, double& S) {
  if (T != 0) S += d8_to_double(T, E - 48);
  T = 0;
  E = -1000000;
}

__global__ void __launch_bounds__(GP_THREADS, 1)
    k_gram_pp(const uint8_t* __restrict__ vpl, int ldv, int voff, int k1,
              const uint8_t* __restrict__ wpl, int ldw, int woff, int k2, int ntn,
              double* __restrict__ partial, int nchunks, int nraw) {
  extern __shared__ __align__(1024) uint8_t smgc[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int mt = blockIdx.y / ntn, nt = blockIdx.y % ntn;
  const int i0 = mt * GC_MI, j0 = nt * GC_N;
  const int mi = min(GC_MI, k1 - i0), nj = min(GC_N, k2 - j0);
  const int VB = mi * PL_REC, RC = VB + nj * PL_REC;
  constexpr uint32_t ncols = 2 * D8_NL * GC_N;
  uint8_t* base = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smgc) + 1023) & ~(uintptr_t)1023);
  uint8_t* rawbase = base + GP_NS * GC_SB;
  int* cex = reinterpret_cast<int*>(rawbase + nraw * RC);
  uint64_t* mfull = reinterpret_cast<uint64_t*>(cex + 3 * GC_CE);  // stage converted (GP_NS)
  uint64_t* mempty = mfull + GP_NS;  // stage MMAs done (GP_NS)
  uint64_t* maccf = mempty + GP_NS;  // chunk accumulators complete (2)
  uint64_t* macce = maccf + 2;       // chunk accumulators folded (2)
  uint64_t* mraw = macce + 2;        // raw chunk arrived (nraw)
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mraw + GC_MAXRAW);
  const int cbase = nchunks / (int)gridDim.x, crem = nchunks % (int)gridDim.x;
  const int nch = cbase + ((int)blockIdx.x < crem ? 1 : 0);
  const int cfirst = (int)blockIdx.x * cbase + min((int)blockIdx.x, crem);

  if (warp == 0) gcge::tc::tmem_alloc(tslot, ncols);
  if (tid == 0) {
    for (int b = 0; b < GP_NS; b++) {
      gcge::tc::mbar_init(&mfull[b], GP_CW);
      gcge::tc::mbar_init(&mempty[b], 1);
    }
    for (int b = 0; b < 2; b++) {
      gcge::tc::mbar_init(&maccf[b], 1);
      gcge::tc::mbar_init(&macce[b], GP_FW);
    }
    for (int b = 0; b < nraw; b++) gcge::tc::mbar_init(&mraw[b], 1);
  }
  // operand rows past the block's columns (V columns mi .. TC_M - 1, W
  // columns nj .. GC_N - 1) are never converted: they stay zero
  for (int e = tid; e < GP_NS * GC_SB / 16; e += GP_THREADS)
    reinterpret_cast<uint4*>(base)[e] = make_uint4(0u, 0u, 0u, 0u);
  gcge::tc::fence_proxy_async();
  gcge::tc::fence_before();
  __syncthreads();
  gcge::tc::fence_after();
  const uint32_t tmem = *tslot;
  bool ok = true;

  // fold threads: outputs (i, 8 jh + u), u < 8, in registers
  const int fw = warp - 1 - GP_CW;
  const int q4 = warp & 3, jh = fw >> 2;  // lane quadrant, W column half
  const int fi = 32 * q4 + lane;
  double rS[8];
  long long rT[8];
  int rE[8];
#pragma unroll
  for (int u = 0; u < 8; u++) {
    rS[u] = 0.0;
    rT[u] = 0;
    rE[u] = -1000000;
  }

  if (warp == 0) {
    // ------------------------------------------------ copy + MMA thread
    if (lane == 0) {
      // chunk cc of this CTA's run into raw buffer cc % nraw
      auto issue_raw = [&](int cc) {
        const int chunk = cfirst + cc;
        uint64_t* mb = &mraw[cc % nraw];
        uint8_t* dst = rawbase + (cc % nraw) * RC;
        gcge::tc::mbar_arrive_expect_tx(mb, (uint32_t)RC);
        gcge::tc::bulk_g2s(dst, vpl + ((size_t)chunk * ldv + voff + i0) * PL_REC, (uint32_t)VB,
                           mb);
        gcge::tc::bulk_g2s(dst + VB, wpl + ((size_t)chunk * ldw + woff + j0) * PL_REC,
                           (uint32_t)(nj * PL_REC), mb);
      };
      for (int cc = 0; cc < nraw && cc < nch; cc++) issue_raw(cc);
      for (int c = 0; c < nch && ok; c++) {
        const int tb = c & 1;
        for (int st = 0; st < GC_ST; st++) {
          const int g = c * GC_ST + st, buf = g % GP_NS;
          if (!gcge::tc::mbar_wait(&mfull[buf], (g / GP_NS) & 1, TC_WAIT)) ok = false;
          // the accumulator set of this chunk was folded (chunk c - 2)
          if (st == 0 && c >= 2 && !gcge::tc::mbar_wait(&macce[tb], ((c >> 1) - 1) & 1, TC_WAIT))
            ok = false;
          if (!ok) break;
          gcge::tc::fence_after();
          uint8_t* As = base + buf * GC_SB;
          const uint32_t acc = tmem + (uint32_t)(tb * D8_NL * GC_N);
          if (st == 0)
            gp_issue<true>(acc, gcge::tc::smem_u32(As), gcge::tc::smem_u32(As + TC_ABYTES));
          else
            gp_issue<false>(acc, gcge::tc::smem_u32(As), gcge::tc::smem_u32(As + TC_ABYTES));
          gcge::tc::commit(&mempty[buf]);
          if (st == GC_ST - 1) {
            gcge::tc::commit(&maccf[tb]);
            // every converter is past this chunk's raw buffer: refill it
            if (c + nraw < nch) issue_raw(c + nraw);
          }
        }
      }
    }
    __syncwarp();
  } else if (warp <= GP_CW) {
    // ------------------------------------------------ converter warps
    const int ctid = tid - 32;
    const int nwq = 4 * nj, nvq = 4 * mi;
    for (int c = 0; c < nch; c++) {
      const int rb = c % nraw;
      const uint8_t* rbuf = rawbase + rb * RC;
      if (!gcge::tc::mbar_wait_warp(&mraw[rb], (c / nraw) & 1, TC_WAIT)) ok = false;
      if (!ok) break;
      int* ce = cex + (c % 3) * GC_CE;
      for (int i = ctid; i < mi + nj; i += GP_CW * 32) {
        const int e = *reinterpret_cast<const int*>(rbuf + i * PL_REC);
        ce[i < mi ? i : TC_M + i - mi] = e;
      }
      for (int st = 0; st < GC_ST; st++) {
        const int g = c * GC_ST + st, buf = g % GP_NS;
        // the buffer's previous use (stage g - GP_NS) has finished its MMAs
        if (g >= GP_NS &&
            !gcge::tc::mbar_wait_warp(&mempty[buf], ((g / GP_NS) - 1) & 1, TC_WAIT))
          ok = false;
        if (!ok) break;
        uint8_t* As = base + buf * GC_SB;
        uint8_t* Bs = As + TC_ABYTES;
        // operands in the 32-byte swizzled K-major layout: digit planes of
        // TC_M rows (A: V columns) and GC_N rows (B: W columns)
        for (int u = ctid; u < nwq + nvq; u += GP_CW * 32) {
          if (u < nwq) {
            const int col = u >> 2, q = u & 3;
            pl_quad(rbuf + VB + col * PL_REC, st, q, Bs + gcge::tc::sw32_off(col, 4 * q),
                    GC_N * 32);
          } else {
            const int vq = u - nwq, col = vq >> 2, q = vq & 3;
            pl_quad(rbuf + col * PL_REC, st, q, As + gcge::tc::sw32_off(col, 4 * q), TC_M * 32);
          }
        }
        gcge::tc::fence_proxy_async();
        __syncwarp();
        if (lane == 0) gcge::tc::mbar_arrive(&mfull[buf]);
      }
      if (!ok) break;
    }
  } else {
    // ------------------------------------------------ fold warps
    for (int c = 0; c < nch; c++) {
      const int tb = c & 1;
      if (!gcge::tc::mbar_wait_warp(&maccf[tb], (c >> 1) & 1, TC_WAIT)) ok = false;
      if (!ok) break;
      gcge::tc::fence_after();
      if (32 * q4 < mi && 8 * jh < nj) {
        const int* ce = cex + (c % 3) * GC_CE;
        const int ea = ce[fi];
        const uint32_t tacc = tmem + (uint32_t)(tb * D8_NL * GC_N) + ((uint32_t)(32 * q4) << 16);
#pragma unroll
        for (int h = 0; h < 4; h++) {
          const int c0 = 8 * jh + 2 * h;
          uint32_t acc[D8_NL][2];
#pragma unroll
          for (int l = 0; l < D8_NL; l++)
            gcge::tc::tmem_ld2(tacc + (uint32_t)(l * GC_N + c0), acc[l]);
          gcge::tc::tmem_wait_ld();
#pragma unroll
          for (int jj = 0; jj < 2; jj++) {
            const int j = c0 + jj, u = 2 * h + jj;
            if (fi >= mi || j >= nj) continue;
            const int eb = ce[TC_M + j];
            if (ea >= 4096 || eb >= 4096) {
              rS[u] = __longlong_as_double(0x7ff8000000000000ll);
            } else if (ea > -2000 && eb > -2000) {
              int lv[D8_NL];
#pragma unroll
              for (int l = 0; l < D8_NL; l++) lv[l] = __float2int_rn(__uint_as_float(acc[l][jj]));
              const int p0 = lv[0] * 256 + lv[1], p1 = lv[2] * 256 + lv[3];
              const int p2 = lv[4] * 256 + lv[5], p3 = lv[6] * 256 + lv[7];
              const long long T = ((long long)p0 << 26) + ((long long)p1 << 10) +
                                  (long long)((p2 + 32) >> 6) +
                                  (long long)((p3 + (1 << 21)) >> 22);
              const int E = ea + eb;
              const long long t = rT[u], r = t + T;
              if (rE[u] != E || ((t ^ r) & (T ^ r)) < 0) {
                gp_flush(rT[u], rE[u], rS[u]);
                rT[u] = T;
                rE[u] = E;
              } else {
                rT[u] = r;
              }
            }
          }
        }
      }
      gcge::tc::fence_before();
      __syncwarp();
      if (lane == 0) gcge::tc::mbar_arrive(&macce[tb]);
    }
  }
  const int anybad = __syncthreads_or(ok ? 0 : 1);
  if (anybad && tid == 0) atomicExch(&g_oz_tc_status, 1);
  if (warp > GP_CW && fi < mi) {
    double* out = partial + (size_t)blockIdx.x * k1 * k2;
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const int j = 8 * jh + u;
      if (j < nj) {
        gp_flush(rT[u], rE[u], rS[u]);
        out[(i0 + fi) + (size_t)(j0 + j) * k1] =
            anybad ? __longlong_as_double(0x7ff8000000000000ll) : rS[u];
      }
    }
  }
  gcge::tc::fence_before();
  __syncthreads();
  if (warp == 0) {
    gcge::tc::fence_after();
    gcge::tc::tmem_dealloc(tmem, ncols);
  }
}

int gram_pp_all(const uint8_t* vpl, int ldv, int voff, int k1, const uint8_t* wpl, int ldw,
                int woff, int k2, int n, double* partial, cudaStream_t st) {
  const int ntm = (k1 + GC_MI - 1) / GC_MI, ntn = (k2 + GC_N - 1) / GC_N;
  const int nchunks = (n + GC_K - 1) / GC_K;
  const int mi = k1 < GC_MI ? k1 : GC_MI, nj = k2 < GC_N ? k2 : GC_N;
  const int nraw = gp_nraw(mi, nj);
  const int nblk = nchunks < 152 ? nchunks : 152;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_gram_pp, cudaFuncAttributeMaxDynamicSharedMemorySize, GC_SMEM_CAP);
    attr = true;
  }
  k_gram_pp<<<dim3(nblk, ntm * ntn), GP_THREADS, gp_smem(mi, nj), st>>>(
      vpl, ldv, voff, k1, wpl, ldw, woff, k2, ntn, partial, nchunks, nraw);
  return nblk;
}

}  // namespace

size_t lincomb_oz_scratch_bytes(int k1, int k2) {
  const int kb = k1 < 128 ? (k1 > 0 ? k1 : 1) : 128;
  const int k1p = tc_round16(kb);
  const int k2p = (k2 + TC_NMAX - 1) / TC_NMAX * TC_NMAX;
  return (size_t)k2p * k1p * (D8_S * 2) + sizeof(int) * (size_t)(k2p + (k1 > 0 ? k1 : 1)) + 512;
}

// Y_j = beta Y_j + sum_i X_i C[i + j*ldc], FP64 accuracy on the tcgen05
// tensor cores.  scratch: lincomb_oz_scratch_bytes(k1, k2) bytes, 16-byte
// aligned.  balance: scale the columns of X by powers of two (and the rows of
// C inversely) first, for blocks whose columns differ widely in magnitude
// (the product is unchanged: the scaling is exact).  negate: use -C.  k1 >
// 128 runs in blocks of 128 rows of C, each added to Y in FP64.  Y must not
// alias X.
void lincomb_oz(const ColList<double>& X, int k1, const double* C, int ldc,
                const ColList<double>& Y, int k2, double beta, int n, void* scratch,
                cudaStream_t st, bool balance, bool negate) {
  if (k2 <= 0 || n <= 0) return;
  if (k1 <= 0) {
    lincomb_f64(X, 0, C, ldc, Y, k2, beta, n, st);
    return;
  }
  const int ntile = (k2 + TC_NMAX - 1) / TC_NMAX;
  const int k2pad = (ntile - 1) * TC_NMAX + tc_tile_n(k2, ntile - 1);
  const int kbmax = k1 < 128 ? k1 : 128;
  uint8_t* Cg = reinterpret_cast<uint8_t*>(scratch);
  int* texp = reinterpret_cast<int*>(
      Cg + (size_t)ntile * TC_NMAX * tc_round16(kbmax) * (D8_S * 2));
  int* xe = balance ? texp + ntile * TC_NMAX : nullptr;
  if (balance) {
    k_fill_int<<<(k1 + 127) / 128, 128, 0, st>>>(xe, -2000, k1);
    const int nb = (n + 255) / 256 < 64 ? (n + 255) / 256 : 64;
    k_oz_colexp<<<dim3(nb, k1), 256, 0, st>>>(X, k1, n, xe);
  }
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_lincomb_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)tc_lincomb_smem(TC_NMAX));
    attr = true;
  }
  const size_t smem = tc_lincomb_smem(tc_tile_n(k2, 0));
  for (int kb = 0; kb < k1; kb += 128) {
    const int kc = (k1 - kb) < 128 ? (k1 - kb) : 128;
    const int k1p = tc_round16(kc);
    ColList<double> Xb;
    for (int i = 0; i < kc; i++) Xb.p[i] = X.p[kb + i];
    const int* xeb = xe ? xe + kb : nullptr;
    k_d8_split_c<<<k2pad, 128, 0, st>>>(C + kb, ldc, kc, k2, k1p, xeb, negate ? 1 : 0, Cg, texp);
    k_lincomb_tc<<<dim3((n + TC_M - 1) / TC_M, ntile), TC_T, smem, st>>>(
        Xb, kc, k1p, Cg, texp, k2, Y, kb == 0 ? beta : 1.0, n, xeb);
  }
}

int oz_tc_status(bool reset) {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_oz_tc_status, sizeof(int)) != cudaSuccess) return -1;
  if (reset && v) {
    const int z = 0;
    cudaMemcpyToSymbol(g_oz_tc_status, &z, sizeof(int));
  }
  return v;
}

size_t gram_oz_partial_doubles(int k1, int k2) {
  return (size_t)304 * k1 * k2;
}

// G = V^T diag(wd) W (k1 x k2, ldg) through per-CTA partials (partial holds
// gram_oz_partial_doubles(k1, k2) doubles); sym: only the upper triangle is
// kept and mirrored.
void gram_oz(const ColList<double>& V, int k1, const ColList<double>& W, int k2, int n, double* G,
             int ldg, bool sym, double* partial, cudaStream_t st, const double* wdiag) {
  if (k1 <= 0 || k2 <= 0 || n <= 0) return;
  bool vec = ((uintptr_t)wdiag & 15) == 0;
  for (int i = 0; i < k1; i++) vec = vec && ((uintptr_t)V.p[i] & 15) == 0;
  for (int j = 0; j < k2; j++) vec = vec && ((uintptr_t)W.p[j] & 15) == 0;
  const int nblk = vec ? gram_tc_all<true>(V, k1, W, k2, n, wdiag, partial, st)
                       : gram_tc_all<false>(V, k1, W, k2, n, wdiag, partial, st);
  gram_reduce_partials(k1, k2, nblk, sym, partial, G, ldg, st);
}

size_t planes_bytes(int n, int ldp) {
  return (size_t)((n + PL_K - 1) / PL_K) * (size_t)ldp * PL_REC;
}

// Digit planes of the k columns of X into plane columns c0 .. c0 + k - 1 of a
// set of ldp columns.
void cut_planes(const ColList<double>& X, int k, int n, uint8_t* planes, int ldp, int c0,
                cudaStream_t st, const double* d) {
  if (k <= 0 || n <= 0) return;
  const int nchunks = (n + PL_K - 1) / PL_K;
  const int gx = (nchunks + 4 * PL_WARPS - 1) / (4 * PL_WARPS);
  k_cut_planes<<<dim3(gx, k), PL_WARPS * 32, 0, st>>>(X, d, n, nchunks, planes, ldp, c0);
}

// G = V^T W with V = plane columns voff .. voff + k1 - 1 of a set of ldv and
// W = plane columns woff .. woff + k2 - 1 of a set of ldw.
void gram_oz_planes(const uint8_t* vpl, int ldv, int voff, int k1, const uint8_t* wpl, int ldw,
                    int woff, int k2, int n, double* G, int ldg, double* partial,
                    cudaStream_t st) {
  if (k1 <= 0 || k2 <= 0 || n <= 0) return;
  const int nblk = gram_pp_all(vpl, ldv, voff, k1, wpl, ldw, woff, k2, n, partial, st);
  gram_reduce_partials(k1, k2, nblk, false, partial, G, ldg, st);
}

}  // namespace gcge
