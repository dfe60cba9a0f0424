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
                         gcge::tc::idesc_bf16(TC_M, cnt * Nw), accum);
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
// G = V^T diag(wd) W (wd NULL: identity) with FP64 accuracy.  One CTA owns up
// to 128 columns of V (MMA M, TMEM lane = column of V) and up to 32 columns
// of W (MMA N) over a strided set of 128-row chunks.  In a chunk every column
// has one power-of-two scale (its largest |value| over the chunk, a W column
// taken with the diagonal applied), the 7 balanced base-256 digits of the
// lincomb are used, and the 8 level sums over the chunk's 128 rows are exact
// in FP32 tensor memory.  The column exponents of chunk c+1 are gathered
// while chunk c is sliced (its values are re-read from L2 one chunk later);
// with two accumulator sets in tensor memory, the fold of chunk c-1
// (tcgen05.ld -> 64-bit fixed point -> FP64 partial sum in shared memory)
// overlaps the MMAs of chunk c.  Each CTA writes its FP64 partial Gram; a
// second kernel adds the partials in a fixed order.
constexpr int GC_K = 128;            // rows per exact chunk
constexpr int GC_ST = GC_K / TC_KS;  // stages per chunk (8)
constexpr int GC_STAGES = 2;         // shared-memory stage buffers
constexpr int GC_NMAX = 32;          // W columns per CTA (MMA N)
constexpr int GC_CE = TC_M + GC_NMAX;

// width (MMA N) of W-column tile nt of the Gram
__host__ __device__ __forceinline__ int gc_tile_n(int k2, int nt) {
  const int rem = k2 - nt * GC_NMAX;
  return rem >= GC_NMAX ? GC_NMAX : tc_round16(rem);
}

__host__ __device__ __forceinline__ uint32_t tc_cols_pow2(int c) {
  uint32_t p = 32;
  while ((int)p < c) p <<= 1;
  return p;
}

__device__ __forceinline__ int d8_prod_exp(int ew, int eb) {
  if (ew >= 4096 || eb >= 4096) return 4096;
  if (ew <= -2000 || eb <= -2000) return -2000;
  return ew + eb;
}

// v[q] = p[r + q] for q < 4 (0 beyond n)
template <bool VEC>
__device__ __forceinline__ void gc_load4(const double* __restrict__ p, int r, int n, double* v) {
  if (VEC && r + 4 <= n) {
    const double2* p2 = reinterpret_cast<const double2*>(p + r);
    const double2 t0 = __ldg(p2), t1 = __ldg(p2 + 1);
    v[0] = t0.x;
    v[1] = t0.y;
    v[2] = t1.x;
    v[3] = t1.y;
  } else {
#pragma unroll
    for (int q = 0; q < 4; q++) v[q] = (r + q < n) ? __ldg(p + r + q) : 0.0;
  }
}

// A quad of the Gram tile: 4 consecutive rows of one column.  Per 16-row
// stage a tile of ncolt = mi + nj columns has 4 * ncolt quads; quad u covers
// half h = u & 1 of the core-matrix row of column col = (u >> 1) % ncolt in
// K slab g = (u >> 1) / ncolt, i.e. rows 8 g + 4 h .. +3 of the stage, so
// the two threads of a lane pair fill one 16-byte core-matrix row.
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

// largest exponent of the 4 values of a quad (W values with the diagonal)
template <bool VEC>
__device__ __forceinline__ int gc_quad_exp(const double* __restrict__ p,
                                           const double* __restrict__ wd, int r, int n) {
  int e = -2000;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    if (r + q >= n) break;
    const int ex = oz_exp_hi(ld_hi(p + r + q));
    e = max(e, wd ? d8_prod_exp(ex, oz_exp_hi(ld_hi(wd + r + q))) : ex);
  }
  return e;
}

// exponents of one 16-row stage of a chunk into ce (atomicMax)
template <bool VEC>
__device__ __forceinline__ void gc_stage_exp(const ColList<double>& V, int i0, int mi,
                                             const ColList<double>& W, int j0, int nj,
                                             const double* __restrict__ wd, int row0, int n,
                                             int* ce, int ufirst) {
  const int ncolt = mi + nj;
  for (int u = ufirst; u < 4 * ncolt; u += TC_T) {
    const GcQuad q = gc_quad(u, ncolt);
    const int r = row0 + q.roff;
    if (r >= n) continue;
    const bool isv = q.col < mi;
    const int e = isv ? gc_quad_exp<VEC>(V.p[i0 + q.col], nullptr, r, n)
                      : gc_quad_exp<VEC>(W.p[j0 + q.col - mi], wd, r, n);
    if (e > -2000) atomicMax(ce + (isv ? q.col : TC_M + q.col - mi), e);
  }
}

// Adds the exact chunk value held in tensor memory at tacc to output (i, j)
// (slot j * TC_M + i); warp w reads lanes 32 (w % 4).. and column quarter
// w / 4.  A chunk's levels combine into T = sum_L acc_L 2^{50-8L} (|T| <
// 2^55 for 128 rows) worth T 2^{ea+eb-48}.  While the chunk exponent ea+eb
// repeats, T is added to a 64-bit accumulator (exactly, until the sum would
// overflow); when it changes the accumulator is rounded to FP64 and added to
// gsum.  gexp holds the exponent of the accumulator (GC_NOEXP: empty).
constexpr int GC_NOEXP = -1000000;

__device__ __forceinline__ void gc_flush(long long* gT, int* gE, double* gs) {
  if (*gT != 0) *gs += d8_to_double(*gT, *gE - 48);
  *gT = 0;
  *gE = GC_NOEXP;
}

__device__ __forceinline__ void gc_fold(uint32_t tacc, int N, int mi, int nj,
                                        const int* __restrict__ ce, double* gsum, long long* gT,
                                        int* gE) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q4 = warp & 3, cg = warp >> 2;
  const int i = 32 * q4 + lane;
  const int ea = ce[i];
  const int quarter = N / 4;
  for (int c0 = cg * quarter; c0 < (cg + 1) * quarter; c0 += 4) {
    uint32_t acc[D8_NL][4];
#pragma unroll
    for (int l = 0; l < D8_NL; l++)
      gcge::tc::tmem_ld4(tacc + ((uint32_t)(32 * q4) << 16) + (uint32_t)(l * N + c0), acc[l]);
    gcge::tc::tmem_wait_ld();
#pragma unroll
    for (int jj = 0; jj < 4; jj++) {
      const int j = c0 + jj;
      if (i >= mi || j >= nj) continue;
      const int eb = ce[TC_M + j];
      const int o = j * TC_M + i;
      if (ea >= 4096 || eb >= 4096) {
        gsum[o] = __longlong_as_double(0x7ff8000000000000ll);
      } else if (ea > -2000 && eb > -2000) {
        long long T = 0;
#pragma unroll
        for (int l = 0; l < D8_NL; l++) {
          const long long v = (long long)__float2int_rn(__uint_as_float(acc[l][jj]));
          const int sh = 50 - 8 * (l + 2);
          T += sh >= 0 ? (v << sh) : ((v + (1ll << (-sh - 1))) >> (-sh));
        }
        const int E = ea + eb;
        long long t = gT[o];
        const long long r = t + T;
        if (gE[o] != E || ((t ^ r) & (T ^ r)) < 0) {
          gc_flush(gT + o, gE + o, gsum + o);
          gT[o] = T;
          gE[o] = E;
        } else {
          gT[o] = r;
        }
      }
    }
  }
  gcge::tc::fence_before();
}

size_t tc_gram_smem(int N) {
  const int SB = (TC_ABYTES + D8_S * N * 32 + 1023) / 1024 * 1024;
  size_t b = (size_t)GC_STAGES * SB + (size_t)TC_M * N * 20 + 3 * GC_CE * 4 + GC_STAGES * 8 + 16 +
             1024;
  // tensor memory: two CTAs per SM only when both fit in its 512 columns
  const int nbuf = N <= 32 ? 2 : 1;
  if (tc_cols_pow2(nbuf * D8_NL * N) > 256 && b < 118 * 1024) b = 118 * 1024;
  return b;
}

template <bool VEC>
__global__ void __launch_bounds__(TC_T, 2)
    k_gram_tc(ColList<double> V, int k1, ColList<double> W, int k2, int n, int ntn,
              const double* __restrict__ wd, double* __restrict__ partial, int nchunks) {
  extern __shared__ __align__(1024) uint8_t smgc[];
  const int tid = threadIdx.x;
  const int mt = blockIdx.y / ntn, nt = blockIdx.y % ntn;
  const int i0 = mt * TC_M, j0 = nt * GC_NMAX;
  const int mi = min(TC_M, k1 - i0), N = gc_tile_n(k2, nt), nj = min(N, k2 - j0);
  const int nbuf = N <= 32 ? 2 : 1;
  const uint32_t ncols = tc_cols_pow2(nbuf * D8_NL * N);
  const int BB = D8_S * N * 32;
  const int SB = (TC_ABYTES + BB + 1023) / 1024 * 1024;
  uint8_t* base = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smgc) + 1023) & ~(uintptr_t)1023);
  double* gsum = reinterpret_cast<double*>(base + GC_STAGES * SB);
  long long* gT = reinterpret_cast<long long*>(gsum + TC_M * N);
  int* gE = reinterpret_cast<int*>(gT + TC_M * N);
  int* cexp = gE + TC_M * N;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(cexp + 3 * GC_CE);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + GC_STAGES);
  const int nch = (nchunks - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
  const int ncolt = mi + nj;
  const int nquads = 4 * ncolt;

  if ((tid >> 5) == 0) gcge::tc::tmem_alloc(tslot, ncols);
  if (tid == 0)
    for (int s = 0; s < GC_STAGES; s++) gcge::tc::mbar_init(&mbar[s], 1);
  for (int e = tid; e < TC_M * N; e += TC_T) {
    gsum[e] = 0.0;
    gT[e] = 0;
    gE[e] = GC_NOEXP;
  }
  for (int e = tid; e < 3 * GC_CE; e += TC_T) cexp[e] = -2000;
  gcge::tc::fence_before();
  __syncthreads();
  gcge::tc::fence_after();
  const uint32_t tmem = *tslot;

  // exponents of the first chunk
  for (int st = 0; st < GC_ST; st++)
    gc_stage_exp<VEC>(V, i0, mi, W, j0, nj, wd, (int)blockIdx.x * GC_K + st * TC_KS, n, cexp,
                      tid);
  __syncthreads();

  // This thread's first quad runs through two register pipelines: the high
  // words for the exponents of global stage g + 9 are loaded during stage g
  // and folded into the exponent slots during stage g + 1 (so a chunk's
  // exponents are complete one stage before its slicing starts), and the
  // values of stage g + 1 are loaded during stage g.  Further quads of wide
  // tiles run synchronously.
  const bool has_u = tid < nquads;
  const GcQuad uq = gc_quad(has_u ? tid : 0, ncolt);
  const bool uisv = uq.col < mi;
  const double* up = has_u ? (uisv ? V.p[i0 + uq.col] : W.p[j0 + uq.col - mi]) : nullptr;
  const double* uwd = (has_u && !uisv) ? wd : nullptr;
  const int uslot = uisv ? uq.col : TC_M + uq.col - mi;
  auto stage_row = [&](int gs) {  // first row of this quad in global stage gs, -1 past the end
    const int c = gs / GC_ST;
    if (c >= nch) return -1;
    return ((int)blockIdx.x + c * (int)gridDim.x) * GC_K + (gs % GC_ST) * TC_KS + uq.roff;
  };
  int xh[4], wh[4];
  auto exp_issue = [&](int gs) {
    const int r = has_u ? stage_row(gs) : -1;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const bool in = r >= 0 && r + q < n;
      xh[q] = in ? ld_hi(up + r + q) : 0;
      wh[q] = (in && uwd) ? ld_hi(uwd + r + q) : 0x3FE00000;  // 0.5 (exponent 0) without
    }
  };
  // exponent of the quad from the raw 11-bit exponent fields: without the
  // diagonal the largest field decides; with it the largest sum of fields of
  // the nonzero products (a field of 0x7FF anywhere flags the quad non-finite)
  auto exp_consume = [&](int* ce) {
    int fmax = 0, bad = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int fx = (xh[q] >> 20) & 0x7FF, fw = (wh[q] >> 20) & 0x7FF;
      bad |= (fx == 0x7FF) | (fw == 0x7FF);
      // fw of 0.5 is 1022; a product at the bottom of the range still gets a field >= 1
      const int f = (fx == 0 || fw == 0) ? 0 : max(fx + fw - 1022, 1);
      fmax = max(fmax, f);
    }
    const int e = bad ? 4096 : (fmax == 0 ? -2000 : fmax - 1022);
    if (has_u && e > -2000) atomicMax(ce + uslot, e);
  };
  double sv[4];
  auto slice_issue = [&](int gs) {
    const int r = has_u ? stage_row(gs) : -1;
    if (r < 0) return;
    gc_load4<VEC>(up, r, n, sv);
    if (uwd) {
      double w[4];
      gc_load4<VEC>(uwd, r, n, w);
#pragma unroll
      for (int q = 0; q < 4; q++) sv[q] *= w[q];
    }
  };
  exp_issue(GC_ST);  // chunk 1, stage 0
  slice_issue(0);

  bool ok = true;
  for (int c = 0; c < nch; c++) {
    const int cb = (int)blockIdx.x + c * (int)gridDim.x;
    const int* ce = cexp + (c % 3) * GC_CE;
    int* ce_next = cexp + ((c + 1) % 3) * GC_CE;
    const uint32_t tacc = tmem + (uint32_t)((c % nbuf) * D8_NL * N);
    for (int st = 0; st < GC_ST; st++) {
      const int g = c * GC_ST + st;
      const int buf = g % GC_STAGES;
      // exponents of global stage g + 8 (chunk c + 1) -> slots; issue g + 9
      exp_consume(ce_next);
      exp_issue(g + GC_ST + 1);
      double v[4];
#pragma unroll
      for (int q = 0; q < 4; q++) v[q] = sv[q];
      slice_issue(g + 1);
      if (g >= GC_STAGES &&
          !gcge::tc::mbar_wait_warp(&mbar[buf], ((g / GC_STAGES) - 1) & 1, TC_WAIT))
        ok = false;
      if (c > 0 && nbuf == 1 && st == 0) {
        // one accumulator set: fold chunk c-1 before this chunk's first MMA
        const int gl = g - 1;
        if (!gcge::tc::mbar_wait_warp(&mbar[gl % GC_STAGES], (gl / GC_STAGES) & 1, TC_WAIT))
          ok = false;
        gcge::tc::fence_after();
        gc_fold(tmem, N, mi, nj, cexp + ((c - 1) % 3) * GC_CE, gsum, gT, gE);
      } else if (c > 0 && nbuf == 2 && st == GC_STAGES - 1) {
        // the wait above covered the last stage of chunk c-1
        gcge::tc::fence_after();
        gc_fold(tmem + (uint32_t)(((c - 1) % 2) * D8_NL * N), N, mi, nj,
                cexp + ((c - 1) % 3) * GC_CE, gsum, gT, gE);
      }
      uint8_t* As = base + buf * SB;
      uint8_t* Bs = As + TC_ABYTES;
      const int row0 = cb * GC_K + st * TC_KS;
      for (int u = tid; u < nquads; u += TC_T) {
        const GcQuad q = (u == tid) ? uq : gc_quad(u, ncolt);
        const int r = row0 + q.roff;
        const bool isv = q.col < mi;
        if (u != tid) {  // a further quad: load now
          if (isv) {
            gc_load4<VEC>(V.p[i0 + q.col], r, n, v);
          } else {
            gc_load4<VEC>(W.p[j0 + q.col - mi], r, n, v);
            if (wd) {
              double w[4];
              gc_load4<VEC>(wd, r, n, w);
#pragma unroll
              for (int t = 0; t < 4; t++) v[t] *= w[t];
            }
          }
        }
        const int E0 = ce[isv ? q.col : TC_M + q.col - mi];
        int E[4];
#pragma unroll
        for (int t = 0; t < 4; t++) {
          E[t] = E0;
          if (E0 >= 4096) v[t] = 0.0;
        }
        const int cc = isv ? q.col : q.col - mi;
        uint8_t* dst = (isv ? As + q.g * (TC_M / 8 * 128) : Bs + q.g * (D8_S * N * 16)) +
                       (cc >> 3) * 128 + (cc & 7) * 16 + q.h * 8;
        d8_slice4(v, E, dst, isv ? TC_M * TC_KS * 2 : N * 16);
      }
      // further quads: exponents of chunk c + 1 now
      if (c + 1 < nch && nquads > TC_T)
        gc_stage_exp<VEC>(V, i0, mi, W, j0, nj, wd, (cb + (int)gridDim.x) * GC_K + st * TC_KS, n,
                          ce_next, tid + TC_T);
      if (st == GC_ST - 1)  // slots of chunk c+2 (last read by the fold of chunk c-1)
        for (int e = tid; e < GC_CE; e += TC_T) cexp[((c + 2) % 3) * GC_CE + e] = -2000;
      gcge::tc::fence_proxy_async();
      __syncthreads();
      if (tid == 0) {
        gcge::tc::fence_after();
        d8_issue(tacc, gcge::tc::smem_u32(As), TC_M * TC_KS * 2, gcge::tc::smem_u32(Bs), N,
                 st == 0);
        gcge::tc::commit(&mbar[buf]);
      }
    }
  }
  if (nch > 0) {
    const int gl = nch * GC_ST - 1;
    if (!gcge::tc::mbar_wait_warp(&mbar[gl % GC_STAGES], (gl / GC_STAGES) & 1, TC_WAIT))
      ok = false;
    gcge::tc::fence_after();
    gc_fold(tmem + (uint32_t)(((nch - 1) % nbuf) * D8_NL * N), N, mi, nj,
            cexp + ((nch - 1) % 3) * GC_CE, gsum, gT, gE);
  }
  __syncthreads();
  for (int e = tid; e < TC_M * N; e += TC_T) gc_flush(gT + e, gE + e, gsum + e);
  const int anybad = __syncthreads_or(ok ? 0 : 1);
  if (anybad && tid == 0) atomicExch(&g_oz_tc_status, 1);
  // partial layout [block][o], o = i + j*k1 (the flex-Gram reduction layout)
  double* out = partial + (size_t)blockIdx.x * k1 * k2;
  for (int e = tid; e < mi * nj; e += TC_T) {
    const int ii = e % mi, jj = e / mi;
    out[(i0 + ii) + (size_t)(j0 + jj) * k1] =
        anybad ? __longlong_as_double(0x7ff8000000000000ll) : gsum[(size_t)jj * TC_M + ii];
  }
  gcge::tc::fence_before();
  __syncthreads();
  if ((tid >> 5) == 0) {
    gcge::tc::fence_after();
    gcge::tc::tmem_dealloc(tmem, ncols);
  }
}

template <bool VEC>
int launch_gram_tc(const ColList<double>& V, int k1, const ColList<double>& W, int k2, int n,
                   const double* wd, double* partial, cudaStream_t st) {
  const int ntm = (k1 + TC_M - 1) / TC_M, ntn = (k2 + GC_NMAX - 1) / GC_NMAX;
  const int nchunks = (n + GC_K - 1) / GC_K;
  const int N0 = gc_tile_n(k2, 0);
  const size_t sm = tc_gram_smem(N0);
  const int per_sm = (227 * 1024) / (int)(sm + 1024) >= 2 ? 2 : 1;
  const int nblk = nchunks < 152 * per_sm ? nchunks : 152 * per_sm;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_gram_tc<VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)tc_gram_smem(GC_NMAX));
    attr = true;
  }
  k_gram_tc<VEC><<<dim3(nblk, ntm * ntn), TC_T, sm, st>>>(V, k1, W, k2, n, ntn, wd, partial,
                                                          nchunks);
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
  const int nblk = vec ? launch_gram_tc<true>(V, k1, W, k2, n, wdiag, partial, st)
                       : launch_gram_tc<false>(V, k1, W, k2, n, wdiag, partial, st);
  gram_reduce_partials(k1, k2, nblk, sym, partial, G, ldg, st);
}

}  // namespace gcge
