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
#include "gcge_cuda_tc.cuh"

namespace gcge {
namespace {

constexpr int OZ_S = 8;           // slices per value
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

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
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
constexpr int TC_T = 256;
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
// stage ks (16 values of i) and digit a at (ks*7 + a) * N*32, then the
// K-major core-matrix image of N columns x 16 values.  Grid: one CTA per
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
    const size_t off = (size_t)(kk >> 3) * (N * 16) + (size_t)(jj >> 3) * 128 + (jj & 7) * 16 +
                       (kk & 7) * 2;
#pragma unroll
    for (int a = 0; a < D8_S; a++) {
      const unsigned short h = (unsigned short)(__float_as_uint(f[a]) >> 16);
      *reinterpret_cast<unsigned short*>(tile + (size_t)(ks * D8_S + a) * (N * 32) + off) = h;
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

// Y[:, j] = beta Y[:, j] + sum_i X[:, i] C[i][j] for k1 <= 128.  Grid:
// (row tiles of 128, output-column tiles of 64).  Dynamic shared memory:
// tc_lincomb_smem(N).
__global__ void __launch_bounds__(TC_T, 1)
    k_lincomb_tc(ColList<double> X, int k1, int k1p, const uint8_t* __restrict__ Cg,
                 const int* __restrict__ texp, int k2, ColList<double> Y, double beta, int n,
                 const int* __restrict__ xe) {
  extern __shared__ __align__(1024) uint8_t smtc[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nt = blockIdx.y, j0 = nt * TC_NMAX;
  const int N = tc_tile_n(k2, nt);
  const int BB = D8_S * N * 32;                           // B bytes per stage
  const int SB = (TC_ABYTES + BB + 1023) / 1024 * 1024;   // stage stride
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
  // row exponents: two threads per row, loads issued 16 at a time
  {
    const int rr = tid & (TC_M - 1), part = tid >> 7;
    const int r = r0 + rr;
    int e = -2000;
    if (r < n) {
      for (int i0 = part; i0 < k1; i0 += 32) {
        double v[16];
#pragma unroll
        for (int q = 0; q < 16; q++) {
          const int i = i0 + 2 * q;
          v[q] = (i < k1) ? __ldg(X.p[i] + r) : 0.0;
        }
#pragma unroll
        for (int q = 0; q < 16; q++) {
          const int i = i0 + 2 * q;
          if (i < k1) e = max(e, oz_exp_shift(v[q], -oz_bal(xe, i)));
        }
      }
    }
    atomicMax(&rexp[rr], e);
  }
  __syncthreads();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = gcge::tc::idesc_bf16(TC_M, N);

  // slicing role of this thread: row rr, 8 values k = 16 s + 8 kg + q
  const int rr = tid & (TC_M - 1), kg = tid >> 7;
  const int r = r0 + rr;
  const int myexp = rexp[rr];
  const int nks = k1p / TC_KS;
  bool ok = true;
  double vn[8];
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int i = 8 * kg + q;
    vn[q] = (r < n && i < k1) ? __ldg(X.p[i] + r) : 0.0;
  }
  for (int s = 0; s < nks; s++) {
    const int buf = s % TC_STAGES;
    double v[8];
#pragma unroll
    for (int q = 0; q < 8; q++) v[q] = vn[q];
    if (s + 1 < nks) {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int i = (s + 1) * TC_KS + 8 * kg + q;
        vn[q] = (r < n && i < k1) ? __ldg(X.p[i] + r) : 0.0;
      }
    }
    uint8_t* As = base + buf * SB;
    uint8_t* Bs = As + TC_ABYTES;
    if (s >= TC_STAGES) {
      // the MMAs of stage s - TC_STAGES read this buffer
      if (!gcge::tc::mbar_wait(&mbar[buf], ((s / TC_STAGES) - 1) & 1, TC_WAIT)) ok = false;
    }
    // digits of this thread's 8 values -> 7 x 16 bytes
    {
      float f[8][D8_S];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int i = s * TC_KS + 8 * kg + q;
        const int E = (myexp >= 4096) ? 4096 : myexp + ((i < k1) ? oz_bal(xe, i) : 0);
        d8_digits(myexp >= 4096 ? 0.0 : v[q], E, f[q]);
      }
      uint8_t* dst = As + kg * 2048 + (rr >> 3) * 128 + (rr & 7) * 16;
#pragma unroll
      for (int a = 0; a < D8_S; a++) {
        uint4 w;
        w.x = d8_pack(f[0][a], f[1][a]);
        w.y = d8_pack(f[2][a], f[3][a]);
        w.z = d8_pack(f[4][a], f[5][a]);
        w.w = d8_pack(f[6][a], f[7][a]);
        *reinterpret_cast<uint4*>(dst + a * (TC_M * TC_KS * 2)) = w;
      }
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
      const uint32_t abase = gcge::tc::smem_u32(As), bbase = gcge::tc::smem_u32(Bs);
#pragma unroll
      for (int L = 2; L <= D8_NL + 1; L++) {
#pragma unroll
        for (int a = 1; a <= D8_S; a++) {
          const int b = L - a;
          if (b < 1 || b > D8_S) continue;
          const uint64_t ad = gcge::tc::smem_desc(abase + (a - 1) * (TC_M * TC_KS * 2), 2048, 128);
          const uint64_t bd = gcge::tc::smem_desc(bbase + (b - 1) * (N * 32), N * 16, 128);
          const uint32_t accum = (s > 0 || a != (L - D8_S > 1 ? L - D8_S : 1)) ? 1u : 0u;
          gcge::tc::mma_bf16(tmem + (uint32_t)((L - 2) * N), ad, bd, idesc, accum);
        }
      }
      gcge::tc::commit(&mbar[buf]);
    }
  }
  // wait for the last stage (its commit covers every earlier MMA)
  {
    const int s = nks - 1;
    if (!gcge::tc::mbar_wait(&mbar[s % TC_STAGES], (s / TC_STAGES) & 1, TC_WAIT)) ok = false;
  }
  gcge::tc::fence_after();
  const int anybad = __syncthreads_or(ok ? 0 : 1);
  if (anybad) {
    if (tid == 0) atomicExch(&g_oz_tc_status, 1);
    d8_fill_nan(Y, j0, N, k2, n, r0);
  } else {
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31, column half w / 4
    const int q4 = warp & 3, h = warp >> 2;
    const int row = r0 + 32 * q4 + lane;
    const int re = rexp[32 * q4 + lane];
    const int half = N / 2;
    for (int c0 = h * half; c0 < (h + 1) * half; c0 += 8) {
      uint32_t acc[D8_NL][8];
#pragma unroll
      for (int l = 0; l < D8_NL; l++)
        gcge::tc::tmem_ld8(tmem + ((uint32_t)(32 * q4) << 16) + (uint32_t)(l * N + c0), acc[l]);
      gcge::tc::tmem_wait_ld();
#pragma unroll
      for (int jj = 0; jj < 8; jj++) {
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
