// GCGE_CUDA_AMG: a smoothed-aggregation algebraic multigrid hierarchy built
// on the GPU, and GCGE_CUDA_AMGPCG, the W-step solver that uses it.
//
// The reference hands the W step to hypre's BoomerAMG-preconditioned solvers
// through the MultiLinearSolver hook (app/hypre/gcge_app_hypre.c:305-331,
// called at src/gcge_xpw.c:178-191), and its multilevel eigensolver builds
// its level matrices A_l, B_l = P^T B_{l-1} P and prolongations P from a
// BoomerAMG hierarchy (pase/src/pase_mg.c:101-131).  hypre is a third-party
// library the reference links but does not contain; this file is an AMG of its
// own design for one GPU, not a restatement of BoomerAMG:
//
//   set-up (once per matrix, all on the device; the host only sequences the
//   kernels and reads sizes):
//   * strength graph: the off-diagonal entries with |a_ij| >= theta
//     sqrt(|a_ii a_jj|) (theta = 0: every stored off-diagonal entry);
//   * aggregation: a distance-2 maximal independent set of the strength graph
//     by iterated two-hop max-propagation of (state, hash, index) tuples
//     (Bell, Dalton & Olson, SIAM J. Sci. Comput. 34 (2012)); every root
//     starts an aggregate, the other rows join the neighbouring root with the
//     largest tuple, then (second pass) the neighbour aggregated in the first
//     pass with the largest tuple;
//   * prolongation: tentative T (T_{i, agg(i)} = 1) smoothed by one damped
//     Jacobi step, P = (I - omega D^-1 A) T, omega = 4 / (3 lambda_max(D^-1 A))
//     (Vanek, Mandel & Brezina, Computing 56 (1996)); rows longer than
//     kSmoothRowMax entries keep their tentative row;
//   * restriction R = P^T (counting transpose, rows sorted by column);
//   * Galerkin operator A_c = R A P, one coarse row per CTA: the products
//     r_ai a_ij p_jb accumulate in an open-addressing hash table in shared
//     memory (rows with more distinct columns than it holds go to tables in
//     global memory), each row is written sorted by column;
//   * lambda_max(D^-1 A) per level by power iteration (x 1.1);
//   * coarsest level (at most kCoarseMax rows): its dense inverse by
//     Gauss-Jordan elimination on the device.
//
//   solve phase (FP32, row-interleaved n x KW blocks as the mixed block CG
//   uses, so every SpMM gather reads one contiguous row):
//   * V-cycle: Chebyshev smoothing in D^-1 A of degree `cheb_degree` on
//     [lambda_max / cheb_ratio, lambda_max] before and after the coarse
//     correction (the same polynomial both times, so the cycle is symmetric),
//     residual, restriction, recursion, prolongation; the dense inverse at
//     the bottom;
//   * AMG-PCG: per column CG preconditioned by one V-cycle, a column frozen
//     once ||r|| < pcg_rate ||r_0|| or after pcg_max_it steps (the block CG's
//     stopping rule, src/gcge_cg.c:488); step scalars on the device, inner
//     products reduced in a fixed order, the host reads the active count every
//     kCheck steps.  The residual of the FP64 start is formed in FP64, the FP32
//     correction is added to the FP64 columns at the end.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/gcge_cuda.h"
#include "gcge_cuda_amg.cuh"
#include "gcge_cuda_bcg.cuh"
#include "gcge_cuda_common.cuh"

int gcge_record_error(int code, const char* msg);

namespace {

constexpr int kT = 256;
constexpr int kMaxLevels = 16;
constexpr int kCoarseMax = 512;      // dense-inverse limit of the coarsest level
constexpr int kSmoothRowMax = 256;   // longer rows keep the tentative prolongation row
constexpr int kHashCap = 4096;       // shared hash table of the Galerkin product
constexpr int kHashFill = kHashCap / 2;
constexpr int kSortMax = 2048;       // rows sorted by column up to this length
constexpr int kCheck = 4;            // AMG-PCG steps between host reads
constexpr int kRedBlocks = 2 * 152;  // row blocks of the PCG reductions
// resident 256-thread CTAs per SM for the row-gather kernels of width KW that
// fit the cap without spills (the Chebyshev step and the PCG's A p spill under
// it and ran slower: no cap there)
template <int KW>
constexpr int row_blocks_per_sm() { return KW <= 12 ? 6 : (KW <= 20 ? 4 : 2); }

std::mutex g_amg_mu;

#define AMG_CU(call)                                                                    \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      char b_[256];                                                                     \
      snprintf(b_, sizeof b_, "AMG: %s (%s:%d)", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return gcge_record_error(GCGE_CUDA_ERR_CUDA, b_);                                 \
    }                                                                                   \
  } while (0)

#define AMG_CHK(expr)           \
  do {                          \
    const int rc_ = (expr);     \
    if (rc_ != GCGE_CUDA_OK) return rc_; \
  } while (0)

// ------------------------------------------------------------------ small kernels
__device__ __forceinline__ uint32_t amg_hash(uint32_t x) {
  // integer finaliser with good avalanche (Wellons' "lowbias32")
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

// exclusive scan of a[0..len) in place, 2048 entries per CTA (512 threads x 4)
__global__ void k_scan_block(int* a, int len, int* sums) {
  __shared__ int sh[512];
  const int tid = threadIdx.x;
  const long long base = (long long)blockIdx.x * 2048 + tid * 4;
  int v[4];
#pragma unroll
  for (int q = 0; q < 4; q++) v[q] = base + q < len ? a[base + q] : 0;
  const int tot = v[0] + v[1] + v[2] + v[3];
  sh[tid] = tot;
  __syncthreads();
  for (int o = 1; o < 512; o <<= 1) {
    const int t = tid >= o ? sh[tid - o] : 0;
    __syncthreads();
    sh[tid] += t;
    __syncthreads();
  }
  int run = sh[tid] - tot;  // exclusive offset of this thread
#pragma unroll
  for (int q = 0; q < 4; q++) {
    if (base + q < len) a[base + q] = run;
    run += v[q];
  }
  if (tid == 511) sums[blockIdx.x] = sh[511];
}

__global__ void k_scan_add(int* a, int len, const int* sums) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < len) a[i] += sums[i / 2048];
}

int scan_excl(int* a, int len, cudaStream_t st) {
  const int nb = (len + 2047) / 2048;
  int* sums = nullptr;
  AMG_CU(cudaMallocAsync(&sums, sizeof(int) * (nb + 1), st));
  k_scan_block<<<nb, 512, 0, st>>>(a, len, sums);
  if (nb > 1) {
    const int rc = scan_excl(sums, nb, st);
    if (rc != GCGE_CUDA_OK) {
      cudaFreeAsync(sums, st);
      return rc;
    }
    k_scan_add<<<(len + 255) / 256, 256, 0, st>>>(a, len, sums);
  }
  AMG_CU(cudaGetLastError());
  AMG_CU(cudaFreeAsync(sums, st));
  return GCGE_CUDA_OK;
}

// counts c[0..n) -> row pointers rp[0..n] (rp may be c's storage of n + 1)
int counts_to_rowptr(int* rp, int n, int* total, cudaStream_t st) {
  AMG_CU(cudaMemsetAsync(rp + n, 0, sizeof(int), st));
  AMG_CHK(scan_excl(rp, n + 1, st));
  AMG_CU(cudaMemcpyAsync(total, rp + n, sizeof(int), cudaMemcpyDeviceToHost, st));
  AMG_CU(cudaStreamSynchronize(st));
  return GCGE_CUDA_OK;
}

// ------------------------------------------------------------------ level data
struct Mat {  // device CSR (rows x cols), FP64 values and their FP32 copy
  int rows = 0, cols = 0, nnz = 0;
  int* rp = nullptr;
  int* ci = nullptr;
  double* v = nullptr;
  float* v32 = nullptr;
  void release() {
    cudaFree(rp);
    cudaFree(ci);
    cudaFree(v);
    cudaFree(v32);
    rp = ci = nullptr;
    v = nullptr;
    v32 = nullptr;
    rows = cols = nnz = 0;
  }
};

struct Level {
  Mat A;                 // level operator (level 0: a view of the caller's matrix + own v32)
  bool own_A = false;    // level 0 borrows rp / ci / v
  const GcgeDevCsr* heavy = nullptr;  // level 0: the caller's heavy-row chunks
  Mat P, R;              // prolongation (rows x next rows) and restriction P^T
  int* agg = nullptr;    // aggregate of each row
  float* dinv = nullptr; // 1 / a_ii
  double lmax = 0.0;     // lambda_max(D^-1 A) estimate (x 1.1)
  // work blocks, rows x kw floats each
  float *x = nullptr, *b = nullptr, *r = nullptr, *d0 = nullptr, *d1 = nullptr;
};

}  // namespace

struct GCGE_CUDA_AMG_ {
  GCGE_CUDA_AMG_PARAM prm;
  int nlev = 0;
  Level lev[kMaxLevels];
  float* cinv = nullptr;   // dense inverse of the coarsest operator (FP32, row-major)
  int kw = 0;              // width of the allocated work blocks
  // AMG-PCG state
  float *pr = nullptr, *px = nullptr, *pp = nullptr, *pw = nullptr;  // n x kw
  double* tmp64 = nullptr;     // k x n FP64 columns (A x0)
  size_t tmp64_len = 0;
  double* red = nullptr;       // kRedBlocks x 32 partials + scalars
  int* flags = nullptr;        // active flags (32) + nonzero flag
  int* host_cnt = nullptr;     // mapped pinned: active count per check slot
  int* dev_cnt = nullptr;      // its device alias
  int last_steps = 0;
};

namespace {

// ------------------------------------------------------------------ set-up kernels
__global__ void k_diag(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                       const double* __restrict__ v, double* __restrict__ dg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double d = 0.0;
  for (int e = rp[i]; e < rp[i + 1]; e++)
    if (ci[e] == i) d += v[e];
  dg[i] = d;
}

__global__ void k_dinv32(int n, const double* __restrict__ dg, float* __restrict__ dinv, int* bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double d = dg[i];
  if (!(d > 0.0)) atomicExch(bad, 1);
  dinv[i] = d > 0.0 ? (float)(1.0 / d) : 0.f;
}

// strength-graph row lengths (fill = 0) or entries (fill = 1)
__global__ void k_strength(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                           const double* __restrict__ v, const double* __restrict__ dg,
                           double theta, int* __restrict__ cnt, const int* __restrict__ srp,
                           int* __restrict__ sci, int fill) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = 0;
  const double di = fabs(dg[i]);
  int o = fill ? srp[i] : 0;
  for (int e = rp[i]; e < rp[i + 1]; e++) {
    const int j = ci[e];
    if (j == i || v[e] == 0.0) continue;
    if (theta > 0.0 && !(fabs(v[e]) >= theta * sqrt(di * fabs(dg[j])))) continue;
    if (fill)
      sci[o++] = j;
    else
      c++;
  }
  if (!fill) cnt[i] = c;
}

// MIS-2 tuples: state (0 out, 1 undecided, 2 in) in bits 62-63, a hash in
// bits 32-61, the row in bits 0-31
__device__ __forceinline__ unsigned long long mis_tuple(int state, int i) {
  return ((unsigned long long)state << 62) |
         ((unsigned long long)(amg_hash((uint32_t)i) & 0x3FFFFFFFu) << 32) | (uint32_t)i;
}

__global__ void k_mis_init(int n, int* __restrict__ state, unsigned long long* __restrict__ t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  state[i] = 1;
  t[i] = mis_tuple(1, i);
}

// out_i = max of in over the closed neighbourhood of i
__global__ void k_mis_max(int n, const int* __restrict__ srp, const int* __restrict__ sci,
                          const unsigned long long* __restrict__ in,
                          unsigned long long* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned long long m = in[i];
  for (int e = srp[i]; e < srp[i + 1]; e++) {
    const unsigned long long u = in[sci[e]];
    m = u > m ? u : m;
  }
  out[i] = m;
}

__global__ void k_mis_decide(int n, int* __restrict__ state, unsigned long long* __restrict__ t,
                             const unsigned long long* __restrict__ t2, int* __restrict__ undecided) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || state[i] != 1) return;
  const unsigned long long m = t2[i];
  if (m == t[i]) {
    state[i] = 2;
    t[i] = mis_tuple(2, i);
  } else if ((m >> 62) == 2) {
    state[i] = 0;
    t[i] = mis_tuple(0, i);
  } else {
    atomicAdd(undecided, 1);
  }
}

__global__ void k_root_flags(int n, const int* __restrict__ state, int* __restrict__ f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) f[i] = state[i] == 2 ? 1 : 0;
}

// roots take their aggregate number; others -1
__global__ void k_agg_roots(int n, const int* __restrict__ state, const int* __restrict__ num,
                            int* __restrict__ agg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) agg[i] = state[i] == 2 ? num[i] : -1;
}

// pass 1 (from = roots' numbers) / pass 2 (from = a copy after pass 1): an
// unaggregated row joins the aggregate of the neighbour with the largest
// MIS tuple among the neighbours aggregated in `from`
__global__ void k_agg_join(int n, const int* __restrict__ srp, const int* __restrict__ sci,
                           const int* __restrict__ from, int* __restrict__ agg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || from[i] >= 0) return;
  unsigned long long best = 0;
  int a = -1;
  for (int e = srp[i]; e < srp[i + 1]; e++) {
    const int j = sci[e];
    const int aj = from[j];
    if (aj < 0) continue;
    const unsigned long long tj = mis_tuple(1, j);
    if (a < 0 || tj > best) {
      best = tj;
      a = aj;
    }
  }
  if (a >= 0) agg[i] = a;
}

__global__ void k_left_flags(int n, const int* __restrict__ agg, int* __restrict__ f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) f[i] = agg[i] < 0 ? 1 : 0;
}

__global__ void k_left_assign(int n, const int* __restrict__ num, int base, int* __restrict__ agg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && agg[i] < 0) agg[i] = base + num[i];
}

// smoothed prolongation row i: P_{i,a} = [agg(i) = a] - omega/a_ii sum_{j: agg(j) = a} a_ij
// (first-occurrence column order); count (fill = 0) or write (fill = 1)
__global__ void k_prolong(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                          const double* __restrict__ v, const double* __restrict__ dg,
                          const int* __restrict__ agg, double omega, int smooth,
                          int* __restrict__ cnt, const int* __restrict__ prp,
                          int* __restrict__ pci, double* __restrict__ pv, int fill) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int b = rp[i], e = rp[i + 1];
  const int ai = agg[i];
  if (!smooth || e - b > kSmoothRowMax || !(dg[i] > 0.0)) {
    if (fill) {
      pci[prp[i]] = ai;
      pv[prp[i]] = 1.0;
    } else {
      cnt[i] = 1;
    }
    return;
  }
  const double s = omega / dg[i];
  int o = fill ? prp[i] : 0;
  int c = 0;
  // the row's own aggregate first (always present), then the others in
  // first-occurrence order; duplicates are summed into the first occurrence
  for (int pass = 0; pass < 2; pass++) {
    for (int q = b; q < e; q++) {
      const int a = agg[ci[q]];
      if ((pass == 0) != (a == ai)) continue;
      bool seen = false;
      if (pass == 1)
        for (int t = b; t < q && !seen; t++) seen = agg[ci[t]] == a;
      if (pass == 0 && c > 0) seen = true;
      if (seen) continue;
      c++;
      if (fill) {
        double sum = 0.0;
        for (int t = q; t < e; t++)
          if (agg[ci[t]] == a) sum += v[t];
        pci[o] = a;
        pv[o] = (a == ai ? 1.0 : 0.0) - s * sum;
        o++;
      }
    }
    if (pass == 0 && c == 0) {
      // no entry of the row in its own aggregate (zero row): keep T's entry
      c = 1;
      if (fill) {
        pci[o] = ai;
        pv[o] = 1.0;
        o++;
      }
    }
  }
  if (!fill) cnt[i] = c;
}

// transpose: column counts, then scatter (rows of the transpose unordered)
__global__ void k_colcount(int nnz, const int* __restrict__ ci, int* __restrict__ cnt) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nnz) atomicAdd(cnt + ci[e], 1);
}

__global__ void k_transpose_fill(int rows, const int* __restrict__ rp, const int* __restrict__ ci,
                                 const double* __restrict__ v, const int* __restrict__ trp,
                                 int* __restrict__ cur, int* __restrict__ tci,
                                 double* __restrict__ tv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows) return;
  for (int e = rp[i]; e < rp[i + 1]; e++) {
    const int c = ci[e];
    const int pos = trp[c] + atomicAdd(cur + c, 1);
    tci[pos] = i;
    tv[pos] = v[e];
  }
}

// rows sorted by column into (ci2, v2), one warp per row: an entry's place is
// the number of smaller columns in its row (the columns of a row are
// distinct, so the order is canonical and the result deterministic); rows of
// more than kSortMax entries are copied as they are
__global__ void k_rank_rows(int rows, const int* __restrict__ rp, const int* __restrict__ ci,
                            const double* __restrict__ v, int* __restrict__ ci2,
                            double* __restrict__ v2) {
  const int w = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= rows) return;
  const int b = rp[w], e = rp[w + 1];
  if (e - b > kSortMax) {
    // a very long row (a hub of a power-law graph): kept in fill order, since
    // ranking by counting is quadratic in the row length
    for (int p = b + lane; p < e; p += 32) {
      ci2[p] = ci[p];
      v2[p] = v[p];
    }
    return;
  }
  for (int p = b + lane; p < e; p += 32) {
    const int key = ci[p];
    int rk = 0;
    for (int t = b; t < e; t++) rk += ci[t] < key;
    ci2[b + rk] = key;
    v2[b + rk] = v[p];
  }
}

// Galerkin product, one coarse row per CTA: keys / vals is an open-addressing
// table of cap slots (shared memory, or a row's own slice of a global buffer).
// Symbolic (NUM = false): cnt[row] = distinct columns, or -1 past kHashFill
// (shared table) ; bound[row] = number of products.  Numeric: the row's
// entries into cci / cv at crp[row], sorted by column when <= kSortMax.
__device__ __forceinline__ uint32_t slot_of(int key, int cap) {
  return (amg_hash((uint32_t)key)) & (uint32_t)(cap - 1);
}

template <bool NUM>
__global__ void __launch_bounds__(kT) k_rap(const int* __restrict__ rows_list, int nrows_list,
                                            const int* __restrict__ rrp, const int* __restrict__ rci,
                                            const double* __restrict__ rv,
                                            const int* __restrict__ arp, const int* __restrict__ aci,
                                            const double* __restrict__ av,
                                            const int* __restrict__ prp, const int* __restrict__ pci,
                                            const double* __restrict__ pv, int cap,
                                            int* gkeys, double* gvals, const long long* goff,
                                            int* __restrict__ cnt, long long* __restrict__ bound,
                                            const int* __restrict__ crp, int* __restrict__ cci,
                                            double* __restrict__ cv) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int li = blockIdx.x;
  if (li >= nrows_list) return;
  const int row = rows_list ? rows_list[li] : li;
  const bool global = gkeys != nullptr;
  int* keys;
  double* vals;
  if (global) {
    keys = gkeys + goff[li];
    vals = gvals ? gvals + goff[li] : nullptr;
  } else {
    vals = reinterpret_cast<double*>(smem);
    keys = reinterpret_cast<int*>(smem + (NUM ? sizeof(double) * cap : 0));
  }
  __shared__ int s_count, s_over;
  __shared__ long long s_bound;
  if (threadIdx.x == 0) {
    s_count = 0;
    s_over = 0;
    s_bound = 0;
  }
  if (!global) {
    for (int h = threadIdx.x; h < cap; h += kT) {
      keys[h] = -1;
      if (NUM) vals[h] = 0.0;
    }
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  long long nb = 0;
  for (int q = rrp[row] + warp; q < rrp[row + 1]; q += kT / 32) {
    const int i = rci[q];
    const double ri = NUM ? rv[q] : 0.0;
    for (int e = arp[i] + lane; e < arp[i + 1]; e += 32) {
      const int j = aci[e];
      const double ra = NUM ? ri * av[e] : 0.0;
      for (int f = prp[j]; f < prp[j + 1]; f++) {
        const int key = pci[f];
        nb++;
        if (!NUM && s_over) continue;
        uint32_t h = slot_of(key, cap);
        int probes = 0;
        while (true) {
          const int k = keys[h];
          if (k == key) break;
          if (k == -1) {
            const int old = atomicCAS(&keys[h], -1, key);
            if (old == -1) {
              if (!NUM) {
                const int c = atomicAdd(&s_count, 1);
                if (!global && c + 1 > kHashFill) s_over = 1;
              }
              break;
            }
            if (old == key) break;
          }
          h = (h + 1) & (uint32_t)(cap - 1);
          if (++probes >= cap) {  // table full: cannot happen within the fill bounds
            s_over = 1;
            break;
          }
        }
        if (NUM && probes < cap) atomicAdd(&vals[h], ra * pv[f]);
      }
    }
  }
  if (!NUM) atomicAdd((unsigned long long*)&s_bound, (unsigned long long)nb);
  __syncthreads();
  if (!NUM) {
    if (threadIdx.x == 0) {
      cnt[row] = s_over ? -1 : s_count;
      bound[row] = s_bound;
    }
    return;
  }
  // compaction in slot order, then (short rows) a rank sort by column
  __shared__ int s_pos;
  if (threadIdx.x == 0) s_pos = 0;
  __syncthreads();
  const int base = crp[row];
  const int m = crp[row + 1] - base;
  for (int h = threadIdx.x; h < cap; h += kT) {
    const int k = keys[h];
    if (k >= 0) {
      const int p = atomicAdd(&s_pos, 1);
      if (p < m) {
        cci[base + p] = k;
        cv[base + p] = vals[h];
      }
    }
  }
  __syncthreads();
  if (m <= kSortMax && !global) {
    // reuse the table as (key, value) scratch: ranks by counting smaller keys
    int* sk = keys;
    double* sv = vals;
    for (int p = threadIdx.x; p < m; p += kT) {
      sk[p] = cci[base + p];
      sv[p] = cv[base + p];
    }
    __syncthreads();
    for (int p = threadIdx.x; p < m; p += kT) {
      const int k = sk[p];
      int rk = 0;
      for (int t = 0; t < m; t++) rk += sk[t] < k;
      cci[base + rk] = k;
      cv[base + rk] = sv[p];
    }
  }
}

// x <- D^-1 A x / ||.||: one power-iteration step on a single FP64 column
__global__ void k_power_step(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                             const double* __restrict__ v, const double* __restrict__ dg,
                             const double* __restrict__ x, double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int e = rp[i]; e < rp[i + 1]; e++) s += v[e] * x[ci[e]];
  y[i] = dg[i] > 0.0 ? s / dg[i] : 0.0;
}

__global__ void k_power_init(int n, double* x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = 0.5 + (double)(amg_hash((uint32_t)i * 2654435761u + 17u) & 0xFFFF) / 65536.0;
}

__global__ void k_norm2(int n, const double* __restrict__ x, double* __restrict__ out) {
  __shared__ double sh[kT];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += kT) s += x[i] * x[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = kT / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

__global__ void k_scale(int n, double* x, const double* nrm2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const double s = *nrm2 > 0.0 ? 1.0 / sqrt(*nrm2) : 0.0;
  if (i < n) x[i] *= s;
}

__global__ void k_to32(long long n, const double* __restrict__ a, float* __restrict__ b) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

// dense n x 2n [A | I] from CSR (row-major)
__global__ void k_dense_aug(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                            const double* __restrict__ v, double* __restrict__ g) {
  const int i = blockIdx.x;
  for (int j = threadIdx.x; j < 2 * n; j += blockDim.x) g[(size_t)i * 2 * n + j] = j == n + i ? 1.0 : 0.0;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int e = rp[i]; e < rp[i + 1]; e++) g[(size_t)i * 2 * n + ci[e]] += v[e];
}

// Gauss-Jordan step k: piv = row k / a_kk, col = column k (bad set when a_kk <= 0)
__global__ void k_gj_pivot(int n, int k, const double* __restrict__ g, double* __restrict__ piv,
                           double* __restrict__ col, int* bad) {
  const double akk = g[(size_t)k * 2 * n + k];
  if (!(akk > 0.0)) {
    if (threadIdx.x == 0) *bad = 1;
    return;
  }
  for (int j = threadIdx.x; j < 2 * n; j += blockDim.x) piv[j] = g[(size_t)k * 2 * n + j] / akk;
  for (int i = threadIdx.x; i < n; i += blockDim.x) col[i] = g[(size_t)i * 2 * n + k];
}

__global__ void k_gj_elim(int n, int k, double* __restrict__ g, const double* __restrict__ piv,
                          const double* __restrict__ col, const int* bad) {
  if (*bad) return;
  const int i = blockIdx.x;
  for (int j = threadIdx.x; j < 2 * n; j += blockDim.x) {
    const size_t o = (size_t)i * 2 * n + j;
    g[o] = i == k ? piv[j] : g[o] - col[i] * piv[j];
  }
}

__global__ void k_gj_extract(int n, const double* __restrict__ g, float* __restrict__ inv) {
  const int i = blockIdx.x;
  for (int j = threadIdx.x; j < n; j += blockDim.x)
    inv[(size_t)i * n + j] = (float)(0.5 * (g[(size_t)i * 2 * n + n + j] + g[(size_t)j * 2 * n + n + i]));
}

// ------------------------------------------------------------------ V-cycle kernels (rows)
template <int KW>
__device__ __forceinline__ void ld_row(const float* __restrict__ X, int r, float* v) {
  const float4* p = reinterpret_cast<const float4*>(X + (size_t)r * KW);
#pragma unroll
  for (int q = 0; q < KW / 4; q++) {
    const float4 t = p[q];
    v[4 * q] = t.x;
    v[4 * q + 1] = t.y;
    v[4 * q + 2] = t.z;
    v[4 * q + 3] = t.w;
  }
}

template <int KW>
__device__ __forceinline__ void st_row(float* __restrict__ X, int r, const float* v) {
  float4* p = reinterpret_cast<float4*>(X + (size_t)r * KW);
#pragma unroll
  for (int q = 0; q < KW / 4; q++) p[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
}

// acc = (M X)[r]
template <int KW>
__device__ __forceinline__ void gather(const int* __restrict__ rp, const int* __restrict__ ci,
                                       const float* __restrict__ v, const float* __restrict__ X,
                                       int r, float* acc) {
#pragma unroll
  for (int c = 0; c < KW; c++) acc[c] = 0.f;
  const int e1 = __ldg(rp + r + 1);
  for (int e = __ldg(rp + r); e < e1; e++) {
    const float a = __ldg(v + e);
    const float4* xr = reinterpret_cast<const float4*>(X + (size_t)__ldg(ci + e) * KW);
#pragma unroll
    for (int q = 0; q < KW / 4; q++) {
      const float4 t = __ldg(xr + q);
      acc[4 * q] = fmaf(a, t.x, acc[4 * q]);
      acc[4 * q + 1] = fmaf(a, t.y, acc[4 * q + 1]);
      acc[4 * q + 2] = fmaf(a, t.z, acc[4 * q + 2]);
      acc[4 * q + 3] = fmaf(a, t.w, acc[4 * q + 3]);
    }
  }
}

// first smoothing step from x = 0: d = c0 D^-1 b, x = d
template <int KW>
__global__ void k_cheb0(int n, const float* __restrict__ b, const float* __restrict__ dinv, float c0,
                        float* __restrict__ d, float* __restrict__ x) {
  const int r = blockIdx.x * kT + threadIdx.x;
  if (r >= n) return;
  float v[KW];
  ld_row<KW>(b, r, v);
  const float s = c0 * dinv[r];
#pragma unroll
  for (int c = 0; c < KW; c++) v[c] *= s;
  st_row<KW>(d, r, v);
  st_row<KW>(x, r, v);
}

// r_out = r_in - A d_in; d_out = c1 d_in + c2 D^-1 r_out; x += (add_din ? d_in : 0) + d_out
// (x == null: no x update; c2 == 0 and d_out == null: residual update only)
template <int KW>
__global__ void __launch_bounds__(kT) k_cheb_step(int n, const int* __restrict__ rp,
                                                  const int* __restrict__ ci,
                                                  const float* __restrict__ av,
                                                  const float* __restrict__ din,
                                                  const float* rin, float* rout,
                                                  const float* __restrict__ dinv, float c1, float c2,
                                                  float* __restrict__ dout, float* __restrict__ x,
                                                  int add_din) {
  const int r = blockIdx.x * kT + threadIdx.x;
  if (r >= n) return;
  float t[KW], rr[KW];
  gather<KW>(rp, ci, av, din, r, t);
  ld_row<KW>(rin, r, rr);
#pragma unroll
  for (int c = 0; c < KW; c++) rr[c] -= t[c];
  st_row<KW>(rout, r, rr);
  if (!dout) return;
  float dd[KW];
  ld_row<KW>(din, r, dd);
  const float s = c2 * dinv[r];
  float xa[KW];
  if (x) ld_row<KW>(x, r, xa);
#pragma unroll
  for (int c = 0; c < KW; c++) {
    const float dn = c1 * dd[c] + s * rr[c];
    if (x) xa[c] += (add_din ? dd[c] : 0.f) + dn;
    dd[c] = dn;
  }
  st_row<KW>(dout, r, dd);
  if (x) st_row<KW>(x, r, xa);
}

// r = b - A x; d = c0 D^-1 r (x is not written: it is being gathered)
template <int KW>
__global__ void __launch_bounds__(kT, row_blocks_per_sm<KW>()) k_resid_cheb0(int n, const int* __restrict__ rp,
                                                    const int* __restrict__ ci,
                                                    const float* __restrict__ av,
                                                    const float* __restrict__ x,
                                                    const float* __restrict__ b,
                                                    const float* __restrict__ dinv, float c0,
                                                    float* __restrict__ rout, float* __restrict__ d) {
  const int r = blockIdx.x * kT + threadIdx.x;
  if (r >= n) return;
  float t[KW], bb[KW];
  gather<KW>(rp, ci, av, x, r, t);
  ld_row<KW>(b, r, bb);
#pragma unroll
  for (int c = 0; c < KW; c++) bb[c] -= t[c];
  st_row<KW>(rout, r, bb);
  const float s = c0 * dinv[r];
#pragma unroll
  for (int c = 0; c < KW; c++) bb[c] *= s;
  st_row<KW>(d, r, bb);
}

// y = M x (plain) or y += M x (add)
template <int KW>
__global__ void __launch_bounds__(kT, row_blocks_per_sm<KW>()) k_spmv(int n, const int* __restrict__ rp,
                                             const int* __restrict__ ci,
                                             const float* __restrict__ mv,
                                             const float* __restrict__ x, float* __restrict__ y,
                                             int add) {
  const int r = blockIdx.x * kT + threadIdx.x;
  if (r >= n) return;
  float t[KW];
  gather<KW>(rp, ci, mv, x, r, t);
  if (add) {
    float yy[KW];
    ld_row<KW>(y, r, yy);
#pragma unroll
    for (int c = 0; c < KW; c++) t[c] += yy[c];
  }
  st_row<KW>(y, r, t);
}

// warp-per-row forms of the smoothing kernels for levels with long rows (the
// Galerkin operators of smoothed aggregation: a hundred or more entries a row):
// the lanes share the row's gathers, a shuffle reduction gives every lane the
// row's product, and lane q < KW / 4 finishes columns 4q .. 4q + 3
template <int KW>
__device__ __forceinline__ void warp_row_product(const int* __restrict__ rp,
                                                 const int* __restrict__ ci,
                                                 const float* __restrict__ av,
                                                 const float* __restrict__ X, int r, int lane,
                                                 float* t) {
#pragma unroll
  for (int c = 0; c < KW; c++) t[c] = 0.f;
  const int e1 = rp[r + 1];
  for (int e = rp[r] + lane; e < e1; e += 32) {
    const float a = av[e];
    const float4* xr = reinterpret_cast<const float4*>(X + (size_t)ci[e] * KW);
#pragma unroll
    for (int q = 0; q < KW / 4; q++) {
      const float4 u = __ldg(xr + q);
      t[4 * q] = fmaf(a, u.x, t[4 * q]);
      t[4 * q + 1] = fmaf(a, u.y, t[4 * q + 1]);
      t[4 * q + 2] = fmaf(a, u.z, t[4 * q + 2]);
      t[4 * q + 3] = fmaf(a, u.w, t[4 * q + 3]);
    }
  }
#pragma unroll
  for (int c = 0; c < KW; c++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t[c] += __shfl_xor_sync(0xffffffffu, t[c], o);
  }
}

// the four product values of lane q's columns
template <int KW>
__device__ __forceinline__ float4 lane_quad(const float* t, int q) {
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int p = 0; p < KW / 4; p++)
    if (p == q) v = make_float4(t[4 * p], t[4 * p + 1], t[4 * p + 2], t[4 * p + 3]);
  return v;
}

template <int KW>
__global__ void __launch_bounds__(kT) k_cheb_step_warp(int n, const int* __restrict__ rp,
                                                       const int* __restrict__ ci,
                                                       const float* __restrict__ av,
                                                       const float* __restrict__ din,
                                                       const float* rin, float* rout,
                                                       const float* __restrict__ dinv, float c1,
                                                       float c2, float* __restrict__ dout,
                                                       float* __restrict__ x, int add_din) {
  const int r = (int)(((long long)blockIdx.x * kT + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= n) return;
  float t[KW];
  warp_row_product<KW>(rp, ci, av, din, r, lane, t);
  if (lane >= KW / 4) return;
  const float4 tq = lane_quad<KW>(t, lane);
  const size_t o = (size_t)r * KW / 4 + lane;
  float4 rr = reinterpret_cast<const float4*>(rin)[o];
  rr.x -= tq.x;
  rr.y -= tq.y;
  rr.z -= tq.z;
  rr.w -= tq.w;
  reinterpret_cast<float4*>(rout)[o] = rr;
  if (!dout) return;
  const float4 dd = reinterpret_cast<const float4*>(din)[o];
  const float s = c2 * dinv[r];
  const float4 dn = make_float4(c1 * dd.x + s * rr.x, c1 * dd.y + s * rr.y, c1 * dd.z + s * rr.z,
                                c1 * dd.w + s * rr.w);
  reinterpret_cast<float4*>(dout)[o] = dn;
  if (x) {
    float4 xa = reinterpret_cast<float4*>(x)[o];
    const float k = add_din ? 1.f : 0.f;
    xa.x += k * dd.x + dn.x;
    xa.y += k * dd.y + dn.y;
    xa.z += k * dd.z + dn.z;
    xa.w += k * dd.w + dn.w;
    reinterpret_cast<float4*>(x)[o] = xa;
  }
}

template <int KW>
__global__ void __launch_bounds__(kT) k_resid_cheb0_warp(int n, const int* __restrict__ rp,
                                                         const int* __restrict__ ci,
                                                         const float* __restrict__ av,
                                                         const float* __restrict__ x,
                                                         const float* __restrict__ b,
                                                         const float* __restrict__ dinv, float c0,
                                                         float* __restrict__ rout,
                                                         float* __restrict__ d) {
  const int r = (int)(((long long)blockIdx.x * kT + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= n) return;
  float t[KW];
  warp_row_product<KW>(rp, ci, av, x, r, lane, t);
  if (lane >= KW / 4) return;
  const float4 tq = lane_quad<KW>(t, lane);
  const size_t o = (size_t)r * KW / 4 + lane;
  float4 bb = reinterpret_cast<const float4*>(b)[o];
  bb.x -= tq.x;
  bb.y -= tq.y;
  bb.z -= tq.z;
  bb.w -= tq.w;
  reinterpret_cast<float4*>(rout)[o] = bb;
  const float s = c0 * dinv[r];
  reinterpret_cast<float4*>(d)[o] = make_float4(s * bb.x, s * bb.y, s * bb.z, s * bb.w);
}

// y = M x for matrices with long rows (the restriction): one warp per row,
// lanes over the row's entries, then a shuffle reduction per column
template <int KW>
__global__ void __launch_bounds__(kT) k_spmv_warp(int n, const int* __restrict__ rp,
                                                  const int* __restrict__ ci,
                                                  const float* __restrict__ mv,
                                                  const float* __restrict__ x,
                                                  float* __restrict__ y) {
  const int r = (int)(((long long)blockIdx.x * kT + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= n) return;
  float acc[KW];
#pragma unroll
  for (int c = 0; c < KW; c++) acc[c] = 0.f;
  const int e1 = rp[r + 1];
  for (int e = rp[r] + lane; e < e1; e += 32) {
    const float a = mv[e];
    const float4* xr = reinterpret_cast<const float4*>(x + (size_t)ci[e] * KW);
#pragma unroll
    for (int q = 0; q < KW / 4; q++) {
      const float4 t = __ldg(xr + q);
      acc[4 * q] = fmaf(a, t.x, acc[4 * q]);
      acc[4 * q + 1] = fmaf(a, t.y, acc[4 * q + 1]);
      acc[4 * q + 2] = fmaf(a, t.z, acc[4 * q + 2]);
      acc[4 * q + 3] = fmaf(a, t.w, acc[4 * q + 3]);
    }
  }
#pragma unroll
  for (int c = 0; c < KW; c++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
  }
  if (lane < KW / 4)
    reinterpret_cast<float4*>(y + (size_t)r * KW)[lane] =
        make_float4(acc[4 * lane], acc[4 * lane + 1], acc[4 * lane + 2], acc[4 * lane + 3]);
}

template <int KW>
__global__ void k_axpy_rows(int n, float* __restrict__ x, const float* __restrict__ d) {
  const int r = blockIdx.x * kT + threadIdx.x;
  if (r >= n) return;
  float a[KW], b[KW];
  ld_row<KW>(x, r, a);
  ld_row<KW>(d, r, b);
#pragma unroll
  for (int c = 0; c < KW; c++) a[c] += b[c];
  st_row<KW>(x, r, a);
}

// x = C b with the dense coarsest inverse C (nc x nc, row-major): a warp per
// row, lanes over the row, a shuffle reduction per column
template <int KW>
__global__ void k_dense_apply(int nc, const float* __restrict__ C, const float* __restrict__ b,
                              float* __restrict__ x) {
  const int r = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= nc) return;
  float acc[KW];
#pragma unroll
  for (int c = 0; c < KW; c++) acc[c] = 0.f;
  for (int j = lane; j < nc; j += 32) {
    const float a = C[(size_t)r * nc + j];
    float bb[KW];
    ld_row<KW>(b, j, bb);
#pragma unroll
    for (int c = 0; c < KW; c++) acc[c] = fmaf(a, bb[c], acc[c]);
  }
#pragma unroll
  for (int c = 0; c < KW; c++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
  }
  if (lane < KW / 4)
    reinterpret_cast<float4*>(x + (size_t)r * KW)[lane] =
        make_float4(acc[4 * lane], acc[4 * lane + 1], acc[4 * lane + 2], acc[4 * lane + 3]);
}

// ------------------------------------------------------------------ PCG kernels (rows)
// per-block column sums of X .* Y into partial[blk * 32 + c] (FP64, fixed order)
template <int KW>
__device__ __forceinline__ void block_colsum(const float* v, double* partial) {
  __shared__ double sh[kT / 32][KW];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < KW; c++) {
    double s = (double)v[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) sh[warp][c] = s;
  }
  __syncthreads();
  if (threadIdx.x < KW) {
    double s = 0.0;
    for (int w = 0; w < kT / 32; w++) s += sh[w][threadIdx.x];
    partial[(size_t)blockIdx.x * 32 + threadIdx.x] = s;
  }
}

// W = A P and partial (P . W) per column
template <int KW>
__global__ void __launch_bounds__(kT) k_pcg_ap(int n, const int* __restrict__ rp,
                                               const int* __restrict__ ci,
                                               const float* __restrict__ av,
                                               const float* __restrict__ P, float* __restrict__ W,
                                               double* __restrict__ partial) {
  float acc[KW];
#pragma unroll
  for (int c = 0; c < KW; c++) acc[c] = 0.f;
  for (int r = blockIdx.x * kT + threadIdx.x; r < n; r += gridDim.x * kT) {
    float t[KW], p[KW];
    gather<KW>(rp, ci, av, P, r, t);
    st_row<KW>(W, r, t);
    ld_row<KW>(P, r, p);
#pragma unroll
    for (int c = 0; c < KW; c++) acc[c] = fmaf(p[c], t[c], acc[c]);
  }
  block_colsum<KW>(acc, partial);
}

// partial (X . Y) per column
template <int KW>
__global__ void __launch_bounds__(kT) k_pcg_dot(int n, const float* __restrict__ X,
                                                const float* __restrict__ Y,
                                                double* __restrict__ partial) {
  float acc[KW];
#pragma unroll
  for (int c = 0; c < KW; c++) acc[c] = 0.f;
  for (int r = blockIdx.x * kT + threadIdx.x; r < n; r += gridDim.x * kT) {
    float a[KW], b[KW];
    ld_row<KW>(X, r, a);
    ld_row<KW>(Y, r, b);
#pragma unroll
    for (int c = 0; c < KW; c++) acc[c] = fmaf(a[c], b[c], acc[c]);
  }
  block_colsum<KW>(acc, partial);
}

// X += alpha P, R -= alpha W (alpha per column, 0 for frozen columns); partial (R . R)
template <int KW>
__global__ void __launch_bounds__(kT) k_pcg_update(int n, float* __restrict__ X, float* __restrict__ R,
                                                   const float* __restrict__ P,
                                                   const float* __restrict__ W,
                                                   const float* __restrict__ alpha,
                                                   double* __restrict__ partial) {
  float al[KW], acc[KW];
#pragma unroll
  for (int c = 0; c < KW; c++) {
    al[c] = alpha[c];
    acc[c] = 0.f;
  }
  for (int r = blockIdx.x * kT + threadIdx.x; r < n; r += gridDim.x * kT) {
    float x[KW], rr[KW], p[KW], w[KW];
    ld_row<KW>(X, r, x);
    ld_row<KW>(R, r, rr);
    ld_row<KW>(P, r, p);
    ld_row<KW>(W, r, w);
#pragma unroll
    for (int c = 0; c < KW; c++) {
      x[c] = fmaf(al[c], p[c], x[c]);
      rr[c] = fmaf(-al[c], w[c], rr[c]);
      acc[c] = fmaf(rr[c], rr[c], acc[c]);
    }
    st_row<KW>(X, r, x);
    st_row<KW>(R, r, rr);
  }
  block_colsum<KW>(acc, partial);
}

// P = Z + beta P (beta per column; frozen columns keep P)
template <int KW>
__global__ void k_pcg_dir(int n, const float* __restrict__ Z, float* __restrict__ P,
                          const float* __restrict__ beta, const int* __restrict__ act) {
  const int r = blockIdx.x * kT + threadIdx.x;
  if (r >= n) return;
  float z[KW], p[KW];
  ld_row<KW>(Z, r, z);
  ld_row<KW>(P, r, p);
#pragma unroll
  for (int c = 0; c < KW; c++)
    if (act[c]) p[c] = fmaf(beta[c], p[c], z[c]);
  st_row<KW>(P, r, p);
}

// Scalar block of the PCG (sc, 32 entries each): rz, r0, alpha (float), beta (float)
struct PcgScal {
  double* rz;
  double* r0;
  float* alpha;
  float* beta;
  int* act;
};

__device__ __forceinline__ double sum_partial(const double* partial, int nblk, int c) {
  double s = 0.0;
  for (int b = 0; b < nblk; b++) s += partial[(size_t)b * 32 + c];
  return s;
}

__global__ void k_pcg_alpha(const double* __restrict__ partial, int nblk, int k, PcgScal s) {
  const int c = threadIdx.x;
  if (c >= 32) return;
  float a = 0.f;
  if (c < k && s.act[c]) {
    const double pw = sum_partial(partial, nblk, c);
    a = pw > 0.0 ? (float)(s.rz[c] / pw) : 0.f;
    if (!(pw > 0.0)) s.act[c] = 0;  // breakdown: freeze the column
  }
  s.alpha[c] = a;
}

// after an update: columns below rate ||r0|| freeze; first = 1 sets r0
__global__ void k_pcg_flags(const double* __restrict__ partial, int nblk, int k, PcgScal s,
                            double rate, int first, int* cnt_out) {
  __shared__ int sc;
  const int c = threadIdx.x;
  if (c == 0) sc = 0;
  __syncthreads();
  if (c < 32) {
    if (c < k) {
      const double nr = sqrt(sum_partial(partial, nblk, c));
      if (first) {
        s.r0[c] = nr;
        s.act[c] = nr > 0.0 ? 1 : 0;
      } else if (s.act[c] && !(nr >= rate * s.r0[c])) {
        s.act[c] = 0;
      }
    } else {
      s.act[c] = 0;
    }
    if (s.act[c]) atomicAdd(&sc, 1);
  }
  __syncthreads();
  if (c == 0) *cnt_out = sc;
}

// rz_new from partial; beta = rz_new / rz (0 on the first step); rz = rz_new
__global__ void k_pcg_beta(const double* __restrict__ partial, int nblk, int k, PcgScal s,
                           int first) {
  const int c = threadIdx.x;
  if (c >= 32) return;
  float b = 0.f;
  if (c < k && s.act[c]) {
    const double rzn = sum_partial(partial, nblk, c);
    b = (first || !(s.rz[c] != 0.0)) ? 0.f : (float)(rzn / s.rz[c]);
    s.rz[c] = rzn;
  }
  s.beta[c] = b;
}

// any nonzero entry among k FP64 columns
__global__ void k_any_nonzero(ColList<double> X, int k, int n, int* flag) {
  const int c = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (X.p[c][i] != 0.0) {
      *flag = 1;
      return;
    }
}

// FP64 columns x += rows block X
template <int KW>
__global__ void k_rows_add_cols(int n, const float* __restrict__ X, ColList<double> Y, int k) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  float v[KW];
  ld_row<KW>(X, r, v);
#pragma unroll
  for (int c = 0; c < KW; c++)
    if (c < k) Y.p[c][r] += (double)v[c];
}

// ------------------------------------------------------------------ host helpers
int grid_of(long long n) { return (int)((n + kT - 1) / kT); }

template <typename T>
int dalloc(T** p, size_t count) {
  *p = nullptr;
  if (cudaMalloc(p, sizeof(T) * (count > 0 ? count : 1)) != cudaSuccess) {
    cudaGetLastError();
    return gcge_record_error(GCGE_CUDA_ERR_ALLOC, "AMG: device allocation failed");
  }
  return GCGE_CUDA_OK;
}

// Chebyshev coefficients of degree deg on [lmax / ratio, lmax]: c0 (first
// step), c1[s], c2[s] (s = 1 .. deg - 1)
struct Cheb {
  float c0;
  float c1[64], c2[64];
};

Cheb cheb_coef(double lmax, double ratio, int deg) {
  Cheb c{};
  const double lo = lmax / ratio, theta = 0.5 * (lmax + lo), delta = 0.5 * (lmax - lo);
  c.c0 = (float)(1.0 / theta);
  const double sigma = theta / delta;
  double rho = 1.0 / sigma;
  for (int s = 1; s < deg && s < 64; s++) {
    const double rn = 1.0 / (2.0 * sigma - rho);
    c.c1[s] = (float)(rn * rho);
    c.c2[s] = (float)(2.0 * rn / delta);
    rho = rn;
  }
  return c;
}

// the transpose of M (rows x cols) as a (cols x rows) matrix, rows sorted
int transpose(const Mat& M, Mat& T, cudaStream_t st) {
  T.rows = M.cols;
  T.cols = M.rows;
  T.nnz = M.nnz;
  AMG_CHK(dalloc(&T.rp, (size_t)T.rows + 1));
  AMG_CHK(dalloc(&T.ci, (size_t)M.nnz));
  AMG_CHK(dalloc(&T.v, (size_t)M.nnz));
  AMG_CU(cudaMemsetAsync(T.rp, 0, sizeof(int) * (T.rows + 1), st));
  if (M.nnz > 0) k_colcount<<<grid_of(M.nnz), kT, 0, st>>>(M.nnz, M.ci, T.rp);
  int tot = 0;
  AMG_CHK(counts_to_rowptr(T.rp, T.rows, &tot, st));
  int* cur = nullptr;
  AMG_CHK(dalloc(&cur, (size_t)T.rows));
  AMG_CU(cudaMemsetAsync(cur, 0, sizeof(int) * T.rows, st));
  int* ci_u = nullptr;
  double* v_u = nullptr;
  AMG_CHK(dalloc(&ci_u, (size_t)M.nnz));
  AMG_CHK(dalloc(&v_u, (size_t)M.nnz));
  k_transpose_fill<<<grid_of(M.rows), kT, 0, st>>>(M.rows, M.rp, M.ci, M.v, T.rp, cur, ci_u, v_u);
  k_rank_rows<<<grid_of((long long)T.rows * 32), kT, 0, st>>>(T.rows, T.rp, ci_u, v_u, T.ci, T.v);
  AMG_CU(cudaGetLastError());
  AMG_CU(cudaStreamSynchronize(st));
  cudaFree(cur);
  cudaFree(ci_u);
  cudaFree(v_u);
  return GCGE_CUDA_OK;
}

// A_c = R A P.  With dense_out != null the product is abandoned (and
// *dense_out set) when more than max(64, nc / 16) coarse rows have more
// distinct columns than the shared table holds: the coarse operator would fill
// in (hub rows of power-law graphs make every aggregate a neighbour of every
// other).
int galerkin(const Mat& R, const Mat& A, const Mat& P, Mat& C, cudaStream_t st,
             bool* dense_out = nullptr) {
  const int nc = R.rows;
  C.rows = C.cols = nc;
  int* cnt = nullptr;
  long long* bound = nullptr;
  AMG_CHK(dalloc(&cnt, (size_t)nc + 1));
  AMG_CHK(dalloc(&bound, (size_t)nc));
  const size_t sym_smem = sizeof(int) * kHashCap;
  k_rap<false><<<nc, kT, sym_smem, st>>>(nullptr, nc, R.rp, R.ci, R.v, A.rp, A.ci, A.v, P.rp,
                                         P.ci, P.v, kHashCap, nullptr, nullptr, nullptr, cnt, bound,
                                         nullptr, nullptr, nullptr);
  AMG_CU(cudaGetLastError());
  std::vector<int> hcnt(nc);
  std::vector<long long> hbound(nc);
  AMG_CU(cudaMemcpyAsync(hcnt.data(), cnt, sizeof(int) * nc, cudaMemcpyDeviceToHost, st));
  AMG_CU(cudaMemcpyAsync(hbound.data(), bound, sizeof(long long) * nc, cudaMemcpyDeviceToHost, st));
  AMG_CU(cudaStreamSynchronize(st));
  // rows past the shared table: symbolic pass again in global tables of
  // 2 * min(nc, products) slots (power of two), in batches of bounded memory
  std::vector<int> over;
  for (int i = 0; i < nc; i++)
    if (hcnt[i] < 0) over.push_back(i);
  if (dense_out) {
    *dense_out = (long long)over.size() > std::max(64, nc / 16);
    if (*dense_out) {
      cudaFree(cnt);
      cudaFree(bound);
      return GCGE_CUDA_OK;
    }
  }
  auto gcap_of = [&](int row) {
    long long m = std::min<long long>((long long)nc, std::max<long long>(1, hbound[row]));
    long long c = 1;
    while (c < 2 * m) c <<= 1;
    return c;
  };
  const long long kBatchSlots = 1ll << 26;  // 64 Mi slots (768 MiB with values)
  int* gkeys = nullptr;
  double* gvals = nullptr;
  long long* goff = nullptr;
  int* glist = nullptr;
  if (!over.empty()) {
    long long maxcap = 0;
    for (int r : over) maxcap = std::max(maxcap, gcap_of(r));
    const long long slots = std::max(kBatchSlots, maxcap);
    AMG_CHK(dalloc(&gkeys, (size_t)slots));
    AMG_CHK(dalloc(&gvals, (size_t)slots));
    AMG_CHK(dalloc(&goff, over.size()));
    AMG_CHK(dalloc(&glist, over.size()));
  }
  auto run_batches = [&](bool numeric, const int* crp, int* cci, double* cv) -> int {
    size_t i0 = 0;
    const long long slots = std::max(kBatchSlots, [&] {
      long long m = 0;
      for (int r : over) m = std::max(m, gcap_of(r));
      return m;
    }());
    while (i0 < over.size()) {
      std::vector<long long> off;
      std::vector<int> rows;
      long long used = 0;
      size_t i1 = i0;
      while (i1 < over.size() && (rows.empty() || used + gcap_of(over[i1]) <= slots)) {
        off.push_back(used);
        rows.push_back(over[i1]);
        used += gcap_of(over[i1]);
        i1++;
      }
      AMG_CU(cudaMemsetAsync(gkeys, 0xFF, sizeof(int) * used, st));
      AMG_CU(cudaMemsetAsync(gvals, 0, sizeof(double) * used, st));
      AMG_CU(cudaMemcpyAsync(goff, off.data(), sizeof(long long) * off.size(), cudaMemcpyHostToDevice, st));
      AMG_CU(cudaMemcpyAsync(glist, rows.data(), sizeof(int) * rows.size(), cudaMemcpyHostToDevice, st));
      // a batch shares one capacity per launch: group rows of equal capacity
      // by launching per row (rows here are few; each CTA uses its own slice)
      for (size_t q = 0; q < rows.size(); q++) {
        const int cap = (int)gcap_of(rows[q]);
        if (numeric)
          k_rap<true><<<1, kT, 0, st>>>(glist + q, 1, R.rp, R.ci, R.v, A.rp, A.ci, A.v, P.rp, P.ci,
                                        P.v, cap, gkeys, gvals, goff + q, nullptr, nullptr, crp, cci, cv);
        else
          k_rap<false><<<1, kT, 0, st>>>(glist + q, 1, R.rp, R.ci, R.v, A.rp, A.ci, A.v, P.rp, P.ci,
                                         P.v, cap, gkeys, nullptr, goff + q, cnt, bound, nullptr,
                                         nullptr, nullptr);
      }
      AMG_CU(cudaGetLastError());
      AMG_CU(cudaStreamSynchronize(st));
      i0 = i1;
    }
    return GCGE_CUDA_OK;
  };
  if (!over.empty()) AMG_CHK(run_batches(false, nullptr, nullptr, nullptr));
  int nnz = 0;
  AMG_CHK(counts_to_rowptr(cnt, nc, &nnz, st));
  C.rp = cnt;
  C.nnz = nnz;
  AMG_CHK(dalloc(&C.ci, (size_t)nnz));
  AMG_CHK(dalloc(&C.v, (size_t)nnz));
  // numeric pass: table capacity from the longest shared-path row
  int maxm = 1;
  for (int i = 0; i < nc; i++)
    if (hcnt[i] > maxm) maxm = hcnt[i];
  int cap = 64;
  while (cap < 2 * maxm) cap <<= 1;
  if (cap > kHashCap) cap = kHashCap;
  const size_t num_smem = (sizeof(double) + sizeof(int)) * cap;
  AMG_CU(cudaFuncSetAttribute(k_rap<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)num_smem));
  std::vector<int> shared_rows;
  shared_rows.reserve(nc);
  for (int i = 0; i < nc; i++)
    if (hcnt[i] >= 0) shared_rows.push_back(i);
  int* slist = nullptr;
  AMG_CHK(dalloc(&slist, shared_rows.size()));
  AMG_CU(cudaMemcpyAsync(slist, shared_rows.data(), sizeof(int) * shared_rows.size(),
                         cudaMemcpyHostToDevice, st));
  if (!shared_rows.empty())
    k_rap<true><<<(int)shared_rows.size(), kT, num_smem, st>>>(
        slist, (int)shared_rows.size(), R.rp, R.ci, R.v, A.rp, A.ci, A.v, P.rp, P.ci, P.v, cap,
        nullptr, nullptr, nullptr, nullptr, nullptr, C.rp, C.ci, C.v);
  AMG_CU(cudaGetLastError());
  if (!over.empty()) AMG_CHK(run_batches(true, C.rp, C.ci, C.v));
  AMG_CU(cudaStreamSynchronize(st));
  cudaFree(slist);
  cudaFree(bound);
  cudaFree(gkeys);
  cudaFree(gvals);
  cudaFree(goff);
  cudaFree(glist);
  return GCGE_CUDA_OK;
}

// lambda_max(D^-1 A) by power iteration (x 1.1)
int power_lmax(const Mat& A, const double* dg, double* out, cudaStream_t st) {
  const int n = A.rows;
  double *x = nullptr, *y = nullptr, *nr = nullptr;
  AMG_CHK(dalloc(&x, (size_t)n));
  AMG_CHK(dalloc(&y, (size_t)n));
  AMG_CHK(dalloc(&nr, 2));
  k_power_init<<<grid_of(n), kT, 0, st>>>(n, x);
  k_norm2<<<1, kT, 0, st>>>(n, x, nr);
  k_scale<<<grid_of(n), kT, 0, st>>>(n, x, nr);
  double lam = 0.0;
  for (int it = 0; it < 15; it++) {
    k_power_step<<<grid_of(n), kT, 0, st>>>(n, A.rp, A.ci, A.v, dg, x, y);
    k_norm2<<<1, kT, 0, st>>>(n, y, nr);
    k_scale<<<grid_of(n), kT, 0, st>>>(n, y, nr);
    std::swap(x, y);
  }
  double h = 0.0;
  AMG_CU(cudaMemcpyAsync(&h, nr, sizeof(double), cudaMemcpyDeviceToHost, st));
  AMG_CU(cudaStreamSynchronize(st));
  lam = sqrt(h);  // ||D^-1 A x|| for the unit x of the previous step
  cudaFree(x);
  cudaFree(y);
  cudaFree(nr);
  if (!(lam > 0.0) || !std::isfinite(lam))
    return gcge_record_error(GCGE_CUDA_ERR_NUMERIC, "AMG: no positive spectral bound of D^-1 A");
  *out = 1.1 * lam;
  return GCGE_CUDA_OK;
}

int level_operator_setup(Level& L, double** dg_out, cudaStream_t st) {
  const int n = L.A.rows;
  double* dg = nullptr;
  AMG_CHK(dalloc(&dg, (size_t)n));
  k_diag<<<grid_of(n), kT, 0, st>>>(n, L.A.rp, L.A.ci, L.A.v, dg);
  int* bad = nullptr;
  AMG_CHK(dalloc(&bad, 1));
  AMG_CU(cudaMemsetAsync(bad, 0, sizeof(int), st));
  AMG_CHK(dalloc(&L.dinv, (size_t)n));
  k_dinv32<<<grid_of(n), kT, 0, st>>>(n, dg, L.dinv, bad);
  if (!L.A.v32) {
    AMG_CHK(dalloc(&L.A.v32, (size_t)L.A.nnz));
    if (L.A.nnz > 0) k_to32<<<grid_of(L.A.nnz), kT, 0, st>>>(L.A.nnz, L.A.v, L.A.v32);
  }
  int hbad = 0;
  AMG_CU(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  AMG_CU(cudaStreamSynchronize(st));
  cudaFree(bad);
  if (hbad) {
    cudaFree(dg);
    return gcge_record_error(GCGE_CUDA_ERR_NUMERIC, "AMG: a diagonal entry is not positive");
  }
  AMG_CHK(power_lmax(L.A, dg, &L.lmax, st));
  *dg_out = dg;
  return GCGE_CUDA_OK;
}

// aggregation of level L (its operator and diagonal set): L.agg, count nagg
int aggregate(Level& L, const double* dg, double theta, int* nagg, cudaStream_t st) {
  const int n = L.A.rows;
  int *srp = nullptr, *sci = nullptr;
  AMG_CHK(dalloc(&srp, (size_t)n + 1));
  k_strength<<<grid_of(n), kT, 0, st>>>(n, L.A.rp, L.A.ci, L.A.v, dg, theta, srp, nullptr, nullptr, 0);
  int snnz = 0;
  AMG_CHK(counts_to_rowptr(srp, n, &snnz, st));
  AMG_CHK(dalloc(&sci, (size_t)snnz));
  k_strength<<<grid_of(n), kT, 0, st>>>(n, L.A.rp, L.A.ci, L.A.v, dg, theta, nullptr, srp, sci, 1);
  int* state = nullptr;
  unsigned long long *t = nullptr, *t1 = nullptr, *t2 = nullptr;
  int* und = nullptr;
  AMG_CHK(dalloc(&state, (size_t)n));
  AMG_CHK(dalloc(&t, (size_t)n));
  AMG_CHK(dalloc(&t1, (size_t)n));
  AMG_CHK(dalloc(&t2, (size_t)n));
  AMG_CHK(dalloc(&und, 1));
  k_mis_init<<<grid_of(n), kT, 0, st>>>(n, state, t);
  for (int it = 0; it < 200; it++) {
    k_mis_max<<<grid_of(n), kT, 0, st>>>(n, srp, sci, t, t1);
    k_mis_max<<<grid_of(n), kT, 0, st>>>(n, srp, sci, t1, t2);
    AMG_CU(cudaMemsetAsync(und, 0, sizeof(int), st));
    k_mis_decide<<<grid_of(n), kT, 0, st>>>(n, state, t, t2, und);
    int h = 0;
    AMG_CU(cudaMemcpyAsync(&h, und, sizeof(int), cudaMemcpyDeviceToHost, st));
    AMG_CU(cudaStreamSynchronize(st));
    if (h == 0) break;
    if (it == 199) return gcge_record_error(GCGE_CUDA_ERR_NUMERIC, "AMG: aggregation did not settle");
  }
  int* num = nullptr;
  AMG_CHK(dalloc(&num, (size_t)n + 1));
  k_root_flags<<<grid_of(n), kT, 0, st>>>(n, state, num);
  int nroot = 0;
  AMG_CHK(counts_to_rowptr(num, n, &nroot, st));
  AMG_CHK(dalloc(&L.agg, (size_t)n));
  k_agg_roots<<<grid_of(n), kT, 0, st>>>(n, state, num, L.agg);
  int* snap = nullptr;
  AMG_CHK(dalloc(&snap, (size_t)n));
  AMG_CU(cudaMemcpyAsync(snap, L.agg, sizeof(int) * n, cudaMemcpyDeviceToDevice, st));
  k_agg_join<<<grid_of(n), kT, 0, st>>>(n, srp, sci, snap, L.agg);
  AMG_CU(cudaMemcpyAsync(snap, L.agg, sizeof(int) * n, cudaMemcpyDeviceToDevice, st));
  k_agg_join<<<grid_of(n), kT, 0, st>>>(n, srp, sci, snap, L.agg);
  // rows still alone (not expected on a symmetric pattern) become singletons
  k_left_flags<<<grid_of(n), kT, 0, st>>>(n, L.agg, num);
  int nleft = 0;
  AMG_CHK(counts_to_rowptr(num, n, &nleft, st));
  if (nleft > 0) k_left_assign<<<grid_of(n), kT, 0, st>>>(n, num, nroot, L.agg);
  AMG_CU(cudaGetLastError());
  AMG_CU(cudaStreamSynchronize(st));
  *nagg = nroot + nleft;
  cudaFree(srp);
  cudaFree(sci);
  cudaFree(state);
  cudaFree(t);
  cudaFree(t1);
  cudaFree(t2);
  cudaFree(und);
  cudaFree(num);
  cudaFree(snap);
  return GCGE_CUDA_OK;
}

int prolongation(Level& L, const double* dg, int nagg, int smooth, cudaStream_t st) {
  const int n = L.A.rows;
  Mat& P = L.P;
  P.rows = n;
  P.cols = nagg;
  AMG_CHK(dalloc(&P.rp, (size_t)n + 1));
  const double omega = 4.0 / (3.0 * L.lmax);
  k_prolong<<<grid_of(n), kT, 0, st>>>(n, L.A.rp, L.A.ci, L.A.v, dg, L.agg, omega, smooth, P.rp,
                                       nullptr, nullptr, nullptr, 0);
  AMG_CHK(counts_to_rowptr(P.rp, n, &P.nnz, st));
  AMG_CHK(dalloc(&P.ci, (size_t)P.nnz));
  AMG_CHK(dalloc(&P.v, (size_t)P.nnz));
  k_prolong<<<grid_of(n), kT, 0, st>>>(n, L.A.rp, L.A.ci, L.A.v, dg, L.agg, omega, smooth, nullptr,
                                       P.rp, P.ci, P.v, 1);
  AMG_CU(cudaGetLastError());
  AMG_CHK(transpose(P, L.R, st));
  AMG_CHK(dalloc(&P.v32, (size_t)P.nnz));
  AMG_CHK(dalloc(&L.R.v32, (size_t)L.R.nnz));
  if (P.nnz > 0) {
    k_to32<<<grid_of(P.nnz), kT, 0, st>>>(P.nnz, P.v, P.v32);
    k_to32<<<grid_of(P.nnz), kT, 0, st>>>(L.R.nnz, L.R.v, L.R.v32);
  }
  AMG_CU(cudaGetLastError());
  return GCGE_CUDA_OK;
}

int coarsest_inverse(GCGE_CUDA_AMG_* amg, cudaStream_t st) {
  const Level& L = amg->lev[amg->nlev - 1];
  const int n = L.A.rows;
  if (n > kCoarseMax) return GCGE_CUDA_OK;  // smoothed instead
  // the elimination's scratch is freed however this function returns
  struct Scratch {
    double *g = nullptr, *piv = nullptr, *col = nullptr;
    int* bad = nullptr;
    ~Scratch() {
      cudaFree(g);
      cudaFree(piv);
      cudaFree(col);
      cudaFree(bad);
    }
  } w;
  AMG_CHK(dalloc(&w.g, (size_t)n * 2 * n));
  AMG_CHK(dalloc(&w.piv, (size_t)2 * n));
  AMG_CHK(dalloc(&w.col, (size_t)n));
  AMG_CHK(dalloc(&w.bad, 1));
  double *g = w.g, *piv = w.piv, *col = w.col;
  int* bad = w.bad;
  AMG_CU(cudaMemsetAsync(bad, 0, sizeof(int), st));
  k_dense_aug<<<n, 256, 0, st>>>(n, L.A.rp, L.A.ci, L.A.v, g);
  for (int k = 0; k < n; k++) {
    k_gj_pivot<<<1, 1024, 0, st>>>(n, k, g, piv, col, bad);
    k_gj_elim<<<n, 256, 0, st>>>(n, k, g, piv, col, bad);
  }
  int hbad = 0;
  AMG_CU(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  AMG_CU(cudaStreamSynchronize(st));
  if (!hbad) {
    AMG_CHK(dalloc(&amg->cinv, (size_t)n * n));
    k_gj_extract<<<n, 256, 0, st>>>(n, g, amg->cinv);
    AMG_CU(cudaGetLastError());
    AMG_CU(cudaStreamSynchronize(st));
  }
  return GCGE_CUDA_OK;  // a non-positive pivot leaves the coarsest level smoothed
}

void free_level(Level& L) {
  if (L.own_A) {
    L.A.release();
  } else {
    cudaFree(L.A.v32);
  }
  L.P.release();
  L.R.release();
  cudaFree(L.agg);
  cudaFree(L.dinv);
  cudaFree(L.x);
  cudaFree(L.b);
  cudaFree(L.r);
  cudaFree(L.d0);
  cudaFree(L.d1);
  L = Level();
}

void free_pcg(GCGE_CUDA_AMG_* amg) {
  cudaFree(amg->pr);
  cudaFree(amg->px);
  cudaFree(amg->pp);
  cudaFree(amg->pw);
  amg->pr = amg->px = amg->pp = amg->pw = nullptr;
}

// work blocks of width kw on every level (and the PCG's four at level 0)
int ensure_work(GCGE_CUDA_AMG_* amg, int kw) {
  if (amg->kw >= kw) return GCGE_CUDA_OK;
  for (int l = 0; l < amg->nlev; l++) {
    Level& L = amg->lev[l];
    cudaFree(L.x);
    cudaFree(L.b);
    cudaFree(L.r);
    cudaFree(L.d0);
    cudaFree(L.d1);
    L.x = L.b = L.r = L.d0 = L.d1 = nullptr;
  }
  free_pcg(amg);
  amg->kw = 0;
  for (int l = 0; l < amg->nlev; l++) {
    Level& L = amg->lev[l];
    const size_t len = (size_t)L.A.rows * kw;
    AMG_CHK(dalloc(&L.x, len));
    AMG_CHK(dalloc(&L.b, len));
    AMG_CHK(dalloc(&L.r, len));
    AMG_CHK(dalloc(&L.d0, len));
    AMG_CHK(dalloc(&L.d1, len));
  }
  const size_t len0 = (size_t)amg->lev[0].A.rows * kw;
  AMG_CHK(dalloc(&amg->pr, len0));
  AMG_CHK(dalloc(&amg->px, len0));
  AMG_CHK(dalloc(&amg->pp, len0));
  AMG_CHK(dalloc(&amg->pw, len0));
  amg->kw = kw;
  return GCGE_CUDA_OK;
}

// ------------------------------------------------------------------ V-cycle
template <int KW>
void spmv_rows(const Mat& M, const float* x, float* y, int add, cudaStream_t st,
               const GcgeDevCsr* heavy = nullptr) {
  if (heavy && heavy->nheavy > 0 && !add) {
    gcge::spmm_rows_f32(M.rp, M.ci, M.v32, M.rows, x, y, KW, st, heavy);
    return;
  }
  if (!add && M.nnz >= 32ll * M.rows) {
    // long rows (the restriction of a smoothed prolongation): a warp per row
    k_spmv_warp<KW><<<grid_of((long long)M.rows * 32), kT, 0, st>>>(M.rows, M.rp, M.ci, M.v32, x, y);
    return;
  }
  k_spmv<KW><<<grid_of(M.rows), kT, 0, st>>>(M.rows, M.rp, M.ci, M.v32, x, y, add);
}

// Chebyshev smoothing on level L: from x = 0 (zero_start) or from the
// current x; want_resid: leave b - A x in L.r (pre-smoothing)
template <int KW>
void smooth(const GCGE_CUDA_AMG_* amg, const Level& L, const float* b, int deg, bool zero_start,
            bool want_resid, cudaStream_t st) {
  const int n = L.A.rows;
  const Cheb c = cheb_coef(L.lmax, amg->prm.cheb_ratio, deg);
  const int g = grid_of(n);
  // levels with long rows (coarse Galerkin operators) take a warp per row
  const bool wide = L.A.nnz >= 32ll * n;
  const int gw = grid_of((long long)n * 32);
  auto step = [&](const float* din, const float* rin_, float c1, float c2, float* dout, float* xx,
                  int add) {
    if (wide)
      k_cheb_step_warp<KW><<<gw, kT, 0, st>>>(n, L.A.rp, L.A.ci, L.A.v32, din, rin_, L.r, L.dinv,
                                              c1, c2, dout, xx, add);
    else
      k_cheb_step<KW><<<g, kT, 0, st>>>(n, L.A.rp, L.A.ci, L.A.v32, din, rin_, L.r, L.dinv, c1, c2,
                                        dout, xx, add);
  };
  float* d[2] = {L.d0, L.d1};
  const float* rin = b;
  if (zero_start) {
    k_cheb0<KW><<<g, kT, 0, st>>>(n, b, L.dinv, c.c0, d[0], L.x);
  } else {
    if (wide)
      k_resid_cheb0_warp<KW><<<gw, kT, 0, st>>>(n, L.A.rp, L.A.ci, L.A.v32, L.x, b, L.dinv, c.c0,
                                                L.r, d[0]);
    else
      k_resid_cheb0<KW><<<g, kT, 0, st>>>(n, L.A.rp, L.A.ci, L.A.v32, L.x, b, L.dinv, c.c0, L.r,
                                          d[0]);
    rin = L.r;
  }
  int cur = 0;
  for (int s = 1; s < deg; s++) {
    step(d[cur], rin, c.c1[s], c.c2[s], d[cur ^ 1], L.x, (!zero_start && s == 1) ? 1 : 0);
    rin = L.r;
    cur ^= 1;
  }
  if (!zero_start && deg == 1) k_axpy_rows<KW><<<g, kT, 0, st>>>(n, L.x, d[0]);
  if (want_resid) step(d[cur], rin, 0.f, 0.f, nullptr, nullptr, 0);
}

// x_l = M_l^-1 b (b: level 0's input, or L.b on coarser levels)
template <int KW>
void vcycle(const GCGE_CUDA_AMG_* amg, int l, const float* b, cudaStream_t st) {
  const Level& L = amg->lev[l];
  const int deg = amg->prm.cheb_degree;
  if (l == amg->nlev - 1) {
    if (amg->cinv) {
      k_dense_apply<KW><<<grid_of((long long)L.A.rows * 32), kT, 0, st>>>(L.A.rows, amg->cinv, b,
                                                                           L.x);
    } else {
      smooth<KW>(amg, L, b, 4 * deg, true, false, st);
    }
    return;
  }
  smooth<KW>(amg, L, b, deg, true, true, st);
  const Level& C = amg->lev[l + 1];
  spmv_rows<KW>(L.R, L.r, C.b, 0, st);
  vcycle<KW>(amg, l + 1, C.b, st);
  spmv_rows<KW>(L.P, C.x, L.x, 1, st);
  smooth<KW>(amg, L, b, deg, false, false, st);
}

// ------------------------------------------------------------------ AMG-PCG
template <int KW>
int pcg_rows(GCGE_CUDA_AMG_* amg, int k, cudaStream_t st, int* steps_out) {
  const Level& L0 = amg->lev[0];
  const int n = L0.A.rows;
  const int nb = std::min(kRedBlocks, grid_of(n));
  double* partial = amg->red;
  PcgScal s;
  s.rz = amg->red + (size_t)kRedBlocks * 32;
  s.r0 = s.rz + 32;
  s.alpha = reinterpret_cast<float*>(s.r0 + 32);
  s.beta = s.alpha + 32;
  s.act = amg->flags;
  const int maxit = amg->prm.pcg_max_it;
  const double rate = amg->prm.pcg_rate;
  float *R = amg->pr, *X = amg->px, *P = amg->pp, *W = amg->pw;
  const GcgeDevCsr* hv = L0.heavy;
  // r0 norms and flags; z = M r; rz; p = z
  k_pcg_dot<KW><<<nb, kT, 0, st>>>(n, R, R, partial);
  k_pcg_flags<<<1, 32, 0, st>>>(partial, nb, k, s, rate, 1, amg->dev_cnt);
  vcycle<KW>(amg, 0, R, st);
  k_pcg_dot<KW><<<nb, kT, 0, st>>>(n, R, L0.x, partial);
  k_pcg_beta<<<1, 32, 0, st>>>(partial, nb, k, s, 1);
  k_pcg_dir<KW><<<grid_of(n), kT, 0, st>>>(n, L0.x, P, s.beta, s.act);
  int it = 0;
  while (it < maxit) {
    const int batch = std::min(kCheck, maxit - it);
    for (int j = 0; j < batch; j++) {
      if (hv && hv->nheavy > 0) {
        // heavy rows: the chunked SpMM, then the dot product
        gcge::spmm_rows_f32(L0.A.rp, L0.A.ci, L0.A.v32, n, P, W, KW, st, hv);
        k_pcg_dot<KW><<<nb, kT, 0, st>>>(n, P, W, partial);
      } else {
        k_pcg_ap<KW><<<nb, kT, 0, st>>>(n, L0.A.rp, L0.A.ci, L0.A.v32, P, W, partial);
      }
      k_pcg_alpha<<<1, 32, 0, st>>>(partial, nb, k, s);
      k_pcg_update<KW><<<nb, kT, 0, st>>>(n, X, R, P, W, s.alpha, partial);
      k_pcg_flags<<<1, 32, 0, st>>>(partial, nb, k, s, rate, 0, amg->dev_cnt + 1 + j);
      if (it + j + 1 < maxit) {
        vcycle<KW>(amg, 0, R, st);
        k_pcg_dot<KW><<<nb, kT, 0, st>>>(n, R, L0.x, partial);
        k_pcg_beta<<<1, 32, 0, st>>>(partial, nb, k, s, 0);
        k_pcg_dir<KW><<<grid_of(n), kT, 0, st>>>(n, L0.x, P, s.beta, s.act);
      }
    }
    AMG_CU(cudaStreamSynchronize(st));
    bool done = false;
    for (int j = 0; j < batch; j++) {
      it++;
      if (amg->host_cnt[1 + j] == 0) {
        done = true;
        break;
      }
    }
    if (done) break;
  }
  AMG_CU(cudaGetLastError());
  *steps_out = it;
  return GCGE_CUDA_OK;
}

template <int KW>
int apply_rows(GCGE_CUDA_AMG_* amg, cudaStream_t st) {
  vcycle<KW>(amg, 0, amg->pr, st);
  AMG_CU(cudaGetLastError());
  return GCGE_CUDA_OK;
}

template <int KW>
void add_rows_to_cols(int n, const float* X, const ColList<double>& Y, int k, cudaStream_t st) {
  k_rows_add_cols<KW><<<grid_of(n), kT, 0, st>>>(n, X, Y, k);
}

#define AMG_DISPATCH(kw, CALL)     \
  switch (kw) {                    \
    case 4: { constexpr int KW = 4; CALL; } break;   \
    case 8: { constexpr int KW = 8; CALL; } break;   \
    case 12: { constexpr int KW = 12; CALL; } break; \
    case 16: { constexpr int KW = 16; CALL; } break; \
    case 20: { constexpr int KW = 20; CALL; } break; \
    case 24: { constexpr int KW = 24; CALL; } break; \
    case 28: { constexpr int KW = 28; CALL; } break; \
    case 32: { constexpr int KW = 32; CALL; } break; \
  }

int pcg_state(GCGE_CUDA_AMG_* amg) {
  if (!amg->red) AMG_CHK(dalloc(&amg->red, (size_t)kRedBlocks * 32 + 4 * 32));
  if (!amg->flags) AMG_CHK(dalloc(&amg->flags, 64));
  if (!amg->host_cnt) {
    if (cudaHostAlloc(&amg->host_cnt, sizeof(int) * (kCheck + 2), cudaHostAllocMapped) != cudaSuccess) {
      cudaGetLastError();
      amg->host_cnt = nullptr;
      return gcge_record_error(GCGE_CUDA_ERR_ALLOC, "AMG: pinned allocation failed");
    }
    AMG_CU(cudaHostGetDevicePointer((void**)&amg->dev_cnt, amg->host_cnt, 0));
  }
  return GCGE_CUDA_OK;
}

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" void GCGE_CUDA_AMG_DefaultParam(GCGE_CUDA_AMG_PARAM* p) {
  if (!p) return;
  p->max_levels = 10;
  p->coarse_size = 256;
  p->strength = 0.0;
  p->smooth_p = 1;
  p->cheb_degree = 3;
  p->cheb_ratio = 30.0;
  p->pcg_max_it = 20;
  p->pcg_rate = 1e-2;
}

extern "C" int GCGE_CUDA_AMG_Destroy(GCGE_CUDA_AMG** amg) {
  if (!amg || !*amg) return GCGE_CUDA_OK;
  GCGE_CUDA_AMG_* a = *amg;
  for (int l = 0; l < a->nlev; l++) free_level(a->lev[l]);
  free_pcg(a);
  cudaFree(a->cinv);
  cudaFree(a->tmp64);
  cudaFree(a->red);
  cudaFree(a->flags);
  if (a->host_cnt) cudaFreeHost(a->host_cnt);
  delete a;
  *amg = nullptr;
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_AMG_Create(GCGE_CUDA_AMG** out, const GCGE_CUDA_MAT* A,
                                    const GCGE_CUDA_AMG_PARAM* prm) {
  if (!out || !A || A->m.n <= 0) return gcge_record_error(GCGE_CUDA_ERR_ARG, "AMG_Create: bad arguments");
  GCGE_CUDA_AMG_PARAM p;
  GCGE_CUDA_AMG_DefaultParam(&p);
  if (prm) p = *prm;
  if (p.max_levels < 1 || p.max_levels > kMaxLevels || p.coarse_size < 1 ||
      p.coarse_size > kCoarseMax || !(p.strength >= 0.0 && p.strength < 1.0) ||
      (p.smooth_p != 0 && p.smooth_p != 1) || p.cheb_degree < 1 || p.cheb_degree > 16 ||
      !(p.cheb_ratio > 1.0) || p.pcg_max_it < 1 || !(p.pcg_rate > 0.0 && p.pcg_rate < 1.0))
    return gcge_record_error(GCGE_CUDA_ERR_ARG,
                             "AMG_Create: parameter out of range (levels 1..16, coarse_size "
                             "1..512, strength [0,1), smooth_p 0/1, degree 1..16, ratio > 1, "
                             "pcg_max_it >= 1, pcg_rate (0,1))");
  *out = nullptr;
  std::lock_guard<std::mutex> lk(g_amg_mu);
  GCGE_CUDA_AMG_* amg = new GCGE_CUDA_AMG_();
  amg->prm = p;
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
    delete amg;
    return gcge_record_error(GCGE_CUDA_ERR_CUDA, "AMG_Create: stream creation failed");
  }
  auto fail = [&](int rc) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    GCGE_CUDA_AMG* t = amg;
    GCGE_CUDA_AMG_Destroy(&t);
    return rc;
  };
  Level& L0 = amg->lev[0];
  L0.A.rows = L0.A.cols = A->m.n;
  L0.A.nnz = A->m.nnz;
  L0.A.rp = A->m.rp;
  L0.A.ci = A->m.ci;
  L0.A.v = A->m.v;
  L0.own_A = false;
  L0.heavy = A->m.nheavy > 0 ? &A->m : nullptr;
  amg->nlev = 1;
  for (int l = 0;; l++) {
    Level& L = amg->lev[l];
    double* dg = nullptr;
    int rc = level_operator_setup(L, &dg, st);
    if (rc != GCGE_CUDA_OK) return fail(rc);
    const bool last = L.A.rows <= p.coarse_size || l + 1 >= p.max_levels;
    if (last) {
      cudaFree(dg);
      break;
    }
    int nagg = 0;
    rc = aggregate(L, dg, p.strength, &nagg, st);
    if (rc == GCGE_CUDA_OK && (nagg < 1 || nagg * 6 > L.A.rows * 5)) {
      // coarsening stalls (fewer than 1.2x): this level is the coarsest
      cudaFree(L.agg);
      L.agg = nullptr;
      cudaFree(dg);
      break;
    }
    if (rc == GCGE_CUDA_OK) rc = prolongation(L, dg, nagg, p.smooth_p, st);
    cudaFree(dg);
    if (rc != GCGE_CUDA_OK) return fail(rc);
    Level& C = amg->lev[l + 1];
    C.own_A = true;
    bool dense = false;
    rc = galerkin(L.R, L.A, L.P, C.A, st, &dense);
    if (rc == GCGE_CUDA_OK && dense) {
      // the coarse operator would fill in: level l stays the coarsest
      L.P.release();
      L.R.release();
      cudaFree(L.agg);
      L.agg = nullptr;
      C = Level();
      break;
    }
    amg->nlev = l + 2;
    if (rc != GCGE_CUDA_OK) return fail(rc);
  }
  {
    const int rc = coarsest_inverse(amg, st);
    if (rc != GCGE_CUDA_OK) return fail(rc);
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail(gcge_record_error(GCGE_CUDA_ERR_CUDA, "AMG_Create: set-up kernels failed"));
  cudaStreamDestroy(st);
  *out = amg;
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_AMG_GetNumLevels(const GCGE_CUDA_AMG* amg, int* nlev) {
  if (!amg || !nlev) return gcge_record_error(GCGE_CUDA_ERR_ARG, "AMG_GetNumLevels: bad arguments");
  *nlev = amg->nlev;
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_AMG_GetLevelInfo(const GCGE_CUDA_AMG* amg, int l, int* n, int* nnz_a,
                                          int* nnz_p, double* lmax) {
  if (!amg || l < 0 || l >= amg->nlev)
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "AMG_GetLevelInfo: bad arguments");
  const Level& L = amg->lev[l];
  if (n) *n = L.A.rows;
  if (nnz_a) *nnz_a = L.A.nnz;
  if (nnz_p) *nnz_p = L.P.nnz;
  if (lmax) *lmax = L.lmax;
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_AMG_GetLevelCSR(const GCGE_CUDA_AMG* amg, int l, int which, int* rp,
                                         int* ci, double* v) {
  if (!amg || l < 0 || l >= amg->nlev || which < 0 || which > 2 || !rp || !ci || !v)
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "AMG_GetLevelCSR: bad arguments");
  const Level& L = amg->lev[l];
  const Mat& M = which == 0 ? L.A : (which == 1 ? L.P : L.R);
  if (!M.rp) return gcge_record_error(GCGE_CUDA_ERR_ARG, "AMG_GetLevelCSR: no such matrix on this level");
  AMG_CU(cudaMemcpy(rp, M.rp, sizeof(int) * (M.rows + 1), cudaMemcpyDeviceToHost));
  if (M.nnz > 0) {
    AMG_CU(cudaMemcpy(ci, M.ci, sizeof(int) * M.nnz, cudaMemcpyDeviceToHost));
    AMG_CU(cudaMemcpy(v, M.v, sizeof(double) * M.nnz, cudaMemcpyDeviceToHost));
  }
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_AMG_GetAggregates(const GCGE_CUDA_AMG* amg, int l, int* agg) {
  if (!amg || l < 0 || l >= amg->nlev - 1 || !agg || !amg->lev[l].agg)
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "AMG_GetAggregates: bad arguments");
  AMG_CU(cudaMemcpy(agg, amg->lev[l].agg, sizeof(int) * amg->lev[l].A.rows, cudaMemcpyDeviceToHost));
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_AMG_Apply(GCGE_CUDA_AMG* amg, double* const* b, double* const* x, int k,
                                   void* stream) {
  if (!amg || !b || !x || k < 1 || k > 32)
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "AMG_Apply: bad arguments (1 <= k <= 32)");
  std::lock_guard<std::mutex> lk(g_amg_mu);
  cudaStream_t st = (cudaStream_t)stream;
  const int kw = gcge::bcg_rows_width(k);
  AMG_CHK(ensure_work(amg, kw));
  const int n = amg->lev[0].A.rows;
  ColList<double> B, X;
  for (int c = 0; c < k; c++) {
    B.p[c] = b[c];
    X.p[c] = x[c];
  }
  gcge::cols_to_rows_f32(B, k, amg->pr, n, st);
  int rc = GCGE_CUDA_OK;
  AMG_DISPATCH(kw, rc = apply_rows<KW>(amg, st));
  if (rc != GCGE_CUDA_OK) return rc;
  gcge::rows_to_cols_f64(amg->lev[0].x, k, X, n, st);
  AMG_CU(cudaGetLastError());
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_AMGPCG(void* ctx, const GCGE_CUDA_MAT* A, double* const* rhs,
                                double* const* x, int k, int n, void* stream) {
  GCGE_CUDA_AMG_* amg = static_cast<GCGE_CUDA_AMG_*>(ctx);
  if (!amg || !A || !rhs || !x || k < 1 || k > GCGE_MAXCOLS || n != A->m.n ||
      amg->lev[0].A.rows != n || amg->lev[0].A.rp != A->m.rp)
    return gcge_record_error(GCGE_CUDA_ERR_ARG,
                             "AMGPCG: bad arguments (ctx = a GCGE_CUDA_AMG built on this A, "
                             "1 <= k <= 256)");
  if (k > 32) {
    // wider blocks in groups of 32 columns (the row-interleaved blocks' widest)
    int steps = 0;
    for (int c0 = 0; c0 < k; c0 += 32) {
      const int rc = GCGE_CUDA_AMGPCG(ctx, A, rhs + c0, x + c0, std::min(32, k - c0), n, stream);
      if (rc != GCGE_CUDA_OK) return rc;
      steps = std::max(steps, amg->last_steps);
    }
    amg->last_steps = steps;
    return GCGE_CUDA_OK;
  }
  std::lock_guard<std::mutex> lk(g_amg_mu);
  cudaStream_t st = (cudaStream_t)stream;
  const int kw = gcge::bcg_rows_width(k);
  AMG_CHK(ensure_work(amg, kw));
  AMG_CHK(pcg_state(amg));
  ColList<double> RH, XC;
  for (int c = 0; c < k; c++) {
    RH.p[c] = rhs[c];
    XC.p[c] = x[c];
  }
  // r = rhs - A x0 in FP64, skipped for a zero start
  AMG_CU(cudaMemsetAsync(amg->flags + 32, 0, sizeof(int), st));
  k_any_nonzero<<<dim3(std::min(grid_of(n), 608), k), kT, 0, st>>>(XC, k, n, amg->flags + 32);
  int nz = 0;
  AMG_CU(cudaMemcpyAsync(&nz, amg->flags + 32, sizeof(int), cudaMemcpyDeviceToHost, st));
  AMG_CU(cudaStreamSynchronize(st));
  if (nz) {
    const size_t need = (size_t)k * n;
    if (amg->tmp64_len < need) {
      cudaFree(amg->tmp64);
      amg->tmp64 = nullptr;
      amg->tmp64_len = 0;
      AMG_CHK(dalloc(&amg->tmp64, need));
      amg->tmp64_len = need;
    }
    ColList<double> T;
    for (int c = 0; c < k; c++) T.p[c] = amg->tmp64 + (size_t)c * n;
    gcge::spmm_f64(A->m, XC, T, k, st);
    gcge::axpby_f64(-1.0, T, 1.0, RH, k, n, st);
  }
  gcge::cols_to_rows_f32(RH, k, amg->pr, n, st);
  AMG_CU(cudaMemsetAsync(amg->px, 0, sizeof(float) * (size_t)n * kw, st));
  // p starts at zero: frozen and padding columns then stay exactly zero
  AMG_CU(cudaMemsetAsync(amg->pp, 0, sizeof(float) * (size_t)n * kw, st));
  int steps = 0, rc = GCGE_CUDA_OK;
  AMG_DISPATCH(kw, rc = pcg_rows<KW>(amg, k, st, &steps));
  if (rc != GCGE_CUDA_OK) return rc;
  AMG_DISPATCH(kw, add_rows_to_cols<KW>(n, amg->px, XC, k, st));
  AMG_CU(cudaGetLastError());
  amg->last_steps = steps;
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_AMG_GetLastSteps(const GCGE_CUDA_AMG* amg, int* steps) {
  if (!amg || !steps) return gcge_record_error(GCGE_CUDA_ERR_ARG, "AMG_GetLastSteps: bad arguments");
  *steps = amg->last_steps;
  return GCGE_CUDA_OK;
}

// ------------------------------------------------------------------ internal views
namespace gcge {
namespace amg {

namespace {
View view_of(const Mat& m) {
  View v;
  v.rows = m.rows;
  v.cols = m.cols;
  v.nnz = m.nnz;
  v.rp = m.rp;
  v.ci = m.ci;
  v.v = m.v;
  return v;
}
Mat mat_of(const View& v) {
  Mat m;
  m.rows = v.rows;
  m.cols = v.cols;
  m.nnz = v.nnz;
  m.rp = v.rp;
  m.ci = v.ci;
  m.v = v.v;
  return m;
}

__global__ void k_identity(int n, int* rp, int* ci, double* v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    ci[i] = i;
    v[i] = 1.0;
  }
  if (i <= n) rp[i] = i;
}
}  // namespace

int levels(const GCGE_CUDA_AMG* a) { return a ? a->nlev : 0; }
View op(const GCGE_CUDA_AMG* a, int l) { return view_of(a->lev[l].A); }
View prolong(const GCGE_CUDA_AMG* a, int l) { return view_of(a->lev[l].P); }
View restrict_to(const GCGE_CUDA_AMG* a, int l) { return view_of(a->lev[l].R); }

int galerkin(const View& R, const View& M, const View& P, View* C, cudaStream_t st) {
  Mat c;
  const int rc = ::galerkin(mat_of(R), mat_of(M), mat_of(P), c, st);
  if (rc != GCGE_CUDA_OK) {
    c.release();
    return rc;
  }
  *C = view_of(c);
  return GCGE_CUDA_OK;
}

int identity(int n, View* I, cudaStream_t st) {
  View v;
  v.rows = v.cols = v.nnz = n;
  int rc = dalloc(&v.rp, (size_t)n + 1);
  if (rc == GCGE_CUDA_OK) rc = dalloc(&v.ci, (size_t)n);
  if (rc == GCGE_CUDA_OK) rc = dalloc(&v.v, (size_t)n);
  if (rc != GCGE_CUDA_OK) {
    free_view(v);
    return rc;
  }
  k_identity<<<(n + 256) / 256, 256, 0, st>>>(n, v.rp, v.ci, v.v);
  if (cudaGetLastError() != cudaSuccess) {
    free_view(v);
    return gcge_record_error(GCGE_CUDA_ERR_CUDA, "AMG: identity kernel failed");
  }
  *I = v;
  return GCGE_CUDA_OK;
}

void free_view(View& v) {
  cudaFree(v.rp);
  cudaFree(v.ci);
  cudaFree(v.v);
  v = View();
}

void set_pcg(GCGE_CUDA_AMG* a, int max_it, double rate, int* old_max_it, double* old_rate) {
  std::lock_guard<std::mutex> lk(g_amg_mu);
  if (old_max_it) *old_max_it = a->prm.pcg_max_it;
  if (old_rate) *old_rate = a->prm.pcg_rate;
  a->prm.pcg_max_it = max_it;
  a->prm.pcg_rate = rate;
}

}  // namespace amg
}  // namespace gcge
