// Small dense kernels of the GCG iteration (projected matrices of order
// ldm <= nev + 20 + 2*block_size, Gram blocks of order <= block_size):
//   * dgemm_small: thread-per-entry C = alpha op(A) op(B) + beta C, with an
//     option to read A as a symmetric matrix from its upper triangle (dsymm);
//   * the subspace eigensolver: cyclic two-sided Jacobi with a parallel
//     round-robin pair ordering, one CTA, matrix staged in shared memory;
//   * in-subspace Gram-Schmidt with zero-column dropping (P coefficients);
//   * Cholesky of a Gram block with zero-column dropping and the inverse
//     factor (the CholQR step of the W orthonormalisation).
// All arithmetic is FP64.
#include <math.h>

#include "gcge_cuda_common.cuh"
#include "gcge_cuda_dense.cuh"

namespace gcge {
namespace {

__global__ void k_dgemm_small(int ta, int tb, int symA, int m, int n, int k, double alpha,
                              const double* __restrict__ A, int lda, const double* __restrict__ B,
                              int ldb, double beta, double* __restrict__ C, int ldc) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m * n) return;
  const int i = e % m, j = e / m;
  double s = 0.0;
  for (int l = 0; l < k; l++) {
    double a;
    if (symA) a = (i <= l) ? A[i + (size_t)l * lda] : A[l + (size_t)i * lda];
    else a = ta ? A[l + (size_t)i * lda] : A[i + (size_t)l * lda];
    const double b = tb ? B[j + (size_t)l * ldb] : B[l + (size_t)j * ldb];
    s = fma(a, b, s);
  }
  double* c = C + i + (size_t)j * ldc;
  *c = (beta == 0.0) ? alpha * s : fma(beta, *c, alpha * s);
}

// ------------------------------------------------------------ Jacobi
// Round-robin (circle method) pair k of round r for m players (m even):
// (m-1, r) and ((r+k) mod (m-1), (r-k) mod (m-1)).
__device__ inline void rr_pair(int m, int r, int k, int* p, int* q) {
  int a, b;
  if (k == 0) {
    a = m - 1;
    b = r;
  } else {
    a = (r + k) % (m - 1);
    b = (r - k + (m - 1)) % (m - 1);
  }
  *p = a < b ? a : b;
  *q = a < b ? b : a;
}

__device__ inline double block_sum1024(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += sh[w];
  __syncthreads();
  return s;  // every thread gets the sum
}

// a: nrows x nrows (lda), upper triangle read.  Cyclic two-sided Jacobi in
// precision T with a parallel round-robin ordering (npairs disjoint rotations
// per round), stopping when a whole sweep finds every off-diagonal entry
// below tol * sqrt(|a_pp a_qq|); rotated entries are set to exactly 0.
// mode 0: eigenvalues il..iu (1-based, ascending) to eval[0..] and their
//         eigenvectors to evec (lde), sign fixed so the largest-magnitude
//         entry is positive;
// mode 1: all nrows eigenvectors, unsorted, to evec (lde) (a preconditioning
//         basis for the FP64 pass).
// work: global scratch of 2*mp*mp T.  use_smem 1: M and Q in shared memory;
// 2: M in shared memory, Q in work; 0: both in work.  status[0] = sweeps used
// (or -1 if not converged).
template <typename T>
__global__ void __launch_bounds__(1024, 1)
    k_jacobi(int nrows, const double* __restrict__ a, int lda, double* __restrict__ eval,
             double* __restrict__ evec, int lde, int il, int iu, T* __restrict__ work,
             int use_smem, int* __restrict__ status, int mode, double tol, int max_sweeps,
             const unsigned char* __restrict__ mask, const double* __restrict__ norm_ptr) {
  extern __shared__ __align__(16) unsigned char dyn_raw[];
  __shared__ double red[32];
  __shared__ T cs[128], sn[128];
  __shared__ int rank_of[256];
  __shared__ unsigned char rot[128];
  const int m = nrows;
  const int mp = (m % 2) ? m + 1 : m;  // padded player count
  T* M = use_smem ? reinterpret_cast<T*>(dyn_raw) : work;
  T* Q = use_smem == 2 ? work : M + (size_t)mp * mp;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < mp * mp; e += nt) {
    const int i = e % mp, j = e / mp;
    double v = 0.0;
    if (i < m && j < m) v = (i <= j) ? a[i + (size_t)j * lda] : a[j + (size_t)i * lda];
    M[e] = (T)v;
    Q[e] = (i == j) ? T(1) : T(0);
  }
  __syncthreads();
  double tot = 0.0;
  for (int e = tid; e < m * m; e += nt) {
    const int i = e % m, j = e / m;
    const double v = (double)M[i + (size_t)j * mp];
    tot += v * v;
  }
  tot = block_sum1024(tot, red);
  // pair table of the current round, rotation parameters and flags
  __shared__ short pp_[128], qq_[128];
  int sweep = 0;
  bool converged = false;
  const int npairs = mp / 2;
  const int warp = tid >> 5, lane = tid & 31, nwarps = nt >> 5;
  for (; sweep < max_sweeps; sweep++) {
    int did = 0;
    for (int r = 0; r < mp - 1; r++) {
      // parameters of the npairs disjoint rotations of this round
      for (int k = tid; k < npairs; k += nt) {
        int p, q;
        rr_pair(mp, r, k, &p, &q);
        T c = T(1), s = T(0);
        unsigned char doit = 0;
        if (q < m) {
          const T apq = M[p + (size_t)q * mp];
          const T app = M[p + (size_t)p * mp], aqq = M[q + (size_t)q * mp];
          // with a mask (the refinement's clustered pairs) the other pairs
          // rotate only if a coupling above 1e-14 ||A||_F is left
          bool big;
          if (!mask || mask[p + (size_t)q * m])
            big = fabs((double)apq) > tol * sqrt(fabs((double)app) * fabs((double)aqq));
          else
            big = fabs((double)apq) > 1e-14 * norm_ptr[0];
          if (fabs((double)apq) > 1e-300 && big) {
            const T theta = (aqq - app) / (T(2) * apq);
            const T t = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + sqrt(theta * theta + T(1)));
            c = T(1) / sqrt(t * t + T(1));
            s = t * c;
            doit = 1;
            did = 1;
          }
        }
        pp_[k] = (short)p;
        qq_[k] = (short)q;
        cs[k] = c;
        sn[k] = s;
        rot[k] = doit;
      }
      __syncthreads();
      // rows p, q of M (M <- J^T M): a warp per pair, lanes along the row
      for (int k = warp; k < npairs; k += nwarps) {
        if (!rot[k]) continue;
        const int p = pp_[k], q = qq_[k];
        const T c = cs[k], s = sn[k];
        for (int j = lane; j < m; j += 32) {
          const T mp_ = M[p + (size_t)j * mp], mq = M[q + (size_t)j * mp];
          M[p + (size_t)j * mp] = c * mp_ - s * mq;
          M[q + (size_t)j * mp] = s * mp_ + c * mq;
        }
      }
      __syncthreads();
      // columns p, q of M and Q (M <- M J, Q <- Q J)
      for (int k = warp; k < npairs; k += nwarps) {
        if (!rot[k]) continue;
        const int p = pp_[k], q = qq_[k];
        const T c = cs[k], s = sn[k];
        T* Mp = M + (size_t)p * mp;
        T* Mq = M + (size_t)q * mp;
        T* Qp = Q + (size_t)p * mp;
        T* Qq = Q + (size_t)q * mp;
        for (int i = lane; i < m; i += 32) {
          const T a1 = Mp[i], a2 = Mq[i];
          Mp[i] = c * a1 - s * a2;
          Mq[i] = s * a1 + c * a2;
          const T q1 = Qp[i], q2 = Qq[i];
          Qp[i] = c * q1 - s * q2;
          Qq[i] = s * q1 + c * q2;
        }
        if (lane == 0) {  // the annihilated entries are exactly zero
          Mp[q] = T(0);
          Mq[p] = T(0);
        }
      }
      __syncthreads();
    }
    if (!__syncthreads_or(did)) {
      converged = true;
      break;
    }
  }
  if (!converged) {
    // accept a result whose off-diagonal part is negligible anyway
    double off = 0.0;
    for (int e = tid; e < m * m; e += nt) {
      const int i = e % m, j = e / m;
      if (i != j) {
        const double v = (double)M[i + (size_t)j * mp];
        off += v * v;
      }
    }
    off = block_sum1024(off, red);
    converged = off <= (mode == 1 ? 1e-10 : 1e-28) * tot;
  }
  if (mode == 1) {
    for (int e = tid; e < m * m; e += nt) {
      const int i = e % m, j = e / m;
      evec[i + (size_t)j * lde] = (double)Q[i + (size_t)j * mp];
    }
    if (tid == 0) status[0] = converged ? sweep : -1;
    return;
  }
  // ascending order by rank under a strict total order: NaN sorts as +inf
  // and ties break by index, so rank_of is always a permutation of 0..m-1
  for (int i = tid; i < m; i += nt) {
    double di = (double)M[i + (size_t)i * mp];
    if (di != di) di = INFINITY;
    int rk = 0;
    for (int j = 0; j < m; j++) {
      double dj = (double)M[j + (size_t)j * mp];
      if (dj != dj) dj = INFINITY;
      if (dj < di || (dj == di && j < i)) rk++;
    }
    rank_of[rk] = i;
  }
  __syncthreads();
  const int nout = iu - il + 1;
  for (int kk = tid; kk < nout; kk += nt)
    eval[kk] = (double)M[rank_of[il - 1 + kk] * (size_t)(mp + 1)];
  // eigenvector columns, sign fixed so the largest-magnitude entry is positive
  const int nw = nwarps;
  for (int kk = warp; kk < nout; kk += nw) {
    const int c = rank_of[il - 1 + kk];
    double best = -1.0, bv = 0.0;
    int bi = m;
    for (int i = lane; i < m; i += 32) {
      const double v = (double)Q[i + (size_t)c * mp];
      if (fabs(v) > best || (fabs(v) == best && i < bi)) {
        best = fabs(v);
        bv = v;
        bi = i;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_down_sync(0xffffffffu, best, o);
      const double ov = __shfl_down_sync(0xffffffffu, bv, o);
      const int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bv = ov;
        bi = oi;
      }
    }
    bv = __shfl_sync(0xffffffffu, bv, 0);
    const double sg = bv < 0 ? -1.0 : 1.0;
    for (int i = lane; i < m; i += 32)
      evec[i + (size_t)kk * lde] = sg * (double)Q[i + (size_t)c * mp];
  }
  if (tid == 0) status[0] = converged ? sweep : -1;
}

// ------------------------------------------------------------ subspace MGS
// Orthonormalise columns [start, *end) of V (nrows x ldV, Euclidean inner
// product) against each other, two Gram-Schmidt passes per column; a column
// whose norm after projection is <= tol is dropped by moving the last
// column into its place (GCGE_MultiOrthonormalizationInSubspace semantics,
// src/gcge_orthogonal.c:2278-2352).  Writes the new end to *end_out.
__global__ void __launch_bounds__(256) k_sub_mgs(double* __restrict__ V, int ldV, int nrows,
                                                 int start, int end, double tol,
                                                 int* __restrict__ end_out) {
  __shared__ double red[32];
  __shared__ double proj[256];
  const int tid = threadIdx.x, nt = blockDim.x;
  int cur = start;
  while (cur < end) {
    double* v = V + (size_t)cur * ldV;
    for (int pass = 0; pass < 2; pass++) {
      // projections onto the kept columns start..cur-1 (classical GS, one warp each)
      const int warp = tid >> 5, lane = tid & 31;
      for (int j = start + warp; j < cur; j += nt >> 5) {
        const double* u = V + (size_t)j * ldV;
        double s = 0.0;
        for (int i = lane; i < nrows; i += 32) s = fma(u[i], v[i], s);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) proj[j - start] = s;
      }
      __syncthreads();
      for (int i = tid; i < nrows; i += nt) {
        double x = v[i];
        for (int j = start; j < cur; j++) x = fma(-proj[j - start], V[i + (size_t)j * ldV], x);
        v[i] = x;
      }
      __syncthreads();
    }
    double s = 0.0;
    for (int i = tid; i < nrows; i += nt) s = fma(v[i], v[i], s);
    s = block_sum1024(s, red);
    const double nv = sqrt(s);
    if (nv > tol) {
      for (int i = tid; i < nrows; i += nt) v[i] *= 1.0 / nv;
      __syncthreads();
      cur++;
    } else {
      // move the last column into cur and shrink
      const double* last = V + (size_t)(end - 1) * ldV;
      if (cur < end - 1)
        for (int i = tid; i < nrows; i += nt) v[i] = last[i];
      __syncthreads();
      end--;
    }
  }
  if (tid == 0) *end_out = end;
}

// ------------------------------------------------------------ Cholesky
// G: k x k Gram block (ldg).  Right-looking Cholesky G = R^T R in column
// order; a pivot <= tol^2 drops that column (MGS zero-vector semantics of
// GCGE_SubOrthonormalizationSelfBGS, src/gcge_orthogonal.c:2180-2263).
// Outputs kept[0..nk) (original indices, ascending), *nk_out, and
// T = R^{-1} restricted to the kept columns (nk x nk, ldt = k).
__global__ void __launch_bounds__(256) k_chol_drop(int k, const double* __restrict__ G, int ldg,
                                                   double tol2, double* __restrict__ T,
                                                   int* __restrict__ kept,
                                                   int* __restrict__ nk_out,
                                                   double* __restrict__ gwork) {
  extern __shared__ double sm[];
  // k x k working copy and k x k upper factor (rows of kept pivots): in shared
  // memory, or in gwork when 2 k^2 doubles do not fit
  double* M = gwork ? gwork : sm;
  double* R = M + k * k;
  __shared__ int keep[GCGE_MAXCOLS];
  __shared__ int pos[GCGE_MAXCOLS];
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < k * k; e += nt) {
    const int i = e % k, j = e / k;
    M[e] = G[i + (size_t)j * ldg];
    R[e] = 0.0;
  }
  __syncthreads();
  for (int j = 0; j < k; j++) {
    const double d = M[j + j * k];
    const bool ok = d > tol2;  // false for NaN too
    if (tid == 0) keep[j] = ok ? 1 : 0;
    if (ok) {
      const double r = sqrt(d);
      for (int i = j + tid; i < k; i += nt) R[j + i * k] = (i == j) ? r : M[j + i * k] / r;
      __syncthreads();
      for (int e = tid; e < k * k; e += nt) {
        const int a = e % k, b = e / k;
        if (a > j && b > j) M[e] -= R[j + a * k] * R[j + b * k];
      }
    }
    __syncthreads();
  }
  if (tid == 0) {
    int nk = 0;
    for (int j = 0; j < k; j++) {
      pos[j] = keep[j] ? nk : -1;
      if (keep[j]) kept[nk++] = j;
    }
    *nk_out = nk;
    pos[GCGE_MAXCOLS - 1] = nk;
  }
  __syncthreads();
  const int nk = pos[GCGE_MAXCOLS - 1];
  // T = R_kept^{-1}: thread per column c solves R x = e_c by back substitution
  for (int c = tid; c < nk; c += nt) {
    for (int rI = nk - 1; rI >= 0; rI--) {
      double x = (rI == c) ? 1.0 : 0.0;
      const int gr = kept[rI];
      for (int l = rI + 1; l <= c; l++) x -= R[gr + kept[l] * k] * T[l + (size_t)c * k];
      T[rI + (size_t)c * k] = (rI > c) ? 0.0 : x / R[gr + gr * k];
    }
  }
}

// dst[:, j] rows [0, rows) <- src column idx[j] rows [r0, r0+rows); used to
// build the P coefficient block from the unconverged Ritz coefficient
// columns (GCGE_ComputeP, src/gcge_xpw.c:371-383).
__global__ void k_gather_cols(const double* __restrict__ src, int lds, int r0, int rows,
                              IntList idx, int ncols, double* __restrict__ dst, int ldd) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= rows * ncols) return;
  const int i = e % rows, j = e / rows;
  dst[i + (size_t)j * ldd] = src[r0 + i + (size_t)idx.v[j] * lds];
}

__global__ void k_set_diag(double* __restrict__ M, int ld, const double* __restrict__ d, int k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) M[i + (size_t)i * ld] = d[i];
}

__global__ void k_add_diag(double* __restrict__ M, int ld, double s, int k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) M[i + (size_t)i * ld] += s;
}

__global__ void k_sqrt_div(const double* __restrict__ r2, const double* __restrict__ x2,
                           double* __restrict__ out, int k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) out[i] = sqrt(r2[i]) / sqrt(x2[i]);
}

}  // namespace

void dgemm_small(bool ta, bool tb, bool symA, int m, int n, int k, double alpha, const double* A,
                 int lda, const double* B, int ldb, double beta, double* C, int ldc,
                 cudaStream_t st) {
  if (m <= 0 || n <= 0) return;
  const int tot = m * n;
  k_dgemm_small<<<(tot + 127) / 128, 128, 0, st>>>(ta, tb, symA, m, n, k, alpha, A, lda, B, ldb,
                                                   beta, C, ldc);
}

size_t jacobi_smem_bytes(int nrows) {
  const int mp = (nrows % 2) ? nrows + 1 : nrows;
  return sizeof(double) * 2 * (size_t)mp * mp;
}

// Final stage of jacobi_eig.  After the refinement, S = X^T A X is diagonal
// up to couplings below 1e-14 ||A||_F except between pairs the refinement
// marked as clustered.  Rather than sweeping all m(m-1)/2 pairs (m - 1 rounds
// of block-wide barriers per sweep), the clusters -- connected components of
// the marked pairs and of any coupling still above 1e-14 ||A||_F -- are solved
// independently, one warp each, by cyclic FP64 Jacobi on their principal
// submatrix; Z is block diagonal.  Same rotation formula, thresholds and
// output order as k_jacobi (mode 0): eigenvalues il..iu ascending (NaN last,
// ties by index), eigenvector columns signed so the largest-magnitude entry is
// positive.  work: 2 m^2 doubles (each cluster of size c > 1 takes 2 c^2:
// its submatrix and its eigenvectors).  One CTA; status[0] = sweeps of the
// slowest cluster, or -1 if a cluster did not converge.
__global__ void __launch_bounds__(1024, 1)
    k_cluster_jacobi(int m, const double* __restrict__ S, const unsigned char* __restrict__ mask,
                     const double* __restrict__ normA, double* __restrict__ eval,
                     double* __restrict__ Z, int ldz, int il, int iu, double* __restrict__ work,
                     int* __restrict__ status, double tol, int max_sweeps) {
  __shared__ int label[256], order[256], cstart[257], rank_of[256], cl[256], cpos[256];
  __shared__ size_t coff[257];
  __shared__ int ncl, worst;
  __shared__ double d[256];
  const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31;
  const double thr = 1e-14 * normA[0];
  for (int i = tid; i < m; i += nt) label[i] = i;
  if (tid == 0) worst = 0;
  __syncthreads();
  // connected components by min-label propagation (at most m rounds; the
  // exit test is a block-wide vote, so every thread leaves the loop together)
  for (int round = 0; round < m; round++) {
    int mine = 0;
    for (int e = tid; e < m * m; e += nt) {
      const int i = e % m, j = e / m;
      if (i >= j) continue;
      if (!(mask[e] || fabs(S[e]) > thr)) continue;
      const int a = label[i], b = label[j];
      if (a != b) {
        const int l = a < b ? a : b;
        atomicMin(&label[i], l);
        atomicMin(&label[j], l);
        mine = 1;
      }
    }
    __syncthreads();
    for (int i = tid; i < m; i += nt) {  // pointer jumping
      int l = label[i];
      while (label[l] != l) l = label[l];
      label[i] = l;
    }
    if (!__syncthreads_or(mine)) break;
  }
  // group the members of each cluster, in index order (serial: m <= 256)
  if (tid == 0) {
    int nc = 0, pos = 0;
    size_t off = 0;
    for (int r = 0; r < m; r++) {
      if (label[r] != r) continue;
      cstart[nc] = pos;
      coff[nc] = off;
      for (int i = r; i < m; i++)
        if (label[i] == r) {
          cl[i] = nc;
          cpos[i] = pos - cstart[nc];
          order[pos++] = i;
        }
      const size_t sz = (size_t)(pos - cstart[nc]);
      if (sz > 1) off += 2 * sz * sz;
      nc++;
    }
    cstart[nc] = pos;
    coff[nc] = off;
    ncl = nc;
  }
  __syncthreads();
  for (int i = tid; i < m; i += nt) d[i] = S[i + (size_t)i * m];
  // one warp per cluster of size > 1
  for (int c = warp; c < ncl; c += nt >> 5) {
    const int b0 = cstart[c], sz = cstart[c + 1] - b0;
    if (sz == 1) continue;
    // this cluster's submatrix (from the upper triangle) and eigenvectors
    double* A = work + coff[c];
    double* V = A + (size_t)sz * sz;
    for (int e = lane; e < sz * sz; e += 32) {
      const int a = e % sz, b = e / sz;
      const int ia = order[b0 + a], ib = order[b0 + b];
      A[e] = (ia <= ib) ? S[ia + (size_t)ib * m] : S[ib + (size_t)ia * m];
      V[e] = (a == b) ? 1.0 : 0.0;
    }
    __syncwarp();
    int sweep = 0;
    bool conv = false;
    for (; sweep < max_sweeps; sweep++) {
      int did = 0;
      for (int p = 0; p < sz - 1; p++)
        for (int q = p + 1; q < sz; q++) {
          const double apq = A[p + q * sz], app = A[p + p * sz], aqq = A[q + q * sz];
          if (!(fabs(apq) > 1e-300 && fabs(apq) > tol * sqrt(fabs(app) * fabs(aqq)))) continue;
          const double theta = (aqq - app) / (2.0 * apq);
          const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
          const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
          did = 1;
          __syncwarp();
          for (int j = lane; j < sz; j += 32) {  // rows p, q
            const double x = A[p + j * sz], y = A[q + j * sz];
            A[p + j * sz] = cs * x - sn * y;
            A[q + j * sz] = sn * x + cs * y;
          }
          __syncwarp();
          for (int i = lane; i < sz; i += 32) {  // columns p, q of A and V
            const double x = A[i + p * sz], y = A[i + q * sz];
            A[i + p * sz] = cs * x - sn * y;
            A[i + q * sz] = sn * x + cs * y;
            const double v1 = V[i + p * sz], v2 = V[i + q * sz];
            V[i + p * sz] = cs * v1 - sn * v2;
            V[i + q * sz] = sn * v1 + cs * v2;
          }
          __syncwarp();
          if (lane == 0) {
            A[q + p * sz] = 0.0;
            A[p + q * sz] = 0.0;
          }
          __syncwarp();
        }
      if (!did) {
        conv = true;
        break;
      }
    }
    for (int a = lane; a < sz; a += 32) d[order[b0 + a]] = A[a + a * sz];
    if (lane == 0) atomicMax(&worst, conv ? sweep : 1 << 20);
  }
  __syncthreads();
  // ascending order by rank (NaN as +inf, ties by index)
  for (int i = tid; i < m; i += nt) {
    double di = d[i];
    if (di != di) di = INFINITY;
    int rk = 0;
    for (int j = 0; j < m; j++) {
      double dj = d[j];
      if (dj != dj) dj = INFINITY;
      if (dj < di || (dj == di && j < i)) rk++;
    }
    rank_of[rk] = i;
  }
  __syncthreads();
  const int nout = iu - il + 1;
  for (int kk = tid; kk < nout; kk += nt) eval[kk] = d[rank_of[il - 1 + kk]];
  // eigenvector of index c: column cpos[c] of its cluster's V on the
  // cluster's rows (e_c for a singleton), zero elsewhere
  auto zval = [&](int i, int c) -> double {
    const int k = cl[c];
    if (cl[i] != k) return 0.0;
    const int sz = cstart[k + 1] - cstart[k];
    if (sz == 1) return 1.0;
    const double* V = work + coff[k] + (size_t)sz * sz;
    return V[cpos[i] + (size_t)cpos[c] * sz];
  };
  for (int kk = warp; kk < nout; kk += nt >> 5) {
    const int c = rank_of[il - 1 + kk];
    double best = -1.0, bv = 0.0;
    int bi = m;
    for (int i = lane; i < m; i += 32) {
      const double v = zval(i, c);
      if (fabs(v) > best || (fabs(v) == best && i < bi)) {
        best = fabs(v);
        bv = v;
        bi = i;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_down_sync(0xffffffffu, best, o);
      const double ov = __shfl_down_sync(0xffffffffu, bv, o);
      const int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bv = ov;
        bi = oi;
      }
    }
    bv = __shfl_sync(0xffffffffu, bv, 0);
    const double sg = bv < 0 ? -1.0 : 1.0;
    for (int i = lane; i < m; i += 32) Z[i + (size_t)kk * ldz] = sg * zval(i, c);
  }
  if (tid == 0) status[0] = worst >= (1 << 20) ? -1 : worst;
}

template <typename T>
static void launch_jacobi(int nrows, const double* a, int lda, double* eval, double* evec, int lde,
                          int il, int iu, T* work, int* status, int mode, double tol,
                          int max_sweeps, cudaStream_t st, const unsigned char* mask = nullptr,
                          const double* norm_ptr = nullptr) {
  const int mp = (nrows % 2) ? nrows + 1 : nrows;
  // the rotated matrix in shared memory whenever it fits (its rows and columns
  // are read every round), the eigenvector accumulator too if there is room
  constexpr size_t kCap = 220 * 1024;  // dynamic shared memory left beside the static arrays
  const size_t one = sizeof(T) * (size_t)mp * mp;
  const int use_smem = 2 * one <= kCap ? 1 : (one <= kCap ? 2 : 0);
  if (use_smem) {
    const size_t sm = use_smem == 1 ? 2 * one : one;
    cudaFuncSetAttribute(k_jacobi<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_jacobi<T><<<1, 1024, sm, st>>>(nrows, a, lda, eval, evec, lde, il, iu, work, use_smem,
                                     status, mode, tol, max_sweeps, mask, norm_ptr);
  } else {
    k_jacobi<T><<<1, 1024, 0, st>>>(nrows, a, lda, eval, evec, lde, il, iu, work, 0, status, mode,
                                    tol, max_sweeps, mask, norm_ptr);
  }
}

// One step of the Ogita-Aishima refinement of an approximate eigenvector
// basis X of a symmetric A (Japan J. Indust. Appl. Math. 35 (2018)
// 1007-1035, Algorithm 1), given S = X^T A X and R = I - X^T X:
//   l_i = s_ii / (1 - r_ii),  delta = 2 (||S - diag(l)|| + ||A|| ||R||),
//   E_ij = (s_ij + l_j r_ij) / (l_j - l_i)  if |l_i - l_j| > delta
//        = r_ij / 2                          otherwise (and on the diagonal),
// after which X <- X + X E.  Frobenius norms stand in for 2-norms (larger
// delta: safe); ||A|| is read from device memory.  Pairs within delta are
// "clustered": on the first step the mask records them and later steps keep
// treating them as clustered; the final FP64 Jacobi rotates exactly those
// pairs.  One CTA.
__global__ void __launch_bounds__(1024) k_oa_step_dev(int m, const double* __restrict__ S,
                                                      const double* __restrict__ R,
                                                      const double* __restrict__ normA, int first,
                                                      unsigned char* __restrict__ mask,
                                                      double* __restrict__ E);

__global__ void k_eye_minus(double* __restrict__ R, int m) {
  // R <- I - R  (R holds X^T X on entry)
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m * m) return;
  const int i = e % m, j = e / m;
  R[e] = (i == j ? 1.0 : 0.0) - R[e];
}

__global__ void __launch_bounds__(1024) k_frob_sym(int m, const double* __restrict__ a, int lda,
                                                   double* __restrict__ out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
    const int i = e % m, j = e / m;
    const double v = (i <= j) ? a[i + (size_t)j * lda] : a[j + (size_t)i * lda];
    s += v * v;
  }
  s = block_sum1024(s, red);
  if (threadIdx.x == 0) out[0] = sqrt(s);
}

__global__ void __launch_bounds__(1024) k_oa_step_dev(int m, const double* __restrict__ S,
                                                      const double* __restrict__ R,
                                                      const double* __restrict__ normA, int first,
                                                      unsigned char* __restrict__ mask,
                                                      double* __restrict__ E) {
  __shared__ double lam[256];
  __shared__ double red[32];
  const int tid = threadIdx.x, nt = blockDim.x;
  const double nA = normA[0];
  for (int i = tid; i < m; i += nt) lam[i] = S[i + (size_t)i * m] / (1.0 - R[i + (size_t)i * m]);
  __syncthreads();
  double s2 = 0.0, r2 = 0.0;
  for (int e = tid; e < m * m; e += nt) {
    const int i = e % m, j = e / m;
    const double sv = S[e] - (i == j ? lam[i] : 0.0);
    s2 += sv * sv;
    r2 += R[e] * R[e];
  }
  s2 = block_sum1024(s2, red);
  r2 = block_sum1024(r2, red);
  const double delta = 2.0 * (sqrt(s2) + nA * sqrt(r2));
  for (int e = tid; e < m * m; e += nt) {
    const int i = e % m, j = e / m;
    double v;
    if (i == j) {
      v = 0.5 * R[e];
    } else {
      bool clustered;
      if (first) {
        clustered = !(fabs(lam[i] - lam[j]) > delta);  // NaN -> clustered
        mask[e] = clustered ? 1 : 0;
      } else {
        clustered = mask[e] != 0;
      }
      v = clustered ? 0.5 * R[e] : (S[e] + lam[j] * R[e]) / (lam[j] - lam[i]);
    }
    E[e] = v;
  }
}

void jacobi_eig(int nrows, const double* a, int lda, double* eval, double* evec, int lde, int il,
                int iu, double* work, int* status, cudaStream_t st) {
  if (nrows <= 0) return;
  const int m = nrows;
  if (m <= 16) {
    launch_jacobi<double>(m, a, lda, eval, evec, lde, il, iu, work, status, 0, 1e-15, 60, st);
    return;
  }
  // 1. FP32 Jacobi: a basis X of eigenvectors to single precision
  // 2. three Ogita-Aishima refinement steps in FP64 (matrix products only)
  // 3. S = X^T A X is diagonal to rounding except inside clusters of close
  //    eigenvalues; an FP64 Jacobi restricted to the clustered pairs
  //    finishes it and sorts; eigenvectors = X * (its eigenvectors)
  const size_t mm = (size_t)m * m;
  double* X = work;
  double* AX = X + mm;
  double* S = AX + mm;
  double* R = S + mm;
  double* E = R + mm;
  double* Z = E + mm;
  double* nrm = Z + mm;                                         // 8 doubles
  unsigned char* mask = reinterpret_cast<unsigned char*>(nrm + 8);  // m*m bytes
  void* jw = nrm + 8 + (mm + 7) / 8;                            // Jacobi scratch
  launch_jacobi<float>(m, a, lda, eval, X, m, 1, m, (float*)jw, status, 1, 2e-7, 20, st);
  k_frob_sym<<<1, 1024, 0, st>>>(m, a, lda, nrm);
  double* normA_dev = nrm;
  for (int it = 0; it < 3; it++) {
    dgemm_small(false, false, true, m, m, m, 1.0, a, lda, X, m, 0.0, AX, m, st);
    dgemm_small(true, false, false, m, m, m, 1.0, X, m, AX, m, 0.0, S, m, st);
    dgemm_small(true, false, false, m, m, m, 1.0, X, m, X, m, 0.0, R, m, st);
    k_eye_minus<<<(int)((mm + 255) / 256), 256, 0, st>>>(R, m);
    k_oa_step_dev<<<1, 1024, 0, st>>>(m, S, R, normA_dev, it == 0 ? 1 : 0, mask, E);
    // X <- X + X E
    cudaMemcpyAsync(AX, X, sizeof(double) * mm, cudaMemcpyDeviceToDevice, st);
    dgemm_small(false, false, false, m, m, m, 1.0, AX, m, E, m, 1.0, X, m, st);
  }
  dgemm_small(false, false, true, m, m, m, 1.0, a, lda, X, m, 0.0, AX, m, st);
  dgemm_small(true, false, false, m, m, m, 1.0, X, m, AX, m, 0.0, S, m, st);
  // the masked round-robin Jacobi while the matrix and the rotations fit in
  // shared memory (large clusters parallelise over the whole CTA there); the
  // cluster-wise kernel beyond, where round-robin sweeps would run from global
  // memory
  const int mp = (m % 2) ? m + 1 : m;
  if (sizeof(double) * 2 * (size_t)mp * mp <= 220 * 1024)
    launch_jacobi<double>(m, S, m, eval, Z, m, il, iu, (double*)jw, status, 0, 1e-15, 60, st,
                          mask, normA_dev);
  else
    k_cluster_jacobi<<<1, 1024, 0, st>>>(m, S, mask, normA_dev, eval, Z, m, il, iu, (double*)jw,
                                         status, 1e-15, 60);
  const int nout = iu - il + 1;
  dgemm_small(false, false, false, m, nout, m, 1.0, X, m, Z, m, 0.0, evec, lde, st);
}

size_t jacobi_work_doubles(int nrows) {
  const size_t m = nrows, mp = nrows + 1;
  return 6 * m * m + 8 + (m * m + 7) / 8 + 2 * mp * mp + 16;
}

void sub_mgs(double* V, int ldV, int nrows, int start, int end, double tol, int* end_out,
             cudaStream_t st) {
  k_sub_mgs<<<1, 256, 0, st>>>(V, ldV, nrows, start, end, tol, end_out);
}

void chol_drop(int k, const double* G, int ldg, double tol, double* T, int* kept, int* nk,
               double* work, cudaStream_t st) {
  const size_t sm = sizeof(double) * 2 * (size_t)k * k;
  if (sm > 200 * 1024) {
    k_chol_drop<<<1, 256, 0, st>>>(k, G, ldg, tol * tol, T, kept, nk, work);
    return;
  }
  if (sm > 48 * 1024) cudaFuncSetAttribute(k_chol_drop, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_chol_drop<<<1, 256, sm, st>>>(k, G, ldg, tol * tol, T, kept, nk, nullptr);
}

void gather_cols(const double* src, int lds, int r0, int rows, const IntList& idx, int ncols,
                 double* dst, int ldd, cudaStream_t st) {
  const int tot = rows * ncols;
  if (tot <= 0) return;
  k_gather_cols<<<(tot + 255) / 256, 256, 0, st>>>(src, lds, r0, rows, idx, ncols, dst, ldd);
}

void set_diag(double* M, int ld, const double* d, int k, cudaStream_t st) {
  if (k <= 0) return;
  k_set_diag<<<(k + 127) / 128, 128, 0, st>>>(M, ld, d, k);
}

void add_diag(double* M, int ld, double s, int k, cudaStream_t st) {
  if (k <= 0) return;
  k_add_diag<<<(k + 127) / 128, 128, 0, st>>>(M, ld, s, k);
}

void sqrt_div(const double* r2, const double* x2, double* out, int k, cudaStream_t st) {
  if (k <= 0) return;
  k_sqrt_div<<<(k + 127) / 128, 128, 0, st>>>(r2, x2, out, k);
}

}  // namespace gcge
