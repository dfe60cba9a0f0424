/*
 * ORACLE TEST INFRASTRUCTURE — not part of the product.
 *
 * A plain-C restatement of the reference GCG eigensolver iteration
 * (GCGE_Solve and everything under it with the default parameters), used
 * (1) as the CPU checker for the CUDA solver in tests and smoke() and
 * (2) as the timed CPU baseline on machines where the reference itself
 *     cannot be compiled (the GPU host has no reference checkout).
 * It is pinned against the real reference, compiled by oracle/build_ref.sh,
 * by tests/test_oracle.py and the fixtures under tests/golden/.
 *
 * Vectors are length-n double columns; a multivector is an array of column
 * pointers exactly like the reference's default "void**" multivector, so the
 * reference's pointer swaps (src/gcge_ops.c:383-397) stay pointer swaps.
 * Every function cites the reference function it follows.  The dense
 * partial eigensolve (dsyevx in the reference, src/gcge_ops.c:401-553) is a
 * cyclic Jacobi method here; eigenvalues agree with LAPACK to rounding.
 * Large loops carry OpenMP pragmas so the baseline can use the host cores.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <float.h>

typedef struct {
  int n;
  const int* rp;
  const int* ci;
  const double* v;
} port_csr;

typedef struct {
  int nev, block_size, ev_max_it, cg_max_it, max_reorth_time;
  double ev_tol, cg_rate, orth_zero_tol, reorth_tol, scbgs_reorth_tol, multi_tol_for_lock;
  /* shift (src/gcge_para.h:90-92): use_shift recomputes if_shift/shift after
   * every convergence check; if_shift/shift set by hand give a fixed shift.
   * eval_sm: eval_type "sm" (smallest magnitude) instead of "sa". */
  int use_shift, if_shift, eval_sm;
  double shift;
  /* mixed: the W step of the CUDA solver's mixed precision (not part of the
   * reference): the FP64 residual r = rhs - A w0 of the scaled start w0, the
   * block CG on A e = r in FP32 from e = 0, and W = e (w0 is a scaled column
   * of X, so [X, P, e] spans the subspace of [X, P, w0 + e]) */
  int mixed;
  /* convergence criterion (src/gcge_eigsol.c:713-721): 0 "R", 1 "O" (divide
   * by conv_omega_norm + |lambda|), 2 absolute */
  int conv_type;
  double conv_omega_norm;
} port_para;

typedef struct {
  int n, nev, bs, max_dim_x, V_size, V_tmp_size;
  int dim_x, dim_xp, dim_xpw, last_dim_x, last_dim_xpw, unconv_bs;
  int num_soft_locked_in_last_iter;
  double **V, **V_tmp, **CG_p, **evec;
  double *sub_mat, *sub_evec, *sub_dtmp, *eval, *res;
  int *unlock, *itmp;
  int num_iter, num_unlock, num_conv_continuous;
  double* Bx; /* B x of the shifted block-CG operator */
  float *a32, *b32, *f_r, *f_x, *f_p, *f_w; /* mixed: FP32 values and block-CG columns */
  port_para p;
  const port_csr *A, *B;
  long long spmv_count;
} port_ws;

/* ---------------- vector kernels (app/csr/gcge_app_csr.c:297-378) -------- */
static void spmv(const port_csr* M, const double* x, double* y, port_ws* w) {
  const int n = M->n;
  w->spmv_count++;
#pragma omp parallel for schedule(static) if (n > 32768)
  for (int i = 0; i < n; i++) {
    double s = 0.0;
    for (int k = M->rp[i]; k < M->rp[i + 1]; k++) s += M->v[k] * x[M->ci[k]];
    y[i] = s;
  }
}
static void axpby(int n, double a, const double* x, double b, double* y) {
  if (a == 0.0) {
#pragma omp parallel for schedule(static) if (n > 32768)
    for (int i = 0; i < n; i++) y[i] = b * y[i];
  } else if (b == 0.0) {
#pragma omp parallel for schedule(static) if (n > 32768)
    for (int i = 0; i < n; i++) y[i] = a * x[i];
  } else {
#pragma omp parallel for schedule(static) if (n > 32768)
    for (int i = 0; i < n; i++) y[i] = a * x[i] + b * y[i];
  }
}
static double dot(int n, const double* x, const double* y) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static) if (n > 32768)
  for (int i = 0; i < n; i++) s += x[i] * y[i];
  return s;
}
/* B*x, or a copy when B is the identity (B == NULL in the reference). */
static void apply_b(port_ws* w, const double* x, double* y) {
  if (w->B) spmv(w->B, x, y, w);
  else memcpy(y, x, sizeof(double) * w->n);
}

/* ---------------- multivector defaults (src/gcge_ops.c:149-309) ---------- */
static void mv_axpby(port_ws* w, double a, double** x, double b, double** y, int s0, int e0,
                     int s1) {
  for (int i = 0; i < e0 - s0; i++) axpby(w->n, a, x[s0 + i], b, y[s1 + i]);
}
/* y[s1+j] = sum_i x[s0+i] a[j*lda+i] + beta*y (GCGE_Default_MultiVecLinearComb). */
static void mv_lincomb(port_ws* w, double** x, double** y, int s0, int e0, int s1, int e1,
                       const double* a, int lda, double beta) {
  const int n = w->n, nx = e0 - s0;
  for (int j = s1; j < e1; j++) {
    const double* aj = a + (size_t)(j - s1) * lda;
    double* yj = y[j];
#pragma omp parallel for schedule(static) if (n > 32768)
    for (int r = 0; r < n; r++) {
      double s = beta == 0.0 ? 0.0 : beta * yj[r];
      for (int i = 0; i < nx; i++) s += aj[i] * x[s0 + i][r];
      yj[r] = s;
    }
  }
}
/* a(iv,iw) = V[s0+iv]^T W[s1+iw]; "sym": upper triangle then mirror
 * (GCGE_Default_MultiVecInnerProd, src/gcge_ops.c:226-309). */
static void mv_inner(port_ws* w, double** V, double** W, double* a, int sym, int s0, int e0,
                     int s1, int e1, int lda) {
  const int n = w->n;
  if (sym) {
    int len = e1 - s1;
    for (int iw = 0; iw < len; iw++)
      for (int iv = 0; iv <= iw; iv++) a[iw * lda + iv] = dot(n, V[iv + s0], W[iw + s1]);
    for (int iw = 0; iw < len; iw++)
      for (int iv = iw + 1; iv < len; iv++) a[iw * lda + iv] = a[iv * lda + iw];
  } else {
    for (int iw = s1; iw < e1; iw++)
      for (int iv = s0; iv < e0; iv++) a[(iw - s1) * lda + (iv - s0)] = dot(n, V[iv], W[iw]);
  }
}
static void mv_swap(double** V1, double** V2, int s0, int e0, int s1) {
  for (int i = 0; i < e0 - s0; i++) {
    double* t = V1[s0 + i];
    V1[s0 + i] = V2[s1 + i];
    V2[s1 + i] = t;
  }
}

/* ---------------- dense helpers ----------------------------------------- */
/* C(m x n) = alpha * op(A) * op(B) + beta*C, column-major (dgemm_ semantics). */
static void dgemm(int ta, int tb, int m, int n, int k, double alpha, const double* A, int lda,
                  const double* Bm, int ldb, double beta, double* C, int ldc) {
  for (int j = 0; j < n; j++)
    for (int i = 0; i < m; i++) {
      double s = 0.0;
      for (int l = 0; l < k; l++) {
        double av = ta ? A[i * lda + l] : A[l * lda + i];
        double bv = tb ? Bm[l * ldb + j] : Bm[j * ldb + l];
        s += av * bv;
      }
      C[j * ldc + i] = (beta == 0.0 ? 0.0 : beta * C[j * ldc + i]) + alpha * s;
    }
}

/* Symmetric eigensolver by cyclic Jacobi rotations.  a: n x n (lda), only
 * read.  Returns all eigenvalues ascending in w and eigenvectors in z
 * (n x n, ldz); stands in for dsyev/dsyevx. */
static void jacobi_eig(int n, const double* a, int lda, double* w, double* z, int ldz) {
  double* m = (double*)malloc(sizeof(double) * n * n);
  double* q = (double*)malloc(sizeof(double) * n * n);
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) {
      /* symmetrise from the upper triangle, as LAPACK with uplo='U' reads */
      m[j * n + i] = (i <= j) ? a[j * lda + i] : a[i * lda + j];
      q[j * n + i] = (i == j) ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 60; sweep++) {
    double off = 0.0, tot = 0.0;
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        double v = m[j * n + i] * m[j * n + i];
        tot += v;
        if (i != j) off += v;
      }
    if (off <= 1e-34 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; p++)
      for (int r = p + 1; r < n; r++) {
        double apr = m[r * n + p];
        if (fabs(apr) < 1e-300) continue;
        double app = m[p * n + p], arr = m[r * n + r];
        double theta = (arr - app) / (2.0 * apr);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; k++) { /* columns p, r */
          double mkp = m[p * n + k], mkr = m[r * n + k];
          m[p * n + k] = c * mkp - s * mkr;
          m[r * n + k] = s * mkp + c * mkr;
        }
        for (int k = 0; k < n; k++) { /* rows p, r */
          double mpk = m[k * n + p], mrk = m[k * n + r];
          m[k * n + p] = c * mpk - s * mrk;
          m[k * n + r] = s * mpk + c * mrk;
        }
        for (int k = 0; k < n; k++) {
          double qkp = q[p * n + k], qkr = q[r * n + k];
          q[p * n + k] = c * qkp - s * qkr;
          q[r * n + k] = s * qkp + c * qkr;
        }
      }
  }
  int* idx = (int*)malloc(sizeof(int) * n);
  for (int i = 0; i < n; i++) idx[i] = i;
  for (int i = 1; i < n; i++) { /* insertion sort by eigenvalue */
    int t = idx[i], j = i - 1;
    while (j >= 0 && m[idx[j] * n + idx[j]] > m[t * n + t]) {
      idx[j + 1] = idx[j];
      j--;
    }
    idx[j + 1] = t;
  }
  for (int k = 0; k < n; k++) {
    int c = idx[k];
    w[k] = m[c * n + c];
    /* fix the sign: largest-magnitude component positive */
    int im = 0;
    for (int i = 1; i < n; i++)
      if (fabs(q[c * n + i]) > fabs(q[c * n + im])) im = i;
    double sg = q[c * n + im] < 0 ? -1.0 : 1.0;
    for (int i = 0; i < n; i++) z[k * ldz + i] = sg * q[c * n + i];
  }
  free(idx);
  free(m);
  free(q);
}

/* DenseMatEigenSolver with 1-based il..iu (GCGE_Default_DenseMatEigenSolver,
 * src/gcge_ops.c:401-553): eigenpairs il..iu of the nrows x nrows matrix a. */
static void dense_eig(double* a, int lda, int nrows, double* eval, double* evec, int lde, int il,
                      int iu) {
  double* w = (double*)malloc(sizeof(double) * nrows);
  double* z = (double*)malloc(sizeof(double) * nrows * nrows);
  jacobi_eig(nrows, a, lda, w, z, nrows);
  for (int k = il - 1; k < iu; k++) {
    eval[k - (il - 1)] = w[k];
    memcpy(evec + (size_t)(k - (il - 1)) * lde, z + (size_t)k * nrows, sizeof(double) * nrows);
  }
  free(w);
  free(z);
}

/* ---------------- orthogonalisation (src/gcge_orthogonal.c) ------------- */
/* GCGE_Orthonormalization, block branch (sum_res == 0 at start), :112-308. */
static void orth_mgs(port_ws* w, double** V, int start, int* end) {
  const int n = w->n;
  double* d = w->sub_dtmp;
  double vin, vout = 0.0, ratio;
  for (int cur = start; cur < *end; ++cur) {
    int reorth = 0;
    do {
      apply_b(w, V[cur], w->V_tmp[0]);
      for (int j = 0; j <= cur; j++) d[j] = dot(n, V[j], w->V_tmp[0]);
      if (cur != 0) {
        mv_lincomb(w, V, w->V_tmp, 0, cur, 0, 1, d, cur, 0.0);
        axpby(n, -1.0, w->V_tmp[0], 1.0, V[cur]);
      }
      vin = sqrt(d[cur]);
      double s = 0.0;
      for (int j = 0; j < cur; j++) s += d[j] * d[j];
      d[cur] = d[cur] - s;
      vout = sqrt(d[cur]);
      ratio = vout / vin;
      reorth++;
    } while (ratio < w->p.reorth_tol && reorth < w->p.max_reorth_time &&
             vout > w->p.orth_zero_tol);
    if (vout > w->p.orth_zero_tol) {
      axpby(n, 0.0, V[cur], 1.0 / vout, V[cur]);
    } else {
      if (cur < *end - 1) mv_swap(V, V, cur, cur + 1, *end - 1);
      (*end)--;
      cur--;
    }
  }
}

/* V2 -= V1 (V1^T B V2) (GCGE_SubOrthonormalization, :2022-2071). */
static void sub_orth(port_ws* w, double** V, int s0, int e0, int s1, int e1) {
  int l1 = e0 - s0, l2 = e1 - s1;
  for (int i = 0; i < l2; i++) apply_b(w, V[s1 + i], w->V_tmp[i]);
  mv_inner(w, V, w->V_tmp, w->sub_dtmp, 0, s0, e0, 0, l2, l1);
  mv_lincomb(w, V, w->V_tmp, s0, e0, 0, l2, w->sub_dtmp, l1, 0.0);
  mv_axpby(w, -1.0, w->V_tmp, 1.0, V, 0, l2, s1);
}

/* GCGE_SubOrthonormalizationSelfBGS, :2180-2263. */
static void self_bgs(port_ws* w, double** V, int start, int* end) {
  const int n = w->n;
  double* d = w->sub_dtmp;
  for (int cur = start; cur < *end; cur++) {
    apply_b(w, V[cur], w->V_tmp[0]);
    int len = *end - cur;
    for (int j = 0; j < len; j++) d[j] = dot(n, V[cur + j], w->V_tmp[0]);
    double nv = sqrt(d[0]);
    if (nv > w->p.orth_zero_tol) {
      axpby(n, 0.0, V[cur], 1.0 / nv, V[cur]);
      for (int j = cur + 1; j < *end; j++) axpby(n, -d[j - cur] / nv, V[cur], 1.0, V[j]);
    } else {
      if (cur < *end - 1) mv_swap(V, V, cur, cur + 1, *end - 1);
      (*end)--;
      cur--;
    }
  }
}

/* GCGE_MultiOrthonormalization (recursive halving), :2087-2178. */
static void multi_orth(port_ws* w, double** V, int start, int* end) {
  int length = *end - start;
  int l1 = length / 2, l2 = length - l1, mid = start + l1;
  if (length <= 1) { /* max_direct_orth_length = 1 */
    self_bgs(w, V, start, end);
    return;
  }
  multi_orth(w, V, start, &mid);
  if (mid + l2 < *end) {
    int new_end2 = mid + l2, nz = *end - new_end2;
    mv_swap(V, V, mid, mid + nz, new_end2);
    *end = new_end2;
  }
  if (mid - start > 0) {
    double vi = 1.0;
    int it = 0;
    while (vi > w->p.scbgs_reorth_tol) {
      it++;
      sub_orth(w, V, start, mid, mid, *end);
      vi = 0.0;
      for (int i = 0; i < l1 * l2; i++) vi += w->sub_dtmp[i] * w->sub_dtmp[i];
      vi = sqrt(vi);
      if (it >= w->p.max_reorth_time) break;
    }
  }
  multi_orth(w, V, mid, end);
}

/* GCGE_StableMultiOrthonormalization(+Partly), :1909-2019.  The W block is
 * never longer than V_tmp here, so the chunked branch is not needed. */
static void stable_multi_orth(port_ws* w, double** V, int start, int* end) {
  if (start > 0) {
    double vi = 1.0;
    int it = 0;
    while (vi > w->p.scbgs_reorth_tol) {
      it++;
      sub_orth(w, V, 0, start, start, *end);
      vi = 0.0;
      for (int i = 0; i < start * (*end - start); i++) vi += w->sub_dtmp[i] * w->sub_dtmp[i];
      vi = sqrt(vi);
      if (it >= w->p.max_reorth_time) break;
    }
  }
  multi_orth(w, V, start, end);
}

/* Dense-coefficient versions (:2278-2395). */
static void multi_orth_in_sub(port_ws* w, double* V, int ldV, int nrows, int start, int* end) {
  int length = *end - start, l1 = length / 2, l2 = length - l1, mid = start + l1;
  if (length == 1) {
    double s = 0.0;
    for (int i = 0; i < nrows; i++) s += V[start * ldV + i] * V[start * ldV + i];
    s = sqrt(s);
    if (s > w->p.orth_zero_tol) {
      for (int i = 0; i < nrows; i++) V[start * ldV + i] *= 1.0 / s;
    } else {
      *end = start;
    }
    return;
  }
  if (length <= 0) return;
  multi_orth_in_sub(w, V, ldV, nrows, start, &mid);
  if (mid + l2 < *end) {
    int new_end2 = mid + l2, nz = *end - new_end2;
    l1 -= nz;
    memcpy(V + mid * ldV, V + new_end2 * ldV, sizeof(double) * nz * ldV);
    *end = new_end2;
  }
  if (l1 > 0) {
    for (int rc = 0; rc < w->p.max_reorth_time; rc++) {
      dgemm(1, 0, l1, l2, nrows, 1.0, V + start * ldV, ldV, V + mid * ldV, ldV, 0.0, w->sub_dtmp,
            l1);
      /* the row count is ldV, not nrows, as in the reference (:2338-2340) */
      dgemm(0, 0, ldV, l2, l1, -1.0, V + start * ldV, ldV, w->sub_dtmp, l1, 1.0, V + mid * ldV,
            ldV);
    }
  }
  multi_orth_in_sub(w, V, ldV, nrows, mid, end);
}
static void stable_multi_orth_in_sub(port_ws* w, double* V, int ldV, int nrows, int start,
                                     int* end) {
  if (start != 0) {
    for (int rc = 0; rc < w->p.max_reorth_time; rc++) {
      int ol = *end - start;
      dgemm(1, 0, start, ol, nrows, 1.0, V, ldV, V + start * ldV, ldV, 0.0, w->sub_dtmp, start);
      /* row count ldV as in the reference (:2386-2388) */
      dgemm(0, 0, ldV, ol, start, -1.0, V, ldV, w->sub_dtmp, start, 1.0, V + start * ldV, ldV);
    }
  }
  multi_orth_in_sub(w, V, ldV, nrows, start, end);
}

/* ---------------- Rayleigh-Ritz (src/gcge_rayleighritz.c) --------------- */
/* GCGE_ComputeSubspaceMatrixVTAW, :40-90; AW goes to evec as scratch. */
static void vtaw(port_ws* w, int start_W, int start_V, int end_V, double* smat) {
  int wl = end_V - start_W, xpl = end_V - wl;
  for (int i = 0; i < wl; i++) spmv(w->A, w->V[start_W + i], w->evec[i], w);
  memset(smat, 0, sizeof(double) * end_V * wl);
  mv_inner(w, w->V, w->evec, smat + start_V, 0, start_V, xpl, 0, wl, end_V);
  mv_inner(w, w->V, w->evec, smat + xpl, 1, start_W, end_V, 0, wl, end_V);
}
/* GCGE_ComputeSubspaceMatrix, :121-190. */
static void compute_subspace_matrix(port_ws* w) {
  int dim_xp = w->dim_xp, ldm = w->dim_xpw;
  double* sm = w->sub_mat;
  if (dim_xp != 0) {
    int lde = w->last_dim_xpw, dim_x = w->dim_x, dim_p = dim_xp - dim_x;
    double* pp = w->sub_evec + dim_x * lde;
    double* aapp = w->sub_dtmp;
    /* AApp = AA_last(sym, upper) * pp */
    for (int j = 0; j < dim_p; j++)
      for (int i = 0; i < lde; i++) {
        double s = 0.0;
        for (int l = 0; l < lde; l++) {
          double a = (i <= l) ? sm[l * lde + i] : sm[i * lde + l];
          s += a * pp[j * lde + l];
        }
        aapp[j * lde + i] = s;
      }
    memset(sm, 0, sizeof(double) * ldm * ldm);
    dgemm(1, 0, dim_p, dim_p, lde, 1.0, pp, lde, aapp, lde, 0.0, sm + dim_x * ldm + dim_x, ldm);
    for (int i = 0; i < dim_x; i++) sm[i * ldm + i] = w->eval[i];
  }
  int start_V = w->num_soft_locked_in_last_iter; /* opt_rr_eig_partly */
  vtaw(w, dim_xp, start_V, ldm, sm + dim_xp * ldm);
  if (w->p.if_shift == 1) /* :181-189 */
    for (int i = 0; i < ldm; i++) sm[i * ldm + i] += w->p.shift;
}

/* GCGE_SortByMagnitude (src/gcge_rayleighritz.c:842-874): in-place quicksort
 * of a[left..right] by |a| with the first element as pivot, carrying idx. */
static void sort_by_magnitude(double* a, int* idx, int left, int right) {
  if (left > right) return;
  int i = left, j = right;
  const int pidx = idx[left];
  const double piv = a[left], pm = fabs(a[left]);
  while (i != j) {
    while (fabs(a[j]) >= pm && j > i) j--;
    if (j > i) {
      idx[i] = idx[j];
      a[i++] = a[j];
    }
    while (fabs(a[i]) <= pm && j > i) i++;
    if (j > i) {
      idx[j] = idx[i];
      a[j--] = a[i];
    }
  }
  a[i] = piv;
  idx[i] = pidx;
  sort_by_magnitude(a, idx, left, i - 1);
  sort_by_magnitude(a, idx, i + 1, right);
}
/* GCGE_ComputeSubspaceEigenpairs, :507-805 (serial branch). */
static void compute_subspace_eigenpairs(port_ws* w) {
  int ldm = w->dim_xpw;
  double* tmp = w->sub_dtmp;
  int s = w->unlock[0];
  int il = s + 1;
  w->num_soft_locked_in_last_iter = s;
  int iu = (w->max_dim_x < ldm) ? w->max_dim_x : ldm;
  if (w->p.eval_sm) iu = ldm; /* :748-751: all pairs, then the smallest |lambda| */
  for (int i = 0; i < w->dim_xpw - w->dim_xp; i++)
    memset(w->sub_mat + (w->dim_xp + i) * ldm, 0, sizeof(double) * s);
  memcpy(tmp, w->sub_mat, sizeof(double) * ldm * ldm);
  int nrows = ldm - s;
  dense_eig(tmp + s * ldm + s, ldm, nrows, w->eval + s, w->sub_evec + s * ldm + s, ldm, il - s,
            iu - s);
  if (w->p.eval_sm) { /* :753-769 */
    int* ord = w->itmp;
    for (int i = 0; i < nrows; i++) ord[i] = i;
    sort_by_magnitude(w->eval + s, ord, 0, nrows - 1);
    int len = ((w->max_dim_x < ldm) ? w->max_dim_x : ldm) - s;
    double* start = w->sub_evec + s * ldm + s;
    for (int i = 0; i < len; i++)
      memcpy(tmp + (size_t)i * ldm, start + (size_t)ord[i] * ldm, sizeof(double) * nrows);
    memcpy(start, tmp, sizeof(double) * ((size_t)(len - 1) * ldm + nrows));
  }
  if (w->p.if_shift == 1) { /* :771-783 */
    for (int i = s; i < iu; i++) w->eval[i] -= w->p.shift;
    for (int i = 0; i < ldm; i++) w->sub_mat[i * ldm + i] -= w->p.shift;
  }
}

/* ---------------- X, P, W (src/gcge_xpw.c) ------------------------------ */
static void compute_x(port_ws* w, int size_x, int size_v) { /* :47-76 */
  int sx = w->num_soft_locked_in_last_iter;
  mv_lincomb(w, w->V, w->evec, sx, size_v, sx, size_x, w->sub_evec + sx * size_v + sx, size_v, 0.0);
}

/* GCGE_BCG, src/gcge_cg.c:302-501, including its index bookkeeping: after a
 * column locks out, rho/ptw are addressed by the compacted index "id" in
 * places and by the column index "idx" in others (:411 vs :451,465,474). */
/* y += shift * (B x or x) when a shift is active (src/gcge_cg.c:348-360,
 * 420-432): the block CG then solves (A + shift B) w = rhs. */
static void shift_term(port_ws* w, const double* x, double* y) {
  if (w->p.if_shift != 1) return;
  if (w->B) {
    spmv(w->B, x, w->Bx, w);
    axpby(w->n, w->p.shift, w->Bx, 1.0, y);
  } else {
    axpby(w->n, w->p.shift, x, 1.0, y);
  }
}

static void bcg(port_ws* w, double** RHS, double** X, int s0, int s1, int len, double** P,
                double** Wv) {
  const int n = w->n;
  double* rho1 = w->sub_dtmp;
  double* rho2 = rho1 + len;
  double* err = rho2 + len;
  double* lerr = err + len;
  double* ptw = lerr + len;
  int* unl = w->itmp;
  int nu = 0;
  for (int idx = 0; idx < len; idx++) {
    spmv(w->A, X[s1 + idx], Wv[idx], w);
    shift_term(w, X[s1 + idx], Wv[idx]);
    axpby(n, -1.0, Wv[idx], 1.0, RHS[s0 + idx]);
    rho2[idx] = dot(n, RHS[s0 + idx], RHS[s0 + idx]);
  }
  for (int idx = 0; idx < len; idx++) {
    err[idx] = sqrt(rho2[idx]);
    lerr[idx] = err[idx];
    if (err[idx] >= 1e-15) unl[nu++] = idx;
  }
  int niter = 1;
  while (nu > 0 && niter < w->p.cg_max_it) {
    for (int id = 0; id < nu; id++) {
      int idx = unl[id];
      if (niter == 1) axpby(n, 1.0, RHS[s0 + idx], 0.0, P[idx]);
      else axpby(n, 1.0, RHS[s0 + idx], rho2[idx] / rho1[idx], P[idx]);
      spmv(w->A, P[idx], Wv[idx], w);
      shift_term(w, P[idx], Wv[idx]);
      ptw[id] = dot(n, P[idx], Wv[idx]);
    }
    for (int id = 0; id < nu; id++) {
      int idx = unl[id];
      double alpha = rho2[id] / ptw[id];
      axpby(n, alpha, P[idx], 1.0, X[s1 + idx]);
      axpby(n, -alpha, Wv[idx], 1.0, RHS[s0 + idx]);
      rho1[id] = rho2[id];
      rho2[id] = dot(n, RHS[s0 + idx], RHS[s0 + idx]);
    }
    for (int id = 0; id < nu; id++) lerr[unl[id]] = sqrt(fabs(rho2[id]));
    int old = nu;
    nu = 0;
    for (int id = 0; id < old; id++) {
      int idx = unl[id];
      if (lerr[idx] >= w->p.cg_rate * err[idx] && lerr[idx] >= 1e-15) unl[nu++] = idx;
    }
    niter++;
  }
}

/* FP32 operator of the mixed W step: y = (A + shift B) x in FP32 sums. */
static void spmv32(port_ws* w, const float* x, float* y) {
  const int n = w->n;
  const port_csr* A = w->A;
  const port_csr* B = w->B;
  const int sh = w->p.if_shift == 1;
  const float sigma = (float)w->p.shift;
  w->spmv_count++;
#pragma omp parallel for schedule(static) if (n > 32768)
  for (int i = 0; i < n; i++) {
    float s = 0.f;
    for (int k = A->rp[i]; k < A->rp[i + 1]; k++) s += w->a32[k] * x[A->ci[k]];
    if (sh) {
      float t = 0.f;
      if (B)
        for (int k = B->rp[i]; k < B->rp[i + 1]; k++) t += w->b32[k] * x[B->ci[k]];
      else
        t = x[i];
      s += sigma * t;
    }
    y[i] = s;
  }
}

static double dot32(int n, const float* x, const float* y) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static) if (n > 32768)
  for (int i = 0; i < n; i++) s += (double)(x[i] * y[i]);
  return s;
}

/* The block CG above on FP32 columns (R: right-hand sides, overwritten by the
 * residuals; X: start and result), the same bookkeeping. */
static void bcg32(port_ws* w, int len) {
  const int n = w->n;
  double* rho1 = w->sub_dtmp;
  double* rho2 = rho1 + len;
  double* err = rho2 + len;
  double* lerr = err + len;
  double* ptw = lerr + len;
  int* unl = w->itmp;
  int nu = 0;
  for (int idx = 0; idx < len; idx++) {
    float* r = w->f_r + (size_t)idx * n;
    float* ax = w->f_w + (size_t)idx * n;
    spmv32(w, w->f_x + (size_t)idx * n, ax);
    for (int i = 0; i < n; i++) r[i] -= ax[i];
    rho2[idx] = dot32(n, r, r);
  }
  for (int idx = 0; idx < len; idx++) {
    err[idx] = sqrt(rho2[idx]);
    lerr[idx] = err[idx];
    if (err[idx] >= 1e-15) unl[nu++] = idx;
  }
  int niter = 1;
  while (nu > 0 && niter < w->p.cg_max_it) {
    for (int id = 0; id < nu; id++) {
      const int idx = unl[id];
      float* p = w->f_p + (size_t)idx * n;
      const float* r = w->f_r + (size_t)idx * n;
      float* wv = w->f_w + (size_t)idx * n;
      if (niter == 1) {
        for (int i = 0; i < n; i++) p[i] = r[i];
      } else {
        const float beta = (float)(rho2[idx] / rho1[idx]);
        for (int i = 0; i < n; i++) p[i] = r[i] + beta * p[i];
      }
      spmv32(w, p, wv);
      ptw[id] = dot32(n, p, wv);
    }
    for (int id = 0; id < nu; id++) {
      const int idx = unl[id];
      const float alpha = (float)(rho2[id] / ptw[id]);
      float* x = w->f_x + (size_t)idx * n;
      float* r = w->f_r + (size_t)idx * n;
      const float* p = w->f_p + (size_t)idx * n;
      const float* wv = w->f_w + (size_t)idx * n;
      for (int i = 0; i < n; i++) {
        x[i] += alpha * p[i];
        r[i] -= alpha * wv[i];
      }
      rho1[id] = rho2[id];
      rho2[id] = dot32(n, r, r);
    }
    for (int id = 0; id < nu; id++) lerr[unl[id]] = sqrt(fabs(rho2[id]));
    int old = nu;
    nu = 0;
    for (int id = 0; id < old; id++) {
      int idx = unl[id];
      if (lerr[idx] >= w->p.cg_rate * err[idx] && lerr[idx] >= 1e-15) unl[nu++] = idx;
    }
    niter++;
  }
}

static void compute_w(port_ws* w) { /* :118-260 */
  const int n = w->n;
  int ws = w->dim_xp, wl = w->unconv_bs;
  for (int idx = 0; idx < wl; idx++) {
    double* rhs = w->V_tmp[idx];
    int xi = w->unlock[idx];
    double* x = w->V[xi];
    double* wc = w->V[ws + idx];
    apply_b(w, x, rhs);
    double lam = w->eval[xi];
    /* the reference adds para->shift here whether or not if_shift is set */
    if (fabs(lam) <= 1.0) {
      axpby(n, 0.0, rhs, lam + w->p.shift, rhs);
      axpby(n, 1.0, x, 0.0, wc);
    } else {
      axpby(n, 1.0 / (lam + w->p.shift), x, 0.0, wc);
    }
  }
  if (!w->p.mixed) {
    bcg(w, w->V_tmp, w->V, 0, ws, wl, w->CG_p, w->evec);
    return;
  }
  /* mixed: r = rhs - A w0 in FP64, A e = r in FP32 from e = 0, W = e */
  for (int idx = 0; idx < wl; idx++) {
    double* r = w->V_tmp[idx];
    double* wc = w->V[ws + idx];
    spmv(w->A, wc, w->evec[0], w);
    shift_term(w, wc, w->evec[0]);
    axpby(n, -1.0, w->evec[0], 1.0, r);
    float* fr = w->f_r + (size_t)idx * n;
    float* fx = w->f_x + (size_t)idx * n;
    for (int i = 0; i < n; i++) {
      fr[i] = (float)r[i];
      fx[i] = 0.f;
    }
  }
  bcg32(w, wl);
  for (int idx = 0; idx < wl; idx++) {
    double* wc = w->V[ws + idx];
    const float* fx = w->f_x + (size_t)idx * n;
    for (int i = 0; i < n; i++) wc[i] = (double)fx[i];
  }
}

static void compute_p(port_ws* w) { /* :329-478 */
  double* coef = w->sub_evec;
  int ldc = w->dim_xpw, p_start = w->dim_x, p_ncols = w->unconv_bs, xx_nrows = w->last_dim_x;
  double* px = coef + p_start * ldc;
  double* pp = px + xx_nrows;
  double* xp = coef + xx_nrows;
  memset(px, 0, sizeof(double) * p_ncols * ldc);
  for (int cp = 0; cp < p_ncols; cp++)
    memcpy(pp + cp * ldc, xp + w->unlock[cp] * ldc, sizeof(double) * (ldc - xx_nrows));
  int os = w->num_soft_locked_in_last_iter;
  int ol = ldc - os;
  p_start -= os;
  int p_end = p_start + p_ncols;
  stable_multi_orth_in_sub(w, coef + os * ldc + os, ldc, ol, p_start, &p_end);
  p_end += os;
  int nev = w->nev;
  int pe_tmp = p_end - nev;
  mv_lincomb(w, w->V, w->V_tmp, os, ldc, 0, pe_tmp, coef + nev * ldc + os, ldc, 0.0);
  mv_swap(w->V, w->V_tmp, nev, p_end, 0);
  w->dim_xp = p_end;
}

/* GCGE_CheckConvergence, src/gcge_eigsol.c:663-887 ("R" criterion). */
static void check_convergence(port_ws* w) {
  const int n = w->n, nev = w->nev;
  int* unlock = w->unlock;
  int max_conv_idx = unlock[0] - 1, start = unlock[0], flag = 0, nu = 0;
  int ncc = unlock[0];
  double* res = w->res;
  double* eval = w->eval;
  double* t1 = w->V_tmp[0];
  double* t2 = w->V_tmp[1];
  unlock[0] = -1;
  for (int idx = start; idx < nev; idx++) {
    double* ev = w->evec[idx];
    spmv(w->A, ev, t1, w);
    if (!w->B) {
      axpby(n, -eval[idx], ev, 1.0, t1);
    } else {
      spmv(w->B, ev, t2, w);
      axpby(n, -eval[idx], t2, 1.0, t1);
    }
    double rn = sqrt(dot(n, t1, t1)), en = sqrt(dot(n, ev, ev));
    double r = rn / en, ab = r;
    if (w->p.conv_type == 0) r /= (1.0 > fabs(eval[idx]) ? 1.0 : fabs(eval[idx]));
    else if (w->p.conv_type == 1) r /= (w->p.conv_omega_norm + fabs(eval[idx]));
    res[idx] = r;
    if (r < w->p.ev_tol && ab < 1e-2) {
      if (idx > 0) {
        if (res[idx - 1] < w->p.ev_tol) {
          max_conv_idx = idx;
          if (flag == 0) ncc = idx + 1;
        } else {
          double me = fabs(eval[idx] - eval[idx - 1]) / fabs(eval[idx - 1]);
          if (me < w->p.multi_tol_for_lock) unlock[nu++] = idx;
          else max_conv_idx = idx;
        }
      } else {
        max_conv_idx = 0;
        ncc = 1;
      }
    } else {
      flag = 1;
      if (idx > 0 && res[idx - 1] < w->p.ev_tol) {
        int mmi = idx;
        for (int i = idx; i > 0; i--) {
          double me = fabs(eval[i] - eval[i - 1]) / fabs(eval[i - 1]);
          if (me < w->p.multi_tol_for_lock) mmi = i - 1;
          else break;
        }
        for (int i = mmi; i <= idx; i++) unlock[nu++] = i;
      } else {
        unlock[nu++] = idx;
      }
    }
    if (idx - max_conv_idx > 9) break;
  }
  if (ncc < nev && nu < w->p.block_size) {
    /* the reference reads unlock[nu-1] unguarded; nu == 0 cannot occur with
       ncc < nev, the guard only avoids the out-of-range read */
    if (nu > 0 && unlock[nu - 1] < nev - 1) {
      for (int i = nu; i < w->p.block_size; i++) {
        unlock[i] = unlock[i - 1] + 1;
        nu++;
        if (unlock[i] > nev - 2) break;
      }
    }
  }
  if (ncc < nev && unlock[0] < ncc) ncc = unlock[0];
  if (w->p.use_shift == 1) { /* src/gcge_eigsol.c:827-831 */
    w->p.if_shift = 1;
    w->p.shift = (eval[w->dim_x - 1] - 100.0 * eval[0]) / 99.0;
  }
  if (nu > w->p.block_size) nu = w->p.block_size;
  w->num_unlock = nu;
  w->num_conv_continuous = ncc;
  w->unconv_bs = nu;
  w->num_iter++;
}

static double wall(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static double** alloc_mv(int n, int k) {
  double** m = (double**)malloc(sizeof(double*) * k);
  for (int i = 0; i < k; i++) m[i] = (double*)calloc((size_t)n, sizeof(double));
  return m;
}
static void free_mv(double** m, int k) {
  for (int i = 0; i < k; i++) free(m[i]);
  free(m);
}

/* Defaults of GCGE_PARA_Create (src/gcge_para.c:25-113) plus PARA_Setup's
 * block size rule and DBL_EPSILON increments (:414-448). */
void gcge_port_default_para(port_para* p, int nev) {
  p->nev = nev;
  p->block_size = 0;
  p->ev_max_it = 30;
  p->cg_max_it = 20;
  p->max_reorth_time = 3;
  p->ev_tol = 1e-8;
  p->cg_rate = 1e-2;
  p->orth_zero_tol = 1e-14;
  p->reorth_tol = 0.75;
  p->scbgs_reorth_tol = 1e-16;
  p->multi_tol_for_lock = 1e-6;
  p->use_shift = 0;
  p->if_shift = 0;
  p->eval_sm = 0;
  p->shift = 0.0;
  p->mixed = 0;
  p->conv_type = 0;
  p->conv_omega_norm = 0.0;
}

/* Solve A x = lambda B x for the nev smallest pairs from the initial block x0
 * (column-major n x nev), following GCGE_Solve (src/gcge_eigsol.c:65-646).
 * max_outer < 0 means "run to convergence"; otherwise stop after that many
 * outer iterations (used to time bounded samples).  Returns 0 on success. */
int gcge_port_solve(int n, const int* a_rp, const int* a_ci, const double* a_v, const int* b_rp,
                    const int* b_ci, const double* b_v, const port_para* para_in, const double* x0,
                    int max_outer, double* eval_out, double* evec_out, double* res_out,
                    int* num_iter_out, double* seconds_out, long long* spmv_out,
                    double* phase_out) {
  port_csr A = {n, a_rp, a_ci, a_v}, Bm = {n, b_rp, b_ci, b_v};
  port_ws W;
  port_ws* w = &W;
  memset(w, 0, sizeof(W));
  w->p = *para_in;
  int nev = w->p.nev;
  if (w->p.block_size == 0) {
    w->p.block_size = nev < 10 ? nev : 10;
    w->p.block_size = (nev / 5 > w->p.block_size) ? nev / 5 : w->p.block_size;
  } else if (w->p.block_size > nev) {
    w->p.block_size = nev;
  }
  w->p.orth_zero_tol += DBL_EPSILON;
  w->p.scbgs_reorth_tol += DBL_EPSILON;
  w->A = &A;
  w->B = b_rp ? &Bm : NULL;
  w->n = n;
  w->nev = nev;
  w->bs = w->p.block_size;
  w->max_dim_x = nev + 20;
  w->V_size = w->max_dim_x + 2 * w->bs;
  w->V_tmp_size = w->max_dim_x - nev + w->bs;
  int mx = w->max_dim_x + 2 * w->bs;
  w->V = alloc_mv(n, w->V_size);
  w->V_tmp = alloc_mv(n, w->V_tmp_size);
  w->CG_p = alloc_mv(n, w->bs);
  w->evec = alloc_mv(n, nev);
  w->eval = (double*)calloc(mx, sizeof(double));
  w->sub_dtmp = (double*)calloc((size_t)2 * mx * mx + 40 * mx, sizeof(double));
  w->itmp = (int*)calloc(100 * mx, sizeof(int));
  w->sub_evec = (double*)calloc((size_t)mx * mx, sizeof(double));
  w->sub_mat = (double*)calloc((size_t)mx * mx, sizeof(double));
  w->unlock = (int*)calloc(w->max_dim_x, sizeof(int));
  w->res = (double*)calloc(nev, sizeof(double));
  w->Bx = (double*)calloc(n, sizeof(double));
  if (w->p.mixed) {
    const int annz = a_rp[n], bnnz = b_rp ? b_rp[n] : 0;
    w->a32 = (float*)malloc(sizeof(float) * (annz > 0 ? annz : 1));
    w->b32 = (float*)malloc(sizeof(float) * (bnnz > 0 ? bnnz : 1));
    for (int k = 0; k < annz; k++) w->a32[k] = (float)a_v[k];
    for (int k = 0; k < bnnz; k++) w->b32[k] = (float)b_v[k];
    const size_t fn = (size_t)n * w->bs;
    w->f_r = (float*)calloc(fn, sizeof(float));
    w->f_x = (float*)calloc(fn, sizeof(float));
    w->f_p = (float*)calloc(fn, sizeof(float));
    w->f_w = (float*)calloc(fn, sizeof(float));
  }
  for (int i = 0; i < nev; i++) w->res[i] = 1.0;
  for (int i = 0; i < w->max_dim_x; i++) w->unlock[i] = i;
  w->dim_x = nev;
  w->dim_xp = 0;
  w->dim_xpw = nev;
  w->unconv_bs = nev < w->bs ? nev : w->bs;
  for (int j = 0; j < nev; j++) memcpy(w->evec[j], x0 + (size_t)j * n, sizeof(double) * n);

  double t0 = wall();
  /* num_init_evec == nev: orthonormalise the given block (:219-242) */
  orth_mgs(w, w->evec, 0, &w->dim_x);
  for (int j = 0; j < nev; j++) memcpy(w->V[j], w->evec[j], sizeof(double) * n);
  w->dim_xpw = w->dim_x;
  w->last_dim_x = w->dim_x;
  w->dim_xp = 0;
  compute_subspace_matrix(w);
  compute_subspace_eigenpairs(w);
  compute_x(w, nev, w->dim_xpw);
  check_convergence(w);
  if (w->num_conv_continuous < nev) {
    int s = w->num_soft_locked_in_last_iter;
    mv_swap(w->V, w->evec, s, nev, s);
    w->dim_xp = w->dim_x;
    compute_w(w);
    w->last_dim_xpw = w->dim_xpw;
    w->dim_xpw = w->dim_xp + w->unconv_bs;
    stable_multi_orth(w, w->V, w->dim_x, &w->dim_xpw);
    w->dim_xp = nev;
    compute_subspace_matrix(w);
    compute_subspace_eigenpairs(w);
    compute_x(w, nev, w->dim_xpw);
    check_convergence(w);
  }
  double t_loop = wall();
  int outer = 0;
  while (w->num_conv_continuous < nev && w->num_iter < w->p.ev_max_it) {
    if (max_outer >= 0 && outer >= max_outer) break;
    outer++;
    compute_p(w);
    int s = w->num_soft_locked_in_last_iter;
    mv_swap(w->V, w->evec, s, nev, s);
    compute_w(w);
    w->last_dim_xpw = w->dim_xpw;
    w->dim_xpw = w->dim_xp + w->unconv_bs;
    stable_multi_orth(w, w->V, w->dim_xp, &w->dim_xpw);
    compute_subspace_matrix(w);
    compute_subspace_eigenpairs(w);
    w->last_dim_x = w->dim_x;
    w->dim_x = w->max_dim_x;
    compute_x(w, nev, w->dim_xpw);
    check_convergence(w);
  }
  {
    int s = w->num_soft_locked_in_last_iter;
    for (int j = 0; j < s; j++) memcpy(w->evec[j], w->V[j], sizeof(double) * n);
  }
  double t1 = wall();
  /* phase_out: [time before the loop, time in the loop, loop iterations] */
  if (phase_out) {
    phase_out[0] = t_loop - t0;
    phase_out[1] = t1 - t_loop;
    phase_out[2] = outer;
  }
  for (int j = 0; j < nev; j++) {
    eval_out[j] = w->eval[j];
    if (evec_out) memcpy(evec_out + (size_t)j * n, w->evec[j], sizeof(double) * n);
    if (res_out) res_out[j] = w->res[j];
  }
  if (num_iter_out) *num_iter_out = w->num_iter;
  if (seconds_out) *seconds_out = t1 - t0;
  if (spmv_out) *spmv_out = w->spmv_count;
  free_mv(w->V, w->V_size);
  free_mv(w->V_tmp, w->V_tmp_size);
  free_mv(w->CG_p, w->bs);
  free_mv(w->evec, nev);
  free(w->eval);
  free(w->sub_dtmp);
  free(w->itmp);
  free(w->sub_evec);
  free(w->sub_mat);
  free(w->unlock);
  free(w->res);
  free(w->Bx);
  free(w->a32);
  free(w->b32);
  free(w->f_r);
  free(w->f_x);
  free(w->f_p);
  free(w->f_w);
  return 0;
}

/* Thread count of the OpenMP loops (1 = the reference's single thread). */
#ifdef _OPENMP
#include <omp.h>
#endif
void gcge_port_set_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}
int gcge_port_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* The size of port_para, so callers can check their struct mirror. */
int gcge_port_para_size(void) { return (int)sizeof(port_para); }
