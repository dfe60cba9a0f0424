/* The CUDA app's GCGE_OPS table (include/gcge_cuda_ops.h), driven only
 * through its function pointers as the reference core drives it:
 *   1. every block callback against the same operation done on the host
 *      (the reference defaults' meaning, src/gcge_ops.c);
 *   2. a block eigensolver written against the table alone (LOBPCG-style
 *      Rayleigh-Ritz on [X, W, P] with an SVQB orthonormalisation) finds the
 *      smallest eigenvalues of the 2D Laplacian.
 * Built and run on a GPU by tests/test_c_programs.py:
 *   gcc -I include tests/c/ops_table_gpu.c -L<lib dir> -lgcge_cuda -lm
 * Prints "ops table: OK" and exits 0 when every check holds. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gcge_cuda_ops.h"
#include "lap2d.h"

static int nfail = 0;
#define CHECK(cond, ...)              \
  do {                                \
    if (!(cond)) {                    \
      printf("FAIL %d: ", __LINE__);  \
      printf(__VA_ARGS__);            \
      printf("\n");                   \
      nfail++;                        \
    }                                 \
  } while (0)

static double* host_cols(void** mv, int start, int k, int n) {
  double* h = (double*)malloc(sizeof(double) * (size_t)n * (k > 0 ? k : 1));
  CHECK(GCGE_CUDA_MultiVecGetToHost(mv, start, k, h, n) == GCGE_CUDA_OK, "GetToHost");
  return h;
}

static double dotv(const double* a, const double* b, int n) {
  double s = 0.0;
  for (int i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/* ------------------------------------------------------------ callbacks */
static void check_callbacks(GCGE_CUDA_OPS* ops, GCGE_CUDA_MAT* A, int n, const int* rp,
                            const int* ci, const double* v) {
  const int k = 6;
  void **X = NULL, **Y = NULL;
  CHECK(ops->MatDotVec && ops->VecAxpby && ops->VecInnerProd && ops->VecLocalInnerProd &&
            ops->VecCreateByVec && ops->VecCreateByMat && ops->VecDestroy && ops->VecSetRandomValue,
        "the 8 callbacks GCGE_OPS_Setup requires");
  ops->MultiVecCreateByMat(&X, k, A, ops);
  ops->MultiVecCreateByMat(&Y, k, A, ops);
  CHECK(X && Y, "MultiVecCreateByMat");
  ops->MultiVecSetRandomValue(X, 0, k, ops);
  ops->MultiVecSetRandomValue(Y, 0, k, ops);
  double* hx = host_cols(X, 0, k, n);
  double* hy = host_cols(Y, 0, k, n);
  CHECK(hx[0] >= 0.0 && hx[0] < 1.0 && hx[n] != hx[0] && hy[0] != hx[0], "random values U[0,1)");
  for (int i = 0; i < n * k; i++) CHECK(hx[i] >= 0.0 && hx[i] < 1.0, "random value %g", hx[i]);

  /* MatDotMultiVec: Y(:, 1:k) = A X(:, 0:k-1) */
  int s[2] = {0, 1}, e[2] = {k - 1, k};
  ops->MatDotMultiVec(A, X, Y, s, e, ops);
  double* hy2 = host_cols(Y, 0, k, n);
  double* t = (double*)malloc(sizeof(double) * n);
  for (int j = 0; j < k - 1; j++) {
    csr_mv(n, rp, ci, v, hx + (size_t)j * n, t);
    for (int i = 0; i < n; i++) CHECK(fabs(t[i] - hy2[(size_t)(j + 1) * n + i]) < 1e-14, "MatDotMultiVec");
  }
  CHECK(memcmp(hy2, hy, sizeof(double) * n) == 0, "MatDotMultiVec left column 0 alone");

  /* MultiVecInnerProd "ns": a[(w-s1) lda + (v-s0)] = X_v . Y_w */
  double a[64];
  for (int i = 0; i < 64; i++) a[i] = -7.0;
  int s2[2] = {1, 2}, e2[2] = {4, 5};
  ops->MultiVecInnerProd(X, Y, a, "ns", s2, e2, 5, 0, ops);
  for (int w = 0; w < 3; w++)
    for (int vv = 0; vv < 3; vv++) {
      const double ref = dotv(hx + (size_t)(1 + vv) * n, hy2 + (size_t)(2 + w) * n, n);
      CHECK(fabs(a[w * 5 + vv] - ref) <= 1e-13 * fabs(ref) + 1e-13, "InnerProd ns");
    }
  CHECK(a[3] == -7.0 && a[4] == -7.0, "InnerProd kept the rows past the block");
  /* "sym": upper triangle computed, mirrored */
  int s3[2] = {0, 0}, e3[2] = {4, 4};
  ops->MultiVecInnerProd(X, X, a, "sym", s3, e3, 4, 0, ops);
  for (int w = 0; w < 4; w++)
    for (int vv = 0; vv < 4; vv++) {
      const double ref = dotv(hx + (size_t)vv * n, hx + (size_t)w * n, n);
      CHECK(fabs(a[w * 4 + vv] - ref) <= 1e-13 * fabs(ref), "InnerProd sym");
      CHECK(a[w * 4 + vv] == a[vv * 4 + w], "InnerProd sym is symmetric");
    }

  /* MultiVecLinearComb: Y(:,0:3) = 2 X(:,1:5) C + 0.5 Y(:,0:3), C 4 x 3 with lda 6 */
  double C[18];
  for (int i = 0; i < 18; i++) C[i] = 0.1 * (i + 1) - 0.7;
  int s4[2] = {1, 0}, e4[2] = {5, 3};
  ops->MultiVecLinearComb(X, Y, s4, e4, C, 6, 0, 2.0, 0.5, ops);
  double* hy3 = host_cols(Y, 0, k, n);
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < n; i++) {
      double ref = 0.5 * hy2[(size_t)j * n + i];
      for (int q = 0; q < 4; q++) ref += 2.0 * hx[(size_t)(1 + q) * n + i] * C[j * 6 + q];
      CHECK(fabs(hy3[(size_t)j * n + i] - ref) < 1e-13 * (1.0 + fabs(ref)), "LinearComb");
    }
  /* MultiVecAxpby: Y(:, 3:6) = 0.3 X(:, 0:3) - 1.2 Y(:, 3:6) */
  int s5[2] = {0, 3}, e5[2] = {3, 6};
  ops->MultiVecAxpby(0.3, X, -1.2, Y, s5, e5, ops);
  double* hy4 = host_cols(Y, 0, k, n);
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < n; i++) {
      const double ref = 0.3 * hx[(size_t)j * n + i] - 1.2 * hy3[(size_t)(3 + j) * n + i];
      CHECK(fabs(hy4[(size_t)(3 + j) * n + i] - ref) < 1e-14 * (1.0 + fabs(ref)), "Axpby");
    }
  /* MultiVecSwap: X(:,0) <-> Y(:,5) */
  int s6[2] = {0, 5}, e6[2] = {1, 6};
  ops->MultiVecSwap(X, Y, s6, e6, ops);
  double* hx5 = host_cols(X, 0, 1, n);
  double* hy5 = host_cols(Y, 5, 1, n);
  CHECK(memcmp(hx5, hy4 + (size_t)5 * n, sizeof(double) * n) == 0 &&
            memcmp(hy5, hx, sizeof(double) * n) == 0,
        "MultiVecSwap exchanged the columns");
  /* single vectors through GetVecFromMultiVec */
  void *x2, *y3, *z;
  ops->GetVecFromMultiVec(X, 2, &x2, ops);
  ops->GetVecFromMultiVec(Y, 3, &y3, ops);
  double ip = 0.0;
  ops->VecInnerProd(x2, y3, &ip, ops);
  const double ipref = dotv(hx + (size_t)2 * n, hy4 + (size_t)3 * n, n);
  CHECK(fabs(ip - ipref) <= 1e-13 * fabs(ipref), "VecInnerProd");
  ops->VecCreateByVec(&z, x2, ops);
  ops->VecAxpby(2.0, x2, 0.0, z, ops);  /* z = 2 x2 */
  ops->VecAxpby(-1.0, y3, 1.0, z, ops); /* z = 2 x2 - y3 */
  ops->VecInnerProd(z, z, &ip, ops);
  double nz = 0.0;
  for (int i = 0; i < n; i++) {
    const double d = 2.0 * hx[(size_t)2 * n + i] - hy4[(size_t)3 * n + i];
    nz += d * d;
  }
  CHECK(fabs(ip - nz) <= 1e-12 * nz, "VecAxpby / VecCreateByVec");
  ops->VecDestroy(&z, ops);
  ops->RestoreVecForMultiVec(X, 2, &x2, ops);
  ops->RestoreVecForMultiVec(Y, 3, &y3, ops);
  /* DenseMatEigenSolver: tridiag(-1, 2, -1) of order 7, eigenvalues 2 - 2 cos(k pi / 8) */
  double T[49], ev[7], evec[64];
  int iw[64];
  double dw[256];
  for (int pass = 0; pass < 2; pass++) {
    memset(T, 0, sizeof(T));
    for (int i = 0; i < 7; i++) {
      T[i * 7 + i] = 2.0;
      if (i > 0) T[i * 7 + i - 1] = T[(i - 1) * 7 + i] = -1.0;
    }
    const int il = pass == 0 ? 2 : 1, iu = pass == 0 ? 4 : 7;
    ops->DenseMatEigenSolver(T, 7, 7, ev, evec, 8, il, iu, iw, dw);
    for (int q = il; q <= iu; q++)
      CHECK(fabs(ev[q - il] - (2.0 - 2.0 * cos(q * M_PI / 8.0))) < 1e-13, "DenseMatEigenSolver %d", q);
  }
  CHECK(GCGE_CUDA_OpsGetError() == GCGE_CUDA_OK, "no callback failed (%s)",
        GCGE_CUDA_GetLastErrorMessage());
  /* a bad range sets the sticky error and is ignored */
  int sb[2] = {0, 0}, eb[2] = {k + 3, k + 3};
  ops->MultiVecAxpby(1.0, X, 1.0, Y, sb, eb, ops);
  CHECK(GCGE_CUDA_OpsGetError() == GCGE_CUDA_ERR_ARG, "a range past the block is reported");
  GCGE_CUDA_OpsClearError();
  ops->MultiVecDestroy(&X, k, ops);
  ops->MultiVecDestroy(&Y, k, ops);
  CHECK(!X && !Y, "MultiVecDestroy");
  free(hx); free(hy); free(hy2); free(hy3); free(hy4); free(hx5); free(hy5); free(t);
}

/* ------------------------------------------------------------ a block eigensolver on the table */
/* S(:, 0:ns) <- S B with B = D U Theta^{-1/2} over the kept directions (SVQB):
 * orthonormal columns spanning S; returns how many were kept.  T: scratch
 * multivector of at least ns columns (swapped with S). */
static int svqb(GCGE_CUDA_OPS* ops, void*** S, void*** T, int ns) {
  double G[144], Gs[144], th[12], U[144], B[144];
  int iw[256];
  double dw[1024];
  int s[2] = {0, 0}, e[2] = {ns, ns};
  ops->MultiVecInnerProd(*S, *S, G, "sym", s, e, ns, 0, ops);
  double d[12];
  for (int i = 0; i < ns; i++) d[i] = 1.0 / sqrt(G[i * ns + i]);
  for (int j = 0; j < ns; j++)
    for (int i = 0; i < ns; i++) Gs[j * ns + i] = d[i] * G[j * ns + i] * d[j];
  ops->DenseMatEigenSolver(Gs, ns, ns, th, U, ns, 1, ns, iw, dw);
  int kept = 0;
  for (int q = 0; q < ns; q++)
    if (th[q] > 1e-12 * th[ns - 1]) {
      for (int i = 0; i < ns; i++) B[kept * ns + i] = d[i] * U[q * ns + i] / sqrt(th[q]);
      kept++;
    }
  int s2[2] = {0, 0}, e2[2] = {ns, kept};
  ops->MultiVecLinearComb(*S, *T, s2, e2, B, ns, 0, 1.0, 0.0, ops);
  void** tmp = *S;
  *S = *T;
  *T = tmp;
  return kept;
}

static void check_block_solver(GCGE_CUDA_OPS* ops, GCGE_CUDA_MAT* A, int m) {
  const int nev = 4;
  void **S, **T, **AS, **X;
  ops->MultiVecCreateByMat(&S, 3 * nev, A, ops);   /* [X | W | P] */
  ops->MultiVecCreateByMat(&T, 3 * nev, A, ops);
  ops->MultiVecCreateByMat(&AS, 3 * nev, A, ops);
  ops->MultiVecCreateByMat(&X, nev, A, ops);       /* previous X, for P */
  ops->MultiVecSetRandomValue(S, 0, nev, ops);
  int ns = svqb(ops, &S, &T, nev);
  int np = 0, it = 0;
  double lam[12], H[144], C[144], res = 1.0;
  int iw[256];
  double dw[1024];
  const int maxit = 400;
  for (it = 0; it < maxit; it++) {
    /* Rayleigh-Ritz on S(:, 0:ns) */
    int s[2] = {0, 0}, e[2] = {ns, ns};
    ops->MatDotMultiVec(A, S, AS, s, e, ops);
    ops->MultiVecInnerProd(S, AS, H, "sym", s, e, ns, 0, ops);
    ops->DenseMatEigenSolver(H, ns, ns, lam, C, ns, 1, nev, iw, dw);
    /* X_new = S C and A X_new = AS C (into T), W = A X - X Lambda */
    int s1[2] = {0, 0}, e1[2] = {ns, nev};
    int s2[2] = {0, nev}, e2[2] = {ns, 2 * nev};
    ops->MultiVecLinearComb(S, T, s1, e1, C, ns, 0, 1.0, 0.0, ops);
    ops->MultiVecLinearComb(AS, T, s2, e2, C, ns, 0, 1.0, 0.0, ops);
    res = 0.0;
    for (int j = 0; j < nev; j++) {
      ops->MultiVecAxpbyColumn(-lam[j], T, j, 1.0, T, nev + j, ops);
      void* w;
      double r2 = 0.0;
      ops->GetVecFromMultiVec(T, nev + j, &w, ops);
      ops->VecInnerProd(w, w, &r2, ops);
      ops->RestoreVecForMultiVec(T, nev + j, &w, ops);
      res = fmax(res, sqrt(r2) / fabs(lam[j]));  /* unit columns: ||A x - lambda x|| / |lambda| */
    }
    if (res < 1e-9) break;
    /* P = X_new - X_old (after the first step), then S = [X_new, W, P] */
    int sp[2] = {0, 2 * nev}, ep[2] = {nev, 3 * nev};
    if (it > 0) {
      ops->MultiVecAxpby(1.0, T, 0.0, T, sp, ep, ops);   /* T(:, 2nev:) = X_new */
      ops->MultiVecAxpby(-1.0, X, 1.0, T, sp, ep, ops);  /* - X_old */
      np = nev;
    }
    int sc[2] = {0, 0}, ec[2] = {nev, nev};
    ops->MultiVecAxpby(1.0, T, 0.0, X, sc, ec, ops);     /* X_old = X_new */
    void** tmp = S;
    S = T;
    T = tmp;
    ns = svqb(ops, &S, &T, 2 * nev + np);
  }
  double exact[4];
  lap2d_eigs(m, nev, exact);
  double worst = 0.0;
  for (int j = 0; j < nev; j++) worst = fmax(worst, fabs(lam[j] - exact[j]) / exact[j]);
  printf("block solver on the table: %d iterations, residual %.2e, eigenvalue error %.2e\n", it,
         res, worst);
  CHECK(res < 1e-9, "block solver converged (%.2e)", res);
  CHECK(worst < 1e-12, "eigenvalues of the 2D Laplacian (%.2e)", worst);
  CHECK(GCGE_CUDA_OpsGetError() == GCGE_CUDA_OK, "no callback failed (%s)",
        GCGE_CUDA_GetLastErrorMessage());
  ops->MultiVecDestroy(&S, 3 * nev, ops);
  ops->MultiVecDestroy(&T, 3 * nev, ops);
  ops->MultiVecDestroy(&AS, 3 * nev, ops);
  ops->MultiVecDestroy(&X, nev, ops);
}

int main(void) {
  const int m = 16, n = m * m;
  int *rp, *ci;
  double* v;
  lap2d(m, &rp, &ci, &v);
  GCGE_CUDA_MAT* A = NULL;
  if (GCGE_CUDA_MatCreate(&A, n, rp, ci, v, 0) != GCGE_CUDA_OK) {
    printf("MatCreate failed: %s\n", GCGE_CUDA_GetLastErrorMessage());
    return 1;
  }
  GCGE_CUDA_OPS ops;
  memset(&ops, 0, sizeof(ops));
  CHECK(GCGE_CUDA_SetOps(&ops) == GCGE_CUDA_OK, "SetOps");
  CHECK(GCGE_CUDA_SetOps(NULL) == GCGE_CUDA_ERR_ARG, "SetOps(NULL)");
  check_callbacks(&ops, A, n, rp, ci, v);
  check_block_solver(&ops, A, m);
  GCGE_CUDA_MatDestroy(&A);
  free(rp);
  free(ci);
  free(v);
  if (nfail) {
    printf("ops table: %d checks failed\n", nfail);
    return 1;
  }
  printf("ops table: OK\n");
  return 0;
}
