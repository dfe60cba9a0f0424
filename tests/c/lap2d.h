/* 2D 5-point Laplacian on an m x m grid (Dirichlet), CSR with sorted columns;
 * its eigenvalues are 4 - 2 cos(i pi / (m+1)) - 2 cos(j pi / (m+1)). */
#ifndef TESTS_C_LAP2D_H_
#define TESTS_C_LAP2D_H_
#include <math.h>
#include <stdlib.h>

static inline void lap2d(int m, int** rp_, int** ci_, double** v_) {
  const int n = m * m;
  int* rp = (int*)malloc(sizeof(int) * (n + 1));
  int* ci = (int*)malloc(sizeof(int) * 5 * n);
  double* v = (double*)malloc(sizeof(double) * 5 * n);
  int e = 0;
  for (int r = 0; r < m; r++)
    for (int c = 0; c < m; c++) {
      const int i = r * m + c;
      rp[i] = e;
      if (r > 0) { ci[e] = i - m; v[e++] = -1.0; }
      if (c > 0) { ci[e] = i - 1; v[e++] = -1.0; }
      ci[e] = i; v[e++] = 4.0;
      if (c < m - 1) { ci[e] = i + 1; v[e++] = -1.0; }
      if (r < m - 1) { ci[e] = i + m; v[e++] = -1.0; }
    }
  rp[n] = e;
  *rp_ = rp;
  *ci_ = ci;
  *v_ = v;
}

static inline int cmp_double(const void* a, const void* b) {
  const double x = *(const double*)a, y = *(const double*)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

/* the k smallest eigenvalues, ascending */
static inline void lap2d_eigs(int m, int k, double* out) {
  double* all = (double*)malloc(sizeof(double) * m * m);
  for (int i = 1; i <= m; i++)
    for (int j = 1; j <= m; j++)
      all[(i - 1) * m + j - 1] = 4.0 - 2.0 * cos(i * M_PI / (m + 1)) - 2.0 * cos(j * M_PI / (m + 1));
  qsort(all, (size_t)m * m, sizeof(double), cmp_double);
  for (int i = 0; i < k; i++) out[i] = all[i];
  free(all);
}

/* y = A x on the host */
static inline void csr_mv(int n, const int* rp, const int* ci, const double* v, const double* x,
                   double* y) {
  for (int i = 0; i < n; i++) {
    double s = 0.0;
    for (int e = rp[i]; e < rp[i + 1]; e++) s += v[e] * x[ci[e]];
    y[i] = s;
  }
}
#endif
