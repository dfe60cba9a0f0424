/* A C caller of the device-resident solver (include/gcge_cuda.h), the way an
 * application switches from GCGE_CSR_Solver_Init (app/csr/gcge_app_csr.c:92)
 * to GCGE_CUDA_Solver_Init: host CSR in the reference's CSR_MAT layout,
 * -gcge_* flags, a pseudo-random start (num_init_evec 0), Solve, eigenpairs
 * read back.  Checks the 2D Laplacian's known eigenvalues and each pair's
 * residual ||A x - lambda x|| / (|lambda| ||x||) on the host.
 *   usage: solve_c_api m nev [fp64|mixed]
 * Built and run on a GPU by tests/test_c_programs.py; prints "c api: OK". */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "gcge_cuda.h"
#include "lap2d.h"

int main(int argc, char** argv) {
  const int m = argc > 1 ? atoi(argv[1]) : 32, nev = argc > 2 ? atoi(argv[2]) : 10;
  const char* prec = argc > 3 ? argv[3] : "fp64";
  const int n = m * m;
  int *rp, *ci;
  double* v;
  lap2d(m, &rp, &ci, &v);
  GCGE_CUDA_CSR_HOST A = {n, n, rp[n], ci, rp, v};
  char* flags[] = {"prog", "-gcge_ev_tol", "1e-12", "-gcge_ev_max_it", "300",
                   "-gcge_precision", (char*)prec, "-gcge_print_result", "1", "-gcge_print_conv", "1"};
  GCGE_CUDA_SOLVER* s = GCGE_CUDA_Solver_Init(&A, NULL, nev, 11, flags);
  if (!s) {
    printf("GCGE_CUDA_Solver_Init failed: %s\n", GCGE_CUDA_GetLastErrorMessage());
    return 1;
  }
  if (GCGE_CUDA_SOLVER_Solve(s) != GCGE_CUDA_OK) {
    printf("Solve failed: %s\n", GCGE_CUDA_GetLastErrorMessage());
    return 1;
  }
  double *eval = NULL, *evec = NULL;
  GCGE_CUDA_SOLVER_GetEigenvalues(s, &eval);
  GCGE_CUDA_SOLVER_GetEigenvectors(s, &evec);
  double* exact = (double*)malloc(sizeof(double) * nev);
  lap2d_eigs(m, nev, exact);
  double* ax = (double*)malloc(sizeof(double) * n);
  double worst_ev = 0.0, worst_res = 0.0;
  for (int k = 0; k < nev; k++) {
    const double* x = evec + (size_t)k * n;
    csr_mv(n, rp, ci, v, x, ax);
    double r2 = 0.0, x2 = 0.0;
    for (int i = 0; i < n; i++) {
      const double r = ax[i] - eval[k] * x[i];
      r2 += r * r;
      x2 += x[i] * x[i];
    }
    worst_res = fmax(worst_res, sqrt(r2 / x2) / fabs(eval[k]));
    worst_ev = fmax(worst_ev, fabs(eval[k] - exact[k]) / exact[k]);
  }
  GCGE_CUDA_STATS st;
  GCGE_CUDA_SOLVER_GetStats(s, &st);
  printf("c api: %s, %d iterations, eigenvalue error %.2e, residual %.2e\n", prec, st.num_iter,
         worst_ev, worst_res);
  const int ok = worst_ev < 1e-10 && worst_res < 1e-10 && st.num_conv_continuous == nev;
  GCGE_CUDA_SOLVER_Free_All(&s);
  free(exact);
  free(ax);
  free(rp);
  free(ci);
  free(v);
  printf(ok ? "c api: OK\n" : "c api: FAILED\n");
  return ok ? 0 : 1;
}
