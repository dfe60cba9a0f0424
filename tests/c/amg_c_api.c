/* A C caller of the AMG preconditioner (include/gcge_cuda.h): the device
 * matrix from a host CSR in the reference's CSR_MAT layout, the hierarchy
 * built on the GPU (GCGE_CUDA_AMG_Create), the solver's W step handed to
 * AMG-PCG through the MultiLinearSolver hook (the place where the reference's
 * hypre app plugs in its AMG-PCG), Solve, eigenpairs read back.  Checks the 2D
 * Laplacian's known eigenvalues and each pair's residual on the host.
 *   usage: amg_c_api m nev [fp64|mixed]
 * Built and run on a GPU by tests/test_c_programs.py; prints "amg c api: OK". */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gcge_cuda.h"
#include "lap2d.h"

int main(int argc, char** argv) {
  const int m = argc > 1 ? atoi(argv[1]) : 48, nev = argc > 2 ? atoi(argv[2]) : 10;
  const int mixed = argc > 3 && strcmp(argv[3], "mixed") == 0;
  const int n = m * m;
  int *rp, *ci;
  double* v;
  lap2d(m, &rp, &ci, &v);
  GCGE_CUDA_CSR_HOST Ah = {n, n, rp[n], ci, rp, v};
  GCGE_CUDA_MAT* A = NULL;
  GCGE_CUDA_AMG* amg = NULL;
  GCGE_CUDA_SOLVER* s = NULL;
  double* eval = (double*)calloc(nev, sizeof(double));
  double* evec = (double*)calloc((size_t)n * nev, sizeof(double));
  int ok = 0, levels = 0, rc;
  GCGE_CUDA_AMG_PARAM prm;
  GCGE_CUDA_AMG_DefaultParam(&prm);
  if ((rc = GCGE_CUDA_MatCreateFromCSR(&A, &Ah)) != GCGE_CUDA_OK ||
      (rc = GCGE_CUDA_AMG_Create(&amg, A, &prm)) != GCGE_CUDA_OK ||
      (rc = GCGE_CUDA_AMG_GetNumLevels(amg, &levels)) != GCGE_CUDA_OK ||
      (rc = GCGE_CUDA_SOLVER_Create(&s)) != GCGE_CUDA_OK ||
      (rc = GCGE_CUDA_SOLVER_SetMatA(s, A)) != GCGE_CUDA_OK ||
      (rc = GCGE_CUDA_SOLVER_SetMatB(s, NULL)) != GCGE_CUDA_OK ||
      (rc = GCGE_CUDA_SOLVER_SetNumEigen(s, nev)) != GCGE_CUDA_OK ||
      (rc = GCGE_CUDA_SOLVER_SetEigenvalues(s, eval)) != GCGE_CUDA_OK ||
      (rc = GCGE_CUDA_SOLVER_SetEigenvectors(s, evec)) != GCGE_CUDA_OK ||
      (rc = GCGE_CUDA_SOLVER_SetParamDouble(s, "ev_tol", 1e-12)) != GCGE_CUDA_OK ||
      (rc = GCGE_CUDA_SOLVER_SetParamInt(s, "ev_max_it", 300)) != GCGE_CUDA_OK ||
      (rc = GCGE_CUDA_SOLVER_SetParamInt(s, "precision", mixed)) != GCGE_CUDA_OK ||
      (rc = GCGE_CUDA_SOLVER_Setup(s)) != GCGE_CUDA_OK ||
      (rc = GCGE_CUDA_SOLVER_SetMultiLinearSolver(s, GCGE_CUDA_AMGPCG, amg)) != GCGE_CUDA_OK ||
      (rc = GCGE_CUDA_SOLVER_Solve(s)) != GCGE_CUDA_OK) {
    printf("failed (%d): %s\n", rc, GCGE_CUDA_GetLastErrorMessage());
  } else {
    double* exact = (double*)malloc(sizeof(double) * nev);
    double* ax = (double*)malloc(sizeof(double) * n);
    lap2d_eigs(m, nev, exact);
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
    int steps = 0;
    GCGE_CUDA_AMG_GetLastSteps(amg, &steps);
    printf("amg c api: %s, %d levels, %d GCG iterations, last W step %d AMG-PCG steps, "
           "eigenvalue error %.2e, residual %.2e\n", mixed ? "mixed" : "fp64", levels,
           st.num_iter, steps, worst_ev, worst_res);
    ok = levels >= 2 && worst_ev < 1e-10 && worst_res < 1e-10 && steps >= 1;
    free(exact);
    free(ax);
  }
  GCGE_CUDA_SOLVER_Free(&s);
  GCGE_CUDA_AMG_Destroy(&amg);
  GCGE_CUDA_MatDestroy(&A);
  free(eval);
  free(evec);
  free(rp);
  free(ci);
  free(v);
  printf(ok ? "amg c api: OK\n" : "amg c api: FAILED\n");
  return ok ? 0 : 1;
}
