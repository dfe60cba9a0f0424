/* GCGE_SOLVER set-up on the CUDA app's GCGE_OPS table (see gcge_app_cuda.h).
 * Follows GCGE_CSR_Solver_Init (app/csr/gcge_app_csr.c:92-124): create the
 * solver, read the flags, allocate the eigenpair storage, install the table,
 * Setup. */
#include <stdlib.h>

#include "gcge_app_cuda.h"

GCGE_SOLVER* GCGE_CUDA_Ops_Solver_Init(GCGE_CUDA_MAT* A, GCGE_CUDA_MAT* B, int num_eigenvalues,
                                   int argc, char* argv[]) {
  GCGE_SOLVER* solver;
  void** evec = NULL;
  int nev;
  double* eval;
  GCGE_SOLVER_Create(&solver);
  if (num_eigenvalues != -1) solver->para->nev = num_eigenvalues;
  GCGE_PARA_SetFromCommandLine(solver->para, argc, argv);
  nev = solver->para->nev;
  eval = (double*)calloc((size_t)nev, sizeof(double));
  if (!eval || GCGE_CUDA_MultiVecCreate(&evec, nev, A) != GCGE_CUDA_OK ||
      GCGE_CUDA_SetOps(solver->ops) != GCGE_CUDA_OK) {
    free(eval);
    if (evec) GCGE_CUDA_MultiVecDestroy(&evec);
    GCGE_SOLVER_Free(&solver);
    return NULL;
  }
  GCGE_SOLVER_SetMatA(solver, A);
  if (B != NULL) GCGE_SOLVER_SetMatB(solver, B);
  GCGE_SOLVER_SetEigenvalues(solver, eval);
  GCGE_SOLVER_SetEigenvectors(solver, evec);
  GCGE_SOLVER_Setup(solver);
  if (GCGE_CUDA_OpsGetError() != GCGE_CUDA_OK) {
    GCGE_SOLVER_Free_All(&solver);
    return NULL;
  }
  return solver;
}

GCGE_SOLVER* GCGE_CUDA_Ops_Solver_CreateByOps(GCGE_CUDA_MAT* A, GCGE_CUDA_MAT* B, int nev,
                                          double* eval, void** evec) {
  GCGE_OPS* ops;
  GCGE_OPS_Create(&ops);
  if (GCGE_CUDA_SetOps(ops) != GCGE_CUDA_OK) {
    GCGE_OPS_Free(&ops);
    return NULL;
  }
  return GCGE_SOLVER_CreateByOps(A, B, nev, eval, evec, ops);
}
