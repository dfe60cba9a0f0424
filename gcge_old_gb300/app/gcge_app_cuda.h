/* GCGE_SOLVER set-up on the CUDA app's GCGE_OPS table: the analogue of the
 * reference's GCGE_CSR_Solver_Init (app/csr/gcge_app_csr.c:92-124).  This
 * file and gcge_app_cuda.c belong with the reference core: they are compiled
 * together with its src/ C files (they include its gcge_solver.h) and linked with
 * the CUDA app's library (-lgcge_cuda). */
#ifndef GCGE_APP_CUDA_H_
#define GCGE_APP_CUDA_H_

#include "gcge_cuda_ops.h"
#include "gcge_solver.h"

/* A GCGE_SOLVER whose ops are the CUDA table: flags as GCGE_PARA_SetFromCommandLine
 * reads them, eval (nev doubles) and evec (a CUDA multivector of nev columns)
 * allocated here, Setup done.  GCGE_SOLVER_Free_All releases both.  NULL
 * when the table could not be set up (GCGE_CUDA_OpsGetError tells why). */
GCGE_SOLVER* GCGE_CUDA_Ops_Solver_Init(GCGE_CUDA_MAT* A, GCGE_CUDA_MAT* B, int num_eigenvalues,
                                   int argc, char* argv[]);

/* The same through GCGE_SOLVER_CreateByOps (src/gcge_solver.c:40-57), the entry
 * the reference's PASE uses: a fresh GCGE_OPS filled by GCGE_CUDA_SetOps,
 * with the caller's eval and evec (a CUDA multivector). */
GCGE_SOLVER* GCGE_CUDA_Ops_Solver_CreateByOps(GCGE_CUDA_MAT* A, GCGE_CUDA_MAT* B, int nev,
                                          double* eval, void** evec);

#endif
