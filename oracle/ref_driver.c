/*
 * ORACLE TEST INFRASTRUCTURE — not part of the product.
 *
 * Driver that runs the UNMODIFIED reference GCGE (src/ + app/csr/, compiled
 * out of tree by oracle/build_ref.sh) on caller-provided CSR arrays and a
 * caller-provided initial block, so the reference and the CUDA solver see
 * bit-identical inputs.  It goes through the reference's own public entry
 * points: GCGE_CSR_Solver_Init (app/csr/gcge_app_csr.c:92-124) and
 * GCGE_SOLVER_Solve (src/gcge_solver.c:125-128).  The initial block is passed
 * the way the reference supports warm starts: "-gcge_num_init_evec nev"
 * (src/gcge_eigsol.c:134,219-242) with the values written into solver->evec.
 */
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "gcge_app_csr.h"

static double wall_seconds(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* Returns 0 on success.  x0/evec_out are column-major n x nev.  B may be
 * absent (b_rowptr == NULL) which means B = I, as in the reference. */
int ref_gcge_solve(int n, const int* a_rowptr, const int* a_col, const double* a_val,
                   const int* b_rowptr, const int* b_col, const double* b_val, int nev,
                   const double* x0, int argc, char** argv, double* eval_out, double* evec_out,
                   int* num_iter_out, double* seconds_out, double* res_out) {
  CSR_MAT A, B;
  A.N_Rows = n;
  A.N_Columns = n;
  A.N_Entries = a_rowptr[n];
  A.RowPtr = (int*)a_rowptr;
  A.KCol = (int*)a_col;
  A.Entries = (double*)a_val;
  CSR_MAT* Bp = NULL;
  if (b_rowptr) {
    B.N_Rows = n;
    B.N_Columns = n;
    B.N_Entries = b_rowptr[n];
    B.RowPtr = (int*)b_rowptr;
    B.KCol = (int*)b_col;
    B.Entries = (double*)b_val;
    Bp = &B;
  }
  GCGE_SOLVER* s = GCGE_CSR_Solver_Init(&A, Bp, nev, argc, argv);
  if (!s) return 1;
  /* "-ref_fixed_shift <sigma>" (a flag of this driver, skipped by the
   * reference's own parser): sets the public fields para->if_shift = 1 and
   * para->shift = sigma (src/gcge_para.h:90-92), which the reference reads in
   * GCGE_ComputeW / GCGE_BCG / Rayleigh-Ritz; -gcge_use_shift recomputes them
   * every iteration instead. */
  for (int i = 0; i + 1 < argc; i++)
    if (!strcmp(argv[i], "-ref_fixed_shift")) {
      s->para->if_shift = 1;
      s->para->shift = atof(argv[i + 1]);
    }
  CSR_VEC** ev = (CSR_VEC**)s->evec;
  for (int j = 0; j < nev; j++) memcpy(ev[j]->Entries, x0 + (size_t)j * n, sizeof(double) * n);
  double t0 = wall_seconds();
  GCGE_SOLVER_Solve(s);
  double t1 = wall_seconds();
  for (int j = 0; j < nev; j++) {
    eval_out[j] = s->eval[j];
    memcpy(evec_out + (size_t)j * n, ev[j]->Entries, sizeof(double) * n);
    if (res_out) res_out[j] = s->para->res[j];
  }
  if (num_iter_out) *num_iter_out = s->para->num_iter;
  if (seconds_out) *seconds_out = t1 - t0;
  GCGE_SOLVER_Free_All(&s);
  return 0;
}
