/* The unmodified reference core solving on the CUDA app's GCGE_OPS table:
 * the 2D 5-point Laplacian on an m x m grid (B = I), nev smallest pairs,
 * through GCGE_CUDA_Ops_Solver_Init + GCGE_SOLVER_Solve.  Built against the
 * reference's src/ (compiled with it) and -lgcge_cuda by tests/test_ops_table.py
 * where the reference checkout is present.
 *   usage: ops_ref_driver m nev [-gcge_* flags]
 * Prints one line per pair ("pair k lambda"), then "iterations N".  Exits 3
 * when no CUDA device is usable (the matrix cannot be created). */
#include <stdio.h>
#include <stdlib.h>

#include "gcge_app_cuda.h"
#include "lap2d.h"

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  const int m = atoi(argv[1]), nev = atoi(argv[2]), n = m * m;
  int *rp, *ci;
  double* v;
  lap2d(m, &rp, &ci, &v);
  GCGE_CUDA_MAT* A = NULL;
  if (GCGE_CUDA_MatCreate(&A, n, rp, ci, v, 0) != GCGE_CUDA_OK) {
    printf("no usable CUDA device: %s\n", GCGE_CUDA_GetLastErrorMessage());
    return 3;
  }
  GCGE_SOLVER* s = GCGE_CUDA_Ops_Solver_Init(A, NULL, nev, argc - 3, argv + 3);
  if (!s) {
    printf("set-up failed: %s\n", GCGE_CUDA_GetLastErrorMessage());
    return 1;
  }
  GCGE_SOLVER_Solve(s);
  if (GCGE_CUDA_OpsGetError() != GCGE_CUDA_OK) {
    printf("solve failed: %s\n", GCGE_CUDA_GetLastErrorMessage());
    return 1;
  }
  for (int k = 0; k < nev; k++) printf("pair %d %.17g\n", k, s->eval[k]);
  printf("iterations %d\n", s->para->num_iter);
  GCGE_SOLVER_Free_All(&s);
  GCGE_CUDA_MatDestroy(&A);
  free(rp);
  free(ci);
  free(v);
  return 0;
}
