/* Layout check of include/gcge_cuda_ops.h against the reference's struct
 * GCGE_OPS (src/gcge_ops.h:29-150): every field at the same offset with the
 * same size, and the same total size.  Compiled (not run) by
 * tests/test_ops_table.py where the reference checkout is present:
 *   gcc -fsyntax-only -I <reference>/src -I include tests/c/ops_layout.c */
#include <stddef.h>

#include "gcge_ops.h"
#include "gcge_cuda_ops.h"

#define SAME(f)                                                                  \
  _Static_assert(offsetof(GCGE_OPS, f) == offsetof(GCGE_CUDA_OPS, f) &&          \
                     sizeof(((GCGE_OPS*)0)->f) == sizeof(((GCGE_CUDA_OPS*)0)->f), \
                 #f)

SAME(ops);
SAME(VecSetRandomValue);
SAME(MatDotVec);
SAME(MatTransposeDotVec);
SAME(VecAxpby);
SAME(VecInnerProd);
SAME(VecLocalInnerProd);
SAME(VecCreateByVec);
SAME(VecCreateByMat);
SAME(VecDestroy);
SAME(GetVecFromMultiVec);
SAME(RestoreVecForMultiVec);
SAME(MultiGridCreate);
SAME(MultiGridDestroy);
SAME(VecFromItoJ);
SAME(MultiVecFromItoJ);
SAME(LinearSolver);
SAME(linear_solver_workspace);
SAME(MultiLinearSolver);
SAME(Orthonormalization);
SAME(DenseMatCreate);
SAME(DenseMatDestroy);
SAME(MultiVecCreateByVec);
SAME(MultiVecCreateByMat);
SAME(MultiVecCreateByMultiVec);
SAME(MultiVecDestroy);
SAME(MultiVecSetRandomValue);
SAME(MatDotMultiVec);
SAME(MatTransposeDotMultiVec);
SAME(MultiVecAxpby);
SAME(MultiVecAxpbyColumn);
SAME(MultiVecLinearComb);
SAME(MultiVecInnerProd);
SAME(MultiVecInnerProdLocal);
SAME(MultiVecSwap);
SAME(MultiVecPrint);
SAME(SetDirichletBoundary);
SAME(DenseMatEigenSolver);
SAME(DenseMatDotDenseMat);
SAME(DenseSymMatDotDenseMat);
SAME(ArrayDotArray);
SAME(ArrayNorm);
SAME(ArrayAXPBY);
SAME(ArrayCopy);
SAME(ArrayScale);
_Static_assert(sizeof(GCGE_OPS) == sizeof(GCGE_CUDA_OPS), "size of the table");

/* the table filler takes the reference's own struct */
int fill(GCGE_OPS* ops) { return GCGE_CUDA_SetOps(ops); }
