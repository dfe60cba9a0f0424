/*
 * ORACLE TEST INFRASTRUCTURE — not part of the product.
 *
 * Name shim for building the reference GCGE core as a checker.  The reference
 * calls the Fortran-ABI LAPACK/BLAS names declared in src/gcge_ops.h:152-182
 * (dsyev_, dsyevx_, dgemm_, dsymm_, daxpy_, ddot_, dnrm2_, dscal_, dcopy_).
 * The vendored netlib Fortran (blaslapack/) cannot be compiled here (no
 * Fortran compiler), so these forwarders route each call to the LP64 OpenBLAS
 * bundled with scipy, which exports the same routines under a "scipy_" prefix.
 */
typedef int I;

extern void scipy_dsyev_(char*, char*, I*, double*, I*, double*, double*, I*, I*);
extern void scipy_dsyevx_(char*, char*, char*, I*, double*, I*, double*, double*, I*, I*,
                          double*, I*, double*, double*, I*, double*, I*, I*, I*, I*);
extern void scipy_dgemm_(char*, char*, I*, I*, I*, double*, double*, I*, double*, I*,
                         double*, double*, I*);
extern void scipy_dsymm_(char*, char*, I*, I*, double*, double*, I*, double*, I*, double*,
                         double*, I*);
extern void scipy_daxpy_(I*, double*, double*, I*, double*, I*);
extern double scipy_ddot_(I*, double*, I*, double*, I*);
extern double scipy_dnrm2_(I*, double*, I*);
extern void scipy_dscal_(I*, double*, double*, I*);
extern void scipy_dcopy_(I*, double*, I*, double*, I*);

void dsyev_(char* jobz, char* uplo, I* n, double* a, I* lda, double* w, double* work, I* lwork,
            I* info) {
  scipy_dsyev_(jobz, uplo, n, a, lda, w, work, lwork, info);
}
void dsyevx_(char* jobz, char* range, char* uplo, I* n, double* a, I* lda, double* vl,
             double* vu, I* il, I* iu, double* abstol, I* m, double* w, double* z, I* ldz,
             double* work, I* lwork, I* iwork, I* ifail, I* info) {
  scipy_dsyevx_(jobz, range, uplo, n, a, lda, vl, vu, il, iu, abstol, m, w, z, ldz, work, lwork,
                iwork, ifail, info);
}
void dgemm_(char* ta, char* tb, I* m, I* n, I* k, double* al, double* a, I* lda, double* b,
            I* ldb, double* be, double* c, I* ldc) {
  scipy_dgemm_(ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc);
}
void dsymm_(char* side, char* uplo, I* m, I* n, double* al, double* a, I* lda, double* b, I* ldb,
            double* be, double* c, I* ldc) {
  scipy_dsymm_(side, uplo, m, n, al, a, lda, b, ldb, be, c, ldc);
}
void daxpy_(I* n, double* a, double* x, I* incx, double* y, I* incy) {
  scipy_daxpy_(n, a, x, incx, y, incy);
}
double ddot_(I* n, double* x, I* incx, double* y, I* incy) { return scipy_ddot_(n, x, incx, y, incy); }
double dnrm2_(I* n, double* x, I* incx) { return scipy_dnrm2_(n, x, incx); }
void dscal_(I* n, double* a, double* x, I* incx) { scipy_dscal_(n, a, x, incx); }
void dcopy_(I* n, double* x, I* incx, double* y, I* incy) { scipy_dcopy_(n, x, incx, y, incy); }
