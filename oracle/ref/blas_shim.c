/*
 * Fortran-ABI BLAS/LAPACK entry points for the reference GCGE build, forwarded
 * to the scipy_-prefixed symbols exported by SciPy's bundled OpenBLAS (LP64).
 * Test infrastructure only: it lets the reference CPU path
 * (app/app_lapack.h:304-376 declares the names it calls) link in a container
 * that has no system BLAS/LAPACK.
 *
 * Character arguments are passed with explicit hidden length 1, which is what
 * a gfortran-compiled LAPACK expects; a C-translated LAPACK ignores the extra
 * trailing arguments.
 */
#include <stddef.h>

typedef size_t flen;

extern double scipy_dasum_(int *, double *, int *);
extern void scipy_daxpy_(int *, double *, double *, int *, double *, int *);
extern void scipy_dcopy_(int *, double *, int *, double *, int *);
extern double scipy_ddot_(int *, double *, int *, double *, int *);
extern void scipy_dgemm_(char *, char *, int *, int *, int *, double *, double *, int *,
                         double *, int *, double *, double *, int *, flen, flen);
extern void scipy_dgemv_(char *, int *, int *, double *, double *, int *, double *, int *,
                         double *, double *, int *, flen);
extern int scipy_idamax_(int *, double *, int *);
extern void scipy_dscal_(int *, double *, double *, int *);
extern void scipy_dsymm_(char *, char *, int *, int *, double *, double *, int *, double *,
                         int *, double *, double *, int *, flen, flen);
extern void scipy_dgeqp3_(int *, int *, double *, int *, int *, double *, double *, int *, int *);
extern void scipy_dorgqr_(int *, int *, int *, double *, int *, double *, double *, int *, int *);
extern void scipy_dsyev_(char *, char *, int *, double *, int *, double *, double *, int *, int *,
                         flen, flen);
extern void scipy_dsyevx_(char *, char *, char *, int *, double *, int *, double *, double *,
                          int *, int *, double *, int *, double *, double *, int *, double *,
                          int *, int *, int *, int *, flen, flen, flen);

double dasum_(int *n, double *x, int *incx) { return scipy_dasum_(n, x, incx); }
int daxpy_(int *n, double *a, double *x, int *incx, double *y, int *incy)
{ scipy_daxpy_(n, a, x, incx, y, incy); return 0; }
int dcopy_(int *n, double *x, int *incx, double *y, int *incy)
{ scipy_dcopy_(n, x, incx, y, incy); return 0; }
double ddot_(int *n, double *x, int *incx, double *y, int *incy)
{ return scipy_ddot_(n, x, incx, y, incy); }
int dgemm_(char *ta, char *tb, int *m, int *n, int *k, double *alpha, double *a, int *lda,
           double *b, int *ldb, double *beta, double *c, int *ldc)
{ scipy_dgemm_(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, 1, 1); return 0; }
int dgemv_(char *t, int *m, int *n, double *alpha, double *a, int *lda, double *x, int *incx,
           double *beta, double *y, int *incy)
{ scipy_dgemv_(t, m, n, alpha, a, lda, x, incx, beta, y, incy, 1); return 0; }
int idamax_(int *n, double *x, int *incx) { return scipy_idamax_(n, x, incx); }
int dscal_(int *n, double *a, double *x, int *incx) { scipy_dscal_(n, a, x, incx); return 0; }
int dsymm_(char *side, char *uplo, int *m, int *n, double *alpha, double *a, int *lda,
           double *b, int *ldb, double *beta, double *c, int *ldc)
{ scipy_dsymm_(side, uplo, m, n, alpha, a, lda, b, ldb, beta, c, ldc, 1, 1); return 0; }
int dgeqp3_(int *m, int *n, double *a, int *lda, int *jpvt, double *tau, double *work,
            int *lwork, int *info)
{ scipy_dgeqp3_(m, n, a, lda, jpvt, tau, work, lwork, info); return 0; }
int dorgqr_(int *m, int *n, int *k, double *a, int *lda, double *tau, double *work,
            int *lwork, int *info)
{ scipy_dorgqr_(m, n, k, a, lda, tau, work, lwork, info); return 0; }
int dsyev_(char *jobz, char *uplo, int *n, double *a, int *lda, double *w, double *work,
           int *lwork, int *info)
{ scipy_dsyev_(jobz, uplo, n, a, lda, w, work, lwork, info, 1, 1); return 0; }
int dsyevx_(char *jobz, char *range, char *uplo, int *n, double *a, int *lda, double *vl,
            double *vu, int *il, int *iu, double *abstol, int *m, double *w, double *z,
            int *ldz, double *work, int *lwork, int *iwork, int *ifail, int *info)
{
    scipy_dsyevx_(jobz, range, uplo, n, a, lda, vl, vu, il, iu, abstol, m, w, z, ldz, work,
                  lwork, iwork, ifail, info, 1, 1, 1);
    return 0;
}
