/*
 * Fortran-BLAS entry points for the oracle build of upstream htool
 * (oracle/_ref).  Test infrastructure only.
 *
 * htool declares plain Fortran names (dgemv_, zgemm_, ...) in
 * include/htool/wrappers/wrapper_blas.hpp:11-48.  The only BLAS present on
 * both the x86 container and the Arm GPU host is the LP64 OpenBLAS bundled in
 * the SciPy wheel, which exports the same routines with a "scipy_" prefix.
 * Each wrapper below forwards one name; the argument lists follow the BLAS
 * reference interface (hidden Fortran string lengths are not passed, as in
 * htool's own declarations).
 */
typedef struct {
    double re, im;
} zc;
typedef struct {
    float re, im;
} cc;

#define FWD_AXPY(P, T)                                                                         \
    void scipy_##P##axpy_(const int *, const T *, const T *, const int *, T *, const int *); \
    void P##axpy_(const int *n, const T *a, const T *x, const int *ix, T *y, const int *iy) { scipy_##P##axpy_(n, a, x, ix, y, iy); }

#define FWD_GEMV(P, T)                                                                                                                     \
    void scipy_##P##gemv_(const char *, const int *, const int *, const T *, const T *, const int *, const T *, const int *, const T *, T *, \
                          const int *);                                                                                                    \
    void P##gemv_(const char *t, const int *m, const int *n, const T *al, const T *a, const int *lda, const T *x, const int *ix, const T *be, \
                  T *y, const int *iy) { scipy_##P##gemv_(t, m, n, al, a, lda, x, ix, be, y, iy); }

#define FWD_GEMM(P, T)                                                                                                                   \
    void scipy_##P##gemm_(const char *, const char *, const int *, const int *, const int *, const T *, const T *, const int *, const T *, \
                          const int *, const T *, T *, const int *);                                                                     \
    void P##gemm_(const char *ta, const char *tb, const int *m, const int *n, const int *k, const T *al, const T *a, const int *lda,       \
                  const T *b, const int *ldb, const T *be, T *c, const int *ldc) { scipy_##P##gemm_(ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc); }

#define FWD_SYMV(N, P, T)                                                                                                                 \
    void scipy_##P##N##_(const char *, const int *, const T *, const T *, const int *, const T *, const int *, const T *, T *, const int *); \
    void P##N##_(const char *u, const int *n, const T *al, const T *a, const int *lda, const T *x, const int *ix, const T *be, T *y,       \
                 const int *iy) { scipy_##P##N##_(u, n, al, a, lda, x, ix, be, y, iy); }

#define FWD_SYMM(N, P, T)                                                                                                                  \
    void scipy_##P##N##_(const char *, const char *, const int *, const int *, const T *, const T *, const int *, const T *, const int *, \
                         const T *, T *, const int *);                                                                                      \
    void P##N##_(const char *sd, const char *u, const int *m, const int *n, const T *al, const T *a, const int *lda, const T *b,           \
                 const int *ldb, const T *be, T *c, const int *ldc) { scipy_##P##N##_(sd, u, m, n, al, a, lda, b, ldb, be, c, ldc); }

FWD_AXPY(s, float)
FWD_AXPY(d, double)
FWD_AXPY(c, cc)
FWD_AXPY(z, zc)
FWD_GEMV(s, float)
FWD_GEMV(d, double)
FWD_GEMV(c, cc)
FWD_GEMV(z, zc)
FWD_GEMM(s, float)
FWD_GEMM(d, double)
FWD_GEMM(c, cc)
FWD_GEMM(z, zc)
FWD_SYMV(symv, s, float)
FWD_SYMV(symv, d, double)
FWD_SYMV(symv, c, cc)
FWD_SYMV(symv, z, zc)
FWD_SYMV(hemv, c, cc)
FWD_SYMV(hemv, z, zc)
FWD_SYMM(symm, s, float)
FWD_SYMM(symm, d, double)
FWD_SYMM(symm, c, cc)
FWD_SYMM(symm, z, zc)
FWD_SYMM(hemm, c, cc)
FWD_SYMM(hemm, z, zc)

float scipy_snrm2_(const int *, const float *, const int *);
double scipy_dnrm2_(const int *, const double *, const int *);
float scipy_scnrm2_(const int *, const cc *, const int *);
double scipy_dznrm2_(const int *, const zc *, const int *);
float snrm2_(const int *n, const float *x, const int *i) { return scipy_snrm2_(n, x, i); }
double dnrm2_(const int *n, const double *x, const int *i) { return scipy_dnrm2_(n, x, i); }
float scnrm2_(const int *n, const cc *x, const int *i) { return scipy_scnrm2_(n, x, i); }
double dznrm2_(const int *n, const zc *x, const int *i) { return scipy_dznrm2_(n, x, i); }
