/* Forwarding shim used only by the oracle recipe: the NGT quantizer code calls
 * the Fortran BLAS/LAPACK names (sgemv_, sgemm_, sgesvd_, ...).  No system BLAS
 * is installed in the build container, but scipy ships OpenBLAS with every
 * symbol renamed to scipy_<name>.  These one-line wrappers bind the plain names
 * to that library.  Test infrastructure only: never linked into the product. */
#define FWD(ret, name, params, args) \
  extern ret scipy_##name params;    \
  ret name params { return scipy_##name args; }

FWD(void, sgemv_, (char *t, int *m, int *n, float *al, float *a, int *lda, float *x, int *ix, float *be, float *y, int *iy),
    (t, m, n, al, a, lda, x, ix, be, y, iy))
FWD(void, sgemm_, (char *ta, char *tb, int *m, int *n, int *k, float *al, float *a, int *lda, float *b, int *ldb, float *be, float *c, int *ldc),
    (ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc))
FWD(void, dgemm_, (char *ta, char *tb, int *m, int *n, int *k, double *al, double *a, int *lda, double *b, int *ldb, double *be, double *c, int *ldc),
    (ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc))
FWD(void, sgesvd_, (char *ju, char *jv, int *m, int *n, float *a, int *lda, float *s, float *u, int *ldu, float *vt, int *ldvt, float *w, int *lw, int *info),
    (ju, jv, m, n, a, lda, s, u, ldu, vt, ldvt, w, lw, info))
FWD(void, dgesvd_, (char *ju, char *jv, int *m, int *n, double *a, int *lda, double *s, double *u, int *ldu, double *vt, int *ldvt, double *w, int *lw, int *info),
    (ju, jv, m, n, a, lda, s, u, ldu, vt, ldvt, w, lw, info))
FWD(void, sgeqrf_, (int *m, int *n, float *a, int *lda, float *tau, float *w, int *lw, int *info), (m, n, a, lda, tau, w, lw, info))
FWD(void, sorgqr_, (int *m, int *n, int *k, float *a, int *lda, float *tau, float *w, int *lw, int *info), (m, n, k, a, lda, tau, w, lw, info))
FWD(void, dgeqrf_, (int *m, int *n, double *a, int *lda, double *tau, double *w, int *lw, int *info), (m, n, a, lda, tau, w, lw, info))
FWD(void, dorgqr_, (int *m, int *n, int *k, double *a, int *lda, double *tau, double *w, int *lw, int *info), (m, n, k, a, lda, tau, w, lw, info))
