/* BLAS/LAPACK entry points for compiling QSpace's MEX sources against numpy's
 * bundled ILP64 OpenBLAS (symbols scipy_<name>_64_).  Test infrastructure.
 *
 * The reference calls these routines in two styles: through its own
 * by-reference extern "C" prototypes of <name>_ (Source/wbblas.hh; those
 * symbols are defined in fakemx.cpp) and in the pointer style of MATLAB's
 * blas.h / lapack.h headers.  The pointer style is provided here as C++
 * overloads of the same names that forward to the OpenBLAS symbols. */
#ifndef FAKEMX_BLAS_H
#define FAKEMX_BLAS_H
#ifdef __cplusplus
#define FAKEMX_P const void *
extern "C" {
void scipy_dgemm_64_(FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P,
                     FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P);
void scipy_zgemm_64_(FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P,
                     FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P);
void scipy_dsyevd_64_(FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P,
                      FAKEMX_P, FAKEMX_P);
void scipy_zheevd_64_(FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P,
                      FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P);
void scipy_zheev_64_(FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P,
                     FAKEMX_P);
void scipy_dgesdd_64_(FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P,
                      FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P);
void scipy_zgesdd_64_(FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P,
                      FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P);
void scipy_dgesvd_64_(FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P,
                      FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P);
void scipy_zgesvd_64_(FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P,
                      FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P);
void scipy_dgeev_64_(FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P,
                     FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P);
void scipy_zgeev_64_(FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P,
                     FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P);
void scipy_dgetrf_64_(FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P);
void scipy_dgetri_64_(FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P);
long long scipy_ilaenv_64_(FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P, FAKEMX_P,
                           unsigned long, unsigned long);
}
#define FAKEMX_PTR_STYLE(name)                                                 \
  template <class A, class... T>                                               \
  inline void name##_(A *a0, T *...r) {                                        \
    scipy_##name##_64_(static_cast<const void *>(a0), static_cast<const void *>(r)...); \
  }
FAKEMX_PTR_STYLE(dgemm)
FAKEMX_PTR_STYLE(zgemm)
FAKEMX_PTR_STYLE(dsyevd)
FAKEMX_PTR_STYLE(zheevd)
FAKEMX_PTR_STYLE(zheev)
FAKEMX_PTR_STYLE(dgesdd)
FAKEMX_PTR_STYLE(zgesdd)
FAKEMX_PTR_STYLE(dgesvd)
FAKEMX_PTR_STYLE(zgesvd)
FAKEMX_PTR_STYLE(dgeev)
FAKEMX_PTR_STYLE(zgeev)
FAKEMX_PTR_STYLE(dgetrf)
FAKEMX_PTR_STYLE(dgetri)
/* ilaenv in pointer style, with the two trailing string lengths */
inline int ilaenv_(const long *i, const char *nm, const char *op, const long *a, const long *b, const long *c,
                   const long *d, int lnm, int lop) {
  return (int)scipy_ilaenv_64_(i, nm, op, a, b, c, d, (unsigned long)lnm, (unsigned long)lop);
}
#undef FAKEMX_PTR_STYLE
#undef FAKEMX_P
#endif
#endif
