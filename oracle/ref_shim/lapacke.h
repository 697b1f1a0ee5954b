/* Declaration subset of LAPACKE used by the reference CPU sources (zgesv only).
 * Implemented in dpshim.c by Gaussian elimination with partial pivoting. */
#ifndef DPSHIM_LAPACKE_H
#define DPSHIM_LAPACKE_H
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { double real, imag; } lapack_complex_double;
typedef int lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
lapack_int LAPACKE_zgesv(int matrix_layout, lapack_int n, lapack_int nrhs,
                         lapack_complex_double *a, lapack_int lda, lapack_int *ipiv,
                         lapack_complex_double *b, lapack_int ldb);
#ifdef __cplusplus
}
#endif
#endif
