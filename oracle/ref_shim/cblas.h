/* Declaration subset of CBLAS used by the reference CPU sources (dgemm only).
 * Implemented in dpshim.c as a plain triple loop. */
#ifndef DPSHIM_CBLAS_H
#define DPSHIM_CBLAS_H
#ifdef __cplusplus
extern "C" {
#endif
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
void cblas_dgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb,
                 int m, int n, int k, double alpha, const double *a, int lda,
                 const double *b, int ldb, double beta, double *c, int ldc);
#ifdef __cplusplus
}
#endif
#endif
