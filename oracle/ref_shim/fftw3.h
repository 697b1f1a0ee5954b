/* Declaration subset of the FFTW3 API that the reference CPU sources use.
 * The implementation (dpshim.c) is a plain FP64 mixed-radix DFT written for
 * this project; it exists only so the unmodified reference sources can be
 * compiled as a test oracle.  No FFTW code is used or copied. */
#ifndef DPSHIM_FFTW3_H
#define DPSHIM_FFTW3_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef double fftw_complex[2];
typedef struct dpshim_plan_s *fftw_plan;
typedef struct { int n; int is; int os; } fftw_iodim;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_EXHAUSTIVE (1U << 3)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_WISDOM_ONLY (1U << 21)
void *fftw_malloc(size_t n);
void fftw_free(void *p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
void fftw_cleanup_threads(void);
void fftw_forget_wisdom(void);
int fftw_import_wisdom_from_filename(const char *filename);
int fftw_export_wisdom_to_filename(const char *filename);
fftw_plan fftw_plan_guru_split_dft(int rank, const fftw_iodim *dims, int howmany_rank,
                                   const fftw_iodim *howmany_dims, double *ri, double *ii,
                                   double *ro, double *io, unsigned flags);
void fftw_execute_split_dft(const fftw_plan p, double *ri, double *ii, double *ro, double *io);
fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out);
void fftw_destroy_plan(fftw_plan p);
#ifdef __cplusplus
}
#endif
#endif
