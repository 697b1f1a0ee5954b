/* FP64 stand-ins for the three numerical libraries the reference CPU path links
 * (FFTW3, LAPACKE zgesv, CBLAS dgemm), written for this project so that the
 * unmodified reference sources under source/cpu can be compiled as a test
 * oracle.  Test infrastructure only: nothing in the GPU product links this.
 *
 *  - DFT: recursive mixed-radix decimation in time, twiddles evaluated
 *    directly as cos/sin(2*pi*(j*k mod n)/n) in double, a naive DFT for prime
 *    factors; exact up to FP64 rounding (~1e-15 relative).
 *  - zgesv: Gaussian elimination with partial pivoting on |re|+|im|.
 *  - dgemm: column-major triple loop (no transposes; the reference uses none).
 */
#include "fftw3.h"
#include "lapacke.h"
#include "cblas.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

void *fftw_malloc(size_t n) { return malloc(n ? n : 1); }
void fftw_free(void *p) { free(p); }
int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int nthreads) { (void)nthreads; }
void fftw_cleanup_threads(void) {}
void fftw_forget_wisdom(void) {}
int fftw_import_wisdom_from_filename(const char *f) { (void)f; return 0; }
int fftw_export_wisdom_to_filename(const char *f) { (void)f; return 1; }

struct dpshim_plan_s {
  int kind; /* 0 = guru split (forward), 1 = 1-D interleaved */
  int rank;
  fftw_iodim dims[8];
  int howmany_rank;
  fftw_iodim hm[8];
  int n1;
  int sign;
};

static int smallest_factor(int n) {
  if (n % 4 == 0) return 4;
  for (int p = 2; p * p <= n; ++p)
    if (n % p == 0) return p;
  return n;
}

/* out[k] = sum_j in[j*stride] * exp(sign*2*pi*i*j*k/n), out contiguous. */
static void dft_rec(int n, const double *in_re, const double *in_im, long stride,
                    double *out_re, double *out_im, int sign, int ntot, long tw_step) {
  if (n == 1) {
    out_re[0] = in_re[0];
    out_im[0] = in_im[0];
    return;
  }
  int p = smallest_factor(n);
  if (p == n) { /* naive DFT of a prime (or 4) length */
    for (int k = 0; k < n; ++k) {
      double sr = 0, si = 0;
      for (int j = 0; j < n; ++j) {
        long e = ((long)j * k) % n;
        double ang = sign * 2.0 * M_PI * (double)e / (double)n;
        double c = cos(ang), s = sin(ang);
        double xr = in_re[(long)j * stride], xi = in_im[(long)j * stride];
        sr += xr * c - xi * s;
        si += xr * s + xi * c;
      }
      out_re[k] = sr;
      out_im[k] = si;
    }
    return;
  }
  int m = n / p;
  double *yr = (double *)malloc(sizeof(double) * n);
  double *yi = (double *)malloc(sizeof(double) * n);
  for (int r = 0; r < p; ++r)
    dft_rec(m, in_re + (long)r * stride, in_im + (long)r * stride, stride * p, yr + (long)r * m,
            yi + (long)r * m, sign, ntot, tw_step);
  for (int q = 0; q < p; ++q) {
    for (int k = 0; k < m; ++k) {
      int kk = k + q * m;
      double sr = 0, si = 0;
      for (int r = 0; r < p; ++r) {
        long e = ((long)r * kk) % n;
        double ang = sign * 2.0 * M_PI * (double)e / (double)n;
        double c = cos(ang), s = sin(ang);
        double xr = yr[(long)r * m + k], xi = yi[(long)r * m + k];
        sr += xr * c - xi * s;
        si += xr * s + xi * c;
      }
      out_re[kk] = sr;
      out_im[kk] = si;
    }
  }
  free(yr);
  free(yi);
}

static void dft1d_inplace(int n, double *re, double *im, int sign) {
  double *or_ = (double *)malloc(sizeof(double) * n);
  double *oi = (double *)malloc(sizeof(double) * n);
  dft_rec(n, re, im, 1, or_, oi, sign, n, 1);
  memcpy(re, or_, sizeof(double) * n);
  memcpy(im, oi, sizeof(double) * n);
  free(or_);
  free(oi);
}

fftw_plan fftw_plan_guru_split_dft(int rank, const fftw_iodim *dims, int howmany_rank,
                                   const fftw_iodim *howmany_dims, double *ri, double *ii,
                                   double *ro, double *io, unsigned flags) {
  (void)ri; (void)ii; (void)ro; (void)io; (void)flags;
  if (rank < 1 || rank > 8 || howmany_rank < 0 || howmany_rank > 8) return 0;
  struct dpshim_plan_s *p = (struct dpshim_plan_s *)calloc(1, sizeof(*p));
  p->kind = 0;
  p->rank = rank;
  for (int i = 0; i < rank; ++i) p->dims[i] = dims[i];
  p->howmany_rank = howmany_rank;
  for (int i = 0; i < howmany_rank; ++i) p->hm[i] = howmany_dims[i];
  p->sign = FFTW_FORWARD;
  return p;
}

/* Multi-dimensional split-format forward DFT, in-place safe (gathers into a
 * contiguous buffer first). */
void fftw_execute_split_dft(const fftw_plan p, double *ri, double *ii, double *ro, double *io) {
  long total = 1;
  for (int d = 0; d < p->rank; ++d) total *= p->dims[d].n;
  long nh = 1;
  for (int d = 0; d < p->howmany_rank; ++d) nh *= p->hm[d].n;
  double *br = (double *)malloc(sizeof(double) * total);
  double *bi = (double *)malloc(sizeof(double) * total);
  long maxn = 1;
  for (int d = 0; d < p->rank; ++d)
    if (p->dims[d].n > maxn) maxn = p->dims[d].n;
  double *lr = (double *)malloc(sizeof(double) * maxn);
  double *li = (double *)malloc(sizeof(double) * maxn);
  for (long h = 0; h < nh; ++h) {
    long hin = 0, hout = 0, rem = h;
    for (int d = p->howmany_rank - 1; d >= 0; --d) {
      long c = rem % p->hm[d].n;
      rem /= p->hm[d].n;
      hin += c * p->hm[d].is;
      hout += c * p->hm[d].os;
    }
    for (long t = 0; t < total; ++t) { /* gather, C order over dims */
      long off = hin, r2 = t;
      for (int d = p->rank - 1; d >= 0; --d) {
        long c = r2 % p->dims[d].n;
        r2 /= p->dims[d].n;
        off += c * p->dims[d].is;
      }
      br[t] = ri[off];
      bi[t] = ii[off];
    }
    long inner = 1;
    for (int d = p->rank - 1; d >= 0; --d) {
      int n = p->dims[d].n;
      long outer = total / (inner * n);
      for (long o = 0; o < outer; ++o)
        for (long in = 0; in < inner; ++in) {
          long base = o * n * inner + in;
          for (int j = 0; j < n; ++j) {
            lr[j] = br[base + (long)j * inner];
            li[j] = bi[base + (long)j * inner];
          }
          dft1d_inplace(n, lr, li, p->sign);
          for (int j = 0; j < n; ++j) {
            br[base + (long)j * inner] = lr[j];
            bi[base + (long)j * inner] = li[j];
          }
        }
      inner *= n;
    }
    for (long t = 0; t < total; ++t) { /* scatter */
      long off = hout, r2 = t;
      for (int d = p->rank - 1; d >= 0; --d) {
        long c = r2 % p->dims[d].n;
        r2 /= p->dims[d].n;
        off += c * p->dims[d].os;
      }
      ro[off] = br[t];
      io[off] = bi[t];
    }
  }
  free(br); free(bi); free(lr); free(li);
}

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags) {
  (void)in; (void)out; (void)flags;
  struct dpshim_plan_s *p = (struct dpshim_plan_s *)calloc(1, sizeof(*p));
  p->kind = 1;
  p->n1 = n;
  p->sign = sign;
  return p;
}

void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out) {
  int n = p->n1;
  double *re = (double *)malloc(sizeof(double) * n);
  double *im = (double *)malloc(sizeof(double) * n);
  for (int j = 0; j < n; ++j) { re[j] = in[j][0]; im[j] = in[j][1]; }
  dft1d_inplace(n, re, im, p->sign);
  for (int j = 0; j < n; ++j) { out[j][0] = re[j]; out[j][1] = im[j]; }
  free(re); free(im);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }

/* ---------------- zgesv ---------------- */
lapack_int LAPACKE_zgesv(int layout, lapack_int n, lapack_int nrhs, lapack_complex_double *a,
                         lapack_int lda, lapack_int *ipiv, lapack_complex_double *b,
                         lapack_int ldb) {
  if (layout != LAPACK_COL_MAJOR) return -1;
#define A(i, j) a[(i) + (long)(j) * lda]
#define B(i, j) b[(i) + (long)(j) * ldb]
  for (int k = 0; k < n; ++k) {
    int piv = k;
    double best = -1;
    for (int i = k; i < n; ++i) {
      double v = fabs(A(i, k).real) + fabs(A(i, k).imag);
      if (v > best) { best = v; piv = i; }
    }
    ipiv[k] = piv + 1;
    if (best == 0) return k + 1;
    if (piv != k) {
      for (int j = 0; j < n; ++j) { lapack_complex_double t = A(k, j); A(k, j) = A(piv, j); A(piv, j) = t; }
      for (int j = 0; j < nrhs; ++j) { lapack_complex_double t = B(k, j); B(k, j) = B(piv, j); B(piv, j) = t; }
    }
    double pr = A(k, k).real, pi = A(k, k).imag, den = pr * pr + pi * pi;
    for (int i = k + 1; i < n; ++i) {
      double ar = A(i, k).real, ai = A(i, k).imag;
      double lr = (ar * pr + ai * pi) / den, li = (ai * pr - ar * pi) / den;
      A(i, k).real = lr; A(i, k).imag = li;
      for (int j = k + 1; j < n; ++j) {
        double ur = A(k, j).real, ui = A(k, j).imag;
        A(i, j).real -= lr * ur - li * ui;
        A(i, j).imag -= lr * ui + li * ur;
      }
      for (int j = 0; j < nrhs; ++j) {
        double ur = B(k, j).real, ui = B(k, j).imag;
        B(i, j).real -= lr * ur - li * ui;
        B(i, j).imag -= lr * ui + li * ur;
      }
    }
  }
  for (int j = 0; j < nrhs; ++j)
    for (int i = n - 1; i >= 0; --i) {
      double sr = B(i, j).real, si = B(i, j).imag;
      for (int m = i + 1; m < n; ++m) {
        double ar = A(i, m).real, ai = A(i, m).imag, xr = B(m, j).real, xi = B(m, j).imag;
        sr -= ar * xr - ai * xi;
        si -= ar * xi + ai * xr;
      }
      double pr = A(i, i).real, pi = A(i, i).imag, den = pr * pr + pi * pi;
      B(i, j).real = (sr * pr + si * pi) / den;
      B(i, j).imag = (si * pr - sr * pi) / den;
    }
#undef A
#undef B
  return 0;
}

/* ---------------- dgemm ---------------- */
void cblas_dgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb, int m,
                 int n, int k, double alpha, const double *a, int lda, const double *b, int ldb,
                 double beta, double *c, int ldc) {
  if (order != CblasColMajor || ta != CblasNoTrans || tb != CblasNoTrans) abort();
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      double s = 0;
      for (int l = 0; l < k; ++l) s += a[i + (long)l * lda] * b[l + (long)j * ldb];
      c[i + (long)j * ldc] = alpha * s + (beta == 0 ? 0 : beta * c[i + (long)j * ldc]);
    }
}
