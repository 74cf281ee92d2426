/* Oracle FFT (test infrastructure only): recursive mixed-radix decimation-in-time
 * DFT in double precision, twiddles from libm at full precision. Radix 4, 2, 3, 5
 * butterflies are written out; any other prime factor uses a direct O(p^2) DFT.
 * See orc_fft.h for the layout contract (FFTW r2c, reference main.c:1200, 266-271).
 */
#include "orc_fft.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  int n;
  double *wr, *wi; /* w[j] = exp(-2 pi i j / n) */
} twtab;

static void tw_init(twtab *t, int n) {
  t->n = n;
  t->wr = (double *)malloc(sizeof(double) * (size_t)n);
  t->wi = (double *)malloc(sizeof(double) * (size_t)n);
  for (int j = 0; j < n; j++) {
    double a = -2.0 * M_PI * (double)j / (double)n;
    t->wr[j] = cos(a);
    t->wi[j] = sin(a);
  }
}

static void tw_free(twtab *t) {
  free(t->wr);
  free(t->wi);
}

static int pick_radix(int n) {
  if (n % 4 == 0) return 4;
  if (n % 2 == 0) return 2;
  for (int p = 3; (long)p * p <= n; p += 2)
    if (n % p == 0) return p;
  return n;
}

/* out[k] = sum_j x[j*stride] w_n^{jk}; w_n^{m} = T[m*tstep mod N] with N = T->n */
static void fft_rec(int n, const double *x, long stride, double *out, const twtab *T, long tstep) {
  if (n == 1) {
    out[0] = x[0];
    out[1] = x[1];
    return;
  }
  const int N = T->n;
  const int p = pick_radix(n);
  const int m = n / p;
  for (int r = 0; r < p; r++) fft_rec(m, x + 2 * r * stride, stride * p, out + 2 * (long)r * m, T, tstep * p);

  if (p == 2) {
    for (int k = 0; k < m; k++) {
      long w = ((long)k * tstep) % N;
      double *a = out + 2 * k, *b = out + 2 * (k + m);
      double br = b[0] * T->wr[w] - b[1] * T->wi[w];
      double bi = b[0] * T->wi[w] + b[1] * T->wr[w];
      double ar = a[0], ai = a[1];
      a[0] = ar + br; a[1] = ai + bi;
      b[0] = ar - br; b[1] = ai - bi;
    }
    return;
  }
  if (p == 4) {
    for (int k = 0; k < m; k++) {
      double tr[4], ti[4];
      for (int r = 0; r < 4; r++) {
        long w = ((long)r * k * tstep) % N;
        double *c = out + 2 * (k + (long)r * m);
        tr[r] = c[0] * T->wr[w] - c[1] * T->wi[w];
        ti[r] = c[0] * T->wi[w] + c[1] * T->wr[w];
      }
      /* 4-point DFT with w4 = -i */
      double s02r = tr[0] + tr[2], s02i = ti[0] + ti[2];
      double d02r = tr[0] - tr[2], d02i = ti[0] - ti[2];
      double s13r = tr[1] + tr[3], s13i = ti[1] + ti[3];
      double d13r = tr[1] - tr[3], d13i = ti[1] - ti[3];
      double *o0 = out + 2 * k, *o1 = out + 2 * (k + m), *o2 = out + 2 * (k + 2L * m), *o3 = out + 2 * (k + 3L * m);
      o0[0] = s02r + s13r; o0[1] = s02i + s13i;
      o2[0] = s02r - s13r; o2[1] = s02i - s13i;
      /* X1 = d02 + (-i) d13 ; X3 = d02 + (i) d13 */
      o1[0] = d02r + d13i; o1[1] = d02i - d13r;
      o3[0] = d02r - d13i; o3[1] = d02i + d13r;
    }
    return;
  }
  /* generic radix p (3, 5, or any prime) */
  double *tr = (double *)malloc(sizeof(double) * 2 * (size_t)(unsigned)p);
  double *ti = tr + p;
  const long pstep = N / p; /* w_p^1 = T[N/p] */
  for (int k = 0; k < m; k++) {
    for (int r = 0; r < p; r++) {
      long w = ((long)r * k * tstep) % N;
      double *c = out + 2 * (k + (long)r * m);
      tr[r] = c[0] * T->wr[w] - c[1] * T->wi[w];
      ti[r] = c[0] * T->wi[w] + c[1] * T->wr[w];
    }
    for (int q = 0; q < p; q++) {
      double sr = 0.0, si = 0.0;
      for (int r = 0; r < p; r++) {
        long w = (((long)r * q) % p) * pstep;
        sr += tr[r] * T->wr[w] - ti[r] * T->wi[w];
        si += tr[r] * T->wi[w] + ti[r] * T->wr[w];
      }
      double *o = out + 2 * (k + (long)q * m);
      o[0] = sr;
      o[1] = si;
    }
  }
  free(tr);
}

static void fft_line(int n, const double *in, double *out, const twtab *T) { fft_rec(n, in, 1, out, T, 1); }

void orc_fft_c2c_1d(int n, const double *in, double *out) {
  twtab T;
  tw_init(&T, n);
  fft_line(n, in, out, &T);
  tw_free(&T);
}

/* transform all lines of length n (complex) found at base + l*lstride_outer..., element stride estride
 * (in complex units). sign -1 forward, +1 backward (via conjugation). */
static void lines_c2c(double *data, int n, long estride, long nlines, const long *line_off, const twtab *T,
                      int sign) {
  double *a = (double *)malloc(sizeof(double) * 4 * (size_t)n);
  double *b = a + 2 * n;
  for (long l = 0; l < nlines; l++) {
    double *base = data + 2 * line_off[l];
    for (int j = 0; j < n; j++) {
      a[2 * j] = base[2 * j * estride];
      a[2 * j + 1] = sign > 0 ? -base[2 * j * estride + 1] : base[2 * j * estride + 1];
    }
    fft_line(n, a, b, T);
    for (int j = 0; j < n; j++) {
      base[2 * j * estride] = b[2 * j];
      base[2 * j * estride + 1] = sign > 0 ? -b[2 * j + 1] : b[2 * j + 1];
    }
  }
  free(a);
}

static void axes_xy_c2c(int n0, int n1, int nzc, double *data, int sign) {
  /* along axis 1 (stride nzc), then axis 0 (stride n1*nzc), complex units */
  twtab T1, T0;
  tw_init(&T1, n1);
  tw_init(&T0, n0);
  long nl1 = (long)n0 * nzc;
  long *off = (long *)malloc(sizeof(long) * (size_t)(nl1 > (long)n1 * nzc ? nl1 : (long)n1 * nzc));
  long c = 0;
  for (int i = 0; i < n0; i++)
    for (int k = 0; k < nzc; k++) off[c++] = (long)i * n1 * nzc + k;
  lines_c2c(data, n1, nzc, nl1, off, &T1, sign);
  c = 0;
  for (int j = 0; j < n1; j++)
    for (int k = 0; k < nzc; k++) off[c++] = (long)j * nzc + k;
  lines_c2c(data, n0, (long)n1 * nzc, (long)n1 * nzc, off, &T0, sign);
  free(off);
  tw_free(&T1);
  tw_free(&T0);
}

void orc_fft_r2c_3d_inplace(int n0, int n1, int n2, double *data) {
  const int nzc = n2 / 2 + 1;
  twtab T2;
  tw_init(&T2, n2);
  double *a = (double *)malloc(sizeof(double) * 4 * (size_t)n2);
  double *b = a + 2 * n2;
  for (long row = 0; row < (long)n0 * n1; row++) {
    double *r = data + row * 2 * nzc;
    for (int k = 0; k < n2; k++) {
      a[2 * k] = r[k];
      a[2 * k + 1] = 0.0;
    }
    fft_line(n2, a, b, &T2);
    memcpy(r, b, sizeof(double) * 2 * (size_t)nzc);
  }
  free(a);
  tw_free(&T2);
  axes_xy_c2c(n0, n1, nzc, data, -1);
}

void orc_fft_c2c_3d_inplace(int n0, int n1, int n2, double *data, int sign) {
  twtab T2;
  tw_init(&T2, n2);
  long nl = (long)n0 * n1;
  long *off = (long *)malloc(sizeof(long) * (size_t)nl);
  for (long l = 0; l < nl; l++) off[l] = l * n2;
  lines_c2c(data, n2, 1, nl, off, &T2, sign);
  free(off);
  tw_free(&T2);
  axes_xy_c2c(n0, n1, n2, data, sign);
}

void orc_fft_c2r_3d_inplace(int n0, int n1, int n2, double *data) {
  const int nzc = n2 / 2 + 1;
  axes_xy_c2c(n0, n1, nzc, data, +1);
  twtab T2;
  tw_init(&T2, n2);
  double *a = (double *)malloc(sizeof(double) * 4 * (size_t)n2);
  double *b = a + 2 * n2;
  for (long row = 0; row < (long)n0 * n1; row++) {
    double *r = data + row * 2 * nzc;
    /* Hermitian extension along z, then inverse via conjugation */
    for (int k = 0; k < nzc; k++) {
      a[2 * k] = r[2 * k];
      a[2 * k + 1] = -r[2 * k + 1];
    }
    for (int k = nzc; k < n2; k++) {
      a[2 * k] = r[2 * (n2 - k)];
      a[2 * k + 1] = r[2 * (n2 - k) + 1];
    }
    fft_line(n2, a, b, &T2);
    for (int k = 0; k < n2; k++) r[k] = b[2 * k];
    for (int k = n2; k < 2 * nzc; k++) r[k] = 0.0;
  }
  free(a);
  tw_free(&T2);
}
