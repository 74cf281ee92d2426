/* GSL stand-ins (TEST INFRASTRUCTURE ONLY), linked into the reference build (oracle/Makefile.ref) and
 * into the oracle library: the reference's survey path calls them (src/main.c:1233-1248,
 * src/read_data.c:365-446). */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "shims/gsl/gsl_integration.h"
#include "shims/gsl/gsl_spline.h"

/* GSL is absent here. The survey path of the reference evaluates two splines of the comoving-distance
 * table that create_grids builds (main.c:1233-1248) with gsl_integration_qags, and a spline of the
 * number density (read_data.c:385-446). These stand-ins restate the published methods: a natural
 * cubic spline (second derivatives from the tridiagonal system with zero end curvature, evaluated on
 * the bracketing interval) and adaptive Gauss-Kronrod (7-15 point) quadrature, bisecting the
 * interval of largest error until the estimate meets max(epsabs, epsrel |I|). Results agree with
 * GSL's to the requested tolerance, not bit for bit. */
static const gsl_interp_type g_cspline = {0};
const gsl_interp_type *gsl_interp_cspline = &g_cspline;
gsl_interp_accel *gsl_interp_accel_alloc(void) { return (gsl_interp_accel *)calloc(1, sizeof(gsl_interp_accel)); }
void gsl_interp_accel_free(gsl_interp_accel *a) { free(a); }
gsl_spline *gsl_spline_alloc(const gsl_interp_type *t, size_t n) {
  (void)t;
  gsl_spline *s = (gsl_spline *)calloc(1, sizeof(gsl_spline));
  s->n = n;
  s->x = (double *)calloc(n, sizeof(double));
  s->y = (double *)calloc(n, sizeof(double));
  s->m = (double *)calloc(n, sizeof(double));
  return s;
}
int gsl_spline_init(gsl_spline *s, const double *x, const double *y, size_t n) {
  if (n > s->n || n < 3) return 1;
  s->n = n;
  memcpy(s->x, x, n * sizeof(double));
  memcpy(s->y, y, n * sizeof(double));
  /* natural spline: M_0 = M_{n-1} = 0; Thomas algorithm on the interior equations
     h_{i-1} M_{i-1} + 2 (h_{i-1} + h_i) M_i + h_i M_{i+1} = 6 (d_i - d_{i-1}) */
  double *cp = (double *)calloc(n, sizeof(double)), *dp = (double *)calloc(n, sizeof(double));
  s->m[0] = s->m[n - 1] = 0.0;
  for (size_t i = 1; i + 1 < n; i++) {
    const double h0 = x[i] - x[i - 1], h1 = x[i + 1] - x[i];
    const double rhs = 6.0 * ((y[i + 1] - y[i]) / h1 - (y[i] - y[i - 1]) / h0);
    const double diag = 2.0 * (h0 + h1) - (i > 1 ? h0 * cp[i - 1] : 0.0);
    cp[i] = h1 / diag;
    dp[i] = (rhs - (i > 1 ? h0 * dp[i - 1] : 0.0)) / diag;
  }
  for (size_t i = n - 2; i >= 1; i--) s->m[i] = dp[i] - cp[i] * s->m[i + 1];
  free(cp);
  free(dp);
  return 0;
}
double gsl_spline_eval(const gsl_spline *s, double xv, gsl_interp_accel *a) {
  (void)a;
  size_t lo = 0, hi = s->n - 1;
  while (hi - lo > 1) {
    const size_t mid = (lo + hi) / 2;
    if (s->x[mid] > xv) hi = mid;
    else lo = mid;
  }
  const double h = s->x[lo + 1] - s->x[lo], t = xv - s->x[lo];
  const double b = (s->y[lo + 1] - s->y[lo]) / h - h * (2.0 * s->m[lo] + s->m[lo + 1]) / 6.0;
  const double c = 0.5 * s->m[lo], d = (s->m[lo + 1] - s->m[lo]) / (6.0 * h);
  return s->y[lo] + t * (b + t * (c + t * d));
}
void gsl_spline_free(gsl_spline *s) {
  if (!s) return;
  free(s->x);
  free(s->y);
  free(s->m);
  free(s);
}
gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n) {
  gsl_integration_workspace *w = (gsl_integration_workspace *)calloc(1, sizeof *w);
  w->limit = n;
  return w;
}
void gsl_integration_workspace_free(gsl_integration_workspace *w) { free(w); }

/* Kronrod 15-point rule with its embedded 7-point Gauss rule on [a, b] (QUADPACK's published nodes and
   weights); returns the Kronrod value, the |K - G| error estimate in *err */
static double gk15(const gsl_function *f, double a, double b, double *err) {
  static const double xgk[8] = {0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
                                0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
                                0.586087235467691130294144845693013, 0.405845151377397166906606412076961,
                                0.207784955007898467600689403773245, 0.0};
  static const double wgk[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                                0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                                0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                                0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
  static const double wg[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                               0.381830050505118944950369775488975, 0.417959183673469387755102040816327};
  const double c = 0.5 * (a + b), h = 0.5 * (b - a);
  const double fc = f->function(c, f->params);
  double rk = fc * wgk[7], rg = fc * wg[3];
  for (int j = 0; j < 7; j++) {
    const double dx = h * xgk[j];
    const double fs = f->function(c - dx, f->params) + f->function(c + dx, f->params);
    rk += wgk[j] * fs;
    if (j & 1) rg += wg[j / 2] * fs;
  }
  *err = fabs((rk - rg) * h);
  return rk * h;
}

int gsl_integration_qags(const gsl_function *f, double a, double b, double epsabs, double epsrel, size_t limit,
                         gsl_integration_workspace *w, double *result, double *abserr) {
  (void)w;
  if (limit < 1) limit = 1;
  double *ia = (double *)malloc(limit * sizeof(double)), *ib = (double *)malloc(limit * sizeof(double));
  double *iv = (double *)malloc(limit * sizeof(double)), *ie = (double *)malloc(limit * sizeof(double));
  size_t n = 1;
  ia[0] = a;
  ib[0] = b;
  iv[0] = gk15(f, a, b, &ie[0]);
  for (;;) {
    double tot = 0.0, terr = 0.0;
    size_t worst = 0;
    for (size_t i = 0; i < n; i++) {
      tot += iv[i];
      terr += ie[i];
      if (ie[i] > ie[worst]) worst = i;
    }
    const double tol = fmax(epsabs, epsrel * fabs(tot));
    if (terr <= tol || n == limit) {
      *result = tot;
      *abserr = terr;
      break;
    }
    const double m = 0.5 * (ia[worst] + ib[worst]);  /* bisect the interval of largest error */
    ia[n] = m;
    ib[n] = ib[worst];
    ib[worst] = m;
    iv[worst] = gk15(f, ia[worst], ib[worst], &ie[worst]);
    iv[n] = gk15(f, ia[n], ib[n], &ie[n]);
    n++;
  }
  free(ia);
  free(ib);
  free(iv);
  free(ie);
  return 0;
}
