/* Survey catalogue reader with the reference's format, cut, bounds check and messages
 * (read_survey_serial_ascii, src/read_data.c:184-361), and the redshift-distance table it uses
 * (create_grids, src/main.c:1233-1248; comoving_distance and its integrand, src/read_data.c:365-380).
 *
 * The table: 10000 redshifts z_i = i * 10 / 9999 and their comoving distances
 * r_i = (c / 100) int_0^z_i dz / sqrt(Omega_m (1+z)^3 + 1 - Omega_m) (Mpc/h, c in km/s), with two
 * natural cubic splines through it, z(r) and r(z), as the reference builds them with GSL. The
 * reference integrates each r_i from 0 with adaptive Gauss-Kronrod to a relative 1e-7; here each
 * step [z_{i-1}, z_i] is integrated with 8-point Gauss-Legendre (nodes from Newton's method on P_8)
 * and the steps are summed, which is exact to double rounding for this smooth integrand. So the
 * redshift of an object agrees with the reference's to the table's accuracy: a cut decision can
 * differ only for an object within about 1e-9 of REDMININ or REDMAXIN.
 *
 * Reading (one pass, file order): the leading lines that start with '#' are skipped; then every
 * non-empty line must hold at least 12 (data) or 8 (random) numbers, parsed with the correctly
 * rounded reader of catalogue.c (the reference's sscanf "%lf"). The reference tokenises its buffer
 * with strtok and parses a line only while the lengths of the lines so far, plus one each, fit in
 * the bytes read, so a last line without a newline is parsed only when blank lines before it make
 * room; the same rule is applied here to the whole file. */
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "capow.h"

double capow_parse_number(const char *p, const char *e, const char **end);

#define LIGHT_SPEED 299792.458 /* km/s (src/vars.h LightSpeed) */
#define TABLE_N 10000
#define TABLE_ZMAX 10.0

typedef struct {
  int n;
  double *x, *y, *d2; /* knots, values, second derivatives */
} nspline;

/* natural cubic spline: second derivatives with d2[0] = d2[n-1] = 0 from the tridiagonal system
 * h_{i-1} d2_{i-1} + 2 (h_{i-1} + h_i) d2_i + h_i d2_{i+1} = 6 (s_i - s_{i-1}), s_i the slopes,
 * by forward elimination and back substitution */
static int nspline_init(nspline *s, const double *x, const double *y, int n) {
  s->n = n;
  s->x = (double *)malloc(sizeof(double) * n);
  s->y = (double *)malloc(sizeof(double) * n);
  s->d2 = (double *)calloc(n, sizeof(double));
  double *u = (double *)malloc(sizeof(double) * n), *v = (double *)malloc(sizeof(double) * n);
  if (!s->x || !s->y || !s->d2 || !u || !v) {
    free(u);
    free(v);
    return -1;
  }
  memcpy(s->x, x, sizeof(double) * n);
  memcpy(s->y, y, sizeof(double) * n);
  /* after elimination: d2_i = v_i - u_i d2_{i+1} */
  u[0] = v[0] = 0.0;
  for (int i = 1; i < n - 1; i++) {
    const double hl = x[i] - x[i - 1], hr = x[i + 1] - x[i];
    const double rhs = 6.0 * ((y[i + 1] - y[i]) / hr - (y[i] - y[i - 1]) / hl);
    const double den = 2.0 * (hl + hr) - hl * u[i - 1];
    u[i] = hr / den;
    v[i] = (rhs - hl * v[i - 1]) / den;
  }
  for (int i = n - 2; i >= 1; i--) s->d2[i] = v[i] - u[i] * s->d2[i + 1];
  free(u);
  free(v);
  return 0;
}

static void nspline_free(nspline *s) {
  free(s->x);
  free(s->y);
  free(s->d2);
  memset(s, 0, sizeof *s);
}

/* value at t; returns -1 outside [x_0, x_{n-1}] (GSL's interpolation error) */
static int nspline_eval(const nspline *s, double t, double *out) {
  if (!(t >= s->x[0] && t <= s->x[s->n - 1])) return -1;
  int lo = 0, hi = s->n - 1;
  while (hi - lo > 1) {
    const int mid = (lo + hi) / 2;
    if (s->x[mid] > t) hi = mid;
    else lo = mid;
  }
  const double h = s->x[hi] - s->x[lo];
  const double a = (s->x[hi] - t) / h, b = (t - s->x[lo]) / h;
  *out = a * s->y[lo] + b * s->y[hi] + ((a * a * a - a) * s->d2[lo] + (b * b * b - b) * s->d2[hi]) * (h * h) / 6.0;
  return 0;
}

/* 8-point Gauss-Legendre nodes and weights on [-1, 1]: Newton's method on P_8 from Chebyshev-like
 * starting points, P_8 and P_8' by the three-term recurrence */
static void gauss_legendre8(double xs[8], double ws[8]) {
  const int n = 8;
  for (int i = 0; i < n; i++) {
    double x = cos(M_PI * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = x;
      for (int k = 2; k <= n; k++) {
        const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      const double dp = n * (x * p1 - p0) / (x * x - 1.0);
      const double dx = p1 / dp;
      x -= dx;
      if (fabs(dx) < 1e-16) {
        double q0 = 1.0, q1 = x;
        for (int k = 2; k <= n; k++) {
          const double q2 = ((2.0 * k - 1.0) * x * q1 - (k - 1.0) * q0) / k;
          q0 = q1;
          q1 = q2;
        }
        const double d = n * (x * q1 - q0) / (x * x - 1.0);
        ws[i] = 2.0 / ((1.0 - x * x) * d * d);
        break;
      }
    }
    xs[i] = x;
  }
}

static double hubble_inv(double om, double z) {
  const double a = 1.0 + z;
  return 1.0 / sqrt(om * a * a * a + (1.0 - om));
}

typedef struct {
  nspline z_of_r, r_of_z;
} redshift_table;

static int table_build(redshift_table *t, double omega_m) {
  double *z = (double *)malloc(sizeof(double) * TABLE_N), *r = (double *)malloc(sizeof(double) * TABLE_N);
  if (!z || !r) {
    free(z);
    free(r);
    return -1;
  }
  double gx[8], gw[8];
  gauss_legendre8(gx, gw);
  const double step = TABLE_ZMAX / (double)(TABLE_N - 1);
  z[0] = r[0] = 0.0;
  double acc = 0.0;
  for (int i = 1; i < TABLE_N; i++) {
    z[i] = i * step;
    const double a = z[i - 1], b = z[i], half = 0.5 * (b - a), mid = 0.5 * (a + b);
    double s = 0.0;
    for (int q = 0; q < 8; q++) s += gw[q] * hubble_inv(omega_m, mid + half * gx[q]);
    acc += half * s;
    r[i] = LIGHT_SPEED * acc / 100.0;
  }
  int rc = nspline_init(&t->z_of_r, r, z, TABLE_N);
  if (!rc) rc = nspline_init(&t->r_of_z, z, r, TABLE_N);
  free(z);
  free(r);
  return rc;
}

static void table_free(redshift_table *t) {
  nspline_free(&t->z_of_r);
  nspline_free(&t->r_of_z);
}

/* growable text buffer for the lines the reference prints while reading */
typedef struct {
  char *s;
  size_t len, cap;
} textbuf;

static void tb_add(textbuf *b, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
static void tb_add(textbuf *b, const char *fmt, ...) {
  char tmp[512];
  va_list ap;
  va_start(ap, fmt);
  int k = vsnprintf(tmp, sizeof tmp, fmt, ap);
  va_end(ap);
  if (k < 0) return;
  if ((size_t)k >= sizeof tmp) k = sizeof tmp - 1;
  if (b->len + k + 1 > b->cap) {
    size_t nc = b->cap ? 2 * b->cap : 4096;
    while (nc < b->len + k + 1) nc *= 2;
    char *q = (char *)realloc(b->s, nc);
    if (!q) return;
    b->s = q;
    b->cap = nc;
  }
  memcpy(b->s + b->len, tmp, (size_t)k);
  b->len += k;
  b->s[b->len] = 0;
}

void capow_survey_objects_free(capow_survey_objects *o) {
  if (!o) return;
  free(o->x);
  free(o->y);
  free(o->z);
  free(o->w);
  free(o->nbar);
  free(o->redshift);
  free(o->pv);
  free(o->pverr);
  free(o->log);
  memset(o, 0, sizeof *o);
}

static int grow(capow_survey_objects *o, size_t *cap) {
  size_t nc = *cap ? 2 * *cap : 65536;
  float **arr[8] = {&o->x, &o->y, &o->z, &o->w, &o->nbar, &o->redshift, &o->pv, &o->pverr};
  for (int k = 0; k < 8; k++) {
    float *q = (float *)realloc(*arr[k], sizeof(float) * nc);
    if (!q) return -1;
    *arr[k] = q;
  }
  *cap = nc;
  return 0;
}

/* natural log; capow_read_survey's text buffer is named log */
static double log_of(double a) { return log(a); }

int capow_read_survey(const char *path, const capow_params *p, const capow_survey_params *sv, int randoms,
                      capow_survey_objects *out, char *msg, size_t msglen) {
  if (msg && msglen) msg[0] = 0;
  if (!path || !p || !sv || !out) return CAPOW_EINVAL;
  memset(out, 0, sizeof *out);
  FILE *f = fopen(path, "rb");
  if (!f) { /* src/read_data.c:213 */
    if (msg) snprintf(msg, msglen, "Task 0 cannot open input file\nFatal Error at line 113 in routine read_data\n");
    return CAPOW_EINVAL;
  }
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  char *buf = (char *)malloc((size_t)(sz > 0 ? sz : 0) + 1);
  if (!buf) {
    fclose(f);
    return CAPOW_ENOMEM;
  }
  size_t got = fread(buf, 1, (size_t)(sz > 0 ? sz : 0), f);
  fclose(f);
  buf[got] = 0;
  const char *end = buf + got;
  redshift_table tab;
  memset(&tab, 0, sizeof tab);
  if (table_build(&tab, p->Omega_m)) {
    free(buf);
    return CAPOW_ENOMEM;
  }
  /* the grid less the interpolation margin (src/read_data.c:196-204) */
  const double dx = (p->XMAX - p->XMIN) / (double)p->NX, dy = (p->YMAX - p->YMIN) / (double)p->NY,
               dz = (p->ZMAX - p->ZMIN) / (double)p->NZ;
  const int io = p->InterpOrder - 1;
  const double xlo = p->XMIN + io * dx, ylo = p->YMIN + io * dy, zlo = p->ZMIN + io * dz;
  double xhi = p->XMAX - io * dx, yhi = p->YMAX - io * dy, zhi = p->ZMAX - io * dz;
  if (p->DoInterlacing) {
    xhi -= 0.5 * dx;
    yhi -= 0.5 * dy;
    zhi -= 0.5 * dz;
  }
  /* the leading '#' lines (src/read_data.c:216-221); when every line is one, the reference steps back
     to the last of them and parses it as data */
  const char *q = buf;
  const char *last_comment = NULL;
  while (q < end && *q == '#') {
    last_comment = q;
    const char *nl = memchr(q, '\n', (size_t)(end - q));
    q = nl ? nl + 1 : end;
  }
  if (q >= end && last_comment) q = last_comment;
  const size_t avail = (size_t)(end - q);
  const int need = randoms ? 8 : 12;
  textbuf log = {0};
  size_t cap = 0;
  int rc = CAPOW_OK;
  double lo[3] = {1.0e-30, 1.0e-30, 1.0e-30}, hi[3] = {-1.0e30, -1.0e30, -1.0e30};
  double redmin = 1.0e30, redmax = -1.0e30;
  unsigned long long nread = 0, nkeep = 0;
  size_t used = 0; /* sum of (line length + 1) over the lines so far: the reference's largelen */
  while (q < end) {
    const char *nl = memchr(q, '\n', (size_t)(end - q));
    const char *le = nl ? nl : end;
    if (le == q) { /* strtok skips empty lines */
      q = nl ? nl + 1 : end;
      continue;
    }
    used += (size_t)(le - q) + 1;
    if (used > avail) break;
    double v[12];
    int k = 0;
    const char *s = q;
    while (k < need) {
      while (s < le && (*s == ' ' || *s == '\t' || *s == '\r' || *s == '\v' || *s == '\f')) s++;
      if (s >= le) break;
      const char *ne;
      const double d = capow_parse_number(s, le, &ne);
      if (ne == s || ne > le) break;
      v[k++] = d;
      s = ne;
    }
    if (k != need) { /* src/read_data.c:240-247 */
      if (msg)
        snprintf(msg, msglen, "Task 0 has error reading file: %.*s\nFatal Error at line 102 in routine read_data\n",
                 (int)((le - q) > 1999 ? 1999 : (le - q)), q);
      rc = CAPOW_EINVAL;
      break;
    }
    double tx = v[0], ty = v[1], tz = v[2], tw = v[3];
    const double tnbar = v[4];
    nread++;
    if (nread % 1000000 == 0) tb_add(&log, "Read %llu objects, kept %llu\n", nread, nkeep);
    double tred;
    if (sv->Coord_Type == 0) { /* src/read_data.c:258-266 */
      if (nspline_eval(&tab.z_of_r, sqrt(tx * tx + ty * ty + tz * tz), &tred)) {
        if (msg)
          snprintf(msg, msglen, "interpolation error: distance %g outside the redshift-distance table (z in [0, 10])\n",
                   sqrt(tx * tx + ty * ty + tz * tz));
        rc = CAPOW_EINVAL;
        break;
      }
      if ((tred < sv->REDMININ) || (tred > sv->REDMAXIN)) {
        q = nl ? nl + 1 : end;
        continue;
      }
    } else { /* src/read_data.c:267-291 */
      tred = tz;
      if ((tred < sv->REDMININ) || (tred > sv->REDMAXIN)) {
        q = nl ? nl + 1 : end;
        continue;
      }
      if (tw == 0) {
        tb_add(&log, "%lf, %lf, %lf, %lf, %lf\n", tx, ty, tz, tw, tnbar);
        q = nl ? nl + 1 : end;
        continue;
      }
      double tdist;
      if (nspline_eval(&tab.r_of_z, tred, &tdist)) {
        if (msg) snprintf(msg, msglen, "interpolation error: redshift %g outside the redshift-distance table\n", tred);
        rc = CAPOW_EINVAL;
        break;
      }
      double ra = tx, dec = ty;
      if (sv->Coord_Type == 1) {
        ra *= (M_PI / 180.0);
        dec *= (M_PI / 180.0);
      }
      tx = tdist * cos(dec) * cos(ra);
      ty = tdist * cos(dec) * sin(ra);
      tz = tdist * sin(dec);
    }
    if ((tx < xlo) || (tx >= xhi) || (ty < ylo) || (ty >= yhi) || (tz < zlo) || (tz >= zhi)) { /* :293-299 */
      if (msg)
        snprintf(msg, msglen,
                 "Task 0 has object out of grid bounds for chosen InterpOrder: x=%lf, y=%lf, z=%lf, red=%lf\n"
                 "Fatal Error at line 155 in routine read_data\n",
                 tx, ty, tz, tred);
      rc = CAPOW_EINVAL;
      break;
    }
    if (sv->NOBJ_Max >= 0 && nkeep >= (unsigned long long)sv->NOBJ_Max) {
      /* the reference writes past its NOBJ_Max-object array here */
      if (msg) snprintf(msg, msglen, "more than NOBJ_Max = %lld objects kept\n", sv->NOBJ_Max);
      rc = CAPOW_EINVAL;
      break;
    }
    if (nkeep >= cap && grow(out, &cap)) {
      rc = CAPOW_ENOMEM;
      break;
    }
    out->x[nkeep] = (float)tx;
    out->y[nkeep] = (float)ty;
    out->z[nkeep] = (float)tz;
    out->redshift[nkeep] = (float)tred;
    out->w[nkeep] = (float)tw;
    out->nbar[nkeep] = sv->NBAR_Column > 0 ? (float)tnbar : 0.0f;
    out->pv[nkeep] = out->pverr[nkeep] = 0.0f;
    if (p->Momentum) { /* src/read_data.c:308-316 */
      const double ln10 = log_of(10.0);
      const double q = 3.0 / 2.0 * p->Omega_m - 1.0;
      const double zmod = tred * (1.0 + 0.5 * (1.0 - q) * tred - 1.0 / 6.0 * (2.0 - q - 3.0 * q * q) * tred * tred);
      const double tlogdist = randoms ? 0.0 : v[6], tlogdist_err = randoms ? v[6] : v[7];
      out->pv[nkeep] = (float)(LIGHT_SPEED * zmod * ln10 * tlogdist / (1.0 + zmod));
      out->pverr[nkeep] = (float)(LIGHT_SPEED * zmod * ln10 * tlogdist_err / (1.0 + zmod));
    }
    nkeep++;
    if (tred < redmin) redmin = tred;
    if (tred > redmax) redmax = tred;
    if (tx < lo[0]) lo[0] = tx;
    if (ty < lo[1]) lo[1] = ty;
    if (tz < lo[2]) lo[2] = tz;
    if (tx > hi[0]) hi[0] = tx;
    if (ty > hi[1]) hi[1] = ty;
    if (tz > hi[2]) hi[2] = tz;
    q = nl ? nl + 1 : end;
  }
  free(buf);
  table_free(&tab);
  out->n = (size_t)nkeep;
  out->nread = nread;
  for (int a = 0; a < 3; a++) {
    out->lo[a] = lo[a];
    out->hi[a] = hi[a];
  }
  out->redmin = redmin;
  out->redmax = redmax;
  out->log = log.s;
  if (rc != CAPOW_OK) { /* keep the lines printed before the error */
    char *keep = out->log;
    out->log = NULL;
    capow_survey_objects_free(out);
    out->log = keep;
    return rc;
  }
  if (!out->x && grow(out, &cap)) { /* empty catalogue: valid, non-NULL arrays */
    capow_survey_objects_free(out);
    return CAPOW_ENOMEM;
  }
  return CAPOW_OK;
}

/* compute_nbar (src/read_data.c:385-446), one rank. The number density per redshift bin of width
 * (REDMAX - REDMIN) / nbins, nbins = ceil((REDMAXIN - REDMININ) / 0.002), REDMIN and REDMAX the range of
 * the kept objects of both catalogues; counts over the volume of the bin's shell of sky area SkyArea
 * (square degrees); a natural cubic spline through the bin centres, with the raw end values at half a
 * bin beyond each end; every object's nbar from that spline, stored in its float field. As in the
 * reference, the counts loop runs over the data's indices but reads the randoms' redshifts (:401-405);
 * with more data than randoms the reference reads objects it never filled, which is an error here. */
int capow_survey_nbar(const capow_params *p, const capow_survey_params *sv, capow_survey_objects *data,
                      capow_survey_objects *rand, char **log_out, char *msg, size_t msglen) {
  if (msg && msglen) msg[0] = 0;
  if (log_out) *log_out = NULL;
  if (!p || !sv || !data || !rand) return CAPOW_EINVAL;
  const int nbins = (int)(ceil((sv->REDMAXIN - sv->REDMININ) / 0.002));
  if (nbins < 1) {
    if (msg) snprintf(msg, msglen, "compute_nbar needs REDMAXIN > REDMININ\n");
    return CAPOW_EINVAL;
  }
  if (data->n > rand->n) {
    if (msg)
      snprintf(msg, msglen, "compute_nbar reads the redshifts of the first %zu randoms, but only %zu were kept\n",
               data->n, rand->n);
    return CAPOW_EINVAL;
  }
  const double redmin = data->redmin < rand->redmin ? data->redmin : rand->redmin;
  const double redmax = data->redmax > rand->redmax ? data->redmax : rand->redmax;
  const double rbw = (redmax - redmin) / (float)nbins;
  double *znbar = (double *)calloc((size_t)nbins + 2, sizeof(double));
  double *nbar = (double *)calloc((size_t)nbins + 2, sizeof(double));
  redshift_table tab;
  memset(&tab, 0, sizeof tab);
  nspline sp;
  memset(&sp, 0, sizeof sp);
  textbuf log = {0};
  int rc = CAPOW_OK;
  if (!znbar || !nbar || table_build(&tab, p->Omega_m)) {
    rc = CAPOW_ENOMEM;
    goto done;
  }
  tb_add(&log, "Calculating Number Density...\n");
  for (size_t i = 0; i < data->n; i++) {
    int nb = (int)(floor(((double)rand->redshift[i] - redmin) / rbw)) + 1;
    if (nb == nbins + 1) nb--;
    if (nb < 0 || nb > nbins + 1) {
      if (msg) snprintf(msg, msglen, "compute_nbar: redshift %g outside [%g, %g]\n", (double)rand->redshift[i], redmin,
                        redmax);
      rc = CAPOW_EINVAL;
      goto done;
    }
    nbar[nb]++;
  }
  for (int i = 0; i < nbins; i++) {
    double outer, inner;
    if (nspline_eval(&tab.r_of_z, (i + 1) * rbw + redmin, &outer) || nspline_eval(&tab.r_of_z, i * rbw + redmin, &inner)) {
      if (msg) snprintf(msg, msglen, "interpolation error: redshift outside the redshift-distance table\n");
      rc = CAPOW_EINVAL;
      goto done;
    }
    const double volume =
        sv->SkyArea / (180.0 * 180.0) * M_PI * M_PI * (outer * outer * outer - inner * inner * inner) / 3.0;
    znbar[i + 1] = (i + 0.5) * rbw + redmin;
    nbar[i + 1] /= volume;
    tb_add(&log, "%12.6lf, %12.6lf\n", znbar[i + 1], nbar[i + 1]);
  }
  znbar[0] = redmin - 0.5 * rbw;
  znbar[nbins + 1] = redmax + 0.5 * rbw;
  if (nspline_init(&sp, znbar, nbar, nbins + 2)) {
    rc = CAPOW_ENOMEM;
    goto done;
  }
  capow_survey_objects *cats[2] = {data, rand};
  for (int c = 0; c < 2; c++)
    for (size_t i = 0; i < cats[c]->n; i++) {
      double v;
      if (nspline_eval(&sp, (double)cats[c]->redshift[i], &v)) {
        if (msg) snprintf(msg, msglen, "interpolation error: redshift outside the number-density table\n");
        rc = CAPOW_EINVAL;
        goto done;
      }
      cats[c]->nbar[i] = (float)v;
    }
done:
  free(znbar);
  free(nbar);
  table_free(&tab);
  nspline_free(&sp);
  if (log_out) *log_out = log.s;
  else free(log.s);
  return rc;
}
