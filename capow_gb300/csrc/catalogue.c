/* ASCII particle catalogue reader with the reference's format and error behaviour
 * (src/read_data.c:50-76): one particle per line as `x y z vx vy vz`, lines starting with
 * '#' skipped, any other line that does not hold six numbers is a fatal error. The line of
 * sight picks the velocity column (LOS 1 -> vx, 2 -> vy, otherwise vz).
 *
 * The file is read in one pass into memory and its lines are parsed by several threads, each
 * writing its own contiguous range, so the particle order of the file is kept. Numbers are
 * correctly rounded like the reference's sscanf("%lf"): Clinger's fast path where it is exact
 * (at most 19 significant digits, mantissa <= 2^53, |decimal exponent| <= 22: one IEEE multiply or
 * divide of two exact doubles), else the Eisel-Lemire method for up to 19 digits (a 192-bit product
 * with a 128-bit significand of 5^q), and strtod wherever those cannot decide. */
#include <errno.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "capow.h"
#include "pow5_table.h"

typedef struct {
  const char *b, *e; /* [b, e) whole lines */
  size_t n;          /* particles in this chunk */
  size_t off;        /* output offset */
  int los;
  double *x, *y, *z, *v;
  const char *bad;   /* first bad line, if any */
} chunk;

static int is_hspace(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

static const double pow10_exact[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                       1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

/* w * 10^q correctly rounded, w != 0 with at most 19 digits (Eisel-Lemire). With F the 128-bit
 * significand of 5^q (5^q = F 2^(e5 - 127), e5 = floor(log2 5^q)) and wn = w << lz normalised,
 * w 10^q = P 2^(e5 - 127 + q - lz) for the 192-bit product P = wn F, whose leading bit is bit
 * 190 + u (u = 0 or 1). The top 54 bits of P give the 53-bit significand and its round bit. F is
 * exact for 0 <= q <= 55; otherwise it is truncated and the true product lies in [P, P + 2^64), so
 * a carry into the kept bits (every bit from 64 to the round bit set) or an apparent tie cannot be
 * decided here. Returns 0 then, and for subnormal, zero or infinite results (strtod decides). */
static int eisel_lemire(uint64_t w, int q, int neg, double *out) {
  if (q < POW5_QMIN || q > POW5_QMAX) return 0;
  const int lz = __builtin_clzll(w);
  const uint64_t wn = w << lz;
  const uint64_t fh = pow5_128[q - POW5_QMIN][0], fl = pow5_128[q - POW5_QMIN][1];
  const unsigned __int128 a = (unsigned __int128)wn * fh, b = (unsigned __int128)wn * fl;
  const uint64_t p0 = (uint64_t)b;
  const unsigned __int128 t = (unsigned __int128)(uint64_t)a + (uint64_t)(b >> 64);
  const uint64_t p1 = (uint64_t)t;
  const uint64_t p2 = (uint64_t)(a >> 64) + (uint64_t)(t >> 64);
  const int u = (int)(p2 >> 63);
  const int sh = 9 + u;  /* bits of p2 below the 54 kept ones */
  const uint64_t m54 = p2 >> sh, below = p2 & ((1ULL << sh) - 1);
  if (!(q >= 0 && q <= 55)) {
    if (below == (1ULL << sh) - 1 && p1 == ~0ULL) return 0;
    if ((m54 & 1) && below == 0 && p1 == 0 && p0 == 0) return 0;
  }
  uint64_t m = m54 >> 1;
  int e2 = 63 + u + (((217706 * q) >> 16) - q) + q - lz;  /* binary exponent of the leading bit */
  if ((m54 & 1) && (below != 0 || p1 != 0 || p0 != 0 || (m & 1))) m++;
  if (m == (1ULL << 53)) {
    m >>= 1;
    e2++;
  }
  const int be = e2 + 1023;
  if (be < 1 || be > 2046) return 0;
  const uint64_t bits = ((uint64_t)(neg ? 1 : 0) << 63) | ((uint64_t)be << 52) | (m & ((1ULL << 52) - 1));
  memcpy(out, &bits, sizeof bits);
  return 1;
}

/* One decimal number at p (no leading space), ending before e. Sets *end to the first character
 * after it (p when there is none), with strtod's result. Shared with the survey reader, not exported. */
__attribute__((visibility("hidden"))) double capow_parse_number(const char *p, const char *e, const char **end) {
  const char *s = p;
  int neg = 0;
  if (s < e && (*s == '+' || *s == '-')) neg = *s++ == '-';
  uint64_t m = 0;
  int nd = 0, exp10 = 0, digits = 0, exact = 1;
  while (s < e && *s >= '0' && *s <= '9') {
    if (nd < 19) {
      m = m * 10 + (uint64_t)(*s - '0');
      if (m) nd++;
    } else {
      exact = 0;
    }
    digits++;
    s++;
  }
  if (s < e && *s == '.') {
    s++;
    while (s < e && *s >= '0' && *s <= '9') {
      if (nd < 19) {
        m = m * 10 + (uint64_t)(*s - '0');
        if (m) nd++;
        exp10--;
      } else {
        exact = 0;
      }
      digits++;
      s++;
    }
  }
  if (digits && s < e && (*s == 'e' || *s == 'E')) {
    const char *t = s + 1;
    int eneg = 0, ev = 0, ed = 0;
    if (t < e && (*t == '+' || *t == '-')) eneg = *t++ == '-';
    while (t < e && *t >= '0' && *t <= '9') {
      if (ev < 100000) ev = ev * 10 + (*t - '0');
      ed++;
      t++;
    }
    if (ed) {  /* otherwise the 'e' is not part of the number */
      exp10 += eneg ? -ev : ev;
      s = t;
    }
  }
  /* hex, inf and nan (x, i, n after the digits or none), long mantissas and large exponents */
  const int plain = digits && !(s < e && (*s == 'x' || *s == 'X' || *s == 'i' || *s == 'I' || *s == 'n' || *s == 'N'));
  if (plain && exact && m <= (1ULL << 53) && exp10 >= -22 && exp10 <= 22) {
    double d = (double)m;
    d = exp10 < 0 ? d / pow10_exact[-exp10] : d * pow10_exact[exp10];
    *end = s;
    return neg ? -d : d;
  }
  if (plain && exact && m != 0) {
    double d;
    if (eisel_lemire(m, exp10, neg, &d)) {
      *end = s;
      return d;
    }
  }
  char *q;
  const double d = strtod(p, &q);
  *end = q;
  return d;
}

/* parse up to six numbers of one line [p, e); returns how many were read */
static int parse_line(const char *p, const char *e, double out[6]) {
  int k = 0;
  while (k < 6) {
    while (p < e && is_hspace(*p)) p++;
    if (p >= e) break;
    const char *end;
    double v = capow_parse_number(p, e, &end);
    if (end == p || end > e) break;
    out[k++] = v;
    p = end;
  }
  return k;
}

static void *count_lines(void *arg) {
  chunk *c = (chunk *)arg;
  size_t n = 0;
  const char *p = c->b;
  while (p < c->e) {
    const char *nl = memchr(p, '\n', (size_t)(c->e - p));
    const char *le = nl ? nl : c->e;
    if (!(le > p && *p == '#')) n++;
    p = nl ? nl + 1 : c->e;
  }
  c->n = n;
  return NULL;
}

static void *parse_chunk(void *arg) {
  chunk *c = (chunk *)arg;
  size_t i = c->off;
  const char *p = c->b;
  double v[6];
  while (p < c->e) {
    const char *nl = memchr(p, '\n', (size_t)(c->e - p));
    const char *le = nl ? nl : c->e;
    if (!(le > p && *p == '#')) {
      if (parse_line(p, le, v) != 6) {
        c->bad = p;
        return NULL;
      }
      c->x[i] = v[0];
      c->y[i] = v[1];
      c->z[i] = v[2];
      c->v[i] = (c->los == 1) ? v[3] : (c->los == 2 ? v[4] : v[5]);
      i++;
    }
    p = nl ? nl + 1 : c->e;
  }
  return NULL;
}

int capow_read_catalogue(const char *path, int los, size_t *n_out, double **x, double **y, double **z, double **vlos,
                         char *msg, size_t msglen) {
  if (msg && msglen) msg[0] = 0;
  *n_out = 0;
  *x = *y = *z = *vlos = NULL;
  FILE *f = fopen(path, "rb");
  if (!f) { /* src/read_data.c:51 */
    if (msg) snprintf(msg, msglen, "Task 0 cannot open input file\nFatal Error at line 96 in routine read_data\n");
    return CAPOW_EINVAL;
  }
  if (fseek(f, 0, SEEK_END) != 0) {
    fclose(f);
    return CAPOW_EINVAL;
  }
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  char *buf = (char *)malloc((size_t)sz + 1);
  if (!buf) {
    fclose(f);
    return CAPOW_ENOMEM;
  }
  size_t got = fread(buf, 1, (size_t)sz, f);
  fclose(f);
  buf[got] = 0;
  const char *end = buf + got;
  long ncpu = sysconf(_SC_NPROCESSORS_ONLN);
  int nt = (int)(ncpu > 0 ? ncpu : 1);
  if (nt > 32) nt = 32;
  if (got < (1u << 20)) nt = 1;
  chunk ch[32];
  pthread_t th[32];
  const char *p = buf;
  for (int t = 0; t < nt; t++) {
    memset(&ch[t], 0, sizeof ch[t]);
    ch[t].b = p;
    const char *q = (t == nt - 1) ? end : buf + (size_t)got * (t + 1) / nt;
    if (q < p) q = p;
    if (q < end) {
      const char *nl = memchr(q, '\n', (size_t)(end - q));
      q = nl ? nl + 1 : end;
    }
    ch[t].e = q;
    ch[t].los = los;
    p = q;
  }
  for (int t = 0; t < nt; t++) pthread_create(&th[t], NULL, count_lines, &ch[t]);
  for (int t = 0; t < nt; t++) pthread_join(th[t], NULL);
  size_t total = 0;
  for (int t = 0; t < nt; t++) {
    ch[t].off = total;
    total += ch[t].n;
  }
  double *a = (double *)malloc(sizeof(double) * (total ? total : 1));
  double *b = (double *)malloc(sizeof(double) * (total ? total : 1));
  double *c = (double *)malloc(sizeof(double) * (total ? total : 1));
  double *d = (double *)malloc(sizeof(double) * (total ? total : 1));
  if (!a || !b || !c || !d) {
    free(a); free(b); free(c); free(d); free(buf);
    return CAPOW_ENOMEM;
  }
  for (int t = 0; t < nt; t++) {
    ch[t].x = a; ch[t].y = b; ch[t].z = c; ch[t].v = d;
    pthread_create(&th[t], NULL, parse_chunk, &ch[t]);
  }
  for (int t = 0; t < nt; t++) pthread_join(th[t], NULL);
  for (int t = 0; t < nt; t++) {
    if (ch[t].bad) { /* src/read_data.c:64 */
      const char *le = memchr(ch[t].bad, '\n', (size_t)(end - ch[t].bad));
      size_t len = le ? (size_t)(le - ch[t].bad + 1) : (size_t)(end - ch[t].bad);
      if (len > 1999) len = 1999;
      if (msg)
        snprintf(msg, msglen, "Task 0 has error reading file: %.*s\nFatal Error at line 102 in routine read_data\n",
                 (int)len, ch[t].bad);
      free(a); free(b); free(c); free(d); free(buf);
      return CAPOW_EINVAL;
    }
  }
  free(buf);
  *n_out = total;
  *x = a; *y = b; *z = c; *vlos = d;
  return CAPOW_OK;
}

void capow_free(void *p) { free(p); }

/* ------------------------------------------------------------------ binary SoA catalogues */
/* A catalogue the reference has no reader for: the six columns x y z vx vy vz as little-endian
 * arrays after a 32-byte header (magic "CAPOWSOA", version 1, dtype 0 float32 / 1 float64, n, 6
 * columns). The columns the paint needs (x, y, z and the one LOS selects) are read into one host
 * allocation, page-locked with cudaHostRegister where a device is present, so the paint's
 * host-to-device copies run at the link's full rate. */
#include <cuda_runtime_api.h>

typedef struct {
  char magic[8];
  uint32_t version, dtype;
  uint64_t n;
  uint32_t ncols, reserved;
} soa_header;

void capow_free_host(void *p);

int capow_is_soa_catalogue(const char *path) {
  FILE *f = fopen(path, "rb");
  if (!f) return 0;
  char m[8];
  const int ok = fread(m, 1, 8, f) == 8 && memcmp(m, "CAPOWSOA", 8) == 0;
  fclose(f);
  return ok;
}

int capow_read_catalogue_soa(const char *path, int los, size_t *n_out, int *dtype, void **x, void **y, void **z,
                             void **vlos, char *msg, size_t msglen) {
  if (msg && msglen) msg[0] = 0;
  *n_out = 0;
  *x = *y = *z = *vlos = NULL;
  FILE *f = fopen(path, "rb");
  if (!f) {
    if (msg) snprintf(msg, msglen, "Task 0 cannot open input file\nFatal Error at line 96 in routine read_data\n");
    return CAPOW_EINVAL;
  }
  soa_header h;
  if (fread(&h, sizeof h, 1, f) != 1 || memcmp(h.magic, "CAPOWSOA", 8) != 0 || h.version != 1 || h.dtype > 1 ||
      h.ncols != 6) {
    fclose(f);
    if (msg) snprintf(msg, msglen, "%s: not a version-1 CAPOWSOA catalogue with 6 columns\n", path);
    return CAPOW_EINVAL;
  }
  const size_t eb = h.dtype ? 8 : 4, col = (size_t)h.n * eb;
  fseek(f, 0, SEEK_END);
  const long sz = ftell(f);
  if (sz < 0 || (unsigned long long)sz < sizeof h + 6ULL * col) {
    fclose(f);
    if (msg) snprintf(msg, msglen, "%s: truncated (%llu particles declared)\n", path, (unsigned long long)h.n);
    return CAPOW_EINVAL;
  }
  char *base = NULL;
  const size_t bytes = 4 * (col ? col : 1);
  if (posix_memalign((void **)&base, 4096, bytes) != 0) {
    fclose(f);
    return CAPOW_ENOMEM;
  }
  if (cudaHostRegister(base, bytes, cudaHostRegisterDefault) != cudaSuccess) (void)cudaGetLastError(); /* pageable */
  const int vcol = los == 1 ? 3 : (los == 2 ? 4 : 5); /* src/read_data.c:65-76 */
  const int cols[4] = {0, 1, 2, vcol};
  for (int k = 0; k < 4; k++) {
    if (fseek(f, (long)(sizeof h + (size_t)cols[k] * col), SEEK_SET) != 0 ||
        (col && fread(base + (size_t)k * col, 1, col, f) != col)) {
      fclose(f);
      capow_free_host(base);
      if (msg) snprintf(msg, msglen, "%s: read error\n", path);
      return CAPOW_EINVAL;
    }
  }
  fclose(f);
  *n_out = (size_t)h.n;
  *dtype = h.dtype ? CAPOW_F64 : CAPOW_F32;
  *x = base;
  *y = base + col;
  *z = base + 2 * col;
  *vlos = base + 3 * col;
  return CAPOW_OK;
}

void capow_free_host(void *p) {
  if (!p) return;
  if (cudaHostUnregister(p) != cudaSuccess) (void)cudaGetLastError();
  free(p);
}
