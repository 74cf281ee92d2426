/* CPU oracle: plain-C restatement of the CAPOW periodic path (test infrastructure only;
 * see capow_oracle.h). Single rank: ThisTask == 0 == NTask-1, Local_x_start = 0,
 * Local_nx = NX, Local_nxtra = NX + InterpOrder (src/main.c:1131-1135). */
#include "capow_oracle.h"
#include "orc_fft.h"
#include "shims/gsl/gsl_integration.h"
#include "shims/gsl/gsl_spline.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  double dx, dy, dz;     /* src/main.c:1126-1128 */
  double xmin_l, xmax_l; /* XMIN_LOCAL, XMAX_LOCAL: src/read_data.c:38-39 */
  int nxtra;             /* Local_nxtra: src/main.c:1134 */
  unsigned long long row; /* 2*(NZ/2+1) */
} geom;

static geom mk_geom(const orc_params *p) {
  geom g;
  g.dx = (p->xmax - p->xmin) / (double)p->nx;
  g.dy = (p->ymax - p->ymin) / (double)p->ny;
  g.dz = (p->zmax - p->zmin) / (double)p->nz;
  g.xmin_l = (double)0 * g.dx + p->xmin;
  g.xmax_l = (double)(0 + p->nx) * g.dx + p->xmin;
  g.nxtra = p->nx + p->interp_order;
  g.row = 2ULL * ((unsigned long long)p->nz / 2 + 1);
  return g;
}

int64_t orc_slice_doubles(const orc_params *p) { return 2LL * p->ny * (p->nz / 2 + 1); }

int64_t orc_grid_doubles(const orc_params *p) {
  /* Total_size = 2*alloc_local + InterpOrder*alloc_slice, alloc_local = NX*NY*(NZ/2+1) */
  return (int64_t)(p->nx + p->interp_order) * orc_slice_doubles(p);
}

/* One axis of the assignment stencil: up to three taps (index, weight, written?).
 * Written in the order the reference issues its writes: centre, low, high
 * (TSC, src/read_data.c:690-742) or centre, neighbour (CIC, :592-605). */
typedef struct {
  int idx[3];
  double wt[3];
  int on[3];
} taps;

/* CIC along one axis, src/read_data.c:554-576 (periodic branch).
 * is_x: the x axis uses the slab-local clamp at nx (:572); y/z wrap to 0 only for LOS==0 (:573-576)
 * and their neighbour is written only when < N (:594, :597, :602). */
static void cic_axis(double scale, int is_x, int n, int nxtra, int los, taps *t) {
  int i = (int)scale;
  double d = scale - (double)i;
  int nb = i + 1;
  if (is_x) {
    if (nb == nxtra) nb = nxtra - 1;
  } else if (los == 0) {
    if (nb == n) nb = 0;
  }
  t->idx[0] = i;
  t->wt[0] = 1.0 - d;
  t->on[0] = 1;
  t->idx[1] = nb;
  t->wt[1] = d;
  t->on[1] = is_x ? 1 : (nb < n);
  t->on[2] = 0;
}

/* TSC along one axis, src/read_data.c:629-671 (periodic branch) and the write guards of
 * :690-742: centre written if < N (y, z; always for x), low if index > 0, high if < N (nx for x). */
static void tsc_axis(double scale, int is_x, int n, int nxtra, int los, taps *t) {
  int i = (int)(scale + 0.5);
  double d = scale - (double)i;
  double wc = 0.75 - d * d;
  double wl = 0.5 * (0.5 - d) * (0.5 - d);
  double wh = 0.5 * (0.5 + d) * (0.5 + d);
  int lo = i - 1, hi = i + 1;
  if (is_x) {
    if (hi == nxtra) hi = nxtra - 1;
  } else if (los == 0) {
    if (lo < 0) lo = n - 1;
    if (hi >= n) {
      hi -= n;
      if (i >= n) i = 0;
      if (hi > 1) hi = 1;
    }
  }
  int lim = is_x ? nxtra : n;
  t->idx[0] = i;  t->wt[0] = wc; t->on[0] = is_x ? 1 : (i < n);
  t->idx[1] = lo; t->wt[1] = wl; t->on[1] = (lo > 0);
  t->idx[2] = hi; t->wt[2] = wh; t->on[2] = (hi < lim);
}

static inline void put(const orc_params *p, const geom *g, double *density, int ix, int iy, int iz, double v) {
  unsigned long long ind =
      (unsigned long long)iz + g->row * ((unsigned long long)iy + (unsigned long long)p->ny * (unsigned long long)ix);
  density[ind] += v;
}

double orc_add_to_grid(const orc_params *p, double x, double y, double z, double w, double vr, double *density) {
  const geom g = mk_geom(p);
  const double xmin = g.xmin_l, xmax = g.xmax_l;
  const double wvr = w * vr; /* src/read_data.c:516 */

  if (p->interp_order == 1) { /* nearest neighbour, src/read_data.c:519-541 */
    if ((x < xmin) || (x >= xmax)) return 0.0;
    if ((y < p->ymin) || (y >= p->ymax)) return 0.0;
    if ((z < p->zmin) || (z >= p->zmax)) return 0.0;
    int ix = (int)((x - xmin) / g.dx);
    int iy = (int)((y - p->ymin) / g.dy);
    int iz = (int)((z - p->zmin) / g.dz);
    if (ix == g.nxtra) ix = g.nxtra - 1;
    if (iy == p->ny) iy = p->ny - 1;
    if (iz == p->nz) iz = p->nz - 1;
    put(p, &g, density, ix, iy, iz, wvr);
    return w;
  }

  taps tx, ty, tz;
  if (p->interp_order == 2) { /* CIC, src/read_data.c:544-605 */
    if ((x < xmin) || (x >= xmax)) return 0.0;
    if ((y < p->ymin) || (y >= p->ymax)) return 0.0;
    if ((z < p->zmin) || (z >= p->zmax)) return 0.0;
    cic_axis((x - xmin) / g.dx, 1, p->nx, g.nxtra, p->los, &tx);
    cic_axis((y - p->ymin) / g.dy, 0, p->ny, g.nxtra, p->los, &ty);
    cic_axis((z - p->zmin) / g.dz, 0, p->nz, g.nxtra, p->los, &tz);
    /* write order of src/read_data.c:592-605: (y,z) = (c,c) (n,c) (n,n) (c,n), x = c then n */
    static const int yz[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
    for (int q = 0; q < 4; q++) {
      int a = yz[q][0], b = yz[q][1];
      if (!ty.on[a] || !tz.on[b]) continue;
      for (int c = 0; c < 2; c++)
        put(p, &g, density, tx.idx[c], ty.idx[a], tz.idx[b], wvr * tx.wt[c] * ty.wt[a] * tz.wt[b]);
    }
    return w;
  }

  /* TSC, src/read_data.c:608-743 */
  if (p->los == 0) {
    if (x - p->xmin < g.dx) x += p->xmax - p->xmin; /* :610-611 */
    if ((x < xmin + g.dx) || (x >= xmax + g.dx)) return 0.0; /* :612-613 */
  } else {
    if ((x < xmin) || (x >= xmax + g.dx)) return 0.0; /* :618-619 (rank 0) */
  }
  if ((y < p->ymin) || (y >= p->ymax)) return 0.0;
  if ((z < p->zmin) || (z >= p->zmax)) return 0.0;
  tsc_axis((x - xmin) / g.dx, 1, p->nx, g.nxtra, p->los, &tx);
  tsc_axis((y - p->ymin) / g.dy, 0, p->ny, g.nxtra, p->los, &ty);
  tsc_axis((z - p->zmin) / g.dz, 0, p->nz, g.nxtra, p->los, &tz);
  /* write order of src/read_data.c:690-742: (y,z) = (c,c) (l,c) (l,l) (l,h) (h,c) (h,l) (h,h) (c,l) (c,h),
   * x = c, l, h within each */
  static const int yz[9][2] = {{0, 0}, {1, 0}, {1, 1}, {1, 2}, {2, 0}, {2, 1}, {2, 2}, {0, 1}, {0, 2}};
  for (int q = 0; q < 9; q++) {
    int a = yz[q][0], b = yz[q][1];
    if (!ty.on[a] || !tz.on[b]) continue;
    for (int c = 0; c < 3; c++) {
      if (!tx.on[c]) continue;
      put(p, &g, density, tx.idx[c], ty.idx[a], tz.idx[b], wvr * tx.wt[c] * ty.wt[a] * tz.wt[b]);
    }
  }
  return w;
}

/* src/read_data.c:152-175 on one rank: the InterpOrder halo slices [NX, NX+InterpOrder)
 * are added onto slices [0, InterpOrder) when the box wraps (LOS==0, src/main.c:1153-1160,
 * 1173-1180); otherwise the neighbour is MPI_PROC_NULL and nothing is added. */
static void fold_halo(const orc_params *p, double *grid) {
  if (!grid || p->los != 0) return;
  int64_t slice = orc_slice_doubles(p);
  int64_t n = (int64_t)p->interp_order * slice;
  double *src = grid + (int64_t)p->nx * slice;
  double *tmp = (double *)malloc(sizeof(double) * (size_t)n);
  memcpy(tmp, src, sizeof(double) * (size_t)n);
  for (int64_t i = 0; i < n; i++) grid[i] += tmp[i];
  free(tmp);
}

static int has_mom_grid(int momentum) { return (momentum != 0) && (momentum != 2) && (momentum != 5); }

int orc_paint(const orc_params *p, int momentum, int64_t n, const double *x, const double *y, const double *z,
              const double *vx, const double *vy, const double *vz, const double *w, double *ddg,
              double *ddg_interlace, double *ddg_mom, double *ddg_mom_interlace, orc_stats *st) {
  const geom g = mk_geom(p);
  memset(st, 0, sizeof *st);
  /* RSD displacement factor, src/read_data.c:69, 72, 75 */
  const double opz = 1.0 + p->redshift;
  const double den = 100.0 * sqrt(p->omega_m * pow(opz, 3.0) + 1.0 - p->omega_m);
  const double hx = g.dx / 2.0, hy = g.dy / 2.0, hz = g.dz / 2.0;
  const int il = p->do_interlacing;
  for (int64_t i = 0; i < n; i++) {
    double wi = w ? w[i] : 1.0;
    double tx = x[i], ty = y[i], tz = z[i], tvr;
    if (p->los == 0) {
      tvr = vz[i];
    } else if (p->los == 1) {
      tvr = vx[i];
      tx += tvr * (1.0 + p->redshift) / den;
    } else if (p->los == 2) {
      tvr = vy[i];
      ty += tvr * (1.0 + p->redshift) / den;
    } else {
      tvr = vz[i];
      tz += tvr * (1.0 + p->redshift) / den;
    }
    st->nread += 1;
    if ((tx < p->xmin) || (tx > p->xmax) || (ty < p->ymin) || (ty > p->ymax) || (tz < p->zmin) ||
        (tz > p->zmax)) {
      if (p->los == 0) {
        st->fatal = 1;
        return -1;
      }
      st->nout += 1;
    }
    /* Momentum dispatch, src/read_data.c:91-130: value painted into ddg / ddg_mom */
    const double v1 = tvr, v2 = tvr * tvr, v3 = tvr * tvr * tvr, v4 = tvr * tvr * tvr * tvr;
    double vd, vm;
    switch (momentum) {
      case 0: vd = 1.0; vm = 0.0; break;
      case 1: vd = 1.0; vm = v1; break;
      case 2: vd = v1; vm = 0.0; break;
      case 3: vd = 1.0; vm = v2; break;
      case 4: vd = v1; vm = v2; break;
      case 5: vd = v2; vm = 0.0; break;
      case 6: vd = 1.0; vm = v3; break;
      case 7: vd = v1; vm = v3; break;
      default: vd = 1.0; vm = v4; break;
    }
    st->ngrid += orc_add_to_grid(p, tx, ty, tz, wi, vd, ddg);
    if (il) orc_add_to_grid(p, tx + hx, ty + hy, tz + hz, wi, vd, ddg_interlace);
    if (has_mom_grid(momentum)) {
      st->npv += orc_add_to_grid(p, tx, ty, tz, wi, vm, ddg_mom);
      if (il) orc_add_to_grid(p, tx + hx, ty + hy, tz + hz, wi, vm, ddg_mom_interlace);
    }
    if (momentum) { /* src/read_data.c:132-138 */
      st->nsq += wi;
      st->vr_ave += wi * tvr;
      st->vr2_ave += wi * tvr * tvr;
      st->vr3_ave += wi * tvr * tvr * tvr;
      st->vr4_ave += wi * tvr * tvr * tvr * tvr;
    }
  }
  fold_halo(p, ddg);
  if (il) fold_halo(p, ddg_interlace);
  if (has_mom_grid(momentum)) {
    fold_halo(p, ddg_mom);
    if (il) fold_halo(p, ddg_mom_interlace);
  }
  return 0;
}

void orc_shot_norm(const orc_params *p, int momentum, const orc_stats *st, double *alpha, double *shot,
                   double *norm) {
  const double N = st->ngrid; /* NPERIODIC_TOT, src/main.c:108 */
  *alpha = N / ((double)p->nx * (double)p->ny * (double)p->nz);
  const double nbar = N / ((p->xmax - p->xmin) * (p->ymax - p->ymin) * (p->zmax - p->zmin));
  *shot = N;
  *norm = nbar * N;
  double vr = 0, vr2 = 0, vr3 = 0, vr4 = 0;
  if (momentum) { /* src/main.c:121-127, NTask = 1 */
    double nsq = st->nsq / 1.0;
    vr = st->vr_ave / (nsq * 1.0);
    vr2 = st->vr2_ave / (nsq * 1.0);
    vr3 = st->vr3_ave / (nsq * 1.0);
    vr4 = st->vr4_ave / (nsq * 1.0);
  }
  switch (momentum) { /* src/main.c:141-148 */
    case 1: *shot = vr * N; break;
    case 2: *shot = vr2 * N; break;
    case 3: *shot = vr2 * N; break;
    case 4: *shot = vr3 * N; break;
    case 5: *shot = vr4 * N; break;
    case 6: *shot = vr3 * N; break;
    case 7: *shot = vr4 * N; break;
    case 8: *shot = vr4 * N; break;
    default: break;
  }
}

void orc_subtract_mean(const orc_params *p, int momentum, double alpha, double *ddg, double *ddg_interlace) {
  if (!((momentum == 0) | (momentum == 1) | (momentum == 3) | (momentum == 6) | (momentum == 8))) return;
  const unsigned long long row = 2ULL * ((unsigned long long)p->nz / 2 + 1);
  for (int i = 0; i < p->nx; i++)
    for (int j = 0; j < p->ny; j++)
      for (int k = 0; k < p->nz; k++) {
        unsigned long long ind = (unsigned long long)k + row * ((unsigned long long)j + (unsigned long long)p->ny * i);
        ddg[ind] -= alpha;
        if (p->do_interlacing) ddg_interlace[ind] -= alpha;
      }
}

void orc_fft_grids(const orc_params *p, int momentum, double *ddg, double *ddg_interlace, double *ddg_mom,
                   double *ddg_mom_interlace) {
  orc_fft_r2c_3d_inplace(p->nx, p->ny, p->nz, ddg);
  if (p->do_interlacing) orc_fft_r2c_3d_inplace(p->nx, p->ny, p->nz, ddg_interlace);
  if (has_mom_grid(momentum)) {
    orc_fft_r2c_3d_inplace(p->nx, p->ny, p->nz, ddg_mom);
    if (p->do_interlacing) orc_fft_r2c_3d_inplace(p->nx, p->ny, p->nz, ddg_mom_interlace);
  }
}

/* (int) of a double as the x86-64 and AArch64 builds behave for the values that reach it:
 * out-of-range or NaN give a negative (x86: INT_MIN) or >= NK (AArch64: INT_MAX) bin, both
 * rejected by src/main.c:375; -1 reproduces that rejection portably. */
static int to_bin(double v) {
  if (!(v > -2147483649.0 && v < 2147483648.0)) return -1;
  return (int)v;
}

int orc_kbin(const orc_params *p, double fktot) {
  const double binwidth = (p->maxk - p->mink) / (double)p->nk; /* src/main.c:305 */
  if (p->output_log) return to_bin((float)(log10(fktot) - p->mink) / binwidth); /* :370 */
  return to_bin((float)(fktot - p->mink) / binwidth);                          /* :372 */
}

void orc_compute_power(const orc_params *p, int momentum, const double *ddg, const double *ddg_interlace,
                       const double *ddg_mom, const double *ddg_mom_interlace, double *pk0, double *pk1,
                       double *pk2, double *pk3, double *pk4, int *nmodes, double *pk2d, int *nmodes2d) {
  const geom g = mk_geom(p);
  const int NK = p->nk, NMU = p->nmu;
  memset(pk0, 0, sizeof(double) * NK);
  memset(pk2, 0, sizeof(double) * NK);
  memset(pk4, 0, sizeof(double) * NK);
  if (p->odd_multipoles) {
    memset(pk1, 0, sizeof(double) * NK);
    memset(pk3, 0, sizeof(double) * NK);
  }
  memset(nmodes, 0, sizeof(int) * NK);
  if (p->output_2d) {
    memset(pk2d, 0, sizeof(double) * NK * NMU);
    memset(nmodes2d, 0, sizeof(int) * NK * NMU);
  }
  /* Nyquist, src/main.c:320-325 */
  const double ny_x = M_PI / g.dx, ny_y = M_PI / g.dy, ny_z = M_PI / g.dz;
  double min_nyquist = ny_x;
  if (ny_y < min_nyquist) min_nyquist = ny_y;
  if (ny_z < min_nyquist) min_nyquist = ny_z;
  const unsigned long long NX = p->nx, NY = p->ny, NZ = p->nz;
  const double sx = 1.0 / ((float)NX * g.dx), sy = 1.0 / ((float)NY * g.dy), sz = 1.0 / ((float)NZ * g.dz);
  const int mom = (momentum == 1) | (momentum == 3) | (momentum == 4) | (momentum >= 6);
  const unsigned long long row = 2ULL * (NZ / 2 + 1);
  for (int i = 0; i < p->nx; i++) {
    for (int j = 0; j < p->ny; j++) {
      for (int k = 0; (unsigned long long)k <= NZ / 2; k++) {
        /* frequencies, src/main.c:335-352 */
        double fx = ((unsigned long long)i <= NX / 2) ? (float)i * sx : ((float)i - (float)NX) * sx;
        double fy = ((unsigned long long)j <= NY / 2) ? (float)j * sy : ((float)j - (float)NY) * sy;
        double fz = (float)k * sz;
        double fktot = 2.0 * M_PI * sqrt(fx * fx + fy * fy + fz * fz); /* :355 */
        double mu;
        if (fktot > 0) { /* :357-367 */
          if (p->los == 1) mu = 2.0 * M_PI * fx / fktot;
          else if (p->los == 2) mu = 2.0 * M_PI * fy / fktot;
          else mu = 2.0 * M_PI * fz / fktot;
        } else {
          mu = 0.0;
        }
        int kbin = orc_kbin(p, fktot);
        if (!((kbin >= 0) && (kbin < NK) && (fktot <= min_nyquist))) continue; /* :375 */
        /* deconvolution, :382-389 */
        double sinc_x = 1.0, sinc_y = 1.0, sinc_z = 1.0;
        double ax = M_PI * fx * g.dx, ay = M_PI * fy * g.dy, az = M_PI * fz * g.dz;
        if (fx != 0.0) sinc_x = sin(ax) / ax;
        if (fy != 0.0) sinc_y = sin(ay) / ay;
        if (fz != 0.0) sinc_z = sin(az) / az;
        double grid_cor = pow(1.0 / (sinc_x * sinc_y * sinc_z), 2 * p->interp_order);
        unsigned long long base = row * ((unsigned long long)j + NY * (unsigned long long)i);
        double dkr = ddg[2 * k + base], dki = ddg[2 * k + 1 + base];
        if (p->do_interlacing) { /* :394-403 */
          grid_cor *= 0.25;
          double kh = ax + ay + az, sink = sin(kh), cosk = cos(kh);
          double a = ddg_interlace[2 * k + base], b = ddg_interlace[2 * k + 1 + base];
          dkr += a * cosk - b * sink;
          dki += a * sink + b * cosk;
        }
        double dkr_mom = 0.0, dki_mom = 0.0;
        if (mom) { /* :406-418 */
          dkr_mom = ddg_mom[2 * k + base];
          dki_mom = ddg_mom[2 * k + 1 + base];
          if (p->do_interlacing) {
            double kh = ax + ay + az, sink = sin(kh), cosk = cos(kh);
            double a = ddg_mom_interlace[2 * k + base], b = ddg_mom_interlace[2 * k + 1 + base];
            dkr_mom += a * cosk - b * sink;
            dki_mom += a * sink + b * cosk;
          }
        }
        /* Hermitian weight, :422-429 */
        int NM = 2;
        if (k == 0) {
          if (j == 0) {
            if ((i != 0) && ((unsigned long long)i != NX / 2)) NM = 1;
          } else {
            if ((unsigned long long)i != NX / 2) NM = 1;
          }
        }
        double power; /* :432-441 */
        double L2 = 1.5 * mu * mu - 0.5;
        double L4 = 4.375 * mu * mu * mu * mu - 3.75 * mu * mu + 0.375;
        if ((momentum == 0) | (momentum == 2) | (momentum == 5)) power = (dkr * dkr + dki * dki) * grid_cor;
        else if ((momentum == 1) | (momentum == 4) | (momentum == 6)) power = (dkr * dki_mom - dki * dkr_mom) * grid_cor;
        else power = (dkr * dkr_mom + dki * dki_mom) * grid_cor;
        pk0[kbin] += NM * power;
        pk2[kbin] += NM * L2 * power;
        pk4[kbin] += NM * L4 * power;
        if (p->odd_multipoles) { /* :445-449 */
          double L3 = 2.5 * mu * mu * mu - 1.5 * mu;
          pk1[kbin] += NM * mu * power;
          pk3[kbin] += NM * L3 * power;
        }
        nmodes[kbin] += NM;
        if (p->output_2d) { /* :453-461 */
          int mubin = (int)(((mu + 1.0) / 2.0) * (float)NMU);
          if (mubin >= NMU) mubin = NMU - 1;
          int bin = kbin * NMU + mubin;
          if ((bin >= 0) && (bin < NK * NMU)) {
            pk2d[bin] += NM * power;
            nmodes2d[bin] += NM;
          }
        }
      }
    }
  }
}

int orc_normalise(const orc_params *p, double shot, double norm, double *pk0, double *pk1, double *pk2,
                  double *pk3, double *pk4, int *nmodes, double *pk2d, const int *nmodes2d) {
  const int NK = p->nk;
  int *fill = (int *)calloc((size_t)NK, sizeof(int));
  for (int i = 0; i < NK; i++) { /* src/main.c:1021-1033 */
    if (nmodes[i] > 0.0 && fill[i] == 0) {
      pk0[i] -= nmodes[i] * shot;
      pk0[i] /= nmodes[i] * norm;
      pk2[i] *= 5.0 / (nmodes[i] * norm);
      pk4[i] *= 9.0 / (nmodes[i] * norm);
      if (p->odd_multipoles) {
        pk1[i] *= 3.0 / (nmodes[i] * norm);
        pk3[i] *= 7.0 / (nmodes[i] * norm);
      }
      fill[i] = 1;
    }
  }
  if (p->output_2d) /* :1034-1040 */
    for (int i = 0; i < NK * p->nmu; i++)
      if (nmodes2d[i] > 0.0) pk2d[i] /= nmodes2d[i] * norm;
  int last = -1;
  for (int i = NK - 1; i >= 0; i--) { /* :1043-1056 */
    if (fill[i] == 1) {
      if (p->odd_multipoles) {
        pk1[i] = 0.0;
        pk3[i] = 0.0;
      }
      pk0[i] = 0.0;
      pk2[i] = 0.0;
      pk4[i] = 0.0;
      nmodes[i] = 0;
      last = i;
      break;
    }
  }
  free(fill);
  return last;
}

/* ------------------------------------------------------------------ survey mode */
/* add_to_grid with the Survey branches (src/read_data.c:514-745; single rank: the TSC acceptance of
 * :617-619, the clamps of :577-590 (CIC) and :672-688 (TSC)): a neighbour index reaching the axis
 * limit (Local_nxtra for x, NY, NZ) is pulled back with the centre, the weights staying those of the
 * unclamped position. */
static void cic_axis_s(double scale, int lim, taps *t) {
  int i = (int)scale;
  double d = scale - (double)i;
  int nb = i + 1;
  if (nb == lim) {
    nb = lim - 1;
    i = lim - 2;
  }
  t->idx[0] = i;  t->wt[0] = 1.0 - d; t->on[0] = 1;
  t->idx[1] = nb; t->wt[1] = d;       t->on[1] = 1;
  t->on[2] = 0;
}

static void tsc_axis_s(double scale, int is_x, int n, int lim, taps *t) {
  int i = (int)(scale + 0.5);
  double d = scale - (double)i;
  double wc = 0.75 - d * d;
  double wl = 0.5 * (0.5 - d) * (0.5 - d);
  double wh = 0.5 * (0.5 + d) * (0.5 + d);
  int lo = i - 1, hi = i + 1;
  if (hi == lim) {
    hi = lim - 1;
    i = lim - 2;
    lo = lim - 3;
  }
  t->idx[0] = i;  t->wt[0] = wc; t->on[0] = is_x ? 1 : (i < n);
  t->idx[1] = lo; t->wt[1] = wl; t->on[1] = (lo > 0);
  t->idx[2] = hi; t->wt[2] = wh; t->on[2] = (hi < lim);
}

double orc_survey_add(const orc_params *p, double x, double y, double z, double w, double vr, double *density) {
  const geom g = mk_geom(p);
  const double xmin = g.xmin_l, xmax = g.xmax_l;
  const double wvr = w * vr;
  if (p->interp_order == 1) return orc_add_to_grid(p, x, y, z, w, vr, density); /* NN has no survey branch */
  taps tx, ty, tz;
  if (p->interp_order == 2) {
    if ((x < xmin) || (x >= xmax)) return 0.0;
    if ((y < p->ymin) || (y >= p->ymax)) return 0.0;
    if ((z < p->zmin) || (z >= p->zmax)) return 0.0;
    cic_axis_s((x - xmin) / g.dx, g.nxtra, &tx);
    cic_axis_s((y - p->ymin) / g.dy, p->ny, &ty);
    cic_axis_s((z - p->zmin) / g.dz, p->nz, &tz);
    ty.on[1] = ty.idx[1] < p->ny;
    tz.on[1] = tz.idx[1] < p->nz;
    static const int yz[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
    for (int q = 0; q < 4; q++) {
      int a = yz[q][0], b = yz[q][1];
      if (!ty.on[a] || !tz.on[b]) continue;
      for (int c = 0; c < 2; c++)
        put(p, &g, density, tx.idx[c], ty.idx[a], tz.idx[b], wvr * tx.wt[c] * ty.wt[a] * tz.wt[b]);
    }
    return w;
  }
  if ((x < xmin) || (x >= xmax + g.dx)) return 0.0; /* :617-619, rank 0 */
  if ((y < p->ymin) || (y >= p->ymax)) return 0.0;
  if ((z < p->zmin) || (z >= p->zmax)) return 0.0;
  tsc_axis_s((x - xmin) / g.dx, 1, p->nx, g.nxtra, &tx);
  tsc_axis_s((y - p->ymin) / g.dy, 0, p->ny, p->ny, &ty);
  tsc_axis_s((z - p->zmin) / g.dz, 0, p->nz, p->nz, &tz);
  static const int yz[9][2] = {{0, 0}, {1, 0}, {1, 1}, {1, 2}, {2, 0}, {2, 1}, {2, 2}, {0, 1}, {0, 2}};
  for (int q = 0; q < 9; q++) {
    int a = yz[q][0], b = yz[q][1];
    if (!ty.on[a] || !tz.on[b]) continue;
    for (int c = 0; c < 3; c++) {
      if (!tx.on[c]) continue;
      put(p, &g, density, tx.idx[c], ty.idx[a], tz.idx[b], wvr * tx.wt[c] * ty.wt[a] * tz.wt[b]);
    }
  }
  return w;
}

/* assign_survey_data for the density (src/read_data.c:471-494, Momentum 0): each object, and its
 * copy shifted by half a cell into the interlaced grid, with weight prefactor * w. Returns
 * sum(add_to_grid / w) (the reference's NGRID of the call). */
double orc_survey_assign(const orc_params *p, int momentum, int is_data, int64_t n, const double *x, const double *y,
                         const double *z, const double *w, const double *wpv, const double *pv, double prefactor,
                         double *ddg, double *ddg_i, double *ddg_m, double *ddg_mi) {
  const geom g = mk_geom(p);
  double ngrid = 0.0;
  for (int64_t i = 0; i < n; i++) {
    const double xi = x[i] + g.dx / 2.0, yi = y[i] + g.dy / 2.0, zi = z[i] + g.dz / 2.0;
    if (momentum == 1) { /* :476-478: the divisor pv * weight is a float product */
      const float pw = (float)pv[i] * (float)w[i];
      ngrid += orc_survey_add(p, x[i], y[i], z[i], w[i], prefactor * pv[i], ddg) / (double)pw;
      if (p->do_interlacing) orc_survey_add(p, xi, yi, zi, w[i], prefactor * pv[i], ddg_i);
    } else { /* :479-486 */
      ngrid += orc_survey_add(p, x[i], y[i], z[i], prefactor * w[i], 1.0, ddg) / w[i];
      if (p->do_interlacing) orc_survey_add(p, xi, yi, zi, prefactor * w[i], 1.0, ddg_i);
      if (momentum && is_data) {
        orc_survey_add(p, x[i], y[i], z[i], wpv[i], prefactor * pv[i], ddg_m);
        if (p->do_interlacing) orc_survey_add(p, xi, yi, zi, wpv[i], prefactor * pv[i], ddg_mi);
      }
    }
  }
  return ngrid;
}

/* The unit-vector products of compute_survey_power (src/main.c:472-775) for each multipole: index
 * triples in the reference's loop order, and the power of r^ they multiply the grid by. */
static int survey_terms(int l, int t[15][3]) {
  int n = 0;
  if (l == 0) { t[0][0] = t[0][1] = t[0][2] = 0; return 1; }
  if (l == 1) { for (int i = 0; i < 3; i++) { t[n][0] = i; t[n][1] = t[n][2] = 0; n++; } return n; }
  if (l == 2) {
    for (int i = 0; i < 3; i++) for (int j = i; j < 3; j++) { t[n][0] = i; t[n][1] = j; t[n][2] = 0; n++; }
    return n;
  }
  if (l == 3) { /* :648-655 */
    for (int i = 0; i < 3; i++) {
      int jl = i, jh = i + 1;
      if (i == 0) jh = i + 2;
      for (int j = jl; j < jh; j++) {
        int kl = 0, kh = 3;
        if (j != i) kl = 2;
        for (int k = kl; k < kh; k++) { t[n][0] = i; t[n][1] = j; t[n][2] = k; n++; }
      }
    }
    return n;
  }
  for (int i = 0; i < 3; i++) /* l == 4, :709-727 */
    for (int j = 0; j < 3; j++) {
      int kl = 0, kh = 3;
      if (j != i) {
        if (i == 1) kl = 2;
        else if (i == 2) {
          if (j == 1) continue;
          kl = 1;
          kh = 2;
        } else kl = j;
      }
      for (int k = kl; k < kh; k++) { t[n][0] = i; t[n][1] = j; t[n][2] = k; n++; }
    }
  return n;
}

/* The weighted grid of one term (src/main.c:506-511, 551-559, 604-612, 660-668, 731-742): the first NX
 * slices of src times the r^ products of the cell corner position relative to the origin. */
static void survey_weight(const orc_params *p, const orc_survey *sp, int l, const int *ijk, const double *src,
                          double *dst) {
  const geom g = mk_geom(p);
  for (int ix = 0; ix < p->nx; ix++)
    for (int iy = 0; iy < p->ny; iy++)
      for (int iz = 0; iz < p->nz; iz++) {
        long ind = iz + 2 * (p->nz / 2 + 1) * (iy + p->ny * ix);
        double vec[3] = {ix * g.dx + p->xmin - sp->x_origin, iy * g.dy + p->ymin - sp->y_origin,
                         iz * g.dz + p->zmin - sp->z_origin};
        double r2 = vec[0] * vec[0] + vec[1] * vec[1] + vec[2] * vec[2];
        if (r2 == 0.0) r2 = 1.0;
        double v = src[ind];
        if (l == 1) v = src[ind] * vec[ijk[0]] / sqrt(r2);
        else if (l == 2) v = src[ind] * vec[ijk[0]] * vec[ijk[1]] / r2;
        else if (l == 3) v = src[ind] * vec[ijk[0]] * vec[ijk[1]] * vec[ijk[2]] / (r2 * sqrt(r2));
        else if (l == 4) v = src[ind] * vec[ijk[0]] * vec[ijk[0]] * vec[ijk[1]] * vec[ijk[2]] / (r2 * r2);
        dst[ind] = v;
      }
}

/* assign_survey_power (src/main.c:781-967) over the transformed term grid d2 (and its interlaced copy);
 * multipole 0 stores the combined field in F0. With Momentum 2, 3 the momentum term grid m2 (m2i) is
 * combined too, multipole 0 stores it in F0m, and the power is the cross form of :876-887. */
static void survey_assign(const orc_params *p, int momentum, int l, const int *ijk, const double *d2,
                          const double *d2i, const double *m2, const double *m2i, double *F0, double *F0m,
                          double *pk[5], int *nmodes) {
  const int cross = (momentum != 0) && (momentum != 1);
  const geom g = mk_geom(p);
  const int NK = p->nk;
  const double ny_x = M_PI / g.dx, ny_y = M_PI / g.dy, ny_z = M_PI / g.dz;
  double min_nyquist = ny_x;
  if (ny_y < min_nyquist) min_nyquist = ny_y;
  if (ny_z < min_nyquist) min_nyquist = ny_z;
  const unsigned long long NX = p->nx, NY = p->ny, NZ = p->nz;
  const double sx = 1.0 / ((float)NX * g.dx), sy = 1.0 / ((float)NY * g.dy), sz = 1.0 / ((float)NZ * g.dz);
  const int ii = ijk[0], jj = ijk[1], kk = ijk[2];
  for (int i = 0; i < p->nx; i++)
    for (int j = 0; j < p->ny; j++)
      for (int k = 0; (unsigned long long)k <= NZ / 2; k++) {
        double fx = ((unsigned long long)i <= NX / 2) ? (float)i * sx : ((float)i - (float)NX) * sx;
        double fy = ((unsigned long long)j <= NY / 2) ? (float)j * sy : ((float)j - (float)NY) * sy;
        double fz = (float)k * sz;
        double fktot = 2.0 * M_PI * sqrt(fx * fx + fy * fy + fz * fz);
        int kbin = orc_kbin(p, fktot);
        if (!((kbin >= 0) && (kbin < NK) && (fktot <= min_nyquist))) continue;
        double sinc_x = 1.0, sinc_y = 1.0, sinc_z = 1.0;
        double ax = M_PI * fx * g.dx, ay = M_PI * fy * g.dy, az = M_PI * fz * g.dz;
        if (fx != 0.0) sinc_x = sin(ax) / ax;
        if (fy != 0.0) sinc_y = sin(ay) / ay;
        if (fz != 0.0) sinc_z = sin(az) / az;
        double grid_cor = pow(1.0 / (sinc_x * sinc_y * sinc_z), 2 * p->interp_order);
        double kvec[3] = {2. * M_PI * fx, 2. * M_PI * fy, 2. * M_PI * fz};
        long long ind = (2 * k) + 2 * (NZ / 2 + 1) * (j + NY * i);
        double dkr = d2[ind], dki = d2[ind + 1];
        if (p->do_interlacing) {
          grid_cor *= 0.25;
          double kh = ax + ay + az, sink = sin(kh), cosk = cos(kh);
          double a = d2i[ind], b = d2i[ind + 1];
          dkr += a * cosk - b * sink;
          dki += a * sink + b * cosk;
        }
        double mkr = 0.0, mki = 0.0;
        if (cross) { /* :859-869 */
          mkr = m2[ind];
          mki = m2[ind + 1];
          if (p->do_interlacing) {
            double kh = ax + ay + az, sink = sin(kh), cosk = cos(kh);
            double a = m2i[ind], b = m2i[ind + 1];
            mkr += a * cosk - b * sink;
            mki += a * sink + b * cosk;
          }
        }
        double power;
        if (!cross) {
          if (l == 0) {
            F0[ind] = dkr;
            F0[ind + 1] = dki;
            power = (dkr * dkr + dki * dki) * grid_cor;
          } else if (l % 2) {
            power = (dkr * F0[ind + 1] - dki * F0[ind]) * grid_cor;
          } else {
            power = (dkr * F0[ind] + dki * F0[ind + 1]) * grid_cor;
          }
        } else if (l == 0) {
          F0[ind] = dkr;
          F0[ind + 1] = dki;
          F0m[ind] = mkr;
          F0m[ind + 1] = mki;
          power = (dkr * mki - dki * mkr) * grid_cor;
        } else if (l % 2) {
          power = 0.5 * (dkr * F0m[ind] + dki * F0m[ind + 1] + mkr * F0[ind] + mki * F0[ind + 1]) * grid_cor;
        } else {
          power = 0.5 * (dkr * F0m[ind + 1] - dki * F0m[ind] + mkr * F0[ind + 1] - mki * F0[ind]) * grid_cor;
        }
        int NM = 2;
        if (k == 0) {
          if (j == 0) {
            if ((i != 0) && ((unsigned long long)i != NX / 2)) NM = 1;
          } else {
            if ((unsigned long long)i != NX / 2) NM = 1;
          }
        }
        power *= NM;
        if (l == 0) {
          pk[0][kbin] += power;
          pk[2][kbin] -= 0.5 * power;
          pk[4][kbin] += 0.375 * power;
          nmodes[kbin] += NM;
        } else if (l == 1) {
          if (fktot > 0.0) {
            power *= kvec[ii] / fktot;
            pk[1][kbin] += power;
            pk[3][kbin] -= 1.5 * power;
          }
        } else if (l == 2) {
          if (fktot > 0.0) {
            double kprefac = ii != jj ? 2.0 : 1.0;
            power *= kprefac * kvec[ii] * kvec[jj] / (fktot * fktot);
            pk[2][kbin] += 1.5 * power;
            pk[4][kbin] -= 3.75 * power;
          }
        } else if (l == 3) {
          if (fktot > 0.0) {
            double kprefac = 1.0;
            if (ii != kk) kprefac = (ii != jj) ? 6.0 : 3.0;
            pk[3][kbin] += 2.5 * kprefac * kvec[ii] * kvec[jj] * kvec[kk] / (fktot * fktot * fktot) * power;
          }
        } else {
          if (fktot > 0) {
            double kprefac = 1.0;
            if (ii == jj) {
              if (ii != kk) kprefac = 4.0;
            } else {
              kprefac = (jj == kk) ? 6.0 : 12.0;
            }
            pk[4][kbin] += 4.375 * kprefac * kvec[ii] * kvec[ii] * kvec[jj] * kvec[kk] /
                           (fktot * fktot * fktot * fktot) * power;
          }
        }
      }
}

void orc_survey_power(const orc_params *p, const orc_survey *sp, int momentum, const double *ddg,
                      const double *ddg_interlace, const double *ddg_m, const double *ddg_mi, double *pk0,
                      double *pk1, double *pk2, double *pk3, double *pk4, int *nmodes) {
  const int NK = p->nk;
  const int cross = (momentum != 0) && (momentum != 1);
  double *pk[5] = {pk0, pk1, pk2, pk3, pk4};
  double dummy[NK > 0 ? NK : 1];
  for (int l = 0; l < 5; l++) {
    if (!pk[l]) pk[l] = dummy;
    memset(pk[l], 0, sizeof(double) * NK);
  }
  memset(nmodes, 0, sizeof(int) * NK);
  const int64_t nd = orc_grid_doubles(p);
  double *d2 = (double *)calloc((size_t)nd, sizeof(double));
  double *d2i = p->do_interlacing ? (double *)calloc((size_t)nd, sizeof(double)) : NULL;
  double *F0 = (double *)calloc((size_t)nd, sizeof(double));
  double *m2 = cross ? (double *)calloc((size_t)nd, sizeof(double)) : NULL;
  double *m2i = cross && p->do_interlacing ? (double *)calloc((size_t)nd, sizeof(double)) : NULL;
  double *F0m = cross ? (double *)calloc((size_t)nd, sizeof(double)) : NULL;
  const int step = p->odd_multipoles ? 1 : 2; /* src/main.c:490-492 */
  for (int l = 0; l <= 4; l += step) {
    int t[15][3];
    const int nt = survey_terms(l, t);
    for (int q = 0; q < nt; q++) {
      survey_weight(p, sp, l, t[q], ddg, d2);
      orc_fft_r2c_3d_inplace(p->nx, p->ny, p->nz, d2);
      if (d2i) {
        survey_weight(p, sp, l, t[q], ddg_interlace, d2i);
        orc_fft_r2c_3d_inplace(p->nx, p->ny, p->nz, d2i);
      }
      if (cross) { /* the momentum grids get the same products (src/main.c:515-526, 560-573, ...) */
        survey_weight(p, sp, l, t[q], ddg_m, m2);
        orc_fft_r2c_3d_inplace(p->nx, p->ny, p->nz, m2);
        if (m2i) {
          survey_weight(p, sp, l, t[q], ddg_mi, m2i);
          orc_fft_r2c_3d_inplace(p->nx, p->ny, p->nz, m2i);
        }
      }
      survey_assign(p, momentum, l, t[q], d2, d2i, m2, m2i, F0, F0m, pk, nmodes);
    }
  }
  free(d2);
  free(d2i);
  free(F0);
  free(m2);
  free(m2i);
  free(F0m);
}

/* ---- the redshift-distance table of create_grids (src/main.c:1233-1248) */
static double orc_hubble_inv(double z, void *par) {
  const double om = *(const double *)par;
  return 1.0 / sqrt(om * (1.0 + z) * (1.0 + z) * (1.0 + z) + (1.0 - om)); /* src/read_data.c:376-379 */
}

static double g_table_om = -1.0;
static gsl_spline *g_red_spline = NULL, *g_dist_spline = NULL;

static void survey_table(double omega_m) {
  if (g_red_spline && g_table_om == omega_m) return;
  const int nbins = 10000;
  const double redmin = 0.0, redmax = 10.0, redbinwidth = (redmax - redmin) / (double)(nbins - 1);
  double *zt = (double *)malloc(nbins * sizeof(double)), *rt = (double *)malloc(nbins * sizeof(double));
  double om = omega_m;
  gsl_function F;
  F.function = &orc_hubble_inv;
  F.params = &om;
  zt[0] = 0.0;
  rt[0] = 0.0;
  for (int i = 1; i < nbins; i++) { /* comoving_distance, src/read_data.c:365-373 */
    double result, error;
    zt[i] = i * redbinwidth + redmin;
    gsl_integration_qags(&F, 0.0, zt[i], 0, 1e-7, 1000, NULL, &result, &error);
    rt[i] = 299792.458 * result / 100.0;
  }
  if (g_red_spline) gsl_spline_free(g_red_spline);
  if (g_dist_spline) gsl_spline_free(g_dist_spline);
  g_red_spline = gsl_spline_alloc(gsl_interp_cspline, nbins);
  g_dist_spline = gsl_spline_alloc(gsl_interp_cspline, nbins);
  gsl_spline_init(g_red_spline, rt, zt, nbins); /* src/main.c:1247 */
  gsl_spline_init(g_dist_spline, zt, rt, nbins);
  free(zt);
  free(rt);
  g_table_om = omega_m;
}

double orc_survey_redshift(double omega_m, double r) {
  survey_table(omega_m);
  return gsl_spline_eval(g_red_spline, r, NULL);
}

double orc_survey_distance(double omega_m, double z) {
  survey_table(omega_m);
  return gsl_spline_eval(g_dist_spline, z, NULL);
}

double orc_cspline_eval(int n, const double *x, const double *y, double t) {
  gsl_spline *s = gsl_spline_alloc(gsl_interp_cspline, (size_t)n);
  gsl_spline_init(s, x, y, (size_t)n);
  const double v = gsl_spline_eval(s, t, NULL);
  gsl_spline_free(s);
  return v;
}
