// Shared definitions for libcapow_gpu: geometry constants, the reference's mass-assignment
// tap rules in exact FP64 form (plain FP64 path and near-edge particles) and in FP32
// separable form (tiled FP32 path), error plumbing.
//
// Reference semantics reproduced here (single rank; paths relative to the CAPOW tree):
//   src/read_data.c:514-745  add_to_grid: NN / CIC / TSC acceptance, index and weight rules
//   src/read_data.c:152-175  halo fold: the InterpOrder slices past NX are added onto
//                            slices 0.. when LOS == 0, discarded otherwise
//   src/main.c:1126-1135     dx = (MAX-MIN)/N, padded row 2*(NZ/2+1), XMAX_LOCAL
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/capow.h"

#define CAPOW_HD __host__ __device__ __forceinline__

// Geometry and run constants, passed to kernels by value.
struct Geom {
  int nx, ny, nz;     // NX NY NZ
  int order;          // InterpOrder
  int los;            // LOS (4: survey grid, no RSD shift and no wrap)
  int survey;         // add_to_grid's Survey branches (src/read_data.c:577-590, 672-688) instead of Periodic
  int interlace;      // DoInterlacing
  int nxtra;          // Local_nxtra = NX + InterpOrder (src/main.c:1134)
  int nzc;            // NZ/2 + 1
  long long row;      // 2*(NZ/2+1): padded reals per (x,y) row
  long long slice;    // NY*row
  long long main_sz;  // NX*slice: the FFT region; halo slices start here
  double xmin, ymin, zmin;        // XMIN YMIN ZMIN (XMIN_LOCAL = XMIN on one rank)
  double xmax, ymax, zmax;        // XMAX YMAX ZMAX (box check, src/read_data.c:81)
  double xmax_l;                  // XMAX_LOCAL = NX*dx + XMIN (src/read_data.c:39)
  double lx;                      // XMAX - XMIN (TSC LOS==0 shift, src/read_data.c:611)
  double dx, dy, dz;              // src/main.c:1126-1128
  double hx, hy, hz;              // dx/2.0 ... (interlaced offset, src/read_data.c:93)
  double rsd_opz;                 // 1 + Redshift
  double rsd_den;                 // 100*sqrt(Omega_m*(1+z)^3 + 1 - Omega_m)
  // FP32 path
  float xmin_f, ymin_f, zmin_f;   // float of the box minima
  float idx_f, idy_f, idz_f;      // float(1/d)
  float rsd_f;                    // float((1+z)/den)
  float margin;                   // cells: distance to a discontinuity that sends a particle to FP64
};

// Field exponents: a painted field holds w*v^e (src/read_data.c:91-130).
struct FieldSpec {
  int nfields;   // 1 (field A only) or 2 (A and B)
  int ea, eb;    // exponents of v for field A and B
  int need_v;    // velocities are read (RSD shift, momentum field or moments)
  int moments;   // accumulate sum w v^n (src/read_data.c:132-138, only when Momentum != 0)
};

// ---------------------------------------------------------------------------------------------
// Exact FP64 taps (one stencil) following add_to_grid. Arithmetic uses explicit round-to-nearest
// intrinsics so no FMA contraction changes a rounding relative to the x86-64 reference build.
struct AxisTaps {
  int idx[3];
  double w[3];
  int on[3];
  int n;
};

// Correctly rounded double operations that the compiler may not fuse (device: intrinsics;
// host: plain operators, compiled with -ffp-contract=off).
CAPOW_HD double DADD(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
CAPOW_HD double DSUB(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
CAPOW_HD double DMUL(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
CAPOW_HD double DDIV(double a, double b) {
#ifdef __CUDA_ARCH__
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}

// CIC along one axis: src/read_data.c:554-576 (periodic); neighbour guarded by :594, :597, :602.
CAPOW_HD void cic_axis64(double scale, bool is_x, int n, int nxtra, int los, AxisTaps &t) {
  int i = (int)scale;
  double d = DSUB(scale, (double)i);
  int nb = i + 1;
  if (is_x) {
    if (nb == nxtra) nb = nxtra - 1;
  } else if (los == 0) {
    if (nb == n) nb = 0;
  }
  t.n = 2;
  t.idx[0] = i;  t.w[0] = DSUB(1.0, d); t.on[0] = 1;
  t.idx[1] = nb; t.w[1] = d;            t.on[1] = is_x ? 1 : (nb < n);
  t.on[2] = 0;
}

// TSC along one axis: src/read_data.c:629-671 and the write guards of :690-742.
CAPOW_HD void tsc_axis64(double scale, bool is_x, int n, int nxtra, int los, AxisTaps &t) {
  int i = (int)DADD(scale, 0.5);
  double d = DSUB(scale, (double)i);
  double wc = DSUB(0.75, DMUL(d, d));
  double a = DSUB(0.5, d), b = DADD(0.5, d);
  double wl = DMUL(DMUL(0.5, a), a);
  double wh = DMUL(DMUL(0.5, b), b);
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
  t.n = 3;
  t.idx[0] = i;  t.w[0] = wc; t.on[0] = is_x ? 1 : (i < n);
  t.idx[1] = lo; t.w[1] = wl; t.on[1] = (lo > 0);
  t.idx[2] = hi; t.w[2] = wh; t.on[2] = (hi < lim);
}

// One axis of add_to_grid's Survey branch (single rank). CIC (src/read_data.c:554-590): ix = (int)scale,
// neighbour ix + 1; TSC (:629-688): ix = (int)(scale + 0.5), neighbours ix -/+ 1. When the upper
// neighbour equals lim (Local_nxtra along x, NY or NZ) the stencil moves down one cell, its weights
// unchanged. Write guards (:592-605, :690-742): CIC y/z neighbour < N; TSC centre y/z < N, low > 0,
// high < lim.
CAPOW_HD void survey_cic64(double scale, bool is_x, int n, int lim, AxisTaps &t) {
  int i = (int)scale;
  const double d = DSUB(scale, (double)i);
  int nb = i + 1;
  if (nb == lim) {
    nb = lim - 1;
    i = lim - 2;
  }
  t.n = 2;
  t.idx[0] = i;  t.w[0] = DSUB(1.0, d); t.on[0] = 1;
  t.idx[1] = nb; t.w[1] = d;            t.on[1] = is_x ? 1 : (nb < n);
  t.on[2] = 0;
}

CAPOW_HD void survey_tsc64(double scale, bool is_x, int n, int lim, AxisTaps &t) {
  int i = (int)DADD(scale, 0.5);
  const double d = DSUB(scale, (double)i);
  const double wc = DSUB(0.75, DMUL(d, d));
  const double a = DSUB(0.5, d), b = DADD(0.5, d);
  const double wl = DMUL(DMUL(0.5, a), a);
  const double wh = DMUL(DMUL(0.5, b), b);
  int lo = i - 1, hi = i + 1;
  if (hi == lim) {
    hi = lim - 1;
    i = lim - 2;
    lo = lim - 3;
  }
  t.n = 3;
  t.idx[0] = i;  t.w[0] = wc; t.on[0] = is_x ? 1 : (i < n);
  t.idx[1] = lo; t.w[1] = wl; t.on[1] = (lo > 0);
  t.idx[2] = hi; t.w[2] = wh; t.on[2] = (hi < lim);
}

// Acceptance of one Survey add_to_grid call along one axis a (0 x, 1 y, 2 z; rank 0 of one): x in
// [XMIN, XMAX) for NN and CIC, [XMIN, XMAX + dx) for TSC (:519-527, :546-552, :617-619); y, z in [MIN, MAX).
CAPOW_HD bool survey_accept_axis(const Geom &g, int a, double c) {
  const double mn = a == 0 ? g.xmin : (a == 1 ? g.ymin : g.zmin);
  double mx = a == 0 ? g.xmax_l : (a == 1 ? g.ymax : g.zmax);
  if (a == 0 && g.order == 3) mx = DADD(mx, g.dx);
  return !((c < mn) || (c >= mx));
}

// Taps of one axis for a Survey run (CIC and TSC; NN has no Survey branch: the periodic rule).
CAPOW_HD void survey_axis_taps(const Geom &g, int a, double c, AxisTaps &t) {
  const double mn = a == 0 ? g.xmin : (a == 1 ? g.ymin : g.zmin);
  const double d = a == 0 ? g.dx : (a == 1 ? g.dy : g.dz);
  const int n = a == 0 ? g.nx : (a == 1 ? g.ny : g.nz);
  const int lim = a == 0 ? g.nxtra : n;
  const double s = DDIV(DSUB(c, mn), d);
  if (g.order == 2) survey_cic64(s, a == 0, n, lim, t);
  else survey_tsc64(s, a == 0, n, lim, t);
}

// Acceptance and per-axis taps of one add_to_grid call. (x, y, z) are the coordinates the
// reader passes (already RSD-shifted, +d/2 for the interlaced copy). Returns false when the
// particle is rejected (add_to_grid returns 0.0).
CAPOW_HD bool exact_axes(const Geom &g, double x, double y, double z, AxisTaps &ax, AxisTaps &ay, AxisTaps &az) {
  if (g.survey && g.order > 1) {
    if (!survey_accept_axis(g, 0, x) || !survey_accept_axis(g, 1, y) || !survey_accept_axis(g, 2, z)) return false;
    survey_axis_taps(g, 0, x, ax);
    survey_axis_taps(g, 1, y, ay);
    survey_axis_taps(g, 2, z, az);
    return true;
  }
  const double xmin = g.xmin, xmax = g.xmax_l;
  if (g.order == 1) {  // src/read_data.c:519-541
    if ((x < xmin) || (x >= xmax)) return false;
    if ((y < g.ymin) || (y >= g.ymax)) return false;
    if ((z < g.zmin) || (z >= g.zmax)) return false;
    int ix = (int)DDIV(DSUB(x, xmin), g.dx);
    int iy = (int)DDIV(DSUB(y, g.ymin), g.dy);
    int iz = (int)DDIV(DSUB(z, g.zmin), g.dz);
    if (ix == g.nxtra) ix = g.nxtra - 1;
    if (iy == g.ny) iy = g.ny - 1;
    if (iz == g.nz) iz = g.nz - 1;
    ax.n = ay.n = az.n = 1;
    ax.idx[0] = ix; ay.idx[0] = iy; az.idx[0] = iz;
    ax.w[0] = ay.w[0] = az.w[0] = 1.0;
    ax.on[0] = ay.on[0] = az.on[0] = 1;
    return true;
  }
  if (g.order == 2) {  // src/read_data.c:544-605
    if ((x < xmin) || (x >= xmax)) return false;
    if ((y < g.ymin) || (y >= g.ymax)) return false;
    if ((z < g.zmin) || (z >= g.zmax)) return false;
    cic_axis64(DDIV(DSUB(x, xmin), g.dx), true, g.nx, g.nxtra, g.los, ax);
    cic_axis64(DDIV(DSUB(y, g.ymin), g.dy), false, g.ny, g.nxtra, g.los, ay);
    cic_axis64(DDIV(DSUB(z, g.zmin), g.dz), false, g.nz, g.nxtra, g.los, az);
    return true;
  }
  // TSC, src/read_data.c:608-743
  if (g.los == 0) {
    if (DSUB(x, g.xmin) < g.dx) x = DADD(x, g.lx);                           // :610-611
    if ((x < DADD(xmin, g.dx)) || (x >= DADD(xmax, g.dx))) return false;     // :612-613
  } else {
    if ((x < xmin) || (x >= DADD(xmax, g.dx))) return false;                 // :618-619 (rank 0)
  }
  if ((y < g.ymin) || (y >= g.ymax)) return false;
  if ((z < g.zmin) || (z >= g.zmax)) return false;
  tsc_axis64(DDIV(DSUB(x, xmin), g.dx), true, g.nx, g.nxtra, g.los, ax);
  tsc_axis64(DDIV(DSUB(y, g.ymin), g.dy), false, g.ny, g.nxtra, g.los, ay);
  tsc_axis64(DDIV(DSUB(z, g.zmin), g.dz), false, g.nz, g.nxtra, g.los, az);
  return true;
}

// One axis of exact_axes (0 x, 1 y, 2 z): that axis's acceptance test and taps. A particle is
// accepted when all three axes accept it, so the three can be evaluated independently.
CAPOW_HD bool exact_axis(const Geom &g, int a, double c, AxisTaps &t) {
  if (g.survey && g.order > 1) {
    if (!survey_accept_axis(g, a, c)) return false;
    survey_axis_taps(g, a, c, t);
    return true;
  }
  const double mn = a == 0 ? g.xmin : (a == 1 ? g.ymin : g.zmin);
  const double mx = a == 0 ? g.xmax_l : (a == 1 ? g.ymax : g.zmax);
  const double d = a == 0 ? g.dx : (a == 1 ? g.dy : g.dz);
  const int n = a == 0 ? g.nx : (a == 1 ? g.ny : g.nz);
  if (g.order == 1) {  // src/read_data.c:519-541
    if ((c < mn) || (c >= mx)) return false;
    int i = (int)DDIV(DSUB(c, mn), d);
    if (a == 0) {
      if (i == g.nxtra) i = g.nxtra - 1;
    } else if (i == n) {
      i = n - 1;
    }
    t.n = 1;
    t.idx[0] = i;
    t.w[0] = 1.0;
    t.on[0] = 1;
    return true;
  }
  if (g.order == 2) {  // src/read_data.c:544-605
    if ((c < mn) || (c >= mx)) return false;
    cic_axis64(DDIV(DSUB(c, mn), d), a == 0, n, g.nxtra, g.los, t);
    return true;
  }
  if (a == 0) {  // TSC, src/read_data.c:608-619
    if (g.los == 0) {
      if (DSUB(c, g.xmin) < g.dx) c = DADD(c, g.lx);
      if ((c < DADD(mn, g.dx)) || (c >= DADD(mx, g.dx))) return false;
    } else if ((c < mn) || (c >= DADD(mx, g.dx))) {
      return false;
    }
  } else if ((c < mn) || (c >= mx)) {
    return false;
  }
  tsc_axis64(DDIV(DSUB(c, mn), d), a == 0, n, g.nxtra, g.los, t);
  return true;
}

// Linear padded index of a reference write (src/read_data.c:536 form), then the halo fold:
// indices in the halo slices map onto slice 0.. when LOS == 0 and are dropped otherwise.
// Writes into the padding columns (z >= NZ, reachable only by a rounding edge) are dropped:
// the in-place r2c transform ignores them. Returns -1 when the write does not reach the FFT input.
CAPOW_HD long long canon_index(const Geom &g, int ix, int iy, int iz) {
  unsigned long long L = (unsigned long long)iz +
                         (unsigned long long)g.row * ((unsigned long long)iy + (unsigned long long)g.ny * (unsigned long long)ix);
  if (L >= (unsigned long long)g.main_sz) {
    if (g.los != 0) return -1;
    L -= (unsigned long long)g.main_sz;
    if (L >= (unsigned long long)g.order * (unsigned long long)g.slice) return -1;
  }
  if (iz >= g.nz) return -1;  // iz < row, so iz is L % row before and after the halo fold
  return (long long)L;
}

// RSD shift of the line-of-sight coordinate, src/read_data.c:65-76, operation order preserved:
// pos += tvr*(1+z) / (100*sqrt(...)).
CAPOW_HD double rsd_shift64(const Geom &g, double pos, double v) {
  return DADD(pos, DDIV(DMUL(v, g.rsd_opz), g.rsd_den));
}

// Box check of the reader (src/read_data.c:81): true when outside.
CAPOW_HD bool outside_box(const Geom &g, double x, double y, double z) {
  return (x < g.xmin) || (x > g.xmax) || (y < g.ymin) || (y > g.ymax) || (z < g.zmin) || (z > g.zmax);
}

// w * v^e in the reference's operation order (tvr*tvr*tvr ..., then w*vr).
CAPOW_HD double wpow64(double w, double v, int e) {
  double vr = 1.0;
  if (e >= 1) vr = v;
  if (e >= 2) vr = DMUL(vr, v);
  if (e >= 3) vr = DMUL(vr, v);
  if (e >= 4) vr = DMUL(vr, v);
  return DMUL(w, vr);
}

// ---------------------------------------------------------------------------------------------
// FP32 separable taps for particles away from every discontinuity. Index rules are the same
// as above with the halo fold applied per axis (x) and the wrap rules per axis (y, z).
// kind: 0 = x axis, 1 = y or z axis. A dropped tap has index -1.
struct AxisTapsF {
  int idx[3];
  float w[3];
};

CAPOW_HD void tsc_axis32(float s, int kind, int n, int los, AxisTapsF &t) {
  if (kind == 0 && los == 0 && s < 1.0f) s += (float)n;  // src/read_data.c:611 in cell units
  int i = (int)(s + 0.5f);
  float d = s - (float)i;
  t.w[0] = 0.75f - d * d;
  t.w[1] = 0.5f * (0.5f - d) * (0.5f - d);
  t.w[2] = 0.5f * (0.5f + d) * (0.5f + d);
  int c = i, l = i - 1, h = i + 1;
  if (kind == 0) {
    bool lok = (l > 0);
    if (los == 0) {  // halo slices fold onto 0.. (src/read_data.c:152-175)
      if (c >= n) c -= n;
      if (h >= n) h -= n;
      if (l >= n) l -= n;
    } else {         // halo discarded
      if (c >= n) c = -1;
      if (h >= n) h = -1;
      if (l >= n) l = -1;
    }
    if (!lok) l = -1;
  } else if (los == 0) {
    if (i == n) {
      c = 0; l = n - 1; h = 1;
    } else {
      if (l < 0) l = n - 1;
      if (h >= n) h = 0;
    }
    if (!(l > 0)) l = -1;
  } else {
    if (c >= n) c = -1;
    if (!(l > 0)) l = -1;
    if (h >= n) h = -1;
  }
  t.idx[0] = c; t.idx[1] = l; t.idx[2] = h;
}

CAPOW_HD void cic_axis32(float s, int kind, int n, int los, AxisTapsF &t) {
  int i = (int)s;
  float d = s - (float)i;
  t.w[0] = 1.0f - d;
  t.w[1] = d;
  t.w[2] = 0.0f;
  int c = i, nb = i + 1;
  if (nb >= n) nb = (los == 0) ? nb - n : -1;  // x: halo fold/discard; y,z: wrap/skip (src/read_data.c:571-605)
  if (c >= n) c = -1;                           // unreachable for non-edge particles
  (void)kind;
  t.idx[0] = c; t.idx[1] = nb; t.idx[2] = -1;
}

CAPOW_HD void ngp_axis32(float s, int n, int los, AxisTapsF &t) {
  int i = (int)s;
  if (i >= n) i = (los == 0) ? i - n : -1;
  t.idx[0] = i; t.idx[1] = -1; t.idx[2] = -1;
  t.w[0] = 1.0f; t.w[1] = 0.0f; t.w[2] = 0.0f;
}

CAPOW_HD void axis32(int order, float s, int kind, int n, int los, AxisTapsF &t) {
  if (order == 3) tsc_axis32(s, kind, n, los, t);
  else if (order == 2) cic_axis32(s, kind, n, los, t);
  else ngp_axis32(s, n, los, t);
}

// accepted? (FP32, non-edge particles only). s* are the normal-stencil scales after the RSD shift.
CAPOW_HD bool accept32(const Geom &g, float sx, float sy, float sz) {
  const float nx = (float)g.nx, ny = (float)g.ny, nz = (float)g.nz;
  if (!(sy >= 0.0f && sy < ny && sz >= 0.0f && sz < nz)) return false;
  if (g.order == 3) {
    if (g.los == 0) {
      float s = sx < 1.0f ? sx + nx : sx;
      return s >= 1.0f && s < nx + 1.0f;
    }
    return sx >= 0.0f && sx < nx + 1.0f;
  }
  return sx >= 0.0f && sx < nx;
}
