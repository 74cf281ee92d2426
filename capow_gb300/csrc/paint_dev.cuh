// FP32 device helpers of the paint shared with the adjoint's readout: the per-particle FP32 view
// (RSD-shifted cell-unit positions), the edge test that routes a particle to the exact FP64 rules,
// and the per-axis FP32 taps.
#pragma once
#include "paint.cuh"

struct Prep {
  float sx, sy, sz, v, w;
  bool fin;
};

template <typename T>
__device__ __forceinline__ Prep prep32(const Geom &g, const FieldSpec &fs, const PIn<T> &in, long long i) {
  Prep p;
  float x = (float)in.x[i], y = (float)in.y[i], z = (float)in.z[i];
  p.v = fs.need_v ? (float)in.v[i] : 0.0f;
  p.w = in.w ? (float)in.w[i] : 1.0f;
  if (g.los == 1) x = __fmaf_rn(p.v, g.rsd_f, x);
  else if (g.los == 2) y = __fmaf_rn(p.v, g.rsd_f, y);
  else if (g.los == 3) z = __fmaf_rn(p.v, g.rsd_f, z);
  p.sx = __fmul_rn(__fsub_rn(x, g.xmin_f), g.idx_f);
  p.sy = __fmul_rn(__fsub_rn(y, g.ymin_f), g.idy_f);
  p.sz = __fmul_rn(__fsub_rn(z, g.zmin_f), g.idz_f);
  p.fin = isfinite(p.sx) && isfinite(p.sy) && isfinite(p.sz) && isfinite(p.v) && isfinite(p.w);
  return p;
}

// A particle within the FP32 error margin of a point where the reference's deposit changes
// discontinuously is painted by the exact FP64 rules. Along one axis, for one stencil's scale s:
// the acceptance ends 0 and lim (n, or n + 1 for the TSC x axis), the grid end n (halo and wrap
// rules), the TSC low-tap drop at 0.5, the TSC LOS == 0 x shift at 1, and every cell edge for NN.
// On a periodic axis (LOS == 0) anything outside [m, n - m] is an edge too: such a particle is the
// reference's fatal error, which the exact rules report. Elsewhere a stencil clearly outside the
// acceptance is simply not painted (accept32), and the particle is counted out (outside32).
// (Bitwise logic throughout: every test is cheap, so evaluating all of them beats branching.)
__device__ __forceinline__ bool edge1(float s, int n, float lim, int order, float m, bool wrap) {
  const float nf = (float)n;
  bool e = (fabsf(s) < m) | (fabsf(s - nf) < m) | (fabsf(s - lim) < m) | (fabsf(s - 0.5f) < m) |
           (fabsf(s - 1.0f) < m);
  if (wrap) e |= !(s >= m) | !(s <= nf - m);
  if (order == 1) e |= (fabsf(s - rintf(s)) < m);
  return e;
}

__device__ __forceinline__ bool is_edge(const Geom &g, float sx, float sy, float sz) {
  const bool wrap = g.los == 0;
  const float limx = (float)g.nx + (g.order == 3 ? 1.0f : 0.0f);
  bool e = edge1(sx, g.nx, limx, g.order, g.margin, wrap) | edge1(sy, g.ny, (float)g.ny, g.order, g.margin, wrap) |
           edge1(sz, g.nz, (float)g.nz, g.order, g.margin, wrap);
  if (g.interlace)
    e |= edge1(__fadd_rn(sx, 0.5f), g.nx, limx, g.order, g.margin, wrap) |
         edge1(__fadd_rn(sy, 0.5f), g.ny, (float)g.ny, g.order, g.margin, wrap) |
         edge1(__fadd_rn(sz, 0.5f), g.nz, (float)g.nz, g.order, g.margin, wrap);
  if (g.survey && g.order > 1) {
    // the Survey clamp moves a y or z stencil down one cell when its upper neighbour reaches N:
    // scale in [N - 1, N) for CIC, [N - 1.5, N - 0.5) for TSC (x never gets there inside the
    // acceptance); everything from there up takes the exact rules
    const float up = (g.order == 3 ? 1.5f : 1.0f) + g.margin;
    const float sh = g.interlace ? 0.5f : 0.0f;
    e |= !(__fadd_rn(sy, sh) < (float)g.ny - up) | !(__fadd_rn(sz, sh) < (float)g.nz - up);
  }
  return e;
}

// Outside the box (src/read_data.c:81), for a particle that is not an edge particle: no scale is
// within the margin of 0 or n, so the FP32 test decides exactly.
__device__ __forceinline__ bool outside32(const Geom &g, float sx, float sy, float sz) {
  return (sx < 0.0f) | (sx > (float)g.nx) | (sy < 0.0f) | (sy > (float)g.ny) | (sz < 0.0f) | (sz > (float)g.nz);
}

template <int K>
__device__ __forceinline__ void axis32k(float s, int kind, int n, int los, AxisTapsF &t) {
  if (K == 3) tsc_axis32(s, kind, n, los, t);
  else if (K == 2) cic_axis32(s, kind, n, los, t);
  else ngp_axis32(s, n, los, t);
}
