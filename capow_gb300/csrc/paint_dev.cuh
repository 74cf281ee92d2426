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
// discontinuously (box faces 0 and N, anything outside [0, N], the TSC low-tap drop at 0.5, the
// TSC LOS==0 x shift at 1, every cell edge for NN) is painted by the exact FP64 rules.
// (Bitwise logic throughout: every test is cheap, so evaluating all of them beats branching.)
__device__ __forceinline__ bool edge1(float s, int n, int order, float m) {
  const float nf = (float)n;
  bool e = !(s >= m) | !(s <= nf - m) | (fabsf(s - 0.5f) < m) | (fabsf(s - 1.0f) < m);
  if (order == 1) e |= (fabsf(s - rintf(s)) < m);
  return e;
}

__device__ __forceinline__ bool is_edge(const Geom &g, float sx, float sy, float sz) {
  bool e = edge1(sx, g.nx, g.order, g.margin) | edge1(sy, g.ny, g.order, g.margin) |
           edge1(sz, g.nz, g.order, g.margin);
  if (g.interlace)
    e |= edge1(__fadd_rn(sx, 0.5f), g.nx, g.order, g.margin) | edge1(__fadd_rn(sy, 0.5f), g.ny, g.order, g.margin) |
         edge1(__fadd_rn(sz, 0.5f), g.nz, g.order, g.margin);
  return e;
}

template <int K>
__device__ __forceinline__ void axis32k(float s, int kind, int n, int los, AxisTapsF &t) {
  if (K == 3) tsc_axis32(s, kind, n, los, t);
  else if (K == 2) cic_axis32(s, kind, n, los, t);
  else ngp_axis32(s, n, los, t);
}
