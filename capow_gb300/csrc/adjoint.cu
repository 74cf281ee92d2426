// capow_backward: the adjoint of the periodic multipole pipeline (paint -> mean subtraction -> 3-D FFT ->
// interlace combine -> deconvolved Legendre binning -> output_power normalisation), giving dL/d(x, y, z,
// v_los, w) of every particle from dL/dP_l(k) of every spectrum of the context: the density and the
// momentum fields (any Momentum, or the dd / dp / pp selection) and their products |A|^2, Re A*B, Im A*B,
// |B|^2. The reference has no adjoint; the forward it inverts is src/read_data.c:32-179, 514-745 and
// src/main.c:106-148, 211-225, 266-271, 302-468, 1019-1056.
//
// Steps, all on the context's stream:
//  1. the painted grids of the last catalogue (still in the slots when capow_power took the transposed
//     path, which reads them out of place; repainted otherwise) and their full 3-D R2C transform;
//  2. per half-space mode k, the gradient with respect to each interlace-combined field (as the pair
//     dL/dRe, dL/dIm, written as a complex number):
//       dL/dA' = NM gc sum_l L_l(mu) (2 c_AA,l A' + c_ReAB,l B' - i c_ImAB,l B'),
//       dL/dB' = NM gc sum_l L_l(mu) (c_ReAB,l A' + i c_ImAB,l A' + 2 c_BB,l B'),
//     with c_q,l = sum over the spectra of product q of dL/dP_l * (2l+1) / (Nmodes * norm); the normal
//     slot of a field gets it and the interlaced slot conj(e) times it (A' = A + e A_interlaced);
//  3. Hermitian completion: Phi = Gamma / 2 off the kz = 0 and kz = NZ/2 planes, and
//     Phi(k) = (Gamma(k) + conj Gamma(-k)) / 2 on them, so that the unnormalised C2R transform of Phi
//     is exactly dL/dgrid(x) = Re sum_k Gamma(k) e^{+i k.x};
//  4. per particle: the transpose of its deposit into each field (the same taps, halo fold and dropped
//     writes) read from dL/dgrid with the derivatives of the deposit values w v^e, plus the dependence
//     of NGRID (shot, norm and the mean subtraction of the density) on the accepted weights and of the
//     shot noise's velocity moment sum w v^m / sum w on every particle read.
#include <cuda_runtime.h>
#include <cufft.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "ctx.cuh"
#include "paint_dev.cuh"

template <typename R>
struct AdjC;
template <>
struct AdjC<float> {
  typedef float2 C;
};
template <>
struct AdjC<double> {
  typedef double2 C;
};

// The grid slots, stencil * fields + field: A, (B,) A interlaced, (B interlaced).
template <typename R>
struct AdjSlots {
  typename AdjC<R>::C *s[4];
};

// Hermitian multiplicity NM, src/main.c:422-429 (as in the bin kernels)
__device__ __forceinline__ int adj_nm(int i, int j, int k, int xhalf) {
  if (k != 0) return 2;
  if (j == 0) return ((i != 0) && (i != xhalf)) ? 1 : 2;
  return (i != xhalf) ? 1 : 2;
}

__device__ __forceinline__ int adj_bin(const double *E, int nk, double s) {
  int lo = 0, hi = nk + 2;  // E[lo] <= s < E[hi] (E[0] = -inf, E[nk + 2] = +inf)
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (E[mid] <= s) lo = mid;
    else hi = mid;
  }
  return lo - 1;
}

__device__ __forceinline__ double2 adj_cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// dL/dF(k) of every slot for one half-space mode. coef: [product][5][nk] (products |A|^2, Re A*B, Im A*B,
// |B|^2); pmask: the products with a nonzero coefficient.
template <typename R, int NF>
__device__ __forceinline__ void adj_gamma(const BinParams &bp, const BinTables &t, const double *coef, int pmask,
                                          int i, int j, int k, const AdjSlots<R> &sl, const double *dcv,
                                          double2 *g) {
  constexpr int NSMAX = 2 * NF;
#pragma unroll
  for (int q = 0; q < NSMAX; q++) g[q] = make_double2(0.0, 0.0);
  const double s = __dadd_rn(__dadd_rn(t.fx2d[i], t.fy2d[j]), t.fz2d[k]);
  const int b = adj_bin(t.E, bp.nk, s);
  if (b < 0 || b >= bp.nk) return;
  const long long off = ((long long)i * bp.ny + j) * bp.nzc + k;
  const bool dc = (i == 0 && j == 0 && k == 0);
  double2 F[NSMAX];
  const int ns = bp.interlace ? NSMAX : NF;
  for (int q = 0; q < ns; q++) {
    F[q] = make_double2((double)sl.s[q][off].x, (double)sl.s[q][off].y);
    if (dc) F[q] = make_double2(dcv[q], 0.0);
  }
  double2 e = make_double2(1.0, 0.0);
  double2 A = F[0], B = NF == 2 ? F[1] : make_double2(0.0, 0.0);
  double gc = t.cxd[i] * t.cyd[j] * t.czd[k] * (double)adj_nm(i, j, k, bp.xhalf);
  if (bp.interlace) {
    e = adj_cmul(adj_cmul(t.exd[i], t.eyd[j]), t.ezd[k]);
    const double2 ai = adj_cmul(F[NF], e);
    A = make_double2(A.x + ai.x, A.y + ai.y);
    if (NF == 2) {
      const double2 bi = adj_cmul(F[NF + 1], e);
      B = make_double2(B.x + bi.x, B.y + bi.y);
    }
    gc *= 0.25;
  }
  const double fl = bp.los == 1 ? t.fxd[i] : (bp.los == 2 ? t.fyd[j] : t.fzd[k]);
  const double mu = s > 0.0 ? fl / sqrt(s) : 0.0, mu2 = mu * mu;
  const double Lv[5] = {1.0, mu, 1.5 * mu2 - 0.5, (2.5 * mu2 - 1.5) * mu, (4.375 * mu2 - 3.75) * mu2 + 0.375};
  const int nk = bp.nk;
  double G[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int q = 0; q < 4; q++) {
    if (!((pmask >> q) & 1)) continue;
    for (int l = 0; l < 5; l++) {
      if ((l & 1) && !bp.odd) continue;
      G[q] += coef[(q * 5 + l) * nk + b] * Lv[l];
    }
    G[q] *= gc;
  }
  // dL/dA' and dL/dB' as (dL/dRe, dL/dIm)
  double2 gA = make_double2(2.0 * G[0] * A.x + G[1] * B.x + G[2] * B.y, 2.0 * G[0] * A.y + G[1] * B.y - G[2] * B.x);
  g[0] = gA;
  double2 gB = make_double2(0.0, 0.0);
  if (NF == 2) {
    gB = make_double2(G[1] * A.x - G[2] * A.y + 2.0 * G[3] * B.x, G[1] * A.y + G[2] * A.x + 2.0 * G[3] * B.y);
    g[1] = gB;
  }
  if (bp.interlace) {  // conj(e) times the combined field's gradient
    g[NF] = make_double2(e.x * gA.x + e.y * gA.y, e.x * gA.y - e.y * gA.x);
    if (NF == 2) g[NF + 1] = make_double2(e.x * gB.x + e.y * gB.y, e.x * gB.y - e.y * gB.x);
  }
}

__device__ __forceinline__ float2 adj_cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// adj_gamma for FP32 contexts, in FP32 (the FP32 gradients' tolerance) with the forward's exact bin: the
// FP32 s = fx^2 + (fy^2 + fz^2) of the bin kernels tested against the safe FP32 edges, the exact FP64 s
// for a mode within a few ulps of an edge. coef_f: the per-bin coefficients in FP32.
template <int NF>
__device__ __forceinline__ void adj_gamma32(const BinParams &bp, const BinTables &t, const float *coef_f, int pmask,
                                            int i, int j, int k, const AdjSlots<float> &sl, const double *dcv,
                                            float2 *g) {
  constexpr int NSMAX = 2 * NF;
#pragma unroll
  for (int q = 0; q < NSMAX; q++) g[q] = make_float2(0.0f, 0.0f);
  const int nk = bp.nk;
  const float s = t.fx2f[i] + (t.fy2f[j] + t.fz2f[k]);
  int b;
  if (!bp.lg) {
    const float v = sqrtf(s) * bp.kscale + bp.koff;
    b = v < 0.0f ? -1 : (v >= (float)nk ? nk : (int)v);
  } else {
    int a = 0, z = nk + 2;  // Elo[a] <= s < Elo[z]
    while (z - a > 1) {
      const int mid = (a + z) >> 1;
      if (t.Elo[mid] <= s) a = mid;
      else z = mid;
    }
    b = a - 1;
  }
  while (b < nk && s >= t.Elo[b + 2]) b++;
  while (b > -1 && s < t.Ehi[b + 1]) b--;
  if (!(s >= t.Elo[b + 1] && s < t.Ehi[b + 2])) b = exact_bin(t.E, nk, exact_s(t, i, j, k), b);
  if (b < 0 || b >= nk) return;
  const long long off = ((long long)i * bp.ny + j) * bp.nzc + k;
  const bool dc = (i == 0 && j == 0 && k == 0);
  float2 F[NSMAX];
  const int ns = bp.interlace ? NSMAX : NF;
  for (int q = 0; q < ns; q++) F[q] = dc ? make_float2((float)dcv[q], 0.0f) : sl.s[q][off];
  float2 e = make_float2(1.0f, 0.0f);
  float2 A = F[0], B = NF == 2 ? F[1] : make_float2(0.0f, 0.0f);
  float gc = t.cxf[i] * t.cyf[j] * t.czf[k] * (float)adj_nm(i, j, k, bp.xhalf);
  if (bp.interlace) {
    e = adj_cmulf(t.exf[i], adj_cmulf(t.eyf[j], t.ezf[k]));
    const float2 ai = adj_cmulf(F[NF], e);
    A = make_float2(A.x + ai.x, A.y + ai.y);
    if (NF == 2) {
      const float2 bi = adj_cmulf(F[NF + 1], e);
      B = make_float2(B.x + bi.x, B.y + bi.y);
    }
    gc *= 0.25f;
  }
  const float fl = bp.los == 1 ? t.fxf[i] : (bp.los == 2 ? t.fyf[j] : t.fzf[k]);
  const float mu = s > 0.0f ? fl * rsqrtf(s) : 0.0f, mu2 = mu * mu;
  const float Lv[5] = {1.0f, mu, 1.5f * mu2 - 0.5f, (2.5f * mu2 - 1.5f) * mu, (4.375f * mu2 - 3.75f) * mu2 + 0.375f};
  float G[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int q = 0; q < 4; q++) {
    if (!((pmask >> q) & 1)) continue;
#pragma unroll
    for (int l = 0; l < 5; l++) {
      if ((l & 1) && !bp.odd) continue;
      G[q] += coef_f[(q * 5 + l) * nk + b] * Lv[l];
    }
    G[q] *= gc;
  }
  const float2 gA = make_float2(2.0f * G[0] * A.x + G[1] * B.x + G[2] * B.y, 2.0f * G[0] * A.y + G[1] * B.y - G[2] * B.x);
  g[0] = gA;
  float2 gB = make_float2(0.0f, 0.0f);
  if (NF == 2) {
    gB = make_float2(G[1] * A.x - G[2] * A.y + 2.0f * G[3] * B.x, G[1] * A.y + G[2] * A.x + 2.0f * G[3] * B.y);
    g[1] = gB;
  }
  if (bp.interlace) {  // conj(e) times the combined field's gradient
    g[NF] = make_float2(e.x * gA.x + e.y * gA.y, e.x * gA.y - e.y * gA.x);
    if (NF == 2) g[NF + 1] = make_float2(e.x * gB.x + e.y * gB.y, e.x * gB.y - e.y * gB.x);
  }
}

// Step 2+3 off the self-conjugate planes: Phi = Gamma / 2, in place (FP32 contexts: adj_gamma32 with the
// FP32 coefficients coef_f).
template <typename R, int NF>
__global__ void __launch_bounds__(256) k_adj_modes(BinParams bp, BinTables t, const double *coef, const float *coef_f,
                                                   int pmask, AdjSlots<R> sl, const double *dcv, int kz_lo,
                                                   int kz_hi) {
  const int nkz = kz_hi - kz_lo;
  if (nkz <= 0) return;
  const int ns = bp.interlace ? 2 * NF : NF;
  const long long total = (long long)bp.nx * bp.ny * nkz;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int k = kz_lo + (int)(q % nkz);
    const long long r = q / nkz;
    const int j = (int)(r % bp.ny), i = (int)(r / bp.ny);
    const long long off = ((long long)i * bp.ny + j) * bp.nzc + k;
    if constexpr (sizeof(R) == 4) {
      float2 g[2 * NF];
      adj_gamma32<NF>(bp, t, coef_f, pmask, i, j, k, sl, dcv, g);
      for (int s = 0; s < ns; s++) sl.s[s][off] = make_float2(0.5f * g[s].x, 0.5f * g[s].y);
    } else {
      double2 g[2 * NF];
      adj_gamma<R, NF>(bp, t, coef, pmask, i, j, k, sl, dcv, g);
      for (int s = 0; s < ns; s++) {
        sl.s[s][off].x = (R)(0.5 * g[s].x);
        sl.s[s][off].y = (R)(0.5 * g[s].y);
      }
    }
  }
}

// Step 2+3 on one self-conjugate plane kz: each mode pair (k, -k) by the thread of its lower index.
// Also records Re Gamma(0) of the density's slots (its mean subtraction makes F(0) = sum - NGRID).
template <typename R, int NF>
__global__ void __launch_bounds__(256) k_adj_plane(BinParams bp, BinTables t, const double *coef, int pmask,
                                                   AdjSlots<R> sl, const double *dcv, int kz, double *gamma0) {
  const int ns = bp.interlace ? 2 * NF : NF;
  const long long total = (long long)bp.nx * bp.ny;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q / bp.ny), j = (int)(q % bp.ny);
    const int i2 = (bp.nx - i) % bp.nx, j2 = (bp.ny - j) % bp.ny;
    const long long q2 = (long long)i2 * bp.ny + j2;
    if (q2 < q) continue;  // the partner's thread handles the pair
    double2 a[2 * NF], b[2 * NF];
    adj_gamma<R, NF>(bp, t, coef, pmask, i, j, kz, sl, dcv, a);
    if (kz == 0 && i == 0 && j == 0) {
      gamma0[0] = a[0].x;
      gamma0[1] = bp.interlace ? a[NF].x : 0.0;
    }
    const long long off = ((long long)i * bp.ny + j) * bp.nzc + kz, off2 = ((long long)i2 * bp.ny + j2) * bp.nzc + kz;
    if (q2 == q) {  // self-conjugate mode: Phi = Re Gamma
      for (int s = 0; s < ns; s++) {
        sl.s[s][off].x = (R)a[s].x;
        sl.s[s][off].y = (R)0;
      }
      continue;
    }
    adj_gamma<R, NF>(bp, t, coef, pmask, i2, j2, kz, sl, dcv, b);
    for (int s = 0; s < ns; s++) {
      const double2 p = make_double2(0.5 * (a[s].x + b[s].x), 0.5 * (a[s].y - b[s].y));  // (Gamma(k) + conj Gamma(-k)) / 2
      sl.s[s][off].x = (R)p.x;
      sl.s[s][off].y = (R)p.y;
      sl.s[s][off2].x = (R)p.x;
      sl.s[s][off2].y = (R)(-p.y);
    }
  }
}

// Weight derivatives dW/dscale of the taps exact_axes produced, from the same per-axis offset d.
__device__ __forceinline__ void adj_axis_deriv(int order, double scale, double *dw) {
  if (order == 3) {
    const int i = (int)__dadd_rn(scale, 0.5);
    const double d = __dsub_rn(scale, (double)i);
    dw[0] = -2.0 * d;    // centre: 0.75 - d^2
    dw[1] = -(0.5 - d);  // low: (0.5 - d)^2 / 2
    dw[2] = 0.5 + d;     // high: (0.5 + d)^2 / 2
  } else if (order == 2) {
    dw[0] = -1.0;  // 1 - d
    dw[1] = 1.0;   // d
    dw[2] = 0.0;
  } else {
    dw[0] = dw[1] = dw[2] = 0.0;
  }
}

// What the readout needs beyond the gradient grids: dL/dNGRID (for the accepted weights) and the shot
// noise's moments: dL/d(sum w v^m / sum w) for m = 1..4, with that ratio c[m] and sum w over the catalogue.
struct AdjScalars {
  double dLdN;
  double dLdc[5], c[5];
  double wsum;
};

// dL/d(particle) from the deposit's gradient sums per field: g0 = sum G W, gs = sum G dW/dscale per axis.
template <typename T>
__device__ __forceinline__ void adj_store(const Geom &g, const FieldSpec &fs, double v, double w, const double *g0,
                                          const double (*gs)[3], bool accepted, bool read, const AdjScalars &as,
                                          long long p, T *ox, T *oy, T *oz, T *ov, T *ow) {
  double dxr = 0.0, dyr = 0.0, dzr = 0.0, dw = 0.0, dv = 0.0;
  for (int f = 0; f < fs.nfields; f++) {
    const int e = f ? fs.eb : fs.ea;
    double ve = 1.0, vm = 1.0;
    for (int k = 0; k < e; k++) ve *= v;
    for (int k = 0; k < e - 1; k++) vm *= v;
    const double val = w * ve;  // the field's deposit value w v^e
    dxr += val * gs[f][0] / g.dx;
    dyr += val * gs[f][1] / g.dy;
    dzr += val * gs[f][2] / g.dz;
    dw += ve * g0[f];
    if (e > 0) dv += w * (double)e * vm * g0[f];
  }
  if (accepted) dw += as.dLdN;
  if (read) {  // the shot noise's sum w v^m / sum w over every particle read (src/read_data.c:132-138)
    double vm = 1.0;
    for (int m = 1; m <= 4; m++) {
      if (as.dLdc[m] != 0.0) {
        dw += as.dLdc[m] * (vm * v - as.c[m]) / as.wsum;
        dv += as.dLdc[m] * (double)m * w * vm / as.wsum;
      }
      vm *= v;
    }
  }
  const double rsd = g.rsd_opz / g.rsd_den;  // d(shifted LOS coordinate)/dv
  if (g.los == 1) dv += rsd * dxr;
  else if (g.los == 2) dv += rsd * dyr;
  else if (g.los == 3) dv += rsd * dzr;
  if (ox) ox[p] = (T)dxr;
  if (oy) oy[p] = (T)dyr;
  if (oz) oz[p] = (T)dzr;
  if (ov) ov[p] = (T)dv;
  if (ow) ow[p] = (T)dw;
}

// Step 4 for one particle by the exact FP64 rules: the transpose of its deposits (same taps, halo
// fold and dropped writes) read from dL/dgrid with the weight derivatives. gr: the real slots.
template <typename T, typename R>
__device__ __forceinline__ void adj_particle_exact(const Geom &g, const FieldSpec &fs, const PIn<T> &in, long long p,
                                                   const R *const *gr, const AdjScalars &as, T *ox, T *oy, T *oz,
                                                   T *ov, T *ow) {
  double x = (double)in.x[p], y = (double)in.y[p], z = (double)in.z[p];
  const double v = fs.need_v ? (double)in.v[p] : 0.0, w = in.w ? (double)in.w[p] : 1.0;
  const bool read = isfinite(x) && isfinite(y) && isfinite(z) && isfinite(v) && isfinite(w);
  if (g.los == 1) x = rsd_shift64(g, x, v);
  else if (g.los == 2) y = rsd_shift64(g, y, v);
  else if (g.los == 3) z = rsd_shift64(g, z, v);
  const int nf = fs.nfields;
  double g0[2] = {0.0, 0.0}, gs[2][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
  bool accepted = false;
  {  // a particle outside the box (LOS != 0) is still painted where a stencil accepts it (src/read_data.c:81-97)
    const int nst = g.interlace ? 2 : 1;
    for (int st = 0; st < nst; st++) {
      const double px = st ? DADD(x, g.hx) : x, py = st ? DADD(y, g.hy) : y, pz = st ? DADD(z, g.hz) : z;
      AxisTaps ax, ay, az;
      if (!exact_axes(g, px, py, pz, ax, ay, az)) continue;
      if (st == 0) accepted = true;
      // the scales exact_axes used (TSC with LOS == 0 maps x - XMIN < dx to x + L first)
      double qx = px;
      if (g.order == 3 && g.los == 0 && DSUB(qx, g.xmin) < g.dx) qx = DADD(qx, g.lx);
      double dx3[3], dy3[3], dz3[3];
      adj_axis_deriv(g.order, DDIV(DSUB(qx, g.xmin), g.dx), dx3);
      adj_axis_deriv(g.order, DDIV(DSUB(py, g.ymin), g.dy), dy3);
      adj_axis_deriv(g.order, DDIV(DSUB(pz, g.zmin), g.dz), dz3);
      for (int c = 0; c < az.n; c++)
        for (int b = 0; b < ay.n; b++)
          for (int a = 0; a < ax.n; a++) {
            if (!(ax.on[a] && ay.on[b] && az.on[c])) continue;
            const long long L = canon_index(g, ax.idx[a], ay.idx[b], az.idx[c]);
            if (L < 0) continue;
            for (int f = 0; f < nf; f++) {
              const double G = (double)gr[st * nf + f][L];
              g0[f] += G * ax.w[a] * ay.w[b] * az.w[c];
              gs[f][0] += G * dx3[a] * ay.w[b] * az.w[c];
              gs[f][1] += G * ax.w[a] * dy3[b] * az.w[c];
              gs[f][2] += G * ax.w[a] * ay.w[b] * dz3[c];
            }
          }
    }
  }
  adj_store(g, fs, v, w, g0, gs, accepted, read, as, p, ox, oy, oz, ov, ow);
}

template <typename R>
struct AdjGrids {
  const R *s[4];
};

// dL/dNGRID on the device: the host's part minus Re Gamma(0) of the density's slots
__device__ __forceinline__ AdjScalars adj_scalars(const Geom &g, const AdjScalars &h, const double *gamma0) {
  AdjScalars a = h;
  a.dLdN = h.dLdN - gamma0[0] - (g.interlace ? gamma0[1] : 0.0);
  return a;
}

template <typename T, typename R>
__global__ void __launch_bounds__(128) k_adj_readout(Geom g, FieldSpec fs, PIn<T> in, long long n, AdjGrids<R> gr,
                                                     AdjScalars hs, const double *gamma0, T *ox, T *oy, T *oz,
                                                     T *ov, T *ow) {
  const AdjScalars as = adj_scalars(g, hs, gamma0);
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x)
    adj_particle_exact<T, R>(g, fs, in, p, gr.s, as, ox, oy, oz, ov, ow);
}

// FP32 per-axis weight derivatives of the taps axis32k produced (same offset d).
template <int K>
__device__ __forceinline__ void adj_axis_deriv32(float s, int kind, int n, int los, float *dw) {
  if (K == 3) {
    if (kind == 0 && los == 0 && s < 1.0f) s += (float)n;  // the x shift of tsc_axis32
    const int i = (int)(s + 0.5f);
    const float d = s - (float)i;
    dw[0] = -2.0f * d;
    dw[1] = -(0.5f - d);
    dw[2] = 0.5f + d;
  } else if (K == 2) {
    dw[0] = -1.0f;
    dw[1] = 1.0f;
    dw[2] = 0.0f;
  } else {
    dw[0] = dw[1] = dw[2] = 0.0f;
  }
}

// The constants of adj_store in FP32, formed once per thread: 1/d per axis and d(shifted LOS coordinate)/dv
// as the paint's FP32 scales use them, dL/dNGRID, and dL/dc_m / sum w with c_m.
struct AdjK32 {
  float idx, idy, idz, rsd, dLdN;
  float dLdc_w[5], c[5];
  bool shot_moments;
};

__device__ __forceinline__ AdjK32 adj_k32(const Geom &g, const AdjScalars &as) {
  AdjK32 k;
  k.idx = g.idx_f;
  k.idy = g.idy_f;
  k.idz = g.idz_f;
  k.rsd = g.rsd_f;
  k.dLdN = (float)as.dLdN;
  k.shot_moments = false;
  for (int m = 0; m < 5; m++) {
    k.dLdc_w[m] = m > 0 && as.dLdc[m] != 0.0 ? (float)(as.dLdc[m] / as.wsum) : 0.0f;
    k.c[m] = (float)as.c[m];
    k.shot_moments |= k.dLdc_w[m] != 0.0f;
  }
  return k;
}

// adj_store in FP32 for a particle of the FP32 readout (finite, so read; the gradient sums g0, gs from
// its FP32 gather).
template <int NF, typename T>
__device__ __forceinline__ void adj_store32(const FieldSpec &fs, float v, float w, const float *g0,
                                            const float (*gs)[3], bool accepted, const AdjK32 &k, int los,
                                            long long p, T *ox, T *oy, T *oz, T *ov, T *ow) {
  float dxr = 0.0f, dyr = 0.0f, dzr = 0.0f, dw = 0.0f, dv = 0.0f;
#pragma unroll
  for (int f = 0; f < NF; f++) {
    const int e = f ? fs.eb : fs.ea;
    float ve = 1.0f, vm = 1.0f;
    for (int q = 0; q < e; q++) ve *= v;
    for (int q = 0; q < e - 1; q++) vm *= v;
    const float val = w * ve;  // the field's deposit value w v^e
    dxr += val * gs[f][0];
    dyr += val * gs[f][1];
    dzr += val * gs[f][2];
    dw += ve * g0[f];
    if (e > 0) dv += w * (float)e * vm * g0[f];
  }
  dxr *= k.idx;
  dyr *= k.idy;
  dzr *= k.idz;
  if (accepted) dw += k.dLdN;
  if (k.shot_moments) {  // the shot noise's sum w v^m / sum w over every particle read (src/read_data.c:132-138)
    float vm = 1.0f;
    for (int m = 1; m <= 4; m++) {
      dw += k.dLdc_w[m] * (vm * v - k.c[m]);
      dv += k.dLdc_w[m] * (float)m * w * vm;
      vm *= v;
    }
  }
  if (los == 1) dv += k.rsd * dxr;
  else if (los == 2) dv += k.rsd * dyr;
  else if (los == 3) dv += k.rsd * dzr;
  if (ox) ox[p] = (T)dxr;
  if (oy) oy[p] = (T)dyr;
  if (oz) oz[p] = (T)dzr;
  if (ov) ov[p] = (T)dv;
  if (ow) ow[p] = (T)dw;
}

// Step 4 for FP32 contexts: particles away from every edge of the reference's rules gather their
// taps with the FP32 rules of the paint (the same ones that deposited them) and form their gradient in
// FP32; the others take the exact FP64 path.
template <int K, int NF, typename T>
__global__ void __launch_bounds__(128) k_adj_readout32(Geom g, FieldSpec fs, PIn<T> in, long long n,
                                                       AdjGrids<float> gr, AdjScalars hs, const double *gamma0,
                                                       T *ox, T *oy, T *oz, T *ov, T *ow) {
  const AdjScalars as = adj_scalars(g, hs, gamma0);
  const AdjK32 k32 = adj_k32(g, as);
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const Prep pr = prep32(g, fs, in, p);
    if (!pr.fin || is_edge(g, pr.sx, pr.sy, pr.sz)) {
      adj_particle_exact<T, float>(g, fs, in, p, gr.s, as, ox, oy, oz, ov, ow);
      continue;
    }
    float g0[NF], gs[NF][3];
#pragma unroll
    for (int f = 0; f < NF; f++) g0[f] = gs[f][0] = gs[f][1] = gs[f][2] = 0.0f;
    bool accepted = false;
    const int nst = g.interlace ? 2 : 1;
    for (int st = 0; st < nst; st++) {
      const float sx = st ? __fadd_rn(pr.sx, 0.5f) : pr.sx, sy = st ? __fadd_rn(pr.sy, 0.5f) : pr.sy,
                  sz = st ? __fadd_rn(pr.sz, 0.5f) : pr.sz;
      if (!accept32(g, sx, sy, sz)) continue;
      if (st == 0) accepted = true;
      AxisTapsF ax, ay, az;
      axis32k<K>(sx, 0, g.nx, g.los, ax);
      axis32k<K>(sy, 1, g.ny, g.los, ay);
      axis32k<K>(sz, 1, g.nz, g.los, az);
      float dx3[3], dy3[3], dz3[3];
      adj_axis_deriv32<K>(sx, 0, g.nx, g.los, dx3);
      adj_axis_deriv32<K>(sy, 1, g.ny, g.los, dy3);
      adj_axis_deriv32<K>(sz, 1, g.nz, g.los, dz3);
      // per (x, y) tap pair, the z taps' sums S = sum_c G W_z and D = sum_c G dW_z, then the pair's weights
#pragma unroll
      for (int a = 0; a < K; a++) {
        if (ax.idx[a] < 0) continue;
#pragma unroll
        for (int b = 0; b < K; b++) {
          if (ay.idx[b] < 0) continue;
          const long long rowb = ((long long)ax.idx[a] * g.ny + ay.idx[b]) * g.row;
          float S[NF], D[NF];
#pragma unroll
          for (int f = 0; f < NF; f++) S[f] = D[f] = 0.0f;
#pragma unroll
          for (int c = 0; c < K; c++) {
            if (az.idx[c] < 0) continue;
#pragma unroll
            for (int f = 0; f < NF; f++) {
              const float G = gr.s[st * NF + f][rowb + az.idx[c]];
              S[f] += G * az.w[c];
              D[f] += G * dz3[c];
            }
          }
          const float wxy = ax.w[a] * ay.w[b], dxy = dx3[a] * ay.w[b], xdy = ax.w[a] * dy3[b];
#pragma unroll
          for (int f = 0; f < NF; f++) {
            g0[f] += wxy * S[f];
            gs[f][0] += dxy * S[f];
            gs[f][1] += xdy * S[f];
            gs[f][2] += wxy * D[f];
          }
        }
      }
    }
    adj_store32<NF, T>(fs, pr.v, pr.w, g0, gs, accepted, k32, g.los, p, ox, oy, oz, ov, ow);
  }
}

static int make_3d_plans(capow_ctx *c) {
  if (c->adj_plans) return CAPOW_OK;
  const bool f64 = c->prec == CAPOW_FP64;
  const capow_params *p = &c->p;
  const int nzc = p->NZ / 2 + 1;
  int n[3] = {p->NX, p->NY, p->NZ};
  int inembed[3] = {p->NX, p->NY, 2 * nzc}, onembed[3] = {p->NX, p->NY, nzc};
  const long long idist = (long long)c->grid_elems, odist = (long long)c->grid_elems / 2;
  if (idist > 0x7fffffffLL) FAIL(c, CAPOW_ENOTSUP, "capow_backward: grid too large for one batched plan");
  CKFFT(c, cufftPlanMany(&c->adj_fwd, 3, n, inembed, 1, (int)idist, onembed, 1, (int)odist, f64 ? CUFFT_D2Z : CUFFT_R2C,
                         c->nslot));
  CKFFT(c, cufftPlanMany(&c->adj_inv, 3, n, onembed, 1, (int)odist, inembed, 1, (int)idist, f64 ? CUFFT_Z2D : CUFFT_C2R,
                         c->nslot));
  CKFFT(c, cufftSetStream(c->adj_fwd, c->stream));
  CKFFT(c, cufftSetStream(c->adj_inv, c->stream));
  c->adj_plans = true;
  return CAPOW_OK;
}

// grid-launch helper for the mode kernels
static int adj_blocks(long long work) {
  long long b = (work + 255) / 256;
  if (b > 152LL * 16) b = 152LL * 16;
  return (int)(b < 1 ? 1 : b);
}

template <typename R, int NF>
static void adj_mode_kernels(capow_ctx *c, const double *coef_d, const float *coef_f, int pmask, double *gamma0) {
  const capow_params &p = c->p;
  const size_t eb = sizeof(R);
  AdjSlots<R> sl;
  for (int s = 0; s < 4; s++)
    sl.s[s] = s < c->nslot ? (typename AdjC<R>::C *)((char *)c->grid_base + eb * c->grid_elems * s) : nullptr;
  const int nyq = (p.NZ % 2 == 0) ? p.NZ / 2 : -1;
  const int kz_hi = nyq > 0 ? nyq : c->bp.nzc;
  const long long interior = (long long)p.NX * p.NY * (kz_hi - 1 > 0 ? kz_hi - 1 : 0);
  const int nbm = adj_blocks(interior), nbp = adj_blocks((long long)p.NX * p.NY);
  k_adj_modes<R, NF><<<nbm, 256, 0, c->stream>>>(c->bp, c->bt, coef_d, coef_f, pmask, sl, c->dcv, 1, kz_hi);
  k_adj_plane<R, NF><<<nbp, 256, 0, c->stream>>>(c->bp, c->bt, coef_d, pmask, sl, c->dcv, 0, gamma0);
  if (nyq > 0) k_adj_plane<R, NF><<<nbp, 256, 0, c->stream>>>(c->bp, c->bt, coef_d, pmask, sl, c->dcv, nyq, gamma0);
  c->launches += nyq > 0 ? 3 : 2;
}

template <typename T>
static void adj_readout(capow_ctx *c, long long n, const AdjScalars &hs, const double *gamma0, void *const *dev) {
  const capow_particles &d = c->last;
  const PIn<T> in{(const T *)d.x, (const T *)d.y, (const T *)d.z, (const T *)d.vlos, (const T *)d.w};
  const int nb = (int)((n + 127) / 128 > 152 * 16 ? 152 * 16 : ((n + 127) / 128 < 1 ? 1 : (n + 127) / 128));
  T *o[5];
  for (int k = 0; k < 5; k++) o[k] = (T *)dev[k];
  const size_t eb = c->prec == CAPOW_FP64 ? 8 : 4;
  if (c->prec == CAPOW_FP64) {
    AdjGrids<double> gr;
    for (int s = 0; s < 4; s++) gr.s[s] = s < c->nslot ? (const double *)((char *)c->grid_base + eb * c->grid_elems * s) : nullptr;
    k_adj_readout<T, double><<<nb, 128, 0, c->stream>>>(c->g, c->fs, in, n, gr, hs, gamma0, o[0], o[1], o[2], o[3], o[4]);
    return;
  }
  AdjGrids<float> gr;
  for (int s = 0; s < 4; s++) gr.s[s] = s < c->nslot ? (const float *)((char *)c->grid_base + eb * c->grid_elems * s) : nullptr;
  const int K = c->p.InterpOrder;
#define ADJ_RUN32(KK, NFF) \
  k_adj_readout32<KK, NFF, T><<<nb, 128, 0, c->stream>>>(c->g, c->fs, in, n, gr, hs, gamma0, o[0], o[1], o[2], o[3], o[4])
  if (c->fs.nfields == 2) {
    if (K == 3) ADJ_RUN32(3, 2);
    else if (K == 2) ADJ_RUN32(2, 2);
    else ADJ_RUN32(1, 2);
  } else {
    if (K == 3) ADJ_RUN32(3, 1);
    else if (K == 2) ADJ_RUN32(2, 1);
    else ADJ_RUN32(1, 1);
  }
#undef ADJ_RUN32
}

extern "C" int capow_backward(capow_ctx *c, const double *const *dL_dP, const capow_grads *out) {
  if (!c || !dL_dP || !out) return CAPOW_EINVAL;
  if (c->pending) FAIL(c, CAPOW_ESTATE, "capow_power_result of the power stage in flight first");
  if (!c->powered) FAIL(c, CAPOW_ESTATE, "capow_backward needs capow_paint and capow_power first");
  if (out->dtype != CAPOW_F32 && out->dtype != CAPOW_F64) FAIL(c, CAPOW_EINVAL, "grads dtype must be F32 or F64");
  CK(c, cudaSetDevice(c->o.device));
  const capow_params &p = c->p;
  const int nk = p.NK, nf = c->fs.nfields;
  const long long n = (long long)c->last.n;
  // ---- host: per-product, per-bin coefficients c_q,l(b) = sum over the spectra of product q of
  // dL/dP_l(b) (2l+1) / (Nmodes(b) norm); dL/dNGRID through norm = NGRID^2 / V and shot = NGRID c_m;
  // dL/dc_m through the shot (src/main.c:106-148, 1019-1056)
  const DevStats &st = *c->h_st;
  const double N = st.ngrid;
  const double V = (p.XMAX - p.XMIN) * (p.YMAX - p.YMIN) * (p.ZMAX - p.ZMIN);
  const double norm = N * N / V;
  AdjScalars hs;
  memset(&hs, 0, sizeof hs);
  hs.wsum = st.nsq;
  hs.c[0] = 1.0;
  for (int m = 1; m <= 4; m++) hs.c[m] = c->moments && st.nsq != 0.0 ? st.vr[m - 1] / st.nsq : 0.0;
  int last = -1;  // output_power zeroes the highest filled bin (its output does not depend on anything)
  for (int b = 0; b < nk; b++)
    if (c->nmodes[b] > 0) last = b;
  std::vector<double> coef(NPROD * 5 * nk, 0.0);
  int pmask = 0;
  for (int q = 0; q < c->bp.nspec; q++) {
    const int pq = spectrum_product(nf, c->bp.spec[q]);
    const int m = c->shot_moment[q];
    const double shot = N * hs.c[m];
    for (int b = 0; b < nk; b++) {
      const double nm = (double)c->nmodes[b];
      if (nm <= 0.0 || b == last || norm <= 0.0) continue;
      for (int l = 0; l < 5; l++) {
        if ((l == 1 || l == 3) && !p.Odd_Multipoles) continue;
        const double gl = dL_dP[q * 5 + l] ? dL_dP[q * 5 + l][b] : 0.0;
        if (gl == 0.0) continue;
        coef[(pq * 5 + l) * nk + b] += gl * (double)(2 * l + 1) / (nm * norm);
        pmask |= 1 << pq;
        const double S = c->h_bins[(pq * 5 + l) * nk + b];  // the raw sum of this product and multipole
        const double P = l == 0 ? (S / nm - shot) / norm : (double)(2 * l + 1) * S / (nm * norm);
        hs.dLdN += gl * (l == 0 ? -2.0 * P / N - hs.c[m] / norm : -2.0 * P / N);
        if (l == 0 && m > 0) hs.dLdc[m] += gl * (-N / norm);
      }
    }
  }
  // device: the coefficients in FP64, Re Gamma(0) of the density's two slots, the coefficients in FP32
  const size_t ncoef = (size_t)NPROD * 5 * nk;
  if (!c->adj_coef)
    CK(c, cudaMalloc(&c->adj_coef, sizeof(double) * (ncoef + 2) + sizeof(float) * ncoef));
  double *coef_d = c->adj_coef, *gamma0 = c->adj_coef + ncoef;
  float *coef_f = (float *)(c->adj_coef + ncoef + 2);
  CK(c, cudaMemcpyAsync(coef_d, coef.data(), sizeof(double) * ncoef, cudaMemcpyHostToDevice, c->stream));
  const std::vector<float> coef32(coef.begin(), coef.end());
  CK(c, cudaMemcpyAsync(coef_f, coef32.data(), sizeof(float) * ncoef, cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaMemsetAsync(gamma0, 0, 2 * sizeof(double), c->stream));
  int rc = make_3d_plans(c);
  if (rc) return rc;
  // ---- the forward's grids (repainted unless the power stage left them in place), full 3-D transform
  rc = enqueue_backward_paint(c);
  if (rc) return rc;
  c->grids_intact = false;  // the transform below runs in place
  const bool f64 = c->prec == CAPOW_FP64;
  if (f64) CKFFT(c, cufftExecD2Z(c->adj_fwd, (cufftDoubleReal *)c->grid_base, (cufftDoubleComplex *)c->grid_base));
  else CKFFT(c, cufftExecR2C(c->adj_fwd, (cufftReal *)c->grid_base, (cufftComplex *)c->grid_base));
  // ---- mode gradients and Hermitian completion, then the inverse transform. Re Gamma(0) enters dL/dNGRID
  // only where the density is mean-subtracted (F(0) = sum - NGRID); otherwise gamma0 is cleared after
  if (f64) {
    if (nf == 2) adj_mode_kernels<double, 2>(c, coef_d, coef_f, pmask, gamma0);
    else adj_mode_kernels<double, 1>(c, coef_d, coef_f, pmask, gamma0);
    CKFFT(c, cufftExecZ2D(c->adj_inv, (cufftDoubleComplex *)c->grid_base, (cufftDoubleReal *)c->grid_base));
  } else {
    if (nf == 2) adj_mode_kernels<float, 2>(c, coef_d, coef_f, pmask, gamma0);
    else adj_mode_kernels<float, 1>(c, coef_d, coef_f, pmask, gamma0);
    CKFFT(c, cufftExecC2R(c->adj_inv, (cufftComplex *)c->grid_base, (cufftReal *)c->grid_base));
  }
  if (!c->bp.mean_sub_a) CK(c, cudaMemsetAsync(gamma0, 0, 2 * sizeof(double), c->stream));
  CK(c, cudaGetLastError());
  // ---- per-particle readout into device buffers (the caller's, or staging for host outputs)
  const size_t ob = out->dtype == CAPOW_F64 ? 8 : 4;
  void *dst[5] = {out->dx, out->dy, out->dz, out->dvlos, out->dw};
  void *dev[5];
  for (int k = 0; k < 5; k++) {
    dev[k] = nullptr;
    if (!dst[k]) continue;
    if (out->on_device) {
      dev[k] = dst[k];
    } else {
      if (c->adj_stage_bytes[k] < ob * (size_t)n) {
        if (c->adj_stage[k]) cudaFree(c->adj_stage[k]);
        c->adj_stage[k] = nullptr;
        c->adj_stage_bytes[k] = 0;
        CK(c, cudaMalloc(&c->adj_stage[k], ob * (size_t)(n ? n : 1)));
        c->adj_stage_bytes[k] = ob * (size_t)(n ? n : 1);
      }
      dev[k] = c->adj_stage[k];
    }
  }
  if (c->last.dtype != out->dtype)
    FAIL(c, CAPOW_EINVAL, "capow_backward: gradient dtype must match the painted particles' dtype");
  if (c->last.dtype == CAPOW_F64) adj_readout<double>(c, n, hs, gamma0, dev);
  else adj_readout<float>(c, n, hs, gamma0, dev);
  c->launches++;
  CK(c, cudaGetLastError());
  if (!out->on_device)
    for (int k = 0; k < 5; k++)
      if (dst[k]) CK(c, cudaMemcpyAsync(dst[k], dev[k], ob * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  c->powered = true;  // the grids hold dL/dgrid now: a new paint is needed before capow_power
  c->grids_intact = false;
  return CAPOW_OK;
}
