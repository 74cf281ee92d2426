// capow_backward: the adjoint of the periodic density-multipole pipeline (paint -> mean subtraction
// -> 3-D FFT -> interlace combine -> deconvolved Legendre binning -> output_power normalisation),
// giving dL/d(x, y, z, v_los, w) of every particle from dL/dP_l(k). The reference has no adjoint;
// the forward it inverts is src/read_data.c:32-179, 514-745 and src/main.c:106-148, 211-225,
// 266-271, 302-468, 1019-1056.
//
// Steps, all on the context's stream:
//  1. repaint the last catalogue and take the full 3-D R2C transform of every slot;
//  2. per half-space mode k: Gamma = dL/dF'(k) = 2 NM gc sum_l c_l(bin) L_l(mu) F'(k), with
//     F' = F + e Fi the interlace combine and c_l = dL/dP_l * (2l+1) / (Nmodes * norm); the slots
//     get Gamma and conj(e) Gamma;
//  3. Hermitian completion: Phi = Gamma / 2 off the kz = 0 and kz = NZ/2 planes, and
//     Phi(k) = (Gamma(k) + conj Gamma(-k)) / 2 on them, so that the unnormalised C2R transform of Phi
//     is exactly dL/dgrid(x) = Re sum_k Gamma(k) e^{+i k.x};
//  4. per particle: the transpose of its deposit (the same taps, halo fold and dropped writes) read
//     from dL/dgrid with the weight derivatives, plus the dependence of NGRID (shot, norm and the
//     mean subtraction) for the weights.
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

// dL/dF'(k) for one half-space mode, returned for the normal slot (gA) and the interlaced slot (gAi).
template <typename R>
__device__ __forceinline__ void adj_gamma(const BinParams &bp, const BinTables &t, const double *coef, int i, int j,
                                          int k, const typename AdjC<R>::C *gA, const typename AdjC<R>::C *gAi,
                                          const double *dcv, double2 &gF, double2 &gFi) {
  gF = make_double2(0.0, 0.0);
  gFi = make_double2(0.0, 0.0);
  const double s = __dadd_rn(__dadd_rn(t.fx2d[i], t.fy2d[j]), t.fz2d[k]);
  const int b = adj_bin(t.E, bp.nk, s);
  if (b < 0 || b >= bp.nk) return;
  const long long off = ((long long)i * bp.ny + j) * bp.nzc + k;
  const bool dc = (i == 0 && j == 0 && k == 0);
  double2 F = make_double2((double)gA[off].x, (double)gA[off].y);
  if (dc) F = make_double2(dcv[0], 0.0);
  double2 e = make_double2(1.0, 0.0), Fp = F;
  double gc = t.cxd[i] * t.cyd[j] * t.czd[k] * (double)adj_nm(i, j, k, bp.xhalf);
  if (bp.interlace) {
    double2 Fi = make_double2((double)gAi[off].x, (double)gAi[off].y);
    if (dc) Fi = make_double2(dcv[1], 0.0);
    const double2 ex = t.exd[i], ey = t.eyd[j], ez = t.ezd[k];
    const double2 exy = make_double2(ex.x * ey.x - ex.y * ey.y, ex.x * ey.y + ex.y * ey.x);
    e = make_double2(exy.x * ez.x - exy.y * ez.y, exy.x * ez.y + exy.y * ez.x);
    Fp = make_double2(F.x + Fi.x * e.x - Fi.y * e.y, F.y + Fi.x * e.y + Fi.y * e.x);
    gc *= 0.25;
  }
  const double fl = bp.los == 1 ? t.fxd[i] : (bp.los == 2 ? t.fyd[j] : t.fzd[k]);
  const double mu = s > 0.0 ? fl / sqrt(s) : 0.0, mu2 = mu * mu;
  const int nk = bp.nk;
  double G = coef[0 * nk + b] + coef[2 * nk + b] * (1.5 * mu2 - 0.5) +
             coef[4 * nk + b] * ((4.375 * mu2 - 3.75) * mu2 + 0.375);
  if (bp.odd) G += coef[1 * nk + b] * mu + coef[3 * nk + b] * ((2.5 * mu2 - 1.5) * mu);
  G *= 2.0 * gc;
  gF = make_double2(G * Fp.x, G * Fp.y);
  if (bp.interlace) gFi = make_double2(e.x * gF.x + e.y * gF.y, e.x * gF.y - e.y * gF.x);  // conj(e) * gF
}

// Step 2+3 off the self-conjugate planes: Phi = Gamma / 2, in place.
template <typename R>
__global__ void __launch_bounds__(256) k_adj_modes(BinParams bp, BinTables t, const double *coef,
                                                   typename AdjC<R>::C *gA, typename AdjC<R>::C *gAi,
                                                   const double *dcv, int kz_lo, int kz_hi) {
  const int nkz = kz_hi - kz_lo;
  if (nkz <= 0) return;
  const long long total = (long long)bp.nx * bp.ny * nkz;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int k = kz_lo + (int)(q % nkz);
    const long long r = q / nkz;
    const int j = (int)(r % bp.ny), i = (int)(r / bp.ny);
    double2 gF, gFi;
    adj_gamma<R>(bp, t, coef, i, j, k, gA, gAi, dcv, gF, gFi);
    const long long off = ((long long)i * bp.ny + j) * bp.nzc + k;
    gA[off].x = (R)(0.5 * gF.x);
    gA[off].y = (R)(0.5 * gF.y);
    if (bp.interlace) {
      gAi[off].x = (R)(0.5 * gFi.x);
      gAi[off].y = (R)(0.5 * gFi.y);
    }
  }
}

// Step 2+3 on one self-conjugate plane kz: each mode pair (k, -k) by the thread of its lower index.
// Also records Re Gamma(0) of both slots (the mean subtraction makes F(0) = sum - NGRID).
template <typename R>
__global__ void __launch_bounds__(256) k_adj_plane(BinParams bp, BinTables t, const double *coef,
                                                   typename AdjC<R>::C *gA, typename AdjC<R>::C *gAi,
                                                   const double *dcv, int kz, double *gamma0) {
  const long long total = (long long)bp.nx * bp.ny;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q / bp.ny), j = (int)(q % bp.ny);
    const int i2 = (bp.nx - i) % bp.nx, j2 = (bp.ny - j) % bp.ny;
    const long long q2 = (long long)i2 * bp.ny + j2;
    if (q2 < q) continue;  // the partner's thread handles the pair
    double2 a, ai, b, bi;
    adj_gamma<R>(bp, t, coef, i, j, kz, gA, gAi, dcv, a, ai);
    if (kz == 0 && i == 0 && j == 0) {
      gamma0[0] = a.x;
      gamma0[1] = ai.x;
    }
    const long long off = ((long long)i * bp.ny + j) * bp.nzc + kz, off2 = ((long long)i2 * bp.ny + j2) * bp.nzc + kz;
    if (q2 == q) {  // self-conjugate mode: Phi = Re Gamma
      gA[off].x = (R)a.x;
      gA[off].y = (R)0;
      if (bp.interlace) {
        gAi[off].x = (R)ai.x;
        gAi[off].y = (R)0;
      }
      continue;
    }
    adj_gamma<R>(bp, t, coef, i2, j2, kz, gA, gAi, dcv, b, bi);
    const double2 p = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y));  // (Gamma(k) + conj Gamma(-k)) / 2
    gA[off].x = (R)p.x;
    gA[off].y = (R)p.y;
    gA[off2].x = (R)p.x;
    gA[off2].y = (R)(-p.y);
    if (bp.interlace) {
      const double2 pi = make_double2(0.5 * (ai.x + bi.x), 0.5 * (ai.y - bi.y));
      gAi[off].x = (R)pi.x;
      gAi[off].y = (R)pi.y;
      gAi[off2].x = (R)pi.x;
      gAi[off2].y = (R)(-pi.y);
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

// dL/d(particle) from the deposit's gradient sums: g0 = sum G W, gs = sum G dW/dscale per axis.
template <typename T>
__device__ __forceinline__ void adj_store(const Geom &g, const FieldSpec &fs, double v, double w, double g0,
                                          const double *gs, bool accepted, double dLdN, long long p, T *ox, T *oy,
                                          T *oz, T *ov, T *ow) {
  const int e = fs.ea;
  double ve = 1.0;
  for (int k = 0; k < e; k++) ve *= v;
  const double val = w * ve;  // deposit value w v^e (field A)
  const double dxr = val * gs[0] / g.dx, dyr = val * gs[1] / g.dy, dzr = val * gs[2] / g.dz;
  const double dw = ve * g0 + (accepted ? dLdN : 0.0);
  double dv = 0.0;
  if (e > 0) {
    double vm = 1.0;
    for (int k = 0; k < e - 1; k++) vm *= v;
    dv = w * (double)e * vm * g0;
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

// Step 4 for one particle by the exact FP64 rules: the transpose of its deposit (same taps, halo
// fold and dropped writes) read from dL/dgrid with the weight derivatives.
template <typename T, typename R>
__device__ __forceinline__ void adj_particle_exact(const Geom &g, const FieldSpec &fs, const PIn<T> &in, long long p,
                                                   const R *gA, const R *gAi, double dLdN, T *ox, T *oy, T *oz,
                                                   T *ov, T *ow) {
  double x = (double)in.x[p], y = (double)in.y[p], z = (double)in.z[p];
  const double v = fs.need_v ? (double)in.v[p] : 0.0, w = in.w ? (double)in.w[p] : 1.0;
  if (g.los == 1) x = rsd_shift64(g, x, v);
  else if (g.los == 2) y = rsd_shift64(g, y, v);
  else if (g.los == 3) z = rsd_shift64(g, z, v);
  double g0 = 0.0, gs[3] = {0.0, 0.0, 0.0};
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
      const R *gr = st ? gAi : gA;
      for (int c = 0; c < az.n; c++)
        for (int b = 0; b < ay.n; b++)
          for (int a = 0; a < ax.n; a++) {
            if (!(ax.on[a] && ay.on[b] && az.on[c])) continue;
            const long long L = canon_index(g, ax.idx[a], ay.idx[b], az.idx[c]);
            if (L < 0) continue;
            const double G = (double)gr[L];
            g0 += G * ax.w[a] * ay.w[b] * az.w[c];
            gs[0] += G * dx3[a] * ay.w[b] * az.w[c];
            gs[1] += G * ax.w[a] * dy3[b] * az.w[c];
            gs[2] += G * ax.w[a] * ay.w[b] * dz3[c];
          }
    }
  }
  adj_store(g, fs, v, w, g0, gs, accepted, dLdN, p, ox, oy, oz, ov, ow);
}

template <typename T, typename R>
__global__ void __launch_bounds__(128) k_adj_readout(Geom g, FieldSpec fs, PIn<T> in, long long n, const R *gA,
                                                     const R *gAi, double dLdN_host, const double *gamma0,
                                                     T *ox, T *oy, T *oz, T *ov, T *ow) {
  const double dLdN = dLdN_host - gamma0[0] - (g.interlace ? gamma0[1] : 0.0);
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x)
    adj_particle_exact<T, R>(g, fs, in, p, gA, gAi, dLdN, ox, oy, oz, ov, ow);
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

// Step 4 for FP32 contexts: particles away from every edge of the reference's rules gather their
// taps with the FP32 rules of the paint (the same ones that deposited them); the others take the
// exact FP64 path.
template <int K, typename T>
__global__ void __launch_bounds__(128) k_adj_readout32(Geom g, FieldSpec fs, PIn<T> in, long long n,
                                                       const float *gA, const float *gAi, double dLdN_host,
                                                       const double *gamma0, T *ox, T *oy, T *oz, T *ov, T *ow) {
  const double dLdN = dLdN_host - gamma0[0] - (g.interlace ? gamma0[1] : 0.0);
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const Prep pr = prep32(g, fs, in, p);
    if (!pr.fin || is_edge(g, pr.sx, pr.sy, pr.sz)) {
      adj_particle_exact<T, float>(g, fs, in, p, gA, gAi, dLdN, ox, oy, oz, ov, ow);
      continue;
    }
    float g0 = 0.0f, gs[3] = {0.0f, 0.0f, 0.0f};
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
      const float *gr = st ? gAi : gA;
#pragma unroll
      for (int a = 0; a < K; a++) {
        if (ax.idx[a] < 0) continue;
#pragma unroll
        for (int b = 0; b < K; b++) {
          if (ay.idx[b] < 0) continue;
          const long long rowb = ((long long)ax.idx[a] * g.ny + ay.idx[b]) * g.row;
#pragma unroll
          for (int c = 0; c < K; c++) {
            if (az.idx[c] < 0) continue;
            const float G = gr[rowb + az.idx[c]];
            const float wyz = ay.w[b] * az.w[c];
            g0 += G * ax.w[a] * wyz;
            gs[0] += G * dx3[a] * wyz;
            gs[1] += G * ax.w[a] * dy3[b] * az.w[c];
            gs[2] += G * ax.w[a] * ay.w[b] * dz3[c];
          }
        }
      }
    }
    const double gsd[3] = {(double)gs[0], (double)gs[1], (double)gs[2]};
    adj_store(g, fs, (double)pr.v, (double)pr.w, (double)g0, gsd, accepted, dLdN, p, ox, oy, oz, ov, ow);
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

extern "C" int capow_backward(capow_ctx *c, const double *const dL_dP[5], const capow_grads *out) {
  if (!c || !dL_dP || !out) return CAPOW_EINVAL;
  if (!c->powered) FAIL(c, CAPOW_ESTATE, "capow_backward needs capow_paint and capow_power first");
  if (c->fs.nfields != 1 || c->bp.nspec != 1 || !c->bp.mean_sub_a || c->fs.ea != 0)
    FAIL(c, CAPOW_ENOTSUP, "capow_backward covers the density auto-spectrum (Momentum 0 or spectra = DD)");
  if (out->dtype != CAPOW_F32 && out->dtype != CAPOW_F64) FAIL(c, CAPOW_EINVAL, "grads dtype must be F32 or F64");
  CK(c, cudaSetDevice(c->o.device));
  const capow_params &p = c->p;
  const int nk = p.NK;
  const long long n = (long long)c->last.n;
  // ---- host: per-bin coefficients c_l(b) = dL/dP_l(b) (2l+1) / (Nmodes(b) norm), and dL/dNGRID
  // through norm = NGRID^2 / V and shot = NGRID (src/main.c:106-148, 1019-1056)
  const DevStats &st = *c->h_st;
  const double N = st.ngrid;
  const double V = (p.XMAX - p.XMIN) * (p.YMAX - p.YMIN) * (p.ZMAX - p.ZMIN);
  const double norm = N * N / V;
  int last = -1;  // output_power zeroes the highest filled bin (its output does not depend on anything)
  for (int b = 0; b < nk; b++)
    if (c->nmodes[b] > 0) last = b;
  std::vector<double> coef(5 * nk, 0.0);
  double dLdN = 0.0;
  for (int b = 0; b < nk; b++) {
    const double nm = (double)c->nmodes[b];
    if (nm <= 0.0 || b == last || norm <= 0.0) continue;
    for (int l = 0; l < 5; l++) {
      if ((l == 1 || l == 3) && !p.Odd_Multipoles) continue;
      const double g = dL_dP[l] ? dL_dP[l][b] : 0.0;
      if (g == 0.0) continue;
      coef[l * nk + b] = g * (double)(2 * l + 1) / (nm * norm);
      const double S = c->h_bins[l * nk + b];  // raw sum of product 0 (|A|^2), multipole l
      const double P = l == 0 ? (S - nm * N) / (nm * norm) : (double)(2 * l + 1) * S / (nm * norm);
      const double dPdN = l == 0 ? -2.0 * P / N - V / (N * N) : -2.0 * P / N;
      dLdN += g * dPdN;
    }
  }
  if (!c->adj_coef) {
    CK(c, cudaMalloc(&c->adj_coef, sizeof(double) * 5 * nk + 2 * sizeof(double)));
  }
  double *coef_d = c->adj_coef, *gamma0 = c->adj_coef + 5 * nk;
  CK(c, cudaMemcpyAsync(coef_d, coef.data(), sizeof(double) * 5 * nk, cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaMemsetAsync(gamma0, 0, 2 * sizeof(double), c->stream));
  int rc = make_3d_plans(c);
  if (rc) return rc;
  // ---- forward again: paint, DC values, full 3-D transform
  rc = enqueue_backward_paint(c);
  if (rc) return rc;
  const bool f64 = c->prec == CAPOW_FP64;
  if (f64) CKFFT(c, cufftExecD2Z(c->adj_fwd, (cufftDoubleReal *)c->grid_base, (cufftDoubleComplex *)c->grid_base));
  else CKFFT(c, cufftExecR2C(c->adj_fwd, (cufftReal *)c->grid_base, (cufftComplex *)c->grid_base));
  // ---- mode gradients and Hermitian completion, then the inverse transform
  const size_t eb = f64 ? 8 : 4;
  void *gA = c->grid_base, *gAi = p.DoInterlacing ? (char *)c->grid_base + eb * c->grid_elems : nullptr;
  const int nyq = (p.NZ % 2 == 0) ? p.NZ / 2 : -1;
  const int kz_hi = nyq > 0 ? nyq : c->bp.nzc;
  const long long interior = (long long)p.NX * p.NY * (kz_hi - 1 > 0 ? kz_hi - 1 : 0);
  const int nbm = adj_blocks(interior), nbp = adj_blocks((long long)p.NX * p.NY);
  if (f64) {
    k_adj_modes<double><<<nbm, 256, 0, c->stream>>>(c->bp, c->bt, coef_d, (double2 *)gA, (double2 *)gAi, c->dcv, 1, kz_hi);
    k_adj_plane<double><<<nbp, 256, 0, c->stream>>>(c->bp, c->bt, coef_d, (double2 *)gA, (double2 *)gAi, c->dcv, 0, gamma0);
    if (nyq > 0)
      k_adj_plane<double><<<nbp, 256, 0, c->stream>>>(c->bp, c->bt, coef_d, (double2 *)gA, (double2 *)gAi, c->dcv, nyq,
                                                      gamma0);
    CKFFT(c, cufftExecZ2D(c->adj_inv, (cufftDoubleComplex *)c->grid_base, (cufftDoubleReal *)c->grid_base));
  } else {
    k_adj_modes<float><<<nbm, 256, 0, c->stream>>>(c->bp, c->bt, coef_d, (float2 *)gA, (float2 *)gAi, c->dcv, 1, kz_hi);
    k_adj_plane<float><<<nbp, 256, 0, c->stream>>>(c->bp, c->bt, coef_d, (float2 *)gA, (float2 *)gAi, c->dcv, 0, gamma0);
    if (nyq > 0)
      k_adj_plane<float><<<nbp, 256, 0, c->stream>>>(c->bp, c->bt, coef_d, (float2 *)gA, (float2 *)gAi, c->dcv, nyq,
                                                     gamma0);
    CKFFT(c, cufftExecC2R(c->adj_inv, (cufftComplex *)c->grid_base, (cufftReal *)c->grid_base));
  }
  c->launches += nyq > 0 ? 3 : 2;
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
  const capow_particles &d = c->last;
  const int nb = (int)((n + 127) / 128 > 152 * 16 ? 152 * 16 : ((n + 127) / 128 < 1 ? 1 : (n + 127) / 128));
#define ADJ_IN(TI) \
  PIn<TI> { (const TI *)d.x, (const TI *)d.y, (const TI *)d.z, (const TI *)d.vlos, (const TI *)d.w }
#define ADJ_OUT(TO) (TO *)dev[0], (TO *)dev[1], (TO *)dev[2], (TO *)dev[3], (TO *)dev[4]
#define ADJ_RUN64(T) \
  k_adj_readout<T, double><<<nb, 128, 0, c->stream>>>(c->g, c->fs, ADJ_IN(T), n, (const double *)gA, \
                                                      (const double *)gAi, dLdN, gamma0, ADJ_OUT(T))
#define ADJ_RUN32(K, T) \
  k_adj_readout32<K, T><<<nb, 128, 0, c->stream>>>(c->g, c->fs, ADJ_IN(T), n, (const float *)gA, \
                                                   (const float *)gAi, dLdN, gamma0, ADJ_OUT(T))
  if (d.dtype != out->dtype)
    FAIL(c, CAPOW_EINVAL, "capow_backward: gradient dtype must match the painted particles' dtype");
  if (f64) {
    if (d.dtype == CAPOW_F64) ADJ_RUN64(double);
    else ADJ_RUN64(float);
  } else if (d.dtype == CAPOW_F64) {
    if (p.InterpOrder == 3) ADJ_RUN32(3, double);
    else if (p.InterpOrder == 2) ADJ_RUN32(2, double);
    else ADJ_RUN32(1, double);
  } else {
    if (p.InterpOrder == 3) ADJ_RUN32(3, float);
    else if (p.InterpOrder == 2) ADJ_RUN32(2, float);
    else ADJ_RUN32(1, float);
  }
#undef ADJ_IN
#undef ADJ_OUT
#undef ADJ_RUN64
#undef ADJ_RUN32
  c->launches++;
  CK(c, cudaGetLastError());
  if (!out->on_device)
    for (int k = 0; k < 5; k++)
      if (dst[k]) CK(c, cudaMemcpyAsync(dst[k], dev[k], ob * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  c->powered = true;  // the grids hold dL/dgrid now: a new paint is needed before capow_power
  return CAPOW_OK;
}
