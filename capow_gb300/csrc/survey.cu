// Survey-mode estimator (Periodic 0, Survey 1; Momentum 0 to 3) on one GB300: the C ABI's capow_survey_*.
//
// Reference semantics (single rank; paths relative to the CAPOW source tree):
//   src/read_data.c:450-466  compute_fkp: the FKP weights of the density (Momentum 0), of the velocities
//                            (Momentum 1: 1/((pverr^2 + 300^2) + nbar FKP_Pk_mom)) or both with their
//                            cross factor (Momentum 2, 3: weight and weight_pv), stored in float fields
//   src/main.c:149-204       sums over data and randoms, alpha, shot, norm
//   src/read_data.c:471-494  assign_survey_data: the density of data (prefactor 1) and randoms (-alpha);
//                            Momentum 1: the data's w pv only; Momentum 2, 3: also the data's w_pv pv into
//                            the momentum grid; each object and its copy shifted by half a cell
//   src/read_data.c:514-745  add_to_grid's Survey branches: no wrap; a neighbour that reaches the axis
//                            limit pulls the stencil back by one cell (:577-590, :672-688); the halo
//                            slices past NX are discarded (no neighbour rank, src/main.c:1162-1188)
//   src/main.c:472-775       compute_survey_power: the grids times products of the unit vector r^ from
//                            the observer to every cell corner, one FFT per product (and per grid)
//   src/main.c:781-967       assign_survey_power: interlacing combine, deconvolution, the products'
//                            k^ factors, crossed with F0 (and F0_mom) and binned
//
// Multipoles through solid harmonics. For a unit k^, the reference builds
//   F_l(k) = sum_r L_l(k^.r^) f(r) e^{-ik.r}
// from the Cartesian products r^_i r^_j ... (1, 3, 6, 10, 15 FFTs for l = 0..4). By the addition
// theorem L_l(k^.u) = sum_m c_lm h_lm(k^) h_lm(u) with h_lm the 2l+1 real harmonic polynomials of
// degree l (below), so F_l = sum_m c_lm h_lm(k^) FFT[h_lm(r^) f] takes 1, 3, 5, 7, 9 FFTs. The two
// forms agree on every cell with |r^| = 1. The cell whose corner is the observer (r2 == 0, where the
// reference sets r2 = 1 and all its products vanish) enters the reference's P2 and P4 through the
// constant terms of L_2 and L_4 only: L_l(0) f_o e^{-ik.r_o}, added here in closed form. At k = 0 the
// reference skips every l > 0 product. For the density (and Momentum 1) P_l = sum Re or Im(F_l conj F0),
// and the constant terms of L_2 and L_4 at the other cells cancel against its l = 0 bins except at
// k = 0. For the cross spectra (Momentum 2, 3) each product enters as half the sum of its density
// against F0_mom and its momentum against F0, and that symmetric form of F0 against F0_mom vanishes, so
// the reference's l = 0 terms -0.5 X0 and +0.375 X0 (X0 = its monopole power) stay in P2 and P4 at every
// mode; the l = 0 pass adds them.
#include <cuda_runtime.h>
#include <cufft.h>
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <new>
#include <type_traits>
#include <vector>

#include "ctx.cuh"
#include "harm.cuh"

// ------------------------------------------------------------------------------------ device state
struct SvStats {
  double wsum[2], w2sum[2], w2nsum[2];  // [0] data, [1] randoms: sum w, w^2, w^2 nbar (src/main.c:151-163)
  double vr, vrsq;                      // data: sum w w_pv pv, w^2 pv^2 (Momentum 1-3)
  double w2npv[2];                      // sum w_pv^2 nbar: data (Momentum 1-3), randoms (Momentum 2)
  double ngrid[2];                      // assign_survey_data's NGRID (src/read_data.c:474-491)
  double dc[4];                         // FP64 sum of the deposits reaching the FFT input, per grid slot
  int nonfinite;                        // a non-finite coordinate, weight, number density or velocity
  int pad;
};

// Catalogue arrays on the device. pv, pverr are null for Momentum 0.
template <typename T>
struct SvIn {
  const T *x, *y, *z, *w, *nbar, *pv, *pverr;
};

// Grid slot of (stencil, field): stencil 0 normal, 1 interlaced; field 0 density, 1 momentum (Momentum 2, 3).
// The periodic path's order, so that the FP32 paint context's grids are the survey's slots.
__host__ __device__ __forceinline__ int sv_slot(int stencil, int field, int nf) { return stencil * nf + field; }

static double harm_coef(int l, int m) {
  static const double c1[3] = {1, 1, 1};
  static const double c2[5] = {3, 3, 3, 0.75, 0.25};
  static const double c3[7] = {0.625, 0.625, 3.75, 15, 0.375, 0.375, 0.25};
  static const double c4[9] = {8.75, 35.0 / 64.0, 4.375, 4.375, 1.25, 0.3125, 0.625, 0.625, 1.0 / 64.0};
  const double *c[5] = {nullptr, c1, c2, c3, c4};
  return l == 0 ? 1.0 : c[l][m];
}

// -------------------------------------------------------------------------- paint (exact FP64 rules)
// exact_axes (common.cuh) applies add_to_grid's Survey branches when Geom.survey is set: acceptance as for a
// periodic run with LOS != 0, and the stencil pulled back one cell where its upper neighbour reaches the
// axis limit (src/read_data.c:577-590, 672-688). NN has no Survey branch.

// Linear index of a write (src/read_data.c:536 form) that reaches the FFT input, else -1: the halo
// slices are discarded, the padding columns are not read by the transform, and an index the
// reference would place before the grid (NY or NZ below 3 with a pulled-back TSC stencil) is dropped.
__device__ __forceinline__ long long sv_index(const Geom &g, int ix, int iy, int iz) {
  if (ix < 0 || iy < 0 || iz < 0 || iz >= g.nz) return -1;
  const unsigned long long L =
      (unsigned long long)iz + (unsigned long long)g.row * ((unsigned long long)iy + (unsigned long long)g.ny * (unsigned long long)ix);
  return L < (unsigned long long)g.main_sz ? (long long)L : -1;
}

template <typename R>
__device__ __forceinline__ double sv_deposit(const Geom &g, R *grid, double wv, const AxisTaps &ax,
                                             const AxisTaps &ay, const AxisTaps &az) {
  double s = 0.0;
  for (int c = 0; c < az.n; c++) {
    if (!az.on[c]) continue;
    for (int b = 0; b < ay.n; b++) {
      if (!ay.on[b]) continue;
      for (int a = 0; a < ax.n; a++) {
        if (!ax.on[a]) continue;
        const long long L = sv_index(g, ax.idx[a], ay.idx[b], az.idx[c]);
        if (L < 0) continue;
        const double d = DMUL(DMUL(DMUL(wv, ax.w[a]), ay.w[b]), az.w[c]);
        atomicAdd(grid + L, (R)d);
        s += d;
      }
    }
  }
  return s;
}

__device__ __forceinline__ double sv_warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum NV per-thread doubles over the block and add them to global dst (one atomic per value and block).
template <int NV>
__device__ void sv_block_add(const double (&v)[NV], double *const (&dst)[NV]) {
  __shared__ double red[32][NV];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  double t[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) t[k] = sv_warp_sum(v[k]);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; k++) red[wid][k] = t[k];
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) {
      double a = lane < nw ? red[lane][k] : 0.0;
      a = sv_warp_sum(a);
      if (lane == 0 && a != 0.0) atomicAdd(dst[k], a);
    }
  }
  __syncthreads();
}

__device__ __forceinline__ float sv_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double sv_mul(double a, double b) { return __dmul_rn(a, b); }

// compute_fkp (src/read_data.c:450-466) and the weight sums (src/main.c:151-163) of one catalogue. The FKP
// factors in double, the weights stored back in the catalogue's type (float for the reference's struct):
//   Momentum 0: w *= 1/(1 + nbar FKP_Pk);
//   Momentum 1: w *= 1/((pverr^2 + 300^2) + nbar FKP_Pk_mom), pverr^2 in the catalogue's type;
//   Momentum 2, 3: with t = 1/(1 + nbar FKP_Pk), t_pv the Momentum 1 factor and the cross factor
//     t_c = 1/sqrt(1 + t t_pv nbar nbar FKP_Pk_cross FKP_Pk_cross): w_pv = w t_pv t_c, w = w (t t_c).
// The sums' products are in the catalogue's type, summed in double. which: 0 data, 1 randoms.
template <typename T>
__global__ void __launch_bounds__(256) k_sv_prepare(SvIn<T> in, long long n, int fkp, int mom, double pk, double pk_mom,
                                                    double pk_cross, T *wout, T *wpvout, SvStats *st, int which) {
  double s[6] = {0, 0, 0, 0, 0, 0};  // w, w^2, w^2 nbar, w w_pv pv, w^2 pv^2, w_pv^2 nbar
  int bad = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    T w = in.w[i], wpv = (T)0;
    const T nb = in.nbar[i];
    const T pe = mom ? in.pverr[i] : (T)0;
    if (fkp) {
      const double nbd = (double)nb;
      if (mom == 0) {
        w = (T)__dmul_rn((double)w, __ddiv_rn(1.0, __dadd_rn(1.0, __dmul_rn(nbd, pk))));
      } else {
        const double tpv = __ddiv_rn(1.0, __dadd_rn(__dadd_rn((double)sv_mul(pe, pe), 90000.0), __dmul_rn(nbd, pk_mom)));
        if (mom == 1) {
          w = (T)__dmul_rn((double)w, tpv);
        } else {
          const double tw = __ddiv_rn(1.0, __dadd_rn(1.0, __dmul_rn(nbd, pk)));
          const double q = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(tw, tpv), nbd), nbd), pk_cross), pk_cross);
          const double tc = __ddiv_rn(1.0, __dsqrt_rn(__dadd_rn(1.0, q)));
          wpv = (T)__dmul_rn(__dmul_rn((double)w, tpv), tc);
          w = (T)__dmul_rn((double)w, __dmul_rn(tw, tc));
          wpvout[i] = wpv;
        }
      }
      wout[i] = w;
    }
    if (!isfinite((double)w) || !isfinite((double)nb) || !isfinite((double)pe)) bad = 1;
    const T ww = sv_mul(w, w);
    s[0] += (double)w;
    s[1] += (double)ww;
    s[2] += (double)sv_mul(ww, nb);
    if (mom && which == 0) {
      const T pv = in.pv[i];
      if (!isfinite((double)pv)) bad = 1;
      s[3] += (double)sv_mul(sv_mul(w, wpv), pv);
      s[4] += (double)sv_mul(sv_mul(ww, pv), pv);
      s[5] += (double)sv_mul(sv_mul(wpv, wpv), nb);
    } else if (mom == 2 && which == 1) {
      s[5] += (double)sv_mul(sv_mul(wpv, wpv), nb);
    }
  }
  double *const dst[6] = {&st->wsum[which], &st->w2sum[which], &st->w2nsum[which], &st->vr, &st->vrsq,
                          &st->w2npv[which]};
  if (which == 0) {
    sv_block_add<6>(s, dst);
  } else {
    const double v[4] = {s[0], s[1], s[2], s[5]};
    double *const d4[4] = {dst[0], dst[1], dst[2], dst[5]};
    sv_block_add<4>(v, d4);
  }
  if (bad) atomicOr(&st->nonfinite, 1);
}

// Grid pointers of a survey paint: the slots of sv_slot.
template <typename R>
struct SvGrids {
  R *g[4];
};

// assign_survey_data (src/read_data.c:471-494), FP64: each object and, half a cell up, its interlaced copy.
// Momentum 1 (data only): w pv into the density slots, NGRID += add_to_grid / (pv w) (a product in the
// catalogue's type). Otherwise prefactor w into the density slots, NGRID += add_to_grid / w, and for the
// data of Momentum 2, 3 also w_pv pv into the momentum slots. The randoms' prefactor is -alpha =
// -(sum w_data / sum w_rand) (src/main.c:169, 229), read from the sums on the device.
template <typename T, typename R>
__global__ void __launch_bounds__(256) k_sv_paint(Geom g, SvIn<T> in, const T *wk, const T *wpv, long long n, int which,
                                                  int mom, int nf, SvGrids<R> gr, SvStats *st) {
  const double pref = which ? -__ddiv_rn(st->wsum[0], st->wsum[1]) : 1.0;
  double l_ngrid = 0.0, l_dc[4] = {0, 0, 0, 0};
  int bad = 0;
  const int sd0 = sv_slot(0, 0, nf), sd1 = sv_slot(1, 0, nf), sm0 = sv_slot(0, 1, nf), sm1 = sv_slot(1, 1, nf);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double x = (double)in.x[i], y = (double)in.y[i], z = (double)in.z[i], w = (double)wk[i];
    if (!(isfinite(x) && isfinite(y) && isfinite(z))) {
      bad = 1;
      continue;
    }
    double dval, got = 0.0;  // the density slots' deposit value (add_to_grid's w * vr)
    double div;
    if (mom == 1) {
      dval = __dmul_rn(w, __dmul_rn(pref, (double)in.pv[i]));
      div = (double)sv_mul(in.pv[i], wk[i]);
    } else {
      dval = __dmul_rn(pref, w);
      div = w;
    }
    const bool mfield = mom >= 2 && which == 0;
    const double mval = mfield ? __dmul_rn((double)wpv[i], __dmul_rn(pref, (double)in.pv[i])) : 0.0;
    AxisTaps ax, ay, az;
    if (exact_axes(g, x, y, z, ax, ay, az)) {
      l_dc[sd0] += sv_deposit(g, gr.g[sd0], dval, ax, ay, az);
      if (mfield) l_dc[sm0] += sv_deposit(g, gr.g[sm0], mval, ax, ay, az);
      got = mom == 1 ? w : dval;
    }
    l_ngrid += __ddiv_rn(got, div);
    if (g.interlace && exact_axes(g, DADD(x, g.hx), DADD(y, g.hy), DADD(z, g.hz), ax, ay, az)) {
      l_dc[sd1] += sv_deposit(g, gr.g[sd1], dval, ax, ay, az);
      if (mfield) l_dc[sm1] += sv_deposit(g, gr.g[sm1], mval, ax, ay, az);
    }
  }
  const double v[5] = {l_ngrid, l_dc[0], l_dc[1], l_dc[2], l_dc[3]};
  double *const dst[5] = {&st->ngrid[which], &st->dc[0], &st->dc[1], &st->dc[2], &st->dc[3]};
  sv_block_add<5>(v, dst);
  if (bad) atomicOr(&st->nonfinite, 1);
}

// The FP32 paint takes data and randoms as one catalogue for the tile kernels: this writes object i of one
// catalogue at off + i of the combined float arrays with the weight of its density deposit (prefactor w;
// Momentum 1: w pv) and, for Momentum 2, 3, the v with w v = w_pv pv (the tile kernels' second field is
// w v; 0 for randoms), and adds its assign_survey_data counter (acceptance only, no taps).
template <typename T>
__global__ void __launch_bounds__(256) k_sv_combine(Geom g, SvIn<T> in, const T *wk, const T *wpv, long long n,
                                                    int which, int mom, long long off, float *cx, float *cy, float *cz,
                                                    float *cw, float *cv, SvStats *st) {
  const double pref = which ? -__ddiv_rn(st->wsum[0], st->wsum[1]) : 1.0;
  double l_ngrid = 0.0;
  int bad = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double x = (double)in.x[i], y = (double)in.y[i], z = (double)in.z[i], w = (double)wk[i];
    if (!(isfinite(x) && isfinite(y) && isfinite(z))) bad = 1;
    const bool acc = g.order == 1 ? !((x < g.xmin) || (x >= g.xmax_l) || (y < g.ymin) || (y >= g.ymax) ||
                                      (z < g.zmin) || (z >= g.zmax))
                                  : (survey_accept_axis(g, 0, x) && survey_accept_axis(g, 1, y) &&
                                     survey_accept_axis(g, 2, z));
    double wp;
    if (mom == 1) {
      wp = __dmul_rn(w, (double)in.pv[i]);
      l_ngrid += __ddiv_rn(acc ? w : 0.0, (double)sv_mul(in.pv[i], wk[i]));
    } else {
      wp = __dmul_rn(pref, w);
      // the counter's term (pref w) / w is pref to the last ulp (the sum agrees to ~1e-16); only w == 0
      // takes the quotient, whose 0 / 0 is the reference's NaN (and a rejected object's 0 / 0 too)
      if (w != 0.0) l_ngrid += acc ? pref : 0.0;
      else l_ngrid += __ddiv_rn(acc ? wp : 0.0, w);
    }
    cx[off + i] = (float)x;
    cy[off + i] = (float)y;
    cz[off + i] = (float)z;
    cw[off + i] = (float)wp;
    if (mom >= 2) {
      const double mv = which == 0 ? __dmul_rn((double)wpv[i], (double)in.pv[i]) : 0.0;
      cv[off + i] = (wp != 0.0) ? (float)__ddiv_rn(mv, wp) : 0.0f;
    }
  }
  const double v[1] = {l_ngrid};
  double *const dst[1] = {&st->ngrid[which]};
  sv_block_add<1>(v, dst);
  if (bad) atomicOr(&st->nonfinite, 1);
}

// ------------------------------------------------------------------------ weighted term grids
// w[c] = a[c] h_lm(r^) for every cell c = (ix, iy, iz < NZ) of a painted grid (and its interlaced copy),
// r^ the unit vector from the observer to the cell corner (ix dx + XMIN - X_Origin, ...) (src/main.c:551-559
// and the other product loops). A corner at the observer (r2 == 0) gets r2 = 1, as in the reference, so its
// harmonics vanish. l = 0 copies the grid (src/main.c:503-511). One warp per (x, y) row, grid-stride over
// rows; each lane moves z pairs (rows have an even length, so pairs are aligned vector loads).
template <typename R>
__global__ void __launch_bounds__(256) k_sv_weight(const R *a0, const R *a1, R *w0, R *w1, const R *vx, const R *vy,
                                                   const R *vz, int nx, int ny, int nz, long long row, int l, int m) {
  typedef typename std::conditional<sizeof(R) == 4, float2, double2>::type R2;
  const int lane = threadIdx.x & 31;
  const long long nrows = (long long)nx * ny;
  const int npairs = (nz + 1) >> 1;
  const long long wstride = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long r = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; r < nrows; r += wstride) {
    const int ix = (int)(r / ny), iy = (int)(r - (long long)ix * ny);
    const R px = vx[ix], py = vy[iy];
    const R pxy = px * px + py * py;
    const R2 *s0 = reinterpret_cast<const R2 *>(a0 + r * row);
    const R2 *s1 = a1 ? reinterpret_cast<const R2 *>(a1 + r * row) : nullptr;
    R2 *d0 = reinterpret_cast<R2 *>(w0 + r * row);
    R2 *d1 = a1 ? reinterpret_cast<R2 *>(w1 + r * row) : nullptr;
    for (int p = lane; p < npairs; p += 32) {
      R h0 = (R)1, h1 = (R)1;
      if (l > 0) {
        h0 = sv_cell_weight<R>(l, m, px, py, pxy, vz[2 * p]);
        h1 = 2 * p + 1 < nz ? sv_cell_weight<R>(l, m, px, py, pxy, vz[2 * p + 1]) : (R)0;
      }
      R2 v = s0[p];
      v.x *= h0;
      v.y *= h1;
      d0[p] = v;
      if (s1) {
        R2 u = s1[p];
        u.x *= h0;
        u.y *= h1;
        d1[p] = u;
      }
    }
  }
}

// -------------------------------------------------------------------------------------- binning
template <typename R>
struct SvC;
template <>
struct SvC<float> {
  typedef float2 C;
};
template <>
struct SvC<double> {
  typedef double2 C;
};

// What one assign pass needs beyond the periodic tables.
template <typename R>
struct SvAssign {
  typedef typename SvC<R>::C C;
  const C *gd0, *gd1;   // transformed density term grid(s) [NX][NY][NZ/2+1]: normal, interlaced
  const C *gm0, *gm1;   // the momentum term grids (Momentum 2, 3)
  C *F0, *F0m;          // monopole fields (the l = 0 pass writes them)
  const double *dc;     // exact DC of each painted slot: the l = 0 pass's k = 0 mode
  int sd0, sd1, sm0, sm1;  // slots of dc and of the painted grids
  R coef;               // c_lm
  int m;
  // the observer's cell (l = 0 pass only): painted values there and e^{-2 pi i q o/N} per axis
  int origin;
  const R *a[4];        // painted grids by slot
  long long oind;
  const C *ox, *oy, *oz;
};

constexpr int SV_ICHUNK = 128;

template <typename C, typename R>
__device__ __forceinline__ R sv_imf(const C &a, const C &b) { return a.x * b.y - a.y * b.x; }
template <typename C, typename R>
__device__ __forceinline__ R sv_ref(const C &a, const C &b) { return a.x * b.x + a.y * b.y; }

// assign_survey_power (src/main.c:781-967) for one FFT set; the power forms of :870-887. w = NM times the
// deconvolution (times 0.25 when interlacing, :890-899).
//  Density (CROSS false). L = 0: F0 = the interlacing-combined field, P0 += w |F0|^2; at k = 0 also
//   P2 += L_2(0) w |F0|^2, P4 += L_4(0) w |F0|^2; elsewhere the observer cell's closed-form term.
//   L > 0: P_L += w c_lm h_lm(k^) X.F0 for k != 0, X.F0 = Re(X conj F0) for even L, dkr F0i - dki F0r
//   for odd L.
//  Cross (Momentum 2, 3). L = 0: F0, F0m = the combined density and momentum fields, X0 = Im(conj F0 F0m),
//   P0 += w X0, P2 -= 0.5 w X0, P4 += 0.375 w X0 at every mode, and the observer cell's term.
//   L > 0: P_L += w c_lm h_lm(k^) (G_d.F0m + G_m.F0) / 2, with the Re form for odd L and the Im form
//   (a.r b.i - a.i b.r) for even L.
// One thread per (ky, kz) column walks x over a chunk of SV_ICHUNK; bin sums run per thread over equal-bin
// stretches, then per CTA in shared memory, then FP64 global atomics. Modes beyond the top bin edge are
// skipped as in k_bin.
template <typename R, int L, bool CROSS, bool TR>
__global__ void __launch_bounds__(256) k_sv_assign(BinParams bp, BinTables t, SvAssign<R> sa, double *bins) {
  typedef typename SvC<R>::C C;
  constexpr bool F32 = sizeof(R) == 4;
  const int nk = bp.nk;
  __shared__ R sb[3 * 512];  // [3][nk] (L = 0: P0, P2, P4; else one row)
  __shared__ double sE[515];
  __shared__ float sElo[515], sEhi[515];
  __shared__ R sfx2[SV_ICHUNK], scx[SV_ICHUNK], sfx[SV_ICHUNK];
  __shared__ C sex[SV_ICHUNK], sox[SV_ICHUNK];
  const int i0 = blockIdx.y * SV_ICHUNK, i1 = min(bp.nx, i0 + SV_ICHUNK);
  for (int c = threadIdx.x; c < 3 * nk; c += blockDim.x) sb[c] = (R)0;
  for (int c = threadIdx.x; c < nk + 3; c += blockDim.x) {
    sE[c] = t.E[c];
    sElo[c] = t.Elo[c];
    sEhi[c] = t.Ehi[c];
  }
  for (int c = threadIdx.x; c < i1 - i0; c += blockDim.x) {
    const int i = i0 + c;
    if (F32) {
      sfx2[c] = (R)t.fx2f[i];
      scx[c] = (R)t.cxf[i];
      sfx[c] = (R)t.fxf[i];
      sex[c].x = (R)t.exf[i].x;
      sex[c].y = (R)t.exf[i].y;
    } else {
      sfx2[c] = (R)t.fx2d[i];
      scx[c] = (R)t.cxd[i];
      sfx[c] = (R)t.fxd[i];
      sex[c].x = (R)t.exd[i].x;
      sex[c].y = (R)t.exd[i].y;
    }
    if (L == 0 && sa.origin) sox[c] = sa.ox[i];
  }
  __syncthreads();
  const long long cols = (long long)bp.ny * bp.nzc;
  const long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (col < cols) {
    // the column (ky, kz): [NX][NY][NZ/2+1] grids, or TR: the transposed [NX][NZ/2+1][NY] of the z-pass path
    const int j = TR ? (int)(col % bp.ny) : (int)(col / bp.nzc);
    const int k = TR ? (int)(col / bp.ny) : (int)(col - (long long)j * bp.nzc);
    const R syz = F32 ? (R)(t.fy2f[j] + t.fz2f[k]) : (R)0;
    const double fy2 = t.fy2d[j], fz2 = t.fz2d[k];
    R cyz = F32 ? (R)(t.cyf[j] * t.czf[k]) : (R)(t.cyd[j] * t.czd[k]);
    if (bp.interlace) cyz *= (R)0.25;
    C eyz;
    if (F32) {
      const float2 a = t.eyf[j], b = t.ezf[k];
      eyz.x = a.x * b.x - a.y * b.y;
      eyz.y = a.x * b.y + a.y * b.x;
    } else {
      const double2 a = t.eyd[j], b = t.ezd[k];
      eyz.x = a.x * b.x - a.y * b.y;
      eyz.y = a.x * b.y + a.y * b.x;
    }
    const R fy = F32 ? (R)t.fyf[j] : (R)t.fyd[j], fz = F32 ? (R)t.fzf[k] : (R)t.fzd[k];
    C oyz;
    R od0 = (R)0, od1 = (R)0, om0 = (R)0, om1 = (R)0;  // painted values at the observer's cell
    oyz.x = oyz.y = (R)0;
    if (L == 0 && sa.origin) {
      const C a = sa.oy[j], b = sa.oz[k];
      oyz.x = a.x * b.x - a.y * b.y;
      oyz.y = a.x * b.y + a.y * b.x;
      od0 = sa.a[sa.sd0][sa.oind];
      if (bp.interlace) od1 = sa.a[sa.sd1][sa.oind];
      if (CROSS) {
        om0 = sa.a[sa.sm0][sa.oind];
        if (bp.interlace) om1 = sa.a[sa.sm1][sa.oind];
      }
    }
    const long long base = TR ? (long long)k * bp.ny + j : (long long)j * bp.nzc + k;
    R acc0 = (R)0, acc2 = (R)0, acc4 = (R)0;
    int cur = -1;
    R lo = (R)1, hi = (R)0;
    const float top = sElo[nk + 1] - (float)(F32 ? (float)syz : (float)(fy2 + fz2));
    const int rr = top > 0.0f ? min(bp.xhalf, (int)(sqrtf(top) / bp.fx_step) + 1) : -1;
    for (int i = i0; i < i1; i++) {
      if (i > rr && i < bp.nx - rr) {
        i = bp.nx - rr - 1;
        continue;
      }
      const int li = i - i0;
      R s;
      if (F32) s = sfx2[li] + syz;
      else s = (R)__dadd_rn(__dadd_rn((double)sfx2[li], fy2), fz2);
      if (!(s >= lo && s < hi)) {
        int b = cur < -1 ? -1 : cur;
        if (F32) {
          const float sf = (float)s;
          while (b < nk && sf >= sElo[b + 2]) b++;
          while (b > -1 && sf < sEhi[b + 1]) b--;
          if (sf >= sElo[b + 1] && sf < sEhi[b + 2]) {
            lo = (R)sElo[b + 1];
            hi = (R)sEhi[b + 2];
          } else {  // within a few ulps of an edge: the exact FP64 s decides
            b = exact_bin(sE, nk, __dadd_rn(__dadd_rn(t.fx2d[i], fy2), fz2), b);
            lo = (R)1;
            hi = (R)0;
          }
        } else {
          b = exact_bin(sE, nk, (double)s, b);
          lo = (R)sE[b + 1];
          hi = (R)sE[b + 2];
        }
        if (b != cur) {
          if (cur >= 0 && cur < nk) {
            if (L == 0) {
              if (acc0 != (R)0) atomicAdd(&sb[cur], acc0);
              if (acc2 != (R)0) atomicAdd(&sb[nk + cur], acc2);
              if (acc4 != (R)0) atomicAdd(&sb[2 * nk + cur], acc4);
            } else if (acc0 != (R)0) {
              atomicAdd(&sb[cur], acc0);
            }
            acc0 = acc2 = acc4 = (R)0;
          }
          cur = b;
        }
      }
      if (cur < 0 || cur >= nk) continue;
      const bool kzero = (i == 0 && col == 0);
      if (L > 0 && kzero) continue;
      const long long off = (long long)i * cols + base;
      const C ex = sex[li];
      C e;
      e.x = ex.x * eyz.x - ex.y * eyz.y;
      e.y = ex.x * eyz.y + ex.y * eyz.x;
      C X = sa.gd0[off], M;
      M.x = M.y = (R)0;
      if (L == 0 && kzero) {
        X.x = (R)sa.dc[sa.sd0];
        X.y = (R)0;
      }
      if (CROSS) {
        M = sa.gm0[off];
        if (L == 0 && kzero) {
          M.x = (R)sa.dc[sa.sm0];
          M.y = (R)0;
        }
      }
      if (bp.interlace) {
        C a = sa.gd1[off];
        if (L == 0 && kzero) {
          a.x = (R)sa.dc[sa.sd1];
          a.y = (R)0;
        }
        X.x += a.x * e.x - a.y * e.y;
        X.y += a.x * e.y + a.y * e.x;
        if (CROSS) {
          C b = sa.gm1[off];
          if (L == 0 && kzero) {
            b.x = (R)sa.dc[sa.sm1];
            b.y = (R)0;
          }
          M.x += b.x * e.x - b.y * e.y;
          M.y += b.x * e.y + b.y * e.x;
        }
      }
      const R gc = cyz * scx[li] * (R)herm_nm(i, j, k, bp.xhalf);
      if (L == 0) {
        sa.F0[off] = X;
        if (CROSS) sa.F0m[off] = M;
        // the observer cell's closed-form field, O = (f_o + e f_o,interlaced) e^{-i k.r_o}
        C q;
        q.x = q.y = (R)0;
        if (sa.origin && !kzero) {
          const C ph = sox[li];
          q.x = ph.x * oyz.x - ph.y * oyz.y;
          q.y = ph.x * oyz.y + ph.y * oyz.x;
        }
        if (!CROSS) {
          const R p = (X.x * X.x + X.y * X.y) * gc;
          acc0 += p;
          if (kzero) {
            acc2 += (R)-0.5 * p;
            acc4 += (R)0.375 * p;
          } else if (sa.origin) {
            C O;
            O.x = (od0 + od1 * e.x) * q.x - (od1 * e.y) * q.y;
            O.y = (od0 + od1 * e.x) * q.y + (od1 * e.y) * q.x;
            const R pc = sv_ref<C, R>(O, X) * gc;
            acc2 += (R)-0.5 * pc;
            acc4 += (R)0.375 * pc;
          }
        } else {
          const R x0 = sv_imf<C, R>(X, M) * gc;
          acc0 += x0;
          acc2 += (R)-0.5 * x0;
          acc4 += (R)0.375 * x0;
          if (sa.origin && !kzero) {
            C Od, Om;
            Od.x = (od0 + od1 * e.x) * q.x - (od1 * e.y) * q.y;
            Od.y = (od0 + od1 * e.x) * q.y + (od1 * e.y) * q.x;
            Om.x = (om0 + om1 * e.x) * q.x - (om1 * e.y) * q.y;
            Om.y = (om0 + om1 * e.x) * q.y + (om1 * e.y) * q.x;
            const R pc = (R)0.5 * (sv_imf<C, R>(Od, M) + sv_imf<C, R>(Om, X)) * gc;
            acc2 += (R)-0.5 * pc;
            acc4 += (R)0.375 * pc;
          }
        }
      } else {
        R v;
        if (!CROSS) {
          const C F = sa.F0[off];
          v = (L & 1) ? sv_imf<C, R>(X, F) : sv_ref<C, R>(X, F);
        } else {
          const C F = sa.F0[off], Fm = sa.F0m[off];
          v = (L & 1) ? (R)0.5 * (sv_ref<C, R>(X, Fm) + sv_ref<C, R>(M, F))
                      : (R)0.5 * (sv_imf<C, R>(X, Fm) + sv_imf<C, R>(M, F));
        }
        const R inv = sv_rsqrt(s);
        const R hv = harm<R>(L, sa.m, sfx[li] * inv, fy * inv, fz * inv);
        acc0 += gc * sa.coef * hv * v;
      }
    }
    if (cur >= 0 && cur < nk) {
      if (acc0 != (R)0) atomicAdd(&sb[cur], acc0);
      if (L == 0) {
        if (acc2 != (R)0) atomicAdd(&sb[nk + cur], acc2);
        if (acc4 != (R)0) atomicAdd(&sb[2 * nk + cur], acc4);
      }
    }
  }
  __syncthreads();
  // bins laid out [5][nk]
  for (int c = threadIdx.x; c < (L == 0 ? 3 : 1) * nk; c += blockDim.x) {
    const R v = sb[c];
    if (v == (R)0) continue;
    const int row = L == 0 ? 2 * (c / nk) : L;
    atomicAdd(&bins[row * nk + c % nk], (double)v);
  }
}

// ------------------------------------------------------------------------------------ the context
#define SV_STAGE 9  // staged arrays per catalogue: x, y, z, w, nbar, pv, pverr, FKP w, FKP w_pv

struct capow_survey_ctx {
  capow_params p;
  capow_survey_params sv;
  capow_options o;
  int prec;  // CAPOW_FP64 or CAPOW_FP32_MIXED
  int mom;   // Momentum 0..3
  int nf;    // painted fields: 1, or 2 (density and momentum) for Momentum 2, 3
  Geom g;
  BinParams bp;
  BinTables bt;
  int nslot;  // nf * (1 + DoInterlacing)
  cudaStream_t stream;
  bool own_stream;
  void *paint;  // nslot painted grids, main_sz reals each (FP32: the paint context's grids)
  capow_ctx *pc;  // FP32: the paint-only context whose tile kernels paint data and randoms
  float *comb;    // FP32: the combined catalogue for it, [x | y | z | w | v] of comb_cap objects each
  size_t comb_cap;
  void *work;   // nslot term grids
  void *F0, *F0m;  // main_sz reals each (complex [NX][NY][NZ/2+1]); F0m for Momentum 2, 3
  void *vx, *vy, *vz;  // cell-corner offsets from the observer per axis (R)
  SvStats *st;
  double *bins;  // [5][nk]
  unsigned long long *nmodes_d, *nmodes2d_d;
  std::vector<unsigned long long> nmodes;
  cufftHandle plan;
  bool plan_ok, plan_per_grid;
  // FP32 with a power-of-two NZ: the z axis by the weighted z pass into the transposed [NX][NZ/2+1][NY]
  // work slots, then cuFFT along y (contiguous rows) and along x (strided), in place
  bool tr;
  cufftHandle yplan, xplan;
  bool yplan_ok, xplan_ok;
  // the observer's cell (r2 == 0), if any
  int origin;
  long long oind;
  void *ox, *oy, *oz;
  void *stage[2][SV_STAGE];
  size_t stage_bytes[2][SV_STAGE];
  double *h_bins;
  SvStats *h_st;
  std::vector<void *> allocs;
  cudaEvent_t ev[3];
  int sets;
  long long launches;
  bool done;
  char err[512];
};

static void *sv_dalloc(capow_survey_ctx *c, size_t bytes) {
  void *p = nullptr;
  if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) return nullptr;
  c->allocs.push_back(p);
  return p;
}

static int sv_validate(const capow_params *p, const capow_survey_params *sv, const capow_options *o, char *err,
                       size_t n) {
#define BAD(code, ...)             \
  do {                             \
    snprintf(err, n, __VA_ARGS__); \
    return code;                   \
  } while (0)
  if (!sv) BAD(CAPOW_EINVAL, "no survey parameters");
  if (p->InterpOrder < 1 || p->InterpOrder > 3) BAD(CAPOW_EINVAL, "InterpOrder is neither 1, 2 nor 3");
  if (p->DoInterlacing != 0 && p->DoInterlacing != 1) BAD(CAPOW_EINVAL, "DoInterlacing is neither 0 nor 1");
  if (p->Output2D != 0 && p->Output2D != 1) BAD(CAPOW_EINVAL, "Output2D is neither 0 nor 1");
  if (p->OutputLog != 0 && p->OutputLog != 1) BAD(CAPOW_EINVAL, "OutputLog is neither 0 nor 1");
  if (p->NX <= 0 || p->NY <= 0 || p->NZ <= 0) BAD(CAPOW_EINVAL, "NX, NY and NZ must be > 0");
  if (p->NK <= 0) BAD(CAPOW_EINVAL, "NK is less than 1");
  if (p->NK > 512) BAD(CAPOW_ENOTSUP, "the survey binning holds at most 512 k bins");
  if (!(p->XMAX > p->XMIN) || !(p->YMAX > p->YMIN) || !(p->ZMAX > p->ZMIN)) BAD(CAPOW_EINVAL, "box MAX must exceed MIN");
  if (p->Maxk < p->Mink) BAD(CAPOW_EINVAL, "Maxk is less than Mink");
  if (p->Momentum < 0 || p->Momentum > 3) BAD(CAPOW_ENOTSUP, "the survey estimator has Momentum 0 to 3");
  if (p->Momentum >= 2 && sv->FKP_Column >= 0)
    BAD(CAPOW_EINVAL, "survey Momentum 2 and 3 need the FKP weights (FKP_Column < 0): w_pv is set by them only");
  if (o->precision != CAPOW_FP64 && o->precision != CAPOW_FP32_MIXED)
    BAD(CAPOW_ENOTSUP, "survey precision must be CAPOW_FP64 or CAPOW_FP32_MIXED");
  if ((long long)p->NX * p->NY * 2 * (p->NZ / 2 + 1) >= (1LL << 40)) BAD(CAPOW_EINVAL, "grid too large");
  return CAPOW_OK;
#undef BAD
}

template <typename T>
static T *sv_upload(capow_survey_ctx *c, const std::vector<T> &h) {
  T *d = (T *)sv_dalloc(c, sizeof(T) * h.size());
  if (d && cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
  return d;
}

// cell-corner offset from the observer along one axis, as the reference forms it (src/main.c:554)
static double corner(int i, double d, double mn, double o) { return (double)i * d + mn - o; }

extern "C" int capow_survey_create(const capow_params *p, const capow_survey_params *sv, const capow_options *opt,
                                   capow_survey_ctx **out) {
  if (!p || !out) return CAPOW_EINVAL;
  *out = nullptr;
  capow_options o;
  memset(&o, 0, sizeof o);
  if (opt) o = *opt;
  else o.precision = CAPOW_FP32_MIXED;
  capow_survey_ctx *c = new (std::nothrow) capow_survey_ctx();
  if (!c) return CAPOW_ENOMEM;
  int rc = sv_validate(p, sv, &o, c->err, sizeof c->err);
  if (rc) {
    fprintf(stderr, "capow_survey_create: %s\n", c->err);
    delete c;
    return rc;
  }
  c->p = *p;
  c->sv = *sv;
  c->o = o;
  c->prec = o.precision;
  c->mom = p->Momentum;
  c->nf = c->mom >= 2 ? 2 : 1;
  *out = c;  // from here on capow_survey_destroy releases partial state
  CK(c, cudaSetDevice(o.device));
  if (o.stream) {
    c->stream = (cudaStream_t)o.stream;
    c->own_stream = false;
  } else {
    CK(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->own_stream = true;
  }
  for (int k = 0; k < 3; k++) CK(c, cudaEventCreate(&c->ev[k]));
  c->g = make_geom(*p);
  c->g.los = 4;  // no RSD shift, no wrap, the halo discarded
  c->g.survey = 1;
  c->nslot = c->nf * (1 + p->DoInterlacing);
  const bool f64 = c->prec == CAPOW_FP64;
  const size_t eb = f64 ? 8 : 4;
  const size_t ge = (size_t)c->g.main_sz;
  if (f64) {
    c->paint = sv_dalloc(c, eb * ge * c->nslot);
  } else {  // the FP32 grids are painted by the tile kernels of a paint-only context on this stream
    capow_options po = o;
    po.stream = (void *)c->stream;
    rc = create_paint_ctx(p, &po, c->nf, &c->pc);
    if (rc) FAIL(c, rc, "paint context: %s", c->pc ? capow_last_error(c->pc) : "invalid parameters");
    c->paint = c->pc->grid_base;
    // a survey fills part of the box (a ball or a sky cut), so an occupied tile holds several times the
    // box's mean share of the records: buckets of four mean shares keep them out of the overflow path
    c->pc->bucket_factor = 4.0f;
  }
  c->work = sv_dalloc(c, eb * ge * c->nslot);
  c->F0 = sv_dalloc(c, eb * ge);
  if (c->nf == 2) c->F0m = sv_dalloc(c, eb * ge);
  c->st = (SvStats *)sv_dalloc(c, sizeof(SvStats));
  const int nk = p->NK;
  c->bins = (double *)sv_dalloc(c, sizeof(double) * 5 * nk);
  c->nmodes_d = (unsigned long long *)sv_dalloc(c, sizeof(unsigned long long) * nk);
  c->nmodes2d_d = (unsigned long long *)sv_dalloc(c, sizeof(unsigned long long));
  if (!c->paint || !c->work || !c->F0 || (c->nf == 2 && !c->F0m) || !c->st || !c->bins || !c->nmodes_d ||
      !c->nmodes2d_d)
    FAIL(c, CAPOW_ENOMEM, "device allocation failed (grids need %.2f GB)", eb * ge * (2.0 * c->nslot + c->nf) / 1e9);
  CK(c, cudaMallocHost((void **)&c->h_bins, sizeof(double) * 5 * nk));
  CK(c, cudaMallocHost((void **)&c->h_st, sizeof(SvStats)));
  // corner offsets per axis, and the observer's cell: the corner whose three offsets square to 0
  const Geom &g = c->g;
  std::vector<double> v[3];
  const int nn[3] = {p->NX, p->NY, p->NZ};
  const double dd[3] = {g.dx, g.dy, g.dz}, mn[3] = {p->XMIN, p->YMIN, p->ZMIN},
               org[3] = {sv->X_Origin, sv->Y_Origin, sv->Z_Origin};
  int oc[3], ncand[3] = {0, 0, 0};
  for (int a = 0; a < 3; a++) {
    v[a].resize(nn[a]);
    for (int i = 0; i < nn[a]; i++) {
      v[a][i] = corner(i, dd[a], mn[a], org[a]);
      if (v[a][i] * v[a][i] == 0.0) {
        oc[a] = i;
        ncand[a]++;
      }
    }
  }
  c->origin = ncand[0] && ncand[1] && ncand[2];
  if (ncand[0] > 1 || ncand[1] > 1 || ncand[2] > 1)
    FAIL(c, CAPOW_ENOTSUP, "several cell corners within 1e-154 of the observer along one axis");
  if (f64) {
    c->vx = sv_upload(c, v[0]);
    c->vy = sv_upload(c, v[1]);
    c->vz = sv_upload(c, v[2]);
  } else {
    std::vector<float> f[3];
    for (int a = 0; a < 3; a++) {
      f[a].resize(nn[a]);
      for (int i = 0; i < nn[a]; i++) f[a][i] = (float)v[a][i];
    }
    c->vx = sv_upload(c, f[0]);
    c->vy = sv_upload(c, f[1]);
    c->vz = sv_upload(c, f[2]);
  }
  if (!c->vx || !c->vy || !c->vz) FAIL(c, CAPOW_ENOMEM, "observer offset tables");
  if (c->origin) {
    c->oind = (long long)oc[2] + g.row * ((long long)oc[1] + (long long)p->NY * oc[0]);
    const int len[3] = {p->NX, p->NY, p->NZ / 2 + 1};
    void **dst[3] = {&c->ox, &c->oy, &c->oz};
    for (int a = 0; a < 3; a++) {
      std::vector<double2> e2(len[a]);
      std::vector<float2> e1(len[a]);
      for (int q = 0; q < len[a]; q++) {  // e^{-2 pi i q o / N}, the exponent reduced exactly
        const long long r = ((long long)q * oc[a]) % nn[a];
        const double ang = -2.0 * M_PI * (double)r / (double)nn[a];
        e2[q] = make_double2(cos(ang), sin(ang));
        e1[q] = make_float2((float)cos(ang), (float)sin(ang));
      }
      *dst[a] = f64 ? (void *)sv_upload(c, e2) : (void *)sv_upload(c, e1);
      if (!*dst[a]) FAIL(c, CAPOW_ENOMEM, "observer phase tables");
    }
  }
  // bins: the periodic tables, exact edges and mode counts (the survey's modes, NM and Nyquist rule
  // are the periodic ones, src/main.c:840-905)
  BinParams &bp = c->bp;
  memset(&bp, 0, sizeof bp);
  bp.nx = p->NX; bp.ny = p->NY; bp.nz = p->NZ; bp.nzc = p->NZ / 2 + 1; bp.xhalf = p->NX / 2;
  bp.nk = nk; bp.nmu = p->NMU; bp.los = 3; bp.interlace = p->DoInterlacing;
  bp.odd = p->Odd_Multipoles; bp.out2d = 0; bp.nfields = 1;
  bp.two_pi = 2.0 * M_PI;
  bp.fx_step = (float)(1.0 / ((float)p->NX * g.dx));
  bin_params_kguess(bp, *p);
  if (build_bin_tables(*p, g, c->prec, c->bt, c->allocs, c->stream)) FAIL(c, CAPOW_ENOMEM, "bin tables");
  CK(c, cudaMemsetAsync(c->nmodes_d, 0, sizeof(unsigned long long) * nk, c->stream));
  launch_mode_counts(c->stream, bp, c->bt, c->nmodes_d, c->nmodes2d_d, &c->launches);
  CK(c, cudaGetLastError());
  c->nmodes.resize(nk);
  CK(c, cudaMemcpyAsync(c->nmodes.data(), c->nmodes_d, sizeof(unsigned long long) * nk, cudaMemcpyDeviceToHost,
                        c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  // FP32 with a power-of-two NZ: the transposed path (its z pass weights the painted grids as it reads
  // them, so no weighted grid is written; the y axis is then a contiguous batched transform)
  if (!f64 && c->bt.twz && zr2c_supported(bp)) {
    const long long yrows = (long long)c->nslot * p->NX * bp.nzc, xcols = (long long)bp.nzc * p->NY;
    int ny = p->NY, nx = p->NX, emb = p->NX;
    if (yrows <= 0x7fffffffLL && xcols <= 0x7fffffffLL &&
        cufftPlanMany(&c->yplan, 1, &ny, nullptr, 1, ny, nullptr, 1, ny, CUFFT_C2C, (int)yrows) == CUFFT_SUCCESS) {
      c->yplan_ok = true;
      if (cufftPlanMany(&c->xplan, 1, &nx, &emb, (int)xcols, 1, &emb, (int)xcols, 1, CUFFT_C2C, (int)xcols) ==
          CUFFT_SUCCESS) {
        c->xplan_ok = true;
        c->tr = true;
        CKFFT(c, cufftSetStream(c->yplan, c->stream));
        CKFFT(c, cufftSetStream(c->xplan, c->stream));
        return CAPOW_OK;
      }
    }
    (void)cudaGetLastError();  // no room for the plans: the 3-D transform below
  }
  // one batched in-place real-to-complex plan over the nslot term grids (fftw_execute of plan, plan_interlace,
  // plan_mom and plan_mom_interlace, src/main.c:513-526 and the product loops)
  int n[3] = {p->NX, p->NY, p->NZ};
  int inembed[3] = {p->NX, p->NY, 2 * bp.nzc}, onembed[3] = {p->NX, p->NY, bp.nzc};
  const long long idist = (long long)ge, odist = (long long)ge / 2;
  if (idist > 0x7fffffffLL || c->nslot == 1) {
    CKFFT(c, cufftPlan3d(&c->plan, p->NX, p->NY, p->NZ, f64 ? CUFFT_D2Z : CUFFT_R2C));
    c->plan_per_grid = true;
  } else {
    CKFFT(c, cufftPlanMany(&c->plan, 3, n, inembed, 1, (int)idist, onembed, 1, (int)odist, f64 ? CUFFT_D2Z : CUFFT_R2C,
                           c->nslot));
  }
  c->plan_ok = true;
  CKFFT(c, cufftSetStream(c->plan, c->stream));
  return CAPOW_OK;
}

extern "C" void capow_survey_destroy(capow_survey_ctx *c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->plan_ok) cufftDestroy(c->plan);
  if (c->yplan_ok) cufftDestroy(c->yplan);
  if (c->xplan_ok) cufftDestroy(c->xplan);
  if (c->pc) capow_destroy(c->pc);
  if (c->comb) cudaFree(c->comb);
  for (void *q : c->allocs) cudaFree(q);
  for (int a = 0; a < 2; a++)
    for (int k = 0; k < SV_STAGE; k++)
      if (c->stage[a][k]) cudaFree(c->stage[a][k]);
  if (c->h_bins) cudaFreeHost(c->h_bins);
  if (c->h_st) cudaFreeHost(c->h_st);
  for (int k = 0; k < 3; k++)
    if (c->ev[k]) cudaEventDestroy(c->ev[k]);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" const char *capow_survey_last_error(const capow_survey_ctx *c) { return c ? c->err : "no context"; }
extern "C" int64_t capow_survey_kernel_launches(const capow_survey_ctx *c) { return c ? c->launches : 0; }

// a device buffer of at least `bytes` in staging slot [cat][k]
static int sv_stage_buffer(capow_survey_ctx *c, int cat, int k, size_t bytes) {
  if (c->stage_bytes[cat][k] >= bytes && c->stage[cat][k]) return CAPOW_OK;
  if (c->stage[cat][k]) cudaFree(c->stage[cat][k]);
  c->stage[cat][k] = nullptr;
  c->stage_bytes[cat][k] = 0;
  CK(c, cudaMalloc(&c->stage[cat][k], bytes ? bytes : 16));
  c->stage_bytes[cat][k] = bytes;
  return CAPOW_OK;
}

static int sv_blocks(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152LL * 16) b = 152LL * 16;
  return b < 1 ? 1 : (int)b;
}

// The device view of one catalogue: device arrays as given, host arrays copied into the staging slots.
// *wk and *wpv are the weights to paint: the FKP-weighted copies when FKP_Column < 0.
template <typename T>
static int sv_device_view(capow_survey_ctx *c, int cat, const capow_survey_catalogue *in, bool copy, SvIn<T> *sin,
                          const T **wk, const T **wpv) {
  const size_t bytes = sizeof(T) * in->n;
  const void *src[7] = {in->x, in->y, in->z, in->w, in->nbar, in->pv, in->pverr};
  const void *d[7];
  for (int k = 0; k < 7; k++) {
    if (k >= 5 && !c->mom) {  // pv, pverr: Momentum 1-3 only
      d[k] = nullptr;
      continue;
    }
    if (!src[k] || in->on_device) {
      d[k] = src[k];
      continue;
    }
    if (copy) {
      int rc = sv_stage_buffer(c, cat, k, bytes);
      if (rc) return rc;
      if (bytes) CK(c, cudaMemcpyAsync(c->stage[cat][k], src[k], bytes, cudaMemcpyHostToDevice, c->stream));
    }
    d[k] = c->stage[cat][k];
  }
  *sin = SvIn<T>{(const T *)d[0], (const T *)d[1], (const T *)d[2], (const T *)d[3], (const T *)d[4], (const T *)d[5],
                 (const T *)d[6]};
  const bool fkp = c->sv.FKP_Column < 0;
  if (fkp && copy) {
    int rc = sv_stage_buffer(c, cat, 7, bytes);
    if (!rc && c->mom >= 2) rc = sv_stage_buffer(c, cat, 8, bytes);
    if (rc) return rc;
  }
  *wk = fkp ? (const T *)c->stage[cat][7] : sin->w;
  *wpv = c->mom >= 2 ? (const T *)c->stage[cat][8] : nullptr;
  return CAPOW_OK;
}

template <typename T>
static int sv_enqueue_catalogue(capow_survey_ctx *c, int cat, const capow_survey_catalogue *in) {
  SvIn<T> sin;
  const T *wk, *wpv;
  int rc = sv_device_view<T>(c, cat, in, true, &sin, &wk, &wpv);
  if (rc) return rc;
  if (in->n) {
    k_sv_prepare<T><<<sv_blocks(in->n), 256, 0, c->stream>>>(sin, (long long)in->n, c->sv.FKP_Column < 0, c->mom,
                                                             c->sv.FKP_Pk, c->sv.FKP_Pk_mom, c->sv.FKP_Pk_cross,
                                                             (T *)wk, (T *)wpv, c->st, cat);
    c->launches++;
  }
  return CAPOW_OK;
}

// FP64: every object with global FP64 atomics (k_sv_paint), the reference's per-object double products.
template <typename T, typename R>
static int sv_launch_paint(capow_survey_ctx *c, int cat, const capow_survey_catalogue *in) {
  if (!in->n) return CAPOW_OK;
  SvIn<T> sin;
  const T *wk, *wpv;
  int rc = sv_device_view<T>(c, cat, in, false, &sin, &wk, &wpv);
  if (rc) return rc;
  SvGrids<R> gr;
  for (int s = 0; s < 4; s++) gr.g[s] = s < c->nslot ? (R *)c->paint + s * c->g.main_sz : nullptr;
  k_sv_paint<T, R><<<sv_blocks(in->n), 256, 0, c->stream>>>(c->g, sin, wk, wpv, (long long)in->n, cat, c->mom, c->nf,
                                                            gr, c->st);
  c->launches++;
  return CAPOW_OK;
}

// FP32: data and randoms (Momentum 1: data only) combined into one float catalogue with the prefactors
// applied, painted by the paint context's tile kernels (shared-memory tiles written once; objects near the
// grid's discontinuities, the Survey clamp region included, take the exact FP64 rules). The paint settles on
// the host (one synchronisation) so that a tile-list overflow repaints before the multipoles read the grids.
template <typename T>
static int sv_paint_tiles(capow_survey_ctx *c, const capow_survey_catalogue *data, const capow_survey_catalogue *rand) {
  const int ncat = c->mom == 1 ? 1 : 2;  // src/main.c:229: Momentum 1 paints no randoms
  const size_t n = data->n + (ncat == 2 ? rand->n : 0);
  if (c->comb_cap < n || !c->comb) {
    if (c->comb) cudaFree(c->comb);
    c->comb = nullptr;
    c->comb_cap = 0;
    CK(c, cudaMalloc(&c->comb, sizeof(float) * 5 * (n ? n : 1)));
    c->comb_cap = n ? n : 1;
  }
  float *cx = c->comb, *cy = cx + c->comb_cap, *cz = cy + c->comb_cap, *cw = cz + c->comb_cap, *cv = cw + c->comb_cap;
  const capow_survey_catalogue *cats[2] = {data, rand};
  long long off = 0;
  for (int cat = 0; cat < ncat; cat++) {
    const long long m = (long long)cats[cat]->n;
    if (m) {
      SvIn<T> sin;
      const T *wk, *wpv;
      int rc = sv_device_view<T>(c, cat, cats[cat], false, &sin, &wk, &wpv);
      if (rc) return rc;
      k_sv_combine<T><<<sv_blocks(m), 256, 0, c->stream>>>(c->g, sin, wk, wpv, m, cat, c->mom, off, cx, cy, cz, cw, cv,
                                                           c->st);
      c->launches++;
    }
    off += m;
  }
  CK(c, cudaGetLastError());
  capow_particles d;
  memset(&d, 0, sizeof d);
  d.n = n;
  d.dtype = CAPOW_F32;
  d.on_device = 1;
  d.x = cx;
  d.y = cy;
  d.z = cz;
  d.w = cw;
  d.vlos = c->nf == 2 ? cv : nullptr;
  capow_ctx *pc = c->pc;
  pc->last = d;
  pc->painted = true;
  const long long before = pc->launches;
  int rc = enqueue_paint(pc, d);
  if (!rc) rc = settle_paint(pc);
  c->launches += pc->launches - before;
  if (rc) FAIL(c, rc, "survey paint: %s", capow_last_error(pc));
  return CAPOW_OK;
}

template <typename R, int L>
static void sv_launch_assign(capow_survey_ctx *c, const dim3 &grid, const SvAssign<R> &sa) {
  if (c->tr) {
    if (c->nf == 2) k_sv_assign<R, L, true, true><<<grid, 256, 0, c->stream>>>(c->bp, c->bt, sa, c->bins);
    else k_sv_assign<R, L, false, true><<<grid, 256, 0, c->stream>>>(c->bp, c->bt, sa, c->bins);
  } else if (c->nf == 2) {
    k_sv_assign<R, L, true, false><<<grid, 256, 0, c->stream>>>(c->bp, c->bt, sa, c->bins);
  } else {
    k_sv_assign<R, L, false, false><<<grid, 256, 0, c->stream>>>(c->bp, c->bt, sa, c->bins);
  }
}

template <typename R>
static int sv_multipoles(capow_survey_ctx *c) {
  typedef typename SvC<R>::C C;
  const capow_params &p = c->p;
  const Geom &g = c->g;
  const long long ge = g.main_sz;
  const int nf = c->nf, il = p.DoInterlacing;
  R *a[4], *w[4];
  for (int s = 0; s < 4; s++) {
    a[s] = s < c->nslot ? (R *)c->paint + s * ge : nullptr;
    w[s] = s < c->nslot ? (R *)c->work + s * ge : nullptr;
  }
  const int sd0 = sv_slot(0, 0, nf), sd1 = sv_slot(1, 0, nf), sm0 = sv_slot(0, 1, nf), sm1 = sv_slot(1, 1, nf);
  const long long rows = (long long)p.NX * p.NY;
  // one warp per row, 8 per CTA, grid-stride beyond 16 CTAs per SM
  const unsigned wblocks = (unsigned)std::min<long long>((rows + 7) / 8, 152LL * 16);
  const long long cols = (long long)p.NY * c->bp.nzc;
  const dim3 agrid((unsigned)((cols + 255) / 256), (unsigned)((p.NX + SV_ICHUNK - 1) / SV_ICHUNK));
  SvAssign<R> sa;
  memset(&sa, 0, sizeof sa);
  sa.gd0 = (const C *)w[sd0];
  sa.gd1 = il ? (const C *)w[sd1] : nullptr;
  sa.gm0 = nf == 2 ? (const C *)w[sm0] : nullptr;
  sa.gm1 = nf == 2 && il ? (const C *)w[sm1] : nullptr;
  sa.F0 = (C *)c->F0;
  sa.F0m = (C *)c->F0m;
  sa.dc = c->pc ? (const double *)((const char *)c->pc->st + offsetof(DevStats, dc))
               : (const double *)((const char *)c->st + offsetof(SvStats, dc));
  sa.sd0 = sd0;
  sa.sd1 = sd1;
  sa.sm0 = sm0;
  sa.sm1 = sm1;
  sa.origin = c->origin;
  for (int s = 0; s < 4; s++) sa.a[s] = a[s];
  sa.oind = c->oind;
  sa.ox = (const C *)c->ox;
  sa.oy = (const C *)c->oy;
  sa.oz = (const C *)c->oz;
  const int step = p.Odd_Multipoles ? 1 : 2;  // src/main.c:490-492
  c->sets = 0;
  for (int l = 0; l <= 4; l += step) {
    for (int m = 0; m < 2 * l + 1; m++) {
      bool transformed = false;
      if constexpr (sizeof(R) == 4) {
        if (c->tr) {  // weighted z pass into the transposed work slots, then y and x in place
          const long long tslot = ge / 2;
          if (l == 0)
            launch_zr2c(c->stream, c->bp, c->bt, c->nslot, (const float *)a[0], ge, (int)g.row, (float2 *)w[0],
                        tslot, &c->launches);
          else
            launch_zr2c_weighted(c->stream, c->bp, c->bt, c->nslot, (const float *)a[0], ge, (int)g.row,
                                 (float2 *)w[0], tslot, (const float *)c->vx, (const float *)c->vy,
                                 (const float *)c->vz, l, m, &c->launches);
          CKFFT(c, cufftExecC2C(c->yplan, (cufftComplex *)w[0], (cufftComplex *)w[0], CUFFT_FORWARD));
          for (int s = 0; s < c->nslot; s++)
            CKFFT(c, cufftExecC2C(c->xplan, (cufftComplex *)w[s], (cufftComplex *)w[s], CUFFT_FORWARD));
          transformed = true;
        }
      }
      for (int f = 0; f < nf && !transformed; f++) {  // the density grid (and its interlaced copy), then momentum
        const int s0 = sv_slot(0, f, nf), s1 = sv_slot(1, f, nf);
        k_sv_weight<R><<<wblocks, 256, 0, c->stream>>>(a[s0], il ? a[s1] : nullptr, w[s0], il ? w[s1] : nullptr,
                                                       (const R *)c->vx, (const R *)c->vy, (const R *)c->vz, p.NX,
                                                       p.NY, p.NZ, g.row, l, m);
        c->launches++;
      }
      if (transformed) {
      } else if (c->plan_per_grid) {
        for (int s = 0; s < c->nslot; s++) {
          if (sizeof(R) == 8) CKFFT(c, cufftExecD2Z(c->plan, (cufftDoubleReal *)w[s], (cufftDoubleComplex *)w[s]));
          else CKFFT(c, cufftExecR2C(c->plan, (cufftReal *)w[s], (cufftComplex *)w[s]));
        }
      } else if (sizeof(R) == 8) {
        CKFFT(c, cufftExecD2Z(c->plan, (cufftDoubleReal *)w[0], (cufftDoubleComplex *)w[0]));
      } else {
        CKFFT(c, cufftExecR2C(c->plan, (cufftReal *)w[0], (cufftComplex *)w[0]));
      }
      sa.m = m;
      sa.coef = (R)harm_coef(l, m);
      switch (l) {
        case 0: sv_launch_assign<R, 0>(c, agrid, sa); break;
        case 1: sv_launch_assign<R, 1>(c, agrid, sa); break;
        case 2: sv_launch_assign<R, 2>(c, agrid, sa); break;
        case 3: sv_launch_assign<R, 3>(c, agrid, sa); break;
        default: sv_launch_assign<R, 4>(c, agrid, sa); break;
      }
      c->launches++;
      c->sets++;
    }
  }
  CK(c, cudaGetLastError());
  return CAPOW_OK;
}

template <typename T, typename R>
static int sv_run(capow_survey_ctx *c, const capow_survey_catalogue *data, const capow_survey_catalogue *rand) {
  CK(c, cudaMemsetAsync(c->st, 0, sizeof(SvStats), c->stream));
  CK(c, cudaMemsetAsync(c->bins, 0, sizeof(double) * 5 * c->p.NK, c->stream));
  CK(c, cudaEventRecord(c->ev[0], c->stream));
  int rc = sv_enqueue_catalogue<T>(c, 0, data);
  if (!rc) rc = sv_enqueue_catalogue<T>(c, 1, rand);
  if (rc) return rc;
  if constexpr (sizeof(R) == 8) {
    CK(c, cudaMemsetAsync(c->paint, 0, sizeof(R) * (size_t)c->g.main_sz * c->nslot, c->stream));
    rc = sv_launch_paint<T, R>(c, 0, data);
    if (!rc && c->mom != 1) rc = sv_launch_paint<T, R>(c, 1, rand);  // src/main.c:229
    if (rc) return rc;
  } else {
    rc = sv_paint_tiles<T>(c, data, rand);
    if (rc) return rc;
  }
  CK(c, cudaGetLastError());
  CK(c, cudaEventRecord(c->ev[1], c->stream));
  rc = sv_multipoles<R>(c);
  if (rc) return rc;
  CK(c, cudaEventRecord(c->ev[2], c->stream));
  return CAPOW_OK;
}

static bool sv_cat_ok(const capow_survey_catalogue *c, int mom, bool data) {
  if (!c || (c->dtype != CAPOW_F32 && c->dtype != CAPOW_F64)) return false;
  if (c->n && (!c->x || !c->y || !c->z || !c->w || !c->nbar)) return false;
  if (c->n && mom && !c->pverr) return false;
  if (c->n && mom && data && !c->pv) return false;
  return true;
}

extern "C" int capow_survey_power(capow_survey_ctx *c, const capow_survey_catalogue *data,
                                  const capow_survey_catalogue *rand, capow_spectrum *out, capow_survey_stats *st) {
  if (!c) return CAPOW_EINVAL;
  if (!sv_cat_ok(data, c->mom, true) || !sv_cat_ok(rand, c->mom, false))
    FAIL(c, CAPOW_EINVAL,
         "survey catalogue: dtype must be CAPOW_F32 or CAPOW_F64 with x, y, z, w and nbar given (and pv, pverr for "
         "Momentum 1-3)");
  if (data->dtype != rand->dtype) FAIL(c, CAPOW_EINVAL, "data and randoms must have the same dtype");
  CK(c, cudaSetDevice(c->o.device));
  c->done = false;
  int rc;
  const bool f64 = c->prec == CAPOW_FP64;
  if (data->dtype == CAPOW_F32) rc = f64 ? sv_run<float, double>(c, data, rand) : sv_run<float, float>(c, data, rand);
  else rc = f64 ? sv_run<double, double>(c, data, rand) : sv_run<double, float>(c, data, rand);
  if (rc) return rc;
  const int nk = c->p.NK;
  CK(c, cudaMemcpyAsync(c->h_bins, c->bins, sizeof(double) * 5 * nk, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaMemcpyAsync(c->h_st, c->st, sizeof(SvStats), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  c->done = true;
  const SvStats &s = *c->h_st;
  if (s.nonfinite)
    FAIL(c, CAPOW_EINVAL, "non-finite coordinate, weight, number density or velocity in a survey catalogue");
  // src/main.c:166-186
  const double alpha = s.wsum[0] / s.wsum[1];
  const double rand_nbwsq = s.w2sum[1] * (alpha * alpha);
  const double rand_nbsqwsq = s.w2nsum[1] * alpha;
  double shot, norm;
  switch (c->mom) {
    case 0: shot = s.w2sum[0] + rand_nbwsq; norm = rand_nbsqwsq; break;
    case 1: shot = s.vrsq; norm = rand_nbsqwsq; break;
    case 2: shot = s.vr; norm = sqrt(rand_nbsqwsq * s.w2npv[1]); break;
    default: shot = s.vrsq; norm = sqrt(rand_nbsqwsq * s.w2npv[1]); break;
  }
  if (st) {
    st->ngrid_data = s.ngrid[0];
    st->ngrid_rand = c->mom == 1 ? 0.0 : s.ngrid[1] / -alpha;
    st->data_nbw = s.wsum[0];
    st->data_nbwsq = s.w2sum[0];
    st->data_nbsqwsq = s.w2nsum[0];
    st->rand_nbw = s.wsum[1];
    st->rand_nbwsq = rand_nbwsq;
    st->rand_nbsqwsq = rand_nbsqwsq;
    st->data_vr = s.vr;
    st->data_vrsq = s.vrsq;
    st->data_nbsqwsq_pv = s.w2npv[0];
    st->rand_nbsqwsq_pv = s.w2npv[1];
  }
  if (out) {
    for (int l = 0; l < 5; l++) {
      if (!out->pk[l]) continue;
      const bool have = (l % 2 == 0) || c->p.Odd_Multipoles;
      for (int b = 0; b < nk; b++) out->pk[l][b] = have ? c->h_bins[l * nk + b] : 0.0;
    }
    if (out->nmodes)
      for (int b = 0; b < nk; b++) out->nmodes[b] = (int64_t)c->nmodes[b];
    if (c->p.Output2D) {  // the survey estimator fills no 2-D bins (src/main.c:476-479 only allocates them)
      const int n2 = nk * c->p.NMU;
      if (out->pk2d)
        for (int b = 0; b < n2; b++) out->pk2d[b] = 0.0;
      if (out->nmodes2d)
        for (int b = 0; b < n2; b++) out->nmodes2d[b] = 0;
    }
    out->alpha = alpha;
    out->shot = shot;
    out->norm = norm;
    out->last_bin = -1;
    out->kind = 0;
  }
  return CAPOW_OK;
}

extern "C" int capow_survey_copy_grid(capow_survey_ctx *c, int which, double *host_out) {
  if (!c || !host_out || which < 0 || which >= c->nslot) return CAPOW_EINVAL;
  if (!c->done) FAIL(c, CAPOW_ESTATE, "no survey evaluation yet");
  const size_t ge = (size_t)c->g.main_sz;
  if (c->prec == CAPOW_FP64) {
    CK(c, cudaMemcpy(host_out, (double *)c->paint + which * ge, sizeof(double) * ge, cudaMemcpyDeviceToHost));
  } else {
    std::vector<float> tmp(ge);
    CK(c, cudaMemcpy(tmp.data(), (float *)c->paint + which * ge, sizeof(float) * ge, cudaMemcpyDeviceToHost));
    for (size_t q = 0; q < ge; q++) host_out[q] = tmp[q];
  }
  return CAPOW_OK;
}

extern "C" int capow_survey_stage_ms(capow_survey_ctx *c, float *paint_ms, float *multipole_ms, int *fft_sets) {
  if (!c) return CAPOW_EINVAL;
  if (!c->done) FAIL(c, CAPOW_ESTATE, "no survey evaluation yet");
  if (paint_ms) CK(c, cudaEventElapsedTime(paint_ms, c->ev[0], c->ev[1]));
  if (multipole_ms) CK(c, cudaEventElapsedTime(multipole_ms, c->ev[1], c->ev[2]));
  if (fft_sets) *fft_sets = c->sets;
  return CAPOW_OK;
}
