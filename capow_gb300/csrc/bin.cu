// compute_periodic_power (src/main.c:302-468) on the GPU: one pass over the FFT output that
// applies the window deconvolution, the interlacing phase combine, the delta-delta /
// delta-momentum / momentum-momentum powers and the Legendre-weighted P0..P4 sums.
//
// Bin assignment is bit-exact: the reference's bin is a monotone function of the double
// s = (fx*fx + fy*fy) + fz*fz (src/main.c:355, 369-375), so the host finds, by bisection over
// doubles, the smallest s of every bin edge (merged with the Nyquist cut, :375). The FP32
// kernel compares an FP32 s against those edges and recomputes s exactly in FP64 only for
// modes within a few ulps of an edge. Mode counts do not depend on the fields and are
// computed once per context by k_mode_counts.
//
// Accumulation: each thread walks the x axis of one (y, z) column; along a walk the bin
// changes rarely, so per-thread register sums of the current bin are flushed into shared
// memory bins on a bin change, and each CTA adds its bins to the global FP64 sums.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "bin.cuh"
#include "paint.cuh"

// ------------------------------------------------------------------------------------ host side
int host_kbin_of_s(double s, double mink, double binwidth, int nk, int output_log, double min_nyquist) {
  double fktot = 2.0 * M_PI * sqrt(s);
  double v;
  if (output_log) v = (float)(log10(fktot) - mink) / binwidth;
  else v = (float)(fktot - mink) / binwidth;
  int kb;
  if (v != v) return -1;
  if (v >= 2147483648.0) return nk;
  if (v <= -2147483649.0) return -1;
  kb = (int)v;
  if (kb < 0) return -1;
  if (kb >= nk) return nk;
  if (!(fktot <= min_nyquist)) return nk;
  return kb;
}

static double from_bits(unsigned long long b) {
  double d;
  memcpy(&d, &b, 8);
  return d;
}

// smallest s >= 0 with bin(s) >= b (bin is monotone non-decreasing in s)
static double edge_for(int b, double mink, double bw, int nk, int lg, double ny) {
  unsigned long long lo = 0, hi = 0x7FF0000000000000ULL;  // [0, +inf]
  if (host_kbin_of_s(0.0, mink, bw, nk, lg, ny) >= b) return 0.0;
  while (hi - lo > 1) {
    unsigned long long mid = lo + (hi - lo) / 2;
    if (host_kbin_of_s(from_bits(mid), mink, bw, nk, lg, ny) >= b) hi = mid;
    else lo = mid;
  }
  return from_bits(hi);
}

template <typename T>
static T *upload(const std::vector<T> &h, std::vector<void *> &allocs, cudaStream_t s) {
  T *d = nullptr;
  if (cudaMalloc(&d, sizeof(T) * (h.size() ? h.size() : 1)) != cudaSuccess) return nullptr;
  allocs.push_back(d);
  if (!h.empty()) cudaMemcpyAsync(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s);
  return d;
}

int build_bin_tables(const capow_params &p, const Geom &g, int precision, BinTables &t, std::vector<void *> &allocs,
                     cudaStream_t s) {
  (void)precision;
  const int nx = p.NX, ny = p.NY, nz = p.NZ, nzc = nz / 2 + 1;
  const unsigned long long NX = nx, NY = ny, NZ = nz;
  const double dx = g.dx, dy = g.dy, dz = g.dz;
  // src/main.c:329
  const double sx = 1.0 / ((float)NX * dx), sy = 1.0 / ((float)NY * dy), sz = 1.0 / ((float)NZ * dz);
  auto freq = [](int i, unsigned long long N, double sc) -> double {
    return ((unsigned long long)i <= N / 2) ? (float)i * sc : ((float)i - (float)N) * sc;
  };
  auto fill = [&](int n, unsigned long long N, double sc, double d, bool half, std::vector<double> &f,
                  std::vector<double> &f2, std::vector<double> &c, std::vector<double> &er, std::vector<double> &ei) {
    f.resize(n); f2.resize(n); c.resize(n); er.resize(n); ei.resize(n);
    for (int i = 0; i < n; i++) {
      double fr = half ? (float)i * sc : freq(i, N, sc);  // fz = (float)k*sz (:352)
      f[i] = fr;
      f2[i] = fr * fr;
      double a = M_PI * fr * d;  // :383-385
      double sinc = 1.0;
      if (fr != 0.0) sinc = sin(a) / a;  // :386-388
      c[i] = pow(1.0 / sinc, 2 * p.InterpOrder);
      er[i] = cos(a);
      ei[i] = sin(a);
    }
  };
  std::vector<double> fx, fx2, cx, exr, exi, fy, fy2, cy, eyr, eyi, fz, fz2, cz, ezr, ezi;
  fill(nx, NX, sx, dx, false, fx, fx2, cx, exr, exi);
  fill(ny, NY, sy, dy, false, fy, fy2, cy, eyr, eyi);
  fill(nzc, NZ, sz, dz, true, fz, fz2, cz, ezr, ezi);
  auto tof = [](const std::vector<double> &v) {
    std::vector<float> o(v.size());
    for (size_t i = 0; i < v.size(); i++) o[i] = (float)v[i];
    return o;
  };
  auto tod2 = [](const std::vector<double> &r, const std::vector<double> &im) {
    std::vector<double2> o(r.size());
    for (size_t i = 0; i < r.size(); i++) o[i] = make_double2(r[i], im[i]);
    return o;
  };
  auto tof2 = [](const std::vector<double> &r, const std::vector<double> &im) {
    std::vector<float2> o(r.size());
    for (size_t i = 0; i < r.size(); i++) o[i] = make_float2((float)r[i], (float)im[i]);
    return o;
  };
  t.fxd = upload(fx, allocs, s); t.fyd = upload(fy, allocs, s); t.fzd = upload(fz, allocs, s);
  t.fx2d = upload(fx2, allocs, s); t.fy2d = upload(fy2, allocs, s); t.fz2d = upload(fz2, allocs, s);
  t.fxf = upload(tof(fx), allocs, s); t.fyf = upload(tof(fy), allocs, s); t.fzf = upload(tof(fz), allocs, s);
  t.fx2f = upload(tof(fx2), allocs, s); t.fy2f = upload(tof(fy2), allocs, s); t.fz2f = upload(tof(fz2), allocs, s);
  t.cxd = upload(cx, allocs, s); t.cyd = upload(cy, allocs, s); t.czd = upload(cz, allocs, s);
  t.cxf = upload(tof(cx), allocs, s); t.cyf = upload(tof(cy), allocs, s); t.czf = upload(tof(cz), allocs, s);
  t.exd = upload(tod2(exr, exi), allocs, s); t.eyd = upload(tod2(eyr, eyi), allocs, s);
  t.ezd = upload(tod2(ezr, ezi), allocs, s);
  t.exf = upload(tof2(exr, exi), allocs, s); t.eyf = upload(tof2(eyr, eyi), allocs, s);
  t.ezf = upload(tof2(ezr, ezi), allocs, s);

  // bin edges, src/main.c:305, 320-325, 369-375
  const double binwidth = (p.Maxk - p.Mink) / (double)p.NK;
  double ny_x = M_PI / dx, ny_y = M_PI / dy, ny_z = M_PI / dz;
  double min_ny = ny_x;
  if (ny_y < min_ny) min_ny = ny_y;
  if (ny_z < min_ny) min_ny = ny_z;
  const int NK = p.NK;
  // E with sentinels: E[0] = -inf (bin -1 lower edge), E[b+1] = edge of bin b, E[NK+2] = +inf
  std::vector<double> E(NK + 3);
  E[0] = -INFINITY;
  for (int b = 0; b <= NK; b++) E[b + 1] = edge_for(b, p.Mink, binwidth, NK, p.OutputLog, min_ny);
  E[NK + 2] = INFINITY;
  std::vector<float> Elo(NK + 3), Ehi(NK + 3);
  const double eps = 4e-6;
  for (int b = 0; b < NK + 3; b++) {
    double e = E[b];
    if (std::isinf(e)) {
      Elo[b] = Ehi[b] = (float)e;
      continue;
    }
    // s32 >= Elo  =>  s >= E ;  s32 < Ehi  =>  s < E   (s32 carries < 1e-6 relative error)
    Elo[b] = nextafterf((float)(e * (1.0 + eps)), INFINITY);
    Ehi[b] = nextafterf((float)(e * (1.0 - eps)), -INFINITY);
    if (e == 0.0) { Elo[b] = 0.0f; Ehi[b] = -INFINITY; }
  }
  t.E = upload(E, allocs, s);
  t.Elo = upload(Elo, allocs, s);
  t.Ehi = upload(Ehi, allocs, s);
  return (t.E && t.Elo && t.Ehi && t.ezf) ? 0 : 1;
}

// ---------------------------------------------------------------------------------- device side
// bin in [-1, NK] of an exact s: E[b+1] <= s < E[b+2]
__device__ __forceinline__ int exact_bin(const double *E, int nk, double s, int guess) {
  int b = guess < -1 ? -1 : (guess > nk ? nk : guess);
  while (b < nk && s >= E[b + 2]) b++;
  while (b > -1 && s < E[b + 1]) b--;
  return b;
}

__device__ __forceinline__ double exact_s(const BinTables &t, int i, int j, int k) {
  return __dadd_rn(__dadd_rn(t.fx2d[i], t.fy2d[j]), t.fz2d[k]);
}

// Hermitian multiplicity NM, src/main.c:422-429
__device__ __forceinline__ int herm_nm(int i, int j, int k, int xhalf) {
  if (k != 0) return 2;
  if (j == 0) return ((i != 0) && (i != xhalf)) ? 1 : 2;
  return (i != xhalf) ? 1 : 2;
}

// exact 2-D mu bin, src/main.c:357-367, 454-455
__device__ __forceinline__ int exact_mubin(const BinParams &bp, const BinTables &t, int i, int j, int k, double s) {
  double fk = __dmul_rn(bp.two_pi, __dsqrt_rn(s));
  double f = bp.los == 1 ? t.fxd[i] : (bp.los == 2 ? t.fyd[j] : t.fzd[k]);
  double mu = fk > 0 ? __ddiv_rn(__dmul_rn(bp.two_pi, f), fk) : 0.0;
  int mb = (int)__dmul_rn(__ddiv_rn(__dadd_rn(mu, 1.0), 2.0), (double)(float)bp.nmu);
  if (mb >= bp.nmu) mb = bp.nmu - 1;
  return mb;
}

// One-time mode counts (Nmodes, Nmodes_2D): exact for every mode.
__global__ void __launch_bounds__(256) k_mode_counts(BinParams bp, BinTables t, unsigned long long *nm,
                                                     unsigned long long *nm2d) {
  extern __shared__ unsigned long long scount[];
  const int nk = bp.nk, n2 = bp.out2d ? nk * bp.nmu : 0;
  for (int c = threadIdx.x; c < nk + n2; c += blockDim.x) scount[c] = 0;
  __syncthreads();
  const long long cols = (long long)bp.ny * bp.nzc;
  const long long total = cols * bp.nx;
  int guess = 0;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q / cols);
    const long long col = q - (long long)i * cols;
    const int j = (int)(col / bp.nzc), k = (int)(col - (long long)j * bp.nzc);
    const double s = exact_s(t, i, j, k);
    const int b = exact_bin(t.E, nk, s, guess);
    guess = b;
    if (b < 0 || b >= nk) continue;
    const int NM = herm_nm(i, j, k, bp.xhalf);
    atomicAdd(&scount[b], (unsigned long long)NM);
    if (bp.out2d) {
      const int mb = exact_mubin(bp, t, i, j, k, s);
      const int bin = b * bp.nmu + mb;
      if (bin >= 0 && bin < nk * bp.nmu) atomicAdd(&scount[nk + bin], (unsigned long long)NM);
    }
  }
  __syncthreads();
  for (int c = threadIdx.x; c < nk + n2; c += blockDim.x) {
    unsigned long long v = scount[c];
    if (!v) continue;
    if (c < nk) atomicAdd(nm + c, v);
    else atomicAdd(nm2d + (c - nk), v);
  }
}

template <typename R>
struct CT;
template <>
struct CT<float> {
  typedef float2 C;
};
template <>
struct CT<double> {
  typedef double2 C;
};

template <typename C>
__device__ __forceinline__ C cmul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}

// DC corrections: mean subtraction (src/main.c:211-225) changes only the k = 0 mode, whose
// value after it is sum(grid) - NX*NY*NZ*alpha = painted sum - NGRID. The painted sums are
// exact FP64 (FP32 path: FP64 sum of the stored FP32 cells; deterministic path: exact integers).
__global__ void k_dc_prepare(const DevStats *st, int det, int nslot, int nfields, int mean_sub_a,
                             const double *fixed_scale, double *dcv) {
  const double ngrid = st->ngrid;
  for (int s = 0; s < nslot; s++) {
    const int f = s % nfields;
    double v = det ? (double)(long long)st->dc_fixed[s] / fixed_scale[f] : st->dc[s];
    if (f == 0 && mean_sub_a) v -= ngrid;
    dcv[s] = v;
  }
}

// The fused bin kernel. grid: x = column blocks over the flattened (y, z) columns of the
// half-complex grid, y = chunks of the x axis.
template <typename R>
__global__ void __launch_bounds__(256) k_bin(BinParams bp, BinTables t, const typename CT<R>::C *g0,
                                             const typename CT<R>::C *g1, const typename CT<R>::C *g2,
                                             const typename CT<R>::C *g3, const double *dcv, double *bins,
                                             double *bins2d, int ichunk) {
  typedef typename CT<R>::C C;
  extern __shared__ __align__(16) unsigned char smraw[];
  R *sb = (R *)smraw;                       // [nspec][5][NK]
  R *sb2 = sb + bp.nspec * 5 * bp.nk;       // [nspec][NK*NMU] when out2d fits
  const int nk = bp.nk, ns = bp.nspec, nf = bp.nfields;
  const int n2d = bp.out2d ? nk * bp.nmu : 0;
  const bool sm2d_fit = n2d * ns * sizeof(R) + 5 * nk * ns * sizeof(R) <= 96 * 1024;
  for (int c = threadIdx.x; c < ns * (5 * nk + (sm2d_fit ? n2d : 0)); c += blockDim.x) sb[c] = (R)0;
  __syncthreads();

  const long long cols = (long long)bp.ny * bp.nzc;
  const long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int i0 = blockIdx.y * ichunk, i1 = min(bp.nx, i0 + ichunk);
  if (col < cols) {
    const int j = (int)(col / bp.nzc), k = (int)(col - (long long)j * bp.nzc);
    const bool isf = sizeof(R) == 4;
    // per-column constants
    const R syz = isf ? (R)(t.fy2f[j] + t.fz2f[k]) : (R)0;
    R cyz = isf ? (R)(t.cyf[j] * t.czf[k]) : (R)(t.cyd[j] * t.czd[k]);
    if (bp.interlace) cyz *= (R)0.25;
    C eyz;
    if (isf) {
      float2 a = t.eyf[j], b = t.ezf[k];
      eyz.x = (R)(a.x * b.x - a.y * b.y);
      eyz.y = (R)(a.x * b.y + a.y * b.x);
    } else {
      double2 a = t.eyd[j], b = t.ezd[k];
      eyz.x = (R)(a.x * b.x - a.y * b.y);
      eyz.y = (R)(a.x * b.y + a.y * b.x);
    }
    const R flos_yz = bp.los == 2 ? (isf ? (R)t.fyf[j] : (R)t.fyd[j]) : (isf ? (R)t.fzf[k] : (R)t.fzd[k]);
    const long long base = (long long)j * bp.nzc + k;
    R acc[CAPOW_MAX_SPEC][5];
#pragma unroll
    for (int q = 0; q < CAPOW_MAX_SPEC; q++)
#pragma unroll
      for (int l = 0; l < 5; l++) acc[q][l] = (R)0;
    int cur = -1;
    int guess = 0;
    for (int i = i0; i < i1; i++) {
      // ---- bin of this mode
      int b;
      double sd = -1.0;
      if (isf) {
        const float s32 = t.fx2f[i] + (float)syz;
        b = guess;
        while (b < nk && s32 >= t.Elo[b + 2]) b++;
        while (b > -1 && s32 < t.Ehi[b + 1]) b--;
        // safe iff s32 lies inside [Elo[b+1], Ehi[b+2])
        if (!(s32 >= t.Elo[b + 1] && s32 < t.Ehi[b + 2])) {
          sd = exact_s(t, i, j, k);
          b = exact_bin(t.E, nk, sd, b);
        }
      } else {
        sd = exact_s(t, i, j, k);
        b = exact_bin(t.E, nk, sd, guess);
      }
      guess = b;
      if (b < 0 || b >= nk) continue;
      if (b != cur) {
        if (cur >= 0) {
          for (int q = 0; q < ns; q++)
            for (int l = 0; l < 5; l++) {
              if (acc[q][l] != (R)0) atomicAdd(&sb[(q * 5 + l) * nk + cur], acc[q][l]);
              acc[q][l] = (R)0;
            }
        }
        cur = b;
      }
      // ---- fields at this mode, interlacing combine (src/main.c:392-418)
      const long long off = (long long)i * cols + base;
      C F[2];
      const C *gs[4] = {g0, g1, g2, g3};
      C e;
      if (isf) {
        float2 ex = t.exf[i];
        e.x = (R)ex.x * eyz.x - (R)ex.y * eyz.y;
        e.y = (R)ex.x * eyz.y + (R)ex.y * eyz.x;
      } else {
        double2 ex = t.exd[i];
        e.x = (R)ex.x * eyz.x - (R)ex.y * eyz.y;
        e.y = (R)ex.x * eyz.y + (R)ex.y * eyz.x;
      }
      const bool dc = (i == 0 && col == 0);
      for (int f = 0; f < nf; f++) {
        C a = gs[f][off];
        if (dc) { a.x = (R)dcv[f]; a.y = (R)0; }
        if (bp.interlace) {
          C ai = gs[nf + f][off];
          if (dc) { ai.x = (R)dcv[nf + f]; ai.y = (R)0; }
          C r = cmul(ai, e);
          a.x += r.x;
          a.y += r.y;
        }
        F[f] = a;
      }
      // ---- weights: deconvolution, Hermitian multiplicity, Legendre (src/main.c:382-389, 422-449)
      const R cx = isf ? (R)t.cxf[i] : (R)t.cxd[i];
      const R gc = cyz * cx * (R)herm_nm(i, j, k, bp.xhalf);
      R mu;
      const R fl = bp.los == 1 ? (isf ? (R)t.fxf[i] : (R)t.fxd[i]) : flos_yz;
      if (isf) {
        const float s32 = t.fx2f[i] + (float)syz;
        mu = s32 > 0.0f ? (R)((float)fl * rsqrtf(s32)) : (R)0;
      } else {
        double sq = sqrt(sd);
        mu = sq > 0.0 ? (R)(fl / sq) : (R)0;
      }
      const R mu2 = mu * mu;
      const R L2 = (R)1.5 * mu2 - (R)0.5;
      const R L4 = ((R)4.375 * mu2 - (R)3.75) * mu2 + (R)0.375;
      const R L3 = ((R)2.5 * mu2 - (R)1.5) * mu;
      for (int q = 0; q < ns; q++) {
        const C X = F[bp.spec[q].x], Y = F[bp.spec[q].y];
        R pw = bp.spec[q].imag ? (X.x * Y.y - X.y * Y.x) : (X.x * Y.x + X.y * Y.y);
        pw *= gc;
        acc[q][0] += pw;
        acc[q][2] += pw * L2;
        acc[q][4] += pw * L4;
        if (bp.odd) {
          acc[q][1] += pw * mu;
          acc[q][3] += pw * L3;
        }
        if (bp.out2d) {
          int mb;
          const R tq = (mu + (R)1) * (R)0.5 * (R)bp.nmu;
          const R fr = tq - floor(tq);
          if (isf && (fr < (R)1e-4 || fr > (R)(1 - 1e-4))) {
            if (sd < 0) sd = exact_s(t, i, j, k);
            mb = exact_mubin(bp, t, i, j, k, sd);
          } else if (!isf) {
            mb = exact_mubin(bp, t, i, j, k, sd);
          } else {
            mb = (int)tq;
            if (mb >= bp.nmu) mb = bp.nmu - 1;
          }
          const int bin = b * bp.nmu + mb;
          if (bin >= 0 && bin < n2d) {
            if (sm2d_fit)
              atomicAdd(&sb2[q * n2d + bin], pw);
            else
              atomicAdd(&bins2d[q * n2d + bin], (double)pw);
          }
        }
      }
    }
    if (cur >= 0)
      for (int q = 0; q < ns; q++)
        for (int l = 0; l < 5; l++)
          if (acc[q][l] != (R)0) atomicAdd(&sb[(q * 5 + l) * nk + cur], acc[q][l]);
  }
  __syncthreads();
  const bool sm2d = n2d * ns * sizeof(R) + 5 * nk * ns * sizeof(R) <= 96 * 1024;
  for (int c = threadIdx.x; c < ns * 5 * nk; c += blockDim.x) {
    R v = sb[c];
    if (v != (R)0) atomicAdd(&bins[c], (double)v);
  }
  if (bp.out2d && sm2d)
    for (int c = 0 + threadIdx.x; c < ns * n2d; c += blockDim.x) {
      R v = sb2[c];
      if (v != (R)0) atomicAdd(&bins2d[c], (double)v);
    }
}

void launch_mode_counts(cudaStream_t s, const BinParams &bp, const BinTables &t, unsigned long long *nmodes,
                        unsigned long long *nmodes2d, long long *launches) {
  const size_t smem = sizeof(unsigned long long) * (bp.nk + (bp.out2d ? bp.nk * bp.nmu : 0));
  cudaFuncSetAttribute(k_mode_counts, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_mode_counts<<<152 * 4, 256, smem, s>>>(bp, t, nmodes, nmodes2d);
  (*launches)++;
}

void launch_dc_prepare(cudaStream_t s, const void *st, int deterministic, int nslot, int nfields, int mean_sub_a,
                       const double *fixed_scale, double *dcv, long long *launches) {
  k_dc_prepare<<<1, 1, 0, s>>>((const DevStats *)st, deterministic, nslot, nfields, mean_sub_a, fixed_scale, dcv);
  (*launches)++;
}

void launch_bin(cudaStream_t s, int precision, const BinParams &bp, const BinTables &t, void *const slots[4],
                const double *dcv, double *bins, double *bins2d, long long *launches) {
  const long long cols = (long long)bp.ny * bp.nzc;
  const int th = 256;
  const int nbx = (int)((cols + th - 1) / th);
  // enough CTAs to fill the GPU several times over, each thread walking a chunk of x
  int nchunk = (152 * 8 + nbx - 1) / nbx;
  if (nchunk < 1) nchunk = 1;
  if (nchunk > bp.nx) nchunk = bp.nx;
  const int ichunk = (bp.nx + nchunk - 1) / nchunk;
  nchunk = (bp.nx + ichunk - 1) / ichunk;
  dim3 grid(nbx, nchunk);
  const int n2d = bp.out2d ? bp.nk * bp.nmu : 0;
  if (precision == CAPOW_FP64) {
    size_t eb = sizeof(double);
    bool sm2d = n2d * bp.nspec * eb + 5 * bp.nk * bp.nspec * eb <= 96 * 1024;
    size_t smem = eb * bp.nspec * (5 * bp.nk + (sm2d ? n2d : 0));
    cudaFuncSetAttribute(k_bin<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_bin<double><<<grid, th, smem, s>>>(bp, t, (const double2 *)slots[0], (const double2 *)slots[1],
                                         (const double2 *)slots[2], (const double2 *)slots[3], dcv, bins, bins2d,
                                         ichunk);
  } else {
    size_t eb = sizeof(float);
    bool sm2d = n2d * bp.nspec * eb + 5 * bp.nk * bp.nspec * eb <= 96 * 1024;
    size_t smem = eb * bp.nspec * (5 * bp.nk + (sm2d ? n2d : 0));
    cudaFuncSetAttribute(k_bin<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_bin<float><<<grid, th, smem, s>>>(bp, t, (const float2 *)slots[0], (const float2 *)slots[1],
                                        (const float2 *)slots[2], (const float2 *)slots[3], dcv, bins, bins2d, ichunk);
  }
  (*launches)++;
}
