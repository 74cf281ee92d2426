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
#include "harm.cuh"
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

// When set, upload() appends to this host blob instead (16-byte aligned) and returns the offset as
// a pointer; relocate_bin_tables then rebases every table on the blob's device copy.
static thread_local std::vector<unsigned char> *g_pack = nullptr;

template <typename T>
static T *upload(const std::vector<T> &h, std::vector<void *> &allocs, cudaStream_t s) {
  if (g_pack) {
    size_t off = (g_pack->size() + 15) & ~(size_t)15;
    if (off == 0) off = 16;  // no table at offset 0: a null pointer means "missing"
    g_pack->resize(off + sizeof(T) * (h.size() ? h.size() : 1), 0);
    if (!h.empty()) memcpy(g_pack->data() + off, h.data(), sizeof(T) * h.size());
    return (T *)(uintptr_t)off;
  }
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
  t.twx = nullptr;
  if (nx >= 2 && (nx & (nx - 1)) == 0) {  // twiddles of the fused x-axis FFT (forward, sign -1)
    std::vector<float2> tw(nx);
    for (int q = 0; q < nx; q++) {
      const double a = -2.0 * M_PI * (double)q / (double)nx;
      tw[q] = make_float2((float)cos(a), (float)sin(a));
    }
    t.twx = upload(tw, allocs, s);
    if (!t.twx) return 1;
  }
  t.twy = nullptr;
  if (ny >= 16 && ny <= 2048 && (ny & (ny - 1)) == 0) {  // y pass of the one-launch z + y transform
    std::vector<float2> tw(ny);
    for (int q = 0; q < ny; q++) {
      const double a = -2.0 * M_PI * (double)q / (double)ny;
      tw[q] = make_float2((float)cos(a), (float)sin(a));
    }
    t.twy = upload(tw, allocs, s);
    if (!t.twy) return 1;
  }
  t.twz = t.tpz = nullptr;
  const int nzp = p.NZ;
  if (nzp >= 32 && nzp <= 2048 && (nzp & (nzp - 1)) == 0) {  // z pass of the transposed fused path
    const int m = nzp / 2;
    std::vector<float2> tz(m), tp(m + 1);
    for (int q = 0; q < m; q++) {
      const double a = -2.0 * M_PI * (double)q / (double)m;
      tz[q] = make_float2((float)cos(a), (float)sin(a));
    }
    for (int k = 0; k <= m; k++) {
      const double a = -2.0 * M_PI * (double)k / (double)nzp;
      tp[k] = make_float2((float)cos(a), (float)sin(a));
    }
    t.twz = upload(tz, allocs, s);
    t.tpz = upload(tp, allocs, s);
    if (!t.twz || !t.tpz) return 1;
  }
  return (t.E && t.Elo && t.Ehi && t.ezf) ? 0 : 1;
}

int build_bin_tables_packed(const capow_params &p, const Geom &g, int precision, BinTables &t,
                            std::vector<unsigned char> &blob) {
  std::vector<void *> none;
  g_pack = &blob;
  const int rc = build_bin_tables(p, g, precision, t, none, nullptr);
  g_pack = nullptr;
  return rc;
}

void relocate_bin_tables(BinTables &t, const void *base) {
  void **f[] = {(void **)&t.fx2d, (void **)&t.fy2d, (void **)&t.fz2d, (void **)&t.fx2f, (void **)&t.fy2f,
                (void **)&t.fz2f, (void **)&t.fxd,  (void **)&t.fyd,  (void **)&t.fzd,  (void **)&t.fxf,
                (void **)&t.fyf,  (void **)&t.fzf,  (void **)&t.cxd,  (void **)&t.cyd,  (void **)&t.czd,
                (void **)&t.cxf,  (void **)&t.cyf,  (void **)&t.czf,  (void **)&t.exd,  (void **)&t.eyd,
                (void **)&t.ezd,  (void **)&t.exf,  (void **)&t.eyf,  (void **)&t.ezf,  (void **)&t.E,
                (void **)&t.Elo,  (void **)&t.Ehi,  (void **)&t.twx,  (void **)&t.twz,  (void **)&t.tpz,
                (void **)&t.twy};
  for (void **q : f)
    if (*q) *q = (void *)((const char *)base + (uintptr_t)*q);
}

// ---------------------------------------------------------------------------------- device side

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

// Shared-memory carving of k_bin, used by the kernel and by its launcher. Every region starts
// on a 16-byte boundary (double2 tables and double edges need 16 and 8).
struct BinSmem {
  unsigned sb, sb2, sE, sElo, sEhi, sfx2, scx, sex, sfl, total;
};

CAPOW_HD unsigned align16(unsigned x) { return (x + 15u) & ~15u; }

CAPOW_HD BinSmem bin_smem_layout(unsigned rsize, int np, int nk, int n2d_sm, int ichunk) {
  BinSmem L;
  unsigned o = 0;
  L.sb = o;   o = align16(o + rsize * np * 5 * nk);
  L.sb2 = o;  o = align16(o + rsize * np * n2d_sm);
  L.sE = o;   o = align16(o + 8u * (nk + 3));
  L.sElo = o; o = align16(o + 4u * (nk + 3));
  L.sEhi = o; o = align16(o + 4u * (nk + 3));
  L.sfx2 = o; o = align16(o + rsize * ichunk);
  L.scx = o;  o = align16(o + rsize * ichunk);
  L.sex = o;  o = align16(o + 2u * rsize * ichunk);
  L.sfl = o;  o = align16(o + rsize * ichunk);
  L.total = o;
  return L;
}

// The fused bin kernel. grid.x: blocks of flattened (y, z) columns of the half-complex grid;
// grid.y: chunks of the x axis. Each thread walks x for one (y, z) column.
//
// NF = 1: one painted field (A, and A interlaced); product |A|^2.
// NF = 2: fields A and B; products |A|^2, Re(A* B), Im(A* B), |B|^2 are all accumulated and
//         each requested spectrum reads one of them (src/main.c:435-441).
// ODD: also the odd multipoles (src/main.c:445-449). OUT2D: the (k, mu) histogram (:453-461).
// All accumulator indexing is compile-time, so the per-thread sums live in registers.
template <typename R, int NF, bool ODD, bool OUT2D>
__global__ void __launch_bounds__(256) k_bin(BinParams bp, BinTables t, const typename CT<R>::C *gA,
                                             const typename CT<R>::C *gB, const typename CT<R>::C *gAi,
                                             const typename CT<R>::C *gBi, const double *dcv, double *bins,
                                             double *bins2d, int ichunk, int sm2d) {
  typedef typename CT<R>::C C;
  constexpr int NP = NF == 1 ? 1 : 4;
  constexpr bool F32 = sizeof(R) == 4;
  const int nk = bp.nk;
  const int n2d = OUT2D ? nk * bp.nmu : 0;
  extern __shared__ __align__(16) unsigned char smraw[];
  // shared layout: bins [NP][5][nk] | 2-D bins [NP][n2d] | E (double, nk+3) | Elo, Ehi (float, nk+3)
  //                | per-chunk x tables: fx2 (R), cx (R), ex (C), fl (R)
  const BinSmem L = bin_smem_layout(sizeof(R), NP, nk, sm2d ? n2d : 0, ichunk);
  R *sb = (R *)(smraw + L.sb);
  R *sb2 = (R *)(smraw + L.sb2);
  double *sE = (double *)(smraw + L.sE);
  float *sElo = (float *)(smraw + L.sElo);
  float *sEhi = (float *)(smraw + L.sEhi);
  R *sfx2 = (R *)(smraw + L.sfx2);
  R *scx = (R *)(smraw + L.scx);
  C *sex = (C *)(smraw + L.sex);
  R *sfl = (R *)(smraw + L.sfl);
  const int i0 = blockIdx.y * ichunk, i1 = min(bp.nx, i0 + ichunk);
  for (int c = threadIdx.x; c < NP * (5 * nk + (sm2d ? n2d : 0)); c += blockDim.x) sb[c] = (R)0;
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
      sex[c].x = (R)t.exf[i].x;
      sex[c].y = (R)t.exf[i].y;
      sfl[c] = (R)t.fxf[i];
    } else {
      sfx2[c] = (R)t.fx2d[i];
      scx[c] = (R)t.cxd[i];
      sex[c].x = (R)t.exd[i].x;
      sex[c].y = (R)t.exd[i].y;
      sfl[c] = (R)t.fxd[i];
    }
  }
  __syncthreads();

  const long long cols = (long long)bp.ny * bp.nzc;
  const long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  // DC values converted once per thread (for R = float each conversion is an FP64-pipe slot)
  const int nsl = NF * (bp.interlace ? 2 : 1);
  const R dc0 = (R)dcv[0], dc1 = nsl > 1 ? (R)dcv[1] : (R)0, dc2 = nsl > 2 ? (R)dcv[2] : (R)0,
          dc3 = nsl > 3 ? (R)dcv[3] : (R)0;
  if (col < cols) {
    const int j = (int)(col / bp.nzc), k = (int)(col - (long long)j * bp.nzc);
    // per-column constants
    const R syz = F32 ? (R)(t.fy2f[j] + t.fz2f[k]) : (R)0;
    const double fyz2d_y = t.fy2d[j], fyz2d_z = t.fz2d[k];
    R cyz = F32 ? (R)(t.cyf[j] * t.czf[k]) : (R)(t.cyd[j] * t.czd[k]);
    if (bp.interlace) cyz *= (R)0.25;
    C eyz;
    if (F32) {
      const float2 a = t.eyf[j], b = t.ezf[k];
      eyz.x = (R)(a.x * b.x - a.y * b.y);
      eyz.y = (R)(a.x * b.y + a.y * b.x);
    } else {
      const double2 a = t.eyd[j], b = t.ezd[k];
      eyz.x = (R)(a.x * b.x - a.y * b.y);
      eyz.y = (R)(a.x * b.y + a.y * b.x);
    }
    const R flos_yz = bp.los == 2 ? (F32 ? (R)t.fyf[j] : (R)t.fyd[j]) : (F32 ? (R)t.fzf[k] : (R)t.fzd[k]);
    const long long base = (long long)j * bp.nzc + k;
    R acc[NP][5];
#pragma unroll
    for (int q = 0; q < NP; q++)
#pragma unroll
      for (int l = 0; l < 5; l++) acc[q][l] = (R)0;
    int cur = -1;
    R lo = (R)1, hi = (R)0;  // current bin's safe interval in s (empty: search)
    // modes of this column with |fx| beyond the top bin edge (or Nyquist) are never included:
    // walk only i <= r and i >= NX - r (r rounded up; the exact test below decides each mode)
    const float top = sElo[nk + 1] - (float)(F32 ? (float)syz : (float)(fyz2d_y + fyz2d_z));
    const int r = top > 0.0f ? min(bp.xhalf, (int)(sqrtf(top) / bp.fx_step) + 1) : -1;
    for (int i = i0; i < i1; i++) {
      if (i > r && i < bp.nx - r) {
        i = bp.nx - r - 1;
        continue;
      }
      const int li = i - i0;
      // ---- bin of this mode (src/main.c:355, 369-375)
      R s;
      if (F32) s = sfx2[li] + syz;
      else s = (R)__dadd_rn(__dadd_rn((double)sfx2[li], fyz2d_y), fyz2d_z);
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
            const double sd = __dadd_rn(__dadd_rn(t.fx2d[i], fyz2d_y), fyz2d_z);
            b = exact_bin(sE, nk, sd, b);
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
#pragma unroll
            for (int q = 0; q < NP; q++)
#pragma unroll
              for (int l = 0; l < 5; l++) {
                if ((l == 1 || l == 3) && !ODD) continue;
                if (acc[q][l] != (R)0) atomicAdd(&sb[(q * 5 + l) * nk + cur], acc[q][l]);
                acc[q][l] = (R)0;
              }
          }
          cur = b;
        }
      }
      if (cur < 0 || cur >= nk) continue;
      // ---- fields and interlacing combine (src/main.c:392-418)
      const long long off = (long long)i * cols + base;
      const bool dc = (i == 0 && col == 0);
      C ex = sex[li], e;
      e.x = ex.x * eyz.x - ex.y * eyz.y;
      e.y = ex.x * eyz.y + ex.y * eyz.x;
      C A = gA[off];
      if (dc) { A.x = dc0; A.y = (R)0; }
      C B;
      if (NF == 2) {
        B = gB[off];
        if (dc) { B.x = dc1; B.y = (R)0; }
      }
      if (bp.interlace) {
        C a = gAi[off];
        if (dc) { a.x = NF == 2 ? dc2 : dc1; a.y = (R)0; }
        A.x += a.x * e.x - a.y * e.y;
        A.y += a.x * e.y + a.y * e.x;
        if (NF == 2) {
          C b2 = gBi[off];
          if (dc) { b2.x = dc3; b2.y = (R)0; }
          B.x += b2.x * e.x - b2.y * e.y;
          B.y += b2.x * e.y + b2.y * e.x;
        }
      }
      // ---- weights (src/main.c:382-389, 422-449)
      const R gc = cyz * scx[li] * (R)herm_nm(i, j, k, bp.xhalf);
      const R fl = bp.los == 1 ? sfl[li] : flos_yz;
      R mu;
      if (F32) mu = s > (R)0 ? (R)((float)fl * rsqrtf((float)s)) : (R)0;
      else mu = s > (R)0 ? (R)(fl / sqrt((double)s)) : (R)0;
      const R mu2 = mu * mu;
      const R L2 = (R)1.5 * mu2 - (R)0.5;
      const R L4 = ((R)4.375 * mu2 - (R)3.75) * mu2 + (R)0.375;
      const R L3 = ((R)2.5 * mu2 - (R)1.5) * mu;
      R P[NP];
      P[0] = (A.x * A.x + A.y * A.y) * gc;
      if (NF == 2) {
        P[1] = (A.x * B.x + A.y * B.y) * gc;
        P[2] = (A.x * B.y - A.y * B.x) * gc;
        P[3] = (B.x * B.x + B.y * B.y) * gc;
      }
#pragma unroll
      for (int q = 0; q < NP; q++) {
        if (!(bp.pmask & (1 << q))) continue;  // a product no requested spectrum reads
        acc[q][0] += P[q];
        acc[q][2] += P[q] * L2;
        acc[q][4] += P[q] * L4;
        if (ODD) {
          acc[q][1] += P[q] * mu;
          acc[q][3] += P[q] * L3;
        }
      }
      if (OUT2D) {
        int mb;
        const R tq = (mu + (R)1) * (R)0.5 * (R)bp.nmu;
        const R fr = tq - floor(tq);
        if (!F32 || fr < (R)1e-4 || fr > (R)(1 - 1e-4)) {
          const double sd = __dadd_rn(__dadd_rn(t.fx2d[i], fyz2d_y), fyz2d_z);
          mb = exact_mubin(bp, t, i, j, k, sd);
        } else {
          mb = (int)tq;
          if (mb >= bp.nmu) mb = bp.nmu - 1;
        }
        const int bin = cur * bp.nmu + mb;
        if (bin >= 0 && bin < n2d) {
#pragma unroll
          for (int q = 0; q < NP; q++) {
            if (sm2d) atomicAdd(&sb2[q * n2d + bin], P[q]);
            else atomicAdd(&bins2d[q * n2d + bin], (double)P[q]);
          }
        }
      }
    }
    if (cur >= 0 && cur < nk) {
#pragma unroll
      for (int q = 0; q < NP; q++)
#pragma unroll
        for (int l = 0; l < 5; l++) {
          if ((l == 1 || l == 3) && !ODD) continue;
          if (acc[q][l] != (R)0) atomicAdd(&sb[(q * 5 + l) * nk + cur], acc[q][l]);
        }
    }
  }
  __syncthreads();
  // CTA bins -> global FP64 bins, laid out [product][5][nk]
  for (int c = threadIdx.x; c < NP * 5 * nk; c += blockDim.x) {
    const R v = sb[c];
    if (v != (R)0) atomicAdd(&bins[c], (double)v);
  }
  if (OUT2D && sm2d)
    for (int c = threadIdx.x; c < NP * n2d; c += blockDim.x) {
      const R v = sb2[c];
      if (v != (R)0) atomicAdd(&bins2d[c], (double)v);
    }
}

// ------------------------------------------------------------ fused x-axis FFT + binning (FP32)
// Every x-plane of every grid has been transformed over (y, z) (by cuFFT in place, or by k_zr2c and
// the y-axis C2C into the transposed layout); what is left of the 3-D transform (src/main.c:266-271)
// is the length-NX DFT along x of every (ky, kz) column, and its only consumer is the binning
// (src/main.c:302-468). One pass does both: a CTA transforms a block of columns along x in shared
// memory and bins the modes from there, so the x-transformed grids never go to HBM. Columns whose
// smallest |k| lies beyond the top k-bin edge are not loaded.
//
// A block is `kc` consecutive inner indices (kz of one ky, or ky of one kz on the transposed layout)
// in each of the nslot grids: 8 of them (64 contiguous bytes of every x-row of every grid) for
// NX <= 512. One CTA of XBIN_THREADS threads per SM. The first radix-8 stage reads its inputs
// straight from HBM; the others work in shared memory, where row x holds the block's ncol columns
// (c = slot * kc + inner - first inner) with a pitch of ncol + 1: a butterfly's rows are one base
// plus a fixed stride, a warp's accesses are whole rows, and the pad spreads the rows the binning
// reads at once over the banks.
constexpr int XBIN_THREADS = 1024;

struct XbinSmem {
  unsigned sd, stw, sxt, sfx, sb, sbd, scol, srow, sE, sElo, sEhi, total;
};

// Per-column quantities of the block being binned (one entry per inner index of the block), written
// by kc threads during the first FFT stage: everything of a mode that does not depend on kx.
struct XCol {
  float syz;    // fy^2 + fz^2 (FP32)
  float cyzn;   // y, z deconvolution factors, x 0.25 when interlaced, x 2 off the kz = 0 plane (NM)
  float flos;   // mu numerator when the LOS is y or z (fy or fz)
  int r;        // |kx| index beyond which no mode reaches the top bin edge (-1: none does)
  float2 eyz;   // y, z interlace phase
  int j, kz;    // ky index (-1: inner index beyond the grid), kz index
};

// Twiddle-table entries of the radix-8 stages that have more than one butterfly per group: a
// stage of span 2^l has 2^(l-3) of them, each with its 8 factors w^(p jj NX/span), p < 8.
CAPOW_HD unsigned xbin_tw_entries(int log2n) {
  unsigned e = 0;
  for (int l = log2n; l >= 4; l -= 3) e += 8u << (l - 3);
  return e;
}

// Position in the x-table of kx index i: one pad entry per 64 spreads the starts of the binning
// runs over the banks.
__device__ __forceinline__ int xt_index(int i) { return i + (i >> 6); }

CAPOW_HD XbinSmem xbin_smem_layout(int log2n, int ncol, int np, int nl, int nk, int nbc) {
  const unsigned n = 1u << log2n;
  XbinSmem L;
  unsigned o = 0;
  L.sd = o;   o = align16(o + 8u * n * (ncol + 1));
  L.stw = o;  o = align16(o + 8u * xbin_tw_entries(log2n));
  L.sxt = o;  o = align16(o + 16u * (n + (n >> 6) + 1));
  L.sfx = o;  o = align16(o + 4u * n);
  L.sb = o;   o = align16(o + 4u * np * nl * nk * nbc);
  L.sbd = o;  o = align16(o + 8u * np * nl * nk);
  L.scol = o; o = align16(o + (unsigned)sizeof(XCol) * ncol);
  L.srow = o; o = align16(o + 4u * n);
  L.sE = o;   o = align16(o + 8u * (nk + 3));
  L.sElo = o; o = align16(o + 4u * (nk + 3));
  L.sEhi = o; o = align16(o + 4u * (nk + 3));
  L.total = o;
  return L;
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmul_mi(float2 a) { return make_float2(a.y, -a.x); }  // a * (-i)

// A column element read once: no L1 allocation, and an L2 fetch of the surrounding 256 bytes (the
// neighbouring kz blocks of the same row, which other CTAs read next).
__device__ __forceinline__ float2 ld_col(const float2 *p) {
  float2 v;
  asm("ld.global.nc.L1::no_allocate.L2::256B.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
  return v;
}

// In-place DIF butterflies of one stage, forward sign. Inputs a[q] at span/R spacing; outputs X[p]
// (p in natural order) times the twiddle w^(p*j) are written back at position p.
__device__ __forceinline__ void dft8(float2 *a) {
  const float h = 0.70710678118654752f;
  float2 b0 = cadd(a[0], a[4]), b4 = csub(a[0], a[4]);
  float2 b1 = cadd(a[1], a[5]), t5 = csub(a[1], a[5]);
  float2 b2 = cadd(a[2], a[6]), t6 = csub(a[2], a[6]);
  float2 b3 = cadd(a[3], a[7]), t7 = csub(a[3], a[7]);
  const float2 b5 = make_float2((t5.x + t5.y) * h, (t5.y - t5.x) * h);    // * e^{-i pi/4}
  const float2 b6 = cmul_mi(t6);                                           // * e^{-i pi/2}
  const float2 b7 = make_float2((t7.y - t7.x) * h, -(t7.x + t7.y) * h);   // * e^{-3i pi/4}
  const float2 c0 = cadd(b0, b2), c2 = csub(b0, b2), c1 = cadd(b1, b3), c3 = cmul_mi(csub(b1, b3));
  const float2 c4 = cadd(b4, b6), c6 = csub(b4, b6), c5 = cadd(b5, b7), c7 = cmul_mi(csub(b5, b7));
  a[0] = cadd(c0, c1);
  a[4] = csub(c0, c1);
  a[2] = cadd(c2, c3);
  a[6] = csub(c2, c3);
  a[1] = cadd(c4, c5);
  a[5] = csub(c4, c5);
  a[3] = cadd(c6, c7);
  a[7] = csub(c6, c7);
}

__device__ __forceinline__ void dft4(float2 *a) {
  const float2 b0 = cadd(a[0], a[2]), b2 = csub(a[0], a[2]), b1 = cadd(a[1], a[3]), b3 = cmul_mi(csub(a[1], a[3]));
  a[0] = cadd(b0, b1);
  a[2] = csub(b0, b1);
  a[1] = cadd(b2, b3);
  a[3] = csub(b2, b3);
}

// a[p] *= w[p], p = 1..7, w one 16-byte aligned row of a stage's twiddle table (w[0] = 1)
__device__ __forceinline__ void twiddle8(float2 *a, const float2 *w) {
  const float4 *w4 = (const float4 *)w;
  const float4 t01 = w4[0], t23 = w4[1], t45 = w4[2], t67 = w4[3];
  a[1] = cmulf(a[1], make_float2(t01.z, t01.w));
  a[2] = cmulf(a[2], make_float2(t23.x, t23.y));
  a[3] = cmulf(a[3], make_float2(t23.z, t23.w));
  a[4] = cmulf(a[4], make_float2(t45.x, t45.y));
  a[5] = cmulf(a[5], make_float2(t45.z, t45.w));
  a[6] = cmulf(a[6], make_float2(t67.x, t67.y));
  a[7] = cmulf(a[7], make_float2(t67.z, t67.w));
}

// Position along x, after the in-place DIF stages (log2n / 3 of radix 8, then one of radix
// 2^(log2n % 3) when that is not 1), of frequency index i: its base-8 digits reversed.
__device__ __forceinline__ int xfft_pos(int log2n, int i) {
  int pos = 0, shift = log2n, rem = i;
  for (int st = 0; st < log2n / 3; st++) {
    shift -= 3;
    pos += (rem & 7) << shift;
    rem >>= 3;
  }
  return pos + rem;  // the last digit has span 1
}

// First guess of the bin of an FP32 s (linear bins: from sqrtf(s); log bins: bisection over the safe
// edges). It only starts the walk over the safe edges, which ends on the same bin from any start.
__device__ __forceinline__ int guess_bin(const BinParams &bp, const float *sElo, float s) {
  const int nk = bp.nk;
  if (!bp.lg) {
    const float v = sqrtf(s) * bp.kscale + bp.koff;
    return v < 0.0f ? -1 : (v >= (float)nk ? nk : (int)v);
  }
  int a = 0, z = nk + 2;  // sElo[a] <= s < sElo[z] (sElo[0] = -inf, sElo[nk + 2] = +inf)
  while (z - a > 1) {
    const int mid = (a + z) >> 1;
    if (sElo[mid] <= s) a = mid;
    else z = mid;
  }
  return a - 1;
}

// PM: the products accumulated (bit q: |A|^2, Re A*B, Im A*B, |B|^2); the launcher passes a superset
// of the products the spectra read.
template <int NF, bool IL, bool ODD, int PM>
__global__ void __launch_bounds__(XBIN_THREADS) k_xfft_bin(BinParams bp, BinTables t, XbinGeo xg, const float2 *g0,
                                                           const float2 *g1, const float2 *g2, const float2 *g3,
                                                           const double *dcv, double *bins) {
  constexpr int NS = NF * (IL ? 2 : 1);
  constexpr int NP = NF == 1 ? 1 : 4;
  constexpr int NL = ODD ? 5 : 3;  // stored multipoles: l = 0, 2, 4 (+ 1, 3)
  extern __shared__ __align__(16) unsigned char smraw[];
  const int log2n = xg.log2n, n = 1 << log2n, ncol = xg.ncol, kc_n = xg.kc, nk = bp.nk;
  const int P = ncol + 1;  // row pitch of sd
  const XbinSmem L = xbin_smem_layout(log2n, ncol, NP, NL, nk, xg.nbc);
  float2 *sd = (float2 *)(smraw + L.sd);
  float2 *stw = (float2 *)(smraw + L.stw);
  float4 *sxt = (float4 *)(smraw + L.sxt);  // per kx: fx^2, deconvolution factor, interlace phase
  float *sfx = (float *)(smraw + L.sfx);    // per kx: fx (the mu numerator when LOS = x)
  float *sb = (float *)(smraw + L.sb);      // this block's bins, FP32, xg.nbc copies
  double *sbd = (double *)(smraw + L.sbd);  // the CTA's bins, FP64
  XCol *scol = (XCol *)(smraw + L.scol);
  int *srow = (int *)(smraw + L.srow);
  double *sE = (double *)(smraw + L.sE);
  float *sElo = (float *)(smraw + L.sElo);
  float *sEhi = (float *)(smraw + L.sEhi);
  const int nbins = NP * NL * nk;
  for (int c = threadIdx.x; c < nbins * xg.nbc; c += blockDim.x) sb[c] = 0.0f;
  for (int c = threadIdx.x; c < nbins; c += blockDim.x) sbd[c] = 0.0;
  // this warp's copy of the block bins (flushes from different warps then rarely meet on one address)
  float *sbw = sb + ((threadIdx.x >> 5) & (xg.nbc - 1)) * nbins;
  for (int c = threadIdx.x; c < nk + 3; c += blockDim.x) {
    sE[c] = t.E[c];
    sElo[c] = t.Elo[c];
    sEhi[c] = t.Ehi[c];
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float2 e = IL ? t.exf[i] : make_float2(0.0f, 0.0f);
    sxt[xt_index(i)] = make_float4(t.fx2f[i], t.cxf[i], e.x, e.y);
    sfx[i] = t.fxf[i];
  }
  for (int l = log2n, off = 0; l >= 4; off += 8 << (l - 3), l -= 3) {
    const int step = n >> l;  // NX / span
    for (int e = threadIdx.x; e < (8 << (l - 3)); e += blockDim.x)
      stw[off + e] = t.twx[((e & 7) * (e >> 3) * step) & (n - 1)];
  }
  const float topf32 = (float)t.E[nk + 1] * 1.0001f;
  // binning work items: (kz column of the block, run of mpt consecutive kx), mpt <= 8 chosen so that
  // the kc * NX / mpt items keep every thread busy. Within a column the run index is rotated by 3
  // bits, so that neighbouring lanes start runs far apart in x and their rows (digit-reversed)
  // spread over the shared-memory banks. srow[ch]: row of kx = ch * mpt after the DIF stages; the
  // digit reversal is a permutation of bit positions and the run's offsets m < mpt <= 8 have bits
  // disjoint from ch * mpt, so row(ch * mpt + m) = srow[ch] + m NX/8.
  const int log2mpt = min(3, max(0, log2n + xg.log2kc - (31 - __clz(blockDim.x))));
  const int mpt = 1 << log2mpt, log2nr = log2n - log2mpt, nitems = kc_n << log2nr;
  for (int ch = threadIdx.x; ch < (1 << log2nr); ch += blockDim.x) srow[ch] = xfft_pos(log2n, ch << log2mpt);
  const long long xstride = (long long)bp.ny * bp.nzc;  // = n_outer * n_inner
  const int Q1 = n >> 3, nbf1 = ncol << (log2n - 3);
  const long long qstep = (long long)Q1 * xstride;
  int nproc = 0;
  __syncthreads();
  for (int blk = blockIdx.x; blk < xg.nblocks; blk += gridDim.x) {
    const int bo = blk / xg.nkb, bi0 = (blk - bo * xg.nkb) * kc_n;  // outer index, first inner index
    // every mode of the block has s >= the block's smallest fy^2 + fz^2 (fz^2 grows with kz; fy^2
    // rises to ky = NY/2 and falls after it, so over a run of ky it is smallest at an end): skip the
    // block when that is clearly beyond the top edge (each kept mode is tested exactly)
    const float smin = xg.tr ? t.fz2f[bo] + fminf(t.fy2f[bi0], t.fy2f[min(bi0 + kc_n, bp.ny) - 1])
                             : t.fy2f[bo] + t.fz2f[bi0];
    if (smin > topf32) continue;
    __syncthreads();  // the previous block's binning has read sd and scol
    if (threadIdx.x < kc_n) {  // the block's column table (src/main.c:335-389 for the y, z factors)
      XCol col;
      const int inner = bi0 + threadIdx.x;
      if (inner < xg.n_inner) {
        const int j = xg.tr ? inner : bo, kz = xg.tr ? bo : inner;
        col.syz = t.fy2f[j] + t.fz2f[kz];
        float cyz = t.cyf[j] * t.czf[kz];
        if (IL) cyz *= 0.25f;
        col.cyzn = kz != 0 ? 2.0f * cyz : cyz;  // Hermitian multiplicity off the kz = 0 plane (:422-429)
        col.eyz = IL ? cmulf(t.eyf[j], t.ezf[kz]) : make_float2(0.0f, 0.0f);
        col.flos = bp.los == 2 ? t.fyf[j] : t.fzf[kz];
        const float topf = sElo[nk + 1] - col.syz;
        col.r = topf > 0.0f ? min(bp.xhalf, (int)(sqrtf(topf) / bp.fx_step) + 1) : -1;
        col.j = j;
        col.kz = kz;
      } else {
        col.syz = col.cyzn = col.flos = 0.0f;
        col.eyz = make_float2(0.0f, 0.0f);
        col.r = -1;
        col.j = -1;
        col.kz = 0;
      }
      scol[threadIdx.x] = col;
    }
    // first DIF stage (span NX) straight from HBM: butterfly (column c, jj) reads rows jj + q NX/8
    for (int u = threadIdx.x; u < nbf1; u += blockDim.x) {
      const int c = u & (ncol - 1), jj = u >> xg.log2ncol;
      const int sl = c >> xg.log2kc, inner = bi0 + (c & (kc_n - 1));
      const bool live = sl < NS && inner < xg.n_inner;
      const float2 *g = sl == 0 ? g0 : (sl == 1 ? g1 : (sl == 2 ? g2 : g3));
      const float2 *gp = g + (live ? (long long)jj * xstride + (long long)bo * xg.n_inner + inner : 0ll);
      float2 a[8];
#pragma unroll
      for (int q = 0; q < 8; q++) a[q] = live ? ld_col(gp + q * qstep) : make_float2(0.0f, 0.0f);
      dft8(a);
      if (jj > 0) twiddle8(a, stw + 8 * jj);
      float2 *p = sd + jj * P + c;
#pragma unroll
      for (int q = 0; q < 8; q++) p[q * Q1 * P] = a[q];
    }
    __syncthreads();
    int l = log2n - 3, twoff = 8 * Q1;
    for (; l >= 3; l -= 3) {  // the other radix-8 stages
      const int log2q = l - 3, Q = 1 << log2q, qs = Q * P;
      for (int u = threadIdx.x; u < nbf1; u += blockDim.x) {
        const int c = u & (ncol - 1), v = u >> xg.log2ncol;
        const int jj = v & (Q - 1);
        float2 *p = sd + (((v >> log2q) << l) + jj) * P + c;
        float2 a[8];
#pragma unroll
        for (int q = 0; q < 8; q++) a[q] = p[q * qs];
        dft8(a);
        if (jj > 0) twiddle8(a, stw + twoff + 8 * jj);
#pragma unroll
        for (int q = 0; q < 8; q++) p[q * qs] = a[q];
      }
      __syncthreads();
      if (Q > 1) twoff += 8 * Q;
    }
    if (l == 2) {  // a last radix-4 stage (span 4: no twiddles)
      for (int u = threadIdx.x; u < (ncol << (log2n - 2)); u += blockDim.x) {
        float2 *p = sd + ((u >> xg.log2ncol) << 2) * P + (u & (ncol - 1));
        float2 a[4];
#pragma unroll
        for (int q = 0; q < 4; q++) a[q] = p[q * P];
        dft4(a);
#pragma unroll
        for (int q = 0; q < 4; q++) p[q * P] = a[q];
      }
      __syncthreads();
    } else if (l == 1) {  // a last radix-2 stage
      for (int u = threadIdx.x; u < (ncol << (log2n - 1)); u += blockDim.x) {
        float2 *p = sd + ((u >> xg.log2ncol) << 1) * P + (u & (ncol - 1));
        const float2 a0 = p[0], a1 = p[P];
        p[0] = cadd(a0, a1);
        p[P] = csub(a0, a1);
      }
      __syncthreads();
    }
    // ---- binning (the math of k_bin, src/main.c:355-449), runs of consecutive kx
    for (int w = threadIdx.x; w < nitems; w += blockDim.x) {
      const int my_kc = w >> log2nr, rr = w & ((1 << log2nr) - 1);
      const int ch = log2nr >= 3 ? (((rr & 7) << (log2nr - 3)) | (rr >> 3)) : rr;
      const int i0 = ch << log2mpt;
      const XCol col = scol[my_kc];
      if (col.j < 0) continue;
      const int rowb = srow[ch];
      if (col.j == 0 && col.kz == 0 && i0 == 0) {  // the DC mode: the slots' exact DC values replace F(0)
        float2 *pd = sd + rowb * P + my_kc;
#pragma unroll
        for (int sl = 0; sl < NS; sl++) pd[sl * kc_n] = make_float2((float)dcv[sl], 0.0f);
      }
      // this thread's kx run [i0, i0 + mpt) lies in [0, xhalf) or in [xhalf, NX) (xhalf is a multiple
      // of mpt); keep its modes with i <= r or i >= NX - r (r <= xhalf; the others can not reach the
      // top bin): a prefix of a run in the first half, a suffix in the second
      int m_lo = 0, m_hi = mpt;
      if (i0 < bp.xhalf) m_hi = min(mpt, col.r + 1 - i0);
      else m_lo = max(0, bp.nx - col.r - i0);
      if (m_lo >= m_hi) continue;
      // Hermitian multiplicity NM (src/main.c:422-429): 2 off the kz = 0 plane (in cyzn); on it 1,
      // except at kx = NX/2 and, on ky = 0, at kx = 0; a run holds at most one of those
      int isp = -1;
      if (col.kz == 0) {
        if (bp.xhalf >= i0 && bp.xhalf < i0 + mpt) isp = bp.xhalf;
        else if (col.j == 0 && i0 == 0) isp = 0;
      }
      float acc[NP][NL];
#pragma unroll
      for (int qq = 0; qq < NP; qq++)
#pragma unroll
        for (int l2 = 0; l2 < NL; l2++) acc[qq][l2] = 0.0f;
      int cur = -2;  // no bin yet: the first mode guesses, later ones walk from the last
      float lo = 1.0f, hi = 0.0f;
      for (int m = m_lo; m < m_hi; m++) {
        const int i = i0 + m;
        const float2 *pm = sd + (rowb + m * (n >> 3)) * P + my_kc;
        const float4 xt = sxt[xt_index(i)];
        const float s = xt.x + col.syz;
        if (!(s >= lo && s < hi)) {
          int b = cur == -2 ? guess_bin(bp, sElo, s) : cur;
          while (b < nk && s >= sElo[b + 2]) b++;
          while (b > -1 && s < sEhi[b + 1]) b--;
          if (s >= sElo[b + 1] && s < sEhi[b + 2]) {
            lo = sElo[b + 1];
            hi = sEhi[b + 2];
          } else {  // within a few ulps of an edge: the exact FP64 s decides
            const double sd2 = __dadd_rn(__dadd_rn(t.fx2d[i], t.fy2d[col.j]), t.fz2d[col.kz]);
            b = exact_bin(sE, nk, sd2, b);
            lo = 1.0f;
            hi = 0.0f;
          }
          if (b != cur) {
            if (cur >= 0 && cur < nk) {
#pragma unroll
              for (int qq = 0; qq < NP; qq++)
                if ((PM >> qq) & 1)
#pragma unroll
                  for (int l2 = 0; l2 < NL; l2++) {
                    atomicAdd(&sbw[(qq * NL + l2) * nk + cur], acc[qq][l2]);
                    acc[qq][l2] = 0.0f;
                  }
            }
            cur = b;
          }
        }
        if (cur < 0 || cur >= nk) continue;
        float2 A = pm[0];
        float2 B = make_float2(0.0f, 0.0f);
        if (NF == 2) B = pm[kc_n];
        if (IL) {
          const float2 e = cmulf(make_float2(xt.z, xt.w), col.eyz);
          A = cadd(A, cmulf(pm[NF * kc_n], e));
          if (NF == 2) B = cadd(B, cmulf(pm[3 * kc_n], e));
        }
        float gc = col.cyzn * xt.y;
        if (i == isp) gc *= 2.0f;
        const float fl = bp.los == 1 ? sfx[i] : col.flos;
        const float mu = s > 0.0f ? fl * rsqrtf(s) : 0.0f;
        const float mu2 = mu * mu;
        const float L2 = 1.5f * mu2 - 0.5f;
        const float L4 = (4.375f * mu2 - 3.75f) * mu2 + 0.375f;
        float Pq[NP];
        if (PM & 1) Pq[0] = (A.x * A.x + A.y * A.y) * gc;
        if (NF == 2) {
          if (PM & 2) Pq[1] = (A.x * B.x + A.y * B.y) * gc;
          if (PM & 4) Pq[2] = (A.x * B.y - A.y * B.x) * gc;
          if (PM & 8) Pq[3] = (B.x * B.x + B.y * B.y) * gc;
        }
#pragma unroll
        for (int qq = 0; qq < NP; qq++) {
          if (!((PM >> qq) & 1)) continue;
          acc[qq][0] += Pq[qq];
          acc[qq][1] += Pq[qq] * L2;
          acc[qq][2] += Pq[qq] * L4;
          if (ODD) {
            acc[qq][NL - 2] += Pq[qq] * mu;
            acc[qq][NL - 1] += Pq[qq] * ((2.5f * mu2 - 1.5f) * mu);
          }
        }
      }
      if (cur >= 0 && cur < nk) {
#pragma unroll
        for (int qq = 0; qq < NP; qq++)
          if ((PM >> qq) & 1)
#pragma unroll
            for (int l2 = 0; l2 < NL; l2++) atomicAdd(&sbw[(qq * NL + l2) * nk + cur], acc[qq][l2]);
      }
    }
    // every 8 blocks, the FP32 block bins (a few hundred modes per bin at most) are added into the
    // CTA's FP64 bins and cleared; the next block's first barrier orders the clearing before its flushes
    // (at 512^3: every 8 blocks 1.494 ms, every 4 1.508, every 2 1.535)
    if ((++nproc & 7) == 0) {
      __syncthreads();
      for (int c = threadIdx.x; c < nbins; c += blockDim.x) {
        float v = 0.0f;
        for (int k = 0; k < xg.nbc; k++) {
          v += sb[c + k * nbins];
          sb[c + k * nbins] = 0.0f;
        }
        sbd[c] += (double)v;
      }
    }
  }
  __syncthreads();
  // CTA bins (FP64) -> global FP64 bins [product][5][nk]; stored multipole index -> l
  for (int c = threadIdx.x; c < nbins; c += blockDim.x) {
    double v = sbd[c];
    for (int k = 0; k < xg.nbc; k++) v += (double)sb[c + k * nbins];
    if (v == 0.0) continue;
    const int b = c % nk, ql = c / nk, qq = ql / NL, li = ql - qq * NL;
    const int l = li == 0 ? 0 : (li == 1 ? 2 : (li == 2 ? 4 : (li == 3 ? 1 : 3)));
    atomicAdd(&bins[(qq * 5 + l) * nk + b], v);
  }
}

// ------------------------------------------------------------ z-axis real-to-complex DFT (FP32)
// The first axis of the 3-D transform (src/main.c:266-271) on the transposed fused path: every
// (x, y) row of NZ reals of every painted grid, as the M = NZ/2-point complex DFT Z of
// z[n] = x[2n] + i x[2n+1] followed by the real-input split
//   X[k] = (Z[k] + Z*[M-k]) / 2 - (i/2) e^{-2 pi i k/NZ} (Z[k] - Z*[M-k]),  k = 0..M (Z[M] = Z[0]).
// Written out of place and transposed, [NX][NZ/2+1][NY]: the y axis is then a contiguous row for
// the batched cuFFT C2C that follows, and ZB consecutive ky at one kz are contiguous for the fused
// x-axis pass. A CTA transforms ZB consecutive rows (one x) in shared memory: coalesced row reads,
// the same in-place radix-8 DIF stages as the x-axis pass (rows padded to ZB + 1), and ZB * 8 byte
// segments written per kz.
constexpr int ZR_THREADS = 256;

// twiddle-table entries of the radix-8 stages of an M = 2^log2m point DIF with more than one
// butterfly per group
CAPOW_HD unsigned zr2c_tw_entries(int log2m) {
  unsigned e = 0;
  for (int l = log2m; l >= 4; l -= 3) e += 8u << (l - 3);
  return e;
}

struct ZrGeo {
  int log2m, nx, ny, nzc, row, nyb, ns;
  long long slice, in_slot, out_slot;
};

// Geometry of a z pass over nslot grids ([NX][NY][row] floats, slot stride in_slot) into the transposed
// slots (slot stride out_slot complex); nyb is set by the launcher from its rows per CTA.
static ZrGeo zr2c_geo(const BinParams &bp, int nslot, long long in_slot, int row, long long out_slot) {
  ZrGeo zg;
  int lm = 0;
  while ((2 << lm) < bp.nz) lm++;  // M = NZ / 2 = 2^lm
  zg.log2m = lm;
  zg.nx = bp.nx;
  zg.ny = bp.ny;
  zg.nzc = bp.nzc;
  zg.row = row;
  zg.nyb = 0;
  zg.slice = (long long)bp.ny * row;
  zg.in_slot = in_slot;
  zg.out_slot = out_slot;
  zg.ns = nslot;
  return zg;
}

// Shared tables of the z pass: radix-8 twiddles (stw), the row of Z[k] after the DIF stages (spos)
// and the real-input split twiddles (stp), carved after a data area of `data_bytes`.
struct ZrTables {
  float2 *stw;
  int *spos;
  float2 *stp;
};

CAPOW_HD unsigned zr2c_tables_bytes(int log2m) {
  const unsigned M = 1u << log2m;
  return align16(8u * zr2c_tw_entries(log2m)) + align16(4u * M) + align16(8u * (M + 1));
}

__device__ ZrTables zr2c_load_tables(const BinTables &t, int log2m, unsigned char *base) {
  const int M = 1 << log2m;
  ZrTables z;
  z.stw = (float2 *)base;
  z.spos = (int *)(base + align16(8u * zr2c_tw_entries(log2m)));
  z.stp = (float2 *)(base + align16(8u * zr2c_tw_entries(log2m)) + align16(4u * M));
  for (int k = threadIdx.x; k < M; k += blockDim.x) z.spos[k] = xfft_pos(log2m, k);
  for (int k = threadIdx.x; k <= M; k += blockDim.x) z.stp[k] = t.tpz[k];
  for (int l = log2m, off = 0; l >= 4; off += 8 << (l - 3), l -= 3) {
    const int step = M >> l;  // M / span
    for (int e = threadIdx.x; e < (8 << (l - 3)); e += blockDim.x)
      z.stw[off + e] = t.twz[((e & 7) * (e >> 3) * step) & (M - 1)];
  }
  return z;
}

// The z pass's loads: a pair of consecutive reals of row y of plane x (z = 2n, 2n + 1), read once. A load
// functor's row(x, y) gives what is fixed along one row, and its load(p, n) reads pair n at p.
struct ZrPlainRow {
  __device__ __forceinline__ float2 load(const float2 *p, int) const { return __ldcs(p); }
};
struct ZrPlainLoad {
  __device__ __forceinline__ ZrPlainRow row(int, int) const { return ZrPlainRow(); }
};

// One block of the z pass: ZB rows y0.. of plane x of slot sl, through the shared data area sd
// ([M][ZB + 1]). The caller has synchronised after the tables were written and after any earlier use
// of sd. ld reads the input pairs (ZrPlainLoad, or a weighting load). SP = 2: the block holds ZB / 2
// rows of each of the slots sl and sl + 1 (columns r and r + ZB / 2 are row y0 + r of each), and one
// thread reads the same cells of both, so that a weighting load's weights are evaluated once for both.
template <int ZB, class LD = ZrPlainLoad, int SP = 1>
__device__ __forceinline__ void zr2c_block(const ZrGeo &zg, const ZrTables &z, const float *in, float2 *out,
                                           float2 *sd, int sl, int x, int y0, const LD &ld = LD()) {
  constexpr int LZB = ZB == 16 ? 4 : 3;
  constexpr int RS = ZB / SP;  // rows of each slot
  const int log2m = zg.log2m, M = 1 << log2m, P = ZB + 1, Q1 = M >> 3;
  const float *src = in + sl * zg.in_slot + (long long)x * zg.slice;
  // first DIF stage (span M) straight from the rows: butterfly (row r, jj) reads z[jj + q M/8];
  // lanes run along a row, so each of a warp's 8 loads is one contiguous 256-byte piece
  for (int u = threadIdx.x; u < (RS << (log2m - 3)); u += blockDim.x) {
    const int jj = u & (Q1 - 1), r = u >> (log2m - 3), y = y0 + r;
    const float2 *rp = reinterpret_cast<const float2 *>(src + (long long)(y < zg.ny ? y : 0) * zg.row) + jj;
    const auto rw = ld.row(x, y < zg.ny ? y : 0);  // what the row's loads share (a weighting load's row terms)
    float2 a[8];
    if constexpr (SP == 1) {
#pragma unroll
      for (int q = 0; q < 8; q++) a[q] = y < zg.ny ? rw.load(rp + q * Q1, jj + q * Q1) : make_float2(0.0f, 0.0f);
    } else {
      const float2 *rpb = rp + (zg.in_slot >> 1);  // the same row of slot sl + 1 (in_slot floats is even)
      float2 b[8];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        a[q] = b[q] = make_float2(0.0f, 0.0f);
        if (y < zg.ny) {
          const float2 w = rw.weights(jj + q * Q1), va = __ldcs(rp + q * Q1), vb = __ldcs(rpb + q * Q1);
          a[q] = make_float2(va.x * w.x, va.y * w.y);
          b[q] = make_float2(vb.x * w.x, vb.y * w.y);
        }
      }
      dft8(b);
      if (jj > 0) twiddle8(b, z.stw + 8 * jj);
      float2 *pb = sd + jj * P + r + RS;
#pragma unroll
      for (int q = 0; q < 8; q++) pb[q * Q1 * P] = b[q];
    }
    dft8(a);
    if (jj > 0) twiddle8(a, z.stw + 8 * jj);
    float2 *p = sd + jj * P + r;
#pragma unroll
    for (int q = 0; q < 8; q++) p[q * Q1 * P] = a[q];
  }
  __syncthreads();
  int l = log2m - 3, twoff = 8 * Q1;
  for (; l >= 3; l -= 3) {  // the other radix-8 DIF stages
    const int log2q = l - 3, Q = 1 << log2q, qs = Q * P;
    for (int u = threadIdx.x; u < (ZB << (log2m - 3)); u += blockDim.x) {
      const int c = u & (ZB - 1), v = u >> LZB;
      const int jj = v & (Q - 1);
      float2 *p = sd + (((v >> log2q) << l) + jj) * P + c;
      float2 a[8];
#pragma unroll
      for (int q = 0; q < 8; q++) a[q] = p[q * qs];
      dft8(a);
      if (jj > 0) twiddle8(a, z.stw + twoff + 8 * jj);
#pragma unroll
      for (int q = 0; q < 8; q++) p[q * qs] = a[q];
    }
    __syncthreads();
    if (Q > 1) twoff += 8 * Q;
  }
  if (l == 2) {  // a last radix-4 stage (span 4: no twiddles)
    for (int u = threadIdx.x; u < (ZB << (log2m - 2)); u += blockDim.x) {
      float2 *p = sd + ((u >> LZB) << 2) * P + (u & (ZB - 1));
      float2 a[4];
#pragma unroll
      for (int q = 0; q < 4; q++) a[q] = p[q * P];
      dft4(a);
#pragma unroll
      for (int q = 0; q < 4; q++) p[q * P] = a[q];
    }
    __syncthreads();
  } else if (l == 1) {  // a last radix-2 stage
    for (int u = threadIdx.x; u < (ZB << (log2m - 1)); u += blockDim.x) {
      float2 *p = sd + ((u >> LZB) << 1) * P + (u & (ZB - 1));
      const float2 a0 = p[0], a1 = p[P];
      p[0] = cadd(a0, a1);
      p[P] = csub(a0, a1);
    }
    __syncthreads();
  }
  // real-input split and transposed store, X[k] and X[M-k] from the same pair: with
  // A = Z[k] + conj Z[M-k], B = Z[k] - conj Z[M-k] and w^M = -1, X[k] = (A + (-i) w^k B) / 2 and
  // X[M-k] = (conj A + (-i) conj(w^k B)) / 2. The thread's column r is the same on every step.
  const int r = threadIdx.x & (ZB - 1), y = y0 + r % RS, so = r / RS;
  if (y < zg.ny) {
    float2 *dst = out + (sl + so) * zg.out_slot + (long long)x * zg.nzc * zg.ny + y;
    for (int k = threadIdx.x >> LZB; k <= (M >> 1); k += blockDim.x >> LZB) {
      const float2 zk = sd[z.spos[k & (M - 1)] * P + r];
      const float2 zm = sd[z.spos[(M - k) & (M - 1)] * P + r];
      const float2 A = make_float2(zk.x + zm.x, zk.y - zm.y);
      const float2 B = make_float2(zk.x - zm.x, zk.y + zm.y);
      const float2 wB = cmulf(z.stp[k], B);
      dst[(long long)k * zg.ny] = make_float2(0.5f * (A.x + wB.y), 0.5f * (A.y - wB.x));
      if (2 * k != M) dst[(long long)(M - k) * zg.ny] = make_float2(0.5f * (A.x - wB.y), -0.5f * (A.y + wB.x));
    }
  }
}

template <int ZB>
__global__ void __launch_bounds__(ZR_THREADS) k_zr2c(ZrGeo zg, BinTables t, const float *in, float2 *out) {
  extern __shared__ __align__(16) unsigned char smz[];
  const int M = 1 << zg.log2m;
  float2 *sd = (float2 *)smz;  // [M][ZB + 1]
  const ZrTables z = zr2c_load_tables(t, zg.log2m, smz + align16(8u * (unsigned)M * (ZB + 1)));
  const int per_slot = zg.nx * zg.nyb, nblk = per_slot * zg.ns;
  for (int blk = blockIdx.x; blk < nblk; blk += gridDim.x) {  // (slot, x, block of ZB rows)
    const int sl = blk / per_slot, rem = blk - sl * per_slot;
    const int x = rem / zg.nyb, y0 = (rem - x * zg.nyb) * ZB;
    __syncthreads();  // tables written; the previous block's output has read sd
    // the CTA's next block is ZB contiguous padded rows: one bulk prefetch into L2 while this one runs
    const int nb = blk + (int)gridDim.x;
    if (threadIdx.x == 0 && nb < nblk) {
      const int sl2 = nb / per_slot, rem2 = nb - sl2 * per_slot;
      const int x2 = rem2 / zg.nyb, y2 = (rem2 - x2 * zg.nyb) * ZB;
      const float *nxt = in + sl2 * zg.in_slot + (long long)x2 * zg.slice + (long long)y2 * zg.row;
      const unsigned bytes = ((unsigned)(min(ZB, zg.ny - y2) * zg.row) * 4u) & ~15u;
      if (bytes && (((unsigned long long)nxt & 15ull) == 0))
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(nxt), "r"(bytes) : "memory");
    }
    zr2c_block<ZB>(zg, z, in, out, sd, sl, x, y0);
  }
}

// The survey estimator's weighted z pass: the input of a set (l, m) is the painted grid times h_lm(r^) of
// each cell (harm.cuh), applied as the rows are read, so that no weighted grid is written.
struct ZrWeight {
  const float *vx, *vy, *vz;  // cell-corner offsets from the observer per axis
  int l, m;
};

// One row (plane x, row y) of a set: its harmonic's polynomial in pz (HarmRow, formed once per row), so
// that a cell's weight is a Horner step per degree, one rsqrt and L - 1 products.
template <int L>
struct ZrWeightRow {
  HarmRow<L> h;
  const float *vz;
  // the weights of cells z = 2n and 2n + 1
  __device__ __forceinline__ float2 weights(int n) const {
    const float2 pz = __ldg(reinterpret_cast<const float2 *>(vz) + n);
    return make_float2(h.at(pz.x), h.at(pz.y));
  }
  __device__ __forceinline__ float2 load(const float2 *p, int n) const {
    const float2 v = __ldcs(p), c = weights(n);
    return make_float2(v.x * c.x, v.y * c.y);
  }
};

// The degree L is a compile-time constant, so the polynomial of each m is specialised.
template <int L>
struct ZrWeightLoad {
  ZrWeight w;
  __device__ __forceinline__ ZrWeightRow<L> row(int x, int y) const {
    return ZrWeightRow<L>{HarmRow<L>(w.m, __ldg(w.vx + x), __ldg(w.vy + y)), w.vz};
  }
};

// SP = 2 (an even number of slots): each block takes ZB / 2 rows of a pair of slots, whose cells share
// their weights (the weights depend on the cell only).
template <int ZB, int L, int SP>
__global__ void __launch_bounds__(ZR_THREADS) k_zr2c_w(ZrGeo zg, BinTables t, const float *in, float2 *out,
                                                       ZrWeightLoad<L> ld) {
  extern __shared__ __align__(16) unsigned char smz[];
  constexpr int RS = ZB / SP;
  const int M = 1 << zg.log2m;
  float2 *sd = (float2 *)smz;  // [M][ZB + 1]
  const ZrTables z = zr2c_load_tables(t, zg.log2m, smz + align16(8u * (unsigned)M * (ZB + 1)));
  const int per_group = zg.nx * zg.nyb, nblk = per_group * (zg.ns / SP);
  for (int blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int grp = blk / per_group, rem = blk - grp * per_group;
    const int x = rem / zg.nyb, y0 = (rem - x * zg.nyb) * RS;
    __syncthreads();
    zr2c_block<ZB, ZrWeightLoad<L>, SP>(zg, z, in, out, sd, grp * SP, x, y0, ld);
  }
}

template <int ZB, int L, int SP>
static void launch_zr2c_w_sp(cudaStream_t s, ZrGeo zg, const BinTables &t, int nslot, const float *in,
                             float2 *out, const ZrWeight &w) {
  const int M = 1 << zg.log2m;
  zg.nyb = (zg.ny + ZB / SP - 1) / (ZB / SP);
  const size_t smem = align16(8u * (unsigned)M * (ZB + 1)) + zr2c_tables_bytes(zg.log2m);
  cudaFuncSetAttribute(k_zr2c_w<ZB, L, SP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 1, dev = 0, nsm = 152;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_zr2c_w<ZB, L, SP>, ZR_THREADS, smem);
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long long nblk = (long long)zg.nx * zg.nyb * (nslot / SP);
  long long grid = (long long)(per_sm > 0 ? per_sm : 1) * nsm;
  if (grid > nblk) grid = nblk;
  k_zr2c_w<ZB, L, SP><<<(unsigned)grid, ZR_THREADS, smem, s>>>(zg, t, in, out, ZrWeightLoad<L>{w});
}

template <int ZB, int L>
static void launch_zr2c_w_l(cudaStream_t s, const ZrGeo &zg, const BinTables &t, int nslot, const float *in,
                            float2 *out, const ZrWeight &w) {
  if (nslot % 2 == 0 && (zg.in_slot % 2) == 0) launch_zr2c_w_sp<ZB, L, 2>(s, zg, t, nslot, in, out, w);
  else launch_zr2c_w_sp<ZB, L, 1>(s, zg, t, nslot, in, out, w);
}

template <int ZB>
static void launch_zr2c_w_t(cudaStream_t s, const ZrGeo &zg, const BinTables &t, int nslot, const float *in,
                            float2 *out, const ZrWeight &w) {
  switch (w.l) {
    case 1: launch_zr2c_w_l<ZB, 1>(s, zg, t, nslot, in, out, w); break;
    case 2: launch_zr2c_w_l<ZB, 2>(s, zg, t, nslot, in, out, w); break;
    case 3: launch_zr2c_w_l<ZB, 3>(s, zg, t, nslot, in, out, w); break;
    default: launch_zr2c_w_l<ZB, 4>(s, zg, t, nslot, in, out, w); break;
  }
}

void launch_zr2c_weighted(cudaStream_t s, const BinParams &bp, const BinTables &t, int nslot, const float *in,
                          long long in_slot, int row, float2 *out, long long out_slot, const float *vx,
                          const float *vy, const float *vz, int l, int m, long long *launches) {
  ZrGeo zg = zr2c_geo(bp, nslot, in_slot, row, out_slot);
  const ZrWeight ld{vx, vy, vz, l, m};
  if (bp.nz <= 512) {
    zg.nyb = (bp.ny + 15) / 16;
    launch_zr2c_w_t<16>(s, zg, t, nslot, in, out, ld);
  } else {
    zg.nyb = (bp.ny + 7) / 8;
    launch_zr2c_w_t<8>(s, zg, t, nslot, in, out, ld);
  }
  (*launches)++;
}

// ------------------------------------------------------------ z and y axes in one launch (FP32)
// The z pass above followed by the y-axis C2C over the transposed layout [NX][NZ/2+1][NY], in one
// persistent launch so that each x-plane's z output is read back by its y transforms from L2 and
// overwritten in place, instead of going to HBM and back (4 bytes of grid traffic per real cell less
// in each direction). Work items come from one queue counter in a fixed order: the z items of the
// first `lead` planes, then for each plane p its y items followed by the z items of plane p + lead.
// A y item of plane p (KB consecutive kz rows of one slot) waits until all z items of that plane and
// slot are done (a per-(slot, plane) counter). Every item it waits for was taken from the queue before
// it by a running CTA and waits for nothing, so the wait always ends; it is still bounded: a wait that
// runs out sets the abort flag (every CTA then stops at its next item) and the error flag of the
// paint statistics, which capow_power reports as CAPOW_ETIMEOUT.
constexpr int ZY_KB = 8;                     // kz rows per y item
constexpr unsigned ZY_WAIT_LIMIT = 1u << 22;  // polls of about 0.2 us: about a second

struct ZyGeo {
  ZrGeo zg;
  int log2ny;     // NY = 2^log2ny
  int nkb;        // y items per (plane, slot)
  int lead;       // planes of z items issued ahead of the y items
  int stall;      // test switch: y items wait for one z item more than exists (their waits run out)
  long long nitems;
};

CAPOW_HD unsigned zy_ytables_bytes(int log2ny) { return align16(8u * xbin_tw_entries(log2ny)); }

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// ------------------------------------------------------------ one row per warp (FP32, forward)
// Base-8 digit reversal of g over D digits.
template <int D>
__device__ __forceinline__ int rev8(int g) {
  int r = 0;
#pragma unroll
  for (int t = 0; t < D; t++) {
    r = (r << 3) | (g & 7);
    g >>= 3;
  }
  return r;
}

// Padded position in a warp's row buffer: one pad element per 8 spreads the strided accesses of every
// stage (and the last stage's runs of 8) over the banks.
__device__ __forceinline__ int wpad(int i) { return i + (i >> 3); }

// One complex row of N = 2^LOG2N (16 <= N <= 2048) transformed by one warp with no block barrier: the
// first in-place DIF stage (radix 8, span N) reads src, the middle radix-8 stages work in the warp's
// buffer wb (N + N/8 values), and the last stage (radix 8, 4 or 2) writes dst in natural order (the
// output of butterfly g, entry q, is frequency rev8(g) + q N/R). stw: the stage twiddle tables in the
// layout of xbin_tw_entries. src is read through L2 (other CTAs of a launch may have written it).
template <int LOG2N>
__device__ __forceinline__ void warp_fft_row(const float2 *src, float2 *dst, float2 *wb, const float2 *stw,
                                             int lane) {
  constexpr int N = 1 << LOG2N;
  constexpr int LR = LOG2N % 3 == 0 ? 3 : LOG2N % 3;  // log2 of the last stage's radix
  constexpr int R = 1 << LR;
  constexpr int S8 = (LOG2N - LR) / 3;  // radix-8 stages before the last (>= 1)
  constexpr int Q1 = N >> 3;
  for (int j = lane; j < Q1; j += 32) {
    float2 a[8];
#pragma unroll
    for (int q = 0; q < 8; q++) a[q] = __ldcg(src + j + q * Q1);
    dft8(a);
    if (j > 0) twiddle8(a, stw + 8 * j);
#pragma unroll
    for (int q = 0; q < 8; q++) wb[wpad(j + q * Q1)] = a[q];
  }
  __syncwarp();
  int twoff = 8 * Q1;
#pragma unroll
  for (int t = 1; t < S8; t++) {
    const int l = LOG2N - 3 * t, log2q = l - 3, Q = 1 << log2q;
    for (int u = lane; u < (N >> 3); u += 32) {
      const int jj = u & (Q - 1);
      const int base = ((u >> log2q) << l) + jj;
      float2 a[8];
#pragma unroll
      for (int q = 0; q < 8; q++) a[q] = wb[wpad(base + q * Q)];
      dft8(a);
      if (jj > 0) twiddle8(a, stw + twoff + 8 * jj);
#pragma unroll
      for (int q = 0; q < 8; q++) wb[wpad(base + q * Q)] = a[q];
    }
    __syncwarp();
    if (Q > 1) twoff += 8 * Q;
  }
  constexpr int NG = N / R;
  for (int g = lane; g < NG; g += 32) {
    float2 a[R];
#pragma unroll
    for (int q = 0; q < R; q++) a[q] = wb[wpad(R * g + q)];
    if (R == 8) {
      dft8(a);
    } else if (R == 4) {
      dft4(a);
    } else {
      const float2 a0 = a[0];
      a[0] = cadd(a0, a[1]);
      a[1] = csub(a0, a[1]);
    }
    const int i0 = rev8<S8>(g);
#pragma unroll
    for (int q = 0; q < R; q++) dst[i0 + q * NG] = a[q];
  }
  __syncwarp();
}

// The same transform with the output in natural order in the warp's own row buffer buf (used for the
// stages with wpad positions; N + N/8 values): the last stage's inputs are all read into registers
// before any output is written. STREAM: the source is read once (evict-first loads).
template <int LOG2N, bool STREAM>
__device__ __forceinline__ void warp_fft_row_buf(const float2 *src, float2 *buf, const float2 *stw, int lane) {
  constexpr int N = 1 << LOG2N;
  constexpr int LR = LOG2N % 3 == 0 ? 3 : LOG2N % 3;
  constexpr int R = 1 << LR;
  constexpr int S8 = (LOG2N - LR) / 3;
  constexpr int Q1 = N >> 3;
  for (int j = lane; j < Q1; j += 32) {
    float2 a[8];
#pragma unroll
    for (int q = 0; q < 8; q++) a[q] = STREAM ? __ldcs(src + j + q * Q1) : __ldcg(src + j + q * Q1);
    dft8(a);
    if (j > 0) twiddle8(a, stw + 8 * j);
#pragma unroll
    for (int q = 0; q < 8; q++) buf[wpad(j + q * Q1)] = a[q];
  }
  __syncwarp();
  int twoff = 8 * Q1;
#pragma unroll
  for (int t = 1; t < S8; t++) {
    const int l = LOG2N - 3 * t, log2q = l - 3, Q = 1 << log2q;
    for (int u = lane; u < (N >> 3); u += 32) {
      const int jj = u & (Q - 1);
      const int base = ((u >> log2q) << l) + jj;
      float2 a[8];
#pragma unroll
      for (int q = 0; q < 8; q++) a[q] = buf[wpad(base + q * Q)];
      dft8(a);
      if (jj > 0) twiddle8(a, stw + twoff + 8 * jj);
#pragma unroll
      for (int q = 0; q < 8; q++) buf[wpad(base + q * Q)] = a[q];
    }
    __syncwarp();
    if (Q > 1) twoff += 8 * Q;
  }
  constexpr int NG = N / R, PER = (NG + 31) / 32;  // last-stage butterflies per lane
  float2 a[PER][R];
#pragma unroll
  for (int p = 0; p < PER; p++) {
    const int g = lane + 32 * p;
    if (g < NG) {
#pragma unroll
      for (int q = 0; q < R; q++) a[p][q] = buf[wpad(R * g + q)];
      if (R == 8) {
        dft8(a[p]);
      } else if (R == 4) {
        dft4(a[p]);
      } else {
        const float2 a0 = a[p][0];
        a[p][0] = cadd(a0, a[p][1]);
        a[p][1] = csub(a0, a[p][1]);
      }
    }
  }
  __syncwarp();
#pragma unroll
  for (int p = 0; p < PER; p++) {
    const int g = lane + 32 * p;
    if (g < NG) {
      const int i0 = rev8<S8>(g);
#pragma unroll
      for (int q = 0; q < R; q++) buf[i0 + q * NG] = a[p][q];
    }
  }
  __syncwarp();
}

template <int LOG2N>
__device__ __forceinline__ void warp_fft_rows(const ZyGeo &yg, const float2 *stwy, float2 *rows, float2 *sd, int nrow) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int N = 1 << LOG2N;
  for (int r = w; r < nrow; r += (int)(blockDim.x >> 5))
    warp_fft_row<LOG2N>(rows + (long long)r * N, rows + (long long)r * N, sd + w * (N + N / 8), stwy, lane);
}

// One y item: rows kz0 .. kz0 + ZY_KB - 1 (those below NZ/2+1) of plane x of slot sl, each NY complex
// values along y, transformed in place (forward, unnormalised), one row per warp through that warp's
// part of sd (ZY_KB warps, each NY + NY/8 values).
__device__ __forceinline__ void yfft_block(const ZyGeo &yg, const float2 *stwy, float2 *out, float2 *sd, int sl,
                                           int x, int kz0) {
  const int nrow = min(ZY_KB, yg.zg.nzc - kz0);
  float2 *rows = out + sl * yg.zg.out_slot + ((long long)x * yg.zg.nzc + kz0) * (1LL << yg.log2ny);
  switch (yg.log2ny) {
    case 4: warp_fft_rows<4>(yg, stwy, rows, sd, nrow); break;
    case 5: warp_fft_rows<5>(yg, stwy, rows, sd, nrow); break;
    case 6: warp_fft_rows<6>(yg, stwy, rows, sd, nrow); break;
    case 7: warp_fft_rows<7>(yg, stwy, rows, sd, nrow); break;
    case 8: warp_fft_rows<8>(yg, stwy, rows, sd, nrow); break;
    case 9: warp_fft_rows<9>(yg, stwy, rows, sd, nrow); break;
    case 10: warp_fft_rows<10>(yg, stwy, rows, sd, nrow); break;
    default: warp_fft_rows<11>(yg, stwy, rows, sd, nrow); break;
  }
}

// z items of k_zy with one warp per row (M <= 256): rows of M = 2^LOG2M complex values (z[n] = x[2n] + i x[2n+1])
// transformed into natural order in their own buffer rows (stride M + M/8 + 1: the split's lanes run
// across rows), then the real-input split and transposed store of zr2c_block.
template <int LOG2M>
__device__ __forceinline__ int zy_zrow_stride() {
  return (1 << LOG2M) + (1 << LOG2M) / 8 + 1;
}

CAPOW_HD unsigned zy_zdata_bytes(int log2m, int zb) {
  const unsigned M = 1u << log2m;
  return log2m <= 8 ? align16(8u * zb * (M + M / 8 + 1)) : align16(8u * M * (zb + 1));
}

template <int ZB, int LOG2M>
__device__ __forceinline__ void zr2c_block_warp(const ZrGeo &zg, const ZrTables &z, const float *in, float2 *out,
                                                float2 *sd, int sl, int x, int y0) {
  constexpr int LZB = ZB == 16 ? 4 : 3, M = 1 << LOG2M;
  const int RS = zy_zrow_stride<LOG2M>();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const float *src = in + sl * zg.in_slot + (long long)x * zg.slice;
  for (int r = w; r < ZB; r += nw) {
    const int y = y0 + r;
    if (y < zg.ny)
      warp_fft_row_buf<LOG2M, true>(reinterpret_cast<const float2 *>(src + (long long)y * zg.row), sd + r * RS, z.stw,
                                    lane);
  }
  __syncthreads();
  const int r = threadIdx.x & (ZB - 1), y = y0 + r;
  if (y < zg.ny) {
    const float2 *zr = sd + r * RS;
    float2 *dst = out + sl * zg.out_slot + (long long)x * zg.nzc * zg.ny + y;
    for (int k = threadIdx.x >> LZB; k <= (M >> 1); k += blockDim.x >> LZB) {
      const float2 zk = zr[k & (M - 1)];
      const float2 zm = zr[(M - k) & (M - 1)];
      const float2 A = make_float2(zk.x + zm.x, zk.y - zm.y);
      const float2 B = make_float2(zk.x - zm.x, zk.y + zm.y);
      const float2 wB = cmulf(z.stp[k], B);
      dst[(long long)k * zg.ny] = make_float2(0.5f * (A.x + wB.y), 0.5f * (A.y - wB.x));
      if (2 * k != M) dst[(long long)(M - k) * zg.ny] = make_float2(0.5f * (A.x - wB.y), -0.5f * (A.y + wB.x));
    }
  }
}

template <int ZB>
__device__ __forceinline__ void zy_zblock(const ZrGeo &zg, const ZrTables &z, const float *in, float2 *out,
                                          float2 *sd, int sl, int x, int y0) {
  switch (zg.log2m) {
    case 4: zr2c_block_warp<ZB, 4>(zg, z, in, out, sd, sl, x, y0); break;
    case 5: zr2c_block_warp<ZB, 5>(zg, z, in, out, sd, sl, x, y0); break;
    case 6: zr2c_block_warp<ZB, 6>(zg, z, in, out, sd, sl, x, y0); break;
    case 7: zr2c_block_warp<ZB, 7>(zg, z, in, out, sd, sl, x, y0); break;
    case 8: zr2c_block_warp<ZB, 8>(zg, z, in, out, sd, sl, x, y0); break;
    default: zr2c_block<ZB>(zg, z, in, out, sd, sl, x, y0); break;  // M >= 512: the block stages
  }
}

template <int ZB>
__global__ void __launch_bounds__(ZR_THREADS, 4) k_zy(ZyGeo yg, BinTables t, const float *in, float2 *out,
                                                   unsigned *ctr, DevStats *st) {
  extern __shared__ __align__(16) unsigned char smz[];
  const ZrGeo &zg = yg.zg;
  const int M = 1 << zg.log2m, ny = 1 << yg.log2ny;
  const unsigned zdata = zy_zdata_bytes(zg.log2m, ZB), ydata = align16(8u * ZY_KB * (ny + ny / 8));
  float2 *sd = (float2 *)smz;  // the data area of whichever item runs
  unsigned char *tb = smz + (zdata > ydata ? zdata : ydata);
  const ZrTables z = zr2c_load_tables(t, zg.log2m, tb);
  tb += zr2c_tables_bytes(zg.log2m);
  float2 *stwy = (float2 *)tb;
  for (int l = yg.log2ny, off = 0; l >= 4; off += 8 << (l - 3), l -= 3) {
    const int step = ny >> l;
    for (int e = threadIdx.x; e < (8 << (l - 3)); e += blockDim.x)
      stwy[off + e] = t.twy[((e & 7) * (e >> 3) * step) & (ny - 1)];
  }
  __shared__ long long s_item;
  __shared__ int s_ok;
  unsigned *done = ctr + 2;  // [slot][plane]: finished z items
  const long long nzp = (long long)zg.ns * zg.nyb, nyp = (long long)zg.ns * yg.nkb;
  const long long lead = yg.lead, s0 = lead * nzp, per = nzp + nyp, nper = zg.nx - lead;
  for (;;) {
    __syncthreads();  // the previous item is done with sd (and the tables are written)
    if (threadIdx.x == 0) {
      const unsigned abort = *(volatile unsigned *)(ctr + 1);
      s_item = abort ? yg.nitems : (long long)atomicAdd(ctr, 1u);
    }
    __syncthreads();
    const long long item = s_item;
    if (item >= yg.nitems) break;
    // decode: z items of the first `lead` planes, then (y items of p, z items of p + lead) per plane
    bool is_y;
    long long plane, r;
    if (item < s0) {
      is_y = false;
      plane = item / nzp;
      r = item - plane * nzp;
    } else if (item - s0 < nper * per) {
      const long long t2 = item - s0, q = t2 / per;
      r = t2 - q * per;
      is_y = r < nyp;
      plane = is_y ? q : q + lead;
      if (!is_y) r -= nyp;
    } else {
      const long long t3 = item - s0 - nper * per;
      is_y = true;
      plane = nper + t3 / nyp;
      r = t3 - (plane - nper) * nyp;
    }
    if (!is_y) {
      const int sl = (int)(r / zg.nyb), y0 = (int)(r - (long long)sl * zg.nyb) * ZB;
      zy_zblock<ZB>(zg, z, in, out, sd, sl, (int)plane, y0);
      __threadfence();  // this thread's stores, before the item is counted done
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(done + (long long)sl * zg.nx + plane, 1u);
    } else {
      const int sl = (int)(r / yg.nkb), kz0 = (int)(r - (long long)sl * yg.nkb) * ZY_KB;
      if (threadIdx.x == 0) {
        const unsigned *cnt = done + (long long)sl * zg.nx + plane;
        unsigned polls = 0;
        const unsigned need = (unsigned)(zg.nyb + yg.stall);
        while (ld_acquire_u32(cnt) < need && ++polls < ZY_WAIT_LIMIT && !*(volatile unsigned *)(ctr + 1))
          __nanosleep(200);
        s_ok = polls < ZY_WAIT_LIMIT && !*(volatile unsigned *)(ctr + 1);
        if (!s_ok) {
          atomicExch(ctr + 1, 1u);
          atomicExch(&st->timeout, 1);
        }
      }
      __syncthreads();
      if (!s_ok) break;
      yfft_block(yg, stwy, out, sd, sl, (int)plane, kz0);
    }
  }
}

bool zr2c_supported(const BinParams &bp) {
  return bp.nz >= 32 && bp.nz <= 2048 && (bp.nz & (bp.nz - 1)) == 0;
}

template <int ZB>
static void launch_zr2c_t(cudaStream_t s, const ZrGeo &zg, const BinTables &t, int nslot, const float *in,
                          float2 *out) {
  const int M = 1 << zg.log2m;
  const size_t smem = align16(8u * (unsigned)M * (ZB + 1)) + zr2c_tables_bytes(zg.log2m);
  cudaFuncSetAttribute(k_zr2c<ZB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 1, dev = 0, nsm = 152;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_zr2c<ZB>, ZR_THREADS, smem);
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long long nblk = (long long)zg.nx * zg.nyb * nslot;
  long long grid = (long long)(per_sm > 0 ? per_sm : 1) * nsm;
  if (grid > nblk) grid = nblk;
  k_zr2c<ZB><<<(unsigned)grid, ZR_THREADS, smem, s>>>(zg, t, in, out);
}

void launch_zr2c(cudaStream_t s, const BinParams &bp, const BinTables &t, int nslot, const float *in,
                 long long in_slot, int row, float2 *out, long long out_slot, long long *launches) {
  ZrGeo zg = zr2c_geo(bp, nslot, in_slot, row, out_slot);
  if (bp.nz <= 512) {  // 16 rows per CTA: 128-byte segments per kz
    zg.nyb = (bp.ny + 15) / 16;
    launch_zr2c_t<16>(s, zg, t, nslot, in, out);
  } else {  // 8 rows per CTA keeps the shared rows within 80 KB
    zg.nyb = (bp.ny + 7) / 8;
    launch_zr2c_t<8>(s, zg, t, nslot, in, out);
  }
  (*launches)++;
}

bool zy_supported(const BinParams &bp, const BinTables &t) {
  return zr2c_supported(bp) && t.twy && bp.ny >= 16 && bp.ny <= 2048 && (bp.ny & (bp.ny - 1)) == 0;
}

size_t zy_counter_words(const BinParams &bp, int nslot) { return 2 + (size_t)nslot * bp.nx; }

template <int ZB>
static void launch_zy_t(cudaStream_t s, const ZyGeo &yg, const BinTables &t, const float *in, float2 *out,
                        unsigned *ctr, DevStats *st) {
  const unsigned M = 1u << yg.zg.log2m, ny = 1u << yg.log2ny;
  const unsigned zdata = zy_zdata_bytes(yg.zg.log2m, ZB), ydata = align16(8u * ZY_KB * (ny + ny / 8));
  const size_t smem = (zdata > ydata ? zdata : ydata) + zr2c_tables_bytes(yg.zg.log2m) + zy_ytables_bytes(yg.log2ny);
  cudaFuncSetAttribute(k_zy<ZB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 1, dev = 0, nsm = 152;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_zy<ZB>, ZR_THREADS, smem);
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  long long grid = (long long)(per_sm > 0 ? per_sm : 1) * nsm;
  if (grid > yg.nitems) grid = yg.nitems;
  k_zy<ZB><<<(unsigned)grid, ZR_THREADS, smem, s>>>(yg, t, in, out, ctr, st);
}

void launch_zy(cudaStream_t s, const BinParams &bp, const BinTables &t, int nslot, const float *in, long long in_slot,
               int row, float2 *out, long long out_slot, unsigned *ctr, DevStats *st, int stall,
               long long *launches) {
  ZyGeo yg;
  ZrGeo &zg = yg.zg;
  int lm = 0;
  while ((2 << lm) < bp.nz) lm++;  // M = NZ / 2 = 2^lm
  zg.log2m = lm;
  zg.nx = bp.nx;
  zg.ny = bp.ny;
  zg.nzc = bp.nzc;
  zg.row = row;
  zg.slice = (long long)bp.ny * row;
  zg.in_slot = in_slot;
  zg.out_slot = out_slot;
  zg.ns = nslot;
  const int zb = bp.nz <= 512 ? 16 : 8;
  zg.nyb = (bp.ny + zb - 1) / zb;
  yg.log2ny = 0;
  while ((1 << yg.log2ny) < bp.ny) yg.log2ny++;
  yg.nkb = (bp.nzc + ZY_KB - 1) / ZY_KB;
  yg.lead = bp.nx < 8 ? bp.nx : 8;
  yg.stall = stall ? 1 : 0;
  yg.nitems = (long long)bp.nx * nslot * (zg.nyb + yg.nkb);
  cudaMemsetAsync(ctr, 0, sizeof(unsigned) * zy_counter_words(bp, nslot), s);
  if (zb == 16) launch_zy_t<16>(s, yg, t, in, out, ctr, st);
  else launch_zy_t<8>(s, yg, t, in, out, ctr, st);
  (*launches)++;
}

static int ilog2i(int v) {
  int l = 0;
  while ((1 << l) < v) l++;
  return l;
}

bool xbin_plan(const BinParams &bp, int nslot, XbinGeo &xg, bool transposed) {
  const int n = bp.nx;
  if (n < 16 || n > 2048 || (n & (n - 1)) != 0 || bp.out2d) return false;
  memset(&xg, 0, sizeof xg);
  xg.log2n = ilog2i(n);
  xg.ncol = n <= 512 ? 32 : (n == 1024 ? 16 : 4);
  if (nslot > xg.ncol) return false;
  xg.log2ncol = ilog2i(xg.ncol);
  const int ns = nslot == 3 ? 4 : nslot;
  xg.kc = xg.ncol / ns;
  xg.log2kc = ilog2i(xg.kc);
  xg.tr = transposed ? 1 : 0;
  xg.n_outer = transposed ? bp.nzc : bp.ny;
  xg.n_inner = transposed ? bp.ny : bp.nzc;
  xg.nkb = (xg.n_inner + xg.kc - 1) / xg.kc;
  xg.nblocks = xg.n_outer * xg.nkb;
  const int np = bp.nfields == 1 ? 1 : 4, nl = bp.odd ? 5 : 3;
  // up to 2 bin copies as fit: at 512^3 the bin stage took 1.50 ms with 2, 1.58 with 1 and 1.61 with 4
  // (more copies leave less L1; 8 were slower still)
  for (xg.nbc = 2; xg.nbc > 1; xg.nbc >>= 1)
    if (xbin_smem_layout(xg.log2n, xg.ncol, np, nl, bp.nk, xg.nbc).total <= 220 * 1024) break;
  return xbin_smem_layout(xg.log2n, xg.ncol, np, nl, bp.nk, xg.nbc).total <= 220 * 1024;
}

template <int NF, bool IL, bool ODD, int PM>
static void launch_xbin_t(cudaStream_t s, const BinParams &bp, const BinTables &t, const XbinGeo &xg,
                          void *const slots[4], const double *dcv, double *bins) {
  constexpr int NP = NF == 1 ? 1 : 4, NL = ODD ? 5 : 3;
  const size_t smem = xbin_smem_layout(xg.log2n, xg.ncol, NP, NL, bp.nk, xg.nbc).total;
  cudaFuncSetAttribute(k_xfft_bin<NF, IL, ODD, PM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_xfft_bin<NF, IL, ODD, PM>, XBIN_THREADS, smem);
  int dev = 0, nsm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int grid = (per_sm > 0 ? per_sm : 1) * nsm;
  if (grid > xg.nblocks) grid = xg.nblocks;
  k_xfft_bin<NF, IL, ODD, PM><<<grid, XBIN_THREADS, smem, s>>>(bp, t, xg, (const float2 *)slots[0],
                                                                (const float2 *)slots[1], (const float2 *)slots[2],
                                                                (const float2 *)slots[3], dcv, bins);
}

// Two fields: the products dd + dp + pp read (|A|^2, Im A*B, |B|^2), or all four.
template <bool IL, bool ODD>
static void launch_xbin_f2(cudaStream_t s, const BinParams &bp, const BinTables &t, const XbinGeo &xg,
                           void *const slots[4], const double *dcv, double *bins) {
  if ((bp.pmask & ~0xD) == 0) launch_xbin_t<2, IL, ODD, 0xD>(s, bp, t, xg, slots, dcv, bins);
  else launch_xbin_t<2, IL, ODD, 0xF>(s, bp, t, xg, slots, dcv, bins);
}

void launch_xbin(cudaStream_t s, const BinParams &bp, const BinTables &t, const XbinGeo &xg, void *const slots[4],
                 const double *dcv, double *bins, long long *launches) {
  const bool il = bp.interlace != 0, odd = bp.odd != 0;
  if (bp.nfields == 2) {
    if (il) odd ? launch_xbin_f2<true, true>(s, bp, t, xg, slots, dcv, bins)
            : launch_xbin_f2<true, false>(s, bp, t, xg, slots, dcv, bins);
    else odd ? launch_xbin_f2<false, true>(s, bp, t, xg, slots, dcv, bins)
             : launch_xbin_f2<false, false>(s, bp, t, xg, slots, dcv, bins);
  } else {
    if (il) odd ? launch_xbin_t<1, true, true, 1>(s, bp, t, xg, slots, dcv, bins)
            : launch_xbin_t<1, true, false, 1>(s, bp, t, xg, slots, dcv, bins);
    else odd ? launch_xbin_t<1, false, true, 1>(s, bp, t, xg, slots, dcv, bins)
             : launch_xbin_t<1, false, false, 1>(s, bp, t, xg, slots, dcv, bins);
  }
  (*launches)++;
}

void bin_params_kguess(BinParams &bp, const capow_params &p) {
  const double bw = (p.Maxk - p.Mink) / (double)p.NK;
  bp.lg = p.OutputLog ? 1 : 0;
  bp.kscale = (float)(2.0 * M_PI / bw);
  bp.koff = (float)(-p.Mink / bw);
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

int bin_products(int nfields) { return nfields == 1 ? 1 : 4; }

template <typename R, int NF, bool ODD, bool OUT2D>
static void launch_bin_t(cudaStream_t s, const BinParams &bp, const BinTables &t, void *const slots[4],
                         const double *dcv, double *bins, double *bins2d) {
  typedef typename CT<R>::C C;
  constexpr int NP = NF == 1 ? 1 : 4;
  const long long cols = (long long)bp.ny * bp.nzc;
  const int th = 256;
  const int nbx = (int)((cols + th - 1) / th);
  int nchunk = (152 * 8 + nbx - 1) / nbx;
  if (nchunk < 1) nchunk = 1;
  if (nchunk > bp.nx) nchunk = bp.nx;
  const int ichunk = (bp.nx + nchunk - 1) / nchunk;
  nchunk = (bp.nx + ichunk - 1) / ichunk;
  const int n2d = OUT2D ? bp.nk * bp.nmu : 0;
  const int sm2d = (size_t)(NP * n2d) * sizeof(R) <= 64 * 1024 ? 1 : 0;
  const size_t smem = bin_smem_layout(sizeof(R), NP, bp.nk, sm2d ? n2d : 0, ichunk).total;
  cudaFuncSetAttribute(k_bin<R, NF, ODD, OUT2D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  // slot order: stencil * nfields + field
  const C *gA = (const C *)slots[0];
  const C *gB = NF == 2 ? (const C *)slots[1] : nullptr;
  const C *gAi = bp.interlace ? (const C *)slots[NF] : nullptr;
  const C *gBi = (bp.interlace && NF == 2) ? (const C *)slots[NF + 1] : nullptr;
  k_bin<R, NF, ODD, OUT2D><<<dim3(nbx, nchunk), th, smem, s>>>(bp, t, gA, gB, gAi, gBi, dcv, bins, bins2d, ichunk,
                                                                sm2d);
}

template <typename R, int NF>
static void launch_bin_r(cudaStream_t s, const BinParams &bp, const BinTables &t, void *const slots[4],
                         const double *dcv, double *bins, double *bins2d) {
  if (bp.odd) {
    if (bp.out2d) launch_bin_t<R, NF, true, true>(s, bp, t, slots, dcv, bins, bins2d);
    else launch_bin_t<R, NF, true, false>(s, bp, t, slots, dcv, bins, bins2d);
  } else {
    if (bp.out2d) launch_bin_t<R, NF, false, true>(s, bp, t, slots, dcv, bins, bins2d);
    else launch_bin_t<R, NF, false, false>(s, bp, t, slots, dcv, bins, bins2d);
  }
}

void launch_bin(cudaStream_t s, int precision, const BinParams &bp, const BinTables &t, void *const slots[4],
                const double *dcv, double *bins, double *bins2d, long long *launches) {
  if (precision == CAPOW_FP64) {
    if (bp.nfields == 1) launch_bin_r<double, 1>(s, bp, t, slots, dcv, bins, bins2d);
    else launch_bin_r<double, 2>(s, bp, t, slots, dcv, bins, bins2d);
  } else {
    if (bp.nfields == 1) launch_bin_r<float, 1>(s, bp, t, slots, dcv, bins, bins2d);
    else launch_bin_r<float, 2>(s, bp, t, slots, dcv, bins, bins2d);
  }
  (*launches)++;
}
