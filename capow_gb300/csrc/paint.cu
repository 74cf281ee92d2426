// Mass assignment (the reference's read_periodic_serial_ascii + add_to_grid + halo fold,
// src/read_data.c:32-179, 514-745) on the GPU.
//
// FP64 path (k_paint64): one thread per particle, the reference's double arithmetic,
// global FP64 atomics into zeroed grids. It is the plain FP64 GPU path.
//
// FP32 path (k_count -> k_scan -> k_scatter -> k_tile_paint): particles are bucketed into
// the output tiles their stencils touch (a counting sort; a particle near a tile face is
// listed in each neighbouring tile), then one CTA per tile accumulates every stencil tap of
// its particles in shared memory and writes the tile once with coalesced stores. Every grid
// cell is written exactly once: no memset of the grids, no global atomics on them. Particles
// within a few ulps of a discontinuity of the reference's rules (acceptance bounds, the TSC
// low-tap drop, the LOS==0 x shift, NN cell edges, non-finite input) take the exact FP64 rules
// inside the same tile kernel, so indices and acceptance match the reference bit for bit.
// The deterministic variant accumulates int64 fixed point in shared memory.
#include <cuda_runtime.h>
#include <math.h>

#include "paint.cuh"

#define FULL_MASK 0xffffffffu

// ------------------------------------------------------------------------------------------ util
__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum_f(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
  return v;
}

// Reduce `nv` per-thread doubles over the block and add them to global `dst`.
template <int NV>
__device__ void block_add(const double (&v)[NV], double *const (&dst)[NV]) {
  __shared__ double red[32][NV];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  double t[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) t[k] = warp_sum_d(v[k]);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; k++) red[wid][k] = t[k];
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) {
      double a = lane < nw ? red[lane][k] : 0.0;
      a = warp_sum_d(a);
      if (lane == 0 && a != 0.0) atomicAdd(dst[k], a);
    }
  }
  __syncthreads();
}

template <typename T>
__device__ __forceinline__ double ld64(const T *p, long long i) {
  return (double)p[i];
}

// ===================================================================================== FP64 path
template <typename T>
__global__ void __launch_bounds__(256) k_paint64(Geom g, FieldSpec fs, PIn<T> in, long long n, GridPtrs grids,
                                                 DevStats *st) {
  double l_read = 0, l_out = 0, l_grid = 0, l_nsq = 0, l_v[4] = {0, 0, 0, 0}, l_dc[4] = {0, 0, 0, 0};
  int fatal = 0, nonfin = 0;
  const int nf = fs.nfields;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double x = ld64(in.x, i), y = ld64(in.y, i), z = ld64(in.z, i);
    double v = fs.need_v ? ld64(in.v, i) : 0.0;
    double w = in.w ? ld64(in.w, i) : 1.0;
    if (!(isfinite(x) && isfinite(y) && isfinite(z) && isfinite(v) && isfinite(w))) {
      nonfin = 1;
      continue;
    }
    if (g.los == 1) x = rsd_shift64(g, x, v);
    else if (g.los == 2) y = rsd_shift64(g, y, v);
    else if (g.los == 3) z = rsd_shift64(g, z, v);
    l_read += 1.0;
    if (outside_box(g, x, y, z)) {
      if (g.los == 0) {
        fatal = 1;
        atomicMax(&st->fatal_inv, ~0ULL - (unsigned long long)i);
        continue;
      }
      l_out += 1.0;
    }
    const double val[2] = {wpow64(w, v, fs.ea), wpow64(w, v, fs.eb)};
    for (int stn = 0; stn < (g.interlace ? 2 : 1); stn++) {
      AxisTaps ax, ay, az;
      double px = x, py = y, pz = z;
      if (stn) {
        px = DADD(x, g.hx);
        py = DADD(y, g.hy);
        pz = DADD(z, g.hz);
      }
      if (!exact_axes(g, px, py, pz, ax, ay, az)) continue;
      if (stn == 0) l_grid += w;
      for (int f = 0; f < nf; f++) {
        double *gp = (double *)grids.g[stn * nf + f];
        double dsum = 0.0;
        for (int c = 0; c < az.n; c++) {
          if (!az.on[c]) continue;
          for (int b = 0; b < ay.n; b++) {
            if (!ay.on[b]) continue;
            for (int a = 0; a < ax.n; a++) {
              if (!ax.on[a]) continue;
              long long L = canon_index(g, ax.idx[a], ay.idx[b], az.idx[c]);
              if (L < 0) continue;
              double d = DMUL(DMUL(DMUL(val[f], ax.w[a]), ay.w[b]), az.w[c]);
              atomicAdd(gp + L, d);
              dsum += d;
            }
          }
        }
        l_dc[stn * nf + f] += dsum;
      }
    }
    if (fs.moments) {  // src/read_data.c:132-138
      l_nsq += w;
      double wv = DMUL(w, v);
      l_v[0] += wv;
      wv = DMUL(wv, v);
      l_v[1] += wv;
      wv = DMUL(wv, v);
      l_v[2] += wv;
      wv = DMUL(wv, v);
      l_v[3] += wv;
    }
  }
  const double vals[12] = {l_read, l_out, l_grid, l_nsq, l_v[0], l_v[1], l_v[2], l_v[3], l_dc[0], l_dc[1], l_dc[2], l_dc[3]};
  double *const dst[12] = {&st->nread, &st->nout, &st->ngrid, &st->nsq, &st->vr[0], &st->vr[1], &st->vr[2], &st->vr[3],
                           &st->dc[0], &st->dc[1], &st->dc[2], &st->dc[3]};
  block_add<12>(vals, dst);
  if (fatal) atomicOr(&st->fatal, 1);
  if (nonfin) atomicOr(&st->nonfinite, 1);
}

static int grid_blocks(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b > 152LL * 16) b = 152LL * 16;
  if (b < 1) b = 1;
  return (int)b;
}

void launch_paint64(cudaStream_t s, const Geom &g, const FieldSpec &fs, int dtype, const void *x, const void *y,
                    const void *z, const void *v, const void *w, long long n, const GridPtrs &grids, DevStats *st,
                    long long *launches) {
  const int th = 256, nb = grid_blocks(n, th);
  if (dtype == CAPOW_F64) {
    PIn<double> in{(const double *)x, (const double *)y, (const double *)z, (const double *)v, (const double *)w};
    k_paint64<double><<<nb, th, 0, s>>>(g, fs, in, n, grids, st);
  } else {
    PIn<float> in{(const float *)x, (const float *)y, (const float *)z, (const float *)v, (const float *)w};
    k_paint64<float><<<nb, th, 0, s>>>(g, fs, in, n, grids, st);
  }
  (*launches)++;
}

// ===================================================================================== FP32 path
// Normal-stencil scales of one particle after the RSD shift, in FP32, and whether it must take
// the exact rules. Explicit round-to-nearest intrinsics keep the result identical in every
// kernel that recomputes it (count, scatter and tile kernels must agree on the tap set).
struct Prep {
  float sx, sy, sz, v, w;
  bool edge;
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
  bool fin = isfinite(p.sx) && isfinite(p.sy) && isfinite(p.sz) && isfinite(p.v) && isfinite(p.w);
  bool e = !fin || near_edge(p.sx, g.nx, g.order, g.margin) || near_edge(p.sy, g.ny, g.order, g.margin) ||
           near_edge(p.sz, g.nz, g.order, g.margin);
  if (g.interlace)
    e = e || near_edge(__fadd_rn(p.sx, 0.5f), g.nx, g.order, g.margin) ||
        near_edge(__fadd_rn(p.sy, 0.5f), g.ny, g.order, g.margin) ||
        near_edge(__fadd_rn(p.sz, 0.5f), g.nz, g.order, g.margin);
  p.edge = e;
  return p;
}

struct AxisTiles {
  int n;
  int t[4];
};

__device__ __forceinline__ void add_tile(AxisTiles &a, int v) {
  for (int k = 0; k < a.n; k++)
    if (a.t[k] == v) return;
  if (a.n < 4) a.t[a.n++] = v;
}

// Per-axis tile coordinates touched by the accepted stencils of a regular particle.
__device__ __forceinline__ int regular_tiles(const Geom &g, const TileGeo &tg, float sx, float sy, float sz,
                                             AxisTiles &TX, AxisTiles &TY, AxisTiles &TZ) {
  TX.n = TY.n = TZ.n = 0;
  const int nst = g.interlace ? 2 : 1;
  for (int stn = 0; stn < nst; stn++) {
    float ax = stn ? __fadd_rn(sx, 0.5f) : sx, ay = stn ? __fadd_rn(sy, 0.5f) : sy, az = stn ? __fadd_rn(sz, 0.5f) : sz;
    if (!accept32(g, ax, ay, az)) continue;
    AxisTapsF tx, ty, tz;
    axis32(g.order, ax, 0, g.nx, g.los, tx);
    axis32(g.order, ay, 1, g.ny, g.los, ty);
    axis32(g.order, az, 1, g.nz, g.los, tz);
    for (int k = 0; k < 3; k++) {
      if (tx.idx[k] >= 0 && tx.idx[k] < g.nx) add_tile(TX, tx.idx[k] / tg.tx);
      if (ty.idx[k] >= 0 && ty.idx[k] < g.ny) add_tile(TY, ty.idx[k] / tg.ty);
      if (tz.idx[k] >= 0 && tz.idx[k] < g.nz) add_tile(TZ, tz.idx[k] / tg.tz);
    }
  }
  return TX.n * TY.n * TZ.n;
}

__device__ __forceinline__ int tile_id(const TileGeo &tg, int bx, int by, int bz) {
  return (bx * tg.nby + by) * tg.nbz + bz;
}

// Warp-aggregated atomic add of 1 to counter[key] for active lanes; returns each lane's slot.
__device__ __forceinline__ unsigned agg_inc(unsigned *counter, int key, bool active) {
  const unsigned lane = threadIdx.x & 31;
  unsigned amask = __ballot_sync(FULL_MASK, active);
  unsigned res = 0;
  if (active) {
    unsigned peers = __match_any_sync(amask, key);
    int leader = __ffs(peers) - 1;
    unsigned base = 0;
    if ((int)lane == leader) base = atomicAdd(counter + key, (unsigned)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    res = base + __popc(peers & ((1u << lane) - 1));
  }
  return res;
}

// Exact FP64 view of one particle (RSD shift in the reference's order).
template <typename T>
__device__ __forceinline__ void exact_pos(const Geom &g, const FieldSpec &fs, const PIn<T> &in, long long i, double &x,
                                          double &y, double &z, double &v, double &w) {
  x = (double)in.x[i];
  y = (double)in.y[i];
  z = (double)in.z[i];
  v = fs.need_v ? (double)in.v[i] : 0.0;
  w = in.w ? (double)in.w[i] : 1.0;
  if (g.los == 1) x = rsd_shift64(g, x, v);
  else if (g.los == 2) y = rsd_shift64(g, y, v);
  else if (g.los == 3) z = rsd_shift64(g, z, v);
}

// Decode a canonical padded index into cell coordinates.
__device__ __forceinline__ void decode(const Geom &g, long long L, int &ix, int &iy, int &iz) {
  ix = (int)(L / g.slice);
  long long r = L - (long long)ix * g.slice;
  iy = (int)(r / g.row);
  iz = (int)(r - (long long)iy * g.row);
}

// Tiles touched by the exact taps of an edge particle (both stencils), deduplicated.
// Returns the count; writes at most `cap` ids.
template <int CAP>
__device__ int exact_tiles(const Geom &g, const TileGeo &tg, double x, double y, double z, int (&ids)[CAP]) {
  int n = 0;
  for (int stn = 0; stn < (g.interlace ? 2 : 1); stn++) {
    AxisTaps ax, ay, az;
    double px = stn ? DADD(x, g.hx) : x, py = stn ? DADD(y, g.hy) : y, pz = stn ? DADD(z, g.hz) : z;
    if (!exact_axes(g, px, py, pz, ax, ay, az)) continue;
    for (int c = 0; c < az.n; c++)
      for (int b = 0; b < ay.n; b++)
        for (int a = 0; a < ax.n; a++) {
          if (!(ax.on[a] && ay.on[b] && az.on[c])) continue;
          long long L = canon_index(g, ax.idx[a], ay.idx[b], az.idx[c]);
          if (L < 0) continue;
          int ix, iy, iz;
          decode(g, L, ix, iy, iz);
          int t = tile_id(tg, ix / tg.tx, iy / tg.ty, iz / tg.tz);
          bool seen = false;
          for (int k = 0; k < n; k++) seen |= (ids[k] == t);
          if (!seen && n < CAP) ids[n++] = t;
        }
  }
  return n;
}

// Pass 1: statistics, tile counts for regular particles, list of edge particles.
template <typename T>
__global__ void __launch_bounds__(256) k_count(Geom g, FieldSpec fs, TileGeo tg, PIn<T> in, long long n,
                                               unsigned *counts, unsigned *special, DevStats *st) {
  float f_read = 0, f_out = 0, f_grid = 0, f_nsq = 0, f_v[4] = {0, 0, 0, 0}, f_abs[2] = {0, 0};
  double d_grid = 0, d_out = 0, d_nsq = 0, d_v[4] = {0, 0, 0, 0};
  int fatal = 0, nonfin = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long nround = (n + stride - 1) / stride * stride;  // warp-uniform trip count
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nround; i += stride) {
    const bool live = i < n;
    bool reg = false;
    AxisTiles TX, TY, TZ;
    int ntile = 0;
    if (live) {
      Prep p = prep32(g, fs, in, i);
      if (p.edge) {
        unsigned slot = atomicAdd(&st->nspecial, 1u);
        special[slot] = (unsigned)i;
        double x, y, z, v, w;
        exact_pos(g, fs, in, i, x, y, z, v, w);
        if (!(isfinite(x) && isfinite(y) && isfinite(z) && isfinite(v) && isfinite(w))) {
          nonfin = 1;
        } else {
          f_read += 1.0f;
          bool out = outside_box(g, x, y, z);
          if (out && g.los == 0) {
            fatal = 1;
            atomicMax(&st->fatal_inv, ~0ULL - (unsigned long long)i);
          }
          if (out) d_out += 1.0;
          AxisTaps ax, ay, az;
          if (exact_axes(g, x, y, z, ax, ay, az)) d_grid += w;
          if (fs.moments) {
            d_nsq += w;
            double wv = DMUL(w, v);
            d_v[0] += wv; wv = DMUL(wv, v);
            d_v[1] += wv; wv = DMUL(wv, v);
            d_v[2] += wv; wv = DMUL(wv, v);
            d_v[3] += wv;
          }
          f_abs[0] += (float)fabs(wpow64(w, v, fs.ea));
          f_abs[1] += (float)fabs(wpow64(w, v, fs.eb));
        }
      } else {
        f_read += 1.0f;
        const bool out = (p.sx < 0.0f) || (p.sx > (float)g.nx) || (p.sy < 0.0f) || (p.sy > (float)g.ny) ||
                         (p.sz < 0.0f) || (p.sz > (float)g.nz);
        if (out && g.los == 0) {
          fatal = 1;
          atomicMax(&st->fatal_inv, ~0ULL - (unsigned long long)i);
        }
        if (out) f_out += 1.0f;
        if (accept32(g, p.sx, p.sy, p.sz)) f_grid += p.w;
        if (fs.moments) {
          f_nsq += p.w;
          float wv = p.w * p.v;
          f_v[0] += wv; wv *= p.v;
          f_v[1] += wv; wv *= p.v;
          f_v[2] += wv; wv *= p.v;
          f_v[3] += wv;
        }
        float pa = p.w, pb = p.w;
        for (int e = 0; e < fs.ea; e++) pa *= p.v;
        for (int e = 0; e < fs.eb; e++) pb *= p.v;
        f_abs[0] += fabsf(pa);
        f_abs[1] += fabsf(pb);
        ntile = regular_tiles(g, tg, p.sx, p.sy, p.sz, TX, TY, TZ);
        reg = true;
      }
    }
    // warp-uniform loop over the up-to-8 tiles of each regular particle
    int maxt = __reduce_max_sync(FULL_MASK, reg ? ntile : 0);
    for (int k = 0; k < maxt; k++) {
      bool act = reg && k < ntile;
      int key = 0;
      if (act) {
        int a = k % TX.n, b = (k / TX.n) % TY.n, c = k / (TX.n * TY.n);
        key = tile_id(tg, TX.t[a], TY.t[b], TZ.t[c]);
      }
      agg_inc(counts, key, act);
    }
  }
  // FP32 partials are per thread over ~n/(grid threads) particles; promoted to FP64 per warp
  const double vals[10] = {(double)f_read, d_out + (double)f_out, d_grid + (double)f_grid, d_nsq + (double)f_nsq,
                           d_v[0] + (double)f_v[0], d_v[1] + (double)f_v[1], d_v[2] + (double)f_v[2],
                           d_v[3] + (double)f_v[3], (double)f_abs[0], (double)f_abs[1]};
  double *const dst[10] = {&st->nread, &st->nout, &st->ngrid, &st->nsq, &st->vr[0], &st->vr[1], &st->vr[2], &st->vr[3],
                           &st->absw[0], &st->absw[1]};
  block_add<10>(vals, dst);
  if (fatal) atomicOr(&st->fatal, 1);
  if (nonfin) atomicOr(&st->nonfinite, 1);
}

// Pass 1b: tile counts of the edge particles (exact taps).
template <typename T>
__global__ void k_count_special(Geom g, FieldSpec fs, TileGeo tg, PIn<T> in, const unsigned *special, DevStats *st,
                                unsigned *counts) {
  const unsigned ns = st->nspecial;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < ns; k += gridDim.x * blockDim.x) {
    double x, y, z, v, w;
    exact_pos(g, fs, in, special[k], x, y, z, v, w);
    if (!(isfinite(x) && isfinite(y) && isfinite(z) && isfinite(v) && isfinite(w))) continue;
    int ids[64];
    int nt = exact_tiles<64>(g, tg, x, y, z, ids);
    for (int t = 0; t < nt; t++) atomicAdd(counts + ids[t], 1u);
  }
}

// Pass 2: exclusive scan of the tile counts (one CTA), cursor copy, record total, fixed-point scales.
__global__ void __launch_bounds__(1024) k_scan(const unsigned *counts, int ntiles, unsigned *offsets, unsigned *cursor,
                                               DevStats *st, unsigned long long capacity, double *fixed_scale) {
  __shared__ unsigned long long part[1024];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int per = (ntiles + nt - 1) / nt;
  const int b = tid * per, e = min(ntiles, b + per);
  unsigned long long s = 0;
  for (int i = b; i < e; i++) s += counts[i];
  part[tid] = s;
  __syncthreads();
  for (int o = 1; o < nt; o <<= 1) {  // Hillis-Steele inclusive scan of the per-thread sums
    unsigned long long a = tid >= o ? part[tid - o] : 0;
    __syncthreads();
    part[tid] += a;
    __syncthreads();
  }
  unsigned long long run = part[tid] - s;
  for (int i = b; i < e; i++) {
    offsets[i] = (unsigned)run;
    cursor[i] = (unsigned)run;
    run += counts[i];
  }
  if (tid == nt - 1) {
    offsets[ntiles] = (unsigned)part[nt - 1];
    st->nrecords = (unsigned)part[nt - 1];
    if (part[nt - 1] > capacity) st->overflow = 1;
    // fixed-point scale per field: 2^S with sum|contrib| * 2^S < 2^62
    for (int f = 0; f < 2; f++) {
      double bound = st->absw[f] * 1.0001 + 1.0;
      int S = 62 - (int)ceil(log2(bound));
      if (S > 60) S = 60;
      fixed_scale[f] = ldexp(1.0, S);
    }
  }
}

#define SPECIAL_MARK (-3.0e38f)

// Pass 3: scatter regular particles into their tiles' lists.
template <typename T>
__global__ void __launch_bounds__(256) k_scatter(Geom g, FieldSpec fs, TileGeo tg, PIn<T> in, long long n,
                                                 unsigned *cursor, float4 *recs, float *recw,
                                                 unsigned long long capacity) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long nround = (n + stride - 1) / stride * stride;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nround; i += stride) {
    bool reg = false;
    AxisTiles TX, TY, TZ;
    int ntile = 0;
    Prep p;
    if (i < n) {
      p = prep32(g, fs, in, i);
      if (!p.edge) {
        reg = true;
        ntile = regular_tiles(g, tg, p.sx, p.sy, p.sz, TX, TY, TZ);
      }
    }
    int maxt = __reduce_max_sync(FULL_MASK, reg ? ntile : 0);
    for (int k = 0; k < maxt; k++) {
      bool act = reg && k < ntile;
      int key = 0;
      if (act) {
        int a = k % TX.n, b = (k / TX.n) % TY.n, c = k / (TX.n * TY.n);
        key = tile_id(tg, TX.t[a], TY.t[b], TZ.t[c]);
      }
      unsigned slot = agg_inc(cursor, key, act);
      if (act && slot < capacity) {
        recs[slot] = make_float4(p.sx, p.sy, p.sz, p.v);
        if (recw) recw[slot] = p.w;
      }
    }
  }
}

// Pass 3b: scatter edge particles (record carries the particle index).
template <typename T>
__global__ void k_scatter_special(Geom g, FieldSpec fs, TileGeo tg, PIn<T> in, const unsigned *special,
                                  const DevStats *st, unsigned *cursor, float4 *recs, unsigned long long capacity) {
  const unsigned ns = st->nspecial;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < ns; k += gridDim.x * blockDim.x) {
    const unsigned idx = special[k];
    double x, y, z, v, w;
    exact_pos(g, fs, in, idx, x, y, z, v, w);
    if (!(isfinite(x) && isfinite(y) && isfinite(z) && isfinite(v) && isfinite(w))) continue;
    int ids[64];
    int nt = exact_tiles<64>(g, tg, x, y, z, ids);
    for (int t = 0; t < nt; t++) {
      unsigned slot = atomicAdd(cursor + ids[t], 1u);
      if (slot < capacity) recs[slot] = make_float4(SPECIAL_MARK, __uint_as_float(idx), 0.0f, 0.0f);
    }
  }
}

// Pass 4: one CTA per tile. Shared memory holds the tile of every grid slot; taps outside
// the tile are skipped (another tile owns them).
template <typename Acc>
struct TileAcc;
template <>
struct TileAcc<float> {
  __device__ static void add(float *p, double vd, float vf, double) { atomicAdd(p, vf); (void)vd; }
};
template <>
struct TileAcc<unsigned long long> {
  __device__ static void add(unsigned long long *p, double vd, float, double scale) {
    atomicAdd(p, (unsigned long long)__double2ll_rn(vd * scale));
  }
};

template <typename T, typename Acc>
__global__ void __launch_bounds__(256) k_tile_paint(Geom g, FieldSpec fs, TileGeo tg, PIn<T> in,
                                                    long long n, const unsigned *offsets, const float4 *recs,
                                                    const float *recw, unsigned long long capacity, GridPtrs grids,
                                                    const double *fixed_scale, DevStats *st) {
  extern __shared__ __align__(16) unsigned char smraw[];
  Acc *sm = (Acc *)smraw;
  const int nf = fs.nfields, nst = g.interlace ? 2 : 1, nslot = nf * nst;
  const int tsz = tg.tx * tg.ty * tg.tz;
  const int tile = blockIdx.x;
  const int bz = tile % tg.nbz, by = (tile / tg.nbz) % tg.nby, bx = tile / (tg.nbz * tg.nby);
  const int x0 = bx * tg.tx, y0 = by * tg.ty, z0 = bz * tg.tz;
  const int ex = min(tg.tx, g.nx - x0), ey = min(tg.ty, g.ny - y0), ez = min(tg.tz, g.nz - z0);
  for (int c = threadIdx.x; c < nslot * tsz; c += blockDim.x) sm[c] = (Acc)0;
  __syncthreads();
  const double sc0 = fixed_scale ? fixed_scale[0] : 1.0, sc1 = fixed_scale ? fixed_scale[1] : 1.0;
  unsigned rb = offsets[tile], re = offsets[tile + 1];
  if (re > capacity) re = (unsigned)capacity;
  if (rb > re) rb = re;
  for (unsigned r = rb + threadIdx.x; r < re; r += blockDim.x) {
    const float4 rec = recs[r];
    if (rec.x == SPECIAL_MARK) {  // exact FP64 rules
      const unsigned idx = __float_as_uint(rec.y);
      if ((long long)idx >= n) continue;
      double x, y, z, v, w;
      exact_pos(g, fs, in, idx, x, y, z, v, w);
      const double val[2] = {wpow64(w, v, fs.ea), wpow64(w, v, fs.eb)};
      for (int stn = 0; stn < nst; stn++) {
        AxisTaps ax, ay, az;
        double px = stn ? DADD(x, g.hx) : x, py = stn ? DADD(y, g.hy) : y, pz = stn ? DADD(z, g.hz) : z;
        if (!exact_axes(g, px, py, pz, ax, ay, az)) continue;
        for (int c = 0; c < az.n; c++)
          for (int b = 0; b < ay.n; b++)
            for (int a = 0; a < ax.n; a++) {
              if (!(ax.on[a] && ay.on[b] && az.on[c])) continue;
              long long L = canon_index(g, ax.idx[a], ay.idx[b], az.idx[c]);
              if (L < 0) continue;
              int ix, iy, iz;
              decode(g, L, ix, iy, iz);
              ix -= x0; iy -= y0; iz -= z0;
              if (ix < 0 || ix >= ex || iy < 0 || iy >= ey || iz < 0 || iz >= ez) continue;
              const int cell = (ix * tg.ty + iy) * tg.tz + iz;
              for (int f = 0; f < nf; f++) {
                double d = DMUL(DMUL(DMUL(val[f], ax.w[a]), ay.w[b]), az.w[c]);
                TileAcc<Acc>::add(sm + (stn * nf + f) * tsz + cell, d, (float)d, f ? sc1 : sc0);
              }
            }
      }
      continue;
    }
    const float w = recw ? recw[r] : 1.0f;
    float va = w, vb = w;
    for (int e = 0; e < fs.ea; e++) va *= rec.w;
    for (int e = 0; e < fs.eb; e++) vb *= rec.w;
    for (int stn = 0; stn < nst; stn++) {
      float sx = stn ? __fadd_rn(rec.x, 0.5f) : rec.x, sy = stn ? __fadd_rn(rec.y, 0.5f) : rec.y,
            sz = stn ? __fadd_rn(rec.z, 0.5f) : rec.z;
      if (!accept32(g, sx, sy, sz)) continue;
      AxisTapsF tx, ty, tz;
      axis32(g.order, sx, 0, g.nx, g.los, tx);
      axis32(g.order, sy, 1, g.ny, g.los, ty);
      axis32(g.order, sz, 1, g.nz, g.los, tz);
      int lx[3], ly[3], lz[3];
#pragma unroll
      for (int k = 0; k < 3; k++) {
        int a = tx.idx[k] - x0, b = ty.idx[k] - y0, c = tz.idx[k] - z0;
        lx[k] = (tx.idx[k] >= 0 && a >= 0 && a < ex) ? a : -1;
        ly[k] = (ty.idx[k] >= 0 && b >= 0 && b < ey) ? b : -1;
        lz[k] = (tz.idx[k] >= 0 && c >= 0 && c < ez) ? c : -1;
      }
      Acc *s0 = sm + (stn * nf) * tsz;
#pragma unroll
      for (int a = 0; a < 3; a++) {
        if (lx[a] < 0) continue;
        const float wa = tx.w[a];
#pragma unroll
        for (int b = 0; b < 3; b++) {
          if (ly[b] < 0) continue;
          const float wab = wa * ty.w[b];
          const int rowc = (lx[a] * tg.ty + ly[b]) * tg.tz;
#pragma unroll
          for (int c = 0; c < 3; c++) {
            if (lz[c] < 0) continue;
            const float wt = wab * tz.w[c];
            const int cell = rowc + lz[c];
            TileAcc<Acc>::add(s0 + cell, (double)(va * wt), va * wt, sc0);
            if (nf == 2) TileAcc<Acc>::add(s0 + tsz + cell, (double)(vb * wt), vb * wt, sc1);
          }
        }
      }
    }
  }
  __syncthreads();
  // write the tile: rows along z are contiguous in the padded layout
  double dc[4] = {0, 0, 0, 0};
  unsigned long long dcf[4] = {0, 0, 0, 0};
  const int rows = ex * ey;
  for (int slot = 0; slot < nslot; slot++) {
    float *gp = (float *)grids.g[slot];
    const Acc *s = sm + slot * tsz;
    const double inv = (slot % nf) ? 1.0 / sc1 : 1.0 / sc0;
    for (int q = threadIdx.x; q < rows * ez; q += blockDim.x) {
      const int rz = q % ez, rr = q / ez;
      const int ly = rr % ey, lx = rr / ey;
      const Acc a = s[(lx * tg.ty + ly) * tg.tz + rz];
      float val;
      if (sizeof(Acc) == 8) {
        val = (float)((double)(long long)a * inv);
        dcf[slot] += (unsigned long long)a;
      } else {
        val = (float)a;
        dc[slot] += (double)val;
      }
      gp[(long long)(x0 + lx) * g.slice + (long long)(y0 + ly) * g.row + z0 + rz] = val;
    }
  }
  if (sizeof(Acc) == 8) {
    for (int slot = 0; slot < nslot; slot++) {
      unsigned long long v = dcf[slot];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
      if ((threadIdx.x & 31) == 0 && v) atomicAdd(&st->dc_fixed[slot], v);
    }
  } else {
    const double vals[4] = {dc[0], dc[1], dc[2], dc[3]};
    double *const dst[4] = {&st->dc[0], &st->dc[1], &st->dc[2], &st->dc[3]};
    block_add<4>(vals, dst);
  }
}

TileGeo choose_tiles(const Geom &g, int nslots, int deterministic) {
  TileGeo t;
  // 4 grid slots x 8x16x32 floats = 64 KB (three CTAs per SM); the int64 variant halves the volume.
  t.tx = 8;
  t.ty = 16;
  t.tz = 32;
  if (deterministic) t.tx = (nslots > 2) ? 4 : 8;
  else if (nslots <= 2) t.tx = 16;
  if (t.tz > g.nz) t.tz = g.nz;
  if (t.ty > g.ny) t.ty = g.ny;
  if (t.tx > g.nx) t.tx = g.nx;
  t.nbx = (g.nx + t.tx - 1) / t.tx;
  t.nby = (g.ny + t.ty - 1) / t.ty;
  t.nbz = (g.nz + t.tz - 1) / t.tz;
  t.ntiles = t.nbx * t.nby * t.nbz;
  return t;
}

size_t tile_smem_bytes(const TileGeo &tg, int nslots, int deterministic) {
  return (size_t)nslots * tg.tx * tg.ty * tg.tz * (deterministic ? 8 : 4);
}

double tile_dup_estimate(const Geom &g, const TileGeo &tg) {
  // a particle is listed in a neighbour tile when it lies within ~2.5 cells of the face
  double m = (g.order == 3) ? 2.5 : (g.order == 2 ? 1.5 : 0.5);
  if (!g.interlace) m -= 0.5;
  return (1.0 + m / tg.tx) * (1.0 + m / tg.ty) * (1.0 + m / tg.tz);
}

template <typename T>
static void run_paint32(cudaStream_t s, const Geom &g, const FieldSpec &fs, const TileGeo &tg, int det, PIn<T> in,
                        long long n, const GridPtrs &grids, const PaintBufs &b, DevStats *st, long long *launches) {
  const int th = 256, nb = grid_blocks(n, th) * 2;
  cudaMemsetAsync(b.counts, 0, sizeof(unsigned) * tg.ntiles, s);
  k_count<T><<<nb, th, 0, s>>>(g, fs, tg, in, n, b.counts, b.special, st);
  k_count_special<T><<<152, 128, 0, s>>>(g, fs, tg, in, b.special, st, b.counts);
  k_scan<<<1, 1024, 0, s>>>(b.counts, tg.ntiles, b.offsets, b.cursor, st, b.capacity, b.fixed_scale);
  k_scatter<T><<<nb, th, 0, s>>>(g, fs, tg, in, n, b.cursor, b.recs, in.w ? b.recw : nullptr, b.capacity);
  k_scatter_special<T><<<152, 128, 0, s>>>(g, fs, tg, in, b.special, st, b.cursor, b.recs, b.capacity);
  const int nslot = fs.nfields * (g.interlace ? 2 : 1);
  const size_t smem = tile_smem_bytes(tg, nslot, det);
  if (det) {
    cudaFuncSetAttribute(k_tile_paint<T, unsigned long long>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_tile_paint<T, unsigned long long><<<tg.ntiles, 256, smem, s>>>(g, fs, tg, in, n, b.offsets, b.recs,
                                                                      in.w ? b.recw : nullptr, b.capacity, grids,
                                                                      b.fixed_scale, st);
  } else {
    cudaFuncSetAttribute(k_tile_paint<T, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_tile_paint<T, float><<<tg.ntiles, 256, smem, s>>>(g, fs, tg, in, n, b.offsets, b.recs, in.w ? b.recw : nullptr,
                                                        b.capacity, grids, nullptr, st);
  }
  *launches += 6;
}

void launch_paint32(cudaStream_t s, const Geom &g, const FieldSpec &fs, const TileGeo &tg, int deterministic,
                    int dtype, const void *x, const void *y, const void *z, const void *v, const void *w,
                    long long n, const GridPtrs &grids, const PaintBufs &b, DevStats *st, long long *launches) {
  if (dtype == CAPOW_F64) {
    PIn<double> in{(const double *)x, (const double *)y, (const double *)z, (const double *)v, (const double *)w};
    run_paint32<double>(s, g, fs, tg, deterministic, in, n, grids, b, st, launches);
  } else {
    PIn<float> in{(const float *)x, (const float *)y, (const float *)z, (const float *)v, (const float *)w};
    run_paint32<float>(s, g, fs, tg, deterministic, in, n, grids, b, st, launches);
  }
}
