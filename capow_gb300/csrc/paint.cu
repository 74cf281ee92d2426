// Mass assignment (the reference's read_periodic_serial_ascii + add_to_grid + halo fold,
// src/read_data.c:32-179, 514-745) on the GPU.
//
// FP64 path (k_paint64): one thread per particle, the reference's double arithmetic,
// global FP64 atomics into zeroed grids. It is the plain FP64 GPU path.
//
// FP32 path (k_bucket -> k_tile_rec -> k_edge_fixup; deterministic: k_count -> k_scan -> k_scatter ->
// k_tile_rec_det): particles are bucketed into the output tiles their stencils touch (a counting sort; a particle near a tile face is
// listed in each neighbouring tile), then one CTA per tile accumulates every stencil tap of
// its particles in shared memory and writes the tile once with coalesced stores. Every grid
// cell is written exactly once: no memset of the grids, no global atomics on them. Particles
// within a few ulps of a discontinuity of the reference's rules (acceptance bounds, the TSC
// low-tap drop, the LOS==0 x shift, NN cell edges, non-finite input) take the exact FP64 rules
// (k_edge_fixup; in the deterministic variant, inside the tile kernel), so indices and acceptance match
// the reference bit for bit. The deterministic variant accumulates int64 fixed point in shared memory.
#include <cuda_runtime.h>
#include <math.h>

#include "paint.cuh"
#include "paint_dev.cuh"

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

// Reduce `nv` per-thread floats over the block in FP32 within each warp (32 terms) and in FP64
// across warps, and add them to global `dst` (one FP64 atomic per value and block).
template <int NV>
__device__ void block_add_f(const float (&v)[NV], double *const (&dst)[NV]) {
  __shared__ double redf[32][NV];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  float t[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) t[k] = warp_sum_f(v[k]);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; k++) redf[wid][k] = (double)t[k];
  __syncthreads();
  if (wid == 0 && lane < NV) {
    double a = 0.0;
    for (int w = 0; w < nw; w++) a += redf[w][lane];
    if (a != 0.0) atomicAdd(dst[lane], a);
  }
  __syncthreads();
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
// Normal-stencil scales of one particle after the RSD shift, in FP32. Explicit round-to-nearest
// intrinsics keep the result identical in every kernel that recomputes it (the count, scatter
// and tile kernels must agree on each particle's tiles).
// Distinct tile coordinates along one axis, in registers (at most three: a footprint spans at
// most six cells and tiles are at least four cells long, except a short partial last tile).
struct AxisTiles {
  int t0, t1, t2, n;
};

__device__ __forceinline__ void add_tile(AxisTiles &a, int v) {
  const bool dup = ((a.n > 0) & (v == a.t0)) | ((a.n > 1) & (v == a.t1)) | ((a.n > 2) & (v == a.t2));
  const bool put = !dup;
  a.t0 = (put & (a.n == 0)) ? v : a.t0;
  a.t1 = (put & (a.n == 1)) ? v : a.t1;
  a.t2 = (put & (a.n >= 2)) ? v : a.t2;
  a.n = (put & (a.n < 3)) ? a.n + 1 : a.n;
}

__device__ __forceinline__ int tile_at(const AxisTiles &a, int k) { return k == 0 ? a.t0 : (k == 1 ? a.t1 : a.t2); }

__device__ __forceinline__ int tile_id(const TileGeo &tg, int bx, int by, int bz) {
  return (bx * tg.nby + by) * tg.nbz + bz;
}

// Cells any accepted stencil (normal and interlaced) of a particle at scale s can write along one
// axis, widened by the FP32 margin: [floor(s-m)-1, floor(s+m)+2] for TSC, [floor(s-m), floor(s+m)+2]
// for CIC, [floor(s-m), floor(s+m)+1] for NN. Wrapping axes (LOS == 0: periodic y, z and the x halo
// fold) take the cells modulo N; other axes clip to the grid. Returns false when nothing of the
// footprint lies in the grid (the particle is outside the box and rejected).
// [low, lim): where either stencil of a particle at s is accepted along a non-wrapping axis (lim = n,
// or n + 1 for the TSC x axis; low = 0, or -1/2 when the interlaced copy at s + 1/2 is painted too).
// A particle beyond that range by more than the margin is rejected by both and lies outside the box,
// so it is counted out without the exact rules.
__device__ __forceinline__ bool axis_range(float s, int n, bool wrap, int order, float m, float low, float lim,
                                           int &lo, int &hi) {
  if (!(s > -4.0f && s < (float)n + 4.0f)) return false;
  if (!wrap && (s < low - m || s >= lim + m)) return false;
  lo = __float2int_rd(__fsub_rn(s, m)) - (order == 3 ? 1 : 0);
  hi = __float2int_rd(__fadd_rn(s, m)) + (order == 1 ? 1 : 2);
  if (!wrap) {
    lo = lo < 0 ? 0 : lo;
    hi = hi > n - 1 ? n - 1 : hi;
    return lo <= hi;
  }
  const int span = hi - lo;
  // s > -4 and margin < 0.25 give -6 <= lo <= n + 2, and n >= 4: these corrections bring lo into [0, n)
  lo += lo < 0 ? n : 0;
  lo += lo < 0 ? n : 0;
  lo -= lo >= n ? n : 0;
  hi = lo + span;  // cells beyond n - 1 wrap when used
  return true;
}

// The tiles of the cells lo..hi (hi may pass n - 1 on a wrapping axis): the piece inside the grid
// covers tiles lo >> shift .. min(hi, n - 1) >> shift, the wrapped piece 0 .. (hi - n) >> shift.
__device__ __forceinline__ bool axis_footprint(float s, int n, int shift, bool wrap, int order, float m, float low,
                                               float lim, AxisTiles &T) {
  T.n = 0;
  T.t0 = T.t1 = T.t2 = 0;
  int lo, hi;
  if (!axis_range(s, n, wrap, order, m, low, lim, lo, hi)) return false;
  const int top = hi < n - 1 ? hi : n - 1;
  const int a0 = lo >> shift, a1 = top >> shift;  // a1 - a0 <= 2: the footprint spans at most 6 cells
  T.t0 = a0;
  T.t1 = a0 + 1;
  T.t2 = a0 + 2;
  T.n = a1 - a0 + 1;
  if (hi >= n) {  // the wrapped piece (rare: a periodic axis near its last cell)
    const int wtop = hi - n < n - 1 ? hi - n : n - 1;
    for (int t = 0; t <= (wtop >> shift); t++) add_tile(T, t);
  }
  return true;
}

// All tiles of a particle. The first tile of each axis list gives the particle's home tile (the one
// tile that counts it in the statistics).
__device__ __forceinline__ bool footprint(const Geom &g, const TileGeo &tg, float sx, float sy, float sz,
                                          AxisTiles &TX, AxisTiles &TY, AxisTiles &TZ) {
  const bool wrap = g.los == 0;
  const float limx = (float)g.nx + (g.order == 3 ? 1.0f : 0.0f);  // src/read_data.c:618-619
  const float low = g.interlace ? -0.5f : 0.0f;
  if (!axis_footprint(sx, g.nx, tg.lx, wrap, g.order, g.margin, low, limx, TX)) return false;
  if (!axis_footprint(sy, g.ny, tg.ly, wrap, g.order, g.margin, low, (float)g.ny, TY)) return false;
  if (!axis_footprint(sz, g.nz, tg.lz, wrap, g.order, g.margin, low, (float)g.nz, TZ)) return false;
  // CIC rounding edge: a y index equal to NY makes the reference's linear index land in row 0 of
  // the next x slice (src/read_data.c:592-593); that row's tile joins the list.
  if (g.order == 2 && sy > (float)g.ny - 1.5f - g.margin) add_tile(TY, 0);
  return true;
}

// The home tile without building the lists: the tile of the first cell of each axis range
// (the same tile footprint() puts first). Returns -1 when the footprint misses the grid.
__device__ __forceinline__ int home_of(const Geom &g, const TileGeo &tg, float sx, float sy, float sz) {
  const bool wrap = g.los == 0;
  int lx, hx, ly, hy, lz, hz;
  const float limx = (float)g.nx + (g.order == 3 ? 1.0f : 0.0f);
  const float low = g.interlace ? -0.5f : 0.0f;
  if (!axis_range(sx, g.nx, wrap, g.order, g.margin, low, limx, lx, hx)) return -1;
  if (!axis_range(sy, g.ny, wrap, g.order, g.margin, low, (float)g.ny, ly, hy)) return -1;
  if (!axis_range(sz, g.nz, wrap, g.order, g.margin, low, (float)g.nz, lz, hz)) return -1;
  return tile_id(tg, lx >> tg.lx, ly >> tg.ly, lz >> tg.lz);
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

// Warp-aggregated tile counters over runs: consecutive lanes naming the same tile form a run and
// share one atomic, issued by the run's first lane (particles that arrive in spatial order form
// long runs; any order stays correct). Every lane of the warp must call this; lanes with key < 0
// take no slot. Returns the lane's slot: the counter's old value plus its offset in the run.
__device__ __forceinline__ unsigned warp_run_add(unsigned *counter, int key, bool want_slot) {
  const int lane = threadIdx.x & 31;
  const int prev = __shfl_up_sync(FULL_MASK, key, 1);
  const unsigned heads = __ballot_sync(FULL_MASK, lane == 0 || key != prev);
  const unsigned after = heads & ~((2u << lane) - 1u);  // run heads above this lane (0 for lane 31)
  const int head = 31 - __clz(heads & ((2u << lane) - 1u));
  unsigned base = 0;
  if (head == lane && key >= 0) base = atomicAdd(counter + key, (unsigned)((after ? __ffs(after) - 1 : 32) - lane));
  if (!want_slot) return 0;
  base = __shfl_sync(FULL_MASK, base, head);
  return base + (unsigned)(lane - head);
}

// Tile id of the lane's (a, b, c)-th footprint tile, or -1 when the lane has none there.
__device__ __forceinline__ int tile_key(const TileGeo &tg, bool has, const AxisTiles &TX, const AxisTiles &TY,
                                        const AxisTiles &TZ, int a, int b, int c) {
  const int id = tile_id(tg, tile_at(TX, a), tile_at(TY, b), tile_at(TZ, c));
  return (has & (a < TX.n) & (b < TY.n) & (c < TZ.n)) ? id : -1;
}

// Pass 1: tile counts; statistics that need no exact decision (reads, velocity moments, the
// fixed-point bound); particles whose footprint misses the grid (outside the box, rejected).
// The particle loop is warp-uniform (lanes past n take part without a particle) so the tile counters
// can be aggregated over runs of lanes: particles that arrive in spatial order share their tiles.
template <typename T>
__global__ void __launch_bounds__(256) k_count(Geom g, FieldSpec fs, TileGeo tg, PIn<T> in, long long n,
                                               unsigned *counts, DevStats *st, int split_edge) {
  float f_read = 0, f_out = 0, f_nsq = 0, f_v[4] = {0, 0, 0, 0}, f_abs[2] = {0, 0}, f_grid = 0;
  int fatal = 0, nonfin = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i0 = blockIdx.x * (long long)blockDim.x + (threadIdx.x & ~31); i0 < n; i0 += stride) {
    const long long i = i0 + (threadIdx.x & 31);
    bool has = false;
    AxisTiles TX, TY, TZ;
    TX.n = TY.n = TZ.n = 0;
    if (i < n) {
      const Prep p = prep32(g, fs, in, i);
      if (!p.fin) {
        nonfin = 1;
      } else {
        f_read += 1.0f;
        if (fs.moments) {  // src/read_data.c:132-138, every particle read
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
        if (!footprint(g, tg, p.sx, p.sy, p.sz, TX, TY, TZ)) {
          f_out += 1.0f;  // clearly outside the box (src/read_data.c:81-88)
          if (g.los == 0) {
            fatal = 1;
            atomicMax(&st->fatal_inv, ~0ULL - (unsigned long long)i);
          }
        } else if (split_edge && is_edge(g, p.sx, p.sy, p.sz)) {
          // painted and counted by k_edge_fixup
        } else {
          has = true;
          // NGRID (src/read_data.c:92-126) and NOUT: exact for particles away from every edge
          if (split_edge && accept32(g, p.sx, p.sy, p.sz)) f_grid += p.w;
          if (split_edge && outside32(g, p.sx, p.sy, p.sz)) f_out += 1.0f;
        }
      }
    }
    const int na = __reduce_max_sync(FULL_MASK, has ? TX.n : 0), nb = __reduce_max_sync(FULL_MASK, has ? TY.n : 0),
              nc = __reduce_max_sync(FULL_MASK, has ? TZ.n : 0);
    // runtime loops over the warp's footprint tiles (warp-uniform bounds): one copy of the body
#pragma unroll 1
    for (int a = 0; a < na; a++)
#pragma unroll 1
      for (int b = 0; b < nb; b++)
#pragma unroll 1
        for (int c = 0; c < nc; c++) warp_run_add(counts, tile_key(tg, has, TX, TY, TZ, a, b, c), false);
  }
  // FP32 per-thread partials and warp sums, FP64 across warps
  const float vals[10] = {f_read, f_out, f_nsq, f_v[0], f_v[1], f_v[2], f_v[3], f_abs[0], f_abs[1], f_grid};
  double *const dst[10] = {&st->nread, &st->nout, &st->nsq, &st->vr[0], &st->vr[1], &st->vr[2], &st->vr[3],
                           &st->absw[0], &st->absw[1], &st->ngrid};
  block_add_f<10>(vals, dst);
  if (fatal) atomicOr(&st->fatal, 1);
  if (nonfin) atomicOr(&st->nonfinite, 1);
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

// Pass 3: scatter particles into their tiles' lists. A record holds the normal-stencil scales and
// the velocity, or, for a particle taking the exact rules, a mark and the particle index. Same
// warp-uniform loop and run aggregation of the tile cursors as k_count.
template <typename T>
__global__ void __launch_bounds__(256) k_scatter(Geom g, FieldSpec fs, TileGeo tg, PIn<T> in, long long n,
                                                 unsigned *cursor, float4 *recs, float *recw,
                                                 unsigned long long capacity, unsigned *edge_list,
                                                 unsigned *edge_count) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i0 = blockIdx.x * (long long)blockDim.x + (threadIdx.x & ~31); i0 < n; i0 += stride) {
    const long long i = i0 + (threadIdx.x & 31);
    bool has = false;
    AxisTiles TX, TY, TZ;
    TX.n = TY.n = TZ.n = 0;
    float4 rec = make_float4(0.f, 0.f, 0.f, 0.f);
    float w = 1.0f;
    if (i < n) {
      const Prep p = prep32(g, fs, in, i);
      if (p.fin && footprint(g, tg, p.sx, p.sy, p.sz, TX, TY, TZ)) {
        const bool edge = is_edge(g, p.sx, p.sy, p.sz);
        if (edge && edge_list) {  // painted by k_edge_fixup after the tiles
          edge_list[atomicAdd(edge_count, 1u)] = (unsigned)i;
        } else {
          has = true;
          w = p.w;
          rec = edge ? make_float4(SPECIAL_MARK, __uint_as_float((unsigned)i), 0.0f, 0.0f)
                     : make_float4(p.sx, p.sy, p.sz, p.v);
        }
      }
    }
    const int na = __reduce_max_sync(FULL_MASK, has ? TX.n : 0), nb = __reduce_max_sync(FULL_MASK, has ? TY.n : 0),
              nc = __reduce_max_sync(FULL_MASK, has ? TZ.n : 0);
    // runtime loops over the warp's footprint tiles (warp-uniform bounds): one copy of the body
#pragma unroll 1
    for (int a = 0; a < na; a++)
#pragma unroll 1
      for (int b = 0; b < nb; b++)
#pragma unroll 1
        for (int c = 0; c < nc; c++) {
          const int key = tile_key(tg, has, TX, TY, TZ, a, b, c);
          const unsigned slot = warp_run_add(cursor, key, true);
          if (key >= 0 && slot < capacity) {
            recs[slot] = rec;
            if (recw) recw[slot] = w;
          }
        }
  }
}

// Bucket mode, passes 1-3 in one: the statistics of k_count and the records of k_scatter, each
// written into its tile's fixed-capacity bucket (slot from the run-aggregated tile counter); a
// record that finds its bucket full goes to the overflow list with its tile. (Four CTAs per SM:
// 64 registers, which the overlapped reservations below need without spilling.)
template <typename T>
__global__ void __launch_bounds__(256, 4) k_bucket(Geom g, FieldSpec fs, TileGeo tg, PIn<T> in, long long n,
                                                   long long ibase, unsigned *counts, float4 *recs, float *recw, unsigned cap,
                                                unsigned *edge_list, unsigned *edge_count, float4 *ovf_recs,
                                                float *ovf_w, unsigned *ovf_tile, unsigned *ovf_count,
                                                unsigned long long ovf_cap, DevStats *st) {
  float f_read = 0, f_out = 0, f_nsq = 0, f_v[4] = {0, 0, 0, 0}, f_abs[2] = {0, 0}, f_grid = 0;
  int fatal = 0, nonfin = 0, ovf_full = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i0 = blockIdx.x * (long long)blockDim.x + (threadIdx.x & ~31); i0 < n; i0 += stride) {
    const long long i = i0 + (threadIdx.x & 31);
    bool has = false;
    AxisTiles TX, TY, TZ;
    TX.n = TY.n = TZ.n = 0;
    float4 rec = make_float4(0.f, 0.f, 0.f, 0.f);
    float w = 1.0f;
    if (i < n) {
      const Prep p = prep32(g, fs, in, i);
      if (!p.fin) {
        nonfin = 1;
      } else {
        f_read += 1.0f;
        if (fs.moments) {  // src/read_data.c:132-138, every particle read
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
        if (!footprint(g, tg, p.sx, p.sy, p.sz, TX, TY, TZ)) {
          f_out += 1.0f;  // clearly outside the box (src/read_data.c:81-88)
          if (g.los == 0) {
            fatal = 1;
            atomicMax(&st->fatal_inv, ~0ULL - (unsigned long long)(ibase + i));
          }
        } else if (is_edge(g, p.sx, p.sy, p.sz)) {
          edge_list[atomicAdd(edge_count, 1u)] = (unsigned)(ibase + i);  // painted and counted by k_edge_fixup
        } else {
          has = true;
          w = p.w;
          rec = make_float4(p.sx, p.sy, p.sz, p.v);
          if (accept32(g, p.sx, p.sy, p.sz)) f_grid += p.w;  // NGRID (src/read_data.c:92-126)
          if (outside32(g, p.sx, p.sy, p.sz)) f_out += 1.0f;  // src/read_data.c:81-88
        }
      }
    }
    const int na = __reduce_max_sync(FULL_MASK, has ? TX.n : 0), nb = __reduce_max_sync(FULL_MASK, has ? TY.n : 0),
              nc = __reduce_max_sync(FULL_MASK, has ? TZ.n : 0);
    auto put = [&](int key, unsigned slot) {
      if (key < 0) return;
      if (slot < cap) {
        const unsigned long long r = (unsigned long long)key * cap + slot;
        recs[r] = rec;
        if (recw) recw[r] = w;
      } else {
        const unsigned o = atomicAdd(ovf_count, 1u);
        if (o < ovf_cap) {
          ovf_recs[o] = rec;
          if (ovf_w) ovf_w[o] = w;
          ovf_tile[o] = (unsigned)key;
        } else {
          ovf_full = 1;
        }
      }
    };
    if (na <= 2 && nb <= 2 && nc <= 2) {
      // every (a, b, c) reservation of the warp first (their atomics in flight together), then the
      // records: lane slot = the run head's returned base + the lane's place in its run
      const int lane = threadIdx.x & 31;
      int keys[8], hd[8];
      unsigned base[8];
#pragma unroll
      for (int t = 0; t < 8; t++) {
        const int a = t >> 2, b = (t >> 1) & 1, c = t & 1;
        keys[t] = -1;
        hd[t] = 0;
        base[t] = 0;
        if (a < na && b < nb && c < nc) {  // warp-uniform
          const int key = tile_key(tg, has, TX, TY, TZ, a, b, c);
          const int prev = __shfl_up_sync(FULL_MASK, key, 1);
          const unsigned heads = __ballot_sync(FULL_MASK, lane == 0 || key != prev);
          const unsigned after = heads & ~((2u << lane) - 1u);
          const int head = 31 - __clz(heads & ((2u << lane) - 1u));
          if (head == lane && key >= 0) base[t] = atomicAdd(counts + key, (unsigned)((after ? __ffs(after) - 1 : 32) - lane));
          keys[t] = key;
          hd[t] = head;
        }
      }
#pragma unroll
      for (int t = 0; t < 8; t++) {
        const int a = t >> 2, b = (t >> 1) & 1, c = t & 1;
        if (a < na && b < nb && c < nc) {
          const unsigned b0 = __shfl_sync(FULL_MASK, base[t], hd[t]);
          put(keys[t], b0 + (unsigned)(lane - hd[t]));
        }
      }
    } else {
      // runtime loops over the warp's footprint tiles (warp-uniform bounds): one copy of the body
#pragma unroll 1
      for (int a = 0; a < na; a++)
#pragma unroll 1
        for (int b = 0; b < nb; b++)
#pragma unroll 1
          for (int c = 0; c < nc; c++) {
            const int key = tile_key(tg, has, TX, TY, TZ, a, b, c);
            put(key, warp_run_add(counts, key, true));
          }
    }
  }
  const float vals[10] = {f_read, f_out, f_nsq, f_v[0], f_v[1], f_v[2], f_v[3], f_abs[0], f_abs[1], f_grid};
  double *const dst[10] = {&st->nread, &st->nout, &st->nsq, &st->vr[0], &st->vr[1], &st->vr[2], &st->vr[3],
                           &st->absw[0], &st->absw[1], &st->ngrid};
  block_add_f<10>(vals, dst);
  if (fatal) atomicOr(&st->fatal, 1);
  if (nonfin) atomicOr(&st->nonfinite, 1);
  if (ovf_full) atomicOr(&st->overflow, 1);
}

// Deterministic accumulation: round(value * 2^S) added as an integer (S from k_scan, per field).
__device__ __forceinline__ void acc_add64(unsigned long long *p, double v, double scale) {
  atomicAdd(p, (unsigned long long)__double2ll_rn(v * scale));
}

// One axis of a record's stencil: the taps' offsets in the shared tile
// (index within the tile times the axis pitch) and weights; a tap that the reference drops or that
// lies outside this tile gets weight 0.
__device__ __forceinline__ void stage_axis32(const AxisTapsF &t, int origin, int extent, int pitch, float *W,
                                             int *O) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int l = t.idx[k] - origin;
    const bool ok = t.idx[k] >= 0 && l >= 0 && l < extent;
    W[k] = ok ? t.w[k] : 0.0f;
    O[k] = ok ? l * pitch : 0;
  }
}

// Same for exact taps in the reference's index space. x: halo slices fold onto 0.. (LOS == 0) or are
// dropped; z: the padding column (a CIC rounding edge) is dropped; y == NY (a CIC rounding edge) is
// the aliased write handled by the caller.
__device__ __forceinline__ void stage_axis64(const Geom &g, const AxisTaps &t, int axis, int origin, int extent,
                                             int pitch, float *W, int *O) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    int idx = t.idx[k];
    bool ok = k < t.n && t.on[k];
    const int n = axis == 0 ? g.nx : (axis == 1 ? g.ny : g.nz);
    if (axis == 0 && idx >= n) {
      if (g.los == 0 && idx < n + g.order) idx -= n;
      else ok = false;
    }
    if (idx < 0 || idx >= n) ok = false;
    const int l = idx - origin;
    ok = ok && l >= 0 && l < extent;
    W[k] = ok ? (float)t.w[k] : 0.0f;
    O[k] = ok ? l * pitch : 0;
  }
}

// Compile-time-order FP32 taps of one axis (kind 0: x, 1: y or z).
// Power-of-two scale 2^S for a tile's int32 fixed-point cells. A record's taps add at most |w v^e|
// to one slot, so no cell of the slot exceeds the tile's sum of |w v^e| over its records; that sum
// (FP32, raised by 0.1 % for its own rounding) times 2^S <= 2^30 keeps every partial sum, with the
// half-unit rounding of each deposit (one per record and cell), inside int32.
__device__ __forceinline__ int tile_scale_exp(float sum_abs) {
  const float bound = sum_abs * 1.001f;
  if (!(bound > 0.0f) || !isfinite(bound)) return 0;
  const int e = ilogbf(bound);  // bound < 2^(e+1)
  const int S = 29 - e;
  return S > 100 ? 100 : (S < -100 ? -100 : S);
}

// Largest scale exponent that keeps every single deposit of a tile below 2^22 in magnitude
// (|w v^e| 2^S < 2^22, tap weights <= 1), where rint_small rounds exactly.
__device__ __forceinline__ int tile_scale_max(float max_abs) {
  const float mb = max_abs * 1.001f;
  return (mb > 0.0f && isfinite(mb)) ? 21 - ilogbf(mb) : 100;
}

// Round-to-nearest-even of a * b as an int32, for |a * b| < 2^22: the fused multiply-add rounds the
// exact product plus 1.5 * 2^23 to an integer, whose FP32 bit pattern is 0x4B400000 + that integer.
// (Two FP32/integer-pipe instructions instead of a conversion.)
__device__ __forceinline__ int rint_small(float a, float b) {
  return __float_as_int(__fmaf_rn(a, b, 12582912.0f)) - 0x4B400000;
}

// The int32 quantum of a tile is about 2^-30 of the tile's total |w v^e|, and a cell sums up to one
// rounded deposit per record: the cells' relative error grows with the record count. A tile with
// more records than this (a dense clump; uniform catalogues put about a thousand records in a
// tile) is accumulated in int64 with 2^61 headroom instead, one grid slot and one shared-memory
// chunk of cells per pass over its records (the records are re-read from L2 for each pass).
#define TILE_PRECISE_RECORDS 16384

template <int K, int NF, bool IL>
__device__ void tile_paint_precise(const Geom &g, const FieldSpec &fs, const TileGeo &tg, const float4 *recs,
                                   const float *recw, unsigned long long rb, unsigned long long re, float ta, float tb,
                                   int x0, int y0, int z0, int ex, int ey, int ez, int pyz, int tsz,
                                   long long *sm64, int chunk, GridPtrs grids, DevStats *st) {
  constexpr int NS = IL ? 2 : 1;
  const int S64a = 60 - ilogbf(fmaxf(ta * 1.001f, 1e-30f)), S64b = 60 - ilogbf(fmaxf(tb * 1.001f, 1e-30f));
  for (int slot = 0; slot < NS * NF; slot++) {
    const int sten = slot / NF, fld = slot % NF;
    const int S64 = fld == 0 ? S64a : S64b;
    const float sc = ldexpf(1.0f, S64 > 100 ? 100 : S64);
    float dsum = 0.0f;
    for (int c0 = 0; c0 < tsz; c0 += chunk) {
      const int c1 = min(tsz, c0 + chunk);
      for (int c = threadIdx.x; c < c1 - c0; c += blockDim.x) sm64[c] = 0;
      __syncthreads();
      for (unsigned long long r = rb + threadIdx.x; r < re; r += blockDim.x) {
        const float4 rec = recs[r];
        const float w = recw ? recw[r] : 1.0f;
        float v = w;
        const int e_n = fld == 0 ? fs.ea : fs.eb;
        for (int e = 0; e < e_n; e++) v *= rec.w;
        v *= sc;
        const float sx = sten ? __fadd_rn(rec.x, 0.5f) : rec.x, sy = sten ? __fadd_rn(rec.y, 0.5f) : rec.y,
                    sz = sten ? __fadd_rn(rec.z, 0.5f) : rec.z;
        if (!accept32(g, sx, sy, sz)) continue;
        AxisTapsF ax, ay, az;
        axis32k<K>(sx, 0, g.nx, g.los, ax);
        axis32k<K>(sy, 1, g.ny, g.los, ay);
        axis32k<K>(sz, 1, g.nz, g.los, az);
        float wx[3], wy[3], wz[3];
        int ox[3], oy[3], oz[3];
        stage_axis32(ax, x0, ex, pyz, wx, ox);
        stage_axis32(ay, y0, ey, tg.tz, wy, oy);
        stage_axis32(az, z0, ez, 1, wz, oz);
#pragma unroll
        for (int a = 0; a < K; a++)
#pragma unroll
          for (int b2 = 0; b2 < K; b2++) {
            const float wxy = wx[a] * wy[b2];
            const float pv = v * wxy;
            const int oxy = ox[a] + oy[b2];
#pragma unroll
            for (int c = 0; c < K; c++) {
              const int off = oxy + oz[c] - c0;
              if (wxy != 0.0f && wz[c] != 0.0f && off >= 0 && off < c1 - c0)
                atomicAdd((unsigned long long *)(sm64 + off), (unsigned long long)__float2ll_rn(pv * wz[c]));
            }
          }
      }
      __syncthreads();
      const double inv = ldexp(1.0, -(S64 > 100 ? 100 : S64));
      float *gp = (float *)grids.g[slot];
      for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        const int rz = c & (tg.tz - 1), ly = (c >> tg.lz) & (tg.ty - 1), lx = c >> (tg.lz + tg.ly);
        if (lx >= ex || ly >= ey || rz >= ez) continue;
        const float val = (float)((double)sm64[c - c0] * inv);
        gp[(long long)(x0 + lx) * g.slice + (long long)(y0 + ly) * g.row + z0 + rz] = val;
        dsum += val;
      }
      __syncthreads();
    }
    const double vals[1] = {(double)dsum};
    double *const dst1[1] = {&st->dc[slot]};
    block_add<1>(vals, dst1);
  }
}

// The deposits of a tile's records (lane = record; both stencils) into the int32 shared tile.
// FASTR: rounded by rint_small (every deposit below 2^22); otherwise by conversion.
template <int K, int NF, bool IL, bool FASTR>
__device__ __forceinline__ void tile_rec_deposit(const Geom &g, const FieldSpec &fs, const TileGeo &tg,
                                                 const float4 *recs, const float *recw, unsigned long long rb,
                                                 unsigned long long re, float scA, float scB, int x0, int y0,
                                                 int z0, int ex, int ey, int ez, int *smi) {
  constexpr int NS = IL ? 2 : 1;
  const int slotw = tg.slot;
  for (unsigned long long r = rb + threadIdx.x; r < re; r += blockDim.x) {
    const float4 rec = recs[r];
    const float w = recw ? recw[r] : 1.0f;
    float va = w, vb = w;
    for (int e = 0; e < fs.ea; e++) va *= rec.w;
    for (int e = 0; e < fs.eb; e++) vb *= rec.w;
    va *= scA;
    vb *= scB;
#pragma unroll
    for (int s = 0; s < NS; s++) {
      const float sx = s ? __fadd_rn(rec.x, 0.5f) : rec.x, sy = s ? __fadd_rn(rec.y, 0.5f) : rec.y,
                  sz = s ? __fadd_rn(rec.z, 0.5f) : rec.z;
      if (!accept32(g, sx, sy, sz)) continue;
      AxisTapsF ax, ay, az;
      axis32k<K>(sx, 0, g.nx, g.los, ax);
      axis32k<K>(sy, 1, g.ny, g.los, ay);
      axis32k<K>(sz, 1, g.nz, g.los, az);
      float wx[3], wy[3], wz[3];
      int ox[3], oy[3], oz[3];
      stage_axis32(ax, x0, ex, tg.px, wx, ox);
      stage_axis32(ay, y0, ey, tg.py, wy, oy);
      stage_axis32(az, z0, ez, 1, wz, oz);
      int *sA = smi + (s * NF) * slotw;
#pragma unroll
      for (int a = 0; a < K; a++)
#pragma unroll
        for (int b2 = 0; b2 < K; b2++) {
          const float wxy = wx[a] * wy[b2];
          const float pa = va * wxy, pb = vb * wxy;
          const int oxy = ox[a] + oy[b2];
          // one test per (x, y) tap pair: an x or y tap outside the tile has weight 0. A z tap outside
          // it (the z edge of a tile is 32 cells: rare) has weight 0 and offset 0 and adds 0 there.
          if (wxy != 0.0f) {
#pragma unroll
            for (int c = 0; c < K; c++) {
              atomicAdd(sA + oxy + oz[c], FASTR ? rint_small(pa, wz[c]) : __float2int_rn(pa * wz[c]));
              if (NF == 2)
                atomicAdd(sA + slotw + oxy + oz[c], FASTR ? rint_small(pb, wz[c]) : __float2int_rn(pb * wz[c]));
            }
          }
        }
    }
  }
}

// FP32 tile kernel for particles away from every edge of the reference's rules (those are painted
// by k_edge_fixup). One CTA per tile; shared memory holds the tile of every grid slot, both
// stencils, [tx][ty][tz] with the padded pitches py = 3, px = 9 (mod 32) so that deposits at equal z
// spread over the banks, as int32 fixed point with a per-tile power-of-two scale, so
// every deposit is one native integer shared-memory atomic (an ordinary tile's scale also keeps each
// deposit below 2^22, where rint_small rounds it). Lane = record: each thread reads one record, derives its taps
// once per stencil and adds the K^3 products, so a record is read once and nothing is staged. The
// cells are converted back to FP32 when the tile is written. (NGRID of these particles is counted
// by k_bucket or k_count.)
template <int K, int NF, bool IL>
__global__ void __launch_bounds__(256, 3) k_tile_rec(Geom g, FieldSpec fs, TileGeo tg, const unsigned *offsets,
                                                     const unsigned *counts, unsigned cap, const float4 *recs,
                                                     const float *recw, unsigned long long capacity, GridPtrs grids,
                                                     DevStats *st) {
  extern __shared__ __align__(16) int smi[];
  constexpr int NS = IL ? 2 : 1;
  const int tsz = tg.tx * tg.ty * tg.tz;
  const int pyz = tg.ty * tg.tz;
  const int tile = blockIdx.x;
  const int bz = tile % tg.nbz, by = (tile / tg.nbz) % tg.nby, bx = tile / (tg.nbz * tg.nby);
  const int x0 = bx * tg.tx, y0 = by * tg.ty, z0 = bz * tg.tz;
  const int ex = min(tg.tx, g.nx - x0), ey = min(tg.ty, g.ny - y0), ez = min(tg.tz, g.nz - z0);
  int4 *sm4 = reinterpret_cast<int4 *>(smi);
  const int slotw = tg.slot;  // words per padded slot
  for (int c = threadIdx.x; c < (NS * NF * slotw) >> 2; c += blockDim.x) sm4[c] = make_int4(0, 0, 0, 0);
  for (int c = ((NS * NF * slotw) & ~3) + threadIdx.x; c < NS * NF * slotw; c += blockDim.x) smi[c] = 0;
  __syncthreads();
  unsigned long long rb, re;
  if (cap) {  // bucket mode: the tile's own bucket
    rb = (unsigned long long)tile * cap;
    re = rb + min(counts[tile], cap);
  } else {
    rb = offsets[tile];
    re = offsets[tile + 1];
  }
  if (re > capacity) re = capacity;
  if (rb > re) rb = re;
  // pre-pass over the tile's records: sum |w v^e| per field (the records stay in L1 for the deposits)
  __shared__ float red_abs[4][32];
  {
    float la = 0.0f, lb = 0.0f, ma = 0.0f, mb = 0.0f;
    for (unsigned long long r = rb + threadIdx.x; r < re; r += blockDim.x) {
      const float4 rec = recs[r];
      const float w = recw ? recw[r] : 1.0f;
      float va = w, vb = w;
      for (int e = 0; e < fs.ea; e++) va *= rec.w;
      for (int e = 0; e < fs.eb; e++) vb *= rec.w;
      la += fabsf(va);
      lb += fabsf(vb);
      ma = fmaxf(ma, fabsf(va));
      mb = fmaxf(mb, fabsf(vb));
    }
    la = warp_sum_f(la);
    lb = warp_sum_f(lb);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ma = fmaxf(ma, __shfl_xor_sync(0xffffffffu, ma, o));
      mb = fmaxf(mb, __shfl_xor_sync(0xffffffffu, mb, o));
    }
    if ((threadIdx.x & 31) == 0) {
      red_abs[0][threadIdx.x >> 5] = la;
      red_abs[1][threadIdx.x >> 5] = lb;
      red_abs[2][threadIdx.x >> 5] = ma;
      red_abs[3][threadIdx.x >> 5] = mb;
    }
    __syncthreads();
  }
  float ta = 0.0f, tb = 0.0f, xa = 0.0f, xb = 0.0f;
  for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
    ta += red_abs[0][k];
    tb += red_abs[1][k];
    xa = fmaxf(xa, red_abs[2][k]);
    xb = fmaxf(xb, red_abs[3][k]);
  }
  // The tile's scale is set by its sum (tile_scale_exp). When keeping every deposit below 2^22 costs
  // it at most 2 bits (an ordinary tile: hundreds of comparable records), the tile takes that scale
  // and the fast rounding; otherwise (few records, or one dominant record) it keeps the sum's scale
  // and rounds by conversion.
  const int SAs = tile_scale_exp(ta), SBs = tile_scale_exp(tb);
  const int SAf = min(SAs, tile_scale_max(xa)), SBf = min(SBs, tile_scale_max(xb));
  const bool fast = (SAs - SAf <= 2) && (NF == 1 || SBs - SBf <= 2);
  const int SA = fast ? SAf : SAs, SB = fast ? SBf : SBs;
  if (re - rb > TILE_PRECISE_RECORDS) {  // a dense tile (uniform over the CTA)
    const int words = NS * NF * tsz;  // the int32 tile area, reused as int64 cells
    tile_paint_precise<K, NF, IL>(g, fs, tg, recs, recw, rb, re, ta, tb, x0, y0, z0, ex, ey, ez, pyz, tsz,
                                  reinterpret_cast<long long *>(smi), words / 2, grids, st);
    return;
  }
  const float scA = ldexpf(1.0f, SA), scB = ldexpf(1.0f, SB);
  if (fast) tile_rec_deposit<K, NF, IL, true>(g, fs, tg, recs, recw, rb, re, scA, scB, x0, y0, z0, ex, ey, ez, smi);
  else tile_rec_deposit<K, NF, IL, false>(g, fs, tg, recs, recw, rb, re, scA, scB, x0, y0, z0, ex, ey, ez, smi);
  __syncthreads();
  // write every slot: pairs of cells along z as float2 (8-byte aligned global rows). A thread keeps
  // one (y, z) pair of the tile's x-planes and walks x, all slots per step: the pair's address in
  // shared memory and in the grid only advance by px and the grid slice. The slots' DC sums go to
  // one block reduction at the end (FP32 per thread and warp, FP64 across warps).
  float dsums[NS * NF], invs[NS * NF];
#pragma unroll
  for (int slot = 0; slot < NS * NF; slot++) {
    dsums[slot] = 0.0f;
    invs[slot] = ldexpf(1.0f, -((slot % NF) == 0 ? SA : SB));
  }
  const int ppl = (tg.ty * tg.tz) >> 1;  // pairs per x-plane
  for (int w = threadIdx.x; w < ppl; w += blockDim.x) {
    const int c = w << 1;
    const int rz = c & (tg.tz - 1), ly = c >> tg.lz;
    if (ly >= ey || rz >= ez) continue;
    const bool two = rz + 1 < ez;
    const int cb = ly * tg.py + rz;
    const long long gb = (long long)x0 * g.slice + (long long)(y0 + ly) * g.row + z0 + rz;
    for (int lx = 0; lx < ex; lx++) {
      const int cp = cb + lx * tg.px;
      const long long go = gb + (long long)lx * g.slice;
#pragma unroll
      for (int slot = 0; slot < NS * NF; slot++) {
        const int *sl = smi + slot * slotw + cp;
        const float a0 = (float)sl[0] * invs[slot], a1 = (float)sl[1] * invs[slot];
        float *dst = (float *)grids.g[slot] + go;
        if (two) {
          dsums[slot] += a0 + a1;
          *reinterpret_cast<float2 *>(dst) = make_float2(a0, a1);
        } else {
          dsums[slot] += a0;
          dst[0] = a0;
        }
      }
    }
  }
  double *dsts[NS * NF];
#pragma unroll
  for (int slot = 0; slot < NS * NF; slot++) dsts[slot] = &st->dc[slot];
  block_add_f<NS * NF>(dsums, dsts);
}

// --------------------------------------------------------------------- deterministic tile paint
// Tiles with at most this many records accumulate in two-limb cells at a tile scale; denser ones in
// uint64 cells at the run's global scale (64-bit shared atomics: slower, and rare).
#define DET_FAST_RECORDS 8192u

// A deposit p (an FP32 value already in the tile's fixed point, |p| < 2^40) split as p = h 2^k + l with
// h = floor(p 2^-k) and l = p - h 2^k in [0, 2^k] (k <= 22), both made integers by the FMA rounding of
// rint_small and added with two native int32 shared atomics; the cell's value is hi 2^k + lo. The FMA
// that forms l is exact except for a negative p of magnitude below 2^k, where the deposit may come out
// one unit of the fixed point away from round(p): still a fixed function of p, whatever the order.
__device__ __forceinline__ void limb_add(int *lo, int *hi, float p, float two_mk, float two_k) {
  const float h = floorf(p * two_mk);
  const float l = __fmaf_rn(-h, two_k, p);
  atomicAdd(lo, rint_small(l, 1.0f));
  atomicAdd(hi, rint_small(h, 1.0f));
}

// Scale exponent of a tile: (record count) * (largest |w v^e| of its records) * 2^S < 2^40, so that no
// cell of one pass (each record adds at most |w v^e| 2^S to a cell) leaves the limbs' range. Both inputs
// are independent of the order of the records.
__device__ __forceinline__ int det_scale_exp(unsigned cnt, float max_abs) {
  const float bound = (float)cnt * max_abs * 1.001f;
  if (!(bound > 0.0f) || !isfinite(bound)) return 0;
  const int S = 39 - ilogbf(bound);
  return S > 100 ? 100 : (S < -100 ? -100 : S);
}

struct DetPass {
  int *lo, *hi;                  // two-limb cells of field 0 (field 1: + 2 slot); null in the uint64 mode
  unsigned long long *u;         // uint64 cells of field 0 (field 1: + slot)
  int slotw;
  float scA, scB, two_mk, two_k;  // fixed-point scales of the fields; 2^-k, 2^k
  double sc0, sc1;                // the same scales in FP64 (the CIC rounding-edge products)
};

template <int NF>
__device__ __forceinline__ void det_add(const DetPass &d, int off, float pa, float pb) {
  if (d.lo) {
    limb_add(d.lo + off, d.hi + off, pa, d.two_mk, d.two_k);
    if (NF == 2) limb_add(d.lo + 2 * d.slotw + off, d.hi + 2 * d.slotw + off, pb, d.two_mk, d.two_k);
  } else {
    atomicAdd(d.u + off, (unsigned long long)__float2ll_rn(pa));
    if (NF == 2) atomicAdd(d.u + d.slotw + off, (unsigned long long)__float2ll_rn(pb));
  }
}

// |w v^e| of one record for the tile's scale: the FP32 value, or for a special record its exact one.
template <typename T>
__device__ __forceinline__ void det_record_value(const Geom &g, const FieldSpec &fs, const PIn<T> &in, long long n,
                                                 const float4 &rec, float w, float &va, float &vb) {
  if (rec.x == SPECIAL_MARK) {
    const unsigned idx = __float_as_uint(rec.y);
    va = vb = 0.0f;
    if ((long long)idx >= n) return;
    double x, y, z, v, wd;
    exact_pos(g, fs, in, idx, x, y, z, v, wd);
    va = (float)wpow64(wd, v, fs.ea);
    vb = (float)wpow64(wd, v, fs.eb);
    return;
  }
  va = w;
  vb = w;
  for (int e = 0; e < fs.ea; e++) va *= rec.w;
  for (int e = 0; e < fs.eb; e++) vb *= rec.w;
}

// The exact FP64 rules of one special record (a particle within a few ulps of a discontinuity of the
// reference's rules, listed by its index) for stencil stn: its taps inside this tile. With stats its
// home tile also counts it in NGRID, in the out-of-box count and for the LOS == 0 error.
template <typename T, int NF>
__device__ void det_special(const Geom &g, const FieldSpec &fs, const TileGeo &tg, const PIn<T> &in, long long n,
                            unsigned idx, int tile, int x0, int y0, int z0, int ex, int ey, int ez, int stn,
                            bool stats, const DetPass &d, double &d_grid, double &d_out, int &fatal, DevStats *st) {
  if ((long long)idx >= n) return;
  double x, y, z, v, wd;
  exact_pos(g, fs, in, idx, x, y, z, v, wd);
  if (stats) {
    const Prep p = prep32(g, fs, in, idx);
    if (home_of(g, tg, p.sx, p.sy, p.sz) == tile) {
      if (outside_box(g, x, y, z)) {  // src/read_data.c:81-88
        d_out += 1.0;
        if (g.los == 0) {
          fatal = 1;
          atomicMax(&st->fatal_inv, ~0ULL - (unsigned long long)idx);
        }
      }
      AxisTaps ax, ay, az;
      if (exact_axes(g, x, y, z, ax, ay, az)) d_grid += wd;
    }
  }
  const double va64 = wpow64(wd, v, fs.ea), vb64 = wpow64(wd, v, fs.eb);
  const float va = (float)va64 * d.scA, vb = (float)vb64 * d.scB;
  AxisTaps ax, ay, az;
  const double px = stn ? DADD(x, g.hx) : x, py = stn ? DADD(y, g.hy) : y, pz = stn ? DADD(z, g.hz) : z;
  if (!exact_axes(g, px, py, pz, ax, ay, az)) return;
  float W[9];
  int O[9];
  stage_axis64(g, ax, 0, x0, ex, tg.px, W, O);
  stage_axis64(g, ay, 1, y0, ey, tg.py, W + 3, O + 3);
  stage_axis64(g, az, 2, z0, ez, 1, W + 6, O + 6);
  // CIC rounding edge: y index NY lands in row 0 of the next x slice (src/read_data.c:592-593)
  if (g.order == 2 && ay.n > 0 && ay.idx[0] == g.ny && ay.on[0]) {
    for (int a = 0; a < ax.n; a++)
      for (int c = 0; c < az.n; c++) {
        if (!(ax.on[a] && az.on[c])) continue;
        const long long L = canon_index(g, ax.idx[a], ay.idx[0], az.idx[c]);
        if (L < 0) continue;
        int ix, iy, iz;
        decode(g, L, ix, iy, iz);
        ix -= x0;
        iy -= y0;
        iz -= z0;
        if (ix < 0 || ix >= ex || iy < 0 || iy >= ey || iz < 0 || iz >= ez) continue;
        const double tw = DMUL(DMUL(ax.w[a], ay.w[0]), az.w[c]);
        det_add<NF>(d, ix * tg.px + iy * tg.py + iz, (float)(DMUL(va64, tw) * d.sc0), (float)(DMUL(vb64, tw) * d.sc1));
      }
  }
  for (int a = 0; a < 3; a++)
    for (int b2 = 0; b2 < 3; b2++)
      for (int c = 0; c < 3; c++) {
        const float wt = W[a] * W[3 + b2] * W[6 + c];
        if (wt != 0.0f) det_add<NF>(d, O[a] + O[3 + b2] + O[6 + c], va * wt, vb * wt);
      }
}

// Deterministic tile kernel (k_count -> k_scan -> k_scatter -> here): one CTA per tile and, as in k_tile_rec,
// lane = record; the two stencils one after the other (one pass each over the tile's records), each pass
// holding both fields of its stencil in shared memory as int64 fixed point. The cells of a tile with at most
// DET_FAST_RECORDS records are two int32 limbs at the tile's own scale (det_scale_exp: from the record count
// and the largest |w v^e|, both independent of the order of the records); denser tiles use uint64 cells at
// the run's global scale (k_scan: the catalogue's sum of |w v^e| times 2^S below 2^62). A deposit is the FP32
// product at that scale rounded once to an integer, and integer addition makes every cell, and so the grids,
// independent of the order of the deposits: bit-reproducible. Special records take the exact FP64 rules
// here (det_special). The home tile of each record counts it in NGRID and the out-of-box count (k_count only
// counted the tiles); the slots' DC sums go to the exact global integer sums at the global scale.
template <typename T, int K, int NF, bool IL>
__global__ void __launch_bounds__(256, 3) k_tile_rec_det(Geom g, FieldSpec fs, TileGeo tg, PIn<T> in, long long n,
                                                         const unsigned *offsets, const float4 *recs,
                                                         const float *recw, unsigned long long capacity,
                                                         GridPtrs grids, const double *fixed_scale, DevStats *st) {
  extern __shared__ __align__(16) int smd[];
  constexpr int NS = IL ? 2 : 1;
  const int tile = blockIdx.x;
  const int bz = tile % tg.nbz, by = (tile / tg.nbz) % tg.nby, bx = tile / (tg.nbz * tg.nby);
  const int x0 = bx * tg.tx, y0 = by * tg.ty, z0 = bz * tg.tz;
  const int ex = min(tg.tx, g.nx - x0), ey = min(tg.ty, g.ny - y0), ez = min(tg.tz, g.nz - z0);
  const int slotw = tg.slot;
  unsigned long long rb = offsets[tile], re = offsets[tile + 1];
  if (re > capacity) re = capacity;
  if (rb > re) rb = re;
  const unsigned cnt = (unsigned)(re - rb);
  const bool fast = cnt <= DET_FAST_RECORDS;
  __shared__ float red_max[2][32];
  float ma = 0.0f, mb = 0.0f;
  if (fast) {  // the tile's largest |w v^e| per field
    for (unsigned long long r = rb + threadIdx.x; r < re; r += blockDim.x) {
      float va, vb;
      det_record_value(g, fs, in, n, recs[r], recw ? recw[r] : 1.0f, va, vb);
      ma = fmaxf(ma, fabsf(va));
      mb = fmaxf(mb, fabsf(vb));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ma = fmaxf(ma, __shfl_xor_sync(FULL_MASK, ma, o));
      mb = fmaxf(mb, __shfl_xor_sync(FULL_MASK, mb, o));
    }
    if ((threadIdx.x & 31) == 0) {
      red_max[0][threadIdx.x >> 5] = ma;
      red_max[1][threadIdx.x >> 5] = mb;
    }
    __syncthreads();
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
      ma = fmaxf(ma, red_max[0][k]);
      mb = fmaxf(mb, red_max[1][k]);
    }
  }
  const double G0 = fixed_scale[0], G1 = fixed_scale[1];
  const int SA = det_scale_exp(cnt, ma), SB = det_scale_exp(cnt, mb);
  const int kb = 31 - (32 - __clz(cnt));  // k with cnt 2^k < 2^31
  const int k = kb > 22 ? 22 : kb;
  DetPass d;
  d.slotw = slotw;
  if (fast) {
    d.lo = smd;
    d.hi = smd + slotw;
    d.u = nullptr;
    d.scA = ldexpf(1.0f, SA);
    d.scB = ldexpf(1.0f, SB);
    d.two_mk = ldexpf(1.0f, -k);
    d.two_k = ldexpf(1.0f, k);
  } else {
    d.lo = d.hi = nullptr;
    d.u = reinterpret_cast<unsigned long long *>(smd);
    d.scA = (float)G0;
    d.scB = (float)G1;
    d.two_mk = d.two_k = 1.0f;
  }
  d.sc0 = (double)d.scA;
  d.sc1 = (double)d.scB;
  float f_grid = 0.0f, f_out = 0.0f;
  double d_grid = 0.0, d_out = 0.0;
  int fatal = 0;
#pragma unroll 1
  for (int stn = 0; stn < NS; stn++) {
    for (int c = threadIdx.x; c < NF * 2 * slotw; c += blockDim.x) smd[c] = 0;
    __syncthreads();
    for (unsigned long long r = rb + threadIdx.x; r < re; r += blockDim.x) {
      const float4 rec = recs[r];
      if (rec.x == SPECIAL_MARK) {
        det_special<T, NF>(g, fs, tg, in, n, __float_as_uint(rec.y), tile, x0, y0, z0, ex, ey, ez, stn, stn == 0, d,
                           d_grid, d_out, fatal, st);
        continue;
      }
      const float w = recw ? recw[r] : 1.0f;
      if (stn == 0 && home_of(g, tg, rec.x, rec.y, rec.z) == tile) {
        if (accept32(g, rec.x, rec.y, rec.z)) f_grid += w;
        if (outside32(g, rec.x, rec.y, rec.z)) f_out += 1.0f;  // src/read_data.c:81-88
      }
      float va = w, vb = w;
      for (int e = 0; e < fs.ea; e++) va *= rec.w;
      for (int e = 0; e < fs.eb; e++) vb *= rec.w;
      va *= d.scA;
      vb *= d.scB;
      const float sx = stn ? __fadd_rn(rec.x, 0.5f) : rec.x, sy = stn ? __fadd_rn(rec.y, 0.5f) : rec.y,
                  sz = stn ? __fadd_rn(rec.z, 0.5f) : rec.z;
      if (!accept32(g, sx, sy, sz)) continue;
      AxisTapsF ax, ay, az;
      axis32k<K>(sx, 0, g.nx, g.los, ax);
      axis32k<K>(sy, 1, g.ny, g.los, ay);
      axis32k<K>(sz, 1, g.nz, g.los, az);
      float wx[3], wy[3], wz[3];
      int ox[3], oy[3], oz[3];
      stage_axis32(ax, x0, ex, tg.px, wx, ox);
      stage_axis32(ay, y0, ey, tg.py, wy, oy);
      stage_axis32(az, z0, ez, 1, wz, oz);
#pragma unroll
      for (int a = 0; a < K; a++)
#pragma unroll
        for (int b2 = 0; b2 < K; b2++) {
          const float wxy = wx[a] * wy[b2];
          if (wxy == 0.0f) continue;
          const float pa = va * wxy, pb = vb * wxy;
          const int oxy = ox[a] + oy[b2];
#pragma unroll
          for (int c = 0; c < K; c++)
            if (wz[c] != 0.0f) det_add<NF>(d, oxy + oz[c], pa * wz[c], pb * wz[c]);
        }
    }
    __syncthreads();
    // write this stencil's slots: pairs of cells along z as float2 (rows start 8-byte aligned in global
    // memory: the padded row length 2*(NZ/2+1) is even); the slots' integer DC sums at the global scale
    const int npair = (tg.tx * tg.ty * tg.tz) >> 1;
#pragma unroll
    for (int f = 0; f < NF; f++) {
      const int slot = stn * NF + f;
      float *gp = (float *)grids.g[slot];
      const double inv = fast ? ldexp(1.0, -(f ? SB : SA)) : 1.0 / (f ? G1 : G0);
      long long isum = 0;
      for (int q = threadIdx.x; q < npair; q += blockDim.x) {
        const int c = q << 1;
        const int rz = c & (tg.tz - 1), ly = (c >> tg.lz) & (tg.ty - 1), lx = c >> (tg.lz + tg.ly);
        if (lx >= ex || ly >= ey || rz >= ez) continue;
        const int sidx = lx * tg.px + ly * tg.py + rz;
        long long a0, a1;
        if (fast) {
          const int *lo = smd + 2 * f * slotw, *hi = lo + slotw;
          a0 = (long long)hi[sidx] * (1ll << k) + (long long)lo[sidx];
          a1 = (long long)hi[sidx + 1] * (1ll << k) + (long long)lo[sidx + 1];
        } else {
          const unsigned long long *u = reinterpret_cast<const unsigned long long *>(smd) + f * slotw;
          a0 = (long long)u[sidx];
          a1 = (long long)u[sidx + 1];
        }
        const bool two = rz + 1 < ez;
        isum += a0 + (two ? a1 : 0ll);
        float *dst = gp + (long long)(x0 + lx) * g.slice + (long long)(y0 + ly) * g.row + z0 + rz;
        if (two) *reinterpret_cast<float2 *>(dst) = make_float2((float)((double)a0 * inv), (float)((double)a1 * inv));
        else dst[0] = (float)((double)a0 * inv);
      }
      for (int o = 16; o > 0; o >>= 1) isum += __shfl_xor_sync(FULL_MASK, isum, o);
      if ((threadIdx.x & 31) == 0 && isum) {
        // to the global scale: exact (a power of two) where it is the finer one, else rounded once
        const long long gsum = fast ? __double2ll_rn((double)isum * ((f ? G1 : G0) * inv)) : isum;
        atomicAdd(&st->dc_fixed[slot], (unsigned long long)gsum);
      }
    }
    __syncthreads();
  }
  const double vals[2] = {d_grid + (double)f_grid, d_out + (double)f_out};
  double *const dst[2] = {&st->ngrid, &st->nout};
  block_add<2>(vals, dst);
  if (fatal) atomicOr(&st->fatal, 1);
}

// Bucket mode: records that found their tile's bucket full, deposited after the tiles were written
// (FP32 global atomics), each restricted to the taps inside its own tile, with their DC sums.
template <int K, int NF, bool IL>
__global__ void __launch_bounds__(128) k_ovf_paint(Geom g, FieldSpec fs, TileGeo tg, const float4 *ovf_recs,
                                                   const float *ovf_w, const unsigned *ovf_tile,
                                                   const unsigned *ovf_count, unsigned long long ovf_cap,
                                                   GridPtrs grids, DevStats *st) {
  constexpr int NS = IL ? 2 : 1;
  const unsigned long long no = min((unsigned long long)*ovf_count, ovf_cap);
  double l_dc[4] = {0, 0, 0, 0};
  for (unsigned long long o = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; o < no;
       o += (unsigned long long)gridDim.x * blockDim.x) {
    const float4 rec = ovf_recs[o];
    const float w = ovf_w ? ovf_w[o] : 1.0f;
    const int tile = (int)ovf_tile[o];
    const int bz = tile % tg.nbz, by = (tile / tg.nbz) % tg.nby, bx = tile / (tg.nbz * tg.nby);
    const int x0 = bx * tg.tx, y0 = by * tg.ty, z0 = bz * tg.tz;
    const int ex = min(tg.tx, g.nx - x0), ey = min(tg.ty, g.ny - y0), ez = min(tg.tz, g.nz - z0);
    float va = w, vb = w;
    for (int e = 0; e < fs.ea; e++) va *= rec.w;
    for (int e = 0; e < fs.eb; e++) vb *= rec.w;
#pragma unroll
    for (int s = 0; s < NS; s++) {
      const float sx = s ? __fadd_rn(rec.x, 0.5f) : rec.x, sy = s ? __fadd_rn(rec.y, 0.5f) : rec.y,
                  sz = s ? __fadd_rn(rec.z, 0.5f) : rec.z;
      if (!accept32(g, sx, sy, sz)) continue;
      AxisTapsF ax, ay, az;
      axis32k<K>(sx, 0, g.nx, g.los, ax);
      axis32k<K>(sy, 1, g.ny, g.los, ay);
      axis32k<K>(sz, 1, g.nz, g.los, az);
      float wx[3], wy[3], wz[3];
      int lx[3], ly[3], lz[3];
      stage_axis32(ax, x0, ex, 1, wx, lx);
      stage_axis32(ay, y0, ey, 1, wy, ly);
      stage_axis32(az, z0, ez, 1, wz, lz);
#pragma unroll
      for (int a = 0; a < K; a++)
#pragma unroll
        for (int b2 = 0; b2 < K; b2++) {
          const float wxy = wx[a] * wy[b2];
          const long long rowb = ((long long)(x0 + lx[a]) * g.ny + (y0 + ly[b2])) * g.row + z0;
#pragma unroll
          for (int c = 0; c < K; c++) {
            if (wxy == 0.0f || wz[c] == 0.0f) continue;
            const float da = (va * wxy) * wz[c];
            atomicAdd((float *)grids.g[s * NF] + rowb + lz[c], da);
            l_dc[s * NF] += (double)da;
            if (NF == 2) {
              const float db = (vb * wxy) * wz[c];
              atomicAdd((float *)grids.g[s * NF + 1] + rowb + lz[c], db);
              l_dc[s * NF + 1] += (double)db;
            }
          }
        }
    }
  }
  const double vals[4] = {l_dc[0], l_dc[1], l_dc[2], l_dc[3]};
  double *const dst[4] = {&st->dc[0], &st->dc[1], &st->dc[2], &st->dc[3]};
  block_add<4>(vals, dst);
}

// Particles near an edge of the reference's rules, painted after the tiles with the exact FP64
// rules and global atomics into the FP32 grids; their exact statistics (NGRID, the out-of-box
// count, the LOS == 0 error) are added here. One warp per particle: lanes 0-2 take the taps of the
// three axes, then lane t deposits tap t (each a serial chain of FP64 steps otherwise).
template <typename T>
__global__ void __launch_bounds__(128) k_edge_fixup(Geom g, FieldSpec fs, PIn<T> in, const unsigned *edge_list,
                                                    const unsigned *edge_count, GridPtrs grids, DevStats *st) {
  const unsigned ne = *edge_count;
  const int nf = fs.nfields, nst = g.interlace ? 2 : 1;
  const int lane = threadIdx.x & 31;
  const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarp = (gridDim.x * blockDim.x) >> 5;
  double d_grid = 0.0, d_out = 0.0, l_dc[4] = {0, 0, 0, 0};
  int fatal = 0;
  for (unsigned k = warp; k < ne; k += nwarp) {
    const unsigned idx = edge_list[k];
    double x, y, z, v, w;
    exact_pos(g, fs, in, idx, x, y, z, v, w);
    if (outside_box(g, x, y, z)) {  // src/read_data.c:81-88
      if (lane == 0) d_out += 1.0;
      if (g.los == 0) {
        fatal = 1;
        if (lane == 0) atomicMax(&st->fatal_inv, ~0ULL - (unsigned long long)idx);
        continue;
      }
    }
    const double val[2] = {wpow64(w, v, fs.ea), wpow64(w, v, fs.eb)};
    for (int stn = 0; stn < nst; stn++) {
      const double px = stn ? DADD(x, g.hx) : x, py = stn ? DADD(y, g.hy) : y, pz = stn ? DADD(z, g.hz) : z;
      AxisTaps t;
      t.n = 0;
      bool acc = true;
      if (lane < 3) acc = exact_axis(g, lane, lane == 0 ? px : (lane == 1 ? py : pz), t);
      if (__ballot_sync(FULL_MASK, !acc)) continue;  // rejected by some axis
      if (stn == 0 && lane == 0) d_grid += w;
      // this lane's tap (a, b, c) of a 3 x 3 x 3 block; the axes' taps from lanes 0, 1, 2
      const int ta = lane / 9, tb = (lane / 3) % 3, tc = lane % 3;
      const int nx_ = __shfl_sync(FULL_MASK, t.n, 0), ny_ = __shfl_sync(FULL_MASK, t.n, 1),
                nz_ = __shfl_sync(FULL_MASK, t.n, 2);
      int ix = 0, iy = 0, iz = 0, on = 1;
      double wx = 0.0, wy = 0.0, wz = 0.0;
#pragma unroll
      for (int q = 0; q < 3; q++) {
        const int i0 = __shfl_sync(FULL_MASK, t.idx[q], 0), i1 = __shfl_sync(FULL_MASK, t.idx[q], 1),
                  i2 = __shfl_sync(FULL_MASK, t.idx[q], 2);
        const int o0 = __shfl_sync(FULL_MASK, (int)t.on[q], 0), o1 = __shfl_sync(FULL_MASK, (int)t.on[q], 1),
                  o2 = __shfl_sync(FULL_MASK, (int)t.on[q], 2);
        const double w0 = __shfl_sync(FULL_MASK, t.w[q], 0), w1 = __shfl_sync(FULL_MASK, t.w[q], 1),
                     w2 = __shfl_sync(FULL_MASK, t.w[q], 2);
        if (ta == q) { ix = i0; wx = w0; on &= o0; }
        if (tb == q) { iy = i1; wy = w1; on &= o1; }
        if (tc == q) { iz = i2; wz = w2; on &= o2; }
      }
      if (lane >= 27 || ta >= nx_ || tb >= ny_ || tc >= nz_ || !on) continue;
      const long long L = canon_index(g, ix, iy, iz);
      if (L < 0) continue;
      const double tw = DMUL(DMUL(wx, wy), wz);
      for (int f = 0; f < nf; f++) {
        const float dep = (float)DMUL(val[f], tw);
        atomicAdd((float *)grids.g[stn * nf + f] + L, dep);
        l_dc[stn * nf + f] += (double)dep;
      }
    }
  }
  const double vals[6] = {d_grid, d_out, l_dc[0], l_dc[1], l_dc[2], l_dc[3]};
  double *const dst[6] = {&st->ngrid, &st->nout, &st->dc[0], &st->dc[1], &st->dc[2], &st->dc[3]};
  block_add<6>(vals, dst);
  if (fatal) atomicOr(&st->fatal, 1);
}

static int pow2_at_least(int n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

static int log2i(int p) {
  int l = 0;
  while ((1 << l) < p) l++;
  return l;
}

TileGeo choose_tiles(const Geom &g, int nslots, int deterministic) {
  // 4 grid slots x 8x16x32 floats = 64 KB (three CTAs per SM). The deterministic kernel holds one stencil's
  // fields at a time, as 8-byte cells: the same tiles for two fields (or one field interlaced), the
  // 16x16x32 ones for a single field otherwise.
  if (deterministic) return make_tiles(g, nslots == 1 ? 16 : 8, 16, 32);
  return make_tiles(g, nslots <= 2 ? 16 : 8, 16, 32);
}

// Tile edges are powers of two (tile coordinates are shifts); a grid edge shorter than the tile
// uses the next power of two and the tile is partial.
TileGeo make_tiles(const Geom &g, int tx, int ty, int tz) {
  TileGeo t;
  t.tx = tx;
  t.ty = ty;
  t.tz = tz;
  t.tz = t.tz < pow2_at_least(g.nz) ? t.tz : pow2_at_least(g.nz);
  t.ty = t.ty < pow2_at_least(g.ny) ? t.ty : pow2_at_least(g.ny);
  t.tx = t.tx < pow2_at_least(g.nx) ? t.tx : pow2_at_least(g.nx);
  t.lx = log2i(t.tx);
  t.ly = log2i(t.ty);
  t.lz = log2i(t.tz);
  t.nbx = (g.nx + t.tx - 1) / t.tx;
  t.nby = (g.ny + t.ty - 1) / t.ty;
  t.nbz = (g.nz + t.tz - 1) / t.tz;
  t.ntiles = t.nbx * t.nby * t.nbz;
  t.py = t.tz + 1;  // >= tz + 1 so a z pair never straddles rows; = 3 (mod 32)
  while (t.py % 32 != 3) t.py++;
  t.px = t.ty * t.py;
  while (t.px % 32 != 9) t.px++;
  t.slot = t.px * t.tx;
  return t;
}

size_t tile_smem_bytes(const TileGeo &tg, int nslots, int deterministic) {
  return ((size_t)nslots * tg.slot * (deterministic ? 8 : 4) + 15) & ~(size_t)15;
}

size_t rec_smem_bytes(const TileGeo &tg, int nslots) { return (size_t)nslots * tg.slot * 4; }

double tile_dup_estimate(const Geom &g, const TileGeo &tg) {
  // a footprint spans 4 (TSC, CIC) or 2 (NN) cells plus the margin; it crosses into the next tile
  // with probability (span - 1) / tile edge
  const double span = (g.order == 1 ? 2.0 : (g.order == 2 ? 3.0 : 4.0)) + 2.0 * g.margin;
  return (1.0 + (span - 1.0) / tg.tx) * (1.0 + (span - 1.0) / tg.ty) * (1.0 + (span - 1.0) / tg.tz);
}

template <int K, int NF, bool IL>
static void launch_rec(cudaStream_t s, const Geom &g, const FieldSpec &fs, const TileGeo &tg, const PaintBufs &b,
                       bool weights, const GridPtrs &grids, DevStats *st) {
  const size_t smem = rec_smem_bytes(tg, NF * (IL ? 2 : 1));
  cudaFuncSetAttribute(k_tile_rec<K, NF, IL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_tile_rec<K, NF, IL><<<tg.ntiles, 256, smem, s>>>(g, fs, tg, b.offsets, b.counts, b.bucket_cap, b.recs,
                                                     weights ? b.recw : nullptr, b.capacity, grids, st);
  if (b.bucket_cap)
    k_ovf_paint<K, NF, IL><<<152 * 2, 128, 0, s>>>(g, fs, tg, b.ovf_recs, weights ? b.ovf_w : nullptr, b.ovf_tile,
                                                   b.ovf_count, b.ovf_cap, grids, st);
}

template <int K>
static void launch_rec_k(cudaStream_t s, const Geom &g, const FieldSpec &fs, const TileGeo &tg, const PaintBufs &b,
                         bool weights, const GridPtrs &grids, DevStats *st) {
  if (fs.nfields == 2) {
    if (g.interlace) launch_rec<K, 2, true>(s, g, fs, tg, b, weights, grids, st);
    else launch_rec<K, 2, false>(s, g, fs, tg, b, weights, grids, st);
  } else {
    if (g.interlace) launch_rec<K, 1, true>(s, g, fs, tg, b, weights, grids, st);
    else launch_rec<K, 1, false>(s, g, fs, tg, b, weights, grids, st);
  }
}

template <typename T, int K, int NF, bool IL>
static void launch_det(cudaStream_t s, const Geom &g, const FieldSpec &fs, const TileGeo &tg, const PIn<T> &in,
                       long long n, const PaintBufs &b, const GridPtrs &grids, DevStats *st) {
  const size_t smem = tile_smem_bytes(tg, NF, 1);
  cudaFuncSetAttribute(k_tile_rec_det<T, K, NF, IL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_tile_rec_det<T, K, NF, IL><<<tg.ntiles, 256, smem, s>>>(g, fs, tg, in, n, b.offsets, b.recs,
                                                            in.w ? b.recw : nullptr, b.capacity, grids, b.fixed_scale,
                                                            st);
}

template <typename T, int K>
static void launch_det_k(cudaStream_t s, const Geom &g, const FieldSpec &fs, const TileGeo &tg, const PIn<T> &in,
                         long long n, const PaintBufs &b, const GridPtrs &grids, DevStats *st) {
  if (fs.nfields == 2) {
    if (g.interlace) launch_det<T, K, 2, true>(s, g, fs, tg, in, n, b, grids, st);
    else launch_det<T, K, 2, false>(s, g, fs, tg, in, n, b, grids, st);
  } else {
    if (g.interlace) launch_det<T, K, 1, true>(s, g, fs, tg, in, n, b, grids, st);
    else launch_det<T, K, 1, false>(s, g, fs, tg, in, n, b, grids, st);
  }
}

template <typename T>
static void run_paint32(cudaStream_t s, const Geom &g, const FieldSpec &fs, const TileGeo &tg, int det, PIn<T> in,
                        long long n, const GridPtrs &grids, const PaintBufs &b, DevStats *st, long long *launches) {
  const int th = 256;
  long long nbl = (n + th - 1) / th;
  const int nb = (int)(nbl < 1 ? 1 : (nbl > 152 * 8 ? 152 * 8 : nbl));  // one resident wave of 256-thread blocks
  const bool split = !det;  // FP32: edge particles go to k_edge_fixup; deterministic: exact rules in the tiles
  cudaMemsetAsync(b.counts, 0, sizeof(unsigned) * tg.ntiles, s);
  if (split) cudaMemsetAsync(b.edge_count, 0, sizeof(unsigned), s);
  if (!det && b.bucket_cap) {  // bucket mode: one pass to the tiles' buckets, overflow after the tiles
    cudaMemsetAsync(b.ovf_count, 0, sizeof(unsigned), s);
    const int nch = b.nchunk > 1 ? b.nchunk : 1;
    for (int k = 0; k < nch; k++) {  // one launch per copied chunk of a host catalogue (else one)
      const long long c0 = n * k / nch, c1 = n * (k + 1) / nch;
      if (nch > 1) cudaStreamWaitEvent(s, b.chunk_ev[k], 0);
      PIn<T> ink{in.x + c0, in.y + c0, in.z + c0, in.v ? in.v + c0 : nullptr, in.w ? in.w + c0 : nullptr};
      const long long nbk = (c1 - c0 + th - 1) / th;
      const int nbc = (int)(nbk < 1 ? 1 : (nbk > 152 * 8 ? 152 * 8 : nbk));
      k_bucket<T><<<nbc, th, 0, s>>>(g, fs, tg, ink, c1 - c0, c0, b.counts, b.recs, in.w ? b.recw : nullptr,
                                     b.bucket_cap, b.edge_list, b.edge_count, b.ovf_recs, in.w ? b.ovf_w : nullptr,
                                     b.ovf_tile, b.ovf_count, b.ovf_cap, st);
    }
    *launches += nch - 1;
    const bool wts = in.w != nullptr;
    if (b.tile_ev0) cudaEventRecord(b.tile_ev0, s);
    if (g.order == 3) launch_rec_k<3>(s, g, fs, tg, b, wts, grids, st);
    else if (g.order == 2) launch_rec_k<2>(s, g, fs, tg, b, wts, grids, st);
    else launch_rec_k<1>(s, g, fs, tg, b, wts, grids, st);
    if (b.tile_ev1) cudaEventRecord(b.tile_ev1, s);
    k_edge_fixup<T><<<152 * 2, 128, 0, s>>>(g, fs, in, b.edge_list, b.edge_count, grids, st);
    *launches += 4;
    return;
  }
  k_count<T><<<nb, th, 0, s>>>(g, fs, tg, in, n, b.counts, st, split ? 1 : 0);
  k_scan<<<1, 1024, 0, s>>>(b.counts, tg.ntiles, b.offsets, b.cursor, st, b.capacity, b.fixed_scale);
  k_scatter<T><<<nb, th, 0, s>>>(g, fs, tg, in, n, b.cursor, b.recs, in.w ? b.recw : nullptr, b.capacity,
                                 split ? b.edge_list : nullptr, b.edge_count);
  if (det) {
    if (b.tile_ev0) cudaEventRecord(b.tile_ev0, s);
    if (g.order == 3) launch_det_k<T, 3>(s, g, fs, tg, in, n, b, grids, st);
    else if (g.order == 2) launch_det_k<T, 2>(s, g, fs, tg, in, n, b, grids, st);
    else launch_det_k<T, 1>(s, g, fs, tg, in, n, b, grids, st);
    if (b.tile_ev1) cudaEventRecord(b.tile_ev1, s);
    *launches += 4;
  } else {
    const bool wts = in.w != nullptr;
    if (b.tile_ev0) cudaEventRecord(b.tile_ev0, s);
    if (g.order == 3) launch_rec_k<3>(s, g, fs, tg, b, wts, grids, st);
    else if (g.order == 2) launch_rec_k<2>(s, g, fs, tg, b, wts, grids, st);
    else launch_rec_k<1>(s, g, fs, tg, b, wts, grids, st);
    if (b.tile_ev1) cudaEventRecord(b.tile_ev1, s);
    k_edge_fixup<T><<<152 * 2, 128, 0, s>>>(g, fs, in, b.edge_list, b.edge_count, grids, st);
    *launches += 5;
  }
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
