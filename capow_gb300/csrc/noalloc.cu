// capow_paint_noalloc: the FP32 tile paint of capow_paint with every piece of per-call device
// scratch (tile counts, offsets and cursors, the tile record lists, the edge list) taken from one
// fixed file-scope device array instead of buffers that grow with the catalogue.
//
// Who needs it: capow_paint grows its record, edge and staging buffers on demand, so a larger
// catalogue makes it call cudaMalloc, and cudaFree on the old buffers, which waits for all work on
// the device. A caller that paints between the steps of a running simulation on the same GPU, and
// whose own memory pool holds the rest of the device, can afford neither: the allocation fails
// once the pool has taken the memory, and the implicit device-wide wait stalls the simulation's
// streams. This entry point touches only the context (created beforehand, when allocation is
// still possible) and the fixed array below.
//
// Limits: device-resident particles only (host input would need staging buffers), the two FP32
// precisions only (the FP64 path needs no tile scratch), and at most as many particles as fit the
// array under the worst-case number of tile records per particle; larger catalogues are rejected
// with CAPOW_EINVAL and a message that names the largest count that fits this grid.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "ctx.cuh"

// The scratch array: CAPOW_NOALLOC_SCRATCH_BYTES per device. Everything in it that must start at
// zero (the tile counts and the edge counter) is cleared by the paint itself at the start of every
// call, so nothing carries over from one call to the next.
static __device__ __align__(256) unsigned char g_noalloc_scratch[CAPOW_NOALLOC_SCRATCH_BYTES];

#define NOALLOC_MAX_DEVICES 64
static std::mutex g_noalloc_mu;
static void *g_noalloc_addr[NOALLOC_MAX_DEVICES];

// Set-up, once per device, with that device current: the array's device address. The first call
// also loads this module on the device, which is why the first capow_paint_noalloc on each device
// should come before any stream capture begins.
static int noalloc_scratch(capow_ctx *c, void **out) {
  const int dev = c->o.device;
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) FAIL(c, CAPOW_EINVAL, "device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      FAIL(c, CAPOW_ECUDA, "cudaGetSymbolAddress of the paint scratch failed: %s", cudaGetErrorString(e));
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return CAPOW_OK;
}

// Most distinct tiles the footprint of one particle can touch along one axis, as the count and
// scatter passes build it: `cells` consecutive cells starting anywhere, taken modulo n on a
// periodic axis and clipped to the grid otherwise; the passes keep at most three per axis.
static int axis_max_tiles(int n, int shift, int cells, bool wrap) {
  int best = 1;
  for (int lo = wrap ? 0 : -cells; lo < n && best < 3; lo++) {
    int t[3], nt = 0;
    for (int j = 0; j < cells; j++) {
      int cc = lo + j;
      if (wrap) {
        while (cc >= n) cc -= n;
      } else if (cc < 0 || cc >= n) {
        continue;
      }
      const int tile = cc >> shift;
      bool seen = false;
      for (int k = 0; k < nt; k++) seen = seen || t[k] == tile;
      if (!seen && nt < 3) t[nt++] = tile;
    }
    best = nt > best ? nt : best;
  }
  return best;
}

// Upper bound on the tile records of one particle (the count pass never exceeds it, so the record
// lists cannot overflow): the footprint spans at most order + 1 + ceil(2 * margin) cells per axis
// (one more is allowed for); the CIC row-aliasing rule adds the first y tile.
static unsigned long long records_per_particle(const Geom &g, const TileGeo &tg) {
  const int cells = g.order + 2 + (int)ceil(2.0 * (double)g.margin);
  const bool wrap = g.los == 0;
  const int dx = axis_max_tiles(g.nx, tg.lx, cells, wrap);
  int dy = axis_max_tiles(g.ny, tg.ly, cells, wrap);
  const int dz = axis_max_tiles(g.nz, tg.lz, cells, wrap);
  if (g.order == 2 && dy < 3) dy++;
  return (unsigned long long)dx * dy * dz;
}

static unsigned long long up256(unsigned long long b) { return (b + 255ULL) & ~255ULL; }

// Scratch layout of one call; returns the bytes it needs.
struct NoallocLayout {
  unsigned long long counts, offsets, cursor, edge_count, edge_list, recs, recw, total;
};

static NoallocLayout noalloc_layout(const TileGeo &tg, unsigned long long n, unsigned long long cap, bool edges,
                                    bool weights) {
  NoallocLayout L;
  unsigned long long o = 0;
  L.counts = o; o += up256(4ULL * tg.ntiles);
  L.offsets = o; o += up256(4ULL * (tg.ntiles + 1));
  L.cursor = o; o += up256(4ULL * tg.ntiles);
  L.edge_count = o; o += 256;
  L.edge_list = o; o += edges ? up256(4ULL * (n + 1)) : 0;
  L.recs = o; o += up256(16ULL * (cap ? cap : 1));
  L.recw = o; o += weights ? up256(4ULL * (cap ? cap : 1)) : 0;
  L.total = o;
  return L;
}

extern "C" int capow_paint_noalloc(capow_ctx *c, const capow_particles *parts) {
  if (!c || !parts) return CAPOW_EINVAL;
  if (!c->plan_ok) FAIL(c, CAPOW_ESTATE, "context not fully created");
  if (c->pending) FAIL(c, CAPOW_ESTATE, "capow_power_result of the power stage in flight first");
  if (c->prec == CAPOW_FP64) FAIL(c, CAPOW_ENOTSUP, "capow_paint_noalloc covers the FP32 precisions only");
  if (parts->dtype != CAPOW_F32 && parts->dtype != CAPOW_F64) FAIL(c, CAPOW_EINVAL, "dtype must be F32 or F64");
  if (!parts->on_device) FAIL(c, CAPOW_EINVAL, "capow_paint_noalloc takes device-resident particles only");
  if (!parts->x || !parts->y || !parts->z) FAIL(c, CAPOW_EINVAL, "x, y and z are required");
  if (c->fs.need_v && !parts->vlos) FAIL(c, CAPOW_EINVAL, "vlos is required for LOS != 0 or momentum fields");
  // every input must be device memory of this context's device (another device's memory would be
  // read through peer access or fault, with no clear error)
  {
    const void *arrs[5] = {parts->x, parts->y, parts->z, c->fs.need_v ? parts->vlos : nullptr, parts->w};
    for (int k = 0; k < 5; k++) {
      if (!arrs[k]) continue;
      cudaPointerAttributes a;
      if (cudaPointerGetAttributes(&a, arrs[k]) != cudaSuccess) {
        (void)cudaGetLastError();
        FAIL(c, CAPOW_EINVAL, "capow_paint_noalloc: input array %d is not device memory", k);
      }
      if (a.type != cudaMemoryTypeDevice || a.device != c->o.device)
        FAIL(c, CAPOW_EINVAL, "capow_paint_noalloc: input array %d is not device memory of device %d", k, c->o.device);
    }
  }
  const bool det = c->prec == CAPOW_FP32_DETERMINISTIC, weights = parts->w != nullptr;
  const unsigned long long n = parts->n, per = records_per_particle(c->g, c->tg);
  const unsigned long long limit = CAPOW_NOALLOC_SCRATCH_BYTES;
  // size check before anything touches the device: the record count n * per must fit
  const NoallocLayout fixed = noalloc_layout(c->tg, 0, 0, !det, weights);
  const unsigned long long per_bytes = per * (16ULL + (weights ? 4ULL : 0ULL)) + (det ? 0ULL : 4ULL);
  const unsigned long long fit = fixed.total + 1024 < limit ? (limit - fixed.total - 1024) / per_bytes : 0;
  if (n > fit || n * per >= 0xFFFFFFF0ULL)
    FAIL(c, CAPOW_EINVAL,
         "capow_paint_noalloc: %llu particles exceed the fixed %llu-byte scratch (up to %llu tile records per "
         "particle on this grid); at most %llu particles fit",
         n, limit, per, fit);
  const NoallocLayout L = noalloc_layout(c->tg, n, n * per, !det, weights);
  if (L.total > limit) FAIL(c, CAPOW_EINVAL, "capow_paint_noalloc: scratch layout exceeds the fixed array");
  CK(c, cudaSetDevice(c->o.device));
  void *base = nullptr;
  int rc = noalloc_scratch(c, &base);
  if (rc) return rc;
  char *b8 = (char *)base;
  PaintBufs b;
  memset(&b, 0, sizeof b);
  b.counts = (unsigned *)(b8 + L.counts);
  b.offsets = (unsigned *)(b8 + L.offsets);
  b.cursor = (unsigned *)(b8 + L.cursor);
  b.edge_count = (unsigned *)(b8 + L.edge_count);
  b.edge_list = det ? nullptr : (unsigned *)(b8 + L.edge_list);
  b.edge_cap = det ? 0 : n + 1;
  b.recs = (float4 *)(b8 + L.recs);
  b.recw = weights ? (float *)(b8 + L.recw) : nullptr;
  b.capacity = n * per;
  b.fixed_scale = c->fixed_scale;  // the context's: the DC correction of capow_power reads it
  capow_particles d = *parts;
  if (!c->fs.need_v) d.vlos = nullptr;
  c->last = d;
  c->painted = true;
  c->powered = false;
  // per-paint state of capow_paint that this paint does not produce: no timed tile launch (the record
  // counts live in the shared array, not the context's tables) and no chunked host copy
  c->tile_timed = false;
  c->nchunk = 0;
  GridPtrs gp;
  for (int k = 0; k < 4; k++)
    gp.g[k] = k < c->nslot ? (void *)((float *)c->grid_base + c->grid_elems * k) : nullptr;
  CK(c, cudaMemsetAsync(c->st, 0, sizeof(DevStats), c->stream));
  CK(c, cudaEventRecord(c->ev[0], c->stream));
  launch_paint32(c->stream, c->g, c->fs, c->tg, det ? 1 : 0, d.dtype, d.x, d.y, d.z, d.vlos, d.w, (long long)n, gp,
                 b, c->st, &c->launches);
  CK(c, cudaGetLastError());
  CK(c, cudaEventRecord(c->ev[1], c->stream));
  c->grids_intact = true;
  return CAPOW_OK;
}
