// Paint-stage interfaces shared by paint.cu and capow_api.cu.
#pragma once
#include "common.cuh"

template <typename T>
struct PIn {
  const T *x, *y, *z, *v, *w;  // v, w may be null
};

// Device-side counters of one paint (read back by capow_get_stats / capow_power).
struct DevStats {
  double nread, nout, ngrid, nsq;
  double vr[4];
  double dc[4];              // sum of every value deposited inside the FFT region, per grid slot
  double absw[2];            // sum |w v^e| per field: bound used for the fixed-point scale
  unsigned long long dc_fixed[4];  // deterministic mode: exact integer DC sums
  unsigned int nspecial;     // particles routed to the exact FP64 rules
  unsigned int nrecords;     // tile-list records needed
  unsigned long long fatal_inv;  // max of (~0 - index) over LOS == 0 particles outside the box
  int fatal;                 // LOS == 0 particle outside the box
  int nonfinite;             // NaN/inf coordinate
  int overflow;              // record buffer too small
  int timeout;               // a bounded device wait of the power stage gave up (CAPOW_ETIMEOUT)
};

// Tile decomposition of the grid for the FP32 path.
struct TileGeo {
  int tx, ty, tz;  // powers of two
  int lx, ly, lz;  // log2 of the tile edges
  int nbx, nby, nbz;
  int ntiles;
  // shared-memory tile pitches (elements): row pitch py = 3 (mod 32) and plane pitch px = 9 (mod 32)
  // put the 27 taps of one stencil in 27 distinct banks; slot = px * tx elements
  int py, px, slot;
};

// Grid slot order: slot = stencil * nfields + field (A normal, B normal, A interlaced, B interlaced
// for two fields). Pointers to padded [NX][NY][2(NZ/2+1)] grids.
struct GridPtrs {
  void *g[4];
};

struct PaintBufs {
  unsigned int *counts;    // ntiles
  unsigned int *offsets;   // ntiles + 1
  unsigned int *cursor;    // ntiles
  float4 *recs;            // capacity
  float *recw;             // capacity (only when weights are given)
  unsigned long long capacity;
  double *fixed_scale;     // [2] deterministic mode: 2^S per field (device)
  unsigned int *edge_list; // FP32: indices of particles painted by the exact rules after the tiles
  unsigned int *edge_count;
  unsigned long long edge_cap;
  // bucket mode (bucket_cap > 0): one pass writes each tile's records into its own fixed-capacity
  // bucket recs[tile * bucket_cap ...]; records beyond a full bucket go to the overflow list with
  // their tile and are deposited with global atomics after the tiles
  unsigned bucket_cap;
  float4 *ovf_recs;
  float *ovf_w;
  unsigned *ovf_tile;
  unsigned *ovf_count;
  unsigned long long ovf_cap;
  // when set, recorded on the stream just before and after the tile-deposit kernel
  cudaEvent_t tile_ev0, tile_ev1;
  // bucket mode with host input copied in chunks: the bucket pass runs per chunk k (particles
  // [k n / nchunk, (k + 1) n / nchunk)), each launch after chunk_ev[k]
  int nchunk;
  const cudaEvent_t *chunk_ev;
};

// host launchers (paint.cu)
void launch_paint64(cudaStream_t s, const Geom &g, const FieldSpec &fs, int dtype, const void *x, const void *y,
                    const void *z, const void *v, const void *w, long long n, const GridPtrs &grids, DevStats *st,
                    long long *launches);

void launch_paint32(cudaStream_t s, const Geom &g, const FieldSpec &fs, const TileGeo &tg, int deterministic,
                    int dtype, const void *x, const void *y, const void *z, const void *v, const void *w,
                    long long n, const GridPtrs &grids, const PaintBufs &b, DevStats *st, long long *launches);

// suggested tile geometry for a grid (and whether two fields are painted)
TileGeo choose_tiles(const Geom &g, int nslots, int deterministic);
TileGeo make_tiles(const Geom &g, int tx, int ty, int tz);  // tx, ty, tz powers of two (>= 4)
size_t tile_smem_bytes(const TileGeo &tg, int nslots, int deterministic);
size_t rec_smem_bytes(const TileGeo &tg, int nslots);
double tile_dup_estimate(const Geom &g, const TileGeo &tg);
