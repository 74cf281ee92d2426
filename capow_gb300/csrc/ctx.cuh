// Context of one P(k) configuration (the C ABI's capow_ctx) and the error macros of the entry
// points; shared by capow_api.cu and noalloc.cu.
#pragma once
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdio.h>

#include <vector>

#include "bin.cuh"
#include "paint.cuh"

#define NPROD 4  // bin products when two fields are painted

struct capow_ctx {
  capow_params p;
  capow_options o;
  int prec;
  Geom g;
  FieldSpec fs;
  TileGeo tg;
  BinParams bp;
  BinTables bt;
  int nslot;
  int spec_kind[CAPOW_MAX_SPEC];
  int shot_moment[CAPOW_MAX_SPEC];  // 0: N, n: <v^n> N
  int moments;
  cudaStream_t stream;
  bool own_stream;
  // device buffers
  void *grid_base;      // nslot padded grids, contiguous
  size_t grid_elems;    // reals per padded grid
  DevStats *st;
  PaintBufs pb;
  double *fixed_scale;
  double *dcv;
  double *bins, *bins2d;
  unsigned long long *nmodes_d, *nmodes2d_d;
  std::vector<unsigned long long> nmodes, nmodes2d;
  cufftHandle plan;
  bool plan_ok;
  // transposed fused path (power-of-two NZ): k_zr2c writes [NX][NZ/2+1][NY] complex per slot into
  // tbuf, yplan is the batched C2C along y over it
  bool xtr;
  float2 *tbuf;
  long long tslot;  // complex values per slot of tbuf
  cufftHandle yplan;
  bool yplan_ok;
  // power-of-two NY as well: the z pass and the y axis in one launch (k_zy) instead of k_zr2c + yplan;
  // zy_ctr holds its work-queue and per-plane counters
  bool zy;
  unsigned *zy_ctr;
  int zy_stall;  // CAPOW_TEST_STALL_ZY=1 at creation: k_zy's waits run out (the timeout path's test)
  bool fused;           // FP32: 2-D (y, z) cuFFT + fused x-axis FFT and binning (k_xfft_bin)
  XbinGeo xg;
  // capow_backward (created on first use): full 3-D plans, bin coefficients, host-output staging
  bool quiet;           // skip the stage-timing event records (batched enqueue, graph capture)
  bool two_pass;        // FP32 paint: count/scan/scatter instead of the one-pass buckets
  float bucket_factor;  // one-pass buckets: records per tile = factor * the tile's mean share + 64 (0: 2)
  bool adj_plans;
  cufftHandle adj_fwd, adj_inv;
  double *adj_coef;
  void *adj_stage[5];
  size_t adj_stage_bytes[5];
  // staging for host particle input: two sets, alternating between host-input paints, so that a
  // catalogue's copy can run while the previous one's power stage still reads its own set
  void *stage[2][5];
  size_t stage_bytes[2][5];
  int stage_set;                 // the set the next host-input paint fills
  cudaEvent_t stage_free[2];     // recorded on the context stream after the last paint that read each set
  bool stage_used[2];
  capow_particles last;   // device view of the last painted catalogue
  bool painted, powered;
  bool grids_intact;  // the slots still hold the last paint: the power stage read them out of place
  // capow_power_enqueue .. capow_power_result: the power stage in flight (its catalogue, for a repaint
  // after an overflow) and whether one capow_paint has been queued behind it
  bool pending, pend_paint;
  capow_particles pend_last;
  cudaEvent_t power_ev;
  // host pinned readback
  double *h_bins;
  DevStats *h_st;
  std::vector<void *> allocs;
  cudaEvent_t ev[4];
  cudaEvent_t ev_tile[2];  // around the FP32 tile-deposit kernel of the last paint
  // host catalogues of FP32 bucket-mode paints are copied in CAPOW_CHUNKS chunks on copy_stream, and
  // the bucket pass of each chunk starts when its copy lands (chunk_ev); nchunk > 1 for that paint
  cudaStream_t copy_stream;
  cudaEvent_t chunk_ev[4];
  int nchunk;
  bool tile_timed;         // the last FP32 paint recorded ev_tile
  long long launches;
  char err[512];
};

#define FAIL(ctx, code, ...)                                        \
  do {                                                              \
    if (ctx) snprintf((ctx)->err, sizeof((ctx)->err), __VA_ARGS__); \
    return (code);                                                  \
  } while (0)

#define CK(ctx, call)                                                                                       \
  do {                                                                                                      \
    cudaError_t e_ = (call);                                                                                \
    if (e_ != cudaSuccess) FAIL(ctx, CAPOW_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                                __LINE__);                                                                  \
  } while (0)

#define CKFFT(ctx, call)                                                         \
  do {                                                                           \
    cufftResult r_ = (call);                                                     \
    if (r_ != CUFFT_SUCCESS) FAIL(ctx, CAPOW_ECUFFT, "%s failed: cufft status %d", #call, (int)r_); \
  } while (0)

// capow_api.cu: paint the last catalogue again and prepare the DC values (capow_backward).
int enqueue_backward_paint(capow_ctx *c);
// product of one spectrum in the bin kernels' [product][5][NK] sums: |A|^2, Re(A*B), Im(A*B), |B|^2
int spectrum_product(int nfields, const SpecDef &sd);

// capow_api.cu pieces shared with batch.cu and survey.cu
Geom make_geom(const capow_params &p);
// survey: 0, or the number of survey fields (1: w; 2: w and w vlos)
int create_paint_ctx(const capow_params *p, const capow_options *o, int survey, capow_ctx **out);
// sync, read the paint counters into c->h_st, repaint c->last when the tile lists overflowed
int settle_paint(capow_ctx *c);
int enqueue_paint(capow_ctx *c, const capow_particles &d);
int enqueue_power_kernels(capow_ctx *c);
// Size the FP32 record and edge buffers (and, unless two_pass, the one-pass buckets at bucket_factor and
// their overflow list) for catalogues of up to nmax particles, so that a later enqueue_paint allocates nothing.
int prepare_paint_buffers(capow_ctx *c, unsigned long long nmax, bool weights);
void fill_spectra(const capow_ctx *c, const capow_params &p, const DevStats &st, const double *h_bins,
                  const unsigned long long *nmodes, const unsigned long long *nmodes2d, capow_spectrum *out);
