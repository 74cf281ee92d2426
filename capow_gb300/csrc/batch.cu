// capow_batch: many independent periodic-box mocks (each its own box, grid, interpolation order and
// catalogue) in one call. The reference runs one mock per process (src/main.c:28-298); here:
//  * mocks that share a grid shape share one context: grids, cuFFT plans, tile tables and record
//    buffers are allocated once per shape and sized for its largest catalogue;
//  * each mock has its own bin tables, mode counts, counters and bins (its box sets the k grid);
//  * every mock is enqueued on one stream with no host synchronisation and no allocation, so the
//    whole batch can be captured as one CUDA graph and launched once; the bins, counts and counters
//    of all mocks are read back at the end;
//  * an autotuner times candidate tile shapes of the FP32 paint on the first mock of each shape.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "ctx.cuh"

namespace {

typedef std::tuple<int, int, int, int, int, int, int, int, int, int, int, double, double> ShapeKey;

ShapeKey shape_of(const capow_params &p) {
  return ShapeKey(p.NX, p.NY, p.NZ, p.InterpOrder, p.DoInterlacing, p.NK, p.LOS, p.Momentum, p.Odd_Multipoles,
                  p.Output2D, p.OutputLog, p.Mink, p.Maxk);
}

struct MockDev {
  BinTables bt;
  DevStats *st;
  double *dcv, *bins;
  unsigned long long *nmodes;
  Geom g;
  BinParams bp;
};

// Candidate tile shapes for the FP32 paint: the int32 tiles of every slot within 64 KB per CTA.
std::vector<std::tuple<int, int, int>> tile_candidates(int nslot) {
  if (nslot >= 4) return {{8, 16, 32}, {16, 8, 32}, {4, 32, 32}, {16, 16, 16}, {8, 32, 16}};
  if (nslot == 2) return {{16, 16, 32}, {8, 32, 32}, {32, 16, 16}, {16, 32, 16}};
  return {{16, 32, 32}, {32, 16, 32}, {32, 32, 16}};
}

// Point a shape context at one mock's geometry, tables and output buffers.
void bind_mock(capow_ctx *c, const capow_params &p, const MockDev &m) {
  c->p = p;
  c->g = m.g;
  c->bp = m.bp;
  c->bt = m.bt;
  c->st = m.st;
  c->dcv = m.dcv;
  c->bins = m.bins;
}

int time_paint(capow_ctx *c, const capow_particles &d, float *ms) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, c->stream);
  int rc = CAPOW_OK;
  for (int r = 0; r < 3 && !rc; r++) rc = enqueue_paint(c, d);
  cudaEventRecord(b, c->stream);
  cudaEventSynchronize(b);
  cudaEventElapsedTime(ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return rc;
}

// tile shapes chosen by the autotuner, per grid shape, for the life of the process
std::mutex g_tuned_mu;
std::map<ShapeKey, TileGeo> g_tuned;

}  // namespace

extern "C" int capow_batch(capow_mock *mocks, int nmocks, const capow_options *opt, int flags) {
  if (!mocks || nmocks < 0) return CAPOW_EINVAL;
  if (nmocks == 0) return CAPOW_OK;
  capow_options o;
  memset(&o, 0, sizeof o);
  if (opt) o = *opt;
  else o.precision = CAPOW_FP32_MIXED;
  if (cudaSetDevice(o.device) != cudaSuccess) return CAPOW_ECUDA;
  for (int i = 0; i < nmocks; i++) {
    mocks[i].status = CAPOW_OK;
    if (!mocks[i].parts.on_device || !mocks[i].out || mocks[i].params.Output2D) mocks[i].status = CAPOW_EINVAL;
  }
  // ---- one context per grid shape, on one stream
  cudaStream_t stream = (cudaStream_t)o.stream;
  bool own_stream = false;
  if (!stream) {
    if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) return CAPOW_ECUDA;
    own_stream = true;
  }
  capow_options so = o;
  so.stream = stream;
  std::map<ShapeKey, capow_ctx *> ctxs;
  std::map<ShapeKey, unsigned long long> nmax;
  std::map<ShapeKey, bool> wts;
  std::vector<capow_ctx *> ctx_of(nmocks, nullptr);
  int rc = CAPOW_OK;
  for (int i = 0; i < nmocks; i++) {
    if (mocks[i].status) continue;
    const ShapeKey k = shape_of(mocks[i].params);
    if (!ctxs.count(k)) {
      capow_ctx *c = nullptr;
      const int r = capow_create(&mocks[i].params, &so, &c);
      if (r) {
        if (c) capow_destroy(c);
        mocks[i].status = r;
        continue;
      }
      c->quiet = true;
      c->two_pass = true;  // record buffers sized once per shape (prepare_paint_buffers)
      ctxs[k] = c;
    }
    ctx_of[i] = ctxs[k];
    nmax[k] = std::max(nmax[k], (unsigned long long)mocks[i].parts.n);
    wts[k] = wts[k] || mocks[i].parts.w != nullptr;
  }
  // ---- per-mock tables and output buffers (one device arena for the small per-mock arrays)
  const size_t per = ((sizeof(DevStats) + 255) & ~(size_t)255) + 256;  // counters + 4 DC values
  std::vector<MockDev> md(nmocks);
  std::vector<unsigned char> blob;  // every mock's bin tables, uploaded once
  std::vector<size_t> tab_off(nmocks, 0);
  void *tab_dev = nullptr;
  size_t bins_total = 0, nm_total = 0;
  std::vector<size_t> bins_off(nmocks, 0), nm_off(nmocks, 0);
  for (int i = 0; i < nmocks; i++) {
    if (!ctx_of[i]) continue;
    bins_off[i] = bins_total;
    nm_off[i] = nm_total;
    bins_total += (size_t)NPROD * 5 * mocks[i].params.NK;
    nm_total += mocks[i].params.NK;
  }
  char *arena = nullptr;
  double *bins_d = nullptr;
  unsigned long long *nm_d = nullptr;
  const size_t arena_bytes = per * nmocks + 8 * bins_total + 8 * nm_total + 512;
  if (cudaMalloc(&arena, arena_bytes) != cudaSuccess) rc = CAPOW_ENOMEM;
  if (!rc) {
    bins_d = (double *)(arena + ((per * nmocks + 255) & ~(size_t)255));
    nm_d = (unsigned long long *)(bins_d + bins_total);
  }
  for (int i = 0; i < nmocks && !rc; i++) {
    capow_ctx *c = ctx_of[i];
    if (!c) continue;
    const capow_params &p = mocks[i].params;
    MockDev &m = md[i];
    m.g = make_geom(p);
    if (c->prec != CAPOW_FP64 && !(m.g.margin < 0.25f)) {
      mocks[i].status = CAPOW_ENOTSUP;
      ctx_of[i] = nullptr;
      continue;
    }
    m.bp = c->bp;
    m.bp.fx_step = (float)(1.0 / ((float)p.NX * m.g.dx));
    bin_params_kguess(m.bp, p);
    tab_off[i] = (blob.size() + 255) & ~(size_t)255;
    blob.resize(tab_off[i]);
    std::vector<unsigned char> one;
    if (build_bin_tables_packed(p, m.g, c->prec, m.bt, one)) {
      mocks[i].status = CAPOW_ENOMEM;
      ctx_of[i] = nullptr;
      continue;
    }
    blob.insert(blob.end(), one.begin(), one.end());
    m.st = (DevStats *)(arena + per * i);
    m.dcv = (double *)(arena + per * i + ((sizeof(DevStats) + 255) & ~(size_t)255));
    m.bins = bins_d + bins_off[i];
    m.nmodes = nm_d + nm_off[i];
  }
  if (!rc && !blob.empty()) {
    if (cudaMalloc(&tab_dev, blob.size()) != cudaSuccess ||
        cudaMemcpyAsync(tab_dev, blob.data(), blob.size(), cudaMemcpyHostToDevice, stream) != cudaSuccess)
      rc = CAPOW_ENOMEM;
    for (int i = 0; i < nmocks && !rc; i++)
      if (ctx_of[i]) relocate_bin_tables(md[i].bt, (const char *)tab_dev + tab_off[i]);
  }
  // ---- record buffers for the largest catalogue of each shape; the tile autotuner (its choice is
  // kept per grid shape for later calls)
  for (auto &kv : ctxs) {
    if (rc) break;
    capow_ctx *c = kv.second;
    rc = prepare_paint_buffers(c, nmax[kv.first], wts[kv.first]);
    if (rc || !(flags & CAPOW_BATCH_AUTOTUNE) || c->prec != CAPOW_FP32_MIXED) continue;
    {
      std::lock_guard<std::mutex> lock(g_tuned_mu);
      auto it = g_tuned.find(kv.first);
      if (it != g_tuned.end()) {
        c->tg = it->second;
        continue;
      }
    }
    int first = -1;
    for (int i = 0; i < nmocks; i++)
      if (ctx_of[i] == c) {
        first = i;
        break;
      }
    if (first < 0) continue;
    const TileGeo keep = c->tg;
    const PaintBufs keep_pb = c->pb;
    bind_mock(c, mocks[first].params, md[first]);
    TileGeo best = keep;
    float best_ms = 1e30f;
    for (auto &cand : tile_candidates(c->nslot)) {
      const TileGeo tg = make_tiles(c->g, std::get<0>(cand), std::get<1>(cand), std::get<2>(cand));
      if (tg.ntiles > keep.ntiles) continue;  // the tile tables are sized for the default shape
      if (tile_dup_estimate(c->g, tg) > tile_dup_estimate(c->g, keep) * 1.05) continue;  // records must fit
      c->tg = tg;
      float ms = 0.0f;
      if (time_paint(c, mocks[first].parts, &ms) == CAPOW_OK && ms < best_ms) {
        best_ms = ms;
        best = tg;
      }
    }
    c->tg = best;
    c->pb = keep_pb;
    std::lock_guard<std::mutex> lock(g_tuned_mu);
    g_tuned[kv.first] = best;
  }
  // ---- enqueue every mock (optionally captured as one graph)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool captured = false;
  if (!rc && (flags & CAPOW_BATCH_GRAPH)) {
    // one uncaptured pass over the first mock of each shape: every kernel and plan the graph will
    // hold has run once before the capture starts
    for (auto &kv : ctxs) {
      capow_ctx *c = kv.second;
      for (int i = 0; i < nmocks; i++) {
        if (ctx_of[i] != c) continue;
        bind_mock(c, mocks[i].params, md[i]);
        capow_particles d = mocks[i].parts;
        if (!c->fs.need_v) d.vlos = nullptr;
        launch_mode_counts(stream, c->bp, c->bt, md[i].nmodes, nullptr, &c->launches);
        rc = enqueue_paint(c, d);
        if (!rc) rc = enqueue_power_kernels(c);
        break;
      }
      if (rc) break;
    }
  }
  if (!rc) {
    cudaStreamSynchronize(stream);  // table uploads, tuning and warm-up done
    if ((flags & CAPOW_BATCH_GRAPH) &&
        cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess)
      captured = true;
    for (int i = 0; i < nmocks && !rc; i++) {
      capow_ctx *c = ctx_of[i];
      if (!c) continue;
      bind_mock(c, mocks[i].params, md[i]);
      const int nk = mocks[i].params.NK;
      cudaMemsetAsync(md[i].nmodes, 0, sizeof(unsigned long long) * nk, stream);
      launch_mode_counts(stream, c->bp, c->bt, md[i].nmodes, nullptr, &c->launches);
      capow_particles d = mocks[i].parts;
      if (!c->fs.need_v) d.vlos = nullptr;
      int r = enqueue_paint(c, d);
      if (!r) r = enqueue_power_kernels(c);
      if (r) mocks[i].status = r;
    }
    if (captured) {
      const cudaError_t e = cudaStreamEndCapture(stream, &graph);
      if (e != cudaSuccess || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess ||
          cudaGraphLaunch(exec, stream) != cudaSuccess)
        rc = CAPOW_ECUDA;
    }
    if (!rc && cudaStreamSynchronize(stream) != cudaSuccess) rc = CAPOW_ECUDA;
  }
  // ---- read back and fill every mock's spectra (the host side of capow_power)
  if (!rc) {
    std::vector<unsigned char> hst(per * nmocks);
    std::vector<double> hb(bins_total);
    std::vector<unsigned long long> hnm(nm_total);
    if (cudaMemcpy(hst.data(), arena, per * nmocks, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(hb.data(), bins_d, 8 * bins_total, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(hnm.data(), nm_d, 8 * nm_total, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = CAPOW_ECUDA;
    for (int i = 0; i < nmocks && !rc; i++) {
      capow_ctx *c = ctx_of[i];
      if (!c || mocks[i].status) continue;
      const DevStats &st = *(const DevStats *)(hst.data() + per * i);
      if (st.overflow) {  // rare: the record estimate was short; a context of its own repaints this mock
        capow_ctx *c1 = nullptr;
        capow_options o1 = o;
        o1.stream = nullptr;
        int r = capow_create(&mocks[i].params, &o1, &c1);
        if (!r) r = capow_paint(c1, &mocks[i].parts);
        if (!r) r = capow_power(c1, mocks[i].out, capow_num_spectra(c1));
        if (c1) capow_destroy(c1);
        mocks[i].status = r;
        continue;
      }
      if (st.nonfinite) {
        mocks[i].status = CAPOW_EINVAL;
        continue;
      }
      if (st.fatal) {
        mocks[i].status = CAPOW_EBOUNDS;
        continue;
      }
      fill_spectra(c, mocks[i].params, st, hb.data() + bins_off[i], hnm.data() + nm_off[i], nullptr, mocks[i].out);
    }
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  for (auto &kv : ctxs) capow_destroy(kv.second);  // restores nothing: the contexts are private
  if (tab_dev) cudaFree(tab_dev);
  if (arena) cudaFree(arena);
  if (own_stream) cudaStreamDestroy(stream);
  return rc;
}
