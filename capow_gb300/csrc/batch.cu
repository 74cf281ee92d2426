// capow_batch: many independent periodic-box mocks (each its own box, grid, interpolation order and
// catalogue) in one call. The reference runs one mock per process (src/main.c:28-298); here:
//  * mocks that share a grid shape share a small ring of contexts (BATCH_RING): grids, cuFFT plans, tile
//    tables and record buffers are allocated per context and sized for its largest catalogue, and the
//    shape's mocks alternate between the ring's contexts;
//  * every context runs on a stream of its own, forked from the batch stream by one event and joined
//    back by another, so that the mocks of different contexts (of one shape or of different shapes)
//    overlap on the GPU: small grids do not fill it one kernel at a time;
//  * each mock has its own bin tables, mode counts, counters and bins (its box sets the k grid);
//  * every mock is enqueued with no host synchronisation and no allocation, so the whole batch (the
//    fork, every context's work and the join) can be captured as one CUDA graph and launched once; the
//    bins, counts and counters of all mocks are read back at the end;
//  * the FP32 paint is the one-pass bucket paint, its buffers sized per context before anything is
//    enqueued; an autotuner times candidate tile shapes and then bucket capacity factors on the first
//    mock of each shape.
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

// What the shared device resources of a context depend on: the grid shape (grids, plans, tile tables),
// the painted fields (LOS, Momentum) and the binning kernel's variant (odd multipoles). The box, the
// interpolation order and the k bins are per mock (geometry, tables and bins are bound per mock).
typedef std::tuple<int, int, int, int, int, int, int> ShapeKey;

ShapeKey shape_of(const capow_params &p) {
  return ShapeKey(p.NX, p.NY, p.NZ, p.DoInterlacing, p.LOS, p.Momentum, p.Odd_Multipoles);
}

struct MockDev {
  BinTables bt;
  DevStats *st;
  double *dcv, *bins;
  unsigned long long *nmodes;
  Geom g;
  BinParams bp;
  XbinGeo xg;  // the fused binning pass's blocks for this mock's bins
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
  if (c->fused) c->xg = m.xg;
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

// tile shapes and bucket factors chosen by the autotuner, per grid shape, for the life of the process
struct Tuned {
  TileGeo tg;
  float bucket_factor;
};
std::mutex g_tuned_mu;
std::map<ShapeKey, Tuned> g_tuned;

// Bucket capacity factors the autotuner times (records per tile = factor * mean share + 64): smaller
// buckets write fewer record slots, larger ones send fewer records to the slower overflow path.
const float kBucketFactors[] = {1.5f, 2.0f, 3.0f};

// The device state of one batch signature (the mocks' parameters, sizes and array kinds, the options
// and flags): shared contexts, per-mock tables and outputs, and the instantiated graph. It is kept
// after the call, so that a later call with the same signature (new particle values, or new arrays of
// the same sizes) only launches: the graph as it is when the arrays are the same, or updated in place
// (cudaGraphExecUpdate) when they moved. A call with another signature, or capow_batch_release,
// frees it.
constexpr int BATCH_RING = 2;  // contexts per grid shape

struct BatchState {
  std::vector<unsigned char> sig;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::map<ShapeKey, std::vector<capow_ctx *>> rings;
  std::vector<capow_ctx *> all;          // every context of every ring
  std::vector<cudaStream_t> ctx_streams;  // their streams (owned here)
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;         // one per context
  std::vector<capow_ctx *> ctx_of;
  std::vector<int> status0;  // per-mock status found while setting up (e.g. CAPOW_ENOTSUP)
  std::vector<MockDev> md;
  std::vector<size_t> bins_off, nm_off;
  size_t per = 0, bins_total = 0, nm_total = 0;
  char *arena = nullptr;
  double *bins_d = nullptr;
  unsigned long long *nm_d = nullptr;
  void *tab_dev = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<const void *> ptrs;  // the particle arrays the graph holds
};

std::mutex g_batch_mu;
BatchState *g_batch = nullptr;

void free_batch_state(BatchState *b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (cudaStream_t s : b->ctx_streams) cudaStreamSynchronize(s);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (capow_ctx *c : b->all) capow_destroy(c);
  for (cudaStream_t s : b->ctx_streams) cudaStreamDestroy(s);
  if (b->fork) cudaEventDestroy(b->fork);
  for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
  if (b->tab_dev) cudaFree(b->tab_dev);
  if (b->arena) cudaFree(b->arena);
  if (b->own_stream) cudaStreamDestroy(b->stream);
  delete b;
}

template <typename T>
void put(std::vector<unsigned char> &v, const T &x) {
  const unsigned char *p = (const unsigned char *)&x;
  v.insert(v.end(), p, p + sizeof(T));
}

std::vector<unsigned char> batch_signature(const capow_mock *mocks, int nmocks, const capow_options &o, int flags) {
  std::vector<unsigned char> s;
  put(s, o.precision);
  put(s, o.spectra);
  put(s, o.device);
  put(s, o.stream);
  put(s, o.fft_path);
  put(s, flags & CAPOW_BATCH_AUTOTUNE);
  put(s, nmocks);
  for (int i = 0; i < nmocks; i++) {
    const capow_params &p = mocks[i].params;  // field by field: the struct's padding is not compared
    const int ints[] = {p.NX, p.NY, p.NZ, p.InterpOrder, p.DoInterlacing, p.NK, p.NMU, p.Output2D, p.OutputLog,
                        p.LOS, p.Momentum, p.Odd_Multipoles};
    const double dbls[] = {p.XMIN, p.XMAX, p.YMIN, p.YMAX, p.ZMIN, p.ZMAX, p.Mink, p.Maxk, p.Omega_m, p.Redshift};
    put(s, ints);
    put(s, dbls);
    put(s, mocks[i].parts.n);
    put(s, mocks[i].parts.dtype);
    put(s, mocks[i].parts.on_device);
    put(s, mocks[i].parts.vlos != nullptr);
    put(s, mocks[i].parts.w != nullptr);
  }
  return s;
}

std::vector<const void *> batch_pointers(const capow_mock *mocks, int nmocks) {
  std::vector<const void *> p;
  for (int i = 0; i < nmocks; i++) {
    p.push_back(mocks[i].parts.x);
    p.push_back(mocks[i].parts.y);
    p.push_back(mocks[i].parts.z);
    p.push_back(mocks[i].parts.vlos);
    p.push_back(mocks[i].parts.w);
  }
  return p;
}

// Contexts, tables, buffers and tuning of a new signature. Returns a status; per-mock problems go to
// b->status0.
int setup_batch(BatchState *b, const capow_mock *mocks, int nmocks, const capow_options &o, int flags) {
  b->status0.assign(nmocks, CAPOW_OK);
  for (int i = 0; i < nmocks; i++)
    if (!mocks[i].parts.on_device || !mocks[i].out || mocks[i].params.Output2D) b->status0[i] = CAPOW_EINVAL;
  b->stream = (cudaStream_t)o.stream;
  if (!b->stream) {
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return CAPOW_ECUDA;
    b->own_stream = true;
  }
  if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) return CAPOW_ECUDA;
  std::map<capow_ctx *, unsigned long long> nmax;
  std::map<capow_ctx *, bool> wts;
  b->ctx_of.assign(nmocks, nullptr);
  // the contexts of a shape are created for its largest interpolation order (the record buffers are
  // sized for the widest footprint); the ring has BATCH_RING contexts, or one per mock when fewer
  std::map<ShapeKey, int> max_order, count;
  for (int i = 0; i < nmocks; i++)
    if (!b->status0[i]) {
      int &mo = max_order[shape_of(mocks[i].params)];
      mo = std::max(mo, mocks[i].params.InterpOrder);
      count[shape_of(mocks[i].params)]++;
    }
  std::map<ShapeKey, int> seen;
  for (int i = 0; i < nmocks; i++) {
    if (b->status0[i]) continue;
    const ShapeKey k = shape_of(mocks[i].params);
    std::vector<capow_ctx *> &ring = b->rings[k];
    const int want = std::min(BATCH_RING, count[k]);
    const int slot = seen[k]++ % want;
    if ((int)ring.size() <= slot) {
      cudaStream_t cs = nullptr;
      cudaEvent_t je = nullptr;
      if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) return CAPOW_ECUDA;
      b->ctx_streams.push_back(cs);  // freed with the state whatever follows
      capow_options so = o;
      so.stream = cs;
      capow_ctx *c = nullptr;
      capow_params cp = mocks[i].params;
      cp.InterpOrder = max_order[k];
      const int r = capow_create(&cp, &so, &c);
      if (r) {
        if (c) capow_destroy(c);
        b->status0[i] = r;
        continue;
      }
      if (cudaEventCreateWithFlags(&je, cudaEventDisableTiming) != cudaSuccess) {
        capow_destroy(c);
        return CAPOW_ECUDA;
      }
      c->quiet = true;  // record buffers sized once per context (prepare_paint_buffers)
      ring.push_back(c);
      b->all.push_back(c);
      b->joins.push_back(je);
    }
    if (ring.empty()) {
      b->status0[i] = CAPOW_ECUDA;
      continue;
    }
    capow_ctx *c = ring[slot < (int)ring.size() ? slot : 0];
    b->ctx_of[i] = c;
    nmax[c] = std::max(nmax[c], (unsigned long long)mocks[i].parts.n);
    wts[c] = wts[c] || mocks[i].parts.w != nullptr;
  }
  // ---- per-mock tables and output buffers (one device arena for the small per-mock arrays)
  b->per = ((sizeof(DevStats) + 255) & ~(size_t)255) + 256;  // counters + 4 DC values
  b->md.assign(nmocks, MockDev());
  std::vector<unsigned char> blob;  // every mock's bin tables, uploaded once
  std::vector<size_t> tab_off(nmocks, 0);
  b->bins_off.assign(nmocks, 0);
  b->nm_off.assign(nmocks, 0);
  for (int i = 0; i < nmocks; i++) {
    if (!b->ctx_of[i]) continue;
    b->bins_off[i] = b->bins_total;
    b->nm_off[i] = b->nm_total;
    b->bins_total += (size_t)NPROD * 5 * mocks[i].params.NK;
    b->nm_total += mocks[i].params.NK;
  }
  const size_t arena_bytes = b->per * nmocks + 8 * b->bins_total + 8 * b->nm_total + 512;
  if (cudaMalloc((void **)&b->arena, arena_bytes) != cudaSuccess) return CAPOW_ENOMEM;
  b->bins_d = (double *)(b->arena + ((b->per * nmocks + 255) & ~(size_t)255));
  b->nm_d = (unsigned long long *)(b->bins_d + b->bins_total);
  for (int i = 0; i < nmocks; i++) {
    capow_ctx *c = b->ctx_of[i];
    if (!c) continue;
    const capow_params &p = mocks[i].params;
    MockDev &m = b->md[i];
    m.g = make_geom(p);
    if (c->prec != CAPOW_FP64 && !(m.g.margin < 0.25f)) {
      b->status0[i] = CAPOW_ENOTSUP;
      b->ctx_of[i] = nullptr;
      continue;
    }
    m.bp = c->bp;
    m.bp.nk = p.NK;
    m.bp.out2d = p.Output2D;
    m.bp.fx_step = (float)(1.0 / ((float)p.NX * m.g.dx));
    bin_params_kguess(m.bp, p);
    if (c->fused && !xbin_plan(m.bp, c->nslot, m.xg, c->xtr)) {  // this mock's bins do not fit the pass
      b->status0[i] = CAPOW_ENOTSUP;
      b->ctx_of[i] = nullptr;
      continue;
    }
    tab_off[i] = (blob.size() + 255) & ~(size_t)255;
    blob.resize(tab_off[i]);
    std::vector<unsigned char> one;
    if (build_bin_tables_packed(p, m.g, c->prec, m.bt, one)) {
      b->status0[i] = CAPOW_ENOMEM;
      b->ctx_of[i] = nullptr;
      continue;
    }
    blob.insert(blob.end(), one.begin(), one.end());
    m.st = (DevStats *)(b->arena + b->per * i);
    m.dcv = (double *)(b->arena + b->per * i + ((sizeof(DevStats) + 255) & ~(size_t)255));
    m.bins = b->bins_d + b->bins_off[i];
    m.nmodes = b->nm_d + b->nm_off[i];
  }
  if (!blob.empty()) {
    if (cudaMalloc(&b->tab_dev, blob.size()) != cudaSuccess ||
        cudaMemcpyAsync(b->tab_dev, blob.data(), blob.size(), cudaMemcpyHostToDevice, b->stream) != cudaSuccess)
      return CAPOW_ENOMEM;
    for (int i = 0; i < nmocks; i++)
      if (b->ctx_of[i]) relocate_bin_tables(b->md[i].bt, (const char *)b->tab_dev + tab_off[i]);
    // the contexts' streams read the tables: the upload completes first
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return CAPOW_ECUDA;
  }
  // ---- record buffers for the largest catalogue of each context; the autotuner, on the first context of
  // each shape: the tile shape, then the one-pass buckets' capacity factor (its choice is kept per grid
  // shape for later calls and given to the ring); then the buffers again for the chosen settings
  for (capow_ctx *c : b->all) {
    int rc = prepare_paint_buffers(c, nmax[c], wts[c]);
    if (rc) return rc;
  }
  for (auto &kv : b->rings) {
    if (kv.second.empty()) continue;
    capow_ctx *c = kv.second[0];
    if (!(flags & CAPOW_BATCH_AUTOTUNE) || c->prec != CAPOW_FP32_MIXED) continue;
    {
      std::lock_guard<std::mutex> lock(g_tuned_mu);
      auto it = g_tuned.find(kv.first);
      if (it != g_tuned.end()) {
        for (capow_ctx *r : kv.second) {
          r->tg = it->second.tg;
          r->bucket_factor = it->second.bucket_factor;
        }
        continue;
      }
    }
    int first = -1;
    for (int i = 0; i < nmocks; i++)
      if (b->ctx_of[i] == c) {
        first = i;
        break;
      }
    if (first < 0) continue;
    const TileGeo keep = c->tg;
    bind_mock(c, mocks[first].params, b->md[first]);
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
    float best_f = c->bucket_factor;
    best_ms = 1e30f;
    for (float f : kBucketFactors) {
      c->bucket_factor = f;
      float ms = 0.0f;
      if (time_paint(c, mocks[first].parts, &ms) == CAPOW_OK && ms < best_ms) {
        best_ms = ms;
        best_f = f;
      }
    }
    for (capow_ctx *r : kv.second) {
      r->tg = best;
      r->bucket_factor = best_f;
    }
    std::lock_guard<std::mutex> lock(g_tuned_mu);
    g_tuned[kv.first] = Tuned{best, best_f};
  }
  for (capow_ctx *c : b->all) {  // the buffers for the chosen tiles and buckets: enqueues allocate nothing
    int rc = prepare_paint_buffers(c, nmax[c], wts[c]);
    if (rc) return rc;
  }
  // ---- one uncaptured pass over the first mock of each context: every kernel and plan a graph holds
  // has run once before a capture starts
  if (flags & CAPOW_BATCH_GRAPH) {
    for (capow_ctx *c : b->all) {
      for (int i = 0; i < nmocks; i++) {
        if (b->ctx_of[i] != c) continue;
        bind_mock(c, mocks[i].params, b->md[i]);
        capow_particles d = mocks[i].parts;
        if (!c->fs.need_v) d.vlos = nullptr;
        launch_mode_counts(c->stream, c->bp, c->bt, b->md[i].nmodes, nullptr, &c->launches);
        int rc = enqueue_paint(c, d);
        if (!rc) rc = enqueue_power_kernels(c);
        if (rc) return rc;
        break;
      }
    }
  }
  for (cudaStream_t s : b->ctx_streams)
    if (cudaStreamSynchronize(s) != cudaSuccess) return CAPOW_ECUDA;
  return cudaStreamSynchronize(b->stream) == cudaSuccess ? CAPOW_OK : CAPOW_ECUDA;
}

// Every mock's kernels on its context's stream, forked from the batch stream and joined back to it (no
// host synchronisation, no allocation).
int enqueue_batch(BatchState *b, capow_mock *mocks, int nmocks) {
  cudaEventRecord(b->fork, b->stream);
  for (capow_ctx *c : b->all) cudaStreamWaitEvent(c->stream, b->fork, 0);
  for (int i = 0; i < nmocks; i++) {
    capow_ctx *c = b->ctx_of[i];
    if (!c) continue;
    bind_mock(c, mocks[i].params, b->md[i]);
    const int nk = mocks[i].params.NK;
    cudaMemsetAsync(b->md[i].nmodes, 0, sizeof(unsigned long long) * nk, c->stream);
    launch_mode_counts(c->stream, c->bp, c->bt, b->md[i].nmodes, nullptr, &c->launches);
    capow_particles d = mocks[i].parts;
    if (!c->fs.need_v) d.vlos = nullptr;
    int r = enqueue_paint(c, d);
    if (!r) r = enqueue_power_kernels(c);
    if (r) mocks[i].status = r;
  }
  for (size_t k = 0; k < b->all.size(); k++) {
    cudaEventRecord(b->joins[k], b->all[k]->stream);
    cudaStreamWaitEvent(b->stream, b->joins[k], 0);
  }
  return CAPOW_OK;
}

}  // namespace

extern "C" int capow_batch(capow_mock *mocks, int nmocks, const capow_options *opt, int flags) {
  if (!mocks || nmocks < 0) return CAPOW_EINVAL;
  if (nmocks == 0) return CAPOW_OK;
  capow_options o;
  memset(&o, 0, sizeof o);
  if (opt) o = *opt;
  else o.precision = CAPOW_FP32_MIXED;
  if (cudaSetDevice(o.device) != cudaSuccess) return CAPOW_ECUDA;
  std::lock_guard<std::mutex> lock(g_batch_mu);
  const std::vector<unsigned char> sig = batch_signature(mocks, nmocks, o, flags);
  BatchState *b = g_batch;
  int rc = CAPOW_OK;
  if (!b || b->sig != sig) {  // a new signature: the old state goes, this one is set up
    free_batch_state(g_batch);
    g_batch = nullptr;
    b = new (std::nothrow) BatchState();
    if (!b) return CAPOW_ENOMEM;
    b->sig = sig;
    rc = setup_batch(b, mocks, nmocks, o, flags);
    if (rc) {
      free_batch_state(b);
      return rc;
    }
    g_batch = b;
  }
  for (int i = 0; i < nmocks; i++) mocks[i].status = b->status0[i];
  // ---- enqueue every mock: directly, or as the cached graph (captured on first use, updated in
  // place when the particle arrays moved)
  if (flags & CAPOW_BATCH_GRAPH) {
    const std::vector<const void *> ptrs = batch_pointers(mocks, nmocks);
    if (!b->exec || ptrs != b->ptrs) {
      cudaGraph_t graph = nullptr;
      if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return CAPOW_ECUDA;
      enqueue_batch(b, mocks, nmocks);
      if (cudaStreamEndCapture(b->stream, &graph) != cudaSuccess) return CAPOW_ECUDA;
      bool ok = false;
      if (b->exec) {
        cudaGraphExecUpdateResultInfo info;
        ok = cudaGraphExecUpdate(b->exec, graph, &info) == cudaSuccess;
        if (!ok) {
          (void)cudaGetLastError();
          cudaGraphExecDestroy(b->exec);
          b->exec = nullptr;
        }
      }
      if (!ok) ok = cudaGraphInstantiate(&b->exec, graph, 0) == cudaSuccess;
      cudaGraphDestroy(graph);
      if (!ok) {
        b->exec = nullptr;
        return CAPOW_ECUDA;
      }
      b->ptrs = ptrs;
      for (int i = 0; i < nmocks; i++)  // statuses set while enqueueing under capture
        if (mocks[i].status) b->status0[i] = mocks[i].status;
    }
    if (cudaGraphLaunch(b->exec, b->stream) != cudaSuccess) return CAPOW_ECUDA;
  } else {
    enqueue_batch(b, mocks, nmocks);
  }
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return CAPOW_ECUDA;
  // ---- read back and fill every mock's spectra (the host side of capow_power)
  std::vector<unsigned char> hst(b->per * nmocks);
  std::vector<double> hb(b->bins_total);
  std::vector<unsigned long long> hnm(b->nm_total);
  if (cudaMemcpy(hst.data(), b->arena, b->per * nmocks, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(hb.data(), b->bins_d, 8 * b->bins_total, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(hnm.data(), b->nm_d, 8 * b->nm_total, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = CAPOW_ECUDA;
  for (int i = 0; i < nmocks && !rc; i++) {
    capow_ctx *c = b->ctx_of[i];
    if (!c || mocks[i].status) continue;
    const DevStats &st = *(const DevStats *)(hst.data() + b->per * i);
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
    if (st.timeout) {
      mocks[i].status = CAPOW_ETIMEOUT;
      continue;
    }
    fill_spectra(c, mocks[i].params, st, hb.data() + b->bins_off[i], hnm.data() + b->nm_off[i], nullptr,
                 mocks[i].out);
  }
  return rc;
}

extern "C" void capow_batch_release(void) {
  std::lock_guard<std::mutex> lock(g_batch_mu);
  free_batch_state(g_batch);
  g_batch = nullptr;
}
