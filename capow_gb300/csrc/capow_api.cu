// C ABI of libcapow_gpu (include/capow.h): context, orchestration of paint -> cuFFT -> bin,
// host-side reference arithmetic for alpha / shot / norm (src/main.c:106-148) and the
// output normalisation (src/main.c:1019-1056).
#include <cuda_runtime.h>
#include <cufft.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "ctx.cuh"

extern "C" const char *capow_strerror(int s) {
  switch (s) {
    case CAPOW_OK: return "ok";
    case CAPOW_EINVAL: return "invalid argument or parameter";
    case CAPOW_ENOMEM: return "out of memory";
    case CAPOW_ECUDA: return "CUDA runtime error";
    case CAPOW_EBOUNDS: return "particle out of grid bounds (LOS == 0)";
    case CAPOW_ETIMEOUT: return "device wait timed out";
    case CAPOW_ESTATE: return "call out of order";
    case CAPOW_ECUFFT: return "cuFFT error";
    case CAPOW_ENOTSUP: return "not supported";
  }
  return "unknown status";
}

extern "C" const char *capow_last_error(const capow_ctx *ctx) { return ctx ? ctx->err : "no context"; }

// check_inputs semantics (src/read_params.c:294-428) plus what the GPU layout requires.
static int validate(const capow_params *p, const capow_options *o, char *err, size_t n) {
#define BAD(...)                   \
  do {                             \
    snprintf(err, n, __VA_ARGS__); \
    return CAPOW_EINVAL;           \
  } while (0)
  if (p->LOS < 0 || p->LOS > 3) BAD("LOS is neither 0 (real-space), 1, 2 nor 3");
  if (p->InterpOrder < 1 || p->InterpOrder > 3) BAD("InterpOrder is neither 1, 2 nor 3");
  if (p->DoInterlacing != 0 && p->DoInterlacing != 1) BAD("DoInterlacing is neither 0 nor 1");
  if (p->Output2D != 0 && p->Output2D != 1) BAD("Output2D is neither 0 nor 1");
  if (p->Output2D && p->NMU <= 0) BAD("NMU is less than 1");
  if (p->OutputLog != 0 && p->OutputLog != 1) BAD("OutputLog is neither 0 nor 1");
  if (p->NX <= 0 || p->NY <= 0 || p->NZ <= 0) BAD("NX, NY and NZ must be > 0");
  if (p->NK <= 0) BAD("NK is less than 1");
  if (!(p->XMAX > p->XMIN) || !(p->YMAX > p->YMIN) || !(p->ZMAX > p->ZMIN)) BAD("box MAX must exceed MIN");
  if (p->Maxk < p->Mink) BAD("Maxk is less than Mink");
  if (p->Momentum < 0 || p->Momentum > 8) BAD("Momentum must be 0..8");
  if (o->precision < 0 || o->precision > 2) BAD("unknown precision");
  if (o->fft_path < CAPOW_FFT_AUTO || o->fft_path > CAPOW_FFT_ONE_LAUNCH) BAD("unknown fft_path");
  if (o->spectra < 0 || o->spectra > 7) BAD("unknown spectra mask");
  if (o->precision != CAPOW_FP64 && (p->NX < 4 || p->NY < 4 || p->NZ < 4))
    BAD("the FP32 paths need NX, NY, NZ >= 4");
  long long nzc = p->NZ / 2 + 1;
  if ((long long)p->NX * p->NY * 2 * nzc >= (1LL << 40)) BAD("grid too large");
  return CAPOW_OK;
#undef BAD
}

Geom make_geom(const capow_params &p) {
  Geom g;
  memset(&g, 0, sizeof g);
  g.nx = p.NX; g.ny = p.NY; g.nz = p.NZ;
  g.order = p.InterpOrder;
  g.los = p.LOS;
  g.interlace = p.DoInterlacing;
  g.nxtra = p.NX + p.InterpOrder;
  g.nzc = p.NZ / 2 + 1;
  g.row = 2LL * g.nzc;
  g.slice = (long long)p.NY * g.row;
  g.main_sz = (long long)p.NX * g.slice;
  g.xmin = p.XMIN; g.ymin = p.YMIN; g.zmin = p.ZMIN;
  g.xmax = p.XMAX; g.ymax = p.YMAX; g.zmax = p.ZMAX;
  g.dx = (p.XMAX - p.XMIN) / (double)p.NX;  // src/main.c:1126-1128
  g.dy = (p.YMAX - p.YMIN) / (double)p.NY;
  g.dz = (p.ZMAX - p.ZMIN) / (double)p.NZ;
  g.xmax_l = (double)(0 + p.NX) * g.dx + p.XMIN;  // src/read_data.c:39
  g.lx = p.XMAX - p.XMIN;
  g.hx = g.dx / 2.0; g.hy = g.dy / 2.0; g.hz = g.dz / 2.0;
  g.rsd_opz = 1.0 + p.Redshift;  // src/read_data.c:69
  g.rsd_den = 100.0 * sqrt(p.Omega_m * pow((1.0 + p.Redshift), 3.0) + 1.0 - p.Omega_m);
  g.xmin_f = (float)p.XMIN; g.ymin_f = (float)p.YMIN; g.zmin_f = (float)p.ZMIN;
  g.idx_f = (float)(1.0 / g.dx); g.idy_f = (float)(1.0 / g.dy); g.idz_f = (float)(1.0 / g.dz);
  g.rsd_f = (float)(g.rsd_opz / g.rsd_den);
  // FP32 scale error bound in cells: a few ulps of the coordinate over the cell size plus a few
  // ulps of the scale itself, times a safety factor
  double cmax = 0;
  const double c[6] = {p.XMIN, p.XMAX, p.YMIN, p.YMAX, p.ZMIN, p.ZMAX};
  for (int k = 0; k < 6; k++) cmax = fmax(cmax, fabs(c[k]));
  double dmin = fmin(g.dx, fmin(g.dy, g.dz));
  int nmax = p.NX > p.NY ? (p.NX > p.NZ ? p.NX : p.NZ) : (p.NY > p.NZ ? p.NY : p.NZ);
  double eps = ldexp(1.0, -23);
  g.margin = (float)(16.0 * eps * (2.0 * cmax / dmin + nmax + 2.0) + 1e-6);
  return g;
}

// Product of one spectrum in the bin kernels' [product][5][NK] sums: |A|^2, Re(A*B), Im(A*B), |B|^2.
int spectrum_product(int nfields, const SpecDef &sd) {
  return nfields == 1 ? 0 : (sd.x == sd.y ? (sd.x == 0 ? 0 : 3) : (sd.imag ? 2 : 1));
}

// Fields and spectra of a run (src/read_data.c:91-130, src/main.c:141-148, 214, 406-441).
static void plan_fields(capow_ctx *c) {
  const int m = c->p.Momentum;
  FieldSpec &fs = c->fs;
  memset(&fs, 0, sizeof fs);
  BinParams &bp = c->bp;
  if (c->o.spectra == CAPOW_SPEC_REFERENCE) {
    static const int tab[9][6] = {  // nfields, ea, eb, imag, mean_sub_a, shot moment
        {1, 0, 0, 0, 1, 0}, {2, 0, 1, 1, 1, 1}, {1, 1, 0, 0, 0, 2}, {2, 0, 2, 0, 1, 2}, {2, 1, 2, 1, 0, 3},
        {1, 2, 0, 0, 0, 4}, {2, 0, 3, 1, 1, 3}, {2, 1, 3, 0, 0, 4}, {2, 0, 4, 0, 1, 4}};
    fs.nfields = tab[m][0];
    fs.ea = tab[m][1];
    fs.eb = tab[m][2];
    bp.nspec = 1;
    bp.spec[0].x = 0;
    bp.spec[0].y = fs.nfields == 2 ? 1 : 0;
    bp.spec[0].imag = tab[m][3];
    bp.mean_sub_a = tab[m][4];
    c->shot_moment[0] = tab[m][5];
    c->spec_kind[0] = 0;
    c->moments = (m != 0);
  } else {
    const int mask = c->o.spectra;
    const bool needD = mask & (CAPOW_SPEC_DD | CAPOW_SPEC_DP), needP = mask & (CAPOW_SPEC_DP | CAPOW_SPEC_PP);
    int fd = -1, fp = -1;
    if (needD && needP) {
      fs.nfields = 2; fs.ea = 0; fs.eb = 1; fd = 0; fp = 1;
    } else if (needD) {
      fs.nfields = 1; fs.ea = 0; fd = 0;
    } else {
      fs.nfields = 1; fs.ea = 1; fp = 0;
    }
    bp.mean_sub_a = needD ? 1 : 0;
    int q = 0;
    if (mask & CAPOW_SPEC_DD) {
      bp.spec[q] = SpecDef{fd, fd, 0}; c->shot_moment[q] = 0; c->spec_kind[q] = CAPOW_SPEC_DD; q++;
    }
    if (mask & CAPOW_SPEC_DP) {
      bp.spec[q] = SpecDef{fd, fp, 1}; c->shot_moment[q] = 1; c->spec_kind[q] = CAPOW_SPEC_DP; q++;
    }
    if (mask & CAPOW_SPEC_PP) {
      bp.spec[q] = SpecDef{fp, fp, 0}; c->shot_moment[q] = 2; c->spec_kind[q] = CAPOW_SPEC_PP; q++;
    }
    bp.nspec = q;
    c->moments = needP;
  }
  fs.moments = c->moments;
  fs.need_v = fs.moments || c->p.LOS != 0 || fs.ea > 0 || (fs.nfields == 2 && fs.eb > 0);
  bp.pmask = 0;
  for (int q = 0; q < bp.nspec; q++) bp.pmask |= 1 << spectrum_product(fs.nfields, bp.spec[q]);
  c->nslot = fs.nfields * (c->p.DoInterlacing ? 2 : 1);
}

static void *dalloc(capow_ctx *c, size_t bytes) {
  void *p = nullptr;
  if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) return nullptr;
  c->allocs.push_back(p);
  return p;
}

extern "C" int capow_create(const capow_params *p, const capow_options *opt, capow_ctx **out) {
  if (!p || !out) return CAPOW_EINVAL;
  *out = nullptr;
  capow_options o;
  memset(&o, 0, sizeof o);
  if (opt) o = *opt;
  else o.precision = CAPOW_FP32_MIXED;
  capow_ctx *c = new (std::nothrow) capow_ctx();
  if (!c) return CAPOW_ENOMEM;
  c->p = *p;
  c->o = o;
  int rc = validate(p, &o, c->err, sizeof c->err);
  if (rc) {
    fprintf(stderr, "capow_create: %s\n", c->err);
    delete c;
    return rc;
  }
  c->prec = o.precision;
  *out = c;  // from here on capow_destroy releases partial state
  CK(c, cudaSetDevice(o.device));
  if (o.stream) {
    c->stream = (cudaStream_t)o.stream;
    c->own_stream = false;
  } else {
    CK(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->own_stream = true;
  }
  for (int k = 0; k < 4; k++) CK(c, cudaEventCreate(&c->ev[k]));
  CK(c, cudaEventCreate(&c->ev_tile[0]));
  CK(c, cudaEventCreate(&c->ev_tile[1]));
  c->g = make_geom(*p);
  if (c->prec != CAPOW_FP64 && !(c->g.margin < 0.25f))  // FP32 positions cannot resolve the cells
    FAIL(c, CAPOW_ENOTSUP, "box coordinates too large for FP32 cell positions (error margin %.3g cells); use FP64",
         (double)c->g.margin);
  plan_fields(c);
  const bool f64 = c->prec == CAPOW_FP64;
  const size_t eb = f64 ? 8 : 4;
  c->grid_elems = (size_t)c->g.main_sz;
  c->grid_base = dalloc(c, eb * c->grid_elems * c->nslot);
  c->st = (DevStats *)dalloc(c, sizeof(DevStats));
  c->dcv = (double *)dalloc(c, sizeof(double) * 4);
  c->fixed_scale = (double *)dalloc(c, sizeof(double) * 2);
  const int nk = p->NK, n2d = p->Output2D ? p->NK * p->NMU : 0;
  c->bins = (double *)dalloc(c, sizeof(double) * NPROD * 5 * nk);
  c->bins2d = (double *)dalloc(c, sizeof(double) * NPROD * (n2d ? n2d : 1));
  c->nmodes_d = (unsigned long long *)dalloc(c, sizeof(unsigned long long) * nk);
  c->nmodes2d_d = (unsigned long long *)dalloc(c, sizeof(unsigned long long) * (n2d ? n2d : 1));
  if (!c->grid_base || !c->st || !c->dcv || !c->bins || !c->bins2d || !c->nmodes_d || !c->nmodes2d_d)
    FAIL(c, CAPOW_ENOMEM, "device allocation failed (grids need %.2f GB)", eb * c->grid_elems * c->nslot / 1e9);
  CK(c, cudaMallocHost((void **)&c->h_bins, sizeof(double) * NPROD * (5 * nk + n2d)));
  CK(c, cudaMallocHost((void **)&c->h_st, sizeof(DevStats)));
  if (!f64) {
    c->tg = choose_tiles(c->g, c->nslot, c->prec == CAPOW_FP32_DETERMINISTIC);
    c->pb.counts = (unsigned *)dalloc(c, sizeof(unsigned) * c->tg.ntiles);
    c->pb.offsets = (unsigned *)dalloc(c, sizeof(unsigned) * (c->tg.ntiles + 1));
    c->pb.cursor = (unsigned *)dalloc(c, sizeof(unsigned) * c->tg.ntiles);
    c->pb.fixed_scale = c->fixed_scale;
    if (!c->pb.counts || !c->pb.offsets || !c->pb.cursor) FAIL(c, CAPOW_ENOMEM, "tile table allocation failed");
  }
  // bins: tables, exact edges, one-time mode counts
  BinParams &bp = c->bp;
  bp.nx = p->NX; bp.ny = p->NY; bp.nz = p->NZ; bp.nzc = p->NZ / 2 + 1; bp.xhalf = p->NX / 2;
  bp.nk = nk; bp.nmu = p->NMU; bp.los = p->LOS; bp.interlace = p->DoInterlacing;
  bp.odd = p->Odd_Multipoles; bp.out2d = p->Output2D; bp.nfields = c->fs.nfields;
  bp.two_pi = 2.0 * M_PI;
  bp.fx_step = (float)(1.0 / ((float)p->NX * c->g.dx));
  bin_params_kguess(bp, *p);
  if (build_bin_tables(*p, c->g, c->prec, c->bt, c->allocs, c->stream)) FAIL(c, CAPOW_ENOMEM, "bin tables");
  CK(c, cudaMemsetAsync(c->nmodes_d, 0, sizeof(unsigned long long) * nk, c->stream));
  CK(c, cudaMemsetAsync(c->nmodes2d_d, 0, sizeof(unsigned long long) * (n2d ? n2d : 1), c->stream));
  launch_mode_counts(c->stream, bp, c->bt, c->nmodes_d, c->nmodes2d_d, &c->launches);
  CK(c, cudaGetLastError());
  c->nmodes.resize(nk);
  c->nmodes2d.resize(n2d);
  CK(c, cudaMemcpyAsync(c->nmodes.data(), c->nmodes_d, sizeof(unsigned long long) * nk, cudaMemcpyDeviceToHost,
                        c->stream));
  if (n2d)
    CK(c, cudaMemcpyAsync(c->nmodes2d.data(), c->nmodes2d_d, sizeof(unsigned long long) * n2d,
                          cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  // FP32 with a power-of-two NX: the (y, z) axes first, then k_xfft_bin does the x axis together
  // with the binning (CAPOW_FFT_3D keeps the 3-D transform and k_bin). With a power-of-two NZ the z
  // axis is k_zr2c, out of place and transposed to [NX][NZ/2+1][NY], and the y axis a contiguous
  // batched cuFFT C2C; otherwise one cuFFT 2-D R2C over every x-plane, in place.
  const bool want_fused = !f64 && o.fft_path != CAPOW_FFT_3D && c->bt.twx;
  const long long yrows = (long long)c->nslot * p->NX * bp.nzc;
  const bool tr = want_fused && c->bt.twz && zr2c_supported(bp) && yrows <= 0x7fffffffLL;
  c->fused = want_fused && xbin_plan(bp, c->nslot, c->xg, tr);
  if (c->fused && tr) {
    // the transposed layout needs a second grid-sized buffer and a cuFFT workspace; when the device
    // has no room for them the context keeps the in-place 2-D cuFFT layout instead
    c->tslot = (long long)p->NX * bp.nzc * p->NY;
    void *tb = nullptr;
    int ny = p->NY;
    if (o.fft_path == CAPOW_FFT_ONE_LAUNCH && zy_supported(bp, c->bt)) {  // z and y axes in one launch
      const char *stall = getenv("CAPOW_TEST_STALL_ZY");
      c->zy_stall = stall && stall[0] == '1';
      c->zy_ctr = (unsigned *)dalloc(c, sizeof(unsigned) * zy_counter_words(bp, c->nslot));
      if (c->zy_ctr && cudaMalloc(&tb, sizeof(float2) * (size_t)c->tslot * c->nslot) == cudaSuccess) {
        c->allocs.push_back(tb);
        c->tbuf = (float2 *)tb;
        c->xtr = true;
        c->zy = true;
        c->plan_ok = true;
        return CAPOW_OK;
      }
      tb = nullptr;
    }
    if (cudaMalloc(&tb, sizeof(float2) * (size_t)c->tslot * c->nslot) == cudaSuccess) {
      if (cufftPlanMany(&c->yplan, 1, &ny, nullptr, 1, ny, nullptr, 1, ny, CUFFT_C2C, (int)yrows) == CUFFT_SUCCESS) {
        c->allocs.push_back(tb);
        c->tbuf = (float2 *)tb;
        c->xtr = true;
        c->yplan_ok = true;
        CKFFT(c, cufftSetStream(c->yplan, c->stream));
        c->plan_ok = true;  // the context is complete (c->plan is not used on this path)
        return CAPOW_OK;
      }
      cudaFree(tb);
    }
    (void)cudaGetLastError();  // clear the failed allocation
    c->fused = xbin_plan(bp, c->nslot, c->xg, false);
  }
  if (c->fused) {
    int n2[2] = {p->NY, p->NZ};
    int in2[2] = {p->NY, 2 * bp.nzc}, on2[2] = {p->NY, bp.nzc};
    CKFFT(c, cufftPlanMany(&c->plan, 2, n2, in2, 1, p->NY * 2 * bp.nzc, on2, 1, p->NY * bp.nzc, CUFFT_R2C,
                           p->NX * c->nslot));
    c->plan_ok = true;
    CKFFT(c, cufftSetStream(c->plan, c->stream));
    return CAPOW_OK;
  }
  // one batched in-place r2c plan over all painted grids (replaces the fftw_execute calls,
  // src/main.c:266-271): forward, unnormalised, padded last dimension
  int n[3] = {p->NX, p->NY, p->NZ};
  int inembed[3] = {p->NX, p->NY, 2 * bp.nzc}, onembed[3] = {p->NX, p->NY, bp.nzc};
  long long idist = (long long)c->grid_elems, odist = (long long)c->grid_elems / 2;
  if (idist > 0x7fffffffLL) {
    // cufftPlanMany takes int distances; large grids use one plan per grid instead
    CKFFT(c, cufftPlan3d(&c->plan, p->NX, p->NY, p->NZ, f64 ? CUFFT_D2Z : CUFFT_R2C));
  } else {
    CKFFT(c, cufftPlanMany(&c->plan, 3, n, inembed, 1, (int)idist, onembed, 1, (int)odist,
                           f64 ? CUFFT_D2Z : CUFFT_R2C, c->nslot));
  }
  c->plan_ok = true;
  CKFFT(c, cufftSetStream(c->plan, c->stream));
  return CAPOW_OK;
}

// A context that paints only: the grids, counters and FP32 tile buffers of capow_create, without bin
// tables, plans or FFT buffers (capow_paint and capow_power refuse it: plan_ok stays false). survey != 0
// selects the Survey rules with that many fields: 1 (the particles' w) or 2 (w, and w vlos in the
// second field); no RSD shift and no wrap, the halo slices discarded, the Survey clamps at the upper grid
// edge (Geom.los = 4, Geom.survey = 1). The survey estimator paints its FP32 grids through it, on the
// stream given in o->stream.
int create_paint_ctx(const capow_params *p, const capow_options *o, int survey, capow_ctx **out) {
  *out = nullptr;
  capow_ctx *c = new (std::nothrow) capow_ctx();
  if (!c) return CAPOW_ENOMEM;
  c->p = *p;
  c->o = *o;
  c->o.spectra = CAPOW_SPEC_REFERENCE;
  if (survey) {
    c->p.LOS = 3;
    c->p.Momentum = survey == 2 ? 1 : 0;  // fields w and w v^1
  }
  int rc = validate(&c->p, &c->o, c->err, sizeof c->err);
  if (rc) {
    delete c;
    return rc;
  }
  c->prec = o->precision;
  *out = c;
  CK(c, cudaSetDevice(o->device));
  if (o->stream) {
    c->stream = (cudaStream_t)o->stream;
  } else {
    CK(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->own_stream = true;
  }
  for (int k = 0; k < 4; k++) CK(c, cudaEventCreate(&c->ev[k]));
  CK(c, cudaEventCreate(&c->ev_tile[0]));
  CK(c, cudaEventCreate(&c->ev_tile[1]));
  c->g = make_geom(c->p);
  if (c->prec != CAPOW_FP64 && !(c->g.margin < 0.25f))
    FAIL(c, CAPOW_ENOTSUP, "box coordinates too large for FP32 cell positions (error margin %.3g cells); use FP64",
         (double)c->g.margin);
  plan_fields(c);
  if (survey) {
    c->g.los = 4;
    c->g.survey = 1;
    c->fs.need_v = survey == 2;
    c->fs.moments = 0;
    c->moments = 0;
  }
  const size_t eb = c->prec == CAPOW_FP64 ? 8 : 4;
  c->grid_elems = (size_t)c->g.main_sz;
  c->grid_base = dalloc(c, eb * c->grid_elems * c->nslot);
  c->st = (DevStats *)dalloc(c, sizeof(DevStats));
  c->dcv = (double *)dalloc(c, sizeof(double) * 4);
  c->fixed_scale = (double *)dalloc(c, sizeof(double) * 2);
  if (!c->grid_base || !c->st || !c->dcv || !c->fixed_scale)
    FAIL(c, CAPOW_ENOMEM, "device allocation failed (grids need %.2f GB)", eb * c->grid_elems * c->nslot / 1e9);
  CK(c, cudaMallocHost((void **)&c->h_st, sizeof(DevStats)));
  if (c->prec != CAPOW_FP64) {
    c->tg = choose_tiles(c->g, c->nslot, c->prec == CAPOW_FP32_DETERMINISTIC);
    c->pb.counts = (unsigned *)dalloc(c, sizeof(unsigned) * c->tg.ntiles);
    c->pb.offsets = (unsigned *)dalloc(c, sizeof(unsigned) * (c->tg.ntiles + 1));
    c->pb.cursor = (unsigned *)dalloc(c, sizeof(unsigned) * c->tg.ntiles);
    c->pb.fixed_scale = c->fixed_scale;
    if (!c->pb.counts || !c->pb.offsets || !c->pb.cursor) FAIL(c, CAPOW_ENOMEM, "tile table allocation failed");
  }
  return CAPOW_OK;
}

extern "C" int capow_abi_version(void) { return CAPOW_ABI_VERSION; }

extern "C" int capow_num_spectra(const capow_ctx *c) { return c ? c->bp.nspec : 0; }

extern "C" int64_t capow_kernel_launches(const capow_ctx *c) { return c ? c->launches : 0; }

#define CAPOW_CHUNKS 4
#define CAPOW_CHUNK_MIN_PARTICLES (1LL << 22)

static int stage_input(capow_ctx *c, const capow_particles *in, capow_particles *dev) {
  *dev = *in;
  c->nchunk = 0;
  if (in->on_device) return CAPOW_OK;
  const size_t eb = in->dtype == CAPOW_F64 ? 8 : 4;
  const void *src[5] = {in->x, in->y, in->z, in->vlos, in->w};
  const void **dst[5] = {&dev->x, &dev->y, &dev->z, &dev->vlos, &dev->w};
  // a large catalogue for the one-pass bucket paint is copied in chunks on the copy stream, so the
  // bucket pass of one chunk overlaps the copy of the next (host-to-device runs near 210 GB/s)
  const bool chunked = c->prec == CAPOW_FP32_MIXED && !c->two_pass && (long long)in->n >= CAPOW_CHUNK_MIN_PARTICLES;
  if (chunked && !c->copy_stream) {
    CK(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    for (int k = 0; k < CAPOW_CHUNKS; k++) CK(c, cudaEventCreateWithFlags(&c->chunk_ev[k], cudaEventDisableTiming));
  }
  // the set this catalogue fills is free once the paint that last read it is done (stage_free; the
  // context stream's later work, such as a queued power stage, does not hold the copy back)
  const int set = c->stage_set;
  if (!c->stage_free[set]) CK(c, cudaEventCreateWithFlags(&c->stage_free[set], cudaEventDisableTiming));
  if (chunked && c->stage_used[set]) CK(c, cudaStreamWaitEvent(c->copy_stream, c->stage_free[set], 0));
  for (int k = 0; k < 5; k++) {
    if (!src[k]) {
      *dst[k] = nullptr;
      continue;
    }
    size_t bytes = eb * in->n;
    if (c->stage_bytes[set][k] < bytes) {
      if (c->stage_used[set]) CK(c, cudaEventSynchronize(c->stage_free[set]));
      if (c->stage[set][k]) cudaFree(c->stage[set][k]);
      c->stage[set][k] = nullptr;
      c->stage_bytes[set][k] = 0;
      CK(c, cudaMalloc(&c->stage[set][k], bytes));
      c->stage_bytes[set][k] = bytes;
    }
    if (!chunked) CK(c, cudaMemcpyAsync(c->stage[set][k], src[k], bytes, cudaMemcpyHostToDevice, c->stream));
    *dst[k] = c->stage[set][k];
  }
  if (chunked) {
    const long long n = (long long)in->n;
    for (int q = 0; q < CAPOW_CHUNKS; q++) {
      const long long c0 = n * q / CAPOW_CHUNKS, c1 = n * (q + 1) / CAPOW_CHUNKS;
      for (int k = 0; k < 5; k++)
        if (src[k])
          CK(c, cudaMemcpyAsync((char *)c->stage[set][k] + eb * c0, (const char *)src[k] + eb * c0, eb * (c1 - c0),
                                cudaMemcpyHostToDevice, c->copy_stream));
      CK(c, cudaEventRecord(c->chunk_ev[q], c->copy_stream));
    }
    // everything after the bucket pass (and any repaint) also waits for the last chunk
    c->nchunk = CAPOW_CHUNKS;
  }
  c->stage_set ^= 1;
  dev->on_device = 1;
  return CAPOW_OK;
}

// After a paint of catalogue d has been queued: if d lies in a staging set, that set is free again once
// the context stream passes this point.
static int mark_stage_read(capow_ctx *c, const capow_particles &d) {
  for (int s = 0; s < 2; s++)
    if (d.x && d.x == c->stage[s][0] && c->stage_free[s]) {
      CK(c, cudaEventRecord(c->stage_free[s], c->stream));
      c->stage_used[s] = true;
    }
  return CAPOW_OK;
}

static GridPtrs grid_ptrs(capow_ctx *c) {
  GridPtrs gp;
  const size_t eb = c->prec == CAPOW_FP64 ? 8 : 4;
  for (int k = 0; k < 4; k++)
    gp.g[k] = k < c->nslot ? (void *)((char *)c->grid_base + eb * c->grid_elems * k) : nullptr;
  return gp;
}

static int ensure_records(capow_ctx *c, unsigned long long need, bool weights) {
  if (need <= c->pb.capacity && (!weights || c->pb.recw)) return CAPOW_OK;
  if (c->pb.recs) cudaFree(c->pb.recs);
  if (c->pb.recw) cudaFree(c->pb.recw);
  c->pb.recs = nullptr;
  c->pb.recw = nullptr;
  c->pb.capacity = 0;
  CK(c, cudaMalloc(&c->pb.recs, sizeof(float4) * need));
  if (weights) CK(c, cudaMalloc(&c->pb.recw, sizeof(float) * need));
  c->pb.capacity = need;
  return CAPOW_OK;
}

// Records per tile of a one-pass bucket paint of n particles.
static unsigned bucket_capacity(const capow_ctx *c, unsigned long long n) {
  const double mean = tile_dup_estimate(c->g, c->tg) * (double)n / (double)c->tg.ntiles;
  const double f = c->bucket_factor > 0.0f ? (double)c->bucket_factor : 2.0;
  return ((unsigned)(f * mean) + 64 + 31) & ~31u;
}

// The bucket records and the overflow list of a one-pass paint of up to n particles.
static int ensure_buckets(capow_ctx *c, unsigned long long n, bool weights) {
  int rc = ensure_records(c, (unsigned long long)bucket_capacity(c, n) * c->tg.ntiles, weights);
  if (rc) return rc;
  const unsigned long long ocap = n / 4 + 65536;
  if (!c->pb.ovf_count) CK(c, cudaMalloc(&c->pb.ovf_count, sizeof(unsigned)));
  if (c->pb.ovf_cap < ocap || (weights && !c->pb.ovf_w)) {
    if (c->pb.ovf_recs) cudaFree(c->pb.ovf_recs);
    if (c->pb.ovf_w) cudaFree(c->pb.ovf_w);
    if (c->pb.ovf_tile) cudaFree(c->pb.ovf_tile);
    c->pb.ovf_recs = nullptr;
    c->pb.ovf_w = nullptr;
    c->pb.ovf_tile = nullptr;
    c->pb.ovf_cap = 0;
    CK(c, cudaMalloc(&c->pb.ovf_recs, sizeof(float4) * ocap));
    CK(c, cudaMalloc(&c->pb.ovf_tile, sizeof(unsigned) * ocap));
    if (weights) CK(c, cudaMalloc(&c->pb.ovf_w, sizeof(float) * ocap));
    c->pb.ovf_cap = ocap;
  }
  return CAPOW_OK;
}


int enqueue_paint(capow_ctx *c, const capow_particles &d) {
  const long long n = (long long)d.n;
  GridPtrs gp = grid_ptrs(c);
  CK(c, cudaMemsetAsync(c->st, 0, sizeof(DevStats), c->stream));
  if (!c->quiet) CK(c, cudaEventRecord(c->ev[0], c->stream));
  if (c->prec == CAPOW_FP64) {
    CK(c, cudaMemsetAsync(c->grid_base, 0, 8 * c->grid_elems * c->nslot, c->stream));
    launch_paint64(c->stream, c->g, c->fs, d.dtype, d.x, d.y, d.z, d.vlos, d.w, n, gp, c->st, &c->launches);
  } else {
    if (!c->pb.edge_count) CK(c, cudaMalloc(&c->pb.edge_count, sizeof(unsigned)));
    if (c->pb.edge_cap < (unsigned long long)n + 1) {  // every particle could sit on an edge
      if (c->pb.edge_list) cudaFree(c->pb.edge_list);
      c->pb.edge_list = nullptr;
      c->pb.edge_cap = 0;
      CK(c, cudaMalloc(&c->pb.edge_list, sizeof(unsigned) * (n + 1)));
      c->pb.edge_cap = n + 1;
    }
    c->pb.bucket_cap = 0;
    if (c->prec == CAPOW_FP32_MIXED && !c->two_pass) {
      // bucket mode: each tile gets bucket_factor times its mean share of the records (plus slack); the
      // overflow list takes up to a quarter of the catalogue; beyond that the paint falls back to two passes
      int rc = ensure_buckets(c, (unsigned long long)n, d.w != nullptr);
      if (rc) return rc;
      c->pb.bucket_cap = bucket_capacity(c, (unsigned long long)n);
    } else {
      unsigned long long want = (unsigned long long)(tile_dup_estimate(c->g, c->tg) * 1.25 * n) + 65536;
      if (c->pb.capacity < want / 2 || (d.w && !c->pb.recw)) {
        int rc = ensure_records(c, want, d.w != nullptr);
        if (rc) return rc;
      }
    }
    PaintBufs pb = c->pb;
    pb.tile_ev0 = c->quiet ? nullptr : c->ev_tile[0];
    pb.tile_ev1 = c->quiet ? nullptr : c->ev_tile[1];
    pb.nchunk = c->nchunk;
    pb.chunk_ev = c->chunk_ev;
    if (c->nchunk > 1 && !pb.bucket_cap)  // a two-pass paint of a chunked copy: all of it first
      CK(c, cudaStreamWaitEvent(c->stream, c->chunk_ev[c->nchunk - 1], 0));
    c->tile_timed = !c->quiet;
    launch_paint32(c->stream, c->g, c->fs, c->tg, c->prec == CAPOW_FP32_DETERMINISTIC, d.dtype, d.x, d.y, d.z,
                   d.vlos, d.w, n, gp, pb, c->st, &c->launches);
  }
  CK(c, cudaGetLastError());
  if (!c->quiet) CK(c, cudaEventRecord(c->ev[1], c->stream));
  c->grids_intact = true;
  return mark_stage_read(c, d);
}

// Size the FP32 record and edge buffers for catalogues of up to nmax particles (the one-pass buckets at
// the context's bucket_factor and their overflow list, unless two_pass), so that a later enqueue_paint
// allocates nothing.
int prepare_paint_buffers(capow_ctx *c, unsigned long long nmax, bool weights) {
  if (c->prec == CAPOW_FP64) return CAPOW_OK;
  if (!c->pb.edge_count) CK(c, cudaMalloc(&c->pb.edge_count, sizeof(unsigned)));
  if (c->pb.edge_cap < nmax + 1) {
    if (c->pb.edge_list) cudaFree(c->pb.edge_list);
    c->pb.edge_list = nullptr;
    c->pb.edge_cap = 0;
    CK(c, cudaMalloc(&c->pb.edge_list, sizeof(unsigned) * (nmax + 1)));
    c->pb.edge_cap = nmax + 1;
  }
  if (c->prec == CAPOW_FP32_MIXED && !c->two_pass) return ensure_buckets(c, nmax, weights);
  const unsigned long long want = (unsigned long long)(tile_dup_estimate(c->g, c->tg) * 1.25 * nmax) + 65536;
  return ensure_records(c, want, weights);
}

int enqueue_backward_paint(capow_ctx *c) {
  // the transposed fused power stage reads the slots out of place: the forward's grids and DC values stand
  if (c->grids_intact) return CAPOW_OK;
  int rc = enqueue_paint(c, c->last);
  if (rc) return rc;
  launch_dc_prepare(c->stream, c->st, c->prec == CAPOW_FP32_DETERMINISTIC, c->nslot, c->fs.nfields,
                    c->bp.mean_sub_a, c->fixed_scale, c->dcv, &c->launches);
  CK(c, cudaGetLastError());
  return CAPOW_OK;
}

extern "C" int capow_paint(capow_ctx *c, const capow_particles *parts) {
  if (!c || !parts) return CAPOW_EINVAL;
  if (!c->plan_ok) FAIL(c, CAPOW_ESTATE, "context not fully created");
  if (parts->dtype != CAPOW_F32 && parts->dtype != CAPOW_F64) FAIL(c, CAPOW_EINVAL, "dtype must be F32 or F64");
  if (!parts->x || !parts->y || !parts->z) FAIL(c, CAPOW_EINVAL, "x, y and z are required");
  if (c->fs.need_v && !parts->vlos) FAIL(c, CAPOW_EINVAL, "vlos is required for LOS != 0 or momentum fields");
  if (parts->n >= 0xFFFFFFF0ULL) FAIL(c, CAPOW_EINVAL, "too many particles for one paint");
  if (c->pending && c->pend_paint)
    FAIL(c, CAPOW_ESTATE, "one capow_paint at most between capow_power_enqueue and capow_power_result");
  CK(c, cudaSetDevice(c->o.device));
  capow_particles d;
  int rc = stage_input(c, parts, &d);
  if (rc) return rc;
  if (!c->fs.need_v) d.vlos = nullptr;
  c->last = d;
  c->painted = true;
  c->powered = false;
  if (c->pending) c->pend_paint = true;
  return enqueue_paint(c, d);
}

// Sync, read the counters, repaint once with a larger record buffer when the tile lists
// overflowed. Returns a status for fatal conditions found by the paint.
int settle_paint(capow_ctx *c) {
  CK(c, cudaMemcpyAsync(c->h_st, c->st, sizeof(DevStats), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  if (c->h_st->overflow && c->pb.bucket_cap) {  // the overflow list filled: two passes from now on
    c->two_pass = true;
    int rc = enqueue_paint(c, c->last);
    if (rc) return rc;
    CK(c, cudaMemcpyAsync(c->h_st, c->st, sizeof(DevStats), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
  }
  if (c->h_st->overflow) {
    int rc = ensure_records(c, (unsigned long long)c->h_st->nrecords + 65536, c->last.w != nullptr);
    if (rc) return rc;
    rc = enqueue_paint(c, c->last);
    if (rc) return rc;
    CK(c, cudaMemcpyAsync(c->h_st, c->st, sizeof(DevStats), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    if (c->h_st->overflow) FAIL(c, CAPOW_ENOMEM, "tile record buffer overflow after resize");
  }
  if (c->h_st->nonfinite) FAIL(c, CAPOW_EINVAL, "non-finite particle coordinate, velocity or weight");
  if (c->h_st->fatal) FAIL(c, CAPOW_EBOUNDS, "particle out of grid bounds with LOS == 0");
  return CAPOW_OK;
}

extern "C" int capow_get_stats(capow_ctx *c, capow_stats *out) {
  if (!c || !out) return CAPOW_EINVAL;
  if (c->pending) FAIL(c, CAPOW_ESTATE, "capow_power_result of the power stage in flight first");
  if (!c->painted) FAIL(c, CAPOW_ESTATE, "capow_get_stats before capow_paint");
  int rc = CAPOW_OK;
  if (!c->powered) rc = settle_paint(c);
  if (rc != CAPOW_OK && rc != CAPOW_EBOUNDS) return rc;
  out->nread = c->h_st->nread;
  out->nout = c->h_st->nout;
  out->ngrid = c->h_st->ngrid;
  out->nsq = c->h_st->nsq;
  for (int k = 0; k < 4; k++) out->vr[k] = c->h_st->vr[k];
  out->first_out_of_box = c->h_st->fatal ? (int64_t)(~0ULL - c->h_st->fatal_inv) : -1;
  return rc;
}

extern "C" int capow_copy_grid(capow_ctx *c, int which, double *host_out) {
  if (!c || !host_out) return CAPOW_EINVAL;
  if (c->pending) FAIL(c, CAPOW_ESTATE, "capow_power_result of the power stage in flight first");
  if (!c->painted || c->powered) FAIL(c, CAPOW_ESTATE, "capow_copy_grid is valid between paint and power");
  int slot = which;
  if (c->fs.nfields == 1) {
    if (which == 2 || which == 3) FAIL(c, CAPOW_EINVAL, "field B is not painted in this run");
    slot = which == 1 ? 1 : 0;
  }
  if (!c->p.DoInterlacing && (which & 1)) FAIL(c, CAPOW_EINVAL, "no interlaced grid in this run");
  if (c->fs.nfields == 2) slot = (which & 1) ? c->fs.nfields + (which >> 1) : (which >> 1);
  if (slot >= c->nslot) FAIL(c, CAPOW_EINVAL, "grid index out of range");
  int rc = settle_paint(c);
  if (rc) return rc;
  const size_t n = c->grid_elems;
  if (c->prec == CAPOW_FP64) {
    CK(c, cudaMemcpy(host_out, (double *)c->grid_base + n * slot, 8 * n, cudaMemcpyDeviceToHost));
  } else {
    std::vector<float> tmp(n);
    CK(c, cudaMemcpy(tmp.data(), (float *)c->grid_base + n * slot, 4 * n, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; i++) host_out[i] = tmp[i];
  }
  // padding columns are not part of the FFT input; report them as zero
  for (long long r = 0; r < (long long)c->p.NX * c->p.NY; r++)
    for (long long z = c->p.NZ; z < c->g.row; z++) host_out[r * c->g.row + z] = 0.0;
  return CAPOW_OK;
}

// The kernels of capow_power (DC values, FFT, binning into c->bins); no read-back, no sync.
int enqueue_power_kernels(capow_ctx *c) {
  const bool f64 = c->prec == CAPOW_FP64;
  launch_dc_prepare(c->stream, c->st, c->prec == CAPOW_FP32_DETERMINISTIC, c->nslot, c->fs.nfields,
                    c->bp.mean_sub_a, c->fixed_scale, c->dcv, &c->launches);
  if (c->fused) {
    void *slots[4];
    if (c->xtr && c->zy) {
      launch_zy(c->stream, c->bp, c->bt, c->nslot, (const float *)c->grid_base, (long long)c->grid_elems, c->g.row,
                c->tbuf, c->tslot, c->zy_ctr, c->st, c->zy_stall, &c->launches);
      CK(c, cudaGetLastError());
      for (int k = 0; k < 4; k++) slots[k] = k < c->nslot ? (void *)(c->tbuf + c->tslot * k) : nullptr;
    } else if (c->xtr) {
      launch_zr2c(c->stream, c->bp, c->bt, c->nslot, (const float *)c->grid_base, (long long)c->grid_elems, c->g.row,
                  c->tbuf, c->tslot, &c->launches);
      CKFFT(c, cufftExecC2C(c->yplan, (cufftComplex *)c->tbuf, (cufftComplex *)c->tbuf, CUFFT_FORWARD));
      for (int k = 0; k < 4; k++) slots[k] = k < c->nslot ? (void *)(c->tbuf + c->tslot * k) : nullptr;
    } else {
      c->grids_intact = false;
      CKFFT(c, cufftExecR2C(c->plan, (cufftReal *)c->grid_base, (cufftComplex *)c->grid_base));
      GridPtrs gp = grid_ptrs(c);
      for (int k = 0; k < 4; k++) slots[k] = gp.g[k];
    }
    if (!c->quiet) CK(c, cudaEventRecord(c->ev[2], c->stream));
    const int nk = c->p.NK;
    CK(c, cudaMemsetAsync(c->bins, 0, sizeof(double) * NPROD * 5 * nk, c->stream));
    launch_xbin(c->stream, c->bp, c->bt, c->xg, slots, c->dcv, c->bins, &c->launches);
    CK(c, cudaGetLastError());
    if (!c->quiet) CK(c, cudaEventRecord(c->ev[3], c->stream));
    return CAPOW_OK;
  }
  c->grids_intact = false;  // the 3-D transform below runs in place
  if (c->grid_elems > 0x7fffffffULL) {
    const size_t eb = f64 ? 8 : 4;
    for (int s = 0; s < c->nslot; s++) {
      char *gp = (char *)c->grid_base + eb * c->grid_elems * s;
      if (f64) CKFFT(c, cufftExecD2Z(c->plan, (cufftDoubleReal *)gp, (cufftDoubleComplex *)gp));
      else CKFFT(c, cufftExecR2C(c->plan, (cufftReal *)gp, (cufftComplex *)gp));
    }
  } else {
    if (f64) CKFFT(c, cufftExecD2Z(c->plan, (cufftDoubleReal *)c->grid_base, (cufftDoubleComplex *)c->grid_base));
    else CKFFT(c, cufftExecR2C(c->plan, (cufftReal *)c->grid_base, (cufftComplex *)c->grid_base));
  }
  if (!c->quiet) CK(c, cudaEventRecord(c->ev[2], c->stream));
  const int nk = c->p.NK, n2d = c->p.Output2D ? c->p.NK * c->p.NMU : 0;
  CK(c, cudaMemsetAsync(c->bins, 0, sizeof(double) * NPROD * 5 * nk, c->stream));
  if (n2d) CK(c, cudaMemsetAsync(c->bins2d, 0, sizeof(double) * NPROD * n2d, c->stream));
  void *slots[4];
  GridPtrs gp = grid_ptrs(c);
  for (int k = 0; k < 4; k++) slots[k] = gp.g[k];
  launch_bin(c->stream, c->prec, c->bp, c->bt, slots, c->dcv, c->bins, n2d ? c->bins2d : nullptr, &c->launches);
  CK(c, cudaGetLastError());
  if (!c->quiet) CK(c, cudaEventRecord(c->ev[3], c->stream));
  return CAPOW_OK;
}

static int enqueue_power(capow_ctx *c) {
  int rc = enqueue_power_kernels(c);
  if (rc) return rc;
  const int nk = c->p.NK, n2d = c->p.Output2D ? c->p.NK * c->p.NMU : 0;
  const int np = bin_products(c->fs.nfields);
  CK(c, cudaMemcpyAsync(c->h_bins, c->bins, sizeof(double) * np * 5 * nk, cudaMemcpyDeviceToHost, c->stream));
  if (n2d)
    CK(c, cudaMemcpyAsync(c->h_bins + NPROD * 5 * nk, c->bins2d, sizeof(double) * np * n2d, cudaMemcpyDeviceToHost,
                          c->stream));
  CK(c, cudaMemcpyAsync(c->h_st, c->st, sizeof(DevStats), cudaMemcpyDeviceToHost, c->stream));
  return CAPOW_OK;
}

extern "C" int capow_power_enqueue(capow_ctx *c) {
  if (!c) return CAPOW_EINVAL;
  if (c->pending) FAIL(c, CAPOW_ESTATE, "capow_power_result of the power stage in flight first");
  if (!c->painted) FAIL(c, CAPOW_ESTATE, "capow_power before capow_paint");
  if (c->powered) FAIL(c, CAPOW_ESTATE, "grids already transformed; paint again");
  CK(c, cudaSetDevice(c->o.device));
  int rc = enqueue_power(c);
  if (rc) return rc;
  if (!c->power_ev) CK(c, cudaEventCreateWithFlags(&c->power_ev, cudaEventDisableTiming));
  CK(c, cudaEventRecord(c->power_ev, c->stream));
  c->powered = true;
  c->pending = true;
  c->pend_paint = false;
  c->pend_last = c->last;
  return CAPOW_OK;
}

extern "C" int capow_power_result(capow_ctx *c, capow_spectrum *out, int nout) {
  if (!c) return CAPOW_EINVAL;
  if (!c->pending) FAIL(c, CAPOW_ESTATE, "capow_power_result without capow_power_enqueue");
  if (nout < c->bp.nspec || !out) FAIL(c, CAPOW_EINVAL, "need room for %d spectra", c->bp.nspec);
  CK(c, cudaSetDevice(c->o.device));
  c->pending = false;
  const bool queued = c->pend_paint;  // a paint of the next catalogue runs behind this power stage
  c->pend_paint = false;
  CK(c, cudaEventSynchronize(c->power_ev));
  if (c->h_st->overflow) {  // rare: tile lists outgrew the estimate; repaint this catalogue and redo
    int rc = CAPOW_OK;
    if (c->pb.bucket_cap) c->two_pass = true;  // the bucket overflow list filled
    else rc = ensure_records(c, (unsigned long long)c->h_st->nrecords + 65536, c->pend_last.w != nullptr);
    if (rc) return rc;
    rc = enqueue_paint(c, c->pend_last);
    if (rc) return rc;
    rc = enqueue_power(c);
    if (rc) return rc;
    CK(c, cudaStreamSynchronize(c->stream));
    if (c->h_st->overflow) FAIL(c, CAPOW_ENOMEM, "tile record buffer overflow after resize");
    if (queued) {  // the queued paint ran before this repaint: paint the next catalogue again
      rc = enqueue_paint(c, c->last);
      if (rc) return rc;
    }
  }
  if (c->h_st->nonfinite) FAIL(c, CAPOW_EINVAL, "non-finite particle coordinate, velocity or weight");
  if (c->h_st->fatal) FAIL(c, CAPOW_EBOUNDS, "particle out of grid bounds with LOS == 0");
  if (c->h_st->timeout) FAIL(c, CAPOW_ETIMEOUT, "a bounded wait of the z + y transform gave up");
  fill_spectra(c, c->p, *c->h_st, c->h_bins, c->nmodes.data(), c->nmodes2d.data(), out);
  return CAPOW_OK;
}

extern "C" int capow_power(capow_ctx *c, capow_spectrum *out, int nout) {
  if (!c) return CAPOW_EINVAL;
  if (c->pending) FAIL(c, CAPOW_ESTATE, "capow_power_result of the power stage in flight first");
  if (!c->painted) FAIL(c, CAPOW_ESTATE, "capow_power before capow_paint");
  if (c->powered) FAIL(c, CAPOW_ESTATE, "grids already transformed; paint again");
  if (nout < c->bp.nspec || !out) FAIL(c, CAPOW_EINVAL, "need room for %d spectra", c->bp.nspec);
  int rc = capow_power_enqueue(c);
  if (rc) return rc;
  return capow_power_result(c, out, nout);
}

// Host side of capow_power for one catalogue: shot noise and normalisation (src/main.c:117-148,
// one rank: NTask = 1) and the raw sums of each spectrum out of the [product][5][NK] bins.
void fill_spectra(const capow_ctx *c, const capow_params &p, const DevStats &st, const double *h_bins,
                  const unsigned long long *nmodes, const unsigned long long *nmodes2d, capow_spectrum *out) {
  const double N = st.ngrid;
  const double alpha = N / ((double)p.NX * (double)p.NY * (double)p.NZ);
  const double nbar = N / ((p.XMAX - p.XMIN) * (p.YMAX - p.YMIN) * (p.ZMAX - p.ZMIN));
  const double norm = nbar * N;
  double vr[5] = {1.0, 0, 0, 0, 0};
  if (c->moments) {
    const double nsq = st.nsq / 1.0;
    for (int k = 0; k < 4; k++) vr[k + 1] = st.vr[k] / (nsq * 1.0);
  }
  const int nk = p.NK, n2d = p.Output2D ? p.NK * p.NMU : 0;
  for (int q = 0; q < c->bp.nspec; q++) {
    capow_spectrum &s = out[q];
    const int m = c->shot_moment[q];
    // product of this spectrum in the kernel's [product][5][NK] bins: |A|^2, Re(A*B), Im(A*B), |B|^2
    const int pq = spectrum_product(c->fs.nfields, c->bp.spec[q]);
    s.shot = m == 0 ? N : vr[m] * N;
    s.norm = norm;
    s.alpha = alpha;
    s.kind = c->spec_kind[q];
    s.last_bin = -1;
    for (int l = 0; l < 5; l++) {
      if (!s.pk[l]) continue;
      if ((l == 1 || l == 3) && !p.Odd_Multipoles) {
        memset(s.pk[l], 0, sizeof(double) * nk);
        continue;
      }
      memcpy(s.pk[l], h_bins + (pq * 5 + l) * nk, sizeof(double) * nk);
    }
    if (s.nmodes)
      for (int b = 0; b < nk; b++) s.nmodes[b] = (int64_t)nmodes[b];
    if (n2d && s.pk2d) memcpy(s.pk2d, h_bins + NPROD * 5 * nk + pq * n2d, sizeof(double) * n2d);
    if (n2d && s.nmodes2d)
      for (int b = 0; b < n2d; b++) s.nmodes2d[b] = (int64_t)nmodes2d[b];
  }
}

extern "C" int capow_normalise(const capow_params *p, capow_spectrum *s) {
  if (!p || !s || !s->pk[0] || !s->pk[2] || !s->pk[4] || !s->nmodes) return CAPOW_EINVAL;
  const int NK = p->NK;
  std::vector<int> fill(NK, 0);
  const double shot = s->shot, norm = s->norm;
  for (int i = 0; i < NK; i++) {  // src/main.c:1021-1033
    const double nm = (double)s->nmodes[i];
    if (s->nmodes[i] > 0 && fill[i] == 0) {
      s->pk[0][i] -= nm * shot;
      s->pk[0][i] /= nm * norm;
      s->pk[2][i] *= 5.0 / (nm * norm);
      s->pk[4][i] *= 9.0 / (nm * norm);
      if (p->Odd_Multipoles && s->pk[1] && s->pk[3]) {
        s->pk[1][i] *= 3.0 / (nm * norm);
        s->pk[3][i] *= 7.0 / (nm * norm);
      }
      fill[i] = 1;
    }
  }
  if (p->Output2D && s->pk2d && s->nmodes2d)  // :1034-1040
    for (int i = 0; i < NK * p->NMU; i++)
      if (s->nmodes2d[i] > 0) s->pk2d[i] /= (double)s->nmodes2d[i] * norm;
  s->last_bin = -1;
  for (int i = NK - 1; i >= 0; i--) {  // :1043-1056
    if (fill[i] == 1) {
      if (p->Odd_Multipoles && s->pk[1] && s->pk[3]) {
        s->pk[1][i] = 0.0;
        s->pk[3][i] = 0.0;
      }
      s->pk[0][i] = 0.0;
      s->pk[2][i] = 0.0;
      s->pk[4][i] = 0.0;
      s->nmodes[i] = 0;
      s->last_bin = i;
      break;
    }
  }
  return CAPOW_OK;
}

extern "C" int capow_stage_ms(capow_ctx *c, float *paint_ms, float *fft_ms, float *bin_ms) {
  if (!c) return CAPOW_EINVAL;
  if (c->pending) FAIL(c, CAPOW_ESTATE, "capow_power_result of the power stage in flight first");
  CK(c, cudaEventSynchronize(c->ev[3]));
  float a = 0, b = 0, d = 0;
  CK(c, cudaEventElapsedTime(&a, c->ev[0], c->ev[1]));
  CK(c, cudaEventElapsedTime(&b, c->ev[1], c->ev[2]));
  CK(c, cudaEventElapsedTime(&d, c->ev[2], c->ev[3]));
  if (paint_ms) *paint_ms = a;
  if (fft_ms) *fft_ms = b;
  if (bin_ms) *bin_ms = d;
  return CAPOW_OK;
}

extern "C" int capow_tile_kernel_ms(capow_ctx *c, float *ms, int64_t *records) {
  if (!c) return CAPOW_EINVAL;
  if (c->pending) FAIL(c, CAPOW_ESTATE, "capow_power_result of the power stage in flight first");
  if (c->prec == CAPOW_FP64 || !c->tile_timed)
    FAIL(c, CAPOW_ESTATE, "no timed FP32 tile deposit: paint an FP32 context first");
  CK(c, cudaEventSynchronize(c->ev_tile[1]));
  float t = 0.0f;
  CK(c, cudaEventElapsedTime(&t, c->ev_tile[0], c->ev_tile[1]));
  if (ms) *ms = t;
  if (records) {
    std::vector<unsigned> cnt(c->tg.ntiles);
    CK(c, cudaMemcpy(cnt.data(), c->pb.counts, sizeof(unsigned) * cnt.size(), cudaMemcpyDeviceToHost));
    long long tot = 0;
    for (unsigned v : cnt) tot += c->pb.bucket_cap ? (v < c->pb.bucket_cap ? v : c->pb.bucket_cap) : v;
    *records = tot;
  }
  return CAPOW_OK;
}

extern "C" void capow_destroy(capow_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->o.device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->plan_ok && !c->xtr) cufftDestroy(c->plan);
  if (c->yplan_ok) cufftDestroy(c->yplan);
  if (c->adj_plans) {
    cufftDestroy(c->adj_fwd);
    cufftDestroy(c->adj_inv);
  }
  if (c->adj_coef) cudaFree(c->adj_coef);
  for (int k = 0; k < 5; k++)
    if (c->adj_stage[k]) cudaFree(c->adj_stage[k]);
  for (void *p : c->allocs) cudaFree(p);
  for (int s = 0; s < 2; s++) {
    for (int k = 0; k < 5; k++)
      if (c->stage[s][k]) cudaFree(c->stage[s][k]);
    if (c->stage_free[s]) cudaEventDestroy(c->stage_free[s]);
  }
  if (c->power_ev) cudaEventDestroy(c->power_ev);
  if (c->pb.recs) cudaFree(c->pb.recs);
  if (c->pb.recw) cudaFree(c->pb.recw);
  if (c->pb.edge_list) cudaFree(c->pb.edge_list);
  if (c->pb.edge_count) cudaFree(c->pb.edge_count);
  if (c->pb.ovf_recs) cudaFree(c->pb.ovf_recs);
  if (c->pb.ovf_w) cudaFree(c->pb.ovf_w);
  if (c->pb.ovf_tile) cudaFree(c->pb.ovf_tile);
  if (c->pb.ovf_count) cudaFree(c->pb.ovf_count);
  if (c->h_bins) cudaFreeHost(c->h_bins);
  if (c->h_st) cudaFreeHost(c->h_st);
  for (int k = 0; k < 4; k++)
    if (c->ev[k]) cudaEventDestroy(c->ev[k]);
  for (int k = 0; k < 2; k++)
    if (c->ev_tile[k]) cudaEventDestroy(c->ev_tile[k]);
  if (c->copy_stream) {
    cudaStreamSynchronize(c->copy_stream);
    cudaStreamDestroy(c->copy_stream);
    for (int k = 0; k < CAPOW_CHUNKS; k++) cudaEventDestroy(c->chunk_ev[k]);
  }
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
}
