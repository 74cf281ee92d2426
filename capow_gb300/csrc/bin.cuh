// Binning-stage interfaces (bin.cu) and the host-side threshold construction.
#pragma once
#include <vector>

#include "common.cuh"

#define CAPOW_MAX_SPEC 3

// One spectrum: power = Re or Im of conj(X) * Y for X, Y in {field A = 0, field B = 1}
// (src/main.c:432-441: |F|^2, Im(F* P) as dkr*dki_mom - dki*dkr_mom, Re(F* P)).
struct SpecDef {
  int x, y;   // field index
  int imag;   // 1: imaginary part
};

// Device tables for one grid geometry. All "f" quantities follow src/main.c:335-352, 382-389.
struct BinTables {
  // exact squared frequencies, fl(f*f), for the reference's s = (fx*fx + fy*fy) + fz*fz
  double *fx2d, *fy2d, *fz2d;
  float *fx2f, *fy2f, *fz2f;
  double *fxd, *fyd, *fzd;  // signed frequencies (mu numerator, 2-D bins)
  float *fxf, *fyf, *fzf;
  // deconvolution factors sinc^(-2p) per axis and interlacing phases e^{i pi f d} per axis
  double *cxd, *cyd, *czd;
  float *cxf, *cyf, *czf;
  double2 *exd, *eyd, *ezd;
  float2 *exf, *eyf, *ezf;
  // merged k-bin edges E[0..NK] in s (bin b iff E[b] <= s < E[b+1]) and FP32 safe edges
  double *E;
  float *Elo, *Ehi;  // E[b]*(1+eps), E[b]*(1-eps) rounded outward/inward: safe FP32 tests
  float2 *twx;       // exp(-2 pi i q / NX), q < NX (fused x-axis FFT; power-of-two NX only)
  float2 *twy;       // exp(-2 pi i q / NY), q < NY (y pass of the one-launch z + y transform; power-of-two NY)
  // z-axis pass of the fused path (power-of-two NZ >= 32 only): exp(-2 pi i q / M), q < M = NZ/2,
  // for the M-point complex DFT, and exp(-2 pi i k / NZ), k <= M, for its real-input split
  float2 *twz, *tpz;
};

// Geometry of the fused x-axis FFT + binning pass (k_xfft_bin): blocks of `ncol` columns of the
// (y, z)-transformed grids, `kc` consecutive "inner" indices of one "outer" index in each of the
// nslot grids. Layout [NX][outer][inner]: tr = 0, [NX][NY][NZ/2+1] (outer ky, inner kz, after the
// cuFFT 2-D transform); tr = 1, [NX][NZ/2+1][NY] (outer kz, inner ky, after k_zr2c and the y pass).
struct XbinGeo {
  int log2n, ncol, log2ncol, kc, log2kc, nkb, nblocks;
  int tr, n_outer, n_inner;
  int nbc;  // copies of the CTA's bins in shared memory (warps spread over them), a power of two
};

struct BinParams {
  int nx, ny, nz, nzc, xhalf;
  int nk, nmu, los, interlace, odd, out2d;
  int nspec, nfields;
  SpecDef spec[CAPOW_MAX_SPEC];
  int mean_sub_a;           // field A had the mean subtracted (DC correction)
  int pmask;                // products the spectra read (bit q: |A|^2, Re A*B, Im A*B, |B|^2)
  double two_pi;
  float fx_step;            // x frequency spacing 1/((float)NX*dx) (src/main.c:329), for per-column x ranges
  // first guess of a mode's bin from FP32 s = |f|^2 for linear bins: (int)(sqrtf(s) * kscale + koff), i.e.
  // (2 pi |f| - Mink) / binwidth (src/main.c:369-373); lg = 1 (log bins) bisects instead. The guess only
  // starts the walk over the safe FP32 edges, so its rounding does not matter.
  float kscale, koff;
  int lg;
};

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

// Fill kscale, koff and lg of bp for a run's k binning.
void bin_params_kguess(BinParams &bp, const capow_params &p);

// Host: exact k-bin of one |k|^2 value s, following src/main.c:355, 369-375.
// Returns -1 (below), 0..NK-1, or NK (above or beyond Nyquist).
int host_kbin_of_s(double s, double mink, double binwidth, int nk, int output_log, double min_nyquist);

// Host: build and upload tables. Returns 0 on success.
int build_bin_tables(const capow_params &p, const Geom &g, int precision, BinTables &t, std::vector<void *> &allocs,
                     cudaStream_t s);

// The same tables appended to a host blob (offsets in place of pointers), for many grids in one
// allocation; relocate_bin_tables rebases them on the blob's device copy.
int build_bin_tables_packed(const capow_params &p, const Geom &g, int precision, BinTables &t,
                            std::vector<unsigned char> &blob);
void relocate_bin_tables(BinTables &t, const void *base);

// launchers
void launch_mode_counts(cudaStream_t s, const BinParams &bp, const BinTables &t, unsigned long long *nmodes,
                        unsigned long long *nmodes2d, long long *launches);
void launch_bin(cudaStream_t s, int precision, const BinParams &bp, const BinTables &t, void *const slots[4],
                const double *dcv, double *bins, double *bins2d, long long *launches);
// products accumulated by the bin kernel: 1 for one field, 4 (|A|^2, Re A*B, Im A*B, |B|^2) for two
int bin_products(int nfields);

// Fused path: plan for a grid (returns false when NX is not a power of two in [16, 2048], the 2-D
// bins are requested, or the shared-memory bins do not fit), and its launcher. The slots hold the
// (y, z)-transformed grids, x in real space, in the layout xg.tr names.
bool xbin_plan(const BinParams &bp, int nslot, XbinGeo &xg, bool transposed);
// The z-axis pass of the transposed fused layout: true when NZ is a power of two in [32, 2048].
bool zr2c_supported(const BinParams &bp);
// The z pass and the y-axis C2C of the transposed layout in one launch (power-of-two NZ and NY, the
// tables' twy present). ctr: 2 + nslot * NX device counters, cleared by the launcher; a wait that gave
// up sets st->timeout. stall != 0 (tests of the timeout path only) makes every wait run out.
struct DevStats;
bool zy_supported(const BinParams &bp, const BinTables &t);
size_t zy_counter_words(const BinParams &bp, int nslot);
void launch_zy(cudaStream_t s, const BinParams &bp, const BinTables &t, int nslot, const float *in, long long in_slot,
               int row, float2 *out, long long out_slot, unsigned *ctr, DevStats *st, int stall,
               long long *launches);
// Real-to-complex DFT along z of every row of every painted grid (in: [NX][NY][row] floats, slot
// stride in_slot floats), out of place into out (slot stride out_slot complex) as [NX][NZ/2+1][NY].
// The same z pass with the survey estimator's cell weights h_lm(r^) applied to the input as it is read (vx,
// vy, vz: the cell-corner offsets from the observer per axis).
void launch_zr2c_weighted(cudaStream_t s, const BinParams &bp, const BinTables &t, int nslot, const float *in,
                          long long in_slot, int row, float2 *out, long long out_slot, const float *vx,
                          const float *vy, const float *vz, int l, int m, long long *launches);
void launch_zr2c(cudaStream_t s, const BinParams &bp, const BinTables &t, int nslot, const float *in,
                 long long in_slot, int row, float2 *out, long long out_slot, long long *launches);
void launch_xbin(cudaStream_t s, const BinParams &bp, const BinTables &t, const XbinGeo &xg, void *const slots[4],
                 const double *dcv, double *bins, long long *launches);
// DC corrections: dcv[slot] = painted sum (minus NGRID for mean-subtracted field A slots)
void launch_dc_prepare(cudaStream_t s, const void *st, int deterministic, int nslot, int nfields, int mean_sub_a,
                       const double *fixed_scale, double *dcv, long long *launches);
