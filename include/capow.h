/* capow.h -- C ABI of libcapow_gpu, the GB300 (sm_103a) implementation of CAPOW's
 * periodic-box power-spectrum path, and of its survey estimator (capow_survey_*, below).
 *
 * The reference has no plugin interface: its periodic path is a chain of C functions
 * sharing globals (src/proto.h:25-46, src/vars.h). Each entry point below replaces one
 * link of that chain; the file:line it replaces is given beside it. Paths are relative
 * to the CAPOW source tree.
 *
 *   reference (src/main.c:28-298, periodic branch)      this library
 *   ------------------------------------------------      -----------------------------
 *   read_parameterfile / check_inputs (read_params.c)    capow_params (+ driver parser)
 *   create_grids            (main.c:1123-1251)           capow_create
 *   read_periodic_serial_ascii + add_to_grid
 *                           (read_data.c:32-179, 514-745) capow_paint
 *   shot / norm             (main.c:106-148)             capow_get_stats + capow_power
 *   mean subtraction        (main.c:211-225)             capow_power (exact DC correction)
 *   fftw_execute            (main.c:266-271)             capow_power (cuFFT)
 *   compute_periodic_power  (main.c:302-468)             capow_power
 *   output_power arithmetic (main.c:1019-1056)           capow_normalise
 *   destroy_grids           (main.c:1255-1294)           capow_destroy
 *
 * Conventions: every call returns an int status (CAPOW_OK = 0); nothing in the library
 * exits or aborts (the reference calls FatalError -> MPI_Abort, main.c:1298-1303; the
 * driver maps a nonzero status to the same message-and-exit). No torch types; plain
 * pointers and sizes only. A context is not thread-safe; all its GPU work runs on the
 * context's CUDA stream.
 */
#ifndef CAPOW_H
#define CAPOW_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Version of the structs and entry points below. 2: capow_survey_catalogue, capow_survey_stats and
 * capow_survey_objects carry the velocity fields of Momentum 1-3, and capow_backward takes 5 gradient
 * arrays per spectrum. 3: capow_power_enqueue and capow_power_result. A caller compiled against one
 * version checks capow_abi_version() at run time. */
#define CAPOW_ABI_VERSION 3
int capow_abi_version(void); /* CAPOW_ABI_VERSION of the loaded library */

/* ---------------------------------------------------------------- status codes */
#define CAPOW_OK 0
#define CAPOW_EINVAL 1   /* bad argument or parameter (read_params.c:294-428 checks) */
#define CAPOW_ENOMEM 2   /* device or host allocation failed */
#define CAPOW_ECUDA 3    /* CUDA runtime error */
#define CAPOW_EBOUNDS 4  /* LOS==0 particle outside the box: the reference aborts (read_data.c:81-85) */
#define CAPOW_ETIMEOUT 5 /* a bounded device wait gave up */
#define CAPOW_ESTATE 6   /* call out of order (e.g. capow_power before capow_paint) */
#define CAPOW_ECUFFT 7   /* cuFFT error */
#define CAPOW_ENOTSUP 8  /* combination not supported */

/* ---------------------------------------------------------------- parameters */
/* The run_parameters.dat tags that drive the periodic path (read_params.c:65-227), with the
 * reference's names and meanings. The survey tags are in capow_survey_params (below). */
typedef struct capow_params {
  int NX, NY, NZ;                           /* grid cells per axis (vars.h:79-81) */
  double XMIN, XMAX, YMIN, YMAX, ZMIN, ZMAX; /* box (vars.h:83-85) */
  int InterpOrder;                          /* 1 NN, 2 CIC, 3 TSC (vars.h:78) */
  int DoInterlacing;                        /* 0/1 (vars.h:77) */
  int NK, NMU;                              /* k bins, mu bins for the 2-D output (vars.h:88-89) */
  int Output2D, OutputLog;                  /* (vars.h:90-91) */
  double Mink, Maxk;                        /* (vars.h:92-93) */
  double Omega_m, Redshift;                 /* RSD shift factor (read_data.c:69-75) */
  int LOS;                                  /* 0 real space (mu about z), 1/2/3 RSD along x/y/z (vars.h:108) */
  int Momentum;                             /* 0..8: which fields and which spectrum (vars.h:113) */
  int Odd_Multipoles;                       /* also P1, P3 (vars.h:121) */
} capow_params;

/* numeric path */
#define CAPOW_FP64 0          /* plain double path: FP64 grids, FFT and bins */
#define CAPOW_FP32_MIXED 1    /* FP32 grids and FFT; FP64 per-bin sums, scalars, near-edge indices */
#define CAPOW_FP32_DETERMINISTIC 2 /* as FP32_MIXED with int64 fixed-point painting: bit-reproducible grids */

/* spectra selection (capow_options.spectra) */
#define CAPOW_SPEC_REFERENCE 0 /* one spectrum chosen by params.Momentum, as one reference run */
#define CAPOW_SPEC_DD 1        /* density auto (the reference's Momentum 0)                   */
#define CAPOW_SPEC_DP 2        /* density x LOS momentum, Im(D* P) (Momentum 1)                */
#define CAPOW_SPEC_PP 4        /* LOS momentum auto (Momentum 2)                               */

typedef struct capow_options {
  int precision; /* CAPOW_FP64 / CAPOW_FP32_MIXED / CAPOW_FP32_DETERMINISTIC */
  int spectra;   /* CAPOW_SPEC_REFERENCE, or an OR of CAPOW_SPEC_DD|DP|PP (one paint, one set of FFTs) */
  int device;    /* CUDA device ordinal */
  void *stream;  /* cudaStream_t to run on, or NULL for a stream owned by the context */
  int fft_path;  /* CAPOW_FFT_AUTO, CAPOW_FFT_3D or CAPOW_FFT_ONE_LAUNCH (below) */
  int reserved[7];
} capow_options;

/* FFT and binning path (capow_options.fft_path). AUTO: FP32 contexts with a power-of-two NX in
 * [16, 2048] and no 2-D output transform each x-plane over (y, z) with cuFFT and do the x axis
 * together with the binning in one kernel; everything else, or 3D, runs the full 3-D cuFFT
 * transform and a separate binning kernel. Both give the same spectra within FP32 rounding. */
#define CAPOW_FFT_AUTO 0
#define CAPOW_FFT_3D 1
/* ONE_LAUNCH: as AUTO, but where NY and NZ are powers of two (NY in [16, 2048], NZ in [32, 2048]) the
 * z and y axes run in one launch of the library's own kernel, each x-plane's z output read back from
 * L2 by its y transforms (no HBM round trip between the axes) instead of the z kernel followed by
 * cuFFT along y. Same spectra within FP32 rounding. */
#define CAPOW_FFT_ONE_LAUNCH 2

/* particle input: structure of arrays */
#define CAPOW_F32 0
#define CAPOW_F64 1
typedef struct capow_particles {
  size_t n;
  int dtype;         /* CAPOW_F32 or CAPOW_F64, applies to every array */
  int on_device;     /* 1: device pointers (resident in HBM); 0: host pointers (copied in) */
  const void *x, *y, *z; /* positions, box units */
  const void *vlos;  /* velocity along the line of sight in km/s: the vz column for LOS 0 and 3,
                        vx for 1, vy for 2 (read_data.c:65-76). May be NULL when no momentum
                        field is painted and LOS == 0. */
  const void *w;     /* per-particle weights, or NULL for w = 1 (read_data.c:60) */
} capow_particles;

/* counters of the paint pass (read_data.c:37, 78-88, 92-138) */
typedef struct capow_stats {
  double nread;   /* particles read */
  double nout;    /* outside the box after the RSD shift (LOS != 0) */
  double ngrid;   /* sum of w over accepted particles = NPERIODIC (main.c:76) */
  double nsq;     /* sum of w over all particles */
  double vr[4];   /* sum of w*v^n, n = 1..4, over all particles */
  int64_t first_out_of_box; /* LOS == 0: index of the first particle outside the box (the one the
                               reference reports before aborting, read_data.c:81-84), else -1 */
} capow_stats;

/* one spectrum. The caller owns every array; NULL arrays are skipped. */
typedef struct capow_spectrum {
  double *pk[5];       /* P0..P4, NK each (P1, P3 only when Odd_Multipoles) */
  int64_t *nmodes;     /* NK */
  double *pk2d;        /* NK*NMU when Output2D */
  int64_t *nmodes2d;   /* NK*NMU when Output2D */
  double shot, norm, alpha; /* filled by capow_power (main.c:117-148) */
  int last_bin;        /* filled by capow_normalise: the zeroed highest filled bin, or -1 */
  int kind;            /* filled by capow_power: CAPOW_SPEC_DD / DP / PP, or 0 for a reference Momentum run */
} capow_spectrum;

typedef struct capow_ctx capow_ctx;

/* create_grids (main.c:1123-1251): validates params (read_params.c:294-428 semantics),
 * allocates device grids, cuFFT plans and the k-bin threshold tables. */
int capow_create(const capow_params *p, const capow_options *opt, capow_ctx **out);

/* read_periodic_serial_ascii + add_to_grid (read_data.c:32-179, 514-745): RSD shift,
 * bounds count, mass assignment of every requested field with the interlaced copy, the
 * halo fold and the velocity moments, for one catalogue. Replaces any previous paint. */
int capow_paint(capow_ctx *ctx, const capow_particles *parts);

/* Size of the fixed device scratch of capow_paint_noalloc: 64 MiB per device. With lazy module
 * loading (the CUDA default since 12.2) it is reserved when the first call on a device loads it;
 * with CUDA_MODULE_LOADING=EAGER every process that links the library holds it on every device it
 * uses from context creation on. */
#define CAPOW_NOALLOC_SCRATCH_BYTES (64ull << 20)

/* capow_paint without any device allocation. No counterpart in the reference (its paint runs on
 * the host). capow_paint grows its scratch buffers with the catalogue (cudaMalloc, and cudaFree,
 * which waits for the whole device); a caller that paints between the steps of a simulation
 * running on the same GPU, with the rest of the device held by its own memory pool, can neither
 * allocate nor stall the simulation's streams. This call paints the same grids, with the same
 * statistics, as capow_paint on an FP32 context, taking its scratch from one fixed device array of
 * CAPOW_NOALLOC_SCRATCH_BYTES instead; it calls no cudaMalloc, cudaFree or allocating library.
 * - particles must be device-resident (on_device = 1); FP64 contexts return CAPOW_ENOTSUP;
 * - n beyond what the array holds for this grid (worst-case tile records per particle) returns
 *   CAPOW_EINVAL before any device work; capow_last_error names the largest n that fits
 *   (about 500000 unweighted particles for a 512^3 TSC grid);
 * - the first call on each device looks up the array's address and loads its code: make it
 *   before any stream capture begins;
 * - every call on a device shares the one array: calls that overlap on the GPU (other streams,
 *   other contexts on the same device) race; order them, e.g. on one stream.
 * - every input array must be device memory of the context's device (CAPOW_EINVAL otherwise).
 * capow_get_stats, capow_copy_grid and capow_power then work as after capow_paint and allocate
 * nothing (the worst-case bound keeps the record lists from overflowing, so the repaint that
 * capow_power does after an overflow cannot happen). capow_backward is not covered: it creates its 3-D
 * plans and coefficient buffers on first use and, when capow_power transformed the grids in place,
 * repaints the catalogue through capow_paint's buffers, so a caller that cannot allocate must not
 * call it on a context painted this way. capow_tile_kernel_ms returns
 * CAPOW_ESTATE after this paint (its tile launch is not timed). */
int capow_paint_noalloc(capow_ctx *ctx, const capow_particles *parts);

/* counters from the last paint (ends with a stream synchronisation). The counters are filled
 * even when the status is CAPOW_EBOUNDS, so the caller can report the offending particle. */
int capow_get_stats(capow_ctx *ctx, capow_stats *out);

/* mean subtraction, FFT and compute_periodic_power (main.c:211-225, 266-271, 302-468):
 * raw bin sums (not normalised) for each requested spectrum, in the order DD, DP, PP
 * (or the single Momentum spectrum). `out` has room for `nout` spectra. Ends with a
 * stream synchronisation and the device-to-host copy of the bins. */
int capow_power(capow_ctx *ctx, capow_spectrum *out, int nout);

/* capow_power in two halves, for a stream of catalogues through one context: capow_power_enqueue queues
 * the power stage and the read-back of its sums and returns at once; capow_power_result waits for them
 * and fills `out` as capow_power does (CAPOW_ESTATE without a pending power stage). Between the two the
 * context takes one capow_paint of the next catalogue: its kernels run after this power stage, and a
 * host catalogue's copy into the other of two staging buffers starts at once, so that it overlaps this
 * power stage. Every other call on the context returns CAPOW_ESTATE until capow_power_result. If this
 * catalogue's tile lists overflowed, capow_power_result repaints it, redoes the power stage and paints
 * the queued catalogue again. capow_power is capow_power_enqueue followed by capow_power_result. */
int capow_power_enqueue(capow_ctx *ctx);
int capow_power_result(capow_ctx *ctx, capow_spectrum *out, int nout);

/* gradients of a loss with respect to every particle of the last paint (capow_backward) */
typedef struct capow_grads {
  int on_device;     /* 1: device pointers; 0: host pointers (copied out at the end of the call) */
  int dtype;         /* CAPOW_F32 / CAPOW_F64: must match the painted particles */
  void *dx, *dy, *dz; /* dL/d(position), n each; NULL to skip one */
  void *dvlos;       /* dL/d(v_los): through the RSD shift (LOS != 0) */
  void *dw;          /* dL/d(weight), including its effect on NGRID (norm, shot, mean subtraction) */
} capow_grads;

/* Adjoint of capow_power + capow_normalise for every spectrum of the context (any Momentum, or the
 * dd / dp / pp selection): given dL/dP_l(k) of the normalised multipoles, 5 entries per spectrum in the
 * order capow_power returns them (dL_dP[5 q + l] = double[NK] for spectrum q and multipole l = 0..4;
 * NULL for a multipole the loss does not use; one spectrum: 5 entries, as before), writes dL/dx, dL/dy,
 * dL/dz, dL/dv_los and dL/dw of every particle of the last capow_paint. The velocity enters through the
 * RSD shift (LOS != 0), the momentum fields' w v^e deposits and the shot noise's sum w v^m / sum w. The
 * reference has no adjoint; this inverts read_data.c:32-179, 514-745 and main.c:106-148, 211-225,
 * 266-271, 302-468, 1019-1056: the painted grids (still in place after the transposed power stage,
 * repainted after one that transformed them in place), full 3-D R2C, per-mode dL/dF of both fields, Hermitian
 * completion, C2R, and the transposed deposits with the weight derivatives. Call after capow_power; it
 * leaves the grids holding dL/dgrid, so paint again before the next capow_power. The output_power rule
 * that zeroes the highest filled bin makes that bin's gradient zero. */
int capow_backward(capow_ctx *ctx, const double *const *dL_dP, const capow_grads *out);

/* ---------------------------------------------------------------- batched mocks */
/* One mock of a batch: its own parameters (box, grid, order, ...) and device-resident catalogue.
 * `out` has room for capow_num_spectra entries (the spectra selected by the batch's options);
 * the call fills them as capow_power does (raw sums, shot, norm, alpha, Nmodes) and sets status. */
typedef struct capow_mock {
  capow_params params;
  capow_particles parts; /* on_device = 1 */
  capow_spectrum *out;
  int status;            /* CAPOW_OK or this mock's error (e.g. CAPOW_EBOUNDS) */
} capow_mock;

#define CAPOW_BATCH_GRAPH 1    /* capture the whole batch as one CUDA graph and launch it once */
#define CAPOW_BATCH_AUTOTUNE 2 /* time candidate tile shapes of the FP32 paint per grid shape first */

/* Run many independent mocks (the reference runs one per process, main.c:28-298). Mocks with the
 * same grid shape (NX, NY, NZ, interlacing, LOS, Momentum, odd multipoles) share grids, plans and
 * record buffers whatever their boxes, orders and k bins; every mock is enqueued on one stream with
 * no host synchronisation and read back once. Output2D is not supported here. Returns CAPOW_OK when
 * the batch ran; per-mock errors are in mocks[i].status.
 * The device state of the batch (contexts, tables, outputs and, with CAPOW_BATCH_GRAPH, the
 * instantiated graph) is kept for the next call: a call with the same signature (parameters,
 * particle counts and array kinds of every mock, options and flags) only launches, the graph as it
 * is or updated in place when the particle arrays moved. A call with another signature replaces it;
 * capow_batch_release frees it. Calls are serialised by the library. */
int capow_batch(capow_mock *mocks, int nmocks, const capow_options *opt, int flags);

/* Free the device state capow_batch keeps between calls. No reference counterpart. */
void capow_batch_release(void);

/* output_power arithmetic (main.c:1019-1056) in place on one spectrum's raw sums. Host only. */
int capow_normalise(const capow_params *p, capow_spectrum *s);

/* number of spectra capow_power will produce for this context */
int capow_num_spectra(const capow_ctx *ctx);

/* copy one painted real grid to the host in the reference's padded layout
 * [NX][NY][2*(NZ/2+1)] as float64 (after the halo fold, before mean subtraction).
 * which: 0 field A, 1 field A interlaced, 2 field B, 3 field B interlaced. Valid between
 * capow_paint and capow_power. For parity tests. */
int capow_copy_grid(capow_ctx *ctx, int which, double *host_out);

/* device milliseconds of the last paint, FFT and bin stages (CUDA events on the context stream) */
int capow_stage_ms(capow_ctx *ctx, float *paint_ms, float *fft_ms, float *bin_ms);

/* device milliseconds of the tile-deposit kernel of the last FP32 paint (CUDA events on the context
 * stream, around that one launch) and the number of particle records it deposited (each record is
 * one particle's footprint within one tile). For roofline measurements; no reference counterpart.
 * CAPOW_ESTATE on FP64 contexts or before an FP32 paint. */
int capow_tile_kernel_ms(capow_ctx *ctx, float *ms, int64_t *records);

/* total number of kernels this library launched on the context since creation */
int64_t capow_kernel_launches(const capow_ctx *ctx);

void capow_destroy(capow_ctx *ctx);

/* ---------------------------------------------------------------- survey estimator */
/* The reference's other estimator (Periodic 0, Survey 1; src/main.c:77-95, 149-204, 226-258, 279-288,
 * 472-967): data and random catalogues in a non-periodic box seen from an observer, FKP weights,
 * the random counts subtracted in the painted grid, and the Yamamoto multipoles, each an FFT of the
 * density weighted by functions of the line of sight r^ to every cell, crossed with the monopole
 * field F0. params.Momentum selects, as in the reference:
 *   0  the density multipoles;
 *   1  the velocity multipoles: the data's w pv painted (no randoms), FKP weights from pverr,
 *      shot = sum w^2 pv^2, norm = alpha sum w_r^2 nbar_r;
 *   2  the density-velocity cross multipoles: the density (data minus alpha randoms) and the data's
 *      w_pv pv, crossed with F0 and F0_mom (main.c:876-887), shot = sum w w_pv pv,
 *      norm = sqrt(alpha sum w_r^2 nbar_r * sum w_pv,r^2 nbar_r). The reference itself crashes here
 *      (its survey paint writes the momentum grid create_grids leaves unallocated for Momentum 2,
 *      main.c:1198); this library computes what that code describes;
 *   3  the cross multipoles with shot = sum w^2 pv^2 and the reference's norm, which is zero (the
 *      randoms' w_pv sum is taken for Momentum 2 only, main.c:164-165), so the normalised spectra
 *      are infinite as the reference's are.
 *
 *   reference                                             this library
 *   ----------------------------------------------------   -----------------------------------
 *   read_survey_serial_ascii (read_data.c:184-361)         capow_read_survey (host)
 *   compute_fkp              (read_data.c:450-466)         capow_survey_power (on the GPU)
 *   sums, alpha, shot, norm  (main.c:149-204)              capow_survey_power (on the GPU)
 *   assign_survey_data       (read_data.c:471-494, 514-745) capow_survey_power (on the GPU)
 *   compute_survey_power + assign_survey_power
 *                            (main.c:472-967)              capow_survey_power (on the GPU)
 *   output_power arithmetic  (main.c:1019-1056)            capow_normalise
 *
 * The reference forms P_l from the Cartesian products of r^ (1, 3, 6, 10 and 15 FFTs for l = 0..4);
 * this library uses the equivalent real solid harmonics of r^ (1, 3, 5, 7 and 9 FFTs), and adds the
 * one cell the two forms treat differently (a cell whose corner is exactly the observer, where the
 * reference's r^ products are 0) as a closed-form term. Same multipoles within FP64 rounding. */

/* the survey tags of run_parameters.dat (read_params.c:145-222, vars.h) */
typedef struct capow_survey_params {
  int Periodic, Survey;                 /* estimator switches: Periodic 0, Survey 1 selects this one */
  int Coord_Type;                       /* 0: Cartesian x y z; 1: RA, Dec (degrees), z; 2: RA, Dec (radians), z */
  double X_Origin, Y_Origin, Z_Origin;  /* observer position, box units */
  double REDMININ, REDMAXIN;            /* redshift cut of the reader */
  long long NOBJ_Max;                   /* capacity of the reference's object arrays */
  int NBAR_Column;                      /* > 0: number density from the catalogue (its 5th number);
                                           < 0: the reference's compute_nbar (capow_survey_nbar) */
  double SkyArea;
  int FKP_Column;                       /* < 0: FKP weights w *= 1/(1 + nbar FKP_Pk) (main.c:89-94) */
  double FKP_Pk, FKP_Pk_mom, FKP_Pk_cross;
} capow_survey_params;

/* One catalogue as the reference holds it after reading (struct survey_data, vars.h:136-142: float
 * fields). dtype CAPOW_F32 reproduces the reference's float storage of the FKP weights bit for bit;
 * CAPOW_F64 keeps every per-object value in double. */
typedef struct capow_survey_catalogue {
  size_t n;
  int dtype;            /* CAPOW_F32 or CAPOW_F64, every array */
  int on_device;        /* 1: device pointers; 0: host pointers (copied in) */
  const void *x, *y, *z; /* Cartesian positions, box units */
  const void *w;        /* weights as read (before FKP) */
  const void *nbar;     /* number density */
  const void *pv, *pverr; /* peculiar velocity and its error (Momentum 1-3; NULL for Momentum 0). The
                             randoms' pv is not used. */
} capow_survey_catalogue;

/* counters of one survey evaluation */
typedef struct capow_survey_stats {
  double ngrid_data, ngrid_rand; /* assign_survey_data's "gridded" sums: accepted objects counted w/w
                                    (read_data.c:474-491; the randoms' sum divided by -alpha; Momentum 1
                                    counts w/(pv w) and paints no randoms) */
  double data_nbw, data_nbwsq, data_nbsqwsq; /* sum w, w^2, w^2 nbar over the data (main.c:151-156) */
  double rand_nbw, rand_nbwsq, rand_nbsqwsq; /* the same over the randoms, the last two after the alpha
                                                scaling of main.c:170-171 */
  double data_vr, data_vrsq, data_nbsqwsq_pv; /* sum w w_pv pv, w^2 pv^2, w_pv^2 nbar (Momentum 1-3) */
  double rand_nbsqwsq_pv;                     /* sum w_pv^2 nbar over the randoms (Momentum 2) */
} capow_survey_stats;

typedef struct capow_survey_ctx capow_survey_ctx;

/* create_grids for a survey run (main.c:1123-1251): params as for capow_create (LOS is not used;
 * Momentum 0 to 3; Output2D gives the reference's all-zero 2-D bins), the observer and FKP settings
 * from sv. Precision CAPOW_FP64 or CAPOW_FP32_MIXED (FP32 grids and FFTs, FP64 sums and bins);
 * fft_path is ignored. Allocates, per painted field (two for Momentum 2, 3), the painted grid and its
 * interlaced copy, as many work grids for the FFTs, and a complex F0 grid. Momentum 2 and 3 need the
 * FKP weights (FKP_Column < 0): the reference leaves w_pv unset otherwise (CAPOW_EINVAL). */
int capow_survey_create(const capow_params *p, const capow_survey_params *sv, const capow_options *opt,
                        capow_survey_ctx **out);

/* One survey evaluation: FKP weights (when FKP_Column < 0), the weight sums, alpha = sum w_d / sum w_r,
 * the data painted with weight w and the randoms with -alpha w into the same grid(s), then every
 * multipole (P1, P3 only with Odd_Multipoles). Momentum 1 paints only the data's w pv (its auto spectrum;
 * shot sum w^2 pv^2); Momentum 2 and 3 also paint the data's w_pv pv and cross it with the density (shot
 * sum w w_pv pv or sum w^2 pv^2, norm sqrt(rand_nbsqwsq rand_nbsqwsq_pv): 0 for Momentum 3, as in the
 * reference, whose Momentum 3 output is therefore infinite). Fills out's raw sums, Nmodes, shot, norm and alpha as
 * capow_power does (normalise with capow_normalise); st may be NULL. Ends with a stream
 * synchronisation. CAPOW_EINVAL for a non-finite coordinate, weight, number density or velocity. */
int capow_survey_power(capow_survey_ctx *ctx, const capow_survey_catalogue *data, const capow_survey_catalogue *rand,
                       capow_spectrum *out, capow_survey_stats *st);

/* a painted grid of the last evaluation, as float64 in the reference's padded layout [NX][NY][2*(NZ/2+1)]:
 * which = stencil * fields + field, field 0 the density (data minus alpha randoms; Momentum 1: the data's
 * w pv) and, for Momentum 2 and 3, field 1 the data's w_pv pv; stencil 1 the interlaced copy. For parity
 * tests. */
int capow_survey_copy_grid(capow_survey_ctx *ctx, int which, double *host_out);

/* device milliseconds of the last evaluation: weights, sums and painting; the multipole FFTs and
 * binning. And the number of FFT sets it ran (1 + 5 + 9, or 25 with odd multipoles). */
int capow_survey_stage_ms(capow_survey_ctx *ctx, float *paint_ms, float *multipole_ms, int *fft_sets);

int64_t capow_survey_kernel_launches(const capow_survey_ctx *ctx);
const char *capow_survey_last_error(const capow_survey_ctx *ctx);
void capow_survey_destroy(capow_survey_ctx *ctx);

/* ---------------------------------------------------------------- host-side file formats */

/* read_parameterfile + check_inputs (read_params.c:30-428): parse a run_parameters.dat with
 * the same 41 mandatory tags, `%` comments, duplicate/missing-tag errors and range checks.
 * On failure returns CAPOW_EINVAL (CAPOW_ENOTSUP for Periodic 0) and writes the reference's
 * message text into msg. Warnings the reference prints are also appended to msg on success. */
int capow_read_params(const char *path, capow_params *out, char *msg, size_t msglen);

/* the periodic reader's parse loop (read_data.c:50-76): `x y z vx vy vz` per line, `#` lines
 * skipped, malformed lines fatal. Returns malloc'd float64 arrays (free with capow_free);
 * vlos holds the column LOS selects. */
int capow_read_catalogue(const char *path, int los, size_t *n, double **x, double **y, double **z, double **vlos,
                         char *msg, size_t msglen);
void capow_free(void *p);

/* Binary catalogues (no reference counterpart; the reference reads ASCII only). A file that starts
 * with the 8 bytes "CAPOWSOA" holds a 32-byte little-endian header -- magic, uint32 version (1),
 * uint32 dtype (0 float32, 1 float64), uint64 n, uint32 ncols (6), uint32 reserved -- then the six
 * columns x, y, z, vx, vy, vz, each n values. capow_read_catalogue_soa reads x, y, z and the column
 * LOS selects into one host allocation, page-locked where a device is present (x is its base: free
 * with capow_free_host), and reports
 * their dtype (CAPOW_F32 / CAPOW_F64). The driver reads such a DataFile instead of parsing text. */
int capow_is_soa_catalogue(const char *path);
int capow_read_catalogue_soa(const char *path, int los, size_t *n, int *dtype, void **x, void **y, void **z,
                             void **vlos, char *msg, size_t msglen);
void capow_free_host(void *p);

/* read_parameterfile + check_inputs for either estimator: as capow_read_params, but a survey run
 * (Periodic 0) is accepted and the survey tags are returned in sv (Periodic and Survey included). */
int capow_read_survey_params(const char *path, capow_params *out, capow_survey_params *sv, char *msg, size_t msglen);

/* One survey catalogue as read_survey_serial_ascii (read_data.c:184-361) keeps it: the reference's float
 * fields of every object that passed the redshift cut, in file order. */
typedef struct capow_survey_objects {
  size_t n;                 /* objects kept (NKEEP) */
  unsigned long long nread; /* catalogue lines read (NREAD) */
  float *x, *y, *z;         /* Cartesian positions (converted from RA, Dec, z for Coord_Type 1, 2) */
  float *w, *nbar, *redshift;
  float *pv, *pverr;        /* Momentum != 0: c zmod ln10 logdist / (1 + zmod) and the same of the error
                               (read_data.c:308-316, zmod the redshift's second-order distance factor);
                               the data's 7th and 8th numbers, the randoms' 7th (their pv is 0: unused) */
  double lo[3], hi[3];      /* the "X, Y, Z" ranges the reference prints: min and max of the kept objects'
                               coordinates, starting from 1e-30 and -1e30 (read_data.c:192-194, 344-349) */
  double redmin, redmax;    /* min and max redshift of the kept objects (read_data.c:327-328) */
  char *log;                /* what the reference prints while reading: the "Read N objects, kept K" progress
                               lines and the objects skipped for zero weight (Coord_Type 1, 2) */
} capow_survey_objects;

/* read_survey_serial_ascii: `#` lines at the top skipped; per line 12 numbers for data (x y z w nbar
 * ..., the reader keeps the 5th as nbar, read_data.c:244-250) or 8 for randoms; Coord_Type 0 takes the
 * redshift from the distance |x| through the reference's 10000-point redshift-distance table
 * (main.c:1233-1248: a natural cubic spline of z(r)); objects outside [REDMININ, REDMAXIN] are
 * dropped; an object outside the grid less the interpolation margin is fatal (read_data.c:293-299).
 * Errors (CAPOW_EINVAL) carry the reference's message in msg. Free with capow_survey_objects_free. */
int capow_read_survey(const char *path, const capow_params *p, const capow_survey_params *sv, int randoms,
                      capow_survey_objects *out, char *msg, size_t msglen);
void capow_survey_objects_free(capow_survey_objects *o);

/* compute_nbar (read_data.c:385-446) for NBAR_Column < 0, after both catalogues are read (their nbar
 * fields are overwritten): counts per redshift bin (ceil((REDMAXIN - REDMININ) / 0.002) bins over the
 * kept objects' redshift range) over the volume of the bin's shell of SkyArea square degrees, a natural
 * cubic spline through the bin centres, and every object's nbar from it. As in the reference the counts
 * come from the redshifts of the first NDATA randoms (:401-405); more data than randoms is CAPOW_EINVAL
 * (the reference reads objects it never filled). *log receives the reference's printed lines (malloc'd,
 * free with capow_free). */
int capow_survey_nbar(const capow_params *p, const capow_survey_params *sv, capow_survey_objects *data,
                      capow_survey_objects *rand, char **log, char *msg, size_t msglen);

/* output_power's file format (main.c:1058-1101), plus `<path>_2D` when Output2D. */
int capow_write_output(const char *path, const capow_params *p, const capow_spectrum *s);

/* centre of k bin i as the output file prints it (main.c:1070-1075) */
double capow_bin_centre(const capow_params *p, int i);

const char *capow_strerror(int status);

/* text of the last error recorded on this context (e.g. the failing CUDA call) */
const char *capow_last_error(const capow_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif /* CAPOW_H */
