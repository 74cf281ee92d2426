/* CPU oracle for the CAPOW periodic power-spectrum path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference algorithm,
 * used by tests/ as the checker, by __graft_entry__.smoke() as the checker and by
 * bench.py as the CPU baseline. The product (capow_gb300/) never links, loads or
 * calls it. Every function cites the reference file:line it restates (paths are
 * relative to the CAPOW source tree, e.g. src/read_data.c).
 *
 * All arithmetic is double precision in the reference's own operation order, built
 * with -ffp-contract=off so results are bit-identical to the reference compiled for
 * x86-64 (no FMA) when particles are processed in the same order.
 */
#ifndef CAPOW_ORACLE_H
#define CAPOW_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int nx, ny, nz;                           /* NX NY NZ            (src/vars.h:79-81) */
  double xmin, xmax, ymin, ymax, zmin, zmax; /* box                 (src/vars.h:83-85) */
  int interp_order;                         /* 1 NN, 2 CIC, 3 TSC  (src/vars.h:78) */
  int do_interlacing;                       /*                     (src/vars.h:77) */
  int los;                                  /* 0 real space, 1/2/3 = x/y/z RSD (src/vars.h:108) */
  double omega_m, redshift;                 /*                     (src/vars.h:102-103) */
  int nk, nmu, output_2d, output_log, odd_multipoles;
  double mink, maxk;                        /*                     (src/vars.h:88-93, 121) */
} orc_params;

typedef struct {
  double nread;  /* lines read                      (src/read_data.c:78) */
  double nout;   /* out of bounds after RSD         (src/read_data.c:81-88) */
  double ngrid;  /* sum of w over accepted particles (src/read_data.c:92-126) */
  double npv;    /* same for the momentum grid      */
  double nsq, vr_ave, vr2_ave, vr3_ave, vr4_ave; /* sums over all lines (src/read_data.c:132-138) */
  int fatal;     /* 1 if LOS==0 saw an out-of-box particle (src/read_data.c:82-84) */
} orc_stats;

/* doubles per grid, including the InterpOrder halo slices (src/main.c:1131-1135) */
int64_t orc_grid_doubles(const orc_params *p);
/* doubles in one padded x-slice: 2*NY*(NZ/2+1) (src/main.c:1132) */
int64_t orc_slice_doubles(const orc_params *p);

/* src/read_data.c:514-745: deposit w*vr of one particle; returns w if accepted else 0 */
double orc_add_to_grid(const orc_params *p, double x, double y, double z, double w, double vr, double *density);

/* src/read_data.c:32-179 without file parsing: RSD shift, bounds count, Momentum
 * dispatch into up to four grids (NULL = not allocated), moments, then the halo fold.
 * x..vz are the six catalogue columns; w may be NULL (w = 1, src/read_data.c:60). */
int orc_paint(const orc_params *p, int momentum, int64_t n, const double *x, const double *y, const double *z,
              const double *vx, const double *vy, const double *vz, const double *w, double *ddg,
              double *ddg_interlace, double *ddg_mom, double *ddg_mom_interlace, orc_stats *st);

/* src/main.c:106-148: alpha, shot and norm for a periodic run */
void orc_shot_norm(const orc_params *p, int momentum, const orc_stats *st, double *alpha, double *shot,
                   double *norm);

/* src/main.c:211-225 */
void orc_subtract_mean(const orc_params *p, int momentum, double alpha, double *ddg, double *ddg_interlace);

/* src/main.c:266-271 (FFT of each allocated grid, oracle FFT in place of FFTW) */
void orc_fft_grids(const orc_params *p, int momentum, double *ddg, double *ddg_interlace, double *ddg_mom,
                   double *ddg_mom_interlace);

/* src/main.c:302-468: raw bin sums. pk has 5 arrays of NK (P0..P4; P1/P3 only filled
 * when odd_multipoles), nmodes NK; pk2d/nmodes2d NK*NMU (may be NULL when !output_2d). */
void orc_compute_power(const orc_params *p, int momentum, const double *ddg, const double *ddg_interlace,
                       const double *ddg_mom, const double *ddg_mom_interlace, double *pk0, double *pk1,
                       double *pk2, double *pk3, double *pk4, int *nmodes, double *pk2d, int *nmodes2d);

/* src/main.c:1019-1056: normalise in place, zero the last filled bin; returns its index (-1 if none) */
int orc_normalise(const orc_params *p, double shot, double norm, double *pk0, double *pk1, double *pk2,
                  double *pk3, double *pk4, int *nmodes, double *pk2d, const int *nmodes2d);

/* the k-bin of one |k| value, src/main.c:369-373 (exposed for tests) */
int orc_kbin(const orc_params *p, double fktot);

/* ---- survey mode (Periodic 0, Survey 1), density (Momentum 0) */
typedef struct {
  double x_origin, y_origin, z_origin; /* observer position (X_Origin, ...) */
} orc_survey;

/* add_to_grid with the Survey branches (src/read_data.c:514-745) */
double orc_survey_add(const orc_params *p, double x, double y, double z, double w, double vr, double *density);

/* assign_survey_data (src/read_data.c:471-494) for every Momentum. The object fields are the reference's
 * floats, passed as doubles (exact). Momentum 1: w * prefactor pv into ddg (and, half a cell up, ddg_i),
 * NGRID += add_to_grid / (float)(pv w); otherwise: prefactor w into ddg, NGRID += add_to_grid / w, and for
 * data with Momentum 2, 3: w_pv * prefactor pv into ddg_m (ddg_mi). wpv and pv may be NULL for Momentum 0.
 * Returns NGRID. */
double orc_survey_assign(const orc_params *p, int momentum, int is_data, int64_t n, const double *x, const double *y,
                         const double *z, const double *w, const double *wpv, const double *pv, double prefactor,
                         double *ddg, double *ddg_i, double *ddg_m, double *ddg_mi);

/* compute_survey_power + assign_survey_power (src/main.c:472-967): raw bin sums of the Yamamoto multipoles
 * from the painted grids; Momentum 2, 3 also transform the momentum grids and bin the cross terms with F0 and
 * F0_mom (ddg_m, ddg_mi NULL otherwise); the oracle FFT in place of FFTW */
void orc_survey_power(const orc_params *p, const orc_survey *sp, int momentum, const double *ddg,
                      const double *ddg_interlace, const double *ddg_m, const double *ddg_mi, double *pk0,
                      double *pk1, double *pk2, double *pk3, double *pk4, int *nmodes);

/* the redshift of comoving distance r from the table create_grids builds (src/main.c:1233-1248,
 * comoving_distance src/read_data.c:365-380), through the GSL stand-ins (orc_gsl.c) */
double orc_survey_redshift(double omega_m, double r);
/* the comoving distance of redshift z from the same table (dist_spline, src/main.c:1246-1247) */
double orc_survey_distance(double omega_m, double z);
/* a natural cubic spline through (x[i], y[i]), i < n, at t (gsl_interp_cspline through the stand-ins;
 * compute_nbar's nbar_spline, src/read_data.c:428-438) */
double orc_cspline_eval(int n, const double *x, const double *y, double t);

#ifdef __cplusplus
}
#endif
#endif
