/* capow -- drop-in command-line driver for the periodic-box path, with the reference's
 * argument contract, parameter file, catalogue format, stdout summary and output files
 * (src/main.c:28-298). The work runs on one GB300 through libcapow_gpu (include/capow.h).
 *
 *   capow <ParameterFile> <DataFile> <RandomFile> <OutputFile>
 *
 * RandomFile is accepted and unused, as in the reference's periodic branch.
 * Optional environment (the reference's parser rejects unknown tags, so these are not tags):
 *   CAPOW_PRECISION = fp32 (default) | fp64 | det
 *   CAPOW_SPECTRA   = e.g. "dd,dp,pp": one paint and one set of FFTs for several spectra;
 *                     each is written to <OutputFile>.<name>
 *   CAPOW_DEVICE    = CUDA device ordinal
 * Any failure prints the reference's message and exits with status 1 (FatalError,
 * src/main.c:1298-1303). */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "capow.h"

static void banner(const char *t) {
  printf("\n%s\n", t);
  size_t n = strlen(t);
  for (size_t i = 0; i < n; i++) putchar('=');
  printf("\n");
  fflush(stdout);
}

static void die(const char *msg) {
  if (msg && *msg) printf("%s", msg);
  fflush(stdout);
  exit(1);
}

static void die_status(capow_ctx *ctx, int rc, const char *where) {
  if (rc == CAPOW_EBOUNDS) {
    printf("Task 0 has particle out of grid bounds\n");
    printf("Fatal Error at line 110 in routine read_data\n");
  } else {
    printf("%s: %s (%s)\n", where, capow_strerror(rc), ctx ? capow_last_error(ctx) : "");
  }
  fflush(stdout);
  exit(1);
}

int main(int argc, char **argv) {
  if (argc < 5) { /* src/main.c:39-47 */
    printf("Input parameters not found\n");
    printf("Call with <ParameterFile, DataFile, RandomFile, OutputFile>\n");
    fflush(stdout);
    exit(1);
  }
  banner("Reading Input Parameters and setting up CAPOW");
  capow_params p;
  char msg[8192];
  int rc = capow_read_params(argv[1], &p, msg, sizeof msg);
  if (rc != CAPOW_OK) die(msg);
  if (msg[0]) printf("%s", msg); /* warnings */
  const char *datafile = argv[2], *outfile = argv[4];

  capow_options opt;
  memset(&opt, 0, sizeof opt);
  opt.precision = CAPOW_FP32_MIXED;
  const char *pe = getenv("CAPOW_PRECISION");
  if (pe && !strcmp(pe, "fp64")) opt.precision = CAPOW_FP64;
  else if (pe && !strcmp(pe, "det")) opt.precision = CAPOW_FP32_DETERMINISTIC;
  const char *de = getenv("CAPOW_DEVICE");
  if (de) opt.device = atoi(de);
  const char *se = getenv("CAPOW_SPECTRA");
  opt.spectra = CAPOW_SPEC_REFERENCE;
  if (se && *se) {
    if (strstr(se, "dd")) opt.spectra |= CAPOW_SPEC_DD;
    if (strstr(se, "dp")) opt.spectra |= CAPOW_SPEC_DP;
    if (strstr(se, "pp")) opt.spectra |= CAPOW_SPEC_PP;
  }

  banner("Allocating grid"); /* src/main.c:61-66, create_grids prints */
  printf("Setting neighbours...\n");
  printf("Reserving memory...\n");
  fflush(stdout);
  capow_ctx *ctx = NULL;
  rc = capow_create(&p, &opt, &ctx);
  if (rc != CAPOW_OK) die_status(ctx, rc, "capow_create");
  printf("Creating redshift-distance lookup table...\n");

  banner("Reading input data and assigning to grid");
  printf("\nReading: %s\n", datafile);
  fflush(stdout);
  size_t n = 0;
  double *x, *y, *z, *v;
  rc = capow_read_catalogue(datafile, p.LOS, &n, &x, &y, &z, &v, msg, sizeof msg);
  if (rc != CAPOW_OK) die(msg);
  capow_particles parts;
  memset(&parts, 0, sizeof parts);
  parts.n = n;
  parts.dtype = CAPOW_F64;
  parts.on_device = 0;
  parts.x = x; parts.y = y; parts.z = z; parts.vlos = v; parts.w = NULL;
  rc = capow_paint(ctx, &parts);
  if (rc != CAPOW_OK) die_status(ctx, rc, "capow_paint");
  capow_stats st;
  rc = capow_get_stats(ctx, &st);
  if (rc == CAPOW_EBOUNDS && st.first_out_of_box >= 0) { /* src/read_data.c:81-84 */
    const int64_t i = st.first_out_of_box;
    printf("Task 0 has particle out of grid bounds: x=%lf, y=%lf, z=%lf\n", x[i], y[i], z[i]);
    printf("Fatal Error at line 110 in routine read_data\n");
    fflush(stdout);
    exit(1);
  }
  if (rc != CAPOW_OK) die_status(ctx, rc, "capow_paint");
  if (p.LOS == 0) printf("Task 0 read %lf particles, gridded %lf\n", st.nread, st.ngrid);
  else printf("Task 0 read %lf particles, gridded %lf (%lf out of bounds due to RSD)\n", st.nread, st.ngrid, st.nout);
  fflush(stdout);

  const int ns = capow_num_spectra(ctx);
  capow_spectrum spec[3];
  double *store = (double *)calloc((size_t)ns * (5 * p.NK + (p.Output2D ? p.NK * p.NMU : 0)), sizeof(double));
  int64_t *mstore = (int64_t *)calloc((size_t)ns * (p.NK + (p.Output2D ? p.NK * p.NMU : 0)), sizeof(int64_t));
  for (int q = 0; q < ns; q++) {
    memset(&spec[q], 0, sizeof spec[q]);
    double *base = store + (size_t)q * (5 * p.NK + (p.Output2D ? p.NK * p.NMU : 0));
    for (int l = 0; l < 5; l++) spec[q].pk[l] = base + l * p.NK;
    int64_t *mb = mstore + (size_t)q * (p.NK + (p.Output2D ? p.NK * p.NMU : 0));
    spec[q].nmodes = mb;
    if (p.Output2D) {
      spec[q].pk2d = base + 5 * p.NK;
      spec[q].nmodes2d = mb + p.NK;
    }
  }

  banner("Computing shot-noise and normalisation"); /* src/main.c:97-140 */
  const double N = st.ngrid;
  const double alpha = N / ((double)p.NX * (double)p.NY * (double)p.NZ);
  const double nbar = N / ((p.XMAX - p.XMIN) * (p.YMAX - p.YMIN) * (p.ZMAX - p.ZMIN));
  printf("mean          = %g\n", alpha);
  printf("nbar          = %g\n", nbar);
  printf("shot-noise    = %g\n", N);
  printf("normalisation = %g\n", nbar * N);
  const int moments = (opt.spectra == CAPOW_SPEC_REFERENCE) ? (p.Momentum != 0)
                                                             : ((opt.spectra & (CAPOW_SPEC_DP | CAPOW_SPEC_PP)) != 0);
  if (moments) {
    printf("vr_ave = %g\n", st.vr[0] / st.nsq);
    printf("vr2_ave = %g\n", st.vr[1] / st.nsq);
    printf("vr3_ave = %g\n", st.vr[2] / st.nsq);
    printf("vr4_ave = %g\n", st.vr[3] / st.nsq);
  }
  fflush(stdout);
  banner("Subtracting off expected density");
  banner("Fourier transforming overdensity field");
  banner("Iterating over grid cells");
  rc = capow_power(ctx, spec, ns);
  if (rc != CAPOW_OK) die_status(ctx, rc, "capow_power");

  banner("Outputting power spectra"); /* src/main.c:1004-1101 */
  for (int q = 0; q < ns; q++) {
    char name[4096];
    if (opt.spectra == CAPOW_SPEC_REFERENCE) snprintf(name, sizeof name, "%s", outfile);
    else
      snprintf(name, sizeof name, "%s.%s", outfile,
               spec[q].kind == CAPOW_SPEC_DD ? "dd" : (spec[q].kind == CAPOW_SPEC_DP ? "dp" : "pp"));
    printf("Writing multipoles to file: %s\n", name);
    if (p.Output2D) printf("Writing 2D power spectrum to file:%s_2D\n", name);
    fflush(stdout);
    capow_normalise(&p, &spec[q]);
    if (spec[q].last_bin >= 0) {
      printf("Last full bin: %d (k=%g)\n", spec[q].last_bin, capow_bin_centre(&p, spec[q].last_bin));
      fflush(stdout);
    }
    if (capow_write_output(name, &p, &spec[q]) != CAPOW_OK) {
      printf("cannot open output file: %s\n", name);
      printf("Fatal Error at line 142 in routine read_data\n");
      exit(1);
    }
  }
  banner("Cleaning up");
  capow_destroy(ctx);
  capow_free(x); capow_free(y); capow_free(z); capow_free(v);
  free(store);
  free(mstore);
  return 0;
}
