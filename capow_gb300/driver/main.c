/* capow -- drop-in command-line driver for the periodic-box and survey paths, with the reference's
 * argument contract, parameter file, catalogue format, stdout summary and output files
 * (src/main.c:28-298). The work runs on one GB300 through libcapow_gpu (include/capow.h).
 *
 *   capow <ParameterFile> <DataFile> <RandomFile> <OutputFile>
 *
 * Periodic 1 reads DataFile only (RandomFile is accepted and unused, as in the reference's periodic
 * branch); Periodic 0 with Survey 1 runs the survey estimator on DataFile and RandomFile.
 * Optional environment (the reference's parser rejects unknown tags, so these are not tags):
 *   CAPOW_PRECISION = fp32 (default) | fp64 | det
 *   CAPOW_SPECTRA   = e.g. "dd,dp,pp": one paint and one set of FFTs for several spectra;
 *                     each is written to <OutputFile>.<name>
 *   CAPOW_DEVICE    = CUDA device ordinal
 *   CAPOW_TIMING    = 1: wall-clock phases of a periodic run on stderr
 * A periodic DataFile that starts with "CAPOWSOA" is read as binary columns (capow_read_catalogue_soa)
 * instead of text. Any failure prints the reference's message and exits with status 1 (FatalError,
 * src/main.c:1298-1303). */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "capow.h"

static void banner(const char *t) {
  printf("\n%s\n", t);
  size_t n = strlen(t);
  for (size_t i = 0; i < n; i++) putchar('=');
  printf("\n");
  fflush(stdout);
}

/* CAPOW_TIMING=1: wall-clock phases of a periodic run on stderr (stdout stays the reference's) */
enum { T_START, T_CREATE, T_READ, T_POWER, T_END, T_N };
static double g_t[T_N];

static void stamp(int k) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  g_t[k] = ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static void report_times(void) {
  const char *e = getenv("CAPOW_TIMING");
  if (!e || e[0] != '1') return;
  fprintf(stderr,
          "capow timing (s): params+create %.4f read %.4f paint+power %.4f output+cleanup %.4f total %.4f\n",
          g_t[T_CREATE] - g_t[T_START], g_t[T_READ] - g_t[T_CREATE], g_t[T_POWER] - g_t[T_READ],
          g_t[T_END] - g_t[T_POWER], g_t[T_END] - g_t[T_START]);
}

static double value_at(const void *a, int dtype, int64_t i) {
  return dtype == CAPOW_F64 ? ((const double *)a)[i] : (double)((const float *)a)[i];
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

/* output_power's part of main (src/main.c:1004-1101) for one spectrum */
static void write_spectrum(const capow_params *p, capow_spectrum *s, const char *name) {
  printf("Writing multipoles to file: %s\n", name);
  if (p->Output2D) printf("Writing 2D power spectrum to file:%s_2D\n", name);
  fflush(stdout);
  capow_normalise(p, s);
  if (s->last_bin >= 0) {
    printf("Last full bin: %d (k=%g)\n", s->last_bin, capow_bin_centre(p, s->last_bin));
    fflush(stdout);
  }
  if (capow_write_output(name, p, s) != CAPOW_OK) {
    printf("cannot open output file: %s\n", name);
    printf("Fatal Error at line 142 in routine read_data\n");
    exit(1);
  }
}

/* read_survey_serial_ascii's stdout (src/read_data.c:207-210, 229-233, 343-349) around one read */
static void read_one(const capow_params *p, const capow_survey_params *sv, const char *path, int randoms,
                     capow_survey_objects *o) {
  char msg[8192];
  printf("Reading: %s\n", path);
  fflush(stdout);
  int rc = capow_read_survey(path, p, sv, randoms, o, msg, sizeof msg);
  if (o->log) printf("%s", o->log);
  if (rc != CAPOW_OK) die(msg);
  printf("Have %llu objects\n", (unsigned long long)o->n);
  printf("%12.6lf <   X  < %12.6lf\n", o->lo[0], o->hi[0]);
  printf("%12.6lf <   Y  < %12.6lf\n", o->lo[1], o->hi[1]);
  printf("%12.6lf <   Z  < %12.6lf\n", o->lo[2], o->hi[2]);
  fflush(stdout);
}

/* The survey branch of main (src/main.c:77-95, 149-204, 226-258, 279-298): the stdout lines of
 * compute_survey_power's Cartesian products (src/main.c:497-760) are printed as the reference prints
 * them; the library computes the same multipoles through solid harmonics. */
static int run_survey(const capow_params *p, const capow_survey_params *sv, const char *datafile,
                      const char *randfile, const char *outfile) {
  capow_options opt;
  memset(&opt, 0, sizeof opt);
  opt.precision = CAPOW_FP32_MIXED;
  const char *pe = getenv("CAPOW_PRECISION");
  if (pe && !strcmp(pe, "fp64")) opt.precision = CAPOW_FP64;
  else if (pe && !strcmp(pe, "det")) die("CAPOW_PRECISION=det is not provided for the survey estimator\n");
  const char *de = getenv("CAPOW_DEVICE");
  if (de) opt.device = atoi(de);

  banner("Allocating grid");
  printf("Setting neighbours...\n");
  printf("Reserving memory...\n");
  fflush(stdout);
  capow_survey_ctx *ctx = NULL;
  int rc = capow_survey_create(p, sv, &opt, &ctx);
  if (rc != CAPOW_OK) {
    printf("capow_survey_create: %s (%s)\n", capow_strerror(rc), ctx ? capow_survey_last_error(ctx) : "");
    fflush(stdout);
    exit(1);
  }
  printf("Creating redshift-distance lookup table...\n");

  banner("Reading input data and assigning to grid");
  capow_survey_objects data, rand;
  read_one(p, sv, datafile, 0, &data);
  read_one(p, sv, randfile, 1, &rand);
  if (sv->NBAR_Column < 0) { /* compute_nbar, src/main.c:88 */
    char *nlog = NULL;
    char msg[1024];
    rc = capow_survey_nbar(p, sv, &data, &rand, &nlog, msg, sizeof msg);
    if (nlog) printf("%s", nlog);
    capow_free(nlog);
    if (rc != CAPOW_OK) die(msg);
  }
  if (sv->FKP_Column < 0) printf("Computing FKP Weights...\n");
  fflush(stdout);

  const int nk = p->NK, n2 = p->Output2D ? p->NK * p->NMU : 0;
  double *store = (double *)calloc((size_t)(5 * nk + n2), sizeof(double));
  int64_t *mstore = (int64_t *)calloc((size_t)(nk + n2), sizeof(int64_t));
  capow_spectrum spec;
  memset(&spec, 0, sizeof spec);
  for (int l = 0; l < 5; l++) spec.pk[l] = store + l * nk;
  spec.nmodes = mstore;
  if (n2) {
    spec.pk2d = store + 5 * nk;
    spec.nmodes2d = mstore + nk;
  }
  capow_survey_catalogue dc = {data.n, CAPOW_F32, 0, data.x, data.y, data.z, data.w, data.nbar, data.pv, data.pverr};
  capow_survey_catalogue rc_ = {rand.n, CAPOW_F32, 0, rand.x, rand.y, rand.z, rand.w, rand.nbar, rand.pv, rand.pverr};
  capow_survey_stats st;
  rc = capow_survey_power(ctx, &dc, &rc_, &spec, &st);
  if (rc != CAPOW_OK) {
    printf("capow_survey_power: %s (%s)\n", capow_strerror(rc), capow_survey_last_error(ctx));
    fflush(stdout);
    exit(1);
  }
  printf("Task 0 has %llu objects, gridded %lf\n", (unsigned long long)data.n, st.ngrid_data);

  banner("Computing shot-noise and normalisation"); /* src/main.c:189-203 */
  if (p->Momentum == 0) {
    printf("alpha = %g\n", spec.alpha);
    printf("shot-noise [data, randoms]    = %g, %g\n", st.data_nbwsq, st.rand_nbwsq);
    printf("normalisation [data, randoms] = %g, %g\n", st.data_nbsqwsq, st.rand_nbsqwsq);
  } else if (p->Momentum == 1) {
    printf("shot-noise [data]    = %g \n", st.data_vrsq);
    printf("normalisation [data, randoms] = %g, %g\n", st.data_nbsqwsq, st.rand_nbsqwsq);
  } else {
    printf("alpha = %g\n", spec.alpha);
    printf("shot-noise    = %g\n", st.data_vr);
    printf("normalisation = %g\n", spec.norm);
  }
  fflush(stdout);
  banner("Subtracting off expected density");
  if (p->Momentum != 1) /* src/main.c:229: Momentum 1 assigns no randoms */
    printf("Task 0 has %llu objects, gridded %lf\n", (unsigned long long)rand.n, st.ngrid_rand);

  const int step = p->Odd_Multipoles ? 1 : 2;
  for (int l = 0; l <= 4; l += step) {
    static const char *const title[5] = {"monopole", "dipole", "quadrupole", "octopole", "hexadecapole"};
    static const char *const rule[5] = {"===============================================",
                                        "=================================================",
                                        "=================================================",
                                        "=================================================",
                                        "==================================================="};
    printf("\nFourier transforming %s overdensity field\n%s\n", title[l], rule[l]);
    if (l == 1)
      for (int i = 0; i < 3; i++) printf("Indices: %d\n", i);
    if (l == 2)
      for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++) printf("Indices: %d %d\n", i, j);
    if (l == 3) /* src/main.c:648-657 */
      for (int i = 0; i < 3; i++)
        for (int j = i; j < (i == 0 ? i + 2 : i + 1); j++)
          for (int k = (j != i ? 2 : 0); k < 3; k++) printf("Indices: %d %d %d\n", i, j, k);
    if (l == 4) /* src/main.c:709-730 */
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          int klo = 0, khi = 3;
          if (j != i) {
            if (i == 1) klo = 2;
            else if (i == 2) {
              if (j == 1) continue;
              klo = 1;
              khi = 2;
            } else klo = j;
          }
          for (int k = klo; k < khi; k++) printf("Indices: %d %d %d\n", i, j, k);
        }
  }
  fflush(stdout);

  banner("Outputting power spectra");
  write_spectrum(p, &spec, outfile);
  banner("Cleaning up");
  capow_survey_destroy(ctx);
  capow_survey_objects_free(&data);
  capow_survey_objects_free(&rand);
  free(store);
  free(mstore);
  return 0;
}

int main(int argc, char **argv) {
  stamp(T_START);
  if (capow_abi_version() != CAPOW_ABI_VERSION) {
    printf("libcapow_gpu has ABI version %d, this driver was built for %d\n", capow_abi_version(), CAPOW_ABI_VERSION);
    fflush(stdout);
    exit(1);
  }
  if (argc < 5) { /* src/main.c:39-47 */
    printf("Input parameters not found\n");
    printf("Call with <ParameterFile, DataFile, RandomFile, OutputFile>\n");
    fflush(stdout);
    exit(1);
  }
  banner("Reading Input Parameters and setting up CAPOW");
  capow_params p;
  capow_survey_params sv;
  char msg[8192];
  int rc = capow_read_survey_params(argv[1], &p, &sv, msg, sizeof msg);
  if (rc != CAPOW_OK) die(msg);
  if (msg[0]) printf("%s", msg); /* warnings */
  const char *datafile = argv[2], *outfile = argv[4];
  if (!sv.Periodic) {
    if (!sv.Survey) die("\nERROR: neither Periodic nor Survey is set.\n\n");
    return run_survey(&p, &sv, datafile, argv[3], outfile);
  }

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
  stamp(T_CREATE);

  banner("Reading input data and assigning to grid");
  printf("\nReading: %s\n", datafile);
  fflush(stdout);
  size_t n = 0;
  void *x = NULL, *y = NULL, *z = NULL, *v = NULL;
  int dtype = CAPOW_F64;
  const int soa = capow_is_soa_catalogue(datafile); /* binary columns instead of text */
  if (soa) {
    rc = capow_read_catalogue_soa(datafile, p.LOS, &n, &dtype, &x, &y, &z, &v, msg, sizeof msg);
  } else {
    double *ax = NULL, *ay = NULL, *az = NULL, *av = NULL;
    rc = capow_read_catalogue(datafile, p.LOS, &n, &ax, &ay, &az, &av, msg, sizeof msg);
    x = ax; y = ay; z = az; v = av;
  }
  if (rc != CAPOW_OK) die(msg);
  stamp(T_READ);
  capow_particles parts;
  memset(&parts, 0, sizeof parts);
  parts.n = n;
  parts.dtype = dtype;
  parts.on_device = 0;
  parts.x = x; parts.y = y; parts.z = z; parts.vlos = v; parts.w = NULL;
  rc = capow_paint(ctx, &parts);
  if (rc != CAPOW_OK) die_status(ctx, rc, "capow_paint");
  capow_stats st;
  rc = capow_get_stats(ctx, &st);
  if (rc == CAPOW_EBOUNDS && st.first_out_of_box >= 0) { /* src/read_data.c:81-84 */
    const int64_t i = st.first_out_of_box;
    printf("Task 0 has particle out of grid bounds: x=%lf, y=%lf, z=%lf\n", value_at(x, dtype, i),
           value_at(y, dtype, i), value_at(z, dtype, i));
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
  stamp(T_POWER);

  banner("Outputting power spectra"); /* src/main.c:1004-1101 */
  for (int q = 0; q < ns; q++) {
    char name[4096];
    if (opt.spectra == CAPOW_SPEC_REFERENCE) snprintf(name, sizeof name, "%s", outfile);
    else
      snprintf(name, sizeof name, "%s.%s", outfile,
               spec[q].kind == CAPOW_SPEC_DD ? "dd" : (spec[q].kind == CAPOW_SPEC_DP ? "dp" : "pp"));
    write_spectrum(&p, &spec[q], name);
  }
  banner("Cleaning up");
  capow_destroy(ctx);
  if (soa) {
    capow_free_host(x);
  } else {
    capow_free(x); capow_free(y); capow_free(z); capow_free(v);
  }
  free(store);
  free(mstore);
  stamp(T_END);
  report_times();
  return 0;
}
