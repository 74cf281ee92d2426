/* Single-rank MPI / FFTW3(-MPI) / GSL stand-ins plus raw-state dump hooks.
 *
 * TEST INFRASTRUCTURE ONLY. Linked with the UNMODIFIED reference sources
 * (src/main.c, src/read_data.c, src/read_params.c, src/vars.c) into
 * oracle/_ref/capow_ref by oracle/Makefile.ref. Nothing in the product links it.
 *
 * Dump hooks (environment variables), used to pull full-precision state out of the
 * unmodified reference program:
 *   CAPOW_REF_DUMP=<file>   at MPI_Finalize (main.c:295) write NK, every scalar that
 *                           passed through MPI_Allreduce (main.c:108-114: NPERIODIC,
 *                           nsq, vr_ave..vr4_ave), and the raw bin sums Pk0..Pk4,
 *                           Nmodes (and the 2-D bins) that compute_periodic_power
 *                           (main.c:302-468) left in the globals, as %.17g text.
 *   CAPOW_REF_GRIDS=<prefix> at the first MPI_Allreduce (i.e. right after
 *                           read_periodic_serial_ascii returned, halo already folded,
 *                           before mean subtraction) write the first NX padded slices
 *                           of ddg, ddg_interlace, ddg_mom, ddg_mom_interlace as raw
 *                           float64 to <prefix>.<name>.bin.
 */
#include "vars.h"
#include "../orc_fft.h"

#include <stdint.h>

/* ------------------------------------------------------------------ MPI */
static double g_allreduce[64];
static int g_nallreduce = 0;
static int g_grids_dumped = 0;

static size_t type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_DOUBLE: return sizeof(double);
    case MPI_INT: return sizeof(int);
    case MPI_UNSIGNED_LONG_LONG: return sizeof(unsigned long long);
  }
  return 1;
}

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Comm_rank(MPI_Comm c, int *rank) { (void)c; *rank = 0; return 0; }
int MPI_Comm_size(MPI_Comm c, int *size) { (void)c; *size = 1; return 0; }
int MPI_Abort(MPI_Comm c, int code) { (void)c; fflush(stdout); exit(code); }

static void dump_grid(const char *prefix, const char *name, const double *g) {
  if (!g) return;
  char path[4096];
  snprintf(path, sizeof path, "%s.%s.bin", prefix, name);
  FILE *f = fopen(path, "wb");
  if (!f) return;
  fwrite(g, sizeof(double), (size_t)(Local_nx * alloc_slice), f);
  fclose(f);
}

int MPI_Allreduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
  (void)op; (void)c;
  if (!g_grids_dumped) {
    g_grids_dumped = 1;
    const char *prefix = getenv("CAPOW_REF_GRIDS");
    if (prefix && *prefix) {
      dump_grid(prefix, "ddg", ddg);
      dump_grid(prefix, "ddg_interlace", ddg_interlace);
      dump_grid(prefix, "ddg_mom", ddg_mom);
      dump_grid(prefix, "ddg_mom_interlace", ddg_mom_interlace);
    }
  }
  if (t == MPI_DOUBLE && count == 1 && g_nallreduce < 64) g_allreduce[g_nallreduce++] = *(const double *)s;
  memcpy(r, s, (size_t)count * type_size(t));
  return 0;
}

int MPI_Reduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c) {
  (void)op; (void)root; (void)c;
  memcpy(r, s, (size_t)count * type_size(t));
  return 0;
}

int MPI_Allgather(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, MPI_Comm c) {
  (void)rc; (void)rt; (void)c;
  memcpy(r, s, (size_t)sc * type_size(st));
  return 0;
}

int MPI_Sendrecv(const void *s, int sc, MPI_Datatype st, int dest, int stag, void *r, int rc, MPI_Datatype rt,
                 int src, int rtag, MPI_Comm c, MPI_Status *status) {
  (void)stag; (void)rc; (void)rt; (void)rtag; (void)c; (void)status;
  if (src == MPI_PROC_NULL || dest == MPI_PROC_NULL) return 0; /* nothing arrives */
  memmove(r, s, (size_t)sc * type_size(st));
  return 0;
}

static void dump_vec_d(FILE *f, const char *name, const double *v, long n) {
  fprintf(f, "%s", name);
  for (long i = 0; i < n; i++) fprintf(f, " %.17g", v ? v[i] : 0.0);
  fprintf(f, "\n");
}

static void dump_vec_i(FILE *f, const char *name, const int *v, long n) {
  fprintf(f, "%s", name);
  for (long i = 0; i < n; i++) fprintf(f, " %d", v ? v[i] : 0);
  fprintf(f, "\n");
}

int MPI_Finalize(void) {
  const char *path = getenv("CAPOW_REF_DUMP");
  if (path && *path && Pk0) {
    FILE *f = fopen(path, "w");
    if (f) {
      fprintf(f, "NK %d\n", NK);
      fprintf(f, "NMU %d\n", NMU);
      fprintf(f, "binwidth %.17g\n", binwidth);
      dump_vec_d(f, "allreduce", g_allreduce, g_nallreduce);
      dump_vec_d(f, "Pk0", Pk0, NK);
      dump_vec_d(f, "Pk1", Pk1, NK);
      dump_vec_d(f, "Pk2", Pk2, NK);
      dump_vec_d(f, "Pk3", Pk3, NK);
      dump_vec_d(f, "Pk4", Pk4, NK);
      dump_vec_i(f, "Nmodes", Nmodes, NK);
      if (Output2D) {
        dump_vec_d(f, "Pk_2D", Pk_2D, (long)NK * NMU);
        dump_vec_i(f, "Nmodes_2D", Nmodes_2D, (long)NK * NMU);
      }
      fclose(f);
    }
  }
  fflush(stdout);
  return 0;
}

/* ------------------------------------------------------------------ FFTW */
struct capow_shim_plan {
  int n0, n1, n2;
  double *data;
};

void fftw_mpi_init(void) {}

ptrdiff_t fftw_mpi_local_size_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, MPI_Comm comm, ptrdiff_t *local_n0,
                                 ptrdiff_t *local_0_start) {
  (void)comm;
  *local_n0 = n0;
  *local_0_start = 0;
  return n0 * n1 * n2;
}

fftw_plan fftw_mpi_plan_dft_r2c_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, double *in, fftw_complex *out,
                                   MPI_Comm comm, unsigned flags) {
  (void)out; (void)comm; (void)flags;
  fftw_plan p = (fftw_plan)malloc(sizeof *p);
  p->n0 = (int)n0;
  p->n1 = (int)n1;
  p->n2 = (int)n2;
  p->data = in;
  return p;
}

void fftw_execute(const fftw_plan p) { orc_fft_r2c_3d_inplace(p->n0, p->n1, p->n2, p->data); }

void fftw_destroy_plan(fftw_plan p) { free(p); }

/* ------------------------------------------------------------------ GSL: oracle/orc_gsl.c */
