/* Output files in the reference's format (src/main.c:1058-1101): a multipole file with a
 * `# shot`, `# norm` and column header then one %g row per k bin, and, with Output2D, a
 * `_2D` file with one row per (k, mu) bin. Kept byte-compatible so existing readers of
 * CAPOW output work unchanged. */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "capow.h"

static double kcentre(const capow_params *p, int i) {
  const double binwidth = (p->Maxk - p->Mink) / (double)p->NK; /* src/main.c:305 */
  if (p->OutputLog) return pow(10.0, p->Mink + ((float)i + 0.5) * binwidth);
  return p->Mink + ((float)i + 0.5) * binwidth;
}

double capow_bin_centre(const capow_params *p, int i) { return kcentre(p, i); }

int capow_write_output(const char *path, const capow_params *p, const capow_spectrum *s) {
  if (!path || !p || !s || !s->pk[0] || !s->pk[2] || !s->pk[4] || !s->nmodes) return CAPOW_EINVAL;
  FILE *f = fopen(path, "w");
  if (!f) return CAPOW_EINVAL;
  const int odd = p->Odd_Multipoles && s->pk[1] && s->pk[3];
  fprintf(f, "# shot = %g\n", s->shot / s->norm);
  fprintf(f, "# norm = %g\n", s->norm);
  fprintf(f, odd ? "# k  pk0  pk1  pk2  pk3  pk4  Nmodes\n" : "# k  pk0  pk2  pk4  Nmodes\n");
  for (int i = 0; i < p->NK; i++) {
    const double kp = kcentre(p, i);
    if (odd)
      fprintf(f, "%g %g %g %g %g %g %d\n", kp, s->pk[0][i], s->pk[1][i], s->pk[2][i], s->pk[3][i], s->pk[4][i],
              (int)s->nmodes[i]);
    else
      fprintf(f, "%g %g %g %g %d\n", kp, s->pk[0][i], s->pk[2][i], s->pk[4][i], (int)s->nmodes[i]);
  }
  fclose(f);
  if (p->Output2D && s->pk2d && s->nmodes2d) {
    char name[4096];
    snprintf(name, sizeof name, "%s_2D", path);
    FILE *g = fopen(name, "w");
    if (!g) return CAPOW_EINVAL;
    fprintf(g, "# shot = %g\n", s->shot / s->norm);
    fprintf(g, "# norm = %g\n", s->norm);
    fprintf(g, "# k, mu, pk, Nmodes\n");
    for (int i = 0; i < p->NK; i++) {
      const double kp = kcentre(p, i);
      for (int j = 0; j < p->NMU; j++) {
        const double mup = 2.0 * ((float)j + 0.5) / p->NMU - 1.0;
        fprintf(g, "%g %g %g %d\n", kp, mup, s->pk2d[i * p->NMU + j], (int)s->nmodes2d[i * p->NMU + j]);
      }
    }
    fclose(g);
  }
  return CAPOW_OK;
}
