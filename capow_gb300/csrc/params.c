/* run_parameters.dat reader with the reference's file format, tag table, error messages
 * and checks (src/read_params.c:30-290 read_parameterfile, :294-428 check_inputs).
 *
 * The tag set and the message texts are kept identical on purpose: the same parameter file
 * must drive both the reference and this library, and scripts that parse the reference's
 * stdout keep working. capow_read_params serves the periodic path and refuses a survey run;
 * capow_read_survey_params accepts both and also returns the survey tags. */
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "capow.h"

enum { T_FLOAT = 1, T_INT = 3 };

typedef struct {
  const char *name;
  int type;
  int slot; /* index into the int or double scratch arrays */
} tagdef;

/* slots */
enum {
  I_NumFilesInParallel, I_NX, I_NY, I_NZ, I_DoInterlacing, I_InterpOrder, I_NK, I_NMU, I_Output2D, I_OutputLog,
  I_Periodic, I_LOS, I_Survey, I_Momentum, I_NOBJ_Max, I_Coord_Type, I_x_Column, I_y_Column, I_z_Column,
  I_NBAR_Column, I_FKP_Column, I_Odd_Multipoles, I_COUNT
};
enum {
  D_XMIN, D_XMAX, D_YMIN, D_YMAX, D_ZMIN, D_ZMAX, D_Mink, D_Maxk, D_Omega_m, D_Redshift, D_X_Origin, D_Y_Origin,
  D_Z_Origin, D_REDMININ, D_REDMAXIN, D_SkyArea, D_FKP_Pk, D_FKP_Pk_mom, D_FKP_Pk_cross, D_COUNT
};

/* the 41 active tags of src/read_params.c:65-227, in the same order */
static const tagdef TAGS[] = {
    {"NumFilesInParallel", T_INT, I_NumFilesInParallel},
    {"NX", T_INT, I_NX}, {"NY", T_INT, I_NY}, {"NZ", T_INT, I_NZ},
    {"XMIN", T_FLOAT, D_XMIN}, {"XMAX", T_FLOAT, D_XMAX}, {"YMIN", T_FLOAT, D_YMIN}, {"YMAX", T_FLOAT, D_YMAX},
    {"ZMIN", T_FLOAT, D_ZMIN}, {"ZMAX", T_FLOAT, D_ZMAX},
    {"DoInterlacing", T_INT, I_DoInterlacing}, {"InterpOrder", T_INT, I_InterpOrder},
    {"NK", T_INT, I_NK}, {"NMU", T_INT, I_NMU}, {"Output2D", T_INT, I_Output2D}, {"OutputLog", T_INT, I_OutputLog},
    {"Mink", T_FLOAT, D_Mink}, {"Maxk", T_FLOAT, D_Maxk}, {"Omega_m", T_FLOAT, D_Omega_m},
    {"Redshift", T_FLOAT, D_Redshift},
    {"Periodic", T_INT, I_Periodic}, {"LOS", T_INT, I_LOS}, {"Survey", T_INT, I_Survey},
    {"Momentum", T_INT, I_Momentum},
    {"X_Origin", T_FLOAT, D_X_Origin}, {"Y_Origin", T_FLOAT, D_Y_Origin}, {"Z_Origin", T_FLOAT, D_Z_Origin},
    {"REDMININ", T_FLOAT, D_REDMININ}, {"REDMAXIN", T_FLOAT, D_REDMAXIN},
    {"NOBJ_Max", T_INT, I_NOBJ_Max}, {"Coord_Type", T_INT, I_Coord_Type},
    {"x_Column", T_INT, I_x_Column}, {"y_Column", T_INT, I_y_Column}, {"z_Column", T_INT, I_z_Column},
    {"NBAR_Column", T_INT, I_NBAR_Column}, {"SkyArea", T_FLOAT, D_SkyArea}, {"FKP_Column", T_INT, I_FKP_Column},
    {"FKP_Pk", T_FLOAT, D_FKP_Pk}, {"FKP_Pk_mom", T_FLOAT, D_FKP_Pk_mom}, {"FKP_Pk_cross", T_FLOAT, D_FKP_Pk_cross},
    {"Odd_Multipoles", T_INT, I_Odd_Multipoles},
};
#define NTAGS ((int)(sizeof(TAGS) / sizeof(TAGS[0])))

static void append(char *msg, size_t len, const char *s) {
  if (!msg || !len) return;
  size_t u = strlen(msg);
  if (u + 1 >= len) return;
  snprintf(msg + u, len - u, "%s", s);
}

static int read_all(const char *fname, capow_params *out, capow_survey_params *sv, char *msg, size_t msglen) {
  int ival[I_COUNT];
  double dval[D_COUNT];
  int used[64];
  char line[600], buf1[500], buf2[500], buf3[500];
  int errorFlag = 0;
  memset(ival, 0, sizeof ival);
  memset(dval, 0, sizeof dval);
  memset(used, 0, sizeof used);
  if (msg && msglen) msg[0] = 0;
  FILE *fd = fopen(fname, "r");
  if (!fd) { /* src/read_params.c:270-273 */
    snprintf(line, sizeof line, "\nERROR: Parameter file '%s' not found.\n\nFatal Error at line 330 in routine read_param.c\n",
             fname);
    append(msg, msglen, line);
    return CAPOW_EINVAL;
  }
  /* src/read_params.c:231-262: the loop reads 500-byte chunks until end of file */
  while (!feof(fd)) {
    char buf[500];
    buf[0] = 0;
    if (!fgets(buf, 500, fd)) buf[0] = 0;
    if (sscanf(buf, "%499s%499s%499s", buf1, buf2, buf3) < 2) continue;
    if (buf1[0] == '%') continue;
    int j = -1;
    for (int i = 0; i < NTAGS; i++) {
      if (!used[i] && strcmp(buf1, TAGS[i].name) == 0) {
        j = i;
        used[i] = 1;
        break;
      }
    }
    if (j >= 0) {
      if (TAGS[j].type == T_FLOAT) dval[TAGS[j].slot] = atof(buf2);
      else ival[TAGS[j].slot] = atoi(buf2);
    } else {
      snprintf(line, sizeof line, "\nERROR: In file %s:  Tag '%s' not allowed or multiple defined.\n\n", fname, buf1);
      append(msg, msglen, line);
      errorFlag = 1;
    }
  }
  fclose(fd);
  for (int i = 0; i < NTAGS; i++) {
    if (!used[i]) {
      snprintf(line, sizeof line, "\nERROR: I miss a value for tag '%s' in parameter file '%s'.\n\n", TAGS[i].name,
               fname);
      append(msg, msglen, line);
      errorFlag = 1;
    }
  }
  if (errorFlag) return CAPOW_EINVAL;

  /* check_inputs, src/read_params.c:294-428 (one task: NTask = 1) */
#define FATAL(text, ln)                                                         \
  do {                                                                          \
    append(msg, msglen, text);                                                  \
    snprintf(line, sizeof line, "Fatal Error at line %d in routine read_param.c\n", ln); \
    append(msg, msglen, line);                                                  \
    return CAPOW_EINVAL;                                                        \
  } while (0)
  if (ival[I_NumFilesInParallel] < 1)
    FATAL("\nERROR: `NumFilesInParallel' is less than 1 so no processors will be writing out the data.\n"
          "        Please set NumFileInParallel > 0'.\n\n", 297);
  if (1 < ival[I_NumFilesInParallel])
    append(msg, msglen,
           "\nWARNING: Number of processors smaller than `NumFilesInParallel'.\n"
           "         Setting NumFilesInParallel = Number of processors'.\n\n");
  if (ival[I_Periodic]) {
    int los = ival[I_LOS];
    if ((los != 0) && (los != 1) && (los != 2) && (los != 3))
      FATAL("\nERROR: `LOS' is neither 0 (real-space), 1, 2 nor 3.\n        Please choose a suitable value for `LOS'.\n\n",
            313);
  }
  if ((ival[I_InterpOrder] != 1) && (ival[I_InterpOrder] != 2) && (ival[I_InterpOrder] != 3))
    FATAL("\nERROR: `InterpOrder' is neither 1, 2 nor 3.\n        Please choose a suitable value for `InterpOrder'.\n\n",
          329);
  if ((ival[I_DoInterlacing] != 0) && (ival[I_DoInterlacing] != 1))
    FATAL("\nERROR: `DoInterlacing' is neither 0 nor 1.\n        Please choose a suitable value for `DoInterlacing'.\n\n",
          337);
  if ((ival[I_Output2D] != 0) && (ival[I_Output2D] != 1))
    FATAL("\nERROR: `Output2D' is neither 0 nor 1.\n        Please choose a suitable value for `Output2D'.\n\n", 345);
  if (ival[I_Output2D] && ival[I_NMU] <= 0)
    FATAL("\nERROR: `NMU' is less than 1.  if Output2D is 1, we must choose some mu-bins to output.\n"
          "        Please set 'NMU' > 0.\n\n", 354);
  if ((ival[I_OutputLog] != 0) && (ival[I_OutputLog] != 1))
    FATAL("\nERROR: `OutputLog' is neither 0 nor 1.\n        Please choose a suitable value for `OutputLog'.\n\n", 363);
  if (ival[I_NX] <= 0)
    FATAL("\nERROR: `NX' is less than 1. We must generate a mesh.\n        Please set 'NX' > 0.\n\n", 371);
  if (ival[I_NY] <= 0)
    FATAL("\nERROR: `NY' is less than 1. We must generate a mesh.\n        Please set 'NY' > 0.\n\n", 379);
  if (ival[I_NZ] <= 0)
    FATAL("\nERROR: `NZ' is less than 1. We must generate a mesh.\n        Please set 'NZ' > 0.\n\n", 387);
  if (ival[I_NK] <= 0)
    FATAL("\nERROR: `NK' is less than 1. We must choose some k-bins to output.\n        Please set 'NK' > 0.\n\n", 395);
  if (dval[D_XMAX] < dval[D_XMIN])
    FATAL("\nERROR: `XMAX' is less than `XMIN'.\n        Please set `XMAX' > `XMIN'.\n\n", 403);
  if (dval[D_YMAX] < dval[D_YMIN])
    FATAL("\nERROR: `XMAX' is less than `XMIN'.\n        Please set `XMAX' > `XMIN'.\n\n", 411);
  if (dval[D_ZMAX] < dval[D_ZMIN])
    FATAL("\nERROR: `XMAX' is less than `XMIN'.\n        Please set `XMAX' > `XMIN'.\n\n", 419);
  if (dval[D_Maxk] < dval[D_Mink])
    FATAL("\nERROR: `Maxk' is less than `Mink'.\n        Please set `Maxk' > `Mink'.\n\n", 427);
#undef FATAL
  if (!ival[I_Periodic] && !sv) {
    append(msg, msglen, "\nERROR: a survey run (Periodic 0) needs capow_read_survey_params.\n\n");
    return CAPOW_ENOTSUP;
  }
  if (sv) {
    memset(sv, 0, sizeof *sv);
    sv->Periodic = ival[I_Periodic];
    sv->Survey = ival[I_Survey];
    sv->Coord_Type = ival[I_Coord_Type];
    sv->X_Origin = dval[D_X_Origin];
    sv->Y_Origin = dval[D_Y_Origin];
    sv->Z_Origin = dval[D_Z_Origin];
    sv->REDMININ = dval[D_REDMININ];
    sv->REDMAXIN = dval[D_REDMAXIN];
    sv->NOBJ_Max = ival[I_NOBJ_Max];
    sv->NBAR_Column = ival[I_NBAR_Column];
    sv->SkyArea = dval[D_SkyArea];
    sv->FKP_Column = ival[I_FKP_Column];
    sv->FKP_Pk = dval[D_FKP_Pk];
    sv->FKP_Pk_mom = dval[D_FKP_Pk_mom];
    sv->FKP_Pk_cross = dval[D_FKP_Pk_cross];
  }
  if (out) {
    memset(out, 0, sizeof *out);
    out->NX = ival[I_NX];
    out->NY = ival[I_NY];
    out->NZ = ival[I_NZ];
    out->XMIN = dval[D_XMIN]; out->XMAX = dval[D_XMAX];
    out->YMIN = dval[D_YMIN]; out->YMAX = dval[D_YMAX];
    out->ZMIN = dval[D_ZMIN]; out->ZMAX = dval[D_ZMAX];
    out->InterpOrder = ival[I_InterpOrder];
    out->DoInterlacing = ival[I_DoInterlacing];
    out->NK = ival[I_NK];
    out->NMU = ival[I_NMU];
    out->Output2D = ival[I_Output2D];
    out->OutputLog = ival[I_OutputLog];
    out->Mink = dval[D_Mink];
    out->Maxk = dval[D_Maxk];
    out->Omega_m = dval[D_Omega_m];
    out->Redshift = dval[D_Redshift];
    out->LOS = ival[I_LOS];
    out->Momentum = ival[I_Momentum];
    out->Odd_Multipoles = ival[I_Odd_Multipoles];
  }
  return CAPOW_OK;
}

int capow_read_params(const char *fname, capow_params *out, char *msg, size_t msglen) {
  return read_all(fname, out, NULL, msg, msglen);
}

int capow_read_survey_params(const char *fname, capow_params *out, capow_survey_params *sv, char *msg,
                             size_t msglen) {
  if (!sv) return CAPOW_EINVAL;
  return read_all(fname, out, sv, msg, msglen);
}
