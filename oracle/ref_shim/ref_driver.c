/*
 * Test infrastructure only: a command-line driver for the reference SFF
 * library (dacase/nabc src/sff) compiled by oracle/Makefile into oracle/_ref.
 * It follows the reference's own C drivers (test/tmd.c:20-80) and the NAB
 * test programs (test/nab/gb5trx.nab:1-16): rdparm, mm_options,
 * mme_init_sff with nothing frozen or constrained, then one of
 *
 *   sp  <out.bin>                     one mme() at iter=-1 (verbose breakdown)
 *   cg  <maxiter> <dfpred> <rmsgrad> [out.bin]   conjgrad() driven by mme
 *   md  <nsteps> [out.bin]            md() driven by mme
 *   time <nevals>                     repeated quiet mme() evaluations
 *   timei <nevals>                    mme() at iter = 0, 1, ..., nevals - 1 after
 *                                     one untimed call: the normal cadence
 *                                     (list rebuilt when iter % nsnb == 0),
 *                                     printing suppressed by a large ntpr
 *   spr <out.bin>                     mme_rattle() at iter=-1 on the input
 *                                     positions shifted by 0.02 ((k mod 3) - 1) A
 *                                     per coordinate k (bond lengths off)
 *   spc <every> <out.bin>             single point with atoms 0, every, 2 every,
 *                                     ... restrained (option wcons) to the
 *                                     input positions shifted by
 *                                     0.05 ((3 i + k) mod 5 - 2) A per coordinate
 *   xmin <method> <maxiter> <grms_tol> <ls_maxatmov> <rattle> <out.bin> <trace.bin>
 *                                     the reference's test/txmin.c: func(x, g, -1),
 *                                     xmin(func) with print_level 10, func(x, g, -1),
 *                                     func = mme_rattle (rattle=1) or mme;
 *                                     trace.bin: every energy xmin asked for (f64)
 *   lmod <niter> <nmod> <kmod> <mc_option> <nof_lmod_steps> <seed> <grms_tol>
 *        <maxiter> <out.bin>        the reference's test/tlmod.c with these
 *                                     options (print_level 2, xmin
 *                                     ls_maxatmov 0.15, the first
 *                                     minimisation to grms_tol in maxiter
 *                                     steps); ARPACK replaced by
 *                                     ref_shim/arpack_standin.cpp; run in an
 *                                     empty directory (conflib.dat);
 *                                     out.bin: natom, nconf (int32), the
 *                                     return value (f64), x, conflib (f64)
 *
 * Coordinates come from a PDB (columns 31-54 of ATOM/HETATM records, the
 * order the prmtop uses) or an Amber ASCII restart read with getxv().
 * out.bin holds natom (int32) then E (f64) then x[3N] and g[3N] (f64).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include "sff.h"

FILE *nabout;
int mytaskid = 0;
int numtasks = 1;

static double now_s(void)
{
  struct timeval tv;
  gettimeofday(&tv, NULL);
  return (double)tv.tv_sec + 1e-6 * (double)tv.tv_usec;
}

static int read_pdb(const char *name, int natom, double *x)
{
  FILE *fp = fopen(name, "r");
  char line[256], field[9];
  int n = 0, k;
  if (!fp) return -1;
  while (fgets(line, sizeof(line), fp) && n < natom) {
    if (strncmp(line, "ATOM", 4) && strncmp(line, "HETATM", 6)) continue;
    for (k = 0; k < 3; k++) {
      memcpy(field, line + 30 + 8 * k, 8);
      field[8] = '\0';
      x[3 * n + k] = atof(field);
    }
    n++;
  }
  fclose(fp);
  return n == natom ? 0 : -1;
}

static double (*traced_func)(double *, double *, int *);
static double trace[100000];
static int ntraced;

static double traced(double *x, double *g, int *iter)
{
  double e = traced_func(x, g, iter);
  if (ntraced < 100000) trace[ntraced] = e;
  ntraced++;
  return e;
}

static void dump(const char *name, int natom, double e, const double *x, const double *g)
{
  FILE *fp;
  if (!name) return;
  fp = fopen(name, "wb");
  if (!fp) { perror(name); exit(2); }
  fwrite(&natom, sizeof(int), 1, fp);
  fwrite(&e, sizeof(double), 1, fp);
  fwrite(x, sizeof(double), 3 * (size_t)natom, fp);
  fwrite(g, sizeof(double), 3 * (size_t)natom, fp);
  fclose(fp);
}

int main(int argc, char **argv)
{
  PARMSTRUCT_T *prm;
  int natom, n3, *frozen, *constrained, iter;
  double *x, *g, *v, e = 0.0;
  const char *mode;
  size_t len;

  nabout = stdout;
  if (argc < 5) {
    fprintf(stderr, "usage: %s prmtop coords sp|cg|md|time opts [args]\n", argv[0]);
    return 2;
  }
  prm = rdparm(argv[1]);
  natom = prm->Natom;
  n3 = 3 * natom;
  x = calloc((size_t)n3, sizeof(double));
  g = calloc((size_t)n3, sizeof(double));
  v = calloc((size_t)n3, sizeof(double));
  len = strlen(argv[2]);
  if (len > 4 && strcmp(argv[2] + len - 4, ".pdb") == 0) {
    if (read_pdb(argv[2], natom, x)) {
      fprintf(stderr, "cannot read %d atoms from %s\n", natom, argv[2]);
      return 2;
    }
  } else {
    getxv(argv[2], natom, 0.0, x, v);
  }
  mm_options(argv[4]);
  frozen = calloc((size_t)natom, sizeof(int));
  constrained = calloc((size_t)natom, sizeof(int));
  mode = argv[3];
  if (strcmp(mode, "spc") == 0) {
    int every = atoi(argv[5]), i;
    double *x0 = calloc((size_t)n3, sizeof(double));
    for (i = 0; i < n3; i++) x0[i] = x[i] + 0.05 * (double)(i % 5 - 2);
    for (i = 0; i < natom; i += every) constrained[i] = 1;
    mme_init_sff(prm, frozen, constrained, x0, NULL);
    iter = -1;
    e = mme(x, g, &iter);
    printf("oracle_total: %.17g\n", e);
    dump(argc > 6 ? argv[6] : NULL, natom, e, x, g);
    return 0;
  }
  mme_init_sff(prm, frozen, constrained, NULL, NULL);
  if (strcmp(mode, "xmin") == 0) {
    XMIN_OPT_T xo;
    double grms = 0.0;
    FILE *fp;
    xmin_opt_init(&xo);
    xo.method = atoi(argv[5]);
    xo.maxiter = atoi(argv[6]);
    xo.grms_tol = atof(argv[7]);
    xo.ls_maxatmov = atof(argv[8]);
    xo.print_level = 10;
    traced_func = atoi(argv[9]) ? mme_rattle : mme;
    iter = -1;
    e = traced_func(x, g, &iter);
    e = xmin(traced, &natom, x, g, &e, &grms, &xo);
    printf("xmin returns %.17g iter %d ls_iter %d error %d grms %.17g\n", e, xo.iter, xo.ls_iter,
           xo.error_flag, grms);
    iter = -1;
    e = traced_func(x, g, &iter);
    printf("oracle_total: %.17g\n", e);
    dump(argv[10], natom, e, x, g);
    fp = fopen(argv[11], "wb");
    if (!fp) { perror(argv[11]); return 2; }
    fwrite(trace, sizeof(double), (size_t)(ntraced < 100000 ? ntraced : 100000), fp);
    fclose(fp);
    return 0;
  }
  if (strcmp(mode, "lmod") == 0) {
    struct xmin_opt xo;
    struct lmod_opt lo;
    double *conflib, *traj, ret;
    int none = 0;
    double zero = 0.0;
    FILE *fp;
    lmod_opt_init(&lo, &xo);
    lo.niter = atoi(argv[5]);
    lo.nmod = atoi(argv[6]);
    lo.kmod = atoi(argv[7]);
    lo.mc_option = atoi(argv[8]);
    lo.nof_lmod_steps = atoi(argv[9]);
    lo.random_seed = atoi(argv[10]);
    lo.print_level = 2;
    xo.grms_tol = atof(argv[11]);
    xo.maxiter = atoi(argv[12]);
    xo.ls_maxatmov = 0.15;
    conflib = calloc((size_t)n3 * (size_t)lo.nconf, sizeof(double));
    traj = calloc((size_t)n3 * (size_t)(lo.niter + 1), sizeof(double));
    iter = -1;
    e = mme(x, g, &iter);
    ret = lmod(&natom, x, g, &e, conflib, traj, &none, &none, &none, &zero, &zero, &zero, &zero, &xo, &lo);
    printf("lmod returns %.17g error %d nconf %d\n", ret, lo.error_flag, lo.nconf);
    fp = fopen(argv[13], "wb");
    if (!fp) { perror(argv[13]); return 2; }
    fwrite(&natom, sizeof(int), 1, fp);
    fwrite(&lo.nconf, sizeof(int), 1, fp);
    fwrite(&ret, sizeof(double), 1, fp);
    fwrite(x, sizeof(double), (size_t)n3, fp);
    fwrite(conflib, sizeof(double), (size_t)n3 * (size_t)lo.nconf, fp);
    fclose(fp);
    return 0;
  }
  if (strcmp(mode, "spr") == 0) {
    int k;
    for (k = 0; k < n3; k++) x[k] += 0.02 * (double)(k % 3 - 1);
    iter = -1;
    e = mme_rattle(x, g, &iter);
    printf("oracle_total: %.17g\n", e);
    dump(argc > 5 ? argv[5] : NULL, natom, e, x, g);
    return 0;
  }

  if (strcmp(mode, "sp") == 0) {
    iter = -1;
    e = mme(x, g, &iter);
    printf("oracle_total: %.17g\n", e);
    dump(argc > 5 ? argv[5] : NULL, natom, e, x, g);
  } else if (strcmp(mode, "cg") == 0) {
    int maxiter = atoi(argv[5]), ier;
    double dfpred = atof(argv[6]), rmsgrad = atof(argv[7]);
    ier = conjgrad(x, &n3, &e, mme, &rmsgrad, &dfpred, &maxiter);
    printf("conjgrad returns %d\n", ier);
    printf("oracle_total: %.17g\n", e);
    dump(argc > 8 ? argv[8] : NULL, natom, e, x, g);
  } else if (strcmp(mode, "md") == 0) {
    int nsteps = atoi(argv[5]);
    md(n3, nsteps, x, g, v, mme);
    dump(argc > 6 ? argv[6] : NULL, natom, 0.0, x, v);
  } else if (strcmp(mode, "time") == 0) {
    int nevals = atoi(argv[5]), k;
    double t0, t1;
    iter = -2;
    e = mme(x, g, &iter); /* first call builds the pair list */
    t0 = now_s();
    for (k = 0; k < nevals; k++) {
      iter = -2;
      e = mme(x, g, &iter);
    }
    t1 = now_s();
    printf("oracle_time: %d evals %.6f s total %.17g\n", nevals, t1 - t0, e);
  } else if (strcmp(mode, "timei") == 0) {
    int nevals = atoi(argv[5]), k;
    double t0, t1;
    iter = -2;
    e = mme(x, g, &iter);
    t0 = now_s();
    for (k = 0; k < nevals; k++) {
      iter = k;
      e = mme(x, g, &iter);
    }
    t1 = now_s();
    printf("oracle_time: %d evals %.6f s total %.17g\n", nevals, t1 - t0, e);
  } else {
    fprintf(stderr, "unknown mode %s\n", mode);
    return 2;
  }
  return 0;
}
