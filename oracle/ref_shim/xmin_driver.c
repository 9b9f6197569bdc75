/*
 * Test infrastructure only: drives the reference's XMIN (src/sff/xminC.c,
 * compiled unchanged by oracle/Makefile into oracle/_ref/xminref) on the
 * objective functions of oracle/xmin_funcs.c, recording every function
 * value XMIN asks for.
 *
 *   xminref <fn> <method> <ls_method> <numdiff> <m_lbfgs> <maxiter>
 *           <grms_tol> <ls_maxatmov> <out.bin>
 *
 * fn: "rosen" (8 variables from (-1.2, 1, -1.2, 1, ...)) or "chain" (12
 * atoms on a helix, atom 4 frozen).  out.bin: ndim (int32), ncalls (int32),
 * iter, ls_iter, error_flag (int32 each), the return value, energy and grms
 * (f64), x[ndim] and g[ndim] (f64), then the ncalls function values (f64)
 * in the order XMIN requested them.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "sff.h"

FILE *nabout;
int get_mytaskid(void) { return 0; }

extern int xf_dim, xf_natom, xf_frozen[64];
double xf_rosenbrock(double *x, double *g, int *iter);
double xf_chain(double *x, double *g, int *iter);

static double (*objective)(double *, double *, int *);
static double trace[200000];
static int ncalls;

static double recorded(double *x, double *g, int *iter)
{
  double f = objective(x, g, iter);
  if (ncalls < 200000) trace[ncalls] = f;
  ncalls++;
  return f;
}

int main(int argc, char **argv)
{
  XMIN_OPT_T xo;
  double x[192], g[192], e = 0.0, grms = 0.0, ret;
  int n, ndim, i, it = 0;
  FILE *fp;

  nabout = stdout;
  if (argc < 10) {
    fprintf(stderr, "usage: %s fn method ls_method numdiff m maxiter grms_tol maxatmov out\n", argv[0]);
    return 2;
  }
  xmin_opt_init(&xo);
  xo.method = atoi(argv[2]);
  xo.ls_method = atoi(argv[3]);
  xo.numdiff = atoi(argv[4]);
  xo.m_lbfgs = atoi(argv[5]);
  xo.maxiter = atoi(argv[6]);
  xo.grms_tol = atof(argv[7]);
  xo.ls_maxatmov = atof(argv[8]);
  xo.print_level = 0;
  if (strcmp(argv[1], "rosen") == 0) {
    objective = xf_rosenbrock;
    xo.mol_struct_opt = 0;
    ndim = n = xf_dim;
    for (i = 0; i < n; i++) x[i] = (i % 2 == 0) ? -1.2 : 1.0;
  } else {
    objective = xf_chain;
    xo.mol_struct_opt = 1;
    n = xf_natom;
    ndim = 3 * n;
    xf_frozen[4] = 1;
    for (i = 0; i < n; i++) {
      double t = 0.9 * (double)i;
      /* a helix of radius 2 and rise 0.6 per bead; the starting point is
       * written to out.bin, so the tests never recompute it */
      x[3 * i] = 2.0 * cos(t);
      x[3 * i + 1] = 2.0 * sin(t);
      x[3 * i + 2] = 0.6 * (double)i;
    }
  }
  objective(x, g, &it); /* the gradient on entry marks frozen atoms */
  ret = xmin(recorded, &n, x, g, &e, &grms, &xo);
  fp = fopen(argv[9], "wb");
  if (!fp) { perror(argv[9]); return 2; }
  {
    double start[192];
    if (strcmp(argv[1], "rosen") == 0) {
      for (i = 0; i < ndim; i++) start[i] = (i % 2 == 0) ? -1.2 : 1.0;
    } else {
      for (i = 0; i < n; i++) {
        double t = 0.9 * (double)i;
        start[3 * i] = 2.0 * cos(t);
        start[3 * i + 1] = 2.0 * sin(t);
        start[3 * i + 2] = 0.6 * (double)i;
      }
    }
    fwrite(&ndim, sizeof(int), 1, fp);
    fwrite(&ncalls, sizeof(int), 1, fp);
    fwrite(&xo.iter, sizeof(int), 1, fp);
    fwrite(&xo.ls_iter, sizeof(int), 1, fp);
    fwrite(&xo.error_flag, sizeof(int), 1, fp);
    fwrite(&ret, sizeof(double), 1, fp);
    fwrite(&e, sizeof(double), 1, fp);
    fwrite(&grms, sizeof(double), 1, fp);
    fwrite(start, sizeof(double), (size_t)ndim, fp);
    fwrite(x, sizeof(double), (size_t)ndim, fp);
    fwrite(g, sizeof(double), (size_t)ndim, fp);
    fwrite(trace, sizeof(double), (size_t)(ncalls < 200000 ? ncalls : 200000), fp);
  }
  fclose(fp);
  printf("xmin returns %.17g iter %d ls_iter %d error %d calls %d\n", ret, xo.iter, xo.ls_iter,
         xo.error_flag, ncalls);
  return 0;
}
