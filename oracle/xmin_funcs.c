/*
 * Test infrastructure only: deterministic objective functions for checking
 * the XMIN minimiser (the reference's src/sff/xminC.c and libsffg's
 * xmin()) against each other bit for bit.  Both the reference driver
 * (ref_shim/xmin_driver.c) and the tests call these same compiled
 * functions, built without floating-point contraction, so any difference in
 * the iterates comes from the minimisers alone.  Only +, -, *, / and sqrt
 * are used (all correctly rounded), so every host computes the same bits.
 *
 * Each has the signature XMIN expects, func(x, g, iter) -> value; iter is
 * ignored.
 */
#include <math.h>

/* Extended Rosenbrock function of xf_dim (even) variables (general
 * optimisation, mol_struct_opt = 0). */
int xf_dim = 8;

double xf_rosenbrock(double *x, double *g, int *iter)
{
  double f = 0.0;
  int i;
  (void)iter;
  for (i = 0; i + 1 < xf_dim; i += 2) {
    double t1 = x[i + 1] - x[i] * x[i];
    double t2 = 1.0 - x[i];
    f += 100.0 * t1 * t1 + t2 * t2;
    g[i] = -400.0 * x[i] * t1 - 2.0 * t2;
    g[i + 1] = 200.0 * t1;
  }
  return f;
}

/* A bead chain of xf_natom atoms (mol_struct_opt = 1): harmonic bonds of
 * length 1.5 between neighbours and a soft-core 12-6 attraction
 * (s/(r^2 + 0.5))^6 - 2 (s/(r^2 + 0.5))^3 with s = 4 between all other pairs.
 * Atoms with xf_frozen[i] != 0 get a zero gradient. */
int xf_natom = 12;
int xf_frozen[64];

double xf_chain(double *x, double *g, int *iter)
{
  double f = 0.0;
  int i, j, k;
  (void)iter;
  for (i = 0; i < 3 * xf_natom; i++) g[i] = 0.0;
  for (i = 0; i < xf_natom; i++) {
    for (j = i + 1; j < xf_natom; j++) {
      double d[3], r2 = 0.0;
      for (k = 0; k < 3; k++) {
        d[k] = x[3 * j + k] - x[3 * i + k];
        r2 += d[k] * d[k];
      }
      if (j == i + 1) {
        double r = sqrt(r2), dr = r - 1.5;
        double de = 2.0 * 10.0 * dr / r;
        f += 10.0 * dr * dr;
        for (k = 0; k < 3; k++) {
          g[3 * j + k] += de * d[k];
          g[3 * i + k] -= de * d[k];
        }
      } else {
        double u = 4.0 / (r2 + 0.5), u3 = u * u * u, u6 = u3 * u3;
        /* dE/dr2 = (-6 u6 + 6 u3) / (r2 + 0.5) */
        double de = 2.0 * (-6.0 * u6 + 6.0 * u3) / (r2 + 0.5);
        f += u6 - 2.0 * u3;
        for (k = 0; k < 3; k++) {
          g[3 * j + k] += de * d[k];
          g[3 * i + k] -= de * d[k];
        }
      }
    }
  }
  for (i = 0; i < xf_natom; i++)
    if (xf_frozen[i])
      for (k = 0; k < 3; k++) g[3 * i + k] = 0.0;
  return f;
}
