/*
 * Test infrastructure only: runs the reference's LMOD (src/sff/lmodC.c,
 * compiled unchanged by oracle/Makefile into oracle/_ref/lmodref) on the
 * bead chain of oracle/xmin_funcs.c.  The reference's lmod() calls mme()
 * and xmin(mme); here mme() is the chain function and xmin() the
 * reference's own (xminC.c).  Its ARPACK driver is replaced by
 * ref_shim/arpack_standin.cpp.
 *
 *   lmodref <natom> <frozen atom or -1> <niter> <nmod> <kmod> <mc_option>
 *           <nof_lmod_steps> <eig_recalc> <ndim_arnoldi> <lmod_restart>
 *           <n_best_struct> <energy_window> <conf_separation_rms>
 *           <nlig> <lig_start> <lig_end> <lig_cent> <print_level> <seed>
 *           <out.bin>
 *
 * Starts from a helix of radius 2 and rise 0.6 per bead (0.9 rad per bead),
 * with xmin's ls_maxatmov 0.15 (as test/tlmod.c); one ligand takes 0.5-1.5 A
 * translations and 10-60 degree rotations, 3 tries every 2 iterations.
 * out.bin: natom, nconf returned, error_flag, ndim_arnoldi after (int32),
 * the return value and the final energy (f64), then the start coordinates,
 * the final xyz, conflib (nconf structures) and the trajectory (niter + 1
 * structures, or the zig-zag frames at print_level 5), f64.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include "sff.h"

FILE *nabout;
int get_mytaskid(void) { return 0; }

extern int xf_natom, xf_frozen[64];
double xf_chain(double *x, double *g, int *iter);

double mme(double *x, double *g, int *iter) { return xf_chain(x, g, iter); }

int main(int argc, char **argv)
{
  struct xmin_opt xo;
  struct lmod_opt lo;
  double *x, *x0, *g, *conflib, *traj, e, ret;
  int n, i, frozen, it = 0, lig_start, lig_end, lig_cent;
  double tr_min = 0.5, tr_max = 1.5, rot_min = 10.0, rot_max = 60.0;
  size_t ntraj;
  FILE *fp;

  nabout = stdout;
  if (argc < 21) {
    fprintf(stderr, "usage: see the header of lmod_driver.c\n");
    return 2;
  }
  n = atoi(argv[1]);
  frozen = atoi(argv[2]);
  xf_natom = n;
  if (frozen >= 0) xf_frozen[frozen] = 1;
  lmod_opt_init(&lo, &xo);
  lo.niter = atoi(argv[3]);
  lo.nmod = atoi(argv[4]);
  lo.kmod = atoi(argv[5]);
  lo.mc_option = atoi(argv[6]);
  lo.nof_lmod_steps = atoi(argv[7]);
  lo.eig_recalc = atoi(argv[8]);
  lo.ndim_arnoldi = atoi(argv[9]);
  lo.lmod_restart = atoi(argv[10]);
  lo.n_best_struct = atoi(argv[11]);
  lo.energy_window = atof(argv[12]);
  lo.conf_separation_rms = atof(argv[13]);
  lo.nlig = atoi(argv[14]);
  lig_start = atoi(argv[15]);
  lig_end = atoi(argv[16]);
  lig_cent = atoi(argv[17]);
  lo.print_level = atoi(argv[18]);
  lo.random_seed = atoi(argv[19]);
  lo.apply_rigdock = 2;
  lo.nof_poses_to_try = 3;
  xo.ls_maxatmov = 0.15;
  x = calloc(3 * (size_t)n, sizeof(double));
  x0 = calloc(3 * (size_t)n, sizeof(double));
  g = calloc(3 * (size_t)n, sizeof(double));
  conflib = calloc(3 * (size_t)n * (size_t)lo.nconf, sizeof(double));
  ntraj = (size_t)(lo.niter + 1);
  if (lo.print_level == 5)
    ntraj = (size_t)(4 * (lo.nof_lmod_steps ? lo.nof_lmod_steps : 20) + 3) *
            (size_t)(lo.niter * lo.kmod + lo.nmod + 2);
  traj = calloc(3 * (size_t)n * ntraj, sizeof(double));
  for (i = 0; i < n; i++) {
    double t = 0.9 * (double)i;
    x[3 * i] = 2.0 * cos(t);
    x[3 * i + 1] = 2.0 * sin(t);
    x[3 * i + 2] = 0.6 * (double)i;
  }
  for (i = 0; i < 3 * n; i++) x0[i] = x[i];
  e = mme(x, g, &it);
  ret = lmod(&n, x, g, &e, conflib, traj, &lig_start, &lig_end, &lig_cent, &tr_min, &tr_max, &rot_min,
             &rot_max, &xo, &lo);
  printf("lmod returns %.17g error %d nconf %d\n", ret, lo.error_flag, lo.nconf);
  fp = fopen(argv[20], "wb");
  if (!fp) { perror(argv[20]); return 2; }
  fwrite(&n, sizeof(int), 1, fp);
  fwrite(&lo.nconf, sizeof(int), 1, fp);
  fwrite(&lo.error_flag, sizeof(int), 1, fp);
  fwrite(&lo.ndim_arnoldi, sizeof(int), 1, fp);
  fwrite(&ret, sizeof(double), 1, fp);
  fwrite(&e, sizeof(double), 1, fp);
  fwrite(x0, sizeof(double), 3 * (size_t)n, fp);
  fwrite(x, sizeof(double), 3 * (size_t)n, fp);
  fwrite(conflib, sizeof(double), 3 * (size_t)n * (size_t)lo.nconf, fp);
  fwrite(traj, sizeof(double), 3 * (size_t)n * ntraj, fp);
  fclose(fp);
  return 0;
}
