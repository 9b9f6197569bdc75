/*
 * sffo.h -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, FP64 restatement of the reference's generalized-Born energy and
 * gradient path (dacase/nabc src/sff), used by the tests, smoke() and the
 * CPU-baseline leg of bench.py as the checker.  The product never links it.
 * Parity of this restatement is pinned against the reference itself
 * (oracle/_ref, compiled from the reference sources in the development
 * container) through the golden fixtures under tests/golden/.
 */
#ifndef SFFO_H
#define SFFO_H

#include "../include/sff.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Options with the reference's defaults (src/sff/sff.c:68-199). */
typedef struct sffo_opts {
  double cut, rgbmax, kappa, epsext, dielc;
  int gb, nsnb, ntpr;
  double dt, temp0, tempi, gamma_ln, tautp, vlimit;
  int zerov, ntpr_md;
  double wcons;   /* restraint weight (econs, src/sff/eff.c:17) */
  int nscm;       /* md: centre-of-mass motion removal period (sff.c:2347) */
} sffo_opts;

typedef struct sffo_session sffo_session;

void sffo_default_opts(sffo_opts *o);

/* Session on a copy of prm's data; prm itself is not modified.  frozen may
 * be NULL (nothing frozen). */
sffo_session *sffo_create(const PARMSTRUCT_T *prm, const sffo_opts *o, const int *frozen);
void sffo_destroy(sffo_session *s);

/* Energy and gradient (reference mme34, src/sff/eff.c:2442).  ene[0..12]
 * follows the reference's ene[] layout: 0 total, 1 enb, 2 eel, 3 bond,
 * 4 angle, 5 dihedral, 7 enb14, 8 eel14, 10 egb.  The pair list is rebuilt
 * when rebuild != 0 or none exists yet.  reff (optional, length Natom)
 * receives the effective Born radii. */
double sffo_mme(sffo_session *s, const double *x, double *g, double *ene, double *reff,
                int rebuild);

/* Harmonic positional restraints: atoms with constrained[i] != 0 are held
 * to x0 (3 per atom) with weight opts.wcons (src/sff/eff.c:17-80).  Both
 * arrays are copied. */
void sffo_set_restraints(sffo_session *s, const int *constrained, const double *x0);

/* Number of unordered pairs on the current pair list. */
long sffo_npairs(const sffo_session *s);

/* Langevin/Berendsen dynamics exactly as the reference md()
 * (src/sff/sff.c:2071-2366), drawing noise from the reference's serial
 * gauss2 stream (src/sff/rand2.c) started from *seed (the reference's
 * default state is seed = -1).  Writes per-step (ekin, epot) pairs into
 * trace[2*(step-1)] when trace is non-NULL. */
int sffo_md(sffo_session *s, int maxstep, double *x, double *f, double *v, int *seed,
            double *trace);

/* Conjugate gradients exactly as the reference conjgrad()
 * (src/sff/conjgrad.c:34-263), evaluating sffo_mme with the reference's
 * iteration-count list-rebuild rule.  Writes each evaluation's energy into
 * etrace[k] (up to maxiter+1 entries) when etrace is non-NULL. */
int sffo_conjgrad(sffo_session *s, double *x, double *fret, double rmsgrad, double dfpred,
                  int maxiter, double *etrace, int *nevals);

/* The reference's gauss2 stream (src/sff/rand2.c:51-128): n draws of
 * N(mean, sd) continuing from *seed. */
void sffo_gauss_stream(int *seed, int n, double mean, const double *sd, double *out);

/* Threads of the OpenMP loops (n > 0 sets it); returns the count in effect. */
int sffo_set_threads(int n);

/* oracle/synth.c: the library generator's molecule (sffg_synth_molecule),
 * made without the library; free with sffo_synth_free. */
PARMSTRUCT_T *sffo_synth_molecule(int natom, unsigned long long seed, double *x, double *radius_out);
void sffo_synth_free(PARMSTRUCT_T *prm);
int sffo_prm_natom(const PARMSTRUCT_T *prm);
double sffo_prm_fsmax(const PARMSTRUCT_T *prm);

#ifdef __cplusplus
}
#endif

#endif
