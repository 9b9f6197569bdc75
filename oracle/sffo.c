/*
 * sffo.c -- TEST INFRASTRUCTURE ONLY: the FP64 CPU oracle.
 *
 * A plain-C restatement of the reference's generalized-Born energy/gradient
 * path (dacase/nabc src/sff).  Each function cites the reference lines whose
 * arithmetic it follows.  The pair list is the reference's (pairs with
 * r < cut, excluded pairs included, pairs of two frozen atoms left out;
 * src/sff/nblist.c:726-746) built by brute force in ascending-j order, which
 * is also the order the reference's sorted kd-tree lists use, so the
 * floating-point summation order per atom is the same.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * this file; the product path never does.
 */
#include "sffo.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../nabc_gb300/csrc/gbneck_tables.h"

#define KSCALE 0.73 /* src/sff/eff.c:1368 */

struct sffo_session {
  int n;
  sffo_opts o;
  int gb;
  double gboffset, gbneckscale, fsmax, rgbmax, cut;
  double *q, *rborn, *fs, *alpha, *beta, *gamma;
  int *neck, *frozen;
  int ntypes, *iac, *cno;
  double *cn1, *cn2;
  const PARMSTRUCT_T *prm;
  /* exclusion lists per atom, 1-based with 0 = none (src/sff/sff.c:1551-1574) */
  int *ex_start, *ex_atoms;
  /* 1-4 list per atom i (src/sff/sff.c:1492-1537) */
  int *n14_start, *n14_atoms;
  double *n14_scee, *n14_scnb;
  /* pair list: per atom lower (j<i) then upper (j>i), ascending */
  long *pl_start;
  int *pl_low, *pl_up, *pl_atoms;
  long npairs;
  int have_list;
  /* scratch */
  double *reff, *psi, *sumdeijda;
  /* positional restraints (src/sff/sff.c:100, 1169-1178) */
  int *constrained;
  double *x0;
  /* gauss2 state (src/sff/rand2.c:22-25) */
  int rng_seed2, rng_iy, rng_iv[32], rng_seed3;
};

void sffo_default_opts(sffo_opts *o)
{
  /* src/sff/sff.c:72-196 */
  o->cut = 20.0;
  o->rgbmax = 15.0;
  o->kappa = 0.0;
  o->epsext = 78.5;
  o->dielc = 1.0;
  o->gb = 0;
  o->nsnb = 10;
  o->ntpr = 10;
  o->dt = 0.001;
  o->temp0 = 300.0;
  o->tempi = 0.0;
  o->gamma_ln = 0.0;
  o->tautp = 999999.0;
  o->vlimit = 10.0;
  o->zerov = 0;
  o->ntpr_md = 10;
  o->wcons = 0.0;
  o->nscm = 0;
}

static void *xcalloc(size_t n, size_t sz)
{
  void *p = calloc(n ? n : 1, sz);
  if (!p) abort();
  return p;
}

/* GB parameters by model: src/sff/sff.c:1186-1333. */
static void setup_gb(sffo_session *s, const PARMSTRUCT_T *prm)
{
  int i;
  s->gboffset = 0.09;
  s->gbneckscale = 0.0;
  for (i = 0; i < s->n; i++) {
    s->fs[i] = prm->Fs[i];
    s->alpha[i] = s->beta[i] = s->gamma[i] = 0.0;
    s->neck[i] = 0;
  }
  if (s->gb == 2 || s->gb == 5) {
    for (i = 0; i < s->n; i++) {
      s->alpha[i] = s->gb == 2 ? 0.8 : 1.0;
      s->beta[i] = s->gb == 2 ? 0.0 : 0.8;
      s->gamma[i] = s->gb == 2 ? 2.909125 : 4.85;
    }
  } else if (s->gb == 7) {
    s->gbneckscale = 0.361825;
    for (i = 0; i < s->n; i++) {
      s->alpha[i] = 1.09511284;
      s->beta[i] = 1.90792938;
      s->gamma[i] = 2.50798245;
      switch (prm->AtomicNum[i]) {
        case 1: s->fs[i] = 1.09085413633e0; break;
        case 6: s->fs[i] = 4.84353823306e-1; break;
        case 7: s->fs[i] = 7.00147318409e-1; break;
        case 8: s->fs[i] = 1.06557401132e0; break;
        case 16: s->fs[i] = 6.02256336067e-1; break;
        default: s->fs[i] = 5.0e-1;
      }
      s->neck[i] = (int)((prm->Rborn[i] - 1.0) * 20.0 + 0.5);
    }
  } else if (s->gb == 8) {
    for (i = 0; i < s->n; i++) {
      double a = 1.0, b = 0.8, g = 4.85, f = 0.5;
      switch (prm->AtomicNum[i]) {
        case 1: a = SFFG_GB8_ALPHA_H; b = SFFG_GB8_BETA_H; g = SFFG_GB8_GAMMA_H; f = SFFG_GB8_SCREEN_H; break;
        case 6: a = SFFG_GB8_ALPHA_C; b = SFFG_GB8_BETA_C; g = SFFG_GB8_GAMMA_C; f = SFFG_GB8_SCREEN_C; break;
        case 7: a = SFFG_GB8_ALPHA_N; b = SFFG_GB8_BETA_N; g = SFFG_GB8_GAMMA_N; f = SFFG_GB8_SCREEN_N; break;
        case 8: a = SFFG_GB8_ALPHA_OS; b = SFFG_GB8_BETA_OS; g = SFFG_GB8_GAMMA_OS; f = SFFG_GB8_SCREEN_O; break;
        case 15: a = SFFG_GB8_ALPHA_P; b = SFFG_GB8_BETA_P; g = SFFG_GB8_GAMMA_P; f = SFFG_GB8_SCREEN_P; break;
        case 16: a = SFFG_GB8_ALPHA_OS; b = SFFG_GB8_BETA_OS; g = SFFG_GB8_GAMMA_OS; f = SFFG_GB8_SCREEN_S; break;
        default: break;
      }
      s->alpha[i] = a;
      s->beta[i] = b;
      s->gamma[i] = g;
      s->fs[i] = f;
      s->neck[i] = (int)((prm->Rborn[i] - 1.0) * 20.0 + 0.5);
    }
    s->gboffset = 0.195141;
    s->gbneckscale = 0.826836;
  }
}

sffo_session *sffo_create(const PARMSTRUCT_T *prm, const sffo_opts *o, const int *frozen)
{
  sffo_session *s = xcalloc(1, sizeof(*s));
  int i, j, k, n = prm->Natom;
  double scale;
  s->n = n;
  s->o = *o;
  s->gb = o->gb;
  s->prm = prm;
  s->rgbmax = o->rgbmax;
  s->cut = o->cut;
  s->fsmax = prm->Fsmax;
  s->q = xcalloc(n, sizeof(double));
  s->rborn = xcalloc(n, sizeof(double));
  s->fs = xcalloc(n, sizeof(double));
  s->alpha = xcalloc(n, sizeof(double));
  s->beta = xcalloc(n, sizeof(double));
  s->gamma = xcalloc(n, sizeof(double));
  s->neck = xcalloc(n, sizeof(int));
  s->frozen = xcalloc(n, sizeof(int));
  /* charges scaled by 1/sqrt(dielc): src/sff/sff.c:1153-1162 */
  scale = o->dielc != 1.0 ? 1.0 / sqrt(o->dielc) : 1.0;
  for (i = 0; i < n; i++) {
    s->q[i] = prm->Charges[i] * scale;
    s->rborn[i] = prm->Rborn[i];
    s->frozen[i] = frozen ? frozen[i] : 0;
  }
  setup_gb(s, prm);
  s->ntypes = prm->Ntypes;
  s->iac = prm->Iac;
  s->cno = prm->Cno;
  s->cn1 = prm->Cn1;
  s->cn2 = prm->Cn2;
  /* exclusion lists (src/sff/sff.c:1551-1574) */
  s->ex_start = xcalloc(n + 1, sizeof(int));
  for (i = 0; i < n; i++) s->ex_start[i + 1] = s->ex_start[i] + prm->Iblo[i];
  s->ex_atoms = xcalloc(s->ex_start[n], sizeof(int));
  memcpy(s->ex_atoms, prm->ExclAt, sizeof(int) * (size_t)s->ex_start[n]);
  /* 1-4 lists (src/sff/sff.c:1492-1537) */
  s->n14_start = xcalloc(n + 1, sizeof(int));
  for (i = 0; i < n; i++) s->n14_start[i + 1] = s->n14_start[i] + prm->N14pairs[i];
  k = s->n14_start[n];
  s->n14_atoms = xcalloc(k, sizeof(int));
  s->n14_scee = xcalloc(k, sizeof(double));
  s->n14_scnb = xcalloc(k, sizeof(double));
  for (j = 0; j < k; j++) {
    s->n14_atoms[j] = prm->N14pairlist[j];
    s->n14_scee[j] = prm->N14sceelist[j];
    s->n14_scnb[j] = prm->N14scnblist[j];
  }
  s->pl_start = xcalloc(n + 1, sizeof(long));
  s->pl_low = xcalloc(n, sizeof(int));
  s->pl_up = xcalloc(n, sizeof(int));
  s->reff = xcalloc(n, sizeof(double));
  s->psi = xcalloc(n, sizeof(double));
  s->sumdeijda = xcalloc(n, sizeof(double));
  s->rng_seed3 = -1;
  return s;
}

void sffo_destroy(sffo_session *s)
{
  if (!s) return;
  free(s->q); free(s->rborn); free(s->fs); free(s->alpha); free(s->beta); free(s->gamma);
  free(s->neck); free(s->frozen); free(s->ex_start); free(s->ex_atoms); free(s->n14_start);
  free(s->n14_atoms); free(s->n14_scee); free(s->n14_scnb); free(s->pl_start); free(s->pl_low);
  free(s->pl_up); free(s->pl_atoms); free(s->reff); free(s->psi); free(s->sumdeijda);
  free(s->constrained); free(s->x0);
  free(s);
}

void sffo_set_restraints(sffo_session *s, const int *constrained, const double *x0)
{
  free(s->constrained);
  free(s->x0);
  s->constrained = xcalloc(s->n, sizeof(int));
  s->x0 = xcalloc(3 * (size_t)s->n, sizeof(double));
  memcpy(s->constrained, constrained, s->n * sizeof(int));
  memcpy(s->x0, x0, 3 * (size_t)s->n * sizeof(double));
}

/* Harmonic positional restraints: src/sff/eff.c:17-80 (econs). */
static double econs(const sffo_session *s, const double *x, double *g)
{
  double e = 0.0;
  int i;
  if (!s->constrained) return 0.0;
  for (i = 0; i < s->n; i++) {
    if (!s->constrained[i]) continue;
    const double rx = x[3 * i] - s->x0[3 * i], ry = x[3 * i + 1] - s->x0[3 * i + 1],
                 rz = x[3 * i + 2] - s->x0[3 * i + 2];
    e += s->o.wcons * (rx * rx + ry * ry + rz * rz);
    g[3 * i] += 2. * s->o.wcons * rx;
    g[3 * i + 1] += 2. * s->o.wcons * ry;
    g[3 * i + 2] += 2. * s->o.wcons * rz;
  }
  return e;
}

/* Centre-of-mass motion removal: src/sff/com.c:10-47 (com2zero) and, with
 * also_v, 53-147 (com_vw2zero, with the cofactor inverse of com_psinv). */
static void com_remove(int n, double *x, double *v, const double *minv, int also_v)
{
  double mt = 0, xs = 0, ys = 0, zs = 0, vx = 0, vy = 0, vz = 0, L[3] = {0, 0, 0}, M[6] = {0, 0, 0, 0, 0, 0};
  const double sc = 1.e-3;
  int i;
  for (i = 0; i < n; i++) mt += 1. / minv[3 * i];
  for (i = 0; i < n; i++) {
    xs += x[3 * i] / minv[3 * i];
    ys += x[3 * i + 1] / minv[3 * i + 1];
    zs += x[3 * i + 2] / minv[3 * i + 2];
  }
  xs /= mt; ys /= mt; zs /= mt;
  for (i = 0; i < n; i++) {
    x[3 * i] -= xs; x[3 * i + 1] -= ys; x[3 * i + 2] -= zs;
  }
  if (!also_v) return;
  for (i = 0; i < n; i++) {
    vx += v[3 * i] / minv[3 * i];
    vy += v[3 * i + 1] / minv[3 * i + 1];
    vz += v[3 * i + 2] / minv[3 * i + 2];
  }
  vx /= mt; vy /= mt; vz /= mt;
  for (i = 0; i < n; i++) {
    v[3 * i] -= vx; v[3 * i + 1] -= vy; v[3 * i + 2] -= vz;
  }
  for (i = 0; i < n; i++) {
    const double m = 1. / minv[3 * i], X = x[3 * i], Y = x[3 * i + 1], Z = x[3 * i + 2];
    L[0] += sc * (Y * v[3 * i + 2] - Z * v[3 * i + 1]) * m;
    L[1] += sc * (Z * v[3 * i] - X * v[3 * i + 2]) * m;
    L[2] += sc * (X * v[3 * i + 1] - Y * v[3 * i]) * m;
  }
  for (i = 0; i < n; i++) {
    const double m = 1. / minv[3 * i], X = x[3 * i], Y = x[3 * i + 1], Z = x[3 * i + 2];
    M[0] += X * X * m; M[1] += X * Y * m; M[2] += X * Z * m;
    M[3] += Y * Y * m; M[4] += Y * Z * m; M[5] += Z * Z * m;
  }
  {
    const double I0 = (M[3] + M[5]) * sc, I1 = -M[1] * sc, I2 = -M[2] * sc;
    const double I4 = (M[0] + M[5]) * sc, I5 = -M[4] * sc, I8 = (M[0] + M[3]) * sc;
    const double c0 = I4 * I8 - I5 * I5, c1 = I1 * I8 - I5 * I2, c2 = I1 * I5 - I4 * I2;
    const double c4 = I0 * I8 - I2 * I2, c5 = I0 * I5 - I1 * I2, c8 = I0 * I4 - I1 * I1;
    const double det = I0 * c0 - I1 * c1 + I2 * c2;
    const double ox = (c0 * L[0] - c1 * L[1] + c2 * L[2]) / det;
    const double oy = (-c1 * L[0] + c4 * L[1] - c5 * L[2]) / det;
    const double oz = (c2 * L[0] - c5 * L[1] + c8 * L[2]) / det;
    for (i = 0; i < n; i++) {
      const double X = x[3 * i], Y = x[3 * i + 1], Z = x[3 * i + 2];
      v[3 * i] = v[3 * i] - oy * Z + oz * Y;
      v[3 * i + 1] = v[3 * i + 1] - oz * X + ox * Z;
      v[3 * i + 2] = v[3 * i + 2] - ox * Y + oy * X;
    }
  }
}

long sffo_npairs(const sffo_session *s) { return s->npairs; }

/* Pair list with the reference's membership rule (src/sff/nblist.c:726-746):
 * r^2 < cut^2 and not both frozen; per atom the lower part then the upper
 * part, each ascending. */
static void build_pairlist(sffo_session *s, const double *x)
{
  int n = s->n, i;
  double cut2 = s->cut * s->cut;
  long total = 0;
  int *cnt_low = xcalloc(n, sizeof(int)), *cnt_up = xcalloc(n, sizeof(int));
#pragma omp parallel for schedule(dynamic, 16)
  for (i = 0; i < n; i++) {
    int j, lo = 0, up = 0;
    for (j = 0; j < n; j++) {
      double dx, dy, dz;
      if (j == i || (s->frozen[i] && s->frozen[j])) continue;
      dx = x[3 * i] - x[3 * j];
      dy = x[3 * i + 1] - x[3 * j + 1];
      dz = x[3 * i + 2] - x[3 * j + 2];
      if (dx * dx + dy * dy + dz * dz < cut2) {
        if (j < i) lo++; else up++;
      }
    }
    cnt_low[i] = lo;
    cnt_up[i] = up;
  }
  for (i = 0; i < n; i++) {
    s->pl_start[i] = total;
    total += cnt_low[i] + cnt_up[i];
  }
  s->pl_start[n] = total;
  free(s->pl_atoms);
  s->pl_atoms = xcalloc((size_t)total, sizeof(int));
#pragma omp parallel for schedule(dynamic, 16)
  for (i = 0; i < n; i++) {
    int j;
    long k = s->pl_start[i];
    for (j = 0; j < n; j++) {
      double dx, dy, dz;
      if (j == i || (s->frozen[i] && s->frozen[j])) continue;
      dx = x[3 * i] - x[3 * j];
      dy = x[3 * i + 1] - x[3 * j + 1];
      dz = x[3 * i + 2] - x[3 * j + 2];
      if (dx * dx + dy * dy + dz * dz < cut2) s->pl_atoms[k++] = j;
    }
  }
  for (i = 0; i < n; i++) {
    s->pl_low[i] = cnt_low[i];
    s->pl_up[i] = cnt_up[i];
  }
  s->npairs = total / 2;
  s->have_list = 1;
  free(cnt_low);
  free(cnt_up);
}

static int nthreads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Threads of the parallel loops (the CPU baseline times 1 thread and all
 * host threads); buffers are sized per call, so this may change between
 * calls.  Returns the count now in effect. */
int sffo_set_threads(int n)
{
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#endif
  (void)n;
  return nthreads();
}

static int thread_id(void)
{
#ifdef _OPENMP
  return omp_get_thread_num();
#else
  return 0;
#endif
}

/* Harmonic bonds: src/sff/eff.c:82-159 (atom fields hold 3*index). */
static double bonds(int nb, const int *a1, const int *a2, const int *t, const double *rk,
                    const double *req, const double *x, double *g)
{
  double e = 0.0;
  int i;
  for (i = 0; i < nb; i++) {
    int p = a1[i], q = a2[i], ty = t[i] - 1;
    double rx = x[p] - x[q], ry = x[p + 1] - x[q + 1], rz = x[p + 2] - x[q + 2];
    double r = sqrt(rx * rx + ry * ry + rz * rz);
    double db = r - req[ty], df = rk[ty] * db;
    e += df * db;
    df *= 2.0 / r;
    g[p] += rx * df; g[p + 1] += ry * df; g[p + 2] += rz * df;
    g[q] -= rx * df; g[q + 1] -= ry * df; g[q + 2] -= rz * df;
  }
  return e;
}

/* Harmonic angles: src/sff/eff.c:168-307. */
static double angles(int na, const int *a1, const int *a2, const int *a3, const int *t,
                     const double *tk, const double *teq, const double *x, double *g)
{
  double e = 0.0;
  int i;
  for (i = 0; i < na; i++) {
    int p = a1[i], q = a2[i], r = a3[i], ty = t[i] - 1;
    double dxi = x[p] - x[q], dyi = x[p + 1] - x[q + 1], dzi = x[p + 2] - x[q + 2];
    double dxj = x[r] - x[q], dyj = x[r + 1] - x[q + 1], dzj = x[r + 2] - x[q + 2];
    double ri = sqrt(dxi * dxi + dyi * dyi + dzi * dzi);
    double rj = sqrt(dxj * dxj + dyj * dyj + dzj * dzj);
    double rir = 1.0 / ri, rjr = 1.0 / rj;
    double uxi = dxi * rir, uyi = dyi * rir, uzi = dzi * rir;
    double uxj = dxj * rjr, uyj = dyj * rjr, uzj = dzj * rjr;
    double cst = uxi * uxj + uyi * uyj + uzi * uzj, at, da, df, sn;
    if (cst > 1.0) cst = 1.0;
    if (cst < -1.0) cst = -1.0;
    at = acos(cst);
    da = at - teq[ty];
    df = da * tk[ty];
    e += df * da;
    df = df + df;
    sn = sin(at);
    if (sn > 0 && sn < 1.e-3) sn = 1.e-3;
    else if (sn < 0 && sn > -1.e-3) sn = -1.e-3;
    df = -df / sn;
    {
      double xa = df * rir * (uxj - cst * uxi), xc = df * rjr * (uxi - cst * uxj);
      double ya = df * rir * (uyj - cst * uyi), yc = df * rjr * (uyi - cst * uyj);
      double za = df * rir * (uzj - cst * uzi), zc = df * rjr * (uzi - cst * uzj);
      g[p] += xa; g[r] += xc; g[q] -= xa + xc;
      g[p + 1] += ya; g[r + 1] += yc; g[q + 1] -= ya + yc;
      g[p + 2] += za; g[r + 2] += zc; g[q + 2] -= za + zc;
    }
  }
  return e;
}

/* Cosine dihedrals: src/sff/eff.c:316-627, including the phase-0/pi
 * Chebyshev forms for n = 1..6, the general-phase path and the
 * negative-periodicity multi-term chaining. */
static double torsions(int nt, const int *a1, const int *a2, const int *a3, const int *a4,
                       const int *t, const double *pk, const double *pn, const double *phase,
                       const double *x, double *g)
{
  double etot = 0.0;
  int i;
  for (i = 0; i < nt; i++) {
    int p = a1[i], q = a2[i], r = abs(a3[i]), w = abs(a4[i]), ty = t[i] - 1;
    double ax = x[q] - x[p], ay = x[q + 1] - x[p + 1], az = x[q + 2] - x[p + 2];
    double bx = x[r] - x[q], by = x[r + 1] - x[q + 1], bz = x[r + 2] - x[q + 2];
    double cx = x[w] - x[r], cy = x[w + 1] - x[r + 1], cz = x[w + 2] - x[r + 2];
    double ab = ax * bx + ay * by + az * bz, bc = bx * cx + by * cy + bz * cz;
    double ac = ax * cx + ay * cy + az * cz, aa = ax * ax + ay * ay + az * az;
    double bb = bx * bx + by * by + bz * bz, cc = cx * cx + cy * cy + cz * cz;
    double uu = aa * bb - ab * ab, vv = bb * cc - bc * bc, uv = ab * bc - ac * bb;
    double den = uu == 0.0 ? 0.0 : 1.0 / sqrt(uu * vv);
    double co = uv * den, co1 = 0.5 * co * den;
    double a0x = -bc * bx + bb * cx, a0y = -bc * by + bb * cy, a0z = -bc * bz + bb * cz;
    double b0x = ab * cx + bc * ax - 2. * ac * bx, b0y = ab * cy + bc * ay - 2. * ac * by;
    double b0z = ab * cz + bc * az - 2. * ac * bz;
    double c0x = ab * bx - bb * ax, c0y = ab * by - bb * ay, c0z = ab * bz - bb * az;
    double a1x = 2. * uu * (-cc * bx + bc * cx), a1y = 2. * uu * (-cc * by + bc * cy);
    double a1z = 2. * uu * (-cc * bz + bc * cz);
    double b1x = 2. * uu * (bb * cx - bc * bx), b1y = 2. * uu * (bb * cy - bc * by);
    double b1z = 2. * uu * (bb * cz - bc * bz);
    double a2x = -2. * vv * (bb * ax - ab * bx), a2y = -2. * vv * (bb * ay - ab * by);
    double a2z = -2. * vv * (bb * az - ab * bz);
    double b2x = 2. * vv * (aa * bx - ab * ax), b2y = 2. * vv * (aa * by - ab * ay);
    double b2z = 2. * vv * (aa * bz - ab * az);
    double d1x = (a0x - a2x * co1) * den, d1y = (a0y - a2y * co1) * den, d1z = (a0z - a2z * co1) * den;
    double d2x = (-a0x - b0x - (a1x - a2x - b2x) * co1) * den;
    double d2y = (-a0y - b0y - (a1y - a2y - b2y) * co1) * den;
    double d2z = (-a0z - b0z - (a1z - a2z - b2z) * co1) * den;
    double d3x = (b0x - c0x - (-a1x - b1x + b2x) * co1) * den;
    double d3y = (b0y - c0y - (-a1y - b1y + b2y) * co1) * den;
    double d3z = (b0z - c0z - (-a1z - b1z + b2z) * co1) * den;
    double d4x = (c0x - b1x * co1) * den, d4y = (c0y - b1y * co1) * den, d4z = (c0z - b1z * co1) * den;
    for (;;) {
      double e, df;
      if (fabs(phase[ty] - 3.142) > 0.01 && fabs(phase[ty]) > 0.01) {
        double c = co > 1.0 ? 1.0 : (co < -1.0 ? -1.0 : co);
        double phi = acos(c), ux, uy, uz, vx, vy, vz, sx, sy, sz, delta, yy;
        ux = ay * bz - az * by; uy = az * bx - ax * bz; uz = ax * by - ay * bx;
        vx = by * cz - bz * cy; vy = bz * cx - bx * cz; vz = bx * cy - by * cx;
        sx = uy * vz - uz * vy; sy = uz * vx - ux * vz; sz = ux * vy - uy * vx;
        if (sx * bx + sy * by + sz * bz < 0.0) phi = -phi;
        delta = pn[ty] * phi - phase[ty];
        e = pk[ty] * (1.0 + cos(delta));
        yy = sin(phi);
        if (fabs(yy) > 0.001) df = pk[ty] * pn[ty] * sin(delta) / yy;
        else if (phi > -1.0 && phi < 1.0) df = pk[ty] * pn[ty] * sin(delta) * 1000.;
        else df = -pk[ty] * pn[ty] * sin(delta) * 1000.;
      } else {
        double sg = fabs(phase[ty] - 3.142) < 0.01 ? -1.0 : 1.0, k = pk[ty], c2;
        switch ((int)fabs(pn[ty])) {
          case 1: e = k * (1.0 + sg * co); df = sg * k; break;
          case 2: e = k * (1.0 + sg * (2. * co * co - 1.)); df = sg * k * 4. * co; break;
          case 3: c2 = co * co; e = k * (1.0 + sg * co * (4. * c2 - 3.)); df = sg * k * (12. * c2 - 3.); break;
          case 4: c2 = co * co; e = k * (1.0 + sg * (8. * c2 * (c2 - 1.) + 1.)); df = sg * k * co * (32. * c2 - 16.); break;
          case 5: c2 = co * co; e = k * (1.0 + sg * (16. * c2 * c2 * co - 20. * c2 * co + 5. * co)); df = sg * k * (80. * c2 * c2 - 60. * c2 + 5.); break;
          case 6: c2 = co * co; e = k * (1.0 + sg * (32. * c2 * c2 * c2 - 48. * c2 * c2 + 18. * c2 - 1.)); df = sg * k * co * (192. * c2 * c2 - 192. * c2 + 36.); break;
          default: abort();
        }
      }
      etot += e;
      g[p] += df * d1x; g[p + 1] += df * d1y; g[p + 2] += df * d1z;
      g[q] += df * d2x; g[q + 1] += df * d2y; g[q + 2] += df * d2z;
      g[r] += df * d3x; g[r + 1] += df * d3y; g[r + 2] += df * d3z;
      g[w] += df * d4x; g[w + 1] += df * d4y; g[w + 2] += df * d4z;
      if (pn[ty] < 0.0) { ty++; continue; }
      break;
    }
  }
  return etot;
}

/* Scaled 1-4 Coulomb + LJ, the diel=C branch of nbond() with N14=1
 * (src/sff/eff.c:1111-1114, 1212-1251, 1262-1310). */
static void nb14(const sffo_session *s, const double *x, double *g, double *enb, double *eel)
{
  const PARMSTRUCT_T *prm = s->prm;
  double evdw = 0.0, elec = 0.0;
  int i, k;
  for (i = 0; i < s->n - 1; i++) {
    int iaci = s->ntypes * (s->iac[i] - 1);
    double cgi = s->q[i], dx = 0.0, dy = 0.0, dz = 0.0;
    for (k = s->n14_start[i]; k < s->n14_start[i + 1]; k++) {
      int j = s->n14_atoms[k], ic;
      double enbfac = s->n14_scnb[k], cgj = s->q[j] * s->n14_scee[k];
      double xij = x[3 * i] - x[3 * j], yij = x[3 * i + 1] - x[3 * j + 1], zij = x[3 * i + 2] - x[3 * j + 2];
      double r2 = xij * xij + yij * yij + zij * zij, r2inv = 1.0 / r2, r = sqrt(r2);
      double rinv = r * r2inv, rs = cgi * cgj * rinv, df2 = -rs, df, f1, f2;
      elec += rs;
      ic = s->cno[iaci + s->iac[j] - 1];
      if (ic > 0 || enbfac != 1.0) {
        double r6 = r2inv * r2inv * r2inv;
        if (ic > 0) {
          ic--;
        } else {
          int ib = s->iac[i] > s->iac[j] ? s->iac[i] : s->iac[j];
          int is = s->iac[i] > s->iac[j] ? s->iac[j] : s->iac[i];
          ic = ib * (ib - 1) / 2 + is - 1;
        }
        f2 = s->cn2[ic] * r6;
        f1 = s->cn1[ic] * r6 * r6;
        evdw += (f1 - f2) * enbfac;
        df = (df2 + (6.0 * f2 - 12.0 * f1) * enbfac) * rinv;
      } else {
        double r10 = r2inv * r2inv * r2inv * r2inv * r2inv;
        ic = -ic - 1;
        f2 = prm->HB10[ic] * r10;
        f1 = prm->HB12[ic] * r10 * r2inv;
        evdw += (f1 - f2) * enbfac;
        df = (df2 + (10.0 * f2 - 12.0 * f1) * enbfac) * rinv;
      }
      df *= rinv;
      dx += df * xij; dy += df * yij; dz += df * zij;
      g[3 * j] -= df * xij; g[3 * j + 1] -= df * yij; g[3 * j + 2] -= df * zij;
    }
    g[3 * i] += dx; g[3 * i + 1] += dy; g[3 * i + 2] += dz;
  }
  *enb = evdw;
  *eel = elec;
}

#define TA 0.33333333333333333333
#define TB 0.4
#define TC 0.42857142857142857143
#define TD 0.44444444444444444444
#define TDD 0.45454545454545454545
#define TE 1.33333333333333333333
#define TF 2.4
#define TG 3.42857142857142857143
#define TH 4.44444444444444444444
#define THH 5.45454545454545454545

/* The three GB passes of egb(): src/sff/eff.c:1363-2417. */
static double egb(sffo_session *s, const double *x, double *g, double *enb_out, double *eel_out)
{
  const int n = s->n, nt = nthreads();
  const double rgbmax = s->rgbmax, off = s->gboffset;
  const double rgbmax1i = 1.0 / rgbmax, rgbmax2i = rgbmax1i * rgbmax1i;
  const double rgbmaxpsmax2 = (rgbmax + s->fsmax) * (rgbmax + s->fsmax);
  const double kappa = s->o.kappa, epsext = s->o.epsext;
  double epol = 0.0, elec = 0.0, evdw = 0.0;
  double *sdcopy = xcalloc((size_t)nt * n, sizeof(double));
  double *gcopy = xcalloc((size_t)nt * 3 * n, sizeof(double));
  int i;

  /* Pass 1, effective Born radii: src/sff/eff.c:1566-1733. */
#pragma omp parallel for schedule(dynamic, 8)
  for (i = 0; i < n; i++) {
    double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
    double ri = s->rborn[i] - off, ri1i = 1.0 / ri, sumi = 0.0;
    long k;
    for (k = s->pl_start[i]; k < s->pl_start[i + 1]; k++) {
      int j = s->pl_atoms[k];
      double xij = xi - x[3 * j], yij = yi - x[3 * j + 1], zij = zi - x[3 * j + 2];
      double r2 = xij * xij + yij * yij + zij * zij, dij1i, dij, sj, sj2;
      if (r2 > rgbmaxpsmax2) continue;
      dij1i = 1.0 / sqrt(r2);
      dij = r2 * dij1i;
      sj = s->fs[j] * (s->rborn[j] - off);
      sj2 = sj * sj;
      if (dij > rgbmax + sj) continue;
      if (dij > rgbmax - sj) {
        double uij = 1. / (dij - sj);
        sumi -= 0.125 * dij1i * (1.0 + 2.0 * dij * uij + rgbmax2i * (r2 - 4.0 * rgbmax * dij - sj2) +
                                 2.0 * log((dij - sj) * rgbmax1i));
      } else if (dij > 4.0 * sj) {
        double dij2i = dij1i * dij1i, tmpsd = sj2 * dij2i;
        double dumbo = TA + tmpsd * (TB + tmpsd * (TC + tmpsd * (TD + tmpsd * TDD)));
        sumi -= sj * tmpsd * dij2i * dumbo;
      } else if (dij > ri + sj) {
        sumi -= 0.5 * (sj / (r2 - sj2) + 0.5 * dij1i * log((dij - sj) / (dij + sj)));
      } else if (dij > fabs(ri - sj)) {
        double theta = 0.5 * ri1i * dij1i * (r2 + ri * ri - sj2), uij = 1. / (dij + sj);
        sumi -= 0.25 * (ri1i * (2. - theta) - uij + dij1i * log(ri * uij));
      } else if (ri < sj) {
        sumi -= 0.5 * (sj / (r2 - sj2) + 2. * ri1i + 0.5 * dij1i * log((sj - dij) / (sj + dij)));
      }
      if (s->gb == 7 || s->gb == 8) {
        if (dij < s->rborn[i] + s->rborn[j] + SFFG_GBNECK_CUT) {
          int t = s->neck[i] * 21 + s->neck[j];
          double md = dij - sffg_neck_max_pos[t], md2 = md * md, md6 = md2 * md2 * md2;
          sumi -= s->gbneckscale * (sffg_neck_max_val[t] / (1.0 + md2 + 0.3 * md6));
        }
      }
    }
    if (s->gb == 1) {
      s->reff[i] = 1.0 / (ri1i + sumi);
      if (s->reff[i] < 0.0) s->reff[i] = 30.0;
    } else {
      s->psi[i] = -ri * sumi;
      s->reff[i] = 1.0 / (ri1i - tanh((s->alpha[i] - s->beta[i] * s->psi[i] +
                                       s->gamma[i] * s->psi[i] * s->psi[i]) * s->psi[i]) /
                                      s->rborn[i]);
    }
  }

  /* Pass 2, GB + Coulomb + LJ over the upper list: src/sff/eff.c:1770-2066. */
#pragma omp parallel reduction(+ : epol, elec, evdw)
  {
    int tid = thread_id();
    double *sd = sdcopy + (size_t)tid * n, *gg = gcopy + (size_t)tid * 3 * n;
    int *iexw = xcalloc(n + 1, sizeof(int)) ;
    int ii;
    for (ii = 0; ii <= n; ii++) iexw[ii] = -1;
#pragma omp for schedule(dynamic, 8)
    for (ii = 0; ii < n; ii++) {
      double ri = s->reff[ii], qi = s->q[ii], xi, yi, zi, dax = 0, day = 0, daz = 0;
      int iaci, m;
      long k;
      if (!s->frozen[ii]) {
        double expmkf = exp(-KSCALE * kappa * ri) / epsext, dielfac = 1.0 - expmkf;
        double qi2h = 0.5 * qi * qi, qid2h = qi2h * dielfac;
        epol += -qid2h / ri;
        sd[ii] += qid2h - KSCALE * kappa * qi2h * expmkf * ri;
      }
      if (s->pl_up[ii] <= 0) continue;
      xi = x[3 * ii]; yi = x[3 * ii + 1]; zi = x[3 * ii + 2];
      iaci = s->ntypes * (s->iac[ii] - 1);
      for (m = s->ex_start[ii]; m < s->ex_start[ii + 1]; m++) iexw[s->ex_atoms[m]] = ii; /* 1-based; slot 0 = none */
      for (k = s->pl_start[ii] + s->pl_low[ii]; k < s->pl_start[ii + 1]; k++) {
        int j = s->pl_atoms[k], ic;
        double xij = xi - x[3 * j], yij = yi - x[3 * j + 1], zij = zi - x[3 * j + 2];
        double r2 = xij * xij + yij * yij + zij * zij, qiqj = qi * s->q[j], rj = s->reff[j];
        double rb2 = ri * rj, efac = exp(-r2 / (4.0 * rb2)), fgbi = 1.0 / sqrt(r2 + rb2 * efac);
        double fgbk = -kappa * KSCALE / fgbi, expmkf = exp(fgbk) / epsext, dielfac = 1.0 - expmkf;
        double temp4, temp6, de, temp5;
        epol += -qiqj * dielfac * fgbi;
        temp4 = fgbi * fgbi * fgbi;
        temp6 = qiqj * temp4 * (dielfac + fgbk * expmkf);
        de = temp6 * (1.0 - 0.25 * efac);
        temp5 = 0.5 * efac * temp6 * (rb2 + 0.25 * r2);
        sd[ii] += ri * temp5;
        sd[j] += rj * temp5;
        if (iexw[j + 1] != ii) {
          double rinv = 1. / sqrt(r2), r2inv = rinv * rinv, eel = qiqj * rinv;
          elec += eel;
          de -= eel * r2inv;
          ic = s->cno[iaci + s->iac[j] - 1] - 1;
          if (ic >= 0) {
            double r6inv = r2inv * r2inv * r2inv, f6 = s->cn2[ic] * r6inv, f12 = s->cn1[ic] * r6inv * r6inv;
            evdw += f12 - f6;
            de -= (12. * f12 - 6. * f6) * r2inv;
          }
        }
        dax += de * xij; day += de * yij; daz += de * zij;
        gg[3 * j] -= de * xij; gg[3 * j + 1] -= de * yij; gg[3 * j + 2] -= de * zij;
      }
      gg[3 * ii] += dax; gg[3 * ii + 1] += day; gg[3 * ii + 2] += daz;
    }
    free(iexw);
  }
  /* thread reductions in thread order (src/sff/eff.c:2077-2098) */
  for (i = 0; i < n; i++) {
    int t;
    double v = 0.0;
    for (t = 0; t < nt; t++) v += sdcopy[(size_t)t * n + i];
    s->sumdeijda[i] = v;
  }

  /* Pass 3, chain rule through the Born radii: src/sff/eff.c:2131-2405. */
#pragma omp parallel
  {
    int tid = thread_id(), ii;
    double *gg = gcopy + (size_t)tid * 3 * n;
#pragma omp for schedule(dynamic, 8)
    for (ii = 0; ii < n; ii++) {
      double xi, yi, zi, ri, ri1i, sumda, dax = 0, day = 0, daz = 0;
      long k;
      if (s->frozen[ii] || s->pl_start[ii + 1] == s->pl_start[ii]) continue;
      xi = x[3 * ii]; yi = x[3 * ii + 1]; zi = x[3 * ii + 2];
      ri = s->rborn[ii] - off;
      ri1i = 1.0 / ri;
      sumda = s->sumdeijda[ii];
      if (s->gb > 1) {
        double ps = s->psi[ii];
        double thi = tanh((s->alpha[ii] - s->beta[ii] * ps + s->gamma[ii] * ps * ps) * ps);
        sumda *= (s->alpha[ii] - 2.0 * s->beta[ii] * ps + 3.0 * s->gamma[ii] * ps * ps) *
                 (1.0 - thi * thi) * ri / s->rborn[ii];
      }
      for (k = s->pl_start[ii]; k < s->pl_start[ii + 1]; k++) {
        int j = s->pl_atoms[k];
        double xij = xi - x[3 * j], yij = yi - x[3 * j + 1], zij = zi - x[3 * j + 2];
        double r2 = xij * xij + yij * yij + zij * zij, dij1i, dij2i, dij, sj, sj2, datmp, t1, d3i;
        if (r2 > rgbmaxpsmax2) continue;
        dij1i = 1.0 / sqrt(r2);
        dij2i = dij1i * dij1i;
        dij = r2 * dij1i;
        sj = s->fs[j] * (s->rborn[j] - off);
        sj2 = sj * sj;
        if (dij > rgbmax + sj) continue;
        if (dij > rgbmax - sj) {
          t1 = 1. / (dij - sj);
          d3i = dij1i * dij2i;
          datmp = 0.125 * d3i * ((r2 + sj2) * (t1 * t1 - rgbmax2i) - 2.0 * log(rgbmax * t1));
        } else if (dij > 4.0 * sj) {
          double tmpsd = sj2 * dij2i;
          double dumbo = TE + tmpsd * (TF + tmpsd * (TG + tmpsd * (TH + tmpsd * THH)));
          datmp = tmpsd * sj * dij2i * dij2i * dumbo;
        } else if (dij > ri + sj) {
          t1 = 1. / (r2 - sj2);
          datmp = t1 * sj * (-0.5 * dij2i + t1) + 0.25 * dij1i * dij2i * log((dij - sj) / (dij + sj));
        } else if (dij > fabs(ri - sj)) {
          t1 = 1. / (dij + sj);
          d3i = dij2i * dij1i;
          datmp = -0.25 * (-0.5 * (r2 - ri * ri + sj2) * d3i * ri1i * ri1i + dij1i * t1 * (t1 - dij1i) -
                           d3i * log(ri * t1));
        } else if (ri < sj) {
          t1 = 1. / (r2 - sj2);
          datmp = -0.5 * (sj * dij2i * t1 - 2. * sj * t1 * t1 - 0.5 * dij2i * dij1i * log((sj - dij) / (sj + dij)));
        } else {
          datmp = 0.;
        }
        if (s->gb == 7 || s->gb == 8) {
          if (dij < s->rborn[ii] + s->rborn[j] + SFFG_GBNECK_CUT) {
            int t = s->neck[ii] * 21 + s->neck[j];
            double md = dij - sffg_neck_max_pos[t], md2 = md * md, md6 = md2 * md2 * md2;
            double den = 1.0 + md2 + 0.3 * md6;
            den = den * den * dij;
            datmp += ((2.0 * md + 1.8 * md2 * md2 * md) * sffg_neck_max_val[t] * s->gbneckscale) / den;
          }
        }
        dax += xij * datmp; day += yij * datmp; daz += zij * datmp;
        datmp *= sumda;
        gg[3 * j] += xij * datmp; gg[3 * j + 1] += yij * datmp; gg[3 * j + 2] += zij * datmp;
      }
      gg[3 * ii] -= sumda * dax; gg[3 * ii + 1] -= sumda * day; gg[3 * ii + 2] -= sumda * daz;
    }
  }
  for (i = 0; i < 3 * n; i++) {
    int t;
    for (t = 0; t < nt; t++) g[i] += gcopy[(size_t)t * 3 * n + i];
  }
  free(sdcopy);
  free(gcopy);
  *enb_out = evdw;
  *eel_out = elec;
  return epol;
}

/* mme34 energy assembly: src/sff/eff.c:2564-2874 (dim=3, gb>0). */
double sffo_mme(sffo_session *s, const double *x, double *g, double *ene, double *reff, int rebuild)
{
  const PARMSTRUCT_T *prm = s->prm;
  double e[13] = {0}, enb14, eel14, enb, eel, egbv;
  int i, k;
  if (rebuild || !s->have_list) build_pairlist(s, x);
  for (i = 0; i < 3 * s->n; i++) g[i] = 0.0;
  e[3] = bonds(prm->Nbonh, prm->BondHAt1, prm->BondHAt2, prm->BondHNum, prm->Rk, prm->Req, x, g) +
         bonds(prm->Mbona, prm->BondAt1, prm->BondAt2, prm->BondNum, prm->Rk, prm->Req, x, g);
  e[4] = angles(prm->Ntheth, prm->AngleHAt1, prm->AngleHAt2, prm->AngleHAt3, prm->AngleHNum, prm->Tk,
                prm->Teq, x, g) +
         angles(prm->Ntheta, prm->AngleAt1, prm->AngleAt2, prm->AngleAt3, prm->AngleNum, prm->Tk,
                prm->Teq, x, g);
  e[5] = torsions(prm->Nphih, prm->DihHAt1, prm->DihHAt2, prm->DihHAt3, prm->DihHAt4, prm->DihHNum,
                  prm->Pk, prm->Pn, prm->Phase, x, g) +
         torsions(prm->Mphia, prm->DihAt1, prm->DihAt2, prm->DihAt3, prm->DihAt4, prm->DihNum, prm->Pk,
                  prm->Pn, prm->Phase, x, g);
  nb14(s, x, g, &enb14, &eel14);
  e[7] = enb14;
  e[8] = eel14;
  e[9] = econs(s, x, g); /* eff.c:2663-2680 */
  egbv = egb(s, x, g, &enb, &eel);
  e[1] = enb;
  e[2] = eel;
  e[10] = egbv;
  for (i = 0; i < s->n; i++)
    if (s->frozen[i]) g[3 * i] = g[3 * i + 1] = g[3 * i + 2] = 0.0;
  e[0] = 0.0;
  for (k = 1; k <= 12; k++) e[0] += e[k];
  if (ene)
    for (k = 0; k < 13; k++) ene[k] = e[k];
  if (reff)
    for (i = 0; i < s->n; i++) reff[i] = s->reff[i];
  return e[0];
}

/* ---- the reference's serial random stream: src/sff/rand2.c:51-128 ---- */
#define IM1 2147483563
#define IM2 2147483399
#define AM (1.0 / IM1)
#define IMM1 (IM1 - 1)
#define IA1 40014
#define IA2 40692
#define IQ1 53668
#define IQ2 52774
#define IR1 12211
#define IR2 3791
#define NTAB 32
#define NDIV (1 + IMM1 / NTAB)
#define RNMX (1.0 - 1.2e-13)

static double uniform(sffo_session *s)
{
  int *seed = &s->rng_seed3, j, k;
  double t;
  if (*seed <= 0) {
    *seed = (-*seed < 1) ? 1 : -*seed;
    s->rng_seed2 = *seed;
    for (j = NTAB + 7; j >= 0; j--) {
      k = *seed / IQ1;
      *seed = IA1 * (*seed - k * IQ1) - k * IR1;
      if (*seed < 0) *seed += IM1;
      if (j < NTAB) s->rng_iv[j] = *seed;
    }
    s->rng_iy = s->rng_iv[0];
  }
  k = *seed / IQ1;
  *seed = IA1 * (*seed - k * IQ1) - k * IR1;
  if (*seed < 0) *seed += IM1;
  k = s->rng_seed2 / IQ2;
  s->rng_seed2 = IA2 * (s->rng_seed2 - k * IQ2) - k * IR2;
  if (s->rng_seed2 < 0) s->rng_seed2 += IM2;
  j = s->rng_iy / NDIV;
  s->rng_iy = s->rng_iv[j] - s->rng_seed2;
  s->rng_iv[j] = *seed;
  if (s->rng_iy < 1) s->rng_iy += IMM1;
  t = AM * s->rng_iy;
  return t > RNMX ? RNMX : t;
}

static double gaussian(sffo_session *s, double mean, double sd)
{
  double s1, s2, rsq;
  do {
    s1 = 2. * uniform(s) - 1.;
    s2 = 2. * uniform(s) - 1.;
    rsq = s1 * s1 + s2 * s2;
  } while (rsq >= 1. || rsq == 0.0);
  return sd * (s1 * sqrt(-2. * log(rsq) / rsq)) + mean;
}

void sffo_gauss_stream(int *seed, int n, double mean, const double *sd, double *out)
{
  sffo_session tmp;
  int i;
  memset(&tmp, 0, sizeof(tmp));
  tmp.rng_seed3 = *seed;
  for (i = 0; i < n; i++) out[i] = gaussian(&tmp, mean, sd[i]);
  *seed = tmp.rng_seed3;
}

/* mme() iteration protocol for list rebuilds: src/sff/eff.c:2564-2566. */
static double eval_iter(sffo_session *s, const double *x, double *g, int iter)
{
  int rebuild = !s->have_list || (iter > 0 && iter % s->o.nsnb == 0) || iter == -4;
  return sffo_mme(s, x, g, NULL, NULL, rebuild);
}

/* md(): src/sff/sff.c:2071-2366 (no RATTLE, no COM removal, nothing frozen
 * beyond the frozen mask). */
int sffo_md(sffo_session *s, int maxstep, double *x, double *f, double *v, int *seed, double *trace)
{
  const int n = 3 * s->n;
  const double boltz2 = 9.93595e-4;
  double *minv = xcalloc(n, sizeof(double)), *sqrmass = xcalloc(n, sizeof(double));
  double *accel = xcalloc(n, sizeof(double));
  double dtx = s->o.dt * 20.455, dt5 = 0.5 * dtx, rndf, ekin0, dttp, gammai, c_implic, c_explic, c_ave;
  double sdfac, ekin, epot, tscal;
  int nfrozen = 0, i, nstep;
  for (i = 0; i < s->n; i++) nfrozen += s->frozen[i] ? 1 : 0;
  s->rng_seed3 = *seed;
  rndf = n - 3 * nfrozen;
  ekin0 = boltz2 * rndf * s->o.temp0;
  dttp = s->o.dt / s->o.tautp;
  gammai = s->o.gamma_ln / 20.455;
  c_implic = 1.0 / (1.0 + gammai * dt5);
  c_explic = 1.0 - gammai * dt5;
  c_ave = 1.0 + gammai * dt5;
  sdfac = sqrt(4.0 * gammai * boltz2 * s->o.temp0 / dtx);
  for (i = 0; i < s->n; i++) minv[3 * i] = minv[3 * i + 1] = minv[3 * i + 2] = 1. / s->prm->Masses[i];
  if (s->o.zerov) {
    for (i = 0; i < n; i++) v[i] = 0.0;
    ekin = 0.0;
  } else if (s->o.tempi > 0.0) {
    ekin = 0.0;
    for (i = 0; i < n; i++) {
      if (s->frozen[i / 3]) {
        v[i] = 0.0;
      } else {
        v[i] = gaussian(s, 0.0, sqrt(2. * boltz2 * s->o.tempi * minv[i]));
        ekin += v[i] * v[i] / minv[i];
      }
    }
    ekin *= 0.5;
  } else {
    ekin = 0.0;
    for (i = 0; i < n; i++) ekin += v[i] * v[i] * minv[i];
    ekin *= 0.5;
  }
  epot = eval_iter(s, x, f, 0);
  if (gammai == 0.0) {
    for (i = 0; i < n; i++) accel[i] = -f[i] * minv[i] * dt5;
  } else {
    for (i = 0; i < n; i++) {
      if (s->frozen[i / 3]) {
        accel[i] = 0.0;
      } else {
        sqrmass[i] = 1.0 / sqrt(minv[i]);
        accel[i] = (-f[i] + gaussian(s, 0.0, sdfac * sqrmass[i])) * minv[i] * dt5;
      }
    }
  }
  for (nstep = 1; nstep <= maxstep; nstep++) {
    tscal = ekin > 0.01 ? sqrt(1. + dttp * (ekin0 / ekin - 1.)) : 1.0;
    ekin = 0.0;
    for (i = 0; i < n; i++) {
      v[i] = gammai == 0.0 ? (v[i] + accel[i]) * tscal : c_explic * v[i] + accel[i];
      if (v[i] > s->o.vlimit) v[i] = s->o.vlimit;
      if (v[i] < -s->o.vlimit) v[i] = -s->o.vlimit;
      x[i] += v[i] * dtx;
    }
    epot = eval_iter(s, x, f, nstep);
    if (gammai == 0.0) {
      for (i = 0; i < n; i++) {
        accel[i] = -f[i] * minv[i] * dt5;
        v[i] = (v[i] + accel[i]) * tscal;
      }
    } else {
      for (i = 0; i < n; i++) {
        if (!s->frozen[i / 3]) {
          accel[i] = (-f[i] + gaussian(s, 0.0, sdfac * sqrmass[i])) * minv[i] * dt5;
          v[i] = (v[i] + accel[i]) * c_implic;
        }
      }
    }
    for (i = 0; i < n; i++) ekin += v[i] * v[i] / minv[i];
    ekin *= 0.5;
    if (gammai > 0.) ekin *= c_ave;
    if (trace) {
      trace[2 * (nstep - 1)] = ekin;
      trace[2 * (nstep - 1) + 1] = epot;
    }
    /* sff.c:2346-2351 */
    if (s->o.nscm > 0 && nstep % s->o.nscm == 0) com_remove(s->n, x, v, minv, gammai == 0.0);
  }
  *seed = s->rng_seed3;
  free(minv);
  free(sqrmass);
  free(accel);
  return 0;
}

/* conjgrad(): src/sff/conjgrad.c:34-263, the same labels as a state machine
 * (arrays 1-based as in the reference). */
int sffo_conjgrad(sffo_session *s, double *x0, double *fret, double rmsgrad, double dfpred, int maxiter,
                  double *etrace, int *nevals)
{
  const int n = 3 * s->n, maxlin = 10, mxfcon = 4;
  double *w = xcalloc(6 * (size_t)n + 1, sizeof(double)), *g = xcalloc((size_t)n + 1, sizeof(double));
  double *x = x0 - 1, f = 0.0;
  double dgrad = rmsgrad * rmsgrad * n;
  double gama = 0, beta, fmin = 0, gmin = 0, dfpr = 0, gnew = 0, step = 0, work, finit = 0, ginit = 0;
  double gsqrd = 0, gspln, stmin = 0, gamden = 0, ddspln = 0, stepch = 0, sbound = 0, fch = 0, sum = 0;
  int niter = 0, i, nfbeg = 0, iterc = 0, nfopt = 0, iterfm = 0, iterrs = 0, iretry = 0, ier = 0, ret;
  const int irsdx = n, irsdg = 2 * n, iginit = 3 * n, ixopt = 4 * n, igopt = 5 * n;
  int label = 10;
  for (;;) {
    switch (label) {
      case 10:
        ++niter;
        f = eval_iter(s, x + 1, g + 1, niter - 1);
        if (etrace && niter - 1 <= maxiter) etrace[niter - 1] = f;
        if (niter >= 2) { label = 30; break; }
        /* fall through */
      case 20:
        for (i = 1; i <= n; ++i) w[i] = -g[i];
        iterrs = 0;
        if (iterc > 0) { label = 40; break; }
        /* fall through */
      case 30:
        gnew = 0.0;
        sum = 0.0;
        for (i = 1; i <= n; ++i) {
          gnew += w[i] * g[i];
          sum += g[i] * g[i];
        }
        if (niter == 1) {
          fmin = f;
          gsqrd = sum;
          nfopt = niter;
          for (i = 1; i <= n; ++i) { w[ixopt + i] = x[i]; w[igopt + i] = g[i]; }
          if (sum <= dgrad) { label = 100; break; }
        } else {
          fch = f - fmin;
          if (fch < 0.0 || (fch == 0.0 && gnew / gmin >= -1.0)) {
            fmin = f;
            gsqrd = sum;
            nfopt = niter;
            for (i = 1; i <= n; ++i) { w[ixopt + i] = x[i]; w[igopt + i] = g[i]; }
            if (sum <= dgrad) { label = 100; break; }
          }
        }
        if (niter == maxiter + 1) { ier = -3; label = 100; break; }
        if (niter > 1) { label = 60; break; }
        dfpr = dfpred;
        stmin = dfpred / gsqrd;
        /* fall through */
      case 40:
        ++iterc;
        finit = f;
        ginit = 0.0;
        for (i = 1; i <= n; ++i) {
          w[iginit + i] = g[i];
          ginit += w[i] * g[i];
        }
        if (ginit >= 0.0) { ier = -2; label = 90; break; }
        gmin = ginit;
        sbound = -1.0;
        nfbeg = niter;
        iretry = -1;
        {
          double a = fabs(dfpr / ginit);
          stepch = stmin <= a ? stmin : a;
        }
        stmin = 0.0;
        /* fall through */
      case 50:
        step = stmin + stepch;
        work = 0.0;
        for (i = 1; i <= n; ++i) {
          double d;
          x[i] = w[ixopt + i] + stepch * w[i];
          d = fabs(x[i] - w[ixopt + i]);
          work = work >= d ? work : d;
        }
        if (work > 0.0) { label = 10; break; }
        if (niter > nfbeg + 1) ier = -1;
        if (fabs(gmin / ginit) > 0.2) ier = -1;
        label = 90;
        break;
      case 60:
        work = (fch + fch) / stepch - gnew - gmin;
        ddspln = (gnew - gmin) / stepch;
        if (niter > nfopt) sbound = step;
        if (niter <= nfopt) {
          if (gmin * gnew <= 0.0) sbound = stmin;
          stmin = step;
          gmin = gnew;
          stepch = -stepch;
        }
        if (fch != 0.0) ddspln += (work + work) / stepch;
        if (gmin == 0.0) { label = 90; break; }
        if (niter > nfbeg + 1) {
          if (fabs(gmin / ginit) <= 0.2) { label = 90; break; }
          if (niter >= nfopt + maxlin) { ier = -1; label = 90; break; }
        }
        /* fall through */
      case 70:
        stepch = (sbound - stmin) * 0.5;
        if (sbound < -0.5) stepch = stmin * 9.0;
        gspln = gmin + stepch * ddspln;
        if (gmin * gspln < 0.0) stepch = stepch * gmin / (gmin - gspln);
        label = 50;
        break;
      case 80:
        sum = 0.0;
        for (i = 1; i <= n; ++i) sum += g[i] * w[iginit + i];
        beta = (gsqrd - sum) / (gmin - ginit);
        if (fabs(beta * gmin) > gsqrd * 0.2) {
          ++iretry;
          if (iretry <= 0) {
            if (niter >= nfopt + maxlin) { ier = -1; label = 90; break; }
            label = 70;
            break;
          }
        }
        if (f < finit) iterfm = iterc;
        if (iterc >= iterfm + mxfcon) { ier = -4; label = 100; break; }
        dfpr = stmin * ginit;
        if (iretry > 0) { label = 20; break; }
        if (iterrs != 0 && iterc - iterrs < n && fabs(sum) < gsqrd * 0.2) {
          double gs = 0.0;
          gama = 0.0;
          for (i = 1; i <= n; ++i) {
            gama += g[i] * w[irsdg + i];
            gs += g[i] * w[irsdx + i];
          }
          gama /= gamden;
          if (fabs(beta * gmin + gama * gs) < gsqrd * 0.2) {
            for (i = 1; i <= n; ++i) w[i] = -g[i] + beta * w[i] + gama * w[irsdx + i];
            label = 40;
            break;
          }
        }
        gamden = gmin - ginit;
        for (i = 1; i <= n; ++i) {
          w[irsdx + i] = w[i];
          w[irsdg + i] = g[i] - w[iginit + i];
          w[i] = -g[i] + beta * w[i];
        }
        iterrs = iterc;
        label = 40;
        break;
      case 90:
        if (niter != nfopt) {
          f = fmin;
          for (i = 1; i <= n; ++i) { x[i] = w[ixopt + i]; g[i] = w[igopt + i]; }
        }
        if (ier == 0) { label = 80; break; }
        /* fall through */
      case 100:
        goto done;
    }
  }
done:
  ret = ier == 0 ? niter : ier;
  *fret = f;
  if (nevals) *nevals = niter;
  free(w);
  free(g);
  return ret;
}
