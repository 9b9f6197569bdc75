/*
 * synth.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the library's synthetic-molecule generator
 * (nabc_gb300/csrc/synth.cpp, sffg_synth_molecule), so that the CPU
 * baseline and the reference arm of bench.py can make their inputs without
 * loading the library they are compared with.  tests/test_host.py checks
 * that both produce the same coordinates and topology arrays, bit for bit
 * (both are compiled without floating-point contraction).
 *
 * The molecule: one compact, self-avoiding chain (bond 1.53 A, angle
 * 111 degrees, uniform dihedrals, no atom within 2.5 A of an atom other
 * than its two chain predecessors, inside a sphere of radius
 * (3N/(4 pi 0.09))^(1/3) A that grows by 1% when growth stalls); C/N/O/H
 * atoms with probabilities 0.32/0.09/0.09/0.50; charges N(0, 0.4^2) shifted
 * to net zero; the GB radii, screens, LJ parameters, bonded terms and 1-2 /
 * 1-3 / 1-4 exclusions of the generator.  Only the PARMSTRUCT_T fields the
 * oracle reads are filled (no names, residues or tree data).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "sffo.h"

/* xoshiro256** seeded by splitmix64 */
typedef struct { uint64_t s[4]; } rng_t;

static void rng_seed(rng_t *r, uint64_t seed)
{
  uint64_t z = seed;
  for (int k = 0; k < 4; k++) {
    z += 0x9E3779B97F4A7C15ULL;
    uint64_t t = z;
    t = (t ^ (t >> 30)) * 0xBF58476D1CE4E5B9ULL;
    t = (t ^ (t >> 27)) * 0x94D049BB133111EBULL;
    r->s[k] = t ^ (t >> 31);
  }
}

static uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t rng_next(rng_t *r)
{
  uint64_t *s = r->s;
  const uint64_t out = rotl64(s[1] * 5, 7) * 9, t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl64(s[3], 45);
  return out;
}

static double rng_uniform(rng_t *r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }

static double rng_gaussian(rng_t *r)
{
  double u1 = rng_uniform(r);
  const double u2 = rng_uniform(r);
  if (u1 < 1e-300) u1 = 1e-300;
  return sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}

typedef struct { double x, y, z; } v3;

static v3 vsub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static v3 vadd(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static v3 vscale(double s, v3 a) { v3 r = {s * a.x, s * a.y, s * a.z}; return r; }
static double vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 vcross(v3 a, v3 b)
{
  v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
  return r;
}
static v3 vunit(v3 a) { return vscale(1.0 / sqrt(vdot(a, a)), a); }

/* atom D from A, B, C: |CD| = bond, angle BCD = theta, dihedral ABCD = phi */
static v3 place(v3 a, v3 b, v3 c, double bond, double theta, double phi)
{
  const v3 bc = vunit(vsub(c, b));
  const v3 n = vunit(vcross(vsub(b, a), bc));
  const v3 m = vcross(n, bc);
  const double dx = -bond * cos(theta), dy = bond * sin(theta) * cos(phi), dz = bond * sin(theta) * sin(phi);
  return vadd(c, vadd(vadd(vscale(dx, bc), vscale(dy, m)), vscale(dz, n)));
}

static v3 random_unit(rng_t *r)
{
  const double z = 2.0 * rng_uniform(r) - 1.0;
  const double t = 2.0 * M_PI * rng_uniform(r);
  const double s = sqrt(1.0 - z * z);
  v3 u = {s * cos(t), s * sin(t), z};
  return u;
}

/* Spatial hash of the placed atoms, 2.5 A cells: open addressing on the
 * packed cell key, a singly linked list of atoms per cell. */
typedef struct {
  double h;
  size_t cap, used;       /* cap: a power of two; used: cells ever made */
  uint64_t *key;          /* UINT64_MAX: empty */
  int *head;              /* first atom of the cell, -1 none */
  int *next;              /* per atom */
} grid_t;

static long cellof(const grid_t *g, double v) { return (long)floor(v / g->h); }

static uint64_t pack3(long a, long b, long c)
{
  return ((uint64_t)(a + (1 << 20)) << 42) | ((uint64_t)(b + (1 << 20)) << 21) | (uint64_t)(c + (1 << 20));
}

static size_t probe(const uint64_t *key, size_t cap, uint64_t k)
{
  size_t i = (size_t)((k * 0x9E3779B97F4A7C15ULL) >> 20) & (cap - 1);
  while (key[i] != UINT64_MAX && key[i] != k) i = (i + 1) & (cap - 1);
  return i;
}

/* doubles the table (cells keep their atom lists) */
static void grid_grow(grid_t *g)
{
  const size_t cap = 2 * g->cap;
  uint64_t *key = malloc(cap * sizeof(uint64_t));
  int *head = malloc(cap * sizeof(int));
  for (size_t k = 0; k < cap; k++) key[k] = UINT64_MAX;
  for (size_t k = 0; k < g->cap; k++)
    if (g->key[k] != UINT64_MAX) {
      const size_t i = probe(key, cap, g->key[k]);
      key[i] = g->key[k];
      head[i] = g->head[k];
    }
  free(g->key);
  free(g->head);
  g->key = key;
  g->head = head;
  g->cap = cap;
}

static size_t slot_of(grid_t *g, uint64_t k, int insert)
{
  size_t i = probe(g->key, g->cap, k);
  if (g->key[i] == UINT64_MAX && insert) {
    if (2 * (g->used + 1) > g->cap) {
      grid_grow(g);
      i = probe(g->key, g->cap, k);
    }
    g->key[i] = k;
    g->head[i] = -1;
    g->used++;
  }
  return i;
}

static uint64_t pkey(const grid_t *g, v3 p) { return pack3(cellof(g, p.x), cellof(g, p.y), cellof(g, p.z)); }

static void grid_add(grid_t *g, int i, v3 p)
{
  const size_t c = slot_of(g, pkey(g, p), 1);
  g->next[i] = g->head[c];
  g->head[c] = i;
}

static void grid_remove(grid_t *g, int i, v3 p)
{
  const size_t c = slot_of(g, pkey(g, p), 0);
  int *link = &g->head[c];
  while (*link >= 0 && *link != i) link = &g->next[*link];
  if (*link == i) *link = g->next[i];
}

/* true if an atom other than ex1, ex2 lies within d of p */
static int grid_clash(grid_t *g, v3 p, double d, const v3 *pos, int ex1, int ex2)
{
  const long cx = cellof(g, p.x), cy = cellof(g, p.y), cz = cellof(g, p.z);
  const double d2 = d * d;
  for (long a = cx - 1; a <= cx + 1; a++)
    for (long b = cy - 1; b <= cy + 1; b++)
      for (long c = cz - 1; c <= cz + 1; c++) {
        const size_t s = slot_of(g, pack3(a, b, c), 0);
        if (g->key[s] == UINT64_MAX) continue;
        for (int j = g->head[s]; j >= 0; j = g->next[j]) {
          if (j == ex1 || j == ex2) continue;
          const v3 q = vsub(pos[j], p);
          if (vdot(q, q) < d2) return 1;
        }
      }
  return 0;
}

static int inside(v3 p, double radius) { return vdot(p, p) <= radius * radius; }

/* Grows the chain into pos[n]; returns the realised confining radius. */
static double grow_chain(int n, uint64_t seed, v3 *pos)
{
  const double bond = 1.53, theta = 111.0 * M_PI / 180.0, dmin = 2.5;
  double radius = cbrt(3.0 * n / (4.0 * M_PI * 0.09));
  rng_t rng;
  rng_seed(&rng, seed ^ 0xC0FFEEULL);
  grid_t g;
  g.h = dmin;
  g.used = 0;
  g.cap = 1;
  while (g.cap < 4 * (size_t)n + 64) g.cap <<= 1;
  g.key = malloc(g.cap * sizeof(uint64_t));
  g.head = malloc(g.cap * sizeof(int));
  g.next = malloc((size_t)n * sizeof(int));
  for (size_t k = 0; k < g.cap; k++) g.key[k] = UINT64_MAX;
  memset(pos, 0, (size_t)n * sizeof(v3));
  for (;;) {
    const v3 dir = random_unit(&rng);  /* the direction first, then the distance */
    const v3 p0 = vscale(0.3 * radius * cbrt(rng_uniform(&rng)), dir);
    const v3 p1 = vadd(p0, vscale(bond, random_unit(&rng)));
    const v3 u = vunit(vsub(p1, p0));
    const v3 w = random_unit(&rng);
    const v3 perp = vunit(vsub(w, vscale(vdot(w, u), u)));
    const v3 p2 = vadd(p1, vscale(bond, vadd(vscale(-cos(theta), u), vscale(sin(theta), perp))));
    if (n < 3 || (inside(p0, radius) && inside(p1, radius) && inside(p2, radius))) {
      pos[0] = p0;
      if (n > 1) pos[1] = p1;
      if (n > 2) pos[2] = p2;
      break;
    }
  }
  for (int i = 0; i < n && i < 3; i++) grid_add(&g, i, pos[i]);
  int i = 3, consecutive_fail = 0, best = 3, stall = 0;
  const int tries = 64, kstall = 48;
  while (i < n) {
    int ok = 0;
    for (int t = 0; t < tries; t++) {
      const v3 p = place(pos[i - 3], pos[i - 2], pos[i - 1], bond, theta, 2.0 * M_PI * rng_uniform(&rng));
      if (!inside(p, radius) || grid_clash(&g, p, dmin, pos, i - 1, i - 2)) continue;
      pos[i] = p;
      grid_add(&g, i, p);
      ok = 1;
      break;
    }
    if (ok) {
      i++;
      if (i > best) {
        best = i;
        stall = 0;
        consecutive_fail = 0;
      }
      continue;
    }
    if (++stall > kstall) {
      radius *= 1.01;
      stall = 0;
      consecutive_fail = 0;
    }
    const int back = 1 << (consecutive_fail < 6 ? consecutive_fail : 6);
    consecutive_fail++;
    for (int k = 0; k < back && i > 3; k++) {
      i--;
      grid_remove(&g, i, pos[i]);
    }
  }
  free(g.key);
  free(g.head);
  free(g.next);
  return radius;
}

static void *zalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz); }

/* The molecule of sffg_synth_molecule(natom, seed): x[3 natom] coordinates,
 * *radius_out the confining radius; NULL for natom < 4.  Free with
 * sffo_synth_free. */
PARMSTRUCT_T *sffo_synth_molecule(int natom, unsigned long long seed, double *x, double *radius_out)
{
  if (natom < 4) return NULL;
  v3 *pos = malloc((size_t)natom * sizeof(v3));
  const double radius = grow_chain(natom, seed, pos);
  if (radius_out) *radius_out = radius;
  for (int i = 0; i < natom; i++) {
    x[3 * i] = pos[i].x;
    x[3 * i + 1] = pos[i].y;
    x[3 * i + 2] = pos[i].z;
  }
  free(pos);
  rng_t rng;
  rng_seed(&rng, seed ^ 0xA70B5ULL);
  int *el = malloc((size_t)natom * sizeof(int));  /* 0 C, 1 N, 2 O, 3 H */
  for (int i = 0; i < natom; i++) {
    const double u = rng_uniform(&rng);
    el[i] = u < 0.32 ? 0 : u < 0.41 ? 1 : u < 0.50 ? 2 : 3;
  }
  double *q = malloc((size_t)natom * sizeof(double));
  double mean = 0.0;
  for (int i = 0; i < natom; i++) {
    q[i] = 0.4 * rng_gaussian(&rng);
    mean += q[i];
  }
  mean /= natom;

  static const double rstar[4] = {1.908, 1.824, 1.6612, 0.6};
  static const double eps[4] = {0.086, 0.17, 0.21, 0.0157};
  static const double mass[4] = {12.01, 14.01, 16.00, 1.008};
  static const double radii[4] = {1.7, 1.55, 1.5, 1.2};
  static const double screen[4] = {0.72, 0.79, 0.85, 0.85};
  static const int znum[4] = {6, 7, 8, 1};

  PARMSTRUCT_T *prm = calloc(1, sizeof(PARMSTRUCT_T));
#define ISH(a) (el[(a)] == 3)
  int nbh = 0, nba = 0, nth = 0, nta = 0, nph = 0, npa = 0;
  for (int i = 0; i + 1 < natom; i++) (ISH(i) || ISH(i + 1)) ? nbh++ : nba++;
  for (int i = 0; i + 2 < natom; i++) (ISH(i) || ISH(i + 1) || ISH(i + 2)) ? nth++ : nta++;
  for (int i = 0; i + 3 < natom; i++) (ISH(i) || ISH(i + 1) || ISH(i + 2) || ISH(i + 3)) ? nph++ : npa++;
  prm->Natom = natom;
  prm->Ntypes = 4;
  prm->Nbonh = nbh;
  prm->Mbona = prm->Nbona = nba;
  prm->Ntheth = nth;
  prm->Mtheta = prm->Ntheta = nta;
  prm->Nphih = nph;
  prm->Mphia = prm->Nphia = npa;
  prm->Numbnd = prm->Numang = prm->Nptra = prm->Natyp = 1;
  prm->Nat3 = 3 * natom;
  prm->Ntype2d = 16;
  prm->Nttyp = 10;
  int nnb = 0;
  for (int i = 0; i < natom; i++) {
    const int k = (i + 1 < natom) + (i + 2 < natom) + (i + 3 < natom);
    nnb += k ? k : 1;
  }
  prm->Nnb = nnb;
  prm->Charges = zalloc(natom, sizeof(double));
  prm->Masses = zalloc(natom, sizeof(double));
  prm->Iac = zalloc(natom, sizeof(int));
  prm->Iblo = zalloc(natom, sizeof(int));
  prm->Rborn = zalloc(natom, sizeof(double));
  prm->Fs = zalloc(natom, sizeof(double));
  prm->AtomicNum = zalloc(natom, sizeof(int));
  prm->Cno = zalloc(16, sizeof(int));
  prm->Cn1 = zalloc(10, sizeof(double));
  prm->Cn2 = zalloc(10, sizeof(double));
  prm->HB12 = zalloc(1, sizeof(double));
  prm->HB10 = zalloc(1, sizeof(double));
  prm->ExclAt = zalloc(nnb, sizeof(int));
  prm->Rk = zalloc(1, sizeof(double));
  prm->Req = zalloc(1, sizeof(double));
  prm->Tk = zalloc(1, sizeof(double));
  prm->Teq = zalloc(1, sizeof(double));
  prm->Pk = zalloc(1, sizeof(double));
  prm->Pn = zalloc(1, sizeof(double));
  prm->Phase = zalloc(1, sizeof(double));
  prm->Scee = zalloc(1, sizeof(double));
  prm->Scnb = zalloc(1, sizeof(double));
  prm->BondHAt1 = zalloc(nbh, sizeof(int));
  prm->BondHAt2 = zalloc(nbh, sizeof(int));
  prm->BondHNum = zalloc(nbh, sizeof(int));
  prm->BondAt1 = zalloc(nba, sizeof(int));
  prm->BondAt2 = zalloc(nba, sizeof(int));
  prm->BondNum = zalloc(nba, sizeof(int));
  prm->AngleHAt1 = zalloc(nth, sizeof(int));
  prm->AngleHAt2 = zalloc(nth, sizeof(int));
  prm->AngleHAt3 = zalloc(nth, sizeof(int));
  prm->AngleHNum = zalloc(nth, sizeof(int));
  prm->AngleAt1 = zalloc(nta, sizeof(int));
  prm->AngleAt2 = zalloc(nta, sizeof(int));
  prm->AngleAt3 = zalloc(nta, sizeof(int));
  prm->AngleNum = zalloc(nta, sizeof(int));
  prm->DihHAt1 = zalloc(nph, sizeof(int));
  prm->DihHAt2 = zalloc(nph, sizeof(int));
  prm->DihHAt3 = zalloc(nph, sizeof(int));
  prm->DihHAt4 = zalloc(nph, sizeof(int));
  prm->DihHNum = zalloc(nph, sizeof(int));
  prm->DihAt1 = zalloc(npa, sizeof(int));
  prm->DihAt2 = zalloc(npa, sizeof(int));
  prm->DihAt3 = zalloc(npa, sizeof(int));
  prm->DihAt4 = zalloc(npa, sizeof(int));
  prm->DihNum = zalloc(npa, sizeof(int));
  prm->N14pairs = zalloc(natom, sizeof(int));

  for (int i = 0; i < natom; i++) {
    prm->Charges[i] = (q[i] - mean) * 18.2223;
    prm->Masses[i] = mass[el[i]];
    prm->Iac[i] = el[i] + 1;
    prm->Rborn[i] = radii[el[i]];
    prm->Fs[i] = screen[el[i]];
    prm->AtomicNum[i] = znum[el[i]];
  }
  for (int a = 0; a < 4; a++)
    for (int b = 0; b < 4; b++) {
      const int big = (a > b ? a : b) + 1, small = (a > b ? b : a) + 1;
      const int ic = big * (big - 1) / 2 + small;  /* 1-based */
      prm->Cno[a * 4 + b] = ic;
      const double r = rstar[a] + rstar[b], e = sqrt(eps[a] * eps[b]);
      prm->Cn1[ic - 1] = e * pow(r, 12);
      prm->Cn2[ic - 1] = 2.0 * e * pow(r, 6);
    }
  prm->Rk[0] = 300.0;
  prm->Req[0] = 1.53;
  prm->Tk[0] = 50.0;
  prm->Teq[0] = 111.0 * M_PI / 180.0;
  prm->Pk[0] = 1.4;
  prm->Pn[0] = 3.0;
  prm->Phase[0] = 0.0;
  prm->Scee[0] = 1.0 / 1.2;
  prm->Scnb[0] = 1.0 / 2.0;
  nbh = nba = nth = nta = nph = npa = 0;
  for (int i = 0; i + 1 < natom; i++) {
    if (ISH(i) || ISH(i + 1)) {
      prm->BondHAt1[nbh] = 3 * i; prm->BondHAt2[nbh] = 3 * (i + 1); prm->BondHNum[nbh++] = 1;
    } else {
      prm->BondAt1[nba] = 3 * i; prm->BondAt2[nba] = 3 * (i + 1); prm->BondNum[nba++] = 1;
    }
  }
  for (int i = 0; i + 2 < natom; i++) {
    if (ISH(i) || ISH(i + 1) || ISH(i + 2)) {
      prm->AngleHAt1[nth] = 3 * i; prm->AngleHAt2[nth] = 3 * (i + 1);
      prm->AngleHAt3[nth] = 3 * (i + 2); prm->AngleHNum[nth++] = 1;
    } else {
      prm->AngleAt1[nta] = 3 * i; prm->AngleAt2[nta] = 3 * (i + 1);
      prm->AngleAt3[nta] = 3 * (i + 2); prm->AngleNum[nta++] = 1;
    }
  }
  for (int i = 0; i + 3 < natom; i++) {
    if (ISH(i) || ISH(i + 1) || ISH(i + 2) || ISH(i + 3)) {
      prm->DihHAt1[nph] = 3 * i; prm->DihHAt2[nph] = 3 * (i + 1); prm->DihHAt3[nph] = 3 * (i + 2);
      prm->DihHAt4[nph] = 3 * (i + 3); prm->DihHNum[nph++] = 1;
    } else {
      prm->DihAt1[npa] = 3 * i; prm->DihAt2[npa] = 3 * (i + 1); prm->DihAt3[npa] = 3 * (i + 2);
      prm->DihAt4[npa] = 3 * (i + 3); prm->DihNum[npa++] = 1;
    }
  }
#undef ISH
  int k = 0;
  for (int i = 0; i < natom; i++) {
    int cnt = 0;
    for (int d = 1; d <= 3; d++)
      if (i + d < natom) {
        prm->ExclAt[k++] = i + d + 1;  /* 1-based */
        cnt++;
      }
    if (!cnt) prm->ExclAt[k++] = 0;
    prm->Iblo[i] = cnt ? cnt : 1;
  }
  /* Fsmax with the fixed offset 0.09 (src/sff/prm.c:1652-1656) */
  prm->Fsmax = 0.0;
  for (int i = 0; i < natom; i++) {
    const double s = prm->Fs[i] * (prm->Rborn[i] - 0.09);
    if (s > prm->Fsmax) prm->Fsmax = s;
  }
  /* 1-4 list keyed on the smaller end atom (src/sff/prm.c:1855-1900); a
   * chain's dihedrals i..i+3 give atom i the one partner i+3, in the
   * generator's order: H-containing dihedrals first, then the others */
  for (int d = 0; d < nph; d++) prm->N14pairs[prm->DihHAt1[d] / 3]++;
  for (int d = 0; d < npa; d++) prm->N14pairs[prm->DihAt1[d] / 3]++;
  const int total = nph + npa;
  prm->N14pairlist = zalloc(total, sizeof(int));
  prm->N14sceelist = zalloc(total, sizeof(double));
  prm->N14scnblist = zalloc(total, sizeof(double));
  k = 0;
  for (int i = 0; i < natom - 1; i++)
    for (int m = 0; m < prm->N14pairs[i]; m++) {
      prm->N14pairlist[k] = i + 3;
      prm->N14sceelist[k] = prm->Scee[0];
      prm->N14scnblist[k] = prm->Scnb[0];
      k++;
    }
  free(el);
  free(q);
  return prm;
}

/* Two fields of the struct for callers without its layout (ctypes). */
int sffo_prm_natom(const PARMSTRUCT_T *prm) { return prm->Natom; }
double sffo_prm_fsmax(const PARMSTRUCT_T *prm) { return prm->Fsmax; }

void sffo_synth_free(PARMSTRUCT_T *prm)
{
  if (!prm) return;
  void *p[] = {prm->Charges, prm->Masses, prm->Iac, prm->Iblo, prm->Rborn, prm->Fs, prm->AtomicNum, prm->Cno,
               prm->Cn1, prm->Cn2, prm->HB12, prm->HB10, prm->ExclAt, prm->Rk, prm->Req, prm->Tk, prm->Teq,
               prm->Pk, prm->Pn, prm->Phase, prm->Scee, prm->Scnb, prm->BondHAt1, prm->BondHAt2, prm->BondHNum,
               prm->BondAt1, prm->BondAt2, prm->BondNum, prm->AngleHAt1, prm->AngleHAt2, prm->AngleHAt3,
               prm->AngleHNum, prm->AngleAt1, prm->AngleAt2, prm->AngleAt3, prm->AngleNum, prm->DihHAt1,
               prm->DihHAt2, prm->DihHAt3, prm->DihHAt4, prm->DihHNum, prm->DihAt1, prm->DihAt2, prm->DihAt3,
               prm->DihAt4, prm->DihNum, prm->N14pairs, prm->N14pairlist, prm->N14sceelist, prm->N14scnblist};
  for (size_t k = 0; k < sizeof p / sizeof p[0]; k++) free(p[k]);
  free(prm);
}
