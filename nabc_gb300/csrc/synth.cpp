// Synthetic test molecules for the benchmarks and tests.
//
// A molecule of N atoms is one compact, self-avoiding chain: bond 1.53 A,
// bond angle 111 degrees, dihedrals drawn uniformly; a placement closer than
// 2.5 A to an atom it is not bonded to (its two chain predecessors are
// exempt), or outside the sphere of radius (3N/(4 pi 0.09))^(1/3) A, is
// rejected.  When no placement works the chain backs up a few atoms and
// regrows; when that keeps failing the sphere is enlarged by 1% (a density
// of 0.09/A^3 cannot be packed under the 2.5 A rule, so the realised radius
// is reported and the realised density is lower).  Atom types C/N/O/H are drawn with
// probabilities 0.32/0.09/0.09/0.50 with LJ (R*, eps) = (1.908, 0.086),
// (1.824, 0.17), (1.6612, 0.21), (0.6, 0.0157); charges are N(0, 0.4^2)
// shifted to net zero; intrinsic GB radii 1.7/1.55/1.5/1.2 A and screening
// factors 0.72/0.79/0.85/0.85; bonds k = 300, angles k = 50, dihedrals
// n = 3 with PK = 1.4 and phase 0; 1-2, 1-3 and 1-4 neighbours excluded,
// 1-4 scaled by 1/1.2 (electrostatics) and 1/2 (LJ).
#include "sffg_internal.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <unordered_map>
#include <vector>

namespace {

struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t z = seed;
    for (auto &w : s) {
      z += 0x9E3779B97F4A7C15ULL;
      uint64_t t = z;
      t = (t ^ (t >> 30)) * 0xBF58476D1CE4E5B9ULL;
      t = (t ^ (t >> 27)) * 0x94D049BB133111EBULL;
      w = t ^ (t >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t; s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
  double gaussian() {
    double u1 = uniform(), u2 = uniform();
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
  }
};

struct V3 { double x, y, z; };
V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
V3 unit(V3 a) { return (1.0 / std::sqrt(dot(a, a))) * a; }

// Uniform spatial hash with 2.5 A cells.
class Grid {
 public:
  explicit Grid(double h) : h_(h) {}
  void add(int i, V3 p) { cells_[key(p)].push_back(i); }
  void remove(int i, V3 p) {
    auto &v = cells_[key(p)];
    for (size_t k = 0; k < v.size(); k++)
      if (v[k] == i) { v[k] = v.back(); v.pop_back(); return; }
  }
  // True if some atom other than the exempt ones lies within d of p.
  bool clash(V3 p, double d, const std::vector<V3> &pos, int ex1, int ex2) const {
    long cx = cell(p.x), cy = cell(p.y), cz = cell(p.z);
    double d2 = d * d;
    for (long a = cx - 1; a <= cx + 1; a++)
      for (long b = cy - 1; b <= cy + 1; b++)
        for (long c = cz - 1; c <= cz + 1; c++) {
          auto it = cells_.find(pack(a, b, c));
          if (it == cells_.end()) continue;
          for (int j : it->second) {
            if (j == ex1 || j == ex2) continue;
            V3 q = pos[j] - p;
            if (dot(q, q) < d2) return true;
          }
        }
    return false;
  }

 private:
  long cell(double v) const { return static_cast<long>(std::floor(v / h_)); }
  static uint64_t pack(long a, long b, long c) {
    return (static_cast<uint64_t>(a + (1 << 20)) << 42) | (static_cast<uint64_t>(b + (1 << 20)) << 21) |
           static_cast<uint64_t>(c + (1 << 20));
  }
  uint64_t key(V3 p) const { return pack(cell(p.x), cell(p.y), cell(p.z)); }
  double h_;
  std::unordered_map<uint64_t, std::vector<int>> cells_;
};

// Places atom D given A, B, C with |CD| = b, angle BCD = theta and
// dihedral ABCD = phi.
V3 place(V3 a, V3 b, V3 c, double bond, double theta, double phi) {
  V3 bc = unit(c - b);
  V3 n = unit(cross(b - a, bc));
  V3 m = cross(n, bc);
  double dx = -bond * std::cos(theta), dy = bond * std::sin(theta) * std::cos(phi),
         dz = bond * std::sin(theta) * std::sin(phi);
  return c + (dx * bc + dy * m + dz * n);
}

V3 random_unit(Rng &r) {
  double z = 2.0 * r.uniform() - 1.0, t = 2.0 * M_PI * r.uniform(), s = std::sqrt(1.0 - z * z);
  return {s * std::cos(t), s * std::sin(t), z};
}

}  // namespace

namespace sffg {

// Grows the chain; returns the realised confining radius.
double synth_chain(int n, uint64_t seed, std::vector<V3> &pos) {
  const double bond = 1.53, theta = 111.0 * M_PI / 180.0, dmin = 2.5;
  double radius = std::cbrt(3.0 * n / (4.0 * M_PI * 0.09));
  Rng rng(seed ^ 0xC0FFEEULL);
  pos.assign(n, V3{0, 0, 0});
  Grid grid(dmin);
  auto inside = [&](V3 p) { return dot(p, p) <= radius * radius; };
  // first three atoms
  for (;;) {
    // the direction is drawn before the distance (an explicit order: the
    // two draws must not depend on the compiler's choice of operand order)
    const V3 dir = random_unit(rng);
    V3 p0 = (0.3 * radius * std::cbrt(rng.uniform())) * dir;
    V3 p1 = p0 + bond * random_unit(rng);
    V3 u = unit(p1 - p0), w = random_unit(rng);
    V3 perp = unit(w - dot(w, u) * u);
    V3 p2 = p1 + bond * (-std::cos(theta) * u + std::sin(theta) * perp);
    if (n < 3 || (inside(p0) && inside(p1) && inside(p2))) {
      pos[0] = p0;
      if (n > 1) pos[1] = p1;
      if (n > 2) pos[2] = p2;
      break;
    }
  }
  for (int i = 0; i < n && i < 3; i++) grid.add(i, pos[i]);
  // Backtracking doubles (up to 64 atoms) while the chain fails to pass the
  // furthest point it has reached; after kStall failures without progress
  // the confining sphere grows by 1%.
  int i = 3, consecutive_fail = 0, best = 3, stall = 0;
  const int tries = 64, kStall = 48;
  while (i < n) {
    bool ok = false;
    for (int t = 0; t < tries; t++) {
      V3 p = place(pos[i - 3], pos[i - 2], pos[i - 1], bond, theta, 2.0 * M_PI * rng.uniform());
      if (!inside(p) || grid.clash(p, dmin, pos, i - 1, i - 2)) continue;
      pos[i] = p;
      grid.add(i, p);
      ok = true;
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
    if (++stall > kStall) {
      radius *= 1.01;
      stall = 0;
      consecutive_fail = 0;
    }
    int back = 1 << (consecutive_fail < 6 ? consecutive_fail : 6);
    consecutive_fail++;
    for (int k = 0; k < back && i > 3; k++) {
      i--;
      grid.remove(i, pos[i]);
    }
  }
  return radius;
}

}  // namespace sffg

extern "C" PARMSTRUCT_T *sffg_synth_molecule(int natom, unsigned long long seed, double *x,
                                             double *radius_out) {
  if (natom < 4) return nullptr;
  std::vector<V3> pos;
  double radius = sffg::synth_chain(natom, seed, pos);
  if (radius_out) *radius_out = radius;
  for (int i = 0; i < natom; i++) {
    x[3 * i] = pos[i].x;
    x[3 * i + 1] = pos[i].y;
    x[3 * i + 2] = pos[i].z;
  }
  Rng rng(seed ^ 0xA70B5ULL);
  // element draw: 0 C, 1 N, 2 O, 3 H
  std::vector<int> el(natom);
  for (int i = 0; i < natom; i++) {
    double u = rng.uniform();
    el[i] = u < 0.32 ? 0 : u < 0.41 ? 1 : u < 0.50 ? 2 : 3;
  }
  std::vector<double> q(natom);
  double mean = 0.0;
  for (int i = 0; i < natom; i++) {
    q[i] = 0.4 * rng.gaussian();
    mean += q[i];
  }
  mean /= natom;

  PARMSTRUCT_T *prm = static_cast<PARMSTRUCT_T *>(std::calloc(1, sizeof(PARMSTRUCT_T)));
  std::snprintf(prm->ititl, sizeof prm->ititl, "synthetic chain N=%d seed=%llu", natom, seed);
  const int res_size = 16;
  auto isH = [&](int a) { return el[a] == 3; };
  int nbh = 0, nba = 0, nth = 0, nta = 0, nph = 0, npa = 0;
  for (int i = 0; i + 1 < natom; i++) (isH(i) || isH(i + 1) ? nbh : nba)++;
  for (int i = 0; i + 2 < natom; i++) (isH(i) || isH(i + 1) || isH(i + 2) ? nth : nta)++;
  for (int i = 0; i + 3 < natom; i++) (isH(i) || isH(i + 1) || isH(i + 2) || isH(i + 3) ? nph : npa)++;
  prm->Natom = natom;
  prm->Ntypes = 4;
  prm->Nbonh = nbh; prm->Mbona = nba; prm->Nbona = nba;
  prm->Ntheth = nth; prm->Mtheta = nta; prm->Ntheta = nta;
  prm->Nphih = nph; prm->Mphia = npa; prm->Nphia = npa;
  prm->Nres = (natom + res_size - 1) / res_size;
  prm->Nmxrs = res_size;
  prm->Numbnd = 1; prm->Numang = 1; prm->Nptra = 1; prm->Natyp = 1; prm->Nphb = 0;
  int nnb = 0;
  for (int i = 0; i < natom; i++) {
    int k = 0;
    for (int d = 1; d <= 3; d++)
      if (i + d < natom) k++;
    nnb += k ? k : 1;
  }
  prm->Nnb = nnb;
  sffg::prm_allocate_arrays(prm);

  static const char *names[4] = {"C", "N", "O", "H"};
  static const char *atypes[4] = {"CT", "N", "O", "H"};
  static const double rstar[4] = {1.908, 1.824, 1.6612, 0.6};
  static const double eps[4] = {0.086, 0.17, 0.21, 0.0157};
  static const double mass[4] = {12.01, 14.01, 16.00, 1.008};
  static const double radii[4] = {1.7, 1.55, 1.5, 1.2};
  static const double screen[4] = {0.72, 0.79, 0.85, 0.85};
  static const int znum[4] = {6, 7, 8, 1};
  for (int i = 0; i < natom; i++) {
    std::snprintf(prm->AtomNames[i], NAMESIZE, "%-4s", names[el[i]]);
    std::snprintf(prm->AtomType[i], NAMESIZE, "%-4s", atypes[el[i]]);
    std::snprintf(prm->AtomTree[i], NAMESIZE, "%-4s", "M");
    prm->Charges[i] = (q[i] - mean) * 18.2223;
    prm->Masses[i] = mass[el[i]];
    prm->Iac[i] = el[i] + 1;
    prm->Rborn[i] = radii[el[i]];
    prm->Fs[i] = screen[el[i]];
    prm->AtomicNum[i] = znum[el[i]];
    prm->AtomRes[i] = i / res_size;
  }
  for (int a = 0; a < 4; a++)
    for (int b = 0; b < 4; b++) {
      int big = (a > b ? a : b) + 1, small = (a > b ? b : a) + 1;
      int ic = big * (big - 1) / 2 + small;  // 1-based
      prm->Cno[a * 4 + b] = ic;
      double r = rstar[a] + rstar[b], e = std::sqrt(eps[a] * eps[b]);
      prm->Cn1[ic - 1] = e * std::pow(r, 12);
      prm->Cn2[ic - 1] = 2.0 * e * std::pow(r, 6);
    }
  for (int r = 0; r < prm->Nres; r++) {
    std::snprintf(prm->ResNames[r], NAMESIZE, "%-4s", "SYN");
    prm->Ipres[r] = r * res_size;
  }
  prm->Ipres[prm->Nres] = natom;
  prm->Rk[0] = 300.0; prm->Req[0] = 1.53;
  prm->Tk[0] = 50.0; prm->Teq[0] = 111.0 * M_PI / 180.0;
  prm->Pk[0] = 1.4; prm->Pn[0] = 3.0; prm->Phase[0] = 0.0;
  prm->Scee[0] = 1.0 / 1.2; prm->Scnb[0] = 1.0 / 2.0;
  nbh = nba = nth = nta = nph = npa = 0;
  for (int i = 0; i + 1 < natom; i++) {
    if (isH(i) || isH(i + 1)) {
      prm->BondHAt1[nbh] = 3 * i; prm->BondHAt2[nbh] = 3 * (i + 1); prm->BondHNum[nbh++] = 1;
    } else {
      prm->BondAt1[nba] = 3 * i; prm->BondAt2[nba] = 3 * (i + 1); prm->BondNum[nba++] = 1;
    }
  }
  for (int i = 0; i + 2 < natom; i++) {
    if (isH(i) || isH(i + 1) || isH(i + 2)) {
      prm->AngleHAt1[nth] = 3 * i; prm->AngleHAt2[nth] = 3 * (i + 1);
      prm->AngleHAt3[nth] = 3 * (i + 2); prm->AngleHNum[nth++] = 1;
    } else {
      prm->AngleAt1[nta] = 3 * i; prm->AngleAt2[nta] = 3 * (i + 1);
      prm->AngleAt3[nta] = 3 * (i + 2); prm->AngleNum[nta++] = 1;
    }
  }
  for (int i = 0; i + 3 < natom; i++) {
    if (isH(i) || isH(i + 1) || isH(i + 2) || isH(i + 3)) {
      prm->DihHAt1[nph] = 3 * i; prm->DihHAt2[nph] = 3 * (i + 1); prm->DihHAt3[nph] = 3 * (i + 2);
      prm->DihHAt4[nph] = 3 * (i + 3); prm->DihHNum[nph++] = 1;
    } else {
      prm->DihAt1[npa] = 3 * i; prm->DihAt2[npa] = 3 * (i + 1); prm->DihAt3[npa] = 3 * (i + 2);
      prm->DihAt4[npa] = 3 * (i + 3); prm->DihNum[npa++] = 1;
    }
  }
  int k = 0;
  for (int i = 0; i < natom; i++) {
    int cnt = 0;
    for (int d = 1; d <= 3; d++)
      if (i + d < natom) {
        prm->ExclAt[k++] = i + d + 1;  // 1-based
        cnt++;
      }
    if (!cnt) prm->ExclAt[k++] = 0;
    prm->Iblo[i] = cnt ? cnt : 1;
  }
  sffg::prm_finish_derived(prm, true);
  return prm;
}
