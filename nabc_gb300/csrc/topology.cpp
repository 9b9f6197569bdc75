// Per-system preparation: the work of the reference's mme_init_sff()
// (src/sff/sff.c:858-1846) that the device path needs, done once on the
// host.
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "gbneck_tables.h"
#include "sffg_internal.h"

namespace sffg {

ModelParams model_from_options(const Options &o) {
  ModelParams m;
  m.gb = o.gb;
  m.rgbmax = o.rgbmax;
  m.cut = o.cut;
  m.kappa = o.kappa;
  m.epsext = o.epsext;
  m.gboffset = o.gb == 8 ? 0.195141 : 0.09;           // sff.c:1330
  m.gbneckscale = o.gb == 7 ? 0.361825 : o.gb == 8 ? 0.826836 : 0.0;  // sff.c:1208, 1331
  return m;
}

namespace {

[[noreturn]] void init_fail(const char *msg, int a = 0) {
  std::fprintf(legacy_out(), msg, a);
  std::fputc('\n', legacy_out());
  std::fflush(legacy_out());
  std::exit(1);
}

}  // namespace

void build_host_system(PARMSTRUCT_T *prm, const int *frozen, const Options &o, bool mutate_prm,
                       HostSystem &hs, ModelParams &mp) {
  const int n = prm->Natom;
  mp = model_from_options(o);
  if (prm->IfBox && o.gb) init_fail("Error: gb>0 is incompatible with periodic boundary conditions.");
  if (o.gb == 3 || o.gb > 8 || o.gb == 4 || o.gb == 6)
    init_fail("Error: gb=%d is not supported by this library (gb = 1, 2, 5, 7, 8).", o.gb);
  hs = HostSystem();
  hs.natom = n;
  hs.fsmax = prm->Fsmax;
  hs.q.resize(n);
  hs.rborn.resize(n);
  hs.fs.resize(n);
  hs.alpha.assign(n, 0.0);
  hs.beta.assign(n, 0.0);
  hs.gamma.assign(n, 0.0);
  hs.neck.assign(n, 0);
  hs.type.resize(n);
  hs.frozen.assign(n, 0);
  hs.mass.resize(n);
  // charges scaled by 1/sqrt(dielc): sff.c:1153-1162
  const double scale = o.dielc != 1.0 ? 1.0 / std::sqrt(o.dielc) : 1.0;
  for (int i = 0; i < n; i++) {
    hs.q[i] = prm->Charges[i] * scale;
    if (mutate_prm) prm->Charges[i] = hs.q[i];
    hs.rborn[i] = prm->Rborn[i];
    hs.fs[i] = prm->Fs[i];
    hs.type[i] = prm->Iac[i] - 1;
    hs.frozen[i] = frozen ? (frozen[i] != 0) : 0;
    hs.mass[i] = prm->Masses[i];
  }
  // GB model parameters: sff.c:1186-1333
  if (o.gb == 2 || o.gb == 5) {
    for (int i = 0; i < n; i++) {
      hs.alpha[i] = o.gb == 2 ? 0.8 : 1.0;
      hs.beta[i] = o.gb == 2 ? 0.0 : 0.8;
      hs.gamma[i] = o.gb == 2 ? 2.909125 : 4.85;
    }
  } else if (o.gb == 7 || o.gb == 8) {
    for (int i = 0; i < n; i++) {
      double a = 1.0, b = 0.8, g = 4.85, f = 0.5;
      if (o.gb == 7) {
        a = 1.09511284; b = 1.90792938; g = 2.50798245;
        switch (prm->AtomicNum[i]) {
          case 1: f = 1.09085413633e0; break;
          case 6: f = 4.84353823306e-1; break;
          case 7: f = 7.00147318409e-1; break;
          case 8: f = 1.06557401132e0; break;
          case 16: f = 6.02256336067e-1; break;
          default: f = 5.0e-1;
        }
      } else {
        switch (prm->AtomicNum[i]) {
          case 1: a = SFFG_GB8_ALPHA_H; b = SFFG_GB8_BETA_H; g = SFFG_GB8_GAMMA_H; f = SFFG_GB8_SCREEN_H; break;
          case 6: a = SFFG_GB8_ALPHA_C; b = SFFG_GB8_BETA_C; g = SFFG_GB8_GAMMA_C; f = SFFG_GB8_SCREEN_C; break;
          case 7: a = SFFG_GB8_ALPHA_N; b = SFFG_GB8_BETA_N; g = SFFG_GB8_GAMMA_N; f = SFFG_GB8_SCREEN_N; break;
          case 8: a = SFFG_GB8_ALPHA_OS; b = SFFG_GB8_BETA_OS; g = SFFG_GB8_GAMMA_OS; f = SFFG_GB8_SCREEN_O; break;
          case 15: a = SFFG_GB8_ALPHA_P; b = SFFG_GB8_BETA_P; g = SFFG_GB8_GAMMA_P; f = SFFG_GB8_SCREEN_P; break;
          case 16: a = SFFG_GB8_ALPHA_OS; b = SFFG_GB8_BETA_OS; g = SFFG_GB8_GAMMA_OS; f = SFFG_GB8_SCREEN_S; break;
          default: break;
        }
      }
      hs.alpha[i] = a;
      hs.beta[i] = b;
      hs.gamma[i] = g;
      hs.fs[i] = f;
      if (mutate_prm) prm->Fs[i] = f;
      int idx = static_cast<int>((prm->Rborn[i] - 1.0) * 20.0 + 0.5);
      if (idx < 0 || idx > 20) {
        std::fprintf(stderr, "Atom %i outside the allowed range of 1-2 Angstroms for igb==7.\n", i);
        std::exit(1);
      }
      hs.neck[i] = idx;
    }
  }
  // Lennard-Jones table by type pair; only 6-12 pairs take part in egb()'s
  // pass 2 (eff.c:2015-2016)
  hs.ntypes = prm->Ntypes;
  hs.lj_a.assign(static_cast<size_t>(prm->Ntypes) * prm->Ntypes, 0.0f);
  hs.lj_b.assign(static_cast<size_t>(prm->Ntypes) * prm->Ntypes, 0.0f);
  hs.lj_a64.assign(static_cast<size_t>(prm->Ntypes) * prm->Ntypes, 0.0);
  hs.lj_b64.assign(static_cast<size_t>(prm->Ntypes) * prm->Ntypes, 0.0);
  // the pair kernel reads row type_j, column type_i, which is the
  // reference's row type_i (eff.c:1915, 2015) when the index is symmetric, as
  // Amber's NONBONDED_PARM_INDEX is by construction
  for (int a = 0; a < prm->Ntypes; a++)
    for (int b = 0; b < a; b++)
      if (prm->Cno[a * prm->Ntypes + b] != prm->Cno[b * prm->Ntypes + a])
        init_fail("Error: the Lennard-Jones type index (NONBONDED_PARM_INDEX) is not symmetric.");
  for (int a = 0; a < prm->Ntypes; a++)
    for (int b = 0; b < prm->Ntypes; b++) {
      int ic = prm->Cno[a * prm->Ntypes + b] - 1;
      if (ic >= 0) {
        hs.lj_a[a * prm->Ntypes + b] = static_cast<float>(prm->Cn1[ic]);
        hs.lj_b[a * prm->Ntypes + b] = static_cast<float>(prm->Cn2[ic]);
        hs.lj_a64[a * prm->Ntypes + b] = prm->Cn1[ic];
        hs.lj_b64[a * prm->Ntypes + b] = prm->Cn2[ic];
      }
    }
  // Exclusions: row i marks the listed atoms j > i (1-based, 0 = none); the
  // reference only consults them for the upper-triangle pairs of row i
  // (eff.c:1906-1908, 2004)
  {
    int k = 0;
    for (int i = 0; i < n; i++) {
      for (int m = 0; m < prm->Iblo[i]; m++) {
        int j = prm->ExclAt[k + m] - 1;
        if (j > i) hs.excl.emplace_back(i, j);
      }
      k += prm->Iblo[i];
    }
  }
  // Bonded terms, with frozen-only terms dropped as belly_parm() does
  // (src/sff/mask.c:2-130)
  auto all_frozen = [&](std::initializer_list<int> atoms) {
    for (int a : atoms)
      if (!hs.frozen[a]) return false;
    return true;
  };
  auto add_bonds = [&](int nb, const int *a1, const int *a2, const int *t) {
    for (int i = 0; i < nb; i++) {
      int a = a1[i] / 3, b = a2[i] / 3, ty = t[i] - 1;
      if (all_frozen({a, b})) continue;
      hs.bonds.push_back({a, b, prm->Rk[ty], prm->Req[ty]});
    }
  };
  add_bonds(prm->Nbonh, prm->BondHAt1, prm->BondHAt2, prm->BondHNum);
  add_bonds(prm->Mbona, prm->BondAt1, prm->BondAt2, prm->BondNum);
  for (int i = 0; i < prm->Nbonh; i++)
    hs.rattle_bonds.push_back({prm->BondHAt1[i] / 3, prm->BondHAt2[i] / 3, 0.0, prm->Req[prm->BondHNum[i] - 1]});
  for (int i = 0; i < prm->Mbona; i++)
    hs.rattle_bonds.push_back({prm->BondAt1[i] / 3, prm->BondAt2[i] / 3, 0.0, prm->Req[prm->BondNum[i] - 1]});
  hs.rattle_nh = prm->Nbonh;
  auto add_angles = [&](int na, const int *a1, const int *a2, const int *a3, const int *t) {
    for (int i = 0; i < na; i++) {
      int a = a1[i] / 3, b = a2[i] / 3, c = a3[i] / 3, ty = t[i] - 1;
      if (all_frozen({a, b, c})) continue;
      hs.angles.push_back({a, b, c, prm->Tk[ty], prm->Teq[ty]});
    }
  };
  add_angles(prm->Ntheth, prm->AngleHAt1, prm->AngleHAt2, prm->AngleHAt3, prm->AngleHNum);
  add_angles(prm->Ntheta, prm->AngleAt1, prm->AngleAt2, prm->AngleAt3, prm->AngleNum);
  bool any_frozen = false;
  for (int f : hs.frozen) any_frozen |= f != 0;
  std::vector<int> n14_small, n14_big, n14_type;
  auto add_dihedrals = [&](int nd, const int *a1, const int *a2, const int *a3, const int *a4, const int *t) {
    for (int i = 0; i < nd; i++) {
      int a = a1[i] / 3, b = a2[i] / 3, c3 = a3[i] / 3, d4 = a4[i] / 3;
      int c = std::abs(a3[i]) / 3, d = std::abs(a4[i]) / 3, ty = t[i] - 1;
      if (all_frozen({a, b, c, d})) continue;
      // the multi-term chain of eff.c:619-622: a negative periodicity means
      // the next parameter set applies to the same four atoms
      for (int k = ty;; k++) {
        hs.dihedrals.push_back({a, b, c, d, prm->Pk[k], prm->Pn[k], prm->Phase[k], 0});
        if (!(prm->Pn[k] < 0.0)) break;
      }
      if (any_frozen && c3 >= 0 && d4 >= 0) {
        n14_small.push_back(a < d4 ? a : d4);
        n14_big.push_back(a > d4 ? a : d4);
        n14_type.push_back(ty);
      }
    }
  };
  add_dihedrals(prm->Nphih, prm->DihHAt1, prm->DihHAt2, prm->DihHAt3, prm->DihHAt4, prm->DihHNum);
  add_dihedrals(prm->Mphia, prm->DihAt1, prm->DihAt2, prm->DihAt3, prm->DihAt4, prm->DihNum);
  // 1-4 pairs with the nbond() LJ selection for N14 (eff.c:1262-1310)
  auto add_14 = [&](int i, int j, double scee, double scnb) {
    HostSystem::Pair14 p{i, j, scee, scnb, 0.0, 0.0, 0};
    int ic = prm->Cno[prm->Ntypes * (prm->Iac[i] - 1) + prm->Iac[j] - 1];
    if (ic > 0 || scnb != 1.0) {
      if (ic > 0) {
        ic--;
      } else {
        int big = prm->Iac[i] > prm->Iac[j] ? prm->Iac[i] : prm->Iac[j];
        int small = prm->Iac[i] > prm->Iac[j] ? prm->Iac[j] : prm->Iac[i];
        ic = big * (big - 1) / 2 + small - 1;
      }
      p.c12 = prm->Cn1[ic];
      p.c6 = prm->Cn2[ic];
    } else {
      int h = -ic - 1;
      p.pow10 = 1;
      if (h >= 0 && h < prm->Nphb) {
        p.c12 = prm->HB12[h];
        p.c6 = prm->HB10[h];
      }
    }
    hs.pairs14.push_back(p);
  };
  if (!any_frozen) {
    int k = 0;
    for (int i = 0; i < n; i++)
      for (int m = 0; m < prm->N14pairs[i]; m++, k++)
        add_14(i, prm->N14pairlist[k], prm->N14sceelist[k], prm->N14scnblist[k]);
  } else {
    for (size_t m = 0; m < n14_small.size(); m++)
      add_14(n14_small[m], n14_big[m], prm->Scee[n14_type[m]], prm->Scnb[n14_type[m]]);
  }
}

}  // namespace sffg
