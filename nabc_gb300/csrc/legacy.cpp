// The reference's single-session C API on top of the device engine:
// mme_init_sff (src/sff/sff.c:858), mme (sff.c:1854 -> eff.c:2442),
// md (sff.c:2071), conjgrad (conjgrad.c:34), mme_timer (timer.c:71) and the
// serial random stream md() draws from (rand2.c:51-140).
//
// One session is resident on the GPU, like the reference's process-global
// state.  mme() copies x in and the gradient out; md() and conjgrad() called
// with this library's mme keep coordinates, velocities and the minimiser
// state on the device between evaluations, and fall back to the reference's
// host loop only when handed some other energy function.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

#include "engine.h"

namespace sffg {

namespace {

struct Session {
  PARMSTRUCT_T *prm = nullptr;
  int *frozen = nullptr;
  int *constrained = nullptr;  // borrowed with x0, as the reference does (sff.c:886)
  double *x0 = nullptr;
  std::unique_ptr<Batch> batch;
  int natom = 0;
  bool list_built = false;
  NcTrajectory traj;  // md()'s trajectory when mme_init_sff got a file name
  std::vector<double> scratch;
};

Session &session() {
  static Session s;
  return s;
}

[[noreturn]] void fatal(const std::string &msg) {
  std::fprintf(legacy_out(), "sffg: %s\n", msg.c_str());
  std::fflush(legacy_out());
  std::fprintf(stderr, "sffg: %s\n", msg.c_str());
  std::exit(1);
}

void check(int rc, const char *what) {
  if (rc != SFFG_OK) {
    Session &s = session();
    fatal(std::string(what) + " failed: " + (s.batch ? s.batch->last_error : std::string("no session")));
  }
}

// the reference's RNG (Rand2, sffg_internal.h): one process-global stream
Rand2 &rng() {
  static Rand2 r;
  return r;
}

void reference_noise(void *, int, int n, double *out) {
  for (int i = 0; i < n; i++) out[i] = rng().gauss(0.0, 1.0);
}

double frms_of(const std::vector<double> &g) {
  double s = 0.0;
  for (double v : g) s += v * v;
  return std::sqrt(s / static_cast<double>(g.size()));
}

// The per-evaluation printout of mme34 (src/sff/eff.c:2899-2938).
void print_energies(int iter, const double *ene, double frms) {
  const Options &o = options();
  FILE *out = legacy_out();
  if (iter > -1 && (iter == 0 || iter % o.ntpr == 0)) {
    std::fprintf(out, "ff:%6d %9.2f %9.2f %9.2f %9.2f %9.2f %9.2f %9.2e\n", iter, ene[0], ene[3] + ene[4] + ene[5],
                 ene[1] + ene[7], ene[2] + ene[8], ene[9] + ene[11] + ene[12], ene[10], frms);
    std::fflush(out);
  }
  if (iter == -1) {
    std::fprintf(out, "     bond:  %15.9f\n", ene[3]);
    std::fprintf(out, "    angle:  %15.9f\n", ene[4]);
    std::fprintf(out, " dihedral:  %15.9f\n", ene[5]);
    std::fprintf(out, "    enb14:  %15.9f\n", ene[7]);
    std::fprintf(out, "    eel14:  %15.9f\n", ene[8]);
    std::fprintf(out, "      enb:  %15.9f\n", ene[1]);
    std::fprintf(out, "      eel:  %15.9f\n", ene[2]);
    std::fprintf(out, "      egb:  %15.9f\n", ene[10]);
    std::fprintf(out, "    econs:  %15.9f\n", ene[9]);
    std::fprintf(out, "    esurf:  %15.9f\n", ene[11]);
    std::fprintf(out, "    Total:  %15.9f\n", ene[0]);
    std::fprintf(out, "     frms:  %15.9f\n", frms);
  }
  if (o.e_debug == 2) {
    std::fprintf(out, " BOND    = %13.4lf  ANGLE   = %13.4lf  DIHED      = %13.4lf\n", ene[3], ene[4], ene[5]);
    std::fprintf(out, " VDWAALS = %13.4lf  EEL     = %13.4lf  EGB        = %13.4lf\n", ene[1], ene[2], ene[10]);
    std::fprintf(out, " 1-4 VDW = %13.4lf  1-4 EEL = %13.4lf  RESTRAINT  = %13.4lf\n", ene[7], ene[8], ene[9]);
    std::fprintf(out, " ESURF   = %13.4lf\n", ene[11]);
  }
}

void print_header() {
  std::fprintf(legacy_out(), "      iter    Total       bad      vdW     elect   nonpolar   genBorn      frms\n");
  std::fflush(legacy_out());
}

void print_radii(Batch &b) {
  Session &s = session();
  std::vector<double> reff(s.natom);
  check(b.get_reff(0, reff.data(), nullptr), "get_reff");
  std::fprintf(legacy_out(), "Effective Born radii:\n");
  for (int i = 0; i < s.natom; i++)
    std::fprintf(legacy_out(), "%d\t%15.7f\t%15.7f\n", i + 1, s.prm->Rborn[i], reff[i]);
}

Batch &require_batch() {
  Session &s = session();
  if (!s.batch) fatal("mme called before mme_init_sff");
  return *s.batch;
}

// After an evaluation: energies, gradient to host, printing.
double finish_eval(int iter, double *f) {
  Session &s = session();
  Batch &b = *s.batch;
  double ene[13];
  // the gradient goes straight into the caller's f (scratch when f is NULL)
  double *g = f;
  if (!g) {
    s.scratch.resize(3 * static_cast<size_t>(s.natom));
    g = s.scratch.data();
  }
  check(b.get_energy_grad(0, ene, g, nullptr), "get_energy");
  if (options().gb_debug) print_radii(b);
  // frms only for the lines that print it
  const Options &o = options();
  if (iter == -1 || (iter > -1 && (iter == 0 || iter % o.ntpr == 0))) {
    double frms = 0.0;
    for (int i = 0; i < 3 * s.natom; i++) frms += g[i] * g[i];
    print_energies(iter, ene, std::sqrt(frms / (3 * s.natom)));
  }
  return ene[0];
}

}  // namespace

extern "C" REAL_T mme(REAL_T *x, REAL_T *f, INT_T *iter);

}  // namespace sffg

using namespace sffg;

extern "C" INT_T mme_init_sff(PARMSTRUCT_T *prm, INT_T *frozen, INT_T *constrained, REAL_T *x0, STRING_T *ncname) {
  const double t0 = wall_seconds();
  Session &s = session();
  s.batch.reset();
  s.prm = prm;
  s.frozen = frozen;
  s.natom = prm->Natom;
  s.list_built = false;
  const Options &o = options();
  if (o.gb == 0) fatal("this library implements the generalized-Born path only (gb = 1, 2, 5, 7 or 8)");
  if (o.rgbmax > o.cut) {
    std::fprintf(legacy_out(), "Error in egb: rgbmax = %f is greater than cutoff = %f\n", o.rgbmax, o.cut);
    std::exit(1);
  }
  // md()'s Amber NetCDF trajectory, written every ntwx steps (sff.c:1164-1168)
  s.traj.close();
  if (ncname && !s.traj.create(ncname, prm->Natom))
    std::fprintf(stderr, "Error: cannot create NetCDF trajectory %s\n", ncname);
  // positional restraints (src/sff/sff.c:1169-1178): counted and reported
  // here, applied from the first mme() on
  s.constrained = nullptr;
  s.x0 = x0;
  if (constrained) {
    int nc = 0;
    for (int i = 0; i < prm->Natom; i++) nc += constrained[i] != 0;
    if (nc) {
      std::fprintf(legacy_out(), "constrained %d atoms from input array\n", nc);
      if (!x0) fatal("constrained atoms need the reference positions x0");
      s.constrained = constrained;
    }
  }
  // Validate and apply the reference's in-place changes to prm (charges
  // scaled by 1/sqrt(dielc), gb=7/8 screening factors); the device copy is
  // made at the first mme() call, whose coordinates set the spatial order.
  HostSystem hs;
  ModelParams mp;
  build_host_system(prm, frozen, o, true, hs, mp);
  Options od = o;
  od.dielc = 1.0;  // prm already carries the scaled charges
  s.batch.reset(new Batch(od));
  timers().init += wall_seconds() - t0;
  return 0;
}

namespace {

// Deferred upload: the spatial order is taken from the first coordinates
// mme() sees.
void ensure_finalized(const double *x) {
  Session &s = session();
  Batch &b = require_batch();
  if (!b.finalized()) {
    if (b.add_system(s.prm, s.frozen, x, false) < 0) fatal("mme: " + b.last_error);
    if (s.constrained) b.set_restraints(0, s.constrained, s.x0);
    const int rc = b.finalize();
    if (rc) fatal("mme: device setup failed: " + b.last_error);
  }
}

}  // namespace

// The checkpoint name mm_set_checkpoint() set (sff.c:2056); empty: none.
std::string &checkpoint_name() {
  static std::string name;
  return name;
}

// Coordinates of iteration iter in the Cartesian format of the reference's
// putxyz (sff.c:606-636); the name's leftmost "%d" becomes the iteration
// number, or the number is appended (sff.c:789-830); "-" writes to nabout.
void write_checkpoint(const std::string &tmpl, int natom, const double *x, int iter) {
  if (iter < 0) return;
  const std::string num = std::to_string(iter);
  std::string name = tmpl;
  const size_t at = name.find("%d");
  if (at == std::string::npos) name += num;
  else name.replace(at, 2, num);
  FILE *fp = name == "-" ? legacy_out() : std::fopen(name.c_str(), "w");
  if (!fp) {
    std::fprintf(stderr, "Can't open file %s\n", name.c_str());
    return;
  }
  std::fprintf(fp, "%6d\n", natom);
  for (int i = 0; i < 3 * natom; i += 3) std::fprintf(fp, "%20.15f%20.15f%20.15f\n", x[i], x[i + 1], x[i + 2]);
  if (fp != legacy_out()) std::fclose(fp);
}

extern "C" REAL_T mme(REAL_T *x, REAL_T *f, INT_T *iter) {
  Session &s = session();
  if (*iter == -3) return 0.0;  // the reference frees scratch here (eff.c:2504-2521)
  const double t0 = wall_seconds();
  ensure_finalized(x);
  Batch &b = *s.batch;
  if (*iter == 0) print_header();
  const Options &o = options();
  // checkpoint every nchk iterations once a name is set (eff.c:2536-2538)
  if (!checkpoint_name().empty() && *iter > 0 && o.nchk > 0 && *iter % o.nchk == 0)
    write_checkpoint(checkpoint_name(), s.natom, x, *iter);
  const bool rebuild = !s.list_built || (*iter > 0 && o.nsnb > 0 && *iter % o.nsnb == 0) || *iter == -4;
  check(b.set_coords(0, x, nullptr), "set_coords");
  // a rebuild launches without host round trips; the call redoes it in the
  // rare case that a list store proved too small
  check(b.eval_checked(rebuild, nullptr), "eval");
  s.list_built = true;
  const double e = finish_eval(*iter, f);
  timers().mme += wall_seconds() - t0;
  return e;
}

// mme() on a structure whose bond lengths RATTLE first restores, with the
// gradient projected onto the constraints (src/sff/sff.c:1882-2010).
extern "C" REAL_T mme_rattle(REAL_T *x, REAL_T *f, INT_T *iter);
extern "C" void mm_set_checkpoint(STRING_T **fname);

namespace {

// Centre-of-mass motion removal (src/sff/com.c:10-147): translation to the
// origin and, with also_v, the centre-of-mass velocity and rigid rotation.
void com_remove_host(int n, double *x, double *v, const double *minv, bool also_v) {
  double mt = 0, xs = 0, ys = 0, zs = 0;
  for (int i = 0; i < n / 3; i++) mt += 1. / minv[3 * i];
  for (int i = 0; i < n / 3; i++) {
    xs += x[3 * i] / minv[3 * i];
    ys += x[3 * i + 1] / minv[3 * i + 1];
    zs += x[3 * i + 2] / minv[3 * i + 2];
  }
  xs /= mt;
  ys /= mt;
  zs /= mt;
  for (int i = 0; i < n / 3; i++) {
    x[3 * i] -= xs;
    x[3 * i + 1] -= ys;
    x[3 * i + 2] -= zs;
  }
  if (!also_v) return;
  double vx = 0, vy = 0, vz = 0;
  for (int i = 0; i < n / 3; i++) {
    vx += v[3 * i] / minv[3 * i];
    vy += v[3 * i + 1] / minv[3 * i + 1];
    vz += v[3 * i + 2] / minv[3 * i + 2];
  }
  vx /= mt;
  vy /= mt;
  vz /= mt;
  for (int i = 0; i < n / 3; i++) {
    v[3 * i] -= vx;
    v[3 * i + 1] -= vy;
    v[3 * i + 2] -= vz;
  }
  const double sc = 1.e-3;
  double L[3] = {0, 0, 0}, M[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < n / 3; i++) {
    const double m = 1. / minv[3 * i], X = x[3 * i], Y = x[3 * i + 1], Z = x[3 * i + 2];
    L[0] += sc * (Y * v[3 * i + 2] - Z * v[3 * i + 1]) * m;
    L[1] += sc * (Z * v[3 * i] - X * v[3 * i + 2]) * m;
    L[2] += sc * (X * v[3 * i + 1] - Y * v[3 * i]) * m;
  }
  for (int i = 0; i < n / 3; i++) {
    const double m = 1. / minv[3 * i], X = x[3 * i], Y = x[3 * i + 1], Z = x[3 * i + 2];
    M[0] += X * X * m;
    M[1] += X * Y * m;
    M[2] += X * Z * m;
    M[3] += Y * Y * m;
    M[4] += Y * Z * m;
    M[5] += Z * Z * m;
  }
  const double I0 = (M[3] + M[5]) * sc, I1 = -M[1] * sc, I2 = -M[2] * sc;
  const double I4 = (M[0] + M[5]) * sc, I5 = -M[4] * sc, I8 = (M[0] + M[3]) * sc;
  const double c0 = I4 * I8 - I5 * I5, c1 = I1 * I8 - I5 * I2, c2 = I1 * I5 - I4 * I2;
  const double c4 = I0 * I8 - I2 * I2, c5 = I0 * I5 - I1 * I2, c8 = I0 * I4 - I1 * I1;
  const double det = I0 * c0 - I1 * c1 + I2 * c2;
  const double ox = (c0 * L[0] - c1 * L[1] + c2 * L[2]) / det;
  const double oy = (-c1 * L[0] + c4 * L[1] - c5 * L[2]) / det;
  const double oz = (c2 * L[0] - c5 * L[1] + c8 * L[2]) / det;
  for (int i = 0; i < n / 3; i++) {
    const double X = x[3 * i], Y = x[3 * i + 1], Z = x[3 * i + 2];
    v[3 * i] = v[3 * i] - oy * Z + oz * Y;
    v[3 * i + 1] = v[3 * i + 1] - oz * X + ox * Z;
    v[3 * i + 2] = v[3 * i + 2] - ox * Y + oy * X;
  }
}

// Bond-length constraints (RATTLE, src/sff/rattle.c, following TINKER):
// Gauss-Seidel sweeps over the bonds to hydrogen and, with rattle=1, the
// other bonds, in the topology's order, correcting each bond in turn
// (over-relaxed by 1.2) until every |req^2 - r^2| is within the tolerance.
// The sweeps update positions and velocities in place, so their order is
// part of the result; they run on the host.  Atom indices in the topology
// arrays are coordinate offsets (3 * atom).
constexpr double kRattleFac = 1.2;
// the reference keeps this tolerance in single precision (rattle.c:22-28)
const double kRattleEps = static_cast<double>(static_cast<float>(0.0000001));

template <class F>
void for_constrained_bonds(const PARMSTRUCT_T *prm, int irattle, F &&body) {
  const int nh = prm->Nbonh, nb = irattle == 2 ? 0 : prm->Mbona;
  for (int i = 0; i < nh + nb; i++) {
    if (i < nh) body(prm->BondHAt1[i], prm->BondHAt2[i], prm->Req[prm->BondHNum[i] - 1]);
    else body(prm->BondAt1[i - nh], prm->BondAt2[i - nh], prm->Req[prm->BondNum[i - nh] - 1]);
  }
}

// Position part (rattle.c:12-100); xold may alias x.
int rattle_positions(const PARMSTRUCT_T *prm, int irattle, double dt, double *x, const double *xold, double *v,
                     const double *minv) {
  int niter = 0;
  bool done = false;
  while (!done && niter < 1000) {
    niter++;
    done = true;
    for_constrained_bonds(prm, irattle, [&](int a1, int a2, double req) {
      const double xr = x[a2] - x[a1], yr = x[a2 + 1] - x[a1 + 1], zr = x[a2 + 2] - x[a1 + 2];
      const double delta = req * req - (xr * xr + yr * yr + zr * zr);
      if (std::fabs(delta) <= kRattleEps) return;
      done = false;
      const double xo = xold[a2] - xold[a1], yo = xold[a2 + 1] - xold[a1 + 1], zo = xold[a2 + 2] - xold[a1 + 2];
      const double dot = xr * xo + yr * yo + zr * zo;
      double ra = minv[a1], rb = minv[a2];
      const double term = kRattleFac * delta / (2.0 * (ra + rb) * dot);
      const double tx = xo * term, ty = yo * term, tz = zo * term;
      x[a1] -= tx * ra;
      x[a1 + 1] -= ty * ra;
      x[a1 + 2] -= tz * ra;
      x[a2] += tx * rb;
      x[a2 + 1] += ty * rb;
      x[a2 + 2] += tz * rb;
      ra /= dt;
      rb /= dt;
      v[a1] -= tx * ra;
      v[a1 + 1] -= ty * ra;
      v[a1 + 2] -= tz * ra;
      v[a2] += tx * rb;
      v[a2 + 1] += ty * rb;
      v[a2 + 2] += tz * rb;
    });
  }
  if (niter >= 999) fatal("ERROR in RATTLE");
  return niter;
}

// Velocity part (rattle.c:102-181).
int rattle_velocities(const PARMSTRUCT_T *prm, int irattle, double dt, const double *x, double *v,
                      const double *minv) {
  const double eps = 0.0000001 / dt;
  int niter = 0;
  bool done = false;
  while (!done && niter < 1000) {
    niter++;
    done = true;
    for_constrained_bonds(prm, irattle, [&](int a1, int a2, double req) {
      const double xr = x[a2] - x[a1], yr = x[a2 + 1] - x[a1 + 1], zr = x[a2 + 2] - x[a1 + 2];
      const double xv = v[a2] - v[a1], yv = v[a2 + 1] - v[a1 + 1], zv = v[a2 + 2] - v[a1 + 2];
      const double ra = minv[a1], rb = minv[a2];
      const double term = -(xr * xv + yr * yv + zr * zv) * kRattleFac / ((ra + rb) * req * req);
      if (std::fabs(term) <= eps) return;
      done = false;
      const double tx = xr * term, ty = yr * term, tz = zr * term;
      v[a1] -= tx * ra;
      v[a1 + 1] -= ty * ra;
      v[a1 + 2] -= tz * ra;
      v[a2] += tx * rb;
      v[a2 + 1] += ty * rb;
      v[a2 + 2] += tz * rb;
    });
  }
  if (niter >= 999) fatal("ERROR in RATTLE2");
  return niter;
}

// The reference's md() loop on the host around an arbitrary energy
// function (src/sff/sff.c:2071-2366).
int md_host(int n, int maxstep, double *x, double *f, double *v, REAL_T (*func)(REAL_T *, REAL_T *, INT_T *)) {
  Session &s = session();
  const Options &o = options();
  const double boltz2 = 9.93595e-4;
  std::vector<double> minv(n), xold(n), sqrmass(n), accel(n);
  int nfrozen = 0;
  for (int i = 0; s.frozen && i < s.natom; i++) nfrozen += s.frozen[i] != 0;
  const bool rat = o.irattle && s.prm;
  double rndf = n - 3.0 * nfrozen;  // degrees of freedom (sff.c:2142-2146)
  if (rat) rndf -= s.prm->Nbonh + (o.irattle == 1 ? s.prm->Mbona : 0);
  const double dtx = o.dt * 20.455, dt5 = 0.5 * dtx;
  const double ekin0 = boltz2 * rndf * o.temp0, dttp = o.dt / o.tautp, gammai = o.gamma_ln / 20.455;
  const double c_implic = 1.0 / (1.0 + gammai * dt5), c_explic = 1.0 - gammai * dt5, c_ave = 1.0 + gammai * dt5;
  const double sdfac = std::sqrt(4.0 * gammai * boltz2 * o.temp0 / dtx);
  for (int i = 0; i < n; i++) minv[i] = s.prm ? 1.0 / s.prm->Masses[i / 3] : 1.0 / o.genmass;
  auto frz = [&](int i) { return s.frozen && s.frozen[i / 3]; };
  double ekin = 0.0, epot, tscal, t = o.t;
  if (o.zerov) {
    for (int i = 0; i < n; i++) v[i] = 0.0;
  } else if (o.tempi > 0.0) {
    for (int i = 0; i < n; i++) {
      if (frz(i)) {
        v[i] = 0.0;
      } else {
        v[i] = rng().gauss(0.0, std::sqrt(2. * boltz2 * o.tempi * minv[i]));
        ekin += v[i] * v[i] / minv[i];
      }
    }
    ekin *= 0.5;
  } else {
    for (int i = 0; i < n; i++) ekin += v[i] * v[i] * minv[i];
    ekin *= 0.5;
  }
  int nstep = 0;
  epot = func(x, f, &nstep);
  for (int i = 0; i < n; i++) {
    if (gammai == 0.0) {
      accel[i] = -f[i] * minv[i] * dt5;
    } else if (frz(i)) {
      accel[i] = 0.0;
    } else {
      sqrmass[i] = 1.0 / std::sqrt(minv[i]);
      accel[i] = (-f[i] + rng().gauss(0.0, sdfac * sqrmass[i])) * minv[i] * dt5;
    }
  }
  for (nstep = 1; nstep <= maxstep; nstep++) {
    tscal = ekin > 0.01 ? std::sqrt(1. + dttp * (ekin0 / ekin - 1.)) : 1.0;
    ekin = 0.0;
    for (int i = 0; i < n; i++) {
      xold[i] = x[i];
      v[i] = gammai == 0.0 ? (v[i] + accel[i]) * tscal : c_explic * v[i] + accel[i];
      v[i] = v[i] > o.vlimit ? o.vlimit : v[i];
      v[i] = v[i] < -o.vlimit ? -o.vlimit : v[i];
      x[i] += v[i] * dtx;
    }
    if (rat) rattle_positions(s.prm, o.irattle, dtx, x, xold.data(), v, minv.data());
    epot = func(x, f, &nstep);
    for (int i = 0; i < n; i++) {
      if (gammai == 0.0) {
        accel[i] = -f[i] * minv[i] * dt5;
        v[i] = (v[i] + accel[i]) * tscal;
      } else if (!frz(i)) {
        accel[i] = (-f[i] + rng().gauss(0.0, sdfac * sqrmass[i])) * minv[i] * dt5;
        v[i] = (v[i] + accel[i]) * c_implic;
      }
    }
    if (rat) rattle_velocities(s.prm, o.irattle, dtx, x, v, minv.data());
    for (int i = 0; i < n; i++) ekin += v[i] * v[i] / minv[i];
    ekin *= 0.5;
    if (gammai > 0.) ekin *= c_ave;
    t += o.dt;
    if (nstep % o.ntpr_md == 0 || nstep == 1) {
      std::fprintf(legacy_out(), "md:       %5d %10.3f %10.2f %10.2f %10.2f %10.2f\n", nstep, t, ekin, epot,
                   ekin + epot, ekin / (boltz2 * rndf));
      std::fflush(legacy_out());
    }
    if (o.ntwx > 0 && nstep % o.ntwx == 0 && s.traj.open()) s.traj.write_frame(x, t);
    if (o.nscm > 0 && nstep % o.nscm == 0) com_remove_host(n, x, v, minv.data(), gammai == 0.0 || o.hcp);
  }
  options().t = t;
  nstep = -3;
  func(x, f, &nstep);
  return 0;
}

}  // namespace

extern "C" INT_T md(INT_T n, INT_T maxstep, REAL_T *x, REAL_T *f, REAL_T *v,
                    REAL_T (*func)(REAL_T *, REAL_T *, INT_T *)) {
  Session &s = session();
  const double t0 = wall_seconds();
  // another energy function, coordinates that are not the session's, or a
  // rattle option set after the session's batch was made take the host loop
  if (func != &sffg::mme || !s.batch || n != 3 * s.natom || options().irattle != s.batch->opts().irattle) {
    const int rc = md_host(n, maxstep, x, f, v, func);
    timers().md += wall_seconds() - t0;
    return rc;
  }
  Options &o = options();
  const double boltz2 = 9.93595e-4;
  ensure_finalized(x);
  Batch &b = *s.batch;
  int nfrozen = 0;
  for (int i = 0; s.frozen && i < s.natom; i++) nfrozen += s.frozen[i] != 0;
  // RATTLE's constraints take one degree of freedom each (sff.c:2142-2146)
  const double rndf = n - 3.0 * nfrozen - b.rattle_bonds(0), ekin0 = boltz2 * rndf * o.temp0, dttp = o.dt / o.tautp;
  const double gammai = o.gamma_ln / 20.455;
  // initial velocities (sff.c:2165-2188), drawn from the shared stream
  double ekin = 0.0;
  auto frz = [&](int i) { return s.frozen && s.frozen[i / 3]; };
  if (o.zerov) {
    for (int i = 0; i < n; i++) v[i] = 0.0;
  } else if (o.tempi > 0.0) {
    for (int i = 0; i < n; i++) {
      const double minv = 1.0 / s.prm->Masses[i / 3];
      if (frz(i)) {
        v[i] = 0.0;
      } else {
        v[i] = rng().gauss(0.0, std::sqrt(2. * boltz2 * o.tempi * minv));
        ekin += v[i] * v[i] / minv;
      }
    }
    ekin *= 0.5;
  } else {
    for (int i = 0; i < n; i++) ekin += v[i] * v[i] * (1.0 / s.prm->Masses[i / 3]);
    ekin *= 0.5;
  }
  check(b.set_coords(0, x, nullptr), "set_coords");
  check(b.set_velocities(0, v, nullptr), "set_velocities");
  Batch::NoiseFn noise = o.sffg_noise == 0 ? &reference_noise : nullptr;
  // first force (iter 0): ff: header and line as mme() prints them
  print_header();
  check(b.md_begin(!s.list_built, noise, nullptr, nullptr), "md");
  s.list_built = true;
  {
    double ene[13];
    check(b.get_energy(0, ene, nullptr), "get_energy");
    std::vector<double> g(n);
    check(b.get_grad(0, g.data(), nullptr), "get_grad");
    print_energies(0, ene, frms_of(g));
  }
  int step = 0;
  double t = o.t;
  while (step < maxstep) {
    // run to the next step that prints something
    int next = maxstep;
    const bool frames = o.ntwx > 0 && s.traj.open();
    for (int k = step + 1; k <= maxstep; k++) {
      if (k == 1 || k % o.ntpr_md == 0 || k % o.ntpr == 0 || (frames && k % o.ntwx == 0)) {
        next = k;
        break;
      }
    }
    // a frame is written before that step's centre-of-mass removal (sff.c:2341-2351)
    const bool frame = frames && next % o.ntwx == 0;
    const bool com_after = frame && o.nscm > 0 && next % o.nscm == 0;
    if (step == 0 && gammai == 0.0) {
      // Berendsen: the first step's factor comes from the initial kinetic
      // energy; the device derives the later ones (sff.c:2225-2228)
      std::vector<double> ts(1, ekin > 0.01 ? std::sqrt(1. + dttp * (ekin0 / ekin - 1.)) : 1.0);
      check(b.md_set_tscal(ts, nullptr), "md");
    }
    check(b.md_steps(step, next - step, noise, nullptr, nullptr, !com_after), "md");
    if (o.irattle) {
      std::vector<int> st;
      check(b.system_status(st, nullptr), "md");
      if (st[0] == SFFG_ECONSTRAINT) fatal("ERROR in RATTLE");
    }
    t += o.dt * (next - step);
    step = next;
    std::vector<double> ek;
    check(b.md_kinetic(ek, nullptr), "md");
    ekin = ek[0];
    double ene[13];
    check(b.get_energy(0, ene, nullptr), "get_energy");
    if (step % o.ntpr == 0) {
      std::vector<double> g(n);
      check(b.get_grad(0, g.data(), nullptr), "get_grad");
      print_energies(step, ene, frms_of(g));
    }
    if (step % o.ntpr_md == 0 || step == 1) {
      std::fprintf(legacy_out(), "md:       %5d %10.3f %10.2f %10.2f %10.2f %10.2f\n", step, t, ekin, ene[0],
                   ekin + ene[0], ekin / (boltz2 * rndf));
      std::fflush(legacy_out());
    }
    if (frame) {
      check(b.get_coords(0, x, nullptr), "get_coords");
      s.traj.write_frame(x, t);
      if (com_after) check(b.md_com_remove(nullptr), "md");
    }
  }
  o.t = t;
  check(b.get_coords(0, x, nullptr), "get_coords");
  check(b.get_velocities(0, v, nullptr), "get_velocities");
  check(b.get_grad(0, f, nullptr), "get_grad");
  timers().md += wall_seconds() - t0;
  return 0;
}

namespace {

// The reference's conjgrad() on the host around an arbitrary energy
// function (src/sff/conjgrad.c:34-263).
int conjgrad_host(double *x0, int n, double *fret, REAL_T (*func)(REAL_T *, REAL_T *, INT_T *), double rmsgrad,
                  double dfpred, int maxiter) {
  std::vector<double> wv(6 * static_cast<size_t>(n) + 1), gv(static_cast<size_t>(n) + 1);
  double *w = wv.data(), *g = gv.data(), *x = x0 - 1, f = 0.0;
  const int maxlin = 10, mxfcon = 4;
  const double dgrad = rmsgrad * rmsgrad * n;
  double gama, beta = 0, fmin = 0, gmin = 0, dfpr = 0, gnew = 0, step = 0, finit = 0, ginit = 0, gsqrd = 0,
         stmin = 0, gamden = 0, ddspln = 0, stepch = 0, sbound = 0, fch = 0, sum = 0;
  int niter = 0, nfbeg = 0, iterc = 0, nfopt = 0, iterfm = 0, iterrs = 0, iretry = 0, ier = 0;
  const int irsdx = n, irsdg = 2 * n, iginit = 3 * n, ixopt = 4 * n, igopt = 5 * n;
  int label = 10;
  for (;;) {
    switch (label) {
      case 10: {
        ++niter;
        int it = niter - 1;
        f = func(x + 1, g + 1, &it);
        if (niter >= 2) { label = 30; break; }
      }
        // fall through
      case 20:
        for (int i = 1; i <= n; ++i) w[i] = -g[i];
        iterrs = 0;
        if (iterc > 0) { label = 40; break; }
        // fall through
      case 30:
        gnew = 0.0;
        sum = 0.0;
        for (int i = 1; i <= n; ++i) {
          gnew += w[i] * g[i];
          sum += g[i] * g[i];
        }
        {
          bool take = niter == 1;
          if (!take) {
            fch = f - fmin;
            take = fch < 0.0 || (fch == 0.0 && gnew / gmin >= -1.0);
          }
          if (take) {
            fmin = f;
            gsqrd = sum;
            nfopt = niter;
            for (int i = 1; i <= n; ++i) {
              w[ixopt + i] = x[i];
              w[igopt + i] = g[i];
            }
            if (sum <= dgrad) { label = 100; break; }
          }
        }
        if (niter == maxiter + 1) { ier = -3; label = 100; break; }
        if (niter > 1) { label = 60; break; }
        dfpr = dfpred;
        stmin = dfpred / gsqrd;
        // fall through
      case 40:
        ++iterc;
        finit = f;
        ginit = 0.0;
        for (int i = 1; i <= n; ++i) {
          w[iginit + i] = g[i];
          ginit += w[i] * g[i];
        }
        if (ginit >= 0.0) { ier = -2; label = 90; break; }
        gmin = ginit;
        sbound = -1.0;
        nfbeg = niter;
        iretry = -1;
        stepch = std::min(stmin, std::fabs(dfpr / ginit));
        stmin = 0.0;
        // fall through
      case 50: {
        step = stmin + stepch;
        double work = 0.0;
        for (int i = 1; i <= n; ++i) {
          x[i] = w[ixopt + i] + stepch * w[i];
          work = std::max(work, std::fabs(x[i] - w[ixopt + i]));
        }
        if (work > 0.0) { label = 10; break; }
        if (niter > nfbeg + 1) ier = -1;
        if (std::fabs(gmin / ginit) > 0.2) ier = -1;
        label = 90;
        break;
      }
      case 60: {
        const double work = (fch + fch) / stepch - gnew - gmin;
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
          if (std::fabs(gmin / ginit) <= 0.2) { label = 90; break; }
          if (niter >= nfopt + maxlin) { ier = -1; label = 90; break; }
        }
      }
        // fall through
      case 70: {
        stepch = (sbound - stmin) * 0.5;
        if (sbound < -0.5) stepch = stmin * 9.0;
        const double gspln = gmin + stepch * ddspln;
        if (gmin * gspln < 0.0) stepch = stepch * gmin / (gmin - gspln);
        label = 50;
        break;
      }
      case 80:
        sum = 0.0;
        for (int i = 1; i <= n; ++i) sum += g[i] * w[iginit + i];
        beta = (gsqrd - sum) / (gmin - ginit);
        if (std::fabs(beta * gmin) > gsqrd * 0.2) {
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
        if (iterrs != 0 && iterc - iterrs < n && std::fabs(sum) < gsqrd * 0.2) {
          double gs = 0.0;
          gama = 0.0;
          for (int i = 1; i <= n; ++i) {
            gama += g[i] * w[irsdg + i];
            gs += g[i] * w[irsdx + i];
          }
          gama /= gamden;
          if (std::fabs(beta * gmin + gama * gs) < gsqrd * 0.2) {
            for (int i = 1; i <= n; ++i) w[i] = -g[i] + beta * w[i] + gama * w[irsdx + i];
            label = 40;
            break;
          }
        }
        gamden = gmin - ginit;
        for (int i = 1; i <= n; ++i) {
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
          for (int i = 1; i <= n; ++i) {
            x[i] = w[ixopt + i];
            g[i] = w[igopt + i];
          }
        }
        if (ier == 0) { label = 80; break; }
        // fall through
      default:
        *fret = f;
        return ier == 0 ? niter : ier;
    }
  }
}

}  // namespace

extern "C" INT_T conjgrad(REAL_T *x, INT_T *n, REAL_T *f, REAL_T (*func)(REAL_T *, REAL_T *, INT_T *),
                          REAL_T *rmsgrad, REAL_T *dfpred, INT_T *maxiter) {
  Session &s = session();
  const double t0 = wall_seconds();
  int ret;
  if (func != &sffg::mme || !s.batch || *n != 3 * s.natom) {
    ret = conjgrad_host(x, *n, f, func, *rmsgrad, *dfpred, *maxiter);
  } else {
    ensure_finalized(x);
    Batch &b = *s.batch;
    check(b.set_coords(0, x, nullptr), "set_coords");
    std::vector<int> status;
    std::vector<double> energy;
    const bool first = !s.list_built;
    auto after = [&](int iter) -> int {
      s.list_built = true;
      const Options &o = options();
      if (iter == 0) print_header();
      if (iter == 0 || iter % o.ntpr == 0 || o.gb_debug) {
        double ene[13];
        int rc = b.get_energy(0, ene, nullptr);
        if (rc) return rc;
        std::vector<double> g(*n);
        if ((rc = b.get_grad(0, g.data(), nullptr))) return rc;
        if (o.gb_debug) print_radii(b);
        print_energies(iter, ene, frms_of(g));
      }
      return 0;
    };
    check(b.cg(*maxiter, *rmsgrad, *dfpred, first, status, energy, nullptr, after), "conjgrad");
    check(b.get_coords(0, x, nullptr), "get_coords");
    *f = energy[0];
    ret = status[0];
  }
  timers().cg += wall_seconds() - t0;
  return ret;
}

extern "C" INT_T mme_timer(void) {
  const Timers &t = timers();
  FILE *out = legacy_out();
  std::fprintf(out, "\n|Timing summary:\n");
  std::fprintf(out, "|              Initialize %11.3f\n", t.init);
  std::fprintf(out, "|             Molec. Dyn. %11.3f\n", t.md);
  std::fprintf(out, "|             Normal Mode %11.3f\n", 0.0);
  std::fprintf(out, "|             Conj. Grad. %11.3f\n", t.cg);
  std::fprintf(out, "|                  Newton %11.3f\n", 0.0);
  std::fprintf(out, "|-------------------------\n");
  std::fprintf(out, "|                   Total %11.3f\n\n", t.init + t.md + t.cg);
  std::fprintf(out, "|1st derivative timing summary:\n");
  std::fprintf(out, "|       device mme calls %8ld\n", t.nevals);
  std::fprintf(out, "|       host mme() wall  %11.3f\n", t.mme);
  std::fflush(out);
  return 0;
}

extern "C" REAL_T rand2(void) { return rng().uniform(); }

extern "C" REAL_T gauss2(REAL_T *mean, REAL_T *sd) { return rng().gauss(*mean, *sd); }

extern "C" void mm_set_checkpoint(STRING_T **fname) {
  checkpoint_name() = (fname && *fname) ? *fname : "";
  std::fprintf(legacy_out(), "\tcheckpoint:  %s\n", checkpoint_name().c_str());
  std::fflush(legacy_out());
}

extern "C" INT_T setseed(INT_T *seed) {
  if (*seed >= 0) {
    std::fprintf(stderr, "argument to setseed must be negative!\n");
    return 1;
  }
  rng().seed3 = *seed;
  return 0;
}

extern "C" REAL_T mme_rattle(REAL_T *x, REAL_T *f, INT_T *iter) {
  if (*iter == -3) return mme(x, f, iter);
  Session &s = session();
  const Options &o = options();
  if (!s.prm) fatal("mme_rattle: mme_init_sff has not been called");
  const int n3 = 3 * s.natom;
  // unit-free dummies, as the reference uses (inverse masses 2, velocities 0)
  std::vector<double> minv(n3, 2.0), dumv(n3, 0.0);
  rattle_positions(s.prm, o.irattle, o.dt * 20.455, x, x, dumv.data(), minv.data());
  const double e = mme(x, f, iter);
  int niter = 0;
  bool done = false;
  while (!done && niter < 50) {
    niter++;
    done = true;
    for_constrained_bonds(s.prm, o.irattle, [&](int a1, int a2, double) {
      const double xr = x[a2] - x[a1], yr = x[a2 + 1] - x[a1 + 1], zr = x[a2 + 2] - x[a1 + 2];
      const double d2 = xr * xr + yr * yr + zr * zr;
      const double ip = xr * (f[a1] - f[a2]) + yr * (f[a1 + 1] - f[a2 + 1]) + zr * (f[a1 + 2] - f[a2 + 2]);
      if (ip > 0.0000001) done = false;
      f[a1] -= (xr / (2.0 * d2)) * ip;
      f[a1 + 1] -= (yr / (2.0 * d2)) * ip;
      f[a1 + 2] -= (zr / (2.0 * d2)) * ip;
      f[a2] += (xr / (2.0 * d2)) * ip;
      f[a2 + 1] += (yr / (2.0 * d2)) * ip;
      f[a2 + 2] += (zr / (2.0 * d2)) * ip;
    });
  }
  if (*iter == -1) {
    double frms = 0.0;
    for (int i = 0; i < n3; i++) frms += f[i] * f[i];
    std::fprintf(legacy_out(), "     frms:  %15.9f (corrected for rattle)\n", std::sqrt(frms / n3));
  }
  return e;
}
