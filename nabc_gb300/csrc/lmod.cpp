// LMOD, the reference's low-mode conformational search and docking
// (src/sff/lmodC.c): from a minimised structure, repeatedly push it along
// its lowest vibrational modes, relax and minimise the result, keep the
// low-energy, mutually distinct minima found in an energy-sorted archive
// ("conflib"), pick the next structure by a Monte Carlo rule, restart from
// the archive periodically and, for docking, move ligands rigidly.  The
// interface is the reference's (include/sff.h): lmod() drives mme() and
// xmin() itself; lmodC() is the reverse-communication form; lmod_opt_init()
// sets the defaults.  sffg_lmod_func() (include/sffg.h) is lmod() over any
// energy function.
//
// One C++20 coroutine runs a search.  Each point where the reference's state
// machine hands control back (lmodC.c:2209-2237; return_flag codes 1-7,
// labels 2-7) is a co_yield, and lmodC() resumes it.  The steps follow the
// reference one for one -- the same random-number draws from the rand2()
// stream in the same order, the same sums in index order -- so on a
// deterministic energy function a search takes the reference's path and
// leaves the same archive, trajectory and conflib.dat bit for bit, given
// the same low modes.  Those come from LowModes (lowmodes.h), this
// library's replacement for the reference's Fortran ARPACK driver.
//
// Behaviour kept from the reference, including its quirks:
//  * the sort of the modes by |eigenvalue| never runs (lmodC.c:2403-2409
//    calls it only on an error), so modes are taken in ascending algebraic
//    order of the eigenvalues, the first nrotran_dof skipped;
//  * a conflib.dat left in the working directory seeds the archive and the
//    start structure (lmodC.c:2243-2276), and the file is rewritten every
//    10 iterations and at the end; entries read from it restart with
//    multiplicity 1;
//  * "Rg" is the spread of the atoms' distances from their centre
//    (lmodC.c:624-652), not the radius of gyration;
//  * the finite-difference Hessian product restores coordinates and
//    gradient after each product (lmodC.c:1341-1425);
//  * ndim_arnoldi (the caller's variable) is overwritten with the Krylov
//    dimension used, and nconf with the number of structures returned.
// Atoms whose incoming gradient is exactly zero are frozen and left out of
// the modes, as in the reference.  One search runs at a time per process.
#include <sys/time.h>

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <memory>
#include <vector>

#include "coro.h"
#include "lowmodes.h"
#include "sffg_internal.h"

namespace {

using sffg::Gen;

// return_flag requests (lmodC.c:55-62)
constexpr int kDone = 0, kCalcBothNewList = 2, kCalcGradOldList = 3, kMinimize = 5, kRelax = 6, kFirstMinim = 7;
// statuses (lmodC.c:63-69; -2 is the ARPACK driver's own failure code)
constexpr int kParamsError = -1, kArpackError = -2, kFileError = -4, kConflibError = -7;
constexpr double kBig = 1e10, kTiny = 1e-20, kPi = 3.141592653589793;
constexpr int kMetropolis = 1, kQuickQuenching = 3;
constexpr int kMaxMcTry = 10000, kMaxZigzagIter = 20, kConflibUpdate = 10;
constexpr double kFullyMinimized = 10.0;
constexpr double kArpackTol = 1e-4;
constexpr int kArpackIter = 1000000;

inline double sq(double a) { return a * a; }

// "Rg" of the reference (lmodC.c:624-652): the standard deviation of the
// atoms' distances from their centre.
double calc_rad(int natm, const double *xyz) {
  double avg = 0.0, var = 0.0;
  double c[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < natm; i++) {
    c[0] += xyz[i * 3];
    c[1] += xyz[i * 3 + 1];
    c[2] += xyz[i * 3 + 2];
  }
  c[0] /= natm;
  c[1] /= natm;
  c[2] /= natm;
  for (int i = 0; i < natm; i++) {
    double d = sq(xyz[i * 3] - c[0]) + sq(xyz[i * 3 + 1] - c[1]) + sq(xyz[i * 3 + 2] - c[2]);
    var += d;
    avg += std::sqrt(d);
  }
  avg /= natm;
  var = var / natm - sq(avg);
  return std::sqrt(var > 0.0 ? var : 0.0);
}

// All-atom RMS deviation (want_max: largest single-atom deviation) after
// optimal superposition, by Kabsch's method (Acta Cryst. A32 (1976) 922,
// A34 (1978) 827) as the reference forms it (lmodC.c:845-970): the 0.1-
// scaled correlation matrix R, the eigenvectors of R^T R (largest two, the
// third their cross product), the rotation from them.  Neither input is
// changed.
double rmsfit(int ndim, const double *ref_in, const double *xyz_in, bool want_max) {
  const int natm = ndim / 3;
  std::vector<double> ref(ref_in, ref_in + ndim), xyz(xyz_in, xyz_in + ndim);
  double cr[3] = {0.0, 0.0, 0.0}, cx[3] = {0.0, 0.0, 0.0};
  for (int n = 0; n < natm; n++)
    for (int k = 0; k < 3; k++) {
      cr[k] += ref[n * 3 + k];
      cx[k] += xyz[n * 3 + k];
    }
  for (int k = 0; k < 3; k++) {
    cr[k] /= natm;
    cx[k] /= natm;
  }
  for (int n = 0; n < natm; n++)
    for (int k = 0; k < 3; k++) {
      ref[n * 3 + k] -= cr[k];
      xyz[n * 3 + k] -= cx[k];
    }
  double r[3][3] = {{0.0}};
  for (int n = 0; n < natm; n++)
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++) r[i][j] += 0.1 * ref[n * 3 + i] * xyz[n * 3 + j];
  double rtr[9], d[3], zz[9];
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) rtr[j * 3 + i] = r[0][i] * r[0][j] + r[1][i] * r[1][j] + r[2][i] * r[2][j];
  sffg::sym_eigen(3, rtr, d, zz);
  double z[3][3], b[3][3], u[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) z[i][j] = zz[i * 3 + j];
  z[0][2] = z[1][0] * z[2][1] - z[2][0] * z[1][1];
  z[1][2] = z[2][0] * z[0][1] - z[0][0] * z[2][1];
  z[2][2] = z[0][0] * z[1][1] - z[1][0] * z[0][1];
  for (int j = 0; j < 2; j++) {
    for (int i = 0; i < 3; i++) b[i][j] = r[i][0] * z[0][j] + r[i][1] * z[1][j] + r[i][2] * z[2][j];
    const double fac = std::sqrt(b[0][j] * b[0][j] + b[1][j] * b[1][j] + b[2][j] * b[2][j]);
    for (int i = 0; i < 3; i++) b[i][j] /= (fac > kTiny ? fac : kTiny);
  }
  b[0][2] = b[1][0] * b[2][1] - b[2][0] * b[1][1];
  b[1][2] = b[2][0] * b[0][1] - b[0][0] * b[2][1];
  b[2][2] = b[0][0] * b[1][1] - b[1][0] * b[0][1];
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) u[i][j] = b[i][0] * z[j][0] + b[i][1] * z[j][1] + b[i][2] * z[j][2];
  double dsq = 0.0, dmax = 0.0;
  for (int n = 0; n < natm; n++) {
    const double x = xyz[n * 3], y = xyz[n * 3 + 1], zc = xyz[n * 3 + 2];
    double s[3];
    for (int k = 0; k < 3; k++) {
      const double t = u[k][0] * x + u[k][1] * y + u[k][2] * zc;
      s[k] = sq(t - ref[n * 3 + k]);
      dsq += s[k];
    }
    if (s[0] + s[1] + s[2] > dmax) dmax = s[0] + s[1] + s[2];
  }
  return want_max ? std::sqrt(dmax) : std::sqrt(dsq / natm);
}

// The archive of minima, sorted by increasing energy (lmodC.c:237-352).
struct Entry {
  double energy, rad;
  int mult;
  std::vector<double> xyz;
};

class Archive {
 public:
  std::vector<Entry> e;

  // A new structure goes before the first entry of equal or higher energy.
  void add(int ndim, const double *xyz, double energy, double rad) {
    size_t at = 0;
    while (at < e.size() && !(energy <= e[at].energy)) at++;
    e.insert(e.begin() + static_cast<long>(at), Entry{energy, rad, 1, std::vector<double>(xyz, xyz + ndim)});
  }

  // Drops entries above the energy window, then every entry within
  // separation_rms of a lower one, adding its multiplicity to that one
  // (lmodC.c:354-423); returns the number left.
  int update(int ndim_ext, int ndim_local, double window, double separation) {
    for (size_t i = 0; i < e.size(); i++)
      if (std::fabs(e[i].energy - e[0].energy) > window) {
        e.resize(i);
        break;
      }
    const double scale = std::sqrt(static_cast<double>(ndim_ext) / static_cast<double>(ndim_local));
    for (size_t c = 0; c + 1 < e.size(); c++) {
      for (size_t k = c + 1; k < e.size();) {
        const double rms = rmsfit(ndim_ext, e[c].xyz.data(), e[k].xyz.data(), false) * scale;
        if (rms <= separation) {
          e[c].mult += e[k].mult;
          e.erase(e.begin() + static_cast<long>(k));
        } else {
          k++;
        }
      }
    }
    return static_cast<int>(e.size());
  }

  // conflib.dat: per entry the energy (f64), the spread (f64), the
  // multiplicity (i32) and the coordinates (f64), packed.
  bool write(const char *name, int ndim) const {
    FILE *f = std::fopen(name, "wb");
    if (!f) {
      std::fprintf(stderr, "\nERROR in write_archive(): Cannot open %s.\n", name);
      std::fflush(stderr);
      return false;
    }
    for (const Entry &x : e) {
      std::fwrite(&x.energy, sizeof(double), 1, f);
      std::fwrite(&x.rad, sizeof(double), 1, f);
      std::fwrite(&x.mult, sizeof(int), 1, f);
      std::fwrite(x.xyz.data(), sizeof(double), ndim, f);
    }
    std::fclose(f);
    return true;
  }

  // Adds every complete record of a conflib.dat (multiplicities restart at 1).
  bool read_and_sort(const char *name, int ndim) {
    FILE *f = std::fopen(name, "rb");
    if (!f) {
      std::fprintf(stderr, "\nERROR in read_and_sort_archive(): Cannot open %s.\n", name);
      std::fflush(stderr);
      return false;
    }
    std::vector<double> xyz(ndim);
    for (;;) {
      double energy, rad;
      int mult;
      if (std::fread(&energy, sizeof(double), 1, f) < 1) break;
      if (std::fread(&rad, sizeof(double), 1, f) < 1) break;
      if (std::fread(&mult, sizeof(int), 1, f) < 1) break;
      if (std::fread(xyz.data(), sizeof(double), ndim, f) < static_cast<size_t>(ndim)) break;
      add(ndim, xyz.data(), energy, rad);
    }
    const bool ok = !std::ferror(f);
    if (!ok) {
      std::fprintf(stderr, "\nERROR in read_archive(): Input error in %s.\n", name);
      std::fflush(stderr);
    }
    std::fclose(f);
    return ok;
  }

  // One of the nmax lowest structures, chosen by one uniform draw.
  template <class Draw>
  void restart(int ndim, int nmax, double *xyz, Draw draw) const {
    if (e.empty()) return;
    const int nrand = 1 + static_cast<int>(nmax * draw());
    size_t n = 0;
    for (const Entry &x : e) {
      std::memcpy(xyz, x.xyz.data(), ndim * sizeof(double));
      if (static_cast<int>(++n) == nrand) break;
    }
  }
};

// Pulls atoms closer than 1 A apart to at least 1.2 A along their axis, up
// to five passes (lmodC.c:1520-1683); frozen atoms (zero gradient) stay put
// and their partner moves twice as far.  all_pairs: every pair; else each
// ligand atom against every atom outside its ligand.
void separate_close_pairs(bool all_pairs, int ndim, double *xyz, const double *grad, int nligs,
                          const int *lig_start, const int *lig_end) {
  const int natm = ndim / 3;
  auto frozen = [&](int i) { return grad[i * 3] == 0.0 && grad[i * 3 + 1] == 0.0 && grad[i * 3 + 2] == 0.0; };
  auto fix = [&](int i, int j, bool fi, bool &problem) {
    if (fi && frozen(j)) return;
    const bool fj = frozen(j);
    double dx = xyz[i * 3] - xyz[j * 3], dy = xyz[i * 3 + 1] - xyz[j * 3 + 1], dz = xyz[i * 3 + 2] - xyz[j * 3 + 2];
    const double dist2 = sq(dx) + sq(dy) + sq(dz);
    if (!(dist2 < 1.0)) return;
    problem = true;
    if (dist2 == 0.0) {
      dx = dy = dz = (fi || fj) ? std::sqrt(2. / 5.) : std::sqrt(1. / 5.);
    } else {
      const double dist = std::sqrt(dist2);
      double frac = (1.2 - dist) / (2.0 * dist);
      if (fi || fj) frac *= 2.0;
      dx *= frac;
      dy *= frac;
      dz *= frac;
    }
    if (!fi) {
      xyz[i * 3] += dx;
      xyz[i * 3 + 1] += dy;
      xyz[i * 3 + 2] += dz;
    }
    if (!fj) {
      xyz[j * 3] -= dx;
      xyz[j * 3 + 1] -= dy;
      xyz[j * 3 + 2] -= dz;
    }
  };
  for (int cycle = 0; cycle < 5; cycle++) {
    bool problem = false;
    if (all_pairs) {
      for (int i = 0; i < natm; i++) {
        const bool fi = frozen(i);
        for (int j = i + 1; j < natm; j++) fix(i, j, fi, problem);
      }
    } else {
      for (int l = 0; l < nligs; l++)
        for (int i = lig_start[l] - 1; i < lig_end[l]; i++) {
          const bool fi = frozen(i);
          for (int j = 0; j < lig_start[l] - 1; j++) fix(i, j, fi, problem);
          for (int j = lig_end[l]; j < natm; j++) fix(i, j, fi, problem);
        }
    }
    if (!problem) break;
  }
}

void rot_matrix(double alpha, double ax, double ay, double az, double m[3][3]) {
  const double ca = std::cos(alpha), sa = std::sin(alpha);
  m[0][0] = ax * ax + ca * (1.0 - ax * ax);
  m[0][1] = (1.0 - ca) * ax * ay - sa * az;
  m[0][2] = (1.0 - ca) * ax * az + sa * ay;
  m[1][0] = (1.0 - ca) * ay * ax + sa * az;
  m[1][1] = ay * ay + ca * (1.0 - ay * ay);
  m[1][2] = (1.0 - ca) * ay * az - sa * ax;
  m[2][0] = (1.0 - ca) * az * ax - sa * ay;
  m[2][1] = (1.0 - ca) * az * ay + sa * ax;
  m[2][2] = az * az + ca * (1.0 - az * az);
}

// Arguments of one lmodC() call, as pointers (refreshed on every call).
struct Args {
  int *nlmodit, *nmod, *kmod, *rotran, *natm_ext;
  double *xyz_ext, *enrg, *grad_ext;
  int *nconf;
  double *enrg_win, *separ_rms, *conflib, *trajectory;
  int *arpk_recalc, *arpk_dim, *lmod_restart, *topten, *mc_option;
  double *rtemp, *lmod_step_min, *lmod_step_max;
  int *nof_lmod_step, *nligs, *lig_start, *lig_end, *try_now, *ntry;
  double *trmin, *trmax;
  int *lig_rot_cent;
  double *angmin, *angmax;
  int *seed, *print_level;
  double *lmod_time, *extn_time;
  int *return_flag;
};

// Checks the parameters as the reference does (lmodC.c:1733-1955); prints
// its message and returns false on the first violation.
bool check_params(const Args &a) {
  auto fail = [](const char *msg) {
    std::fprintf(stderr, "\nERROR in lmod(): %s\n", msg);
    std::fflush(stderr);
    return false;
  };
  if (*a.nlmodit < 0) return fail("Requested number of LMOD iterations negative.");
  if (*a.nmod < 1) return fail("Wrong number of vibrational modes.");
  if (*a.kmod < 1) return fail("Wrong number of variable modes.");
  if (*a.kmod > *a.nmod) return fail("Number of variable modes > total number of modes.");
  if (*a.rotran < 0) return fail("Wrong number of trans/rot modes.");
  if (*a.natm_ext < 0) return fail("Number of atoms negative.");
  if (*a.natm_ext < 2) return fail("Too few atoms.");
  if (*a.nconf <= 0) return fail("Requested number of confs zero or negative.");
  if (*a.enrg_win < 0.0) return fail("Energy window negative.");
  if (*a.separ_rms <= 0.0) return fail("Conf separation RMS zero or negative.");
  if (*a.arpk_recalc <= 0) return fail("Eigvec update frequency zero or negative.");
  if (*a.arpk_dim < 0) return fail("Requested number of Arnoldi basis vectors negative.");
  if (*a.arpk_dim > 0 && *a.arpk_dim < *a.nmod + 1)
    return fail(
        "Number of Arnoldi basis vectors should be at least one\n                 more than the requested "
        "number of vibrational modes.");
  if (*a.lmod_restart <= 0) return fail("LMOD restart frequency zero or negative.");
  if (*a.topten <= 0) return fail("Pool of structures for LMOD restart empty.");
  if (*a.mc_option < 1 || *a.mc_option > 3) return fail("Unknown Monte Carlo option.");
  if (*a.rtemp <= 0.0) return fail("RT should be positive.");
  if (*a.lmod_step_min <= 0.0) return fail("Min. LMOD step size should be positive.");
  if (*a.lmod_step_max <= 0.0) return fail("Max. LMOD step size should be positive.");
  if (*a.lmod_step_min > *a.lmod_step_max) return fail("LMOD step min/max reversed.");
  if (*a.nof_lmod_step < 0) return fail("Requested number of LMOD steps negative.");
  if (*a.nligs < 0) return fail("User-defined number of ligands negative.");
  char msg[128];
  for (int i = 0; i < *a.nligs; i++) {
    if (a.lig_start[i] < 1 || a.lig_start[i] > *a.natm_ext || a.lig_end[i] < 1 || a.lig_end[i] > *a.natm_ext ||
        a.lig_start[i] > a.lig_end[i]) {
      std::snprintf(msg, sizeof msg, "Ligand %d's start/end out of range.", i + 1);
      return fail(msg);
    }
    if (a.trmin[i] > a.trmax[i]) {
      std::snprintf(msg, sizeof msg, "Ligand %d's trans min/max reversed.", i + 1);
      return fail(msg);
    }
    if (a.angmin[i] > a.angmax[i]) {
      std::snprintf(msg, sizeof msg, "Ligand %d's rot min/max reversed.", i + 1);
      return fail(msg);
    }
    if (a.lig_rot_cent[i] != 0 &&
        (a.lig_rot_cent[i] < 0 || a.lig_rot_cent[i] < a.lig_start[i] || a.lig_rot_cent[i] > a.lig_end[i])) {
      std::snprintf(msg, sizeof msg, "Ligand %d's rot center out of range.", i + 1);
      return fail(msg);
    }
  }
  if (*a.try_now <= 0) return fail("LMOD iter vs. ligand trans/rot frequency must be positive.");
  if (*a.ntry < 0) return fail("Requested number of ligand trans/rot moves negative.");
  if (*a.seed < 0) return fail("User-defined random seed negative.");
  if (*a.print_level < 0 || *a.print_level > 5) return fail("Print level out of range.");
  return true;
}

// A yield: the request for the caller and the label lmodC() reports.
constexpr int yield_code(int request, int label) { return request * 16 + label; }

class Search {
 public:
  Args a{};
  double hess_eps = 2.2204460492503131e-16;  // relative gradient precision for the Hessian products
  double glob_min = 0.0;
  clock_t lmod_stamp = 0, extn_stamp = 0;
  // a search of its own stream (batched searches) or the process-global
  // rand2() stream (lmod(), lmodC(), as the reference)
  sffg::Rand2 *own_rng = nullptr;
  // conflib.dat read at the start and written as the reference does
  bool use_files = true;

  Gen run() {
    const int pl = *a.print_level;
    print_ = (pl >= 1 && pl <= 3);
    debug_ = (pl == 2 || pl == 3);
    debug_modes_ = (pl == 3 || pl == 4);
    zigzag_ = (pl == 5);
    FILE *out = sffg::legacy_out();
    // atoms with a zero incoming gradient are frozen (lmodC.c:1994-2001)
    const int natm_ext = *a.natm_ext;
    for (int i = 0; i < natm_ext; i++)
      if (a.grad_ext[i * 3] != 0 || a.grad_ext[i * 3 + 1] != 0 || a.grad_ext[i * 3 + 2] != 0) idx_.push_back(i);
    natm_ = static_cast<int>(idx_.size());
    nd_ = 3 * natm_;
    next_ = 3 * natm_ext;
    if (*a.arpk_dim == 0) {
      *a.arpk_dim = nd_;
    } else {
      *a.arpk_dim += *a.rotran;
      *a.arpk_dim = std::min(*a.arpk_dim, nd_);
    }
    int nreq = std::min(*a.nmod, nd_ - 1);
    nreq = std::min(nreq + *a.rotran, nd_ - 1);
    const int max_zz = *a.nof_lmod_step == 0 ? kMaxZigzagIter : *a.nof_lmod_step;
    const bool barrier_test = *a.nof_lmod_step == 0;
    x_.assign(nd_, 0.0);
    g_.assign(nd_, 0.0);
    gather_x();
    int seed3;
    if (*a.seed > 0) {
      seed3 = -*a.seed;
    } else {
      timeval tv;
      gettimeofday(&tv, nullptr);
      seed3 = -static_cast<int>(tv.tv_sec ^ tv.tv_usec);
      if (seed3 == 0) seed3 = -1;
    }
    if (own_rng)
      own_rng->seed3 = seed3;
    else
      setseed(&seed3);

    // a conflib.dat from an earlier search seeds this one
    if (FILE *f = use_files ? std::fopen("conflib.dat", "rb") : nullptr) {
      std::fclose(f);
      std::fprintf(out, "\n*****  W A R N I N G  *****\n\n");
      std::fprintf(out, "It appears that results from a previous LMOD search were found\n");
      std::fprintf(out, "in conflib.dat in the launch directory.  LMOD will assume that\n");
      std::fprintf(out, "those molecules in conflib.dat are low-energy conformations of\n");
      std::fprintf(out, "the current input molecule of the present LMOD run and will be\n");
      std::fprintf(out, "used to seed the new search with multiple conformations.\n\n");
      std::fprintf(out, "If conflib.dat is incompatible with the current search, *KILL*\n");
      std::fprintf(out, "this LMOD job, remove conflib.dat, and restart LMOD.\n\n");
      if (!arch_.read_and_sort("conflib.dat", next_)) co_return kFileError;
      arch_.restart(next_, 1, a.xyz_ext, [this] { return draw(); });
      gather_x();
    }
    // minimise the start structure
    scatter_x();
    co_yield yield_code(kFirstMinim, 2);
    gather_x();
    arch_.add(next_, a.xyz_ext, *a.enrg, calc_rad(natm_, x_.data()));
    if (!zigzag_) std::memcpy(a.trajectory, a.xyz_ext, next_ * sizeof(double));
    if (print_) {
      std::fprintf(out, "__________________________________________________");
      if (debug_) std::fprintf(out, "_________________________");
      std::fprintf(out, "\n                  Low-Mode Simulation\n");
      if (!debug_) std::fprintf(out, "-----------------------------------------------\n");
    }

    std::vector<double> vals, vecs, cent(nd_), vec(nd_), hold(nd_), trot(nd_), pboltz(2 * (nreq + 1));
    std::vector<double> moves(2 * static_cast<size_t>(nreq + 1) * nd_);
    std::vector<int> sign(nreq > 0 ? nreq : 1);
    int ncm = 0, n = 0, size = 0;
    for (int it = 0; it < *a.nlmodit; it++) {
      scatter_x();
      co_yield yield_code(kCalcBothNewList, 3);
      gather_g();
      const double ref_energy = *a.enrg;
      double grad_rms = rms(g_);
      if (it % *a.arpk_recalc == 0) {
        // the low modes: Lanczos over finite-difference Hessian products
        sffg::LowModes lm;
        if (lm.init(nd_, nreq, *a.arpk_dim, kArpackTol, kArpackIter - 1)) co_return kArpackError;
        const double sqrt_eps = std::sqrt(hess_eps);
        std::vector<double> xs(nd_), gs(nd_);
        int r;
        gather_g();  // products are taken about the gradient just evaluated
        while ((r = lm.iterate()) == 1) {
          const double *v = lm.in();
          gs = g_;
          xs = x_;
          double dot = 0.0;
          for (int i = 0; i < nd_; i++) dot += sq(xs[i]);
          const double xnorm = std::sqrt(dot);
          dot = 0.0;
          for (int i = 0; i < nd_; i++) dot += sq(v[i]);
          const double step = 2. * sqrt_eps * (1.0 + xnorm) / std::sqrt(dot);
          for (int i = 0; i < nd_; i++) x_[i] += step * v[i];
          scatter_x();
          co_yield yield_code(kCalcGradOldList, 4);
          gather_g();
          double *hv = lm.out();
          for (int i = 0; i < nd_; i++) hv[i] = (g_[i] - gs[i]) / step;
          x_ = xs;
          g_ = gs;
        }
        if (r < 0) co_return kArpackError;
        ncm = lm.nconv();
        vals.assign(lm.values(), lm.values() + ncm);
        vecs.assign(lm.vectors(), lm.vectors() + static_cast<size_t>(ncm) * nd_);
        if (debug_modes_) {
          std::fprintf(out, "\n low modes: %d of %d converged, %d restarts, %d Hessian products\n", ncm, nreq,
                       lm.restarts(), lm.products());
          for (int k = 0; k < ncm; k++) std::fprintf(out, " %12.5g", vals[k]);
          std::fprintf(out, "\n");
        }
      }
      cent = x_;
      if (debug_) {
        std::fprintf(out, "--------------------------------------");
        std::fprintf(out, "-------------------------------------\n");
      }
      if (print_) {
        std::fprintf(out, "%6d   %cE =%13.3f (%6.3f)  Rg = %8.3f\n", it + 1,
                     (*a.nligs && !(it % *a.arpk_recalc) && it) ? '*' : ' ', ref_energy, grad_rms,
                     calc_rad(natm_, x_.data()));
        std::fflush(out);
      }
      // a random sign for each mode of the mixed mode
      for (int i = 0; i < ncm; i++) sign[i] = draw() < 0.5 ? 1 : -1;
      const int rotran = *a.rotran, kmod = *a.kmod;
      double min_energy = kBig;
      int kk = 0, cnt = 0;
      bool quenched = false;
      for (int k = rotran; k <= ncm && !quenched; k++) {
        // kmod of the modes at random, then the mixed mode
        if (cnt == kmod) k = ncm;
        if (kmod < (ncm - rotran) && (kmod - cnt) < (ncm - k) &&
            draw() >= (static_cast<double>(kmod) / static_cast<double>(ncm - rotran)))
          continue;
        cnt++;
        for (int i = 0; i < nd_; i++) {
          if (k < ncm) {
            vec[i] = vecs[static_cast<size_t>(k) * nd_ + i];
          } else {
            vec[i] = 0.0;
            for (int j = rotran; j < ncm; j++) vec[i] += sign[j] * vecs[static_cast<size_t>(j) * nd_ + i];
          }
        }
        size_t offset = 0;
        if (zigzag_) {
          offset = static_cast<size_t>(next_) * (4 * max_zz + 3) * (it * kmod + k - rotran);
          scatter(cent.data());
          std::memcpy(a.trajectory + offset, a.xyz_ext, next_ * sizeof(double));
        }
        for (int l = 1; l <= 2 && !quenched; l++) {
          // ZIG: the fastest atom moves a random step along the mode;
          // ZAG: relax; until the path has crossed a barrier
          double max_atmov = 0.0;
          for (int i = 0; i < natm_; i++) {
            double s = 0.0;
            for (int j = 0; j < 3; j++) s += sq(vec[i * 3 + j]);
            if (s > max_atmov) max_atmov = s;
          }
          max_atmov = std::sqrt(max_atmov);
          const double step = *a.lmod_step_min + (*a.lmod_step_max - *a.lmod_step_min) * draw();
          const double scale = step / max_atmov;
          double energy_old = ref_energy, rms_old = 0.0;
          int zz;
          for (zz = 0; zz < max_zz; zz++) {
            for (int i = 0; i < nd_; i++) x_[i] += scale * vec[i];
            scatter_x();
            separate_close_pairs(true, next_, a.xyz_ext, a.grad_ext, *a.nligs, a.lig_start, a.lig_end);
            gather_x();
            scatter_x();
            co_yield yield_code(kRelax, 5);
            gather_x();
            if (zigzag_) {
              std::memcpy(a.trajectory + offset + static_cast<size_t>(next_) * ((l - 1) * (2 * max_zz + 1) + zz + 1),
                          a.xyz_ext, next_ * sizeof(double));
              std::memcpy(a.trajectory + offset + static_cast<size_t>(next_) * (2 * max_zz * l + (l - 1) - zz),
                          a.xyz_ext, next_ * sizeof(double));
            }
            if (barrier_test) {
              const double r = rmsfit(nd_, cent.data(), x_.data(), false);
              if (*a.enrg < ref_energy || (*a.enrg < energy_old && r > rms_old)) break;
              energy_old = *a.enrg;
              rms_old = r;
            }
          }
          if (zigzag_) {
            scatter(cent.data());
            std::memcpy(a.trajectory + offset + static_cast<size_t>(next_) * l * (2 * max_zz + 1), a.xyz_ext,
                        next_ * sizeof(double));
          }
          // minimise the end point
          scatter_x();
          co_yield yield_code(kMinimize, 6);
          gather_x();
          gather_g();
          const double energy = *a.enrg;
          grad_rms = rms(g_);
          if (grad_rms <= kFullyMinimized)
            pboltz[kk++] = energy <= ref_energy ? 1.0 : std::exp(-(energy - ref_energy) / *a.rtemp);
          else
            pboltz[kk++] = 0.0;
          arch_.add(next_, a.xyz_ext, energy, calc_rad(natm_, x_.data()));
          for (int i = 0; i < nd_; i++) moves[static_cast<size_t>(kk - 1) * nd_ + i] = x_[i] - cent[i];
          if (debug_) {
            const double r = rmsfit(nd_, cent.data(), x_.data(), false);
            std::fprintf(out, "%3d  /%2d %cE =%13.3f (%6.3f)  Rg = %8.3f  rmsd=%7.3f  p=%7.4f\n",
                         (k < ncm) ? (k - rotran + 1) : 0, std::min(zz + 1, max_zz),
                         (grad_rms <= kFullyMinimized) ? ' ' : '!', energy, grad_rms, calc_rad(natm_, x_.data()), r,
                         pboltz[kk - 1]);
            std::fflush(out);
          }
          // total quenching keeps the lowest neighbour; quick quenching
          // takes the first one below the centre
          if (energy <= min_energy) {
            min_energy = energy;
            n = kk - 1;
            if (*a.mc_option == kQuickQuenching && min_energy < ref_energy) {
              quenched = true;
              break;
            }
          }
          x_ = cent;
          for (int i = 0; i < nd_; i++) vec[i] = -vec[i];
        }
      }
      if (!quenched && *a.mc_option == kMetropolis) {
        int tries = 0;
        do {
          n = static_cast<int>(kk * draw());
        } while (draw() > pboltz[n] && ++tries < kMaxMcTry);
      }
      for (int i = 0; i < nd_; i++) x_[i] = cent[i] + moves[static_cast<size_t>(n) * nd_ + i];
      scatter_x();
      if (!zigzag_)
        std::memcpy(a.trajectory + static_cast<size_t>(it + 1) * next_, a.xyz_ext, next_ * sizeof(double));
      // prune and save the archive; restart from one of its best
      if ((it % *a.lmod_restart == *a.lmod_restart - 1) || (it % kConflibUpdate == kConflibUpdate - 1)) {
        size = arch_.update(next_, nd_, *a.enrg_win, *a.separ_rms);
        if (use_files && !arch_.write("conflib.dat", next_)) co_return kFileError;
        if (print_) {
          std::fprintf(out, "__________________________________________________\n");
          std::fprintf(out, " Top Ten:\n");
          int c = 0;
          for (const Entry &x : arch_.e) {
            std::fprintf(out, "   %5d  E =%13.3f /%2d  Rg = %8.3f\n", ++c, x.energy, x.mult, x.rad);
            if (c == 10) break;
          }
          std::fprintf(out, "--------------------------------------------------\n");
          std::fprintf(out, " Total Nof confs = %5d\n", size);
          std::fprintf(out, "________________________\n");
          std::fflush(out);
        }
        if (it % *a.lmod_restart == *a.lmod_restart - 1) {
          arch_.restart(next_, std::min(*a.topten, size), a.xyz_ext, [this] { return draw(); });
          gather_x();
        }
      }
      // docking: every try_now-th iteration, ntry random rigid moves of the
      // ligands, each minimised; the lowest is kept
      if (*a.nligs && it < *a.nlmodit - 1 && !((it + 1) % *a.try_now)) {
        hold = x_;
        double best = kBig;
        for (int t = 0; t < *a.ntry; t++) {
          for (int l = 0; l < *a.nligs; l++) {
            double tx, ty, tz, tn;
            do {
              tx = 2 * draw() - 1;
              ty = 2 * draw() - 1;
              tz = 2 * draw() - 1;
            } while ((tn = std::sqrt(sq(tx) + sq(ty) + sq(tz))) < kTiny);
            const double ts = a.trmin[l] + (a.trmax[l] - a.trmin[l]) * draw();
            tx *= ts / tn;
            ty *= ts / tn;
            tz *= ts / tn;
            lig_start_ = local_index(a.lig_start[l] - 1, lig_start_);
            lig_end_ = local_index(a.lig_end[l] - 1, lig_end_);
            for (int i = lig_start_; i <= lig_end_; i++) {
              x_[3 * i] += tx;
              x_[3 * i + 1] += ty;
              x_[3 * i + 2] += tz;
            }
            double rx, ry, rz, rn;
            do {
              rx = 2 * draw() - 1;
              ry = 2 * draw() - 1;
              rz = 2 * draw() - 1;
            } while ((rn = std::sqrt(sq(rx) + sq(ry) + sq(rz))) < kTiny);
            rx /= rn;
            ry /= rn;
            rz /= rn;
            const double ang = a.angmin[l] + (a.angmax[l] - a.angmin[l]) * draw();
            double m[3][3];
            rot_matrix((kPi / 180.) * ang, rx, ry, rz, m);
            double c[3] = {0.0, 0.0, 0.0};
            if (a.lig_rot_cent[l]) {
              lig_cent_ = local_index(a.lig_rot_cent[l] - 1, lig_cent_);
              for (int k = 0; k < 3; k++) c[k] = x_[lig_cent_ * 3 + k];
            } else {
              for (int i = lig_start_; i <= lig_end_; i++)
                for (int k = 0; k < 3; k++) c[k] += x_[3 * i + k];
              const int cnt_l = (lig_end_ - lig_start_) + 1;
              for (int k = 0; k < 3; k++) c[k] /= cnt_l;
            }
            for (int i = lig_start_; i <= lig_end_; i++) {
              const double px = x_[3 * i] - c[0], py = x_[3 * i + 1] - c[1], pz = x_[3 * i + 2] - c[2];
              for (int k = 0; k < 3; k++) {
                double v = c[k] + m[k][0] * px + m[k][1] * py + m[k][2] * pz;
                if (std::fabs(v) < 0.0000007) v = 0.0;
                x_[3 * i + k] = v;
              }
            }
          }
          scatter_x();
          separate_close_pairs(false, next_, a.xyz_ext, a.grad_ext, *a.nligs, a.lig_start, a.lig_end);
          gather_x();
          scatter_x();
          co_yield yield_code(kMinimize, 7);
          gather_x();
          if (*a.enrg <= best) {
            best = *a.enrg;
            for (int i = 0; i < nd_; i++) trot[i] = x_[i] - hold[i];
          }
          x_ = hold;
        }
        for (int i = 0; i < nd_; i++) x_[i] = hold[i] + trot[i];
      }
    }
    // final pruning; the archive goes to conflib.dat and conflib[]
    size = arch_.update(next_, nd_, *a.enrg_win, *a.separ_rms);
    if (use_files && !arch_.write("conflib.dat", next_)) co_return kFileError;
    if (print_ || debug_) {
      std::fprintf(out, "__________________________________________________\n");
      std::fprintf(out, debug_ ? " Full list:\n" : " Top Ten:\n");
      int c = 0;
      for (const Entry &x : arch_.e) {
        std::fprintf(out, "   %5d  E =%13.3f /%2d  Rg = %8.3f\n", ++c, x.energy, x.mult, x.rad);
        if (!debug_ && c == 10) break;
        if (debug_ && c == *a.nconf) break;
      }
      std::fprintf(out, "--------------------------------------------------\n");
      std::fprintf(out, " Total Nof confs = %5d\n", size);
      std::fprintf(out, "________________________\n\n");
      std::fflush(out);
    }
    if (zigzag_) {
      // the modes (x 1000) and the last mixed mode, for display
      size_t k = 0;
      for (int j = *a.rotran; j < ncm; j++)
        for (int i = 0; i < nd_; i++) a.conflib[k++] = 1e3 * vecs[static_cast<size_t>(j) * nd_ + i];
      const size_t l0 = k;
      for (int i = 0; i < nd_; i++) a.conflib[k++] = vec[i];
      double s = 0.0;
      for (size_t i = l0; i < l0 + nd_; i++) s += sq(a.conflib[i]);
      s = std::sqrt(s);
      for (size_t i = l0; i < l0 + nd_; i++) a.conflib[i] /= (s * 1e-3);
    } else if (*a.nconf > 0) {
      if (arch_.e.empty()) {
        std::fprintf(stderr, "\nERROR in load_archive(): conflib database is empty.\n");
        std::fflush(stderr);
        co_return kConflibError;
      }
      int c = 0;
      for (const Entry &x : arch_.e) {
        std::memcpy(a.conflib + static_cast<size_t>(c) * next_, x.xyz.data(), next_ * sizeof(double));
        if (++c == *a.nconf) break;
      }
      if (c < *a.nconf) *a.nconf = c;
    }
    glob_min = arch_.e.front().energy;
    std::memcpy(a.xyz_ext, arch_.e.front().xyz.data(), next_ * sizeof(double));
    co_return 0;
  }

 private:
  double draw() { return own_rng ? own_rng->uniform() : rand2(); }
  void gather_x() {
    for (int i = 0; i < natm_; i++)
      for (int k = 0; k < 3; k++) x_[3 * i + k] = a.xyz_ext[3 * idx_[i] + k];
  }
  void gather_g() {
    for (int i = 0; i < natm_; i++)
      for (int k = 0; k < 3; k++) g_[3 * i + k] = a.grad_ext[3 * idx_[i] + k];
  }
  void scatter(const double *x) {
    for (int i = 0; i < natm_; i++)
      for (int k = 0; k < 3; k++) a.xyz_ext[3 * idx_[i] + k] = x[3 * i + k];
  }
  void scatter_x() { scatter(x_.data()); }
  double rms(const std::vector<double> &v) const {
    double s = 0.0;
    for (int i = 0; i < nd_; i++) s += sq(v[i]);
    return std::sqrt(s / nd_);
  }
  // the moving-atom index of an atom (the previous value if it is frozen,
  // as the reference's search leaves its variable unchanged)
  int local_index(int atom, int previous) const {
    for (int i = 0; i < natm_; i++)
      if (idx_[i] == atom) return i;
    return previous;
  }

  bool print_ = false, debug_ = false, debug_modes_ = false, zigzag_ = false;
  std::vector<int> idx_;
  int natm_ = 0, nd_ = 0, next_ = 0;
  int lig_start_ = 0, lig_end_ = 0, lig_cent_ = 0;
  std::vector<double> x_, g_;
  Archive arch_;
};

struct Active {
  std::unique_ptr<Search> search;
  std::unique_ptr<Gen> gen;
};

Active &active() {
  static Active a;
  return a;
}

// Relative precision of the gradients the next lmodC() search gets: FP32's
// for this library's own GPU energy (sets the Hessian-product step).
double g_next_hess_eps = 2.2204460492503131e-16;

}  // namespace

namespace sffg {

struct LmodJob::Impl {
  LMOD_OPT_T lo{};
  int natm = 0, zero_i = 0, return_flag = 0;
  double zero_d = 0.0, lmod_time = 0.0, extn_time = 0.0;
  Rand2 rng;
  Search search;
  std::unique_ptr<Gen> gen;
  int step() {
    if (gen->next()) return gen->request() / 16;
    const int status = gen->status();
    gen.reset();
    return status;
  }
};

LmodJob::LmodJob() : impl_(new Impl) {}
LmodJob::~LmodJob() = default;

int LmodJob::start(const LMOD_OPT_T &lo, int natm, double *xyz, double *grad, double *energy, double *conflib,
                   double *trajectory, int seed, double hess_eps) {
  Impl &m = *impl_;
  m.lo = lo;
  m.lo.print_level = 0;
  m.lo.nlig = 0;
  m.lo.random_seed = seed;
  m.natm = natm;
  LMOD_OPT_T &o = m.lo;
  m.search.a = Args{&o.niter, &o.nmod, &o.kmod, &o.nrotran_dof, &m.natm, xyz, energy, grad, &o.nconf,
                    &o.energy_window, &o.conf_separation_rms, conflib, trajectory, &o.eig_recalc,
                    &o.ndim_arnoldi, &o.lmod_restart, &o.n_best_struct, &o.mc_option, &o.rtemp,
                    &o.lmod_step_size_min, &o.lmod_step_size_max, &o.nof_lmod_steps, &o.nlig, &m.zero_i,
                    &m.zero_i, &o.apply_rigdock, &o.nof_poses_to_try, &m.zero_d, &m.zero_d, &m.zero_i, &m.zero_d,
                    &m.zero_d, &o.random_seed, &o.print_level, &m.lmod_time, &m.extn_time, &m.return_flag};
  if (!check_params(m.search.a)) return kParamsError;
  m.search.own_rng = &m.rng;
  m.search.use_files = false;
  m.search.hess_eps = hess_eps;
  m.gen.reset(new Gen(m.search.run()));
  return m.step();
}

int LmodJob::resume() {
  if (!impl_->gen) return -2;
  return impl_->step();
}

double LmodJob::glob_min() const { return impl_->search.glob_min; }
int LmodJob::nconf() const { return impl_->lo.nconf; }

}  // namespace sffg

extern "C" {

REAL_T lmodC(INT_T *nlmodit, INT_T *nmod, INT_T *kmod, INT_T *rotran, INT_T *natm_ext, REAL_T *xyz_ext, REAL_T *enrg,
             REAL_T *grad_ext, INT_T *nconf, REAL_T *enrg_win, REAL_T *separ_rms, REAL_T *conflib,
             REAL_T *trajectory, INT_T *arpk_recalc, INT_T *arpk_dim, INT_T *lmod_restart, INT_T *topten,
             INT_T *mc_option, REAL_T *rtemp, REAL_T *lmod_step_min, REAL_T *lmod_step_max, INT_T *nof_lmod_step,
             INT_T *nligs, INT_T *lig_start, INT_T *lig_end, INT_T *try_now, INT_T *ntry, REAL_T *trmin,
             REAL_T *trmax, INT_T *lig_rot_cent, REAL_T *angmin, REAL_T *angmax, INT_T *seed, INT_T *print_level,
             REAL_T *lmod_time, REAL_T *extn_time, INT_T *return_flag, INT_T *label) {
  Active &act = active();
  const Args args{nlmodit,    nmod,        kmod,        rotran,        natm_ext,      xyz_ext,       enrg,
                  grad_ext,   nconf,       enrg_win,    separ_rms,     conflib,       trajectory,    arpk_recalc,
                  arpk_dim,   lmod_restart, topten,     mc_option,     rtemp,         lmod_step_min, lmod_step_max,
                  nof_lmod_step, nligs,    lig_start,   lig_end,       try_now,       ntry,          trmin,
                  trmax,      lig_rot_cent, angmin,     angmax,        seed,          print_level,   lmod_time,
                  extn_time,  return_flag};
  if (*label == 0) {
    // the step for this search only, whether or not it starts
    const double hess_eps = g_next_hess_eps;
    g_next_hess_eps = 2.2204460492503131e-16;
    *lmod_time = 0.0;
    *extn_time = 0.0;
    act.gen.reset();
    act.search.reset();
    if (!check_params(args)) {
      *label = kParamsError;
      return 0.0;
    }
    act.search.reset(new Search);
    act.search->a = args;
    act.search->hess_eps = hess_eps;
    act.search->lmod_stamp = clock();
    act.gen.reset(new Gen(act.search->run()));
  } else {
    if (!act.gen) {
      std::fprintf(stderr, "\nERROR in lmod(): Illegal status.\n");
      std::fflush(stderr);
      *label = -2;
      return 0.0;
    }
    act.search->a = args;
    act.search->lmod_stamp = clock();
    *extn_time += static_cast<double>(act.search->lmod_stamp - act.search->extn_stamp);
  }
  Search &s = *act.search;
  if (act.gen->next()) {
    const int code = act.gen->request();
    *return_flag = code / 16;
    *label = code % 16;
    s.extn_stamp = clock();
    *lmod_time += static_cast<double>(s.extn_stamp - s.lmod_stamp);
    return 0.0;
  }
  const int status = act.gen->status();
  const double result = s.glob_min;
  *lmod_time += static_cast<double>(clock() - s.lmod_stamp);
  *lmod_time /= CLOCKS_PER_SEC;
  *extn_time /= CLOCKS_PER_SEC;
  act.gen.reset();
  act.search.reset();
  *return_flag = kDone;
  *label = status;
  return status == 0 ? result : 0.0;
}

INT_T lmod_opt_init(LMOD_OPT_T *lo, XMIN_OPT_T *xo) {
  lo->minim_grms = 0.1;
  lo->niter = 10;
  lo->nmod = 5;
  lo->kmod = 3;
  lo->nrotran_dof = 6;
  lo->nconf = 10;
  lo->energy_window = 50.0;
  lo->conf_separation_rms = 2.0;
  lo->eig_recalc = 5;
  lo->ndim_arnoldi = 0;
  lo->lmod_restart = 10;
  lo->n_best_struct = 10;
  lo->mc_option = 1;
  lo->rtemp = 1.5;
  lo->lmod_step_size_min = 2.0;
  lo->lmod_step_size_max = 5.0;
  lo->nof_lmod_steps = 0;
  lo->lmod_relax_grms = 1.0;
  lo->nlig = 0;
  lo->apply_rigdock = 2;
  lo->nof_poses_to_try = 10;
  lo->random_seed = 314159;
  lo->print_level = 0;
  xo->mol_struct_opt = 1;
  xo->maxiter = 20000;
  xo->grms_tol = 1e-8;
  xo->method = 2;
  xo->numdiff = 1;
  xo->m_lbfgs = 3;
  xo->ls_method = 2;
  xo->ls_maxiter = 20;
  xo->ls_maxatmov = 0.5;
  xo->beta_armijo = 0.5;
  xo->c_armijo = 0.4;
  xo->mu_armijo = 1.0;
  xo->ftol_wolfe = 0.0001;
  xo->gtol_wolfe = 0.9;
  xo->print_level = 0;
  return 0;
}

REAL_T sffg_lmod_func(REAL_T (*func)(REAL_T *, REAL_T *, INT_T *), INT_T *natm, REAL_T *xyz, REAL_T *grad,
                      REAL_T *energy, REAL_T *conflib, REAL_T *lmod_trajectory, INT_T *lig_start, INT_T *lig_end,
                      INT_T *lig_cent, REAL_T *tr_min, REAL_T *tr_max, REAL_T *rot_min, REAL_T *rot_max,
                      XMIN_OPT_T *xo, LMOD_OPT_T *lo) {
  // the reference's lmod() driver loop (lmodC.c:3366-3462) over func
  INT_T return_flag = 0, status_flag = 0, neg_two = -2, neg_four = -4;
  REAL_T glob_min = 0.0, xmin_grms = 0.0;
  if (func == &mme || func == &mme_rattle) g_next_hess_eps = FLT_EPSILON;
  for (lo->error_flag = 0;;) {
    glob_min = lmodC(&lo->niter, &lo->nmod, &lo->kmod, &lo->nrotran_dof, natm, xyz, energy, grad, &lo->nconf,
                     &lo->energy_window, &lo->conf_separation_rms, conflib, lmod_trajectory, &lo->eig_recalc,
                     &lo->ndim_arnoldi, &lo->lmod_restart, &lo->n_best_struct, &lo->mc_option, &lo->rtemp,
                     &lo->lmod_step_size_min, &lo->lmod_step_size_max, &lo->nof_lmod_steps, &lo->nlig, lig_start,
                     lig_end, &lo->apply_rigdock, &lo->nof_poses_to_try, tr_min, tr_max, lig_cent, rot_min, rot_max,
                     &lo->random_seed, &lo->print_level, &lo->lmod_time, &lo->aux_time, &return_flag, &status_flag);
    if (return_flag == 0) {
      lo->error_flag = status_flag >= 0 ? 0 : status_flag;
    } else if (status_flag < 0) {
      lo->error_flag = status_flag;
    } else if (return_flag == 1 || return_flag == 2) {
      *energy = func(xyz, grad, &neg_four);
    } else if (return_flag == 3 || return_flag == 4) {
      *energy = func(xyz, grad, &neg_two);
    } else if (return_flag == 5) {
      xo->grms_tol = lo->minim_grms;
      *energy = xmin(func, natm, xyz, grad, energy, &xmin_grms, xo);
    } else if (return_flag == 6) {
      xo->grms_tol = lo->lmod_relax_grms;
      *energy = xmin(func, natm, xyz, grad, energy, &xmin_grms, xo);
    } else if (return_flag == 7) {
      *energy = xmin(func, natm, xyz, grad, energy, &xmin_grms, xo);
    } else {
      std::fprintf(stderr, "\n LMOD ERROR: return_flag corrupted.\n");
      lo->error_flag = -100;
      return 0.0;
    }
    if (lo->error_flag || !return_flag) break;
  }
  if (lo->error_flag) {
    std::fprintf(stderr, "\n LMOD ERROR: %d\n", status_flag);
    return 0.0;
  }
  return glob_min;
}

REAL_T lmod(INT_T *natm, REAL_T *xyz, REAL_T *grad, REAL_T *energy, REAL_T *conflib, REAL_T *lmod_trajectory,
            INT_T *lig_start, INT_T *lig_end, INT_T *lig_cent, REAL_T *tr_min, REAL_T *tr_max, REAL_T *rot_min,
            REAL_T *rot_max, XMIN_OPT_T *xo, LMOD_OPT_T *lo) {
  return sffg_lmod_func(&mme, natm, xyz, grad, energy, conflib, lmod_trajectory, lig_start, lig_end, lig_cent, tr_min,
                        tr_max, rot_min, rot_max, xo, lo);
}

}  // extern "C"
