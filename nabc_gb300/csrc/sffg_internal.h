// Internal declarations shared by the host (C++) and device (CUDA) parts of
// libsffg.  Nothing here is part of the public ABI (include/sff.h,
// include/sffg.h).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "../../include/sff.h"
#include "../../include/sffg.h"

namespace sffg {

// ---------------------------------------------------------------- options
// Every key of the reference's option grammar (src/sff/mm_options.l:28-97)
// with the reference's defaults (src/sff/sff.c:68-199), plus this library's
// own "sffg_" keys.
struct Options {
  double cut = 20.0, cutnp = 10.0, scnb = 2.0, scee = 1.2, rgbmax = 15.0;
  double hcp_h1 = 15.0, hcp_h2 = 50.0, hcp_h3 = 150.0, dhcp = 0.25;
  int ntpr = 10, nscm = 0, nsnb = 10, nsnp = 10, ntwx = 0, nchk = 10000, nchk2 = 10000;
  double dt = 0.001, t = 0.0, tautp = 999999.0, temp0 = 300.0, tempi = 0.0;
  double vlimit = 10.0, gamma_ln = 0.0, genmass = 10.0, wcons = 0.0, k4d = 0.0;
  int ntpr_md = 10, zerov = 0, ips = 0, gb = 0, gb_debug = 0, nr_debug = 0, gb2_debug = 0;
  int gbsa_debug = 0, e_debug = 0, hcp = 0;
  double epsext = 78.5, kappa = 0.0, surften = 0.005, dradius = 0.5, deltar = 0.5;
  double rwater = 1.4, alphanp = 0.75, kappanp = 2.227, min_volume = 0.01;
  int max_set_size = 20, mpi_min_tasks = 8, cull_np_lists = 1, use_lower_tri = 0;
  int dynamic_loops = 1, blocksize = 8, gbsa = 0, dim = 3, dield = 1, irattle = 0;
  double dielc = 1.0;
  // Library keys: noise source for md() ("reference" replays the reference's
  // serial gauss2 stream on the host; "philox" draws on the device), tile
  // kernel tuning and CUDA-graph use.
  int sffg_noise = 0;           // 0 = reference stream, 1 = device Philox
  unsigned long long sffg_seed = 0x5eedULL;
  int sffg_graph = 1;           // capture the md/cg step in a CUDA graph
  int sffg_tune = 1;            // autotune the pair passes' work split
  int sffg_lj_shared = 1;       // pass 2 reads small Lennard-Jones tables from shared memory
  int sffg_serve_classes = 0;   // serving: one minimisation group per size class (1) or one for all (0)
  int sffg_verbose = 0;
};

Options &options();
FILE *legacy_out();  // the caller's nabout, or stdout
// Parses an option string into o (echoing accepted items when echo is set).
// With fail_stop the process exits on a bad item, as the reference does;
// otherwise -1 is returned and the item copied to *bad.
int parse_options(const char *opts, Options &o, bool echo, bool fail_stop, std::string *bad);

// An Amber NetCDF trajectory (csrc/netcdf.cpp): created by mme_init_sff when
// it gets a file name, appended to by md() every ntwx steps.
class NcTrajectory {
 public:
  ~NcTrajectory() { close(); }
  bool create(const char *path, int natom);
  bool write_frame(const double *x, double time_ps);
  void close();
  bool open() const { return fp_ != nullptr; }
  int frames() const { return frames_; }

 private:
  FILE *fp_ = nullptr;
  int natom_ = 0, frames_ = 0;
  unsigned long long data_begin_ = 0, record_bytes_ = 0;
};

// One XMIN minimisation driven by reverse communication (csrc/xmin.cpp):
// start() takes the options, the coordinates and the gradient at them;
// while start() or resume() return 1, evaluate energy and gradient at xyz
// (request: the reference's return_flag, 4-6 rebuild the pair list, 7-9
// keep it) and resume().  0: done, xyz holds the result; < 0: the
// reference's error status.
class XminJob {
 public:
  XminJob();
  ~XminJob();
  // grad_eps: the gradients' relative precision, which sizes TNCG's
  // finite-difference step (the reference assumes FP64)
  int start(const XMIN_OPT_T &xo, int natm, double *xyz, const double *grad, double energy, int *request,
            double grad_eps = 2.2204460492503131e-16);
  int resume(double energy, const double *grad, double *xyz, int *request);
  int iter() const { return iter_; }
  int ls_iter() const { return ls_iter_; }
  double grms() const { return grms_; }
  double time() const { return time_; }

 private:
  struct Impl;
  std::unique_ptr<Impl> impl_;
  int iter_ = 0, ls_iter_ = 0;
  double grms_ = 0.0, time_ = 0.0;
};

// ------------------------------------------------ the reference's RNG
// L'Ecuyer combined generator with Bays-Durham shuffle and polar
// Box-Muller Gaussians, as published in src/sff/rand2.c:51-128, with the
// same default seed (-1).  md(), rand2() and lmod() share one process-
// global stream as in the reference; batched LMOD searches own one each.
struct Rand2 {
  int seed3 = -1, seed2 = 0, iy = 0, iv[32] = {0};
  double uniform() {
    const int IM1 = 2147483563, IM2 = 2147483399, IA1 = 40014, IA2 = 40692, IQ1 = 53668, IQ2 = 52774,
              IR1 = 12211, IR2 = 3791, NTAB = 32, IMM1 = IM1 - 1, NDIV = 1 + IMM1 / NTAB;
    const double AM = 1.0 / IM1, RNMX = 1.0 - 1.2e-13;
    int k;
    if (seed3 <= 0) {
      seed3 = (-seed3 < 1) ? 1 : -seed3;
      seed2 = seed3;
      for (int j = NTAB + 7; j >= 0; j--) {
        k = seed3 / IQ1;
        seed3 = IA1 * (seed3 - k * IQ1) - k * IR1;
        if (seed3 < 0) seed3 += IM1;
        if (j < NTAB) iv[j] = seed3;
      }
      iy = iv[0];
    }
    k = seed3 / IQ1;
    seed3 = IA1 * (seed3 - k * IQ1) - k * IR1;
    if (seed3 < 0) seed3 += IM1;
    k = seed2 / IQ2;
    seed2 = IA2 * (seed2 - k * IQ2) - k * IR2;
    if (seed2 < 0) seed2 += IM2;
    const int j = iy / NDIV;
    iy = iv[j] - seed2;
    iv[j] = seed3;
    if (iy < 1) iy += IMM1;
    const double t = AM * iy;
    return t > RNMX ? RNMX : t;
  }
  double gauss(double mean, double sd) {
    double s1, s2, rsq;
    do {
      s1 = 2. * uniform() - 1.;
      s2 = 2. * uniform() - 1.;
      rsq = s1 * s1 + s2 * s2;
    } while (rsq >= 1. || rsq == 0.0);
    return sd * (s1 * std::sqrt(-2. * std::log(rsq) / rsq)) + mean;
  }
};

// One LMOD search driven by its caller (the batched searches of
// sffg_batch_lmod): lmodC()'s search with its own random stream, no printout
// and no conflib.dat.  start() and resume() return the next request -- 1-7,
// lmodC()'s return_flag codes, acted on at xyz/grad/energy, which the
// caller updates in place before resuming -- or, when the search ends, 0 or
// a negative status.  conflib holds nconf * 3 natm, trajectory
// (niter + 1) * 3 natm doubles.
class LmodJob {
 public:
  LmodJob();
  ~LmodJob();
  int start(const LMOD_OPT_T &lo, int natm, double *xyz, double *grad, double *energy, double *conflib,
            double *trajectory, int seed, double hess_eps);
  int resume();
  double glob_min() const;
  int nconf() const;

 private:
  struct Impl;
  std::unique_ptr<Impl> impl_;
};

// ---------------------------------------------------------------- model
enum GbModel { GB_NONE = 0, GB_HCT = 1, GB_OBC1 = 2, GB_OBC2 = 5, GB_NECK = 7, GB_NECK2 = 8 };

struct ModelParams {
  int gb = 0;
  double gboffset = 0.09, gbneckscale = 0.0;
  double rgbmax = 15.0, cut = 20.0, kappa = 0.0, epsext = 78.5;
};

// One dihedral term (multi-term dihedrals are expanded into several).
struct DihTerm {
  int a, b, c, d;      // atom indices
  double pk, pn, phase;
  int chain_next;      // unused after expansion
};

// Host-side description of one system, derived from a PARMSTRUCT_T and the
// options exactly as the reference's mme_init_sff (src/sff/sff.c:858-1846).
struct HostSystem {
  int natom = 0;
  double fsmax = 0.0;
  std::vector<double> q, rborn, fs, alpha, beta, gamma, mass;
  std::vector<int> neck, type, frozen;
  int ntypes = 0;
  std::vector<float> lj_a, lj_b;          // ntypes^2, zero where no 6-12 term
  std::vector<double> lj_a64, lj_b64;     // the same in FP64 (close pairs)
  std::vector<std::pair<int, int>> excl;  // excluded pairs i<j (Coulomb/LJ only)
  struct Bond { int a, b; double rk, req; };
  struct Angle { int a, b, c; double tk, teq; };
  struct Pair14 { int a, b; double scee, scnb, c12, c6; int pow10; };
  std::vector<Bond> bonds;
  // RATTLE's bond list (src/sff/rattle.c:41-53): the bonds to hydrogen, then
  // the others, in the topology's order, none left out; rattle_nh of them
  // are bonds to hydrogen
  std::vector<Bond> rattle_bonds;
  int rattle_nh = 0;
  std::vector<Angle> angles;
  std::vector<DihTerm> dihedrals;
  std::vector<Pair14> pairs14;
};

ModelParams model_from_options(const Options &o);
// Builds a HostSystem; prm is read (and, like the reference, modified: the
// charges are scaled by 1/sqrt(dielc) and Fs overwritten for gb=7/8) only
// when mutate_prm is true.
void build_host_system(PARMSTRUCT_T *prm, const int *frozen, const Options &o, bool mutate_prm,
                       HostSystem &out, ModelParams &mp);

void prm_allocate_arrays(PARMSTRUCT_T *prm);
void prm_finish_derived(PARMSTRUCT_T *prm, bool newparm);

// ---------------------------------------------------------------- fixed point
// Scales of the 64-bit fixed-point accumulators.
constexpr double kForceScale = 4294967296.0;      // 2^32 per kcal/mol/A
constexpr double kEnergyScale = 4294967296.0;     // 2^32 per kcal/mol
constexpr double kBornScale = 1099511627776.0;    // 2^40 per 1/A
constexpr double kSumdScale = 4294967296.0;       // 2^32

// Per-system energy slots kept in fixed point on the device.
enum EnergySlot { E_EGB = 0, E_EEL, E_EVDW, E_BOND, E_ANGLE, E_DIHED, E_EEL14, E_ENB14, E_CONS, E_NSLOTS };

// ---------------------------------------------------------------- timing
struct Timers {
  double init = 0, md = 0, cg = 0, mme = 0, pair = 0, born = 0, bonded = 0, other = 0;
  long nevals = 0;
};
Timers &timers();
double wall_seconds();

}  // namespace sffg
