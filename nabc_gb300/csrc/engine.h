// The device engine: a batch of independent systems resident on one GPU.
//
// Layout in device memory (all systems flattened, never mixed in a tile):
//   slot  = position in the spatially sorted atom order; 32 consecutive
//           slots form a tile, tiles never straddle two systems, padding
//           slots are marked invalid in the tile's lane mask;
//   atom  = index in the caller's atom order (systems concatenated).
// Per-slot FP32 arrays feed the pair kernels; FP64 arrays hold coordinates,
// velocities, gradients and the per-atom Born-radius finish; forces, Born
// sums, sumdeijda and energies accumulate in 64-bit fixed point, so results
// do not depend on the order in which tile pairs are processed.
#pragma once

#include <cuda_runtime_api.h>

#include <functional>
#include <memory>
#include <string>
#include <vector>

#include "sffg_internal.h"

namespace sffg {

struct DeviceState;  // defined in engine.cu

// Page-locked host doubles for the per-turn coordinate uploads and gradient
// reads of the batched minimisers (pageable copies go through a staging
// buffer); falls back to pageable memory if pinning fails.
class HostDoubles {
 public:
  explicit HostDoubles(size_t n) : n_(n) {
    if (cudaMallocHost(reinterpret_cast<void **>(&p_), n * sizeof(double) + 8) != cudaSuccess) {
      (void)cudaGetLastError();
      p_ = nullptr;
      fallback_.assign(n, 0.0);
    } else {
      for (size_t i = 0; i < n; i++) p_[i] = 0.0;
    }
  }
  ~HostDoubles() {
    if (p_) cudaFreeHost(p_);
  }
  HostDoubles(const HostDoubles &) = delete;
  HostDoubles &operator=(const HostDoubles &) = delete;
  double *data() { return p_ ? p_ : fallback_.data(); }
  size_t size() const { return n_; }

 private:
  double *p_ = nullptr;
  size_t n_;
  std::vector<double> fallback_;
};
struct ListArgs;     // defined in lists.cuh

// State of one system's conjugate-gradient run (the locals of the
// reference's conjgrad(), src/sff/conjgrad.c:40-55).
struct CgState {
  int done, ret, niter, nfbeg, iterc, nfopt, iterfm, iterrs, iretry, ier, maxiter;
  double f, fmin, gmin, dfpr, gnew, step, finit, ginit, gsqrd, stmin, gamden, ddspln, stepch, sbound,
      fch, sum, beta, gama, dgrad, dfpred;
};

struct SystemInfo {
  int natom = 0, atom_off = 0, slot_off = 0, tile_off = 0, ntile = 0;
  double fsmax = 0.0;
  bool has_frozen = false;
  std::vector<int> frozen;
  std::vector<double> mass;
  int ntypes = 0;
  int lj_off = 0;
  unsigned long long noise_key = 0;  // Philox key of the md noise (default: the system index)
  std::vector<int> constrained;      // positional restraints (econs): flags ...
  std::vector<double> x0;            // ... and reference positions, 3 per atom
};

class Batch {
 public:
  explicit Batch(const Options &opts);
  ~Batch();
  Batch(const Batch &) = delete;
  Batch &operator=(const Batch &) = delete;

  // Returns the system index, or a negative status.
  int add_system(PARMSTRUCT_T *prm, const int *frozen, const double *x, bool mutate_prm);
  // The same for a topology already converted (build_host_system).
  int add_host_system(HostSystem hs, const double *x);
  // Harmonic positional restraints of a system (before finalize): atoms with
  // constrained[i] != 0 are held to x0 with the option wcons.
  int set_restraints(int sys, const int *constrained, const double *x0);
  // Key of a system's md noise (before finalize); systems with equal keys,
  // topologies and coordinates draw equal noise in any batch.
  int set_noise_key(int sys, unsigned long long key);
  // Switches one system's work on or off (stream-ordered).
  int set_active(int sys, bool on, void *stream);
  int finalize();
  bool finalized() const { return finalized_; }
  int num_systems() const { return static_cast<int>(sys_.size()); }
  // RATTLE constraints of system sys under the option rattle (0: none; 1: all
  // bonds; 2: bonds to hydrogen)
  int rattle_bonds(int sys) const {
    return opts_.irattle == 0 ? 0
           : opts_.irattle == 2 ? host_[sys].rattle_nh
                                : static_cast<int>(host_[sys].rattle_bonds.size());
  }
  const SystemInfo &system(int s) const { return sys_[s]; }
  const ModelParams &model() const { return mp_; }
  const Options &opts() const { return opts_; }
  int total_atoms() const { return natom_total_; }

  // Host <-> device transfers of one system (stream-ordered, async unless
  // stated).
  int set_coords(int sys, const double *x, void *stream);
  int get_coords(int sys, double *x, void *stream);      // synchronous
  int get_grad(int sys, double *g, void *stream);        // synchronous
  int get_reff(int sys, double *reff, void *stream);     // synchronous
  int set_velocities(int sys, const double *v, void *stream);
  int get_velocities(int sys, double *v, void *stream);  // synchronous
  // Energy components of the last evaluation in the reference's ene[]
  // layout (13 entries); synchronous.
  int get_energy(int sys, double *ene, void *stream);
  // Energy components and gradient of one system with a single wait.
  int get_energy_grad(int sys, double *ene, double *g, void *stream);
  int get_all_energies(std::vector<double> &ene13, void *stream);
  // Whole-batch transfers with one wait: coordinates of every system (atom
  // order, systems in order), the active flags, and every system's energy
  // components (13 each) with the whole gradient.
  int set_all_coords(const double *x, void *stream);
  // Per system: SFFG_OK; SFFG_ENONFINITE once an evaluation met a
  // non-finite coordinate (cleared when its coordinates are set again);
  // SFFG_ECONSTRAINT once RATTLE's sweeps reached their limit in md.
  int system_status(std::vector<int> &status, void *stream);
  // The md state of every system (coordinates, velocities, accelerations,
  // Berendsen factors) to or from a file.  load_state evaluates at the
  // loaded coordinates with fresh pair lists, so md continued from a state
  // saved right after a list-rebuild step (step % nsnb == 0, without a
  // centre-of-mass removal there) in a batch built from the same
  // topologies and initial coordinates repeats the original run bit for bit.
  int save_state(const char *path, void *stream);
  int load_state(const char *path, void *stream);
  int set_all_active(const std::vector<int> &on, void *stream);
  // status (optional): each system's non-finite flag, read with the same wait
  int get_all_energy_grad(std::vector<double> &ene13, double *grad, void *stream,
                          std::vector<int> *status = nullptr);
  // XMIN on every system at once (csrc/batch_xmin.cpp): status, iteration
  // count and final energy per system.
  int xmin(const XMIN_OPT_T &xo, std::vector<int> &status, std::vector<int> &iters, std::vector<double> &energy,
           void *stream);
  // LMOD searches on every system (csrc/batch_lmod.cpp); conflib: per
  // system lo.nconf structures at lo.nconf * 3 * atom offset (may be null)
  int lmod(const LMOD_OPT_T &lo, const XMIN_OPT_T &xo, std::vector<int> &status, std::vector<double> &glob_min,
           std::vector<int> &nconf, double *conflib, void *stream);

  // One energy+gradient evaluation of every active system.  rebuild
  // requests a pair-list rebuild first (always done on the first call).
  int eval(bool rebuild, void *stream);
  // The same, with a list rebuild that launches without reading counts back
  // (see build_lists); returns once the list build has run on the device,
  // and when a list store was too small it grows the stores and evaluates
  // again, so the results are always complete.
  int eval_checked(bool rebuild, void *stream);
  // Resolves a queued list build still unchecked (waiting for it if need
  // be); after one whose stores were too small, md steps taken since are
  // replayed from their snapshot.  Every method that reads or changes the
  // batch's device state calls it first.
  int settle(void *stream);
  long long num_pairs(int sys);

  // Device-resident Langevin/Berendsen md (the reference's integrator,
  // src/sff/sff.c:2191-2354) over all systems.  md_begin evaluates the first
  // force and sets the initial accelerations; md_steps then advances k
  // steps numbered step0+1 .. step0+k.  noise: nullptr -> device Philox;
  // otherwise a host callback that fills the unit Gaussian draws of every
  // non-frozen coordinate in the reference's order.
  using NoiseFn = void (*)(void *ctx, int sys, int n, double *out);
  int md_begin(bool rebuild, NoiseFn noise, void *noise_ctx, void *stream);
  // com_at_end=false leaves out the centre-of-mass removal a last step that
  // is a multiple of nscm would end with; md_com_remove applies it later
  // (md() writes its trajectory frame between the two, as the reference).
  int md_steps(int step0, int k, NoiseFn noise, void *noise_ctx, void *stream, bool com_at_end = true);
  int md_com_remove(void *stream);
  // Kinetic energy after the last md step (reference convention,
  // sff.c:2294-2306) and Berendsen factor for the next step.
  int md_kinetic(std::vector<double> &ekin, void *stream);
  int md_set_tscal(const std::vector<double> &tscal, void *stream);

  // Batched conjgrad: every system runs the reference's state machine
  // (src/sff/conjgrad.c:34-263).  first_rebuild forces a pair-list build
  // before the first evaluation; after_eval (optional) runs on the host
  // after every evaluation with the evaluation index (the reference's
  // iteration count).
  int cg(int maxiter, double rmsgrad, double dfpred, bool first_rebuild, std::vector<int> &status,
         std::vector<double> &energy, void *stream, const std::function<int(int)> &after_eval);
  // The same in pieces, for drivers that interleave several batches:
  // cg_turns launches up to n turns without waiting (the first with a list
  // rebuild when first_rebuild); cg_poll waits for the stream and reports
  // the systems still running (0 once every system ended or maxiter turns
  // ran) and, optionally, each system's return code (0: running) and
  // energy; cg_end restores every system's active flag.
  int cg_begin(int maxiter, double rmsgrad, double dfpred, void *stream);
  int cg_begin(const std::vector<int> &maxiter, const std::vector<double> &rmsgrad, double dfpred, void *stream);
  int cg_turns(int n, bool first_rebuild, void *stream, const std::function<int(int)> &after_eval = nullptr);
  int cg_poll(int *nactive, std::vector<int> *status, std::vector<double> *energy, void *stream);
  int cg_end(void *stream);
  // Turns cg_turns has run since cg_begin.
  int cg_turn() const { return cg_turn_; }
  // Moving a running minimisation into another batch: cg_export reads one
  // system's state machine, coordinates, gradient and work vectors
  // (synchronous); cg_import writes them into system sys of a batch after
  // its cg_begin and before its first turn.  The system continues
  // bit for bit when the move happens where its own evaluation count is a
  // multiple of nsnb (a list rebuild either way) and the receiving batch
  // was built from the same topology and initial coordinates (which fix
  // the atom order; host_system and initial_coords give them).
  struct CgCarry {
    CgState st;
    std::vector<double> x, g, w;
  };
  int cg_export(int sys, CgCarry &c, void *stream);
  int cg_import(int sys, const CgCarry &c, void *stream);
  const HostSystem &host_system(int sys) const { return host_[sys]; }
  const std::vector<double> &initial_coords(int sys) const { return x0_[sys]; }
  // Takes another batch's tuned work split instead of tuning this one.
  void adopt_split(const Batch &from);
  // True once a pair list has been built.
  bool have_list() const { return have_list_; }

  size_t device_bytes() const;
  std::string last_error;

  // The work split the autotuner chose for pass 0, 1 or 2 (pair passes 1-3):
  // work items claimed per grab and persistent blocks.
  int tuned_split(int pass, int *claim, int *blocks) const;

  // Launch counting and per-pass CUDA-event timing.
  long long launches() const { return launches_; }
  int set_profiling(bool on);
  int kernel_times(double ms[3], long long *nevals);

  // Raw device views used by the legacy session.
  double *d_coords();
  double *d_grad();
  void *default_stream();

 private:
  int upload();
  int run_eval_direct(bool rebuild, void *stream);
  int ensure_tuned(cudaStream_t st);
  std::vector<const void *> list_sig() const;
  bool graphs_ok() const;
  int capture(cudaGraphExec_t &exec, std::vector<const void *> &sig, long long &nlaunch,
              const std::function<int(cudaStream_t)> &body);
  int build_lists(void *stream);
  int build_lists_queued(cudaStream_t st);
  int prepare_queued_builds();
  int resolve_list_check(bool *overflowed);
  int settle_md(cudaStream_t st);
  int md_com_remove_direct(cudaStream_t st);
  void rebuild_list_b(void *stream);
  ListArgs list_args();
  int run_eval(bool rebuild, void *stream);
  void collect_pass_times(DeviceState &d, long long max_evals);
  Options opts_;
  ModelParams mp_;
  std::vector<SystemInfo> sys_;
  std::vector<HostSystem> host_;
  std::vector<std::vector<double>> x0_;
  int natom_total_ = 0, nslot_ = 0, ntile_ = 0;
  unsigned step_host_ = 0;  // staging of the md step counter upload
  // work split of the three pair passes (autotuned, see ensure_tuned)
  struct PassCfg {
    int claim = 4, blocks = 1;
  };
  PassCfg cfg_[3];
  int occ_[3] = {1, 1, 1};
  // every system takes the polynomial rgbmax tail: passes 1 and 3 launch the
  // instantiation without the logarithmic form
  bool tail_poly_all_ = true;
  bool tuned_ = false, tuning_ = false;
  // conjgrad driver state (host copies of the device state machines)
  std::vector<CgState> cg_host_;
  std::vector<int> ones_;  // the active flags last sent to the device
  long long list_builds_ = 0, cg_list_builds_ = 0;
  void note_active(const std::vector<int> &on);
  int cg_nsys_ = 0, cg_turn_ = 0, cg_maxiter_ = 0;
  long long cand_max_ = 0;  // candidate tile pairs the batch could ever need
  int ncand_ = 0;           // candidates of the current pair list
  // Queued list builds: allowed while queued_builds_ is set and a
  // synchronous build has sized the stores (sized_); the last known
  // candidate and chunk counts size the next queued build's stores with
  // headroom.  list_check_pending_: a queued build's overflow flag is still
  // unread.  force_sync_build_: the next build reads its counts back.
  bool queued_builds_ = false, sized_ = false, list_check_pending_ = false, force_sync_build_ = false;
  long long last_ncand_ = 0, last_nch_ = 0;
  // md replay: the state (coordinates, velocities, accelerations, kinetic
  // sums, Berendsen factors) before the md step whose list build was
  // queued, that step's predecessor number and the steps taken since
  bool md_ckpt_valid_ = false;
  int md_ckpt_step_ = 0, md_ckpt_steps_ = 0;
  bool finalized_ = false, have_list_ = false, profile_ = false;
  long long launches_ = 0;
  std::unique_ptr<DeviceState> d_;
};

}  // namespace sffg
