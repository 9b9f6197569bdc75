// LMOD on every system of a batch at once (include/sffg.h,
// sffg_batch_lmod).  No counterpart in the reference, whose lmod()
// (src/sff/lmodC.c:3108) searches one molecule through one energy function.
//
// Each system runs its own search (LmodJob, the coroutine of csrc/lmod.cpp)
// with its own random stream, seeded random_seed + s, and, whenever the
// search asks for a minimisation, its own XMIN run (XminJob) with the
// tolerance the reference's lmod() driver would give it (lmodC.c:3420-3447).
// Every system always waits for exactly one evaluation -- for its search or
// for its minimiser -- so each turn uploads all the waiting systems'
// coordinates, evaluates them together, reads every energy and gradient back
// with one wait and resumes the searches and minimisers on the host's cores.
// Systems end independently; one whose energy turns non-finite ends alone.
//
// The pair lists are rebuilt for the whole batch whenever any system asks
// for it, which regroups every system's chunks and so changes the FP32
// rounding of the others: a system in a mixed batch follows its lone search
// to rounding only (and a random search amplifies that), while a
// one-system batch takes lmod()'s path bit for bit.  Runs are deterministic.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <thread>
#include <vector>

#include "engine.h"

namespace sffg {

namespace {
constexpr int kLmodNonFinite = -8;  // the reference's statuses run to -7
}

int Batch::lmod(const LMOD_OPT_T &lo, const XMIN_OPT_T &xo_in, std::vector<int> &status,
                std::vector<double> &glob_min, std::vector<int> &nconf, double *conflib, void *stream) {
  if (!finalized_) return SFFG_ESTATE;
  if (lo.nconf <= 0 || lo.niter < 0) {
    last_error = "lmod: nconf must be positive and niter non-negative";
    return SFFG_EINVAL;
  }
  const int nsys = num_systems();
  const size_t n3 = 3 * static_cast<size_t>(natom_total_);
  HostDoubles x(n3), g(n3);
  std::vector<double> ene, energy(nsys, 0.0);
  for (int s = 0; s < nsys; s++) {
    int rc = get_coords(s, x.data() + 3 * static_cast<size_t>(sys_[s].atom_off), stream);
    if (rc) return rc;
  }
  std::vector<int> on(nsys, 1);
  int rc = set_all_active(on, stream);
  if (rc) return rc;
  if ((rc = eval(true, stream))) return rc;
  if ((rc = get_all_energy_grad(ene, g.data(), stream))) return rc;
  std::vector<int> health;
  if ((rc = system_status(health, stream))) return rc;

  struct Sys {
    LmodJob search;
    XminJob minimiser;
    XMIN_OPT_T xo;
    std::vector<double> conflib, traj;
    int waiting = 0;  // 0 done, 1 for the search, 2 for the minimiser
    int request = 0;  // the search's request, or the minimiser's
  };
  std::vector<Sys> sys(nsys);
  status.assign(nsys, 0);
  glob_min.assign(nsys, 0.0);
  nconf.assign(nsys, 0);
  XMIN_OPT_T xo0 = xo_in;
  xo0.print_level = 0;

  auto off = [&](int s) { return 3 * static_cast<size_t>(sys_[s].atom_off); };
  // Runs system s's search from request r until it waits for an
  // evaluation or ends.
  auto advance = [&](int s, int r) {
    Sys &y = sys[s];
    double *xs = x.data() + off(s), *gs = g.data() + off(s);
    for (;;) {
      if (r <= 0) {
        y.waiting = 0;
        status[s] = r;
        if (r == 0) {  // the search left its lowest structure in xs
          glob_min[s] = y.search.glob_min();
          nconf[s] = y.search.nconf();
        }
        return;
      }
      if (r <= 4) {  // energy and gradient (1, 2: with new pair lists)
        y.waiting = 1;
        y.request = r;
        return;
      }
      // minimise (5), relax (6) or minimise the start structure (7), as
      // the reference's lmod() driver sets the tolerance
      y.xo = xo0;
      if (r == 5) y.xo.grms_tol = lo.minim_grms;
      if (r == 6) y.xo.grms_tol = lo.lmod_relax_grms;
      int req = 0;
      const int m = y.minimiser.start(y.xo, sys_[s].natom, xs, gs, energy[s], &req, FLT_EPSILON);
      if (m == 1) {
        y.waiting = 2;
        y.request = req;
        return;
      }
      if (m < 0) energy[s] = 0.0;  // xmin() returns 0 on an error, and lmod() goes on
      r = y.search.resume();
    }
  };
  for (int s = 0; s < nsys; s++) {
    Sys &y = sys[s];
    const size_t na = static_cast<size_t>(sys_[s].natom);
    y.conflib.assign(3 * na * lo.nconf, 0.0);
    y.traj.assign(3 * na * (static_cast<size_t>(lo.niter) + 1), 0.0);
    energy[s] = ene[13 * s];
    if (health[s] != SFFG_OK || !std::isfinite(energy[s])) {
      status[s] = kLmodNonFinite;
      continue;
    }
    advance(s, y.search.start(lo, sys_[s].natom, x.data() + off(s), g.data() + off(s), &energy[s],
                              y.conflib.data(), y.traj.data(), lo.random_seed + s, FLT_EPSILON));
  }
  for (;;) {
    bool any = false, rebuild = false;
    for (int s = 0; s < nsys; s++) {
      const Sys &y = sys[s];
      on[s] = y.waiting != 0;
      any = any || on[s];
      if (y.waiting == 1 && y.request <= 2) rebuild = true;
      if (y.waiting == 2 && y.request >= 4 && y.request <= 6) rebuild = true;
    }
    if (!any) break;
    if ((rc = set_all_active(on, stream))) return rc;
    if ((rc = set_all_coords(x.data(), stream))) return rc;
    if ((rc = eval(rebuild, stream))) return rc;
    if ((rc = get_all_energy_grad(ene, g.data(), stream, &health))) return rc;
    auto resume_range = [&](int s0, int s1) {
      for (int s = s0; s < s1; s++) {
        Sys &y = sys[s];
        if (!y.waiting) continue;
        energy[s] = ene[13 * s];
        if (health[s] != SFFG_OK || !std::isfinite(energy[s])) {
          y.waiting = 0;
          status[s] = kLmodNonFinite;
          continue;
        }
        if (y.waiting == 2) {
          int req = 0;
          const int m = y.minimiser.resume(energy[s], g.data() + off(s), x.data() + off(s), &req);
          if (m == 1) {
            y.request = req;
            continue;
          }
          if (m < 0) energy[s] = 0.0;
        }
        advance(s, y.search.resume());
      }
    };
    // host threads pay for themselves only on large systems: a thread is
    // started per turn, about the cost of resuming 10,000 atoms' minimiser
    const int nthr = std::min<int>(std::min<int>(std::max(1u, std::thread::hardware_concurrency()), (nsys + 1) / 2),
                                   std::max(1, natom_total_ / 10000));
    if (nthr <= 1) {
      resume_range(0, nsys);
    } else {
      std::vector<std::thread> pool;
      for (int k = 0; k < nthr; k++)
        pool.emplace_back(resume_range, static_cast<int>(static_cast<long long>(nsys) * k / nthr),
                          static_cast<int>(static_cast<long long>(nsys) * (k + 1) / nthr));
      for (auto &th : pool) th.join();
    }
  }
  // results: each system's conflib (its nconf structures, lowest first)
  // and its lowest structure in the batch, every system switched on again
  if (conflib) {
    for (int s = 0; s < nsys; s++) {
      const size_t na3 = 3 * static_cast<size_t>(sys_[s].natom);
      double *dst = conflib + static_cast<size_t>(lo.nconf) * off(s);
      for (size_t i = 0; i < static_cast<size_t>(nconf[s]) * na3; i++) dst[i] = sys[s].conflib[i];
    }
  }
  if ((rc = set_all_coords(x.data(), stream))) return rc;
  std::fill(on.begin(), on.end(), 1);
  if ((rc = set_all_active(on, stream))) return rc;
  return SFFG_OK;
}

}  // namespace sffg
