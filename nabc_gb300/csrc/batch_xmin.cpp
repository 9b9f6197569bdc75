// XMIN on every system of a batch at once (include/sffg.h,
// sffg_batch_xmin).  No counterpart in the reference, whose xmin()
// (src/sff/xminC.c:2997) minimises one system through one energy function.
//
// Each system runs its own copy of the reference's minimiser (XminJob, the
// coroutine of csrc/xmin.cpp, bit for bit the reference's iterates for a
// given energy function); the systems' evaluations are batched.  Every turn
// uploads the coordinates of the systems that asked for an evaluation,
// evaluates them together in one pass over the batch (the others switched
// off), reads back all energies and gradients with one wait and resumes
// each waiting minimiser.  Systems end independently.
//
// The pair lists are rebuilt for the whole batch whenever any system's
// minimiser asks for a rebuild (each line search starts with one).  A
// rebuild regroups every system's list chunks, which changes the FP32
// rounding of the others' sums (and with a finite cutoff may change their
// pair sets), so a system in a mixed batch follows its lone run to rounding
// only; a one-system batch has the lone run's rebuild points and ends bit
// for bit where xmin() over mme() ends.  Runs are deterministic.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <thread>
#include <vector>

#include "engine.h"

namespace sffg {

// Status of a system whose energy turned non-finite (the reference's own
// codes run from -1 to -6).
constexpr int kXminNonFinite = -7;

int Batch::xmin(const XMIN_OPT_T &xo_in, std::vector<int> &status, std::vector<int> &iters,
                std::vector<double> &energy, void *stream) {
  if (!finalized_) return SFFG_ESTATE;
  if (!xo_in.mol_struct_opt) {
    last_error = "xmin: a batch minimises molecular structures (mol_struct_opt = 1)";
    return SFFG_EINVAL;
  }
  const int nsys = num_systems();
  XMIN_OPT_T xo = xo_in;
  xo.print_level = 0;  // no per-system progress lines
  HostDoubles x(3 * static_cast<size_t>(natom_total_)), g(3 * static_cast<size_t>(natom_total_));
  std::vector<double> ene;
  for (int s = 0; s < nsys; s++) {
    int rc = get_coords(s, x.data() + 3 * static_cast<size_t>(sys_[s].atom_off), stream);
    if (rc) return rc;
  }
  std::vector<int> on(nsys, 1);
  int rc = set_all_active(on, stream);
  if (rc) return rc;
  // the gradient on entry marks frozen atoms (xminC.c:2590-2630)
  if ((rc = eval(true, stream))) return rc;
  if ((rc = get_all_energy_grad(ene, g.data(), stream))) return rc;
  std::vector<XminJob> jobs(nsys);
  std::vector<int> request(nsys, 0), state(nsys, 0);  // state: 1 waiting for an evaluation
  status.assign(nsys, 0);
  iters.assign(nsys, 0);
  energy.assign(nsys, 0.0);
  auto settle = [&](int s, int r) {
    if (r == 1) {
      state[s] = 1;
    } else {
      state[s] = 0;
      status[s] = r;
      iters[s] = jobs[s].iter();
    }
  };
  std::vector<int> health;
  if ((rc = system_status(health, stream))) return rc;
  for (int s = 0; s < nsys; s++) {
    const size_t o = 3 * static_cast<size_t>(sys_[s].atom_off);
    energy[s] = ene[13 * s];
    if (health[s] != SFFG_OK || !std::isfinite(ene[13 * s])) {  // never starts
      status[s] = kXminNonFinite;
      continue;
    }
    settle(s, jobs[s].start(xo, sys_[s].natom, x.data() + o, g.data() + o, ene[13 * s], &request[s], FLT_EPSILON));
  }
  for (;;) {
    bool any = false, rebuild = false;
    for (int s = 0; s < nsys; s++) {
      on[s] = state[s];
      any = any || state[s];
      rebuild = rebuild || (state[s] && request[s] >= 4 && request[s] <= 6);
    }
    if (!any) break;
    if ((rc = set_all_active(on, stream))) return rc;
    if ((rc = set_all_coords(x.data(), stream))) return rc;
    if ((rc = eval(rebuild, stream))) return rc;
    if ((rc = get_all_energy_grad(ene, g.data(), stream, &health))) return rc;
    // the minimisers are independent: resume them on the host's cores
    // (each system's arithmetic is the same on any thread)
    auto resume_range = [&](int s0, int s1) {
      for (int s = s0; s < s1; s++) {
        if (!state[s]) continue;
        const size_t o = 3 * static_cast<size_t>(sys_[s].atom_off);
        energy[s] = ene[13 * s];
        if (health[s] != SFFG_OK || !std::isfinite(ene[13 * s])) {  // a non-finite system ends alone
          state[s] = 0;
          status[s] = kXminNonFinite;
          iters[s] = jobs[s].iter();
          continue;
        }
        settle(s, jobs[s].resume(ene[13 * s], g.data() + o, x.data() + o, &request[s]));
      }
    };
    // host threads pay for themselves only on large systems: a thread is
    // started per turn, about the cost of resuming 10,000 atoms' minimiser
    const int nthr = std::min<int>(std::min<int>(std::max(1u, std::thread::hardware_concurrency()), (nsys + 3) / 4),
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
  // the final structures on the device, every system switched on again
  if ((rc = set_all_coords(x.data(), stream))) return rc;
  std::fill(on.begin(), on.end(), 1);
  if ((rc = set_all_active(on, stream))) return rc;
  for (int s = 0; s < nsys; s++)
    if (status[s] < 0) energy[s] = 0.0;  // xmin() returns 0 on an error
  return SFFG_OK;
}

}  // namespace sffg
