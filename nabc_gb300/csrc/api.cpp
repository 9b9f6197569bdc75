// The batched C API (include/sffg.h): status codes, never exits.
#include <cstring>
#include <string>

#include "engine.h"

namespace {

thread_local std::string g_err;

int fail(int rc, const std::string &msg) {
  g_err = msg;
  return rc;
}

int pass(sffg::Batch *b, int rc) {
  if (rc != SFFG_OK && b) g_err = b->last_error;
  return rc;
}

}  // namespace

struct sffg_batch {
  sffg::Batch *impl;
};

extern "C" const char *sffg_last_error(void) { return g_err.c_str(); }

extern "C" int sffg_batch_create(const char *opts, sffg_batch **out) {
  if (!out) return fail(SFFG_EINVAL, "null output handle");
  sffg::Options o;
  std::string bad;
  if (sffg::parse_options(opts, o, false, false, &bad)) return fail(SFFG_EINVAL, "bad option: " + bad);
  if (o.gb == 0 || o.gb == 3) return fail(SFFG_EINVAL, "gb must be 1, 2, 5, 7 or 8");
  if (o.rgbmax > o.cut) return fail(SFFG_EINVAL, "rgbmax is greater than cut");
  *out = new sffg_batch{new sffg::Batch(o)};
  return SFFG_OK;
}

extern "C" int sffg_batch_add_system(sffg_batch *b, PARMSTRUCT_T *prm, const int *frozen, const double *x,
                                     int *sys_index) {
  if (!b) return fail(SFFG_EINVAL, "null batch");
  const int r = b->impl->add_system(prm, frozen, x, false);
  if (r < 0) return pass(b->impl, r);
  if (sys_index) *sys_index = r;
  return SFFG_OK;
}

extern "C" int sffg_batch_set_restraints(sffg_batch *b, int sys, const int *constrained, const double *x0) {
  if (!b) return fail(SFFG_EINVAL, "null batch");
  const int rc = b->impl->set_restraints(sys, constrained, x0);
  if (rc) return fail(rc, "set_restraints: bad system or arrays, or batch already finalized");
  return SFFG_OK;
}

extern "C" int sffg_batch_finalize(sffg_batch *b) {
  if (!b) return fail(SFFG_EINVAL, "null batch");
  return pass(b->impl, b->impl->finalize());
}

extern "C" int sffg_batch_num_systems(const sffg_batch *b) { return b ? b->impl->num_systems() : 0; }

extern "C" int sffg_batch_num_atoms(const sffg_batch *b, int sys) {
  if (!b || sys < 0 || sys >= b->impl->num_systems()) return -1;
  return b->impl->system(sys).natom;
}

#define SFFG_WRAP(call) \
  do {                   \
    if (!b) return fail(SFFG_EINVAL, "null batch"); \
    return pass(b->impl, (call)); \
  } while (0)

extern "C" int sffg_batch_set_coords(sffg_batch *b, int sys, const double *x, void *stream) {
  SFFG_WRAP(b->impl->set_coords(sys, x, stream));
}
extern "C" int sffg_batch_get_coords(sffg_batch *b, int sys, double *x, void *stream) {
  SFFG_WRAP(b->impl->get_coords(sys, x, stream));
}
extern "C" int sffg_batch_eval(sffg_batch *b, int rebuild, void *stream) {
  SFFG_WRAP(b->impl->eval(rebuild != 0, stream));
}
extern "C" int sffg_batch_get_energy(sffg_batch *b, int sys, double *ene, void *stream) {
  SFFG_WRAP(b->impl->get_energy(sys, ene, stream));
}
extern "C" int sffg_batch_get_grad(sffg_batch *b, int sys, double *g, void *stream) {
  SFFG_WRAP(b->impl->get_grad(sys, g, stream));
}
extern "C" int sffg_batch_get_reff(sffg_batch *b, int sys, double *reff, void *stream) {
  SFFG_WRAP(b->impl->get_reff(sys, reff, stream));
}
extern "C" long long sffg_batch_num_pairs(sffg_batch *b, int sys) { return b ? b->impl->num_pairs(sys) : -1; }

extern "C" int sffg_batch_set_velocities(sffg_batch *b, int sys, const double *v, void *stream) {
  SFFG_WRAP(b->impl->set_velocities(sys, v, stream));
}
extern "C" int sffg_batch_get_velocities(sffg_batch *b, int sys, double *v, void *stream) {
  SFFG_WRAP(b->impl->get_velocities(sys, v, stream));
}

extern "C" int sffg_batch_md(sffg_batch *b, int nsteps, void *stream) {
  if (!b) return fail(SFFG_EINVAL, "null batch");
  int rc = b->impl->md_begin(false, nullptr, nullptr, stream);
  if (rc == SFFG_OK) rc = b->impl->md_steps(0, nsteps, nullptr, nullptr, stream);
  return pass(b->impl, rc);
}

extern "C" int sffg_batch_cg(sffg_batch *b, int maxiter, double rmsgrad, double dfpred, int *status,
                             double *energy, void *stream) {
  if (!b) return fail(SFFG_EINVAL, "null batch");
  std::vector<int> st;
  std::vector<double> en;
  const int rc = b->impl->cg(maxiter, rmsgrad, dfpred, true, st, en, stream, nullptr);
  if (rc) return pass(b->impl, rc);
  for (size_t s = 0; s < st.size(); s++) {
    if (status) status[s] = st[s];
    if (energy) energy[s] = en[s];
  }
  return SFFG_OK;
}

extern "C" int sffg_batch_save(sffg_batch *b, const char *path, void *stream) {
  if (!b || !path) return fail(SFFG_EINVAL, "null batch or path");
  SFFG_WRAP(b->impl->save_state(path, stream));
}

extern "C" int sffg_batch_load(sffg_batch *b, const char *path, void *stream) {
  if (!b || !path) return fail(SFFG_EINVAL, "null batch or path");
  SFFG_WRAP(b->impl->load_state(path, stream));
}

extern "C" int sffg_batch_status(sffg_batch *b, int *status, void *stream) {
  if (!b || !status) return fail(SFFG_EINVAL, "null batch or status");
  std::vector<int> st;
  const int rc = b->impl->system_status(st, stream);
  if (rc) return pass(b->impl, rc);
  for (size_t s = 0; s < st.size(); s++) status[s] = st[s];
  return SFFG_OK;
}

extern "C" int sffg_batch_xmin(sffg_batch *b, const XMIN_OPT_T *xo, int *status, int *iters, double *energy,
                               void *stream) {
  if (!b || !xo) return fail(SFFG_EINVAL, "null batch or options");
  std::vector<int> st, it;
  std::vector<double> en;
  const int rc = b->impl->xmin(*xo, st, it, en, stream);
  if (rc) return pass(b->impl, rc);
  for (size_t s = 0; s < st.size(); s++) {
    if (status) status[s] = st[s];
    if (iters) iters[s] = it[s];
    if (energy) energy[s] = en[s];
  }
  return SFFG_OK;
}

extern "C" int sffg_batch_lmod(sffg_batch *b, const LMOD_OPT_T *lo, const XMIN_OPT_T *xo, int *status,
                               double *glob_min, int *nconf, double *conflib, void *stream) {
  if (!b || !lo || !xo) return fail(SFFG_EINVAL, "null batch or options");
  std::vector<int> st, nc;
  std::vector<double> gm;
  const int rc = b->impl->lmod(*lo, *xo, st, gm, nc, conflib, stream);
  if (rc) return pass(b->impl, rc);
  for (size_t s = 0; s < st.size(); s++) {
    if (status) status[s] = st[s];
    if (glob_min) glob_min[s] = gm[s];
    if (nconf) nconf[s] = nc[s];
  }
  return SFFG_OK;
}

extern "C" int sffg_batch_md_begin(sffg_batch *b, void *stream) {
  SFFG_WRAP(b->impl->md_begin(false, nullptr, nullptr, stream));
}

extern "C" int sffg_batch_md_steps(sffg_batch *b, int step0, int nsteps, void *stream) {
  SFFG_WRAP(b->impl->md_steps(step0, nsteps, nullptr, nullptr, stream));
}

extern "C" long long sffg_batch_launch_count(const sffg_batch *b) { return b ? b->impl->launches() : 0; }

extern "C" int sffg_batch_set_profiling(sffg_batch *b, int on) { SFFG_WRAP(b->impl->set_profiling(on != 0)); }

extern "C" int sffg_batch_kernel_times(sffg_batch *b, double *ms3, long long *nevals) {
  SFFG_WRAP(b->impl->kernel_times(ms3, nevals));
}

extern "C" size_t sffg_batch_device_bytes(const sffg_batch *b) { return b ? b->impl->device_bytes() : 0; }

extern "C" int sffg_batch_destroy(sffg_batch *b) {
  if (!b) return SFFG_OK;
  delete b->impl;
  delete b;
  return SFFG_OK;
}

extern "C" int sffg_batch_tuned_split(const sffg_batch *b, int pass, int *claim, int *blocks) {
  if (!b || !claim || !blocks) return fail(SFFG_EINVAL, "null argument");
  return b->impl->tuned_split(pass, claim, blocks);
}
