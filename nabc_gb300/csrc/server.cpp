// Serving: continuous batching of minimisation (conjgrad) and Langevin md
// requests on one GPU (include/sffg.h, sffg_server_*).  No counterpart in
// the reference, which runs one system per process.
//
// Requests wait in arrival order.  At every pump, the waiting requests at
// the head of the queue that fit the device-memory budget (and are of the
// same kind) are admitted together as a new group: one Batch with its own
// stream, its systems resident on the GPU until the group ends.  Every
// running group is then advanced by a few turns (conjgrad evaluations or md
// steps), launched without waiting, so the groups' kernels overlap on the
// device; groups admitted later join those still running.  A request's
// result (return code, energy, coordinates) is taken as soon as its own
// system ends; the group's memory returns to the budget when all of its
// systems have ended.  A system's result does not depend on the group it
// runs in: the work of every system is independent and its sums are fixed
// point.
#include <chrono>
#include <cmath>
#include <deque>
#include <map>
#include <memory>

#include "engine.h"

namespace sffg {
namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  long long id = 0;
  int kind = 0, nsteps = 0;
  double rmsgrad = 0.0;
  HostSystem hs;
  std::vector<double> x;
  size_t bytes = 0;  // admission estimate
  unsigned long long key = 0;  // md noise key: a hash of the request's coordinates
  double t_submit = 0.0, t_done = 0.0;
  int status = 0;  // 0 waiting or running; the driver's return code when done
  double energy = 0.0;
  bool done = false;
};

struct Group {
  std::unique_ptr<Batch> batch;
  cudaStream_t stream = nullptr;
  std::vector<long long> ids;  // system s of the batch serves ids[s]
  std::vector<bool> finished;
  int kind = 0, turns = 0, max_steps = 0;
  size_t bytes = 0;
  bool first = true;
};

}  // namespace

class Server {
 public:
  Server(const Options &o, size_t budget, int max_groups) : opts_(o), budget_(budget), max_groups_(max_groups) {}
  ~Server() {
    for (auto &g : groups_) release(g);
  }

  // Device bytes a request of n atoms is expected to hold: per-atom state
  // and the pair lists, whose size grows with the atoms within the cutoff
  // (at most 0.12 atoms per cubic Angstrom).
  size_t estimate(int n) const {
    const double within = std::min<double>(n, 0.12 * 4.18879 * std::pow(std::min(opts_.cut, 200.0), 3.0));
    const double pairs = 0.5 * n * within;
    return static_cast<size_t>(2048.0 * n + 6.0 * pairs + (4 << 20));
  }

  int submit(PARMSTRUCT_T *prm, const double *x, int kind, int nsteps, double rmsgrad, long long *id,
             std::string &err) {
    if (!prm || !x || prm->Natom <= 0) {
      err = "submit: null topology or coordinates";
      return SFFG_EINVAL;
    }
    if (kind != SFFG_REQ_MINIMIZE && kind != SFFG_REQ_MD) {
      err = "submit: unknown request kind";
      return SFFG_EINVAL;
    }
    if (nsteps < 1) {
      err = "submit: nsteps must be positive";
      return SFFG_EINVAL;
    }
    auto r = std::make_unique<Request>();
    r->id = next_id_++;
    r->kind = kind;
    r->nsteps = nsteps;
    r->rmsgrad = rmsgrad;
    ModelParams mp;
    build_host_system(prm, nullptr, opts_, false, r->hs, mp);
    r->x.assign(x, x + 3 * static_cast<size_t>(prm->Natom));
    // FNV-1a over the coordinate bytes: the same request draws the same md
    // noise whatever else runs beside it
    unsigned long long h = 1469598103934665603ull;
    const unsigned char *b = reinterpret_cast<const unsigned char *>(r->x.data());
    for (size_t k = 0; k < r->x.size() * sizeof(double); k++) h = (h ^ b[k]) * 1099511628211ull;
    r->key = h;
    r->bytes = estimate(prm->Natom);
    if (r->bytes > budget_) {
      err = "submit: the request alone exceeds the memory budget";
      return SFFG_ENOMEM;
    }
    r->t_submit = now_ms();
    *id = r->id;
    pending_.push_back(r->id);
    reqs_[r->id] = std::move(r);
    return SFFG_OK;
  }

  int pump(int turns, int *nrunning, int *npending, std::string &err) {
    int rc = admit(err);
    if (rc) return rc;
    for (auto &g : groups_) {
      int k = turns;
      if (g.kind == SFFG_REQ_MINIMIZE) {
        rc = g.batch->cg_turns(turns, g.first, g.stream);
      } else {
        k = std::min(turns, g.max_steps - g.turns);
        rc = k > 0 ? g.batch->md_steps(g.turns, k, nullptr, nullptr, g.stream) : SFFG_OK;
      }
      if (rc) {
        err = g.batch->last_error;
        return rc;
      }
      g.first = false;
      g.turns += k;
    }
    if ((rc = collect(err))) return rc;
    if (nrunning) *nrunning = static_cast<int>(groups_.size());
    if (npending) *npending = static_cast<int>(pending_.size());
    return SFFG_OK;
  }

  int result(long long id, int *status, double *energy, double *x, double *latency_ms, std::string &err) {
    auto it = reqs_.find(id);
    if (it == reqs_.end()) {
      err = "result: unknown request";
      return SFFG_EINVAL;
    }
    const Request &r = *it->second;
    if (!r.done) return SFFG_ESTATE;
    if (status) *status = r.status;
    if (energy) *energy = r.energy;
    if (x) std::copy(r.x.begin(), r.x.end(), x);
    if (latency_ms) *latency_ms = r.t_done - r.t_submit;
    return SFFG_OK;
  }

  size_t in_use() const { return in_use_; }

 private:
  // Admits the waiting requests at the head of the queue that fit.
  int admit(std::string &err) {
    while (!pending_.empty() && static_cast<int>(groups_.size()) < max_groups_) {
      const int kind = reqs_[pending_.front()]->kind;
      std::vector<long long> take;
      size_t bytes = 0;
      for (long long id : pending_) {
        const Request &r = *reqs_[id];
        if (r.kind != kind || in_use_ + bytes + r.bytes > budget_) break;
        take.push_back(id);
        bytes += r.bytes;
      }
      if (take.empty()) return SFFG_OK;  // wait for memory
      Group g;
      g.kind = kind;
      g.batch = std::make_unique<Batch>(opts_);
      for (long long id : take) {
        Request &r = *reqs_[id];
        const int s = g.batch->add_host_system(std::move(r.hs), r.x.data());
        if (s < 0) {
          err = g.batch->last_error;
          return s;
        }
        g.batch->set_noise_key(s, r.key);
        g.ids.push_back(id);
        g.max_steps = std::max(g.max_steps, r.nsteps);
      }
      int rc = g.batch->finalize();
      if (rc) {
        err = g.batch->last_error;
        return rc;
      }
      if (cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking) != cudaSuccess) {
        err = "stream creation failed";
        return SFFG_ECUDA;
      }
      g.bytes = std::max(bytes, g.batch->device_bytes());
      g.finished.assign(take.size(), false);
      if (kind == SFFG_REQ_MINIMIZE) {
        std::vector<int> maxit;
        std::vector<double> rms;
        for (long long id : take) {
          maxit.push_back(reqs_[id]->nsteps);
          rms.push_back(reqs_[id]->rmsgrad);
        }
        rc = g.batch->cg_begin(maxit, rms, 1.0, g.stream);
      } else {
        rc = g.batch->md_begin(true, nullptr, nullptr, g.stream);
      }
      if (rc) {
        err = g.batch->last_error;
        return rc;
      }
      for (size_t k = 0; k < take.size(); k++) pending_.pop_front();
      in_use_ += g.bytes;
      groups_.push_back(std::move(g));
    }
    return SFFG_OK;
  }

  // Takes the results of systems that ended and retires finished groups.
  // A request whose coordinates turned non-finite ends at once with
  // SFFG_ENONFINITE; the others in its group go on unaffected.
  int collect(std::string &err) {
    for (size_t gi = 0; gi < groups_.size();) {
      Group &g = groups_[gi];
      const int nsys = static_cast<int>(g.ids.size());
      std::vector<int> health;
      int rc0 = g.batch->system_status(health, g.stream);
      if (rc0) {
        err = g.batch->last_error;
        return rc0;
      }
      for (int s = 0; s < nsys; s++) {
        if (g.finished[s] || health[s] == SFFG_OK) continue;
        g.batch->set_active(s, false, g.stream);
        finish(g, s, SFFG_ENONFINITE, std::nan(""));
      }
      bool all = true;
      if (g.kind == SFFG_REQ_MINIMIZE) {
        int na = 0;
        std::vector<int> st;
        std::vector<double> en;
        int rc = g.batch->cg_poll(&na, &st, &en, g.stream);
        if (rc) {
          err = g.batch->last_error;
          return rc;
        }
        for (int s = 0; s < nsys; s++) {
          if (g.finished[s]) continue;
          if (st[s] != 0) {
            finish(g, s, st[s], en[s]);
          } else {
            all = false;
          }
        }
        if (!all && na == 0) all = true;
      } else {
        std::vector<double> ene;
        for (int s = 0; s < nsys; s++) {
          if (g.finished[s]) continue;
          const Request &r = *reqs_[g.ids[s]];
          if (g.turns >= r.nsteps) {
            if (ene.empty()) g.batch->get_all_energies(ene, g.stream);
            g.batch->set_active(s, false, g.stream);
            finish(g, s, r.nsteps, ene[13 * s]);
          } else {
            all = false;
          }
        }
      }
      if (all) {
        in_use_ -= g.bytes;
        release(g);
        groups_.erase(groups_.begin() + gi);
      } else {
        gi++;
      }
    }
    return SFFG_OK;
  }

  void finish(Group &g, int s, int status, double energy) {
    Request &r = *reqs_[g.ids[s]];
    r.status = status;
    r.energy = energy;
    g.batch->get_coords(s, r.x.data(), g.stream);
    r.t_done = now_ms();
    r.done = true;
    g.finished[s] = true;
  }

  void release(Group &g) {
    g.batch.reset();
    if (g.stream) cudaStreamDestroy(g.stream);
    g.stream = nullptr;
  }

  Options opts_;
  size_t budget_, in_use_ = 0;
  int max_groups_;
  long long next_id_ = 1;
  std::deque<long long> pending_;
  std::map<long long, std::unique_ptr<Request>> reqs_;
  std::vector<Group> groups_;
};

}  // namespace sffg

struct sffg_server {
  sffg::Server *impl;
  std::string err;
};

extern "C" int sffg_server_create(const char *opts, double memory_budget_gb, int max_groups, sffg_server **out) {
  if (!out || !(memory_budget_gb > 0.0) || max_groups < 1) return SFFG_EINVAL;
  sffg::Options o;
  std::string bad;
  if (sffg::parse_options(opts, o, false, false, &bad)) return SFFG_EINVAL;
  if (o.gb == 0 || o.gb == 3 || o.rgbmax > o.cut) return SFFG_EINVAL;
  *out = new sffg_server{new sffg::Server(o, static_cast<size_t>(memory_budget_gb * 1e9), max_groups), {}};
  return SFFG_OK;
}

extern "C" int sffg_server_submit(sffg_server *s, PARMSTRUCT_T *prm, const double *x, int kind, int nsteps,
                                  double rmsgrad, long long *id) {
  if (!s || !id) return SFFG_EINVAL;
  return s->impl->submit(prm, x, kind, nsteps, rmsgrad, id, s->err);
}

extern "C" int sffg_server_pump(sffg_server *s, int turns, int *nrunning, int *npending) {
  if (!s || turns < 1) return SFFG_EINVAL;
  return s->impl->pump(turns, nrunning, npending, s->err);
}

extern "C" int sffg_server_result(sffg_server *s, long long id, int *status, double *energy, double *x,
                                  double *latency_ms) {
  if (!s) return SFFG_EINVAL;
  return s->impl->result(id, status, energy, x, latency_ms, s->err);
}

extern "C" size_t sffg_server_device_bytes(const sffg_server *s) { return s ? s->impl->in_use() : 0; }

extern "C" const char *sffg_server_error(const sffg_server *s) { return s ? s->err.c_str() : ""; }

extern "C" int sffg_server_destroy(sffg_server *s) {
  if (!s) return SFFG_EINVAL;
  delete s->impl;
  delete s;
  return SFFG_OK;
}
