// Serving: continuous batching of minimisation (conjgrad) and Langevin md
// requests on one GPU (include/sffg.h, sffg_server_*).  No counterpart in
// the reference, which runs one system per process.
//
// Requests run in groups: one Batch per group, on its own stream, its
// systems resident on the GPU.  Every group advances on its own: a pump
// launches the next turns (conjgrad evaluations or md steps) of every group
// whose earlier turns have finished, then waits until some group's turns
// finish and takes the results of the systems that ended, so a group of
// small molecules is not held to the pace of a group of large ones.
//
// Admission (in arrival order, under the device-memory budget):
//  * a minimisation joins the running minimisation group -- slot-level
//    admission: its system is added to that group's flattened work queue --
//    or, with none running, starts it;
//  * md requests start a new group (md steps keep no per-system step count
//    that a move could carry).
// Batched conjgrad moves every system in lock step, one evaluation per
// turn, so a group's turn takes as long as its whole queue.  The option
// sffg_serve_classes=1 instead keeps one minimisation group per size class
// (size_class), so that a small molecule is not tied to a large one's
// turns; measured on mixed 500-50,000-atom streams it served fewer requests
// per second at a higher median latency, because a large group's pair
// kernels occupy every SM and the small groups' kernels wait for them
// anyway, so one flattened queue is the default.
//
// A join takes effect where the group's turn count is a multiple of nsnb:
// the running systems' state (conjgrad state machine, coordinates, gradient,
// work vectors) moves into a new batch holding them and the newcomers, the
// systems that ended are left out, and the first evaluation rebuilds the
// pair lists -- as each running system's own next evaluation would, since
// every system joined at such a turn.  So a request's pair lists are built
// at the same evaluations as if it ran alone, its atom order comes from its
// own initial coordinates, and its sums are fixed point: its result does
// not depend on the group it runs in, or on the moves.
#include <chrono>
#include <cmath>
#include <deque>
#include <map>
#include <memory>
#include <thread>

#include "engine.h"

namespace sffg {
namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// Size class of a minimisation under sffg_serve_classes=1: molecules under
// 4,096 atoms, whose evaluations cost little more than their launches,
// share one class; above that, one class per doubling of the atom count
// (pair work within 4x).
int size_class(int natom) {
  int c = 0;
  for (int n = natom / 4096; n > 0; n >>= 1) c++;
  return c;
}

struct Request {
  long long id = 0;
  int kind = 0, nsteps = 0, natom = 0;
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
  cudaEvent_t ev = nullptr;  // recorded after the last turns launched
  bool in_flight = false;
  std::vector<long long> ids;  // system s of the batch serves ids[s]
  std::vector<bool> finished;
  std::vector<long long> joiners;  // admitted, waiting for the next turn that is a multiple of nsnb
  int kind = 0, cls = 0, turns = 0;
  size_t bytes = 0, joiner_bytes = 0;
  bool first = true;
  int nrunning() const {
    int n = 0;
    for (bool f : finished) n += !f;
    return n;
  }
};

}  // namespace

class Server {
 public:
  Server(const Options &o, size_t budget, int max_groups) : opts_(o), budget_(budget), max_groups_(max_groups) {}
  ~Server() {
    for (auto &g : groups_) release(*g);
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
    r->natom = prm->Natom;
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

  // Admit; launch the next turns of every idle group; wait until one group's
  // turns have run; collect.
  int pump(int turns, int *nrunning, int *npending, std::string &err) {
    int rc = admit(err);
    if (rc) return rc;
    for (auto &gp : groups_)
      if (!gp->in_flight && (rc = launch(*gp, turns, err))) return rc;
    bool any = false;
    for (auto &gp : groups_) any |= gp->in_flight;
    // a host-side wait for the first group to finish its turns (no device
    // spin; each query returns at once)
    while (any) {
      bool ready = false;
      for (auto &gp : groups_) {
        if (!gp->in_flight) continue;
        const cudaError_t e = cudaEventQuery(gp->ev);
        if (e == cudaSuccess) {
          gp->in_flight = false;
          ready = true;
        } else if (e != cudaErrorNotReady) {
          err = std::string("serving: ") + cudaGetErrorString(e);
          return SFFG_ECUDA;
        }
      }
      if (ready) break;
      std::this_thread::sleep_for(std::chrono::microseconds(20));
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
  long long groups_started = 0, joins = 0, joined = 0;
  double form_ms = 0.0;

 private:
  Group *min_group(int cls) {
    for (auto &gp : groups_)
      if (gp->kind == SFFG_REQ_MINIMIZE && gp->cls == cls) return gp.get();
    return nullptr;
  }

  // Takes waiting requests, in arrival order, while they fit the budget:
  // minimisations join their class's group (or start it); the md requests
  // taken in one admission start a group together (each runs exactly its
  // own number of steps: launch stops at the nearest end).
  int admit(std::string &err) {
    std::map<int, std::vector<long long>> fresh_min;  // class -> new group
    std::vector<long long> fresh_md;
    int nfresh = 0;
    std::deque<long long> keep;
    bool full = false;
    while (!pending_.empty()) {
      const long long id = pending_.front();
      pending_.pop_front();
      Request &r = *reqs_[id];
      if (full || in_use_ + r.bytes > budget_) {
        full = true;  // strict arrival order under the budget
        keep.push_back(id);
        continue;
      }
      if (r.kind == SFFG_REQ_MINIMIZE) {
        const int c = opts_.sffg_serve_classes ? size_class(r.natom) : 0;
        if (Group *g = min_group(c)) {
          g->joiners.push_back(id);
          g->joiner_bytes += r.bytes;
        } else if (fresh_min.count(c) || static_cast<int>(groups_.size()) + nfresh < max_groups_) {
          nfresh += fresh_min.count(c) ? 0 : 1;
          fresh_min[c].push_back(id);
        } else {
          keep.push_back(id);
          continue;
        }
      } else if (!fresh_md.empty() || static_cast<int>(groups_.size()) + nfresh < max_groups_) {
        nfresh += fresh_md.empty() ? 1 : 0;
        fresh_md.push_back(id);
      } else {
        keep.push_back(id);
        continue;
      }
      in_use_ += r.bytes;
    }
    pending_.swap(keep);
    // every new group is started even if one fails (its requests then end
    // with the failure's status); the first failure is reported
    int first_rc = SFFG_OK;
    for (auto &kv : fresh_min) {
      const int rc = start_group(SFFG_REQ_MINIMIZE, kv.first, kv.second, err);
      if (rc && first_rc == SFFG_OK) first_rc = rc;
    }
    if (!fresh_md.empty()) {
      const int rc = start_group(SFFG_REQ_MD, 0, fresh_md, err);
      if (rc && first_rc == SFFG_OK) first_rc = rc;
    }
    return first_rc;
  }

  // A new group of the given requests (their estimated bytes already in
  // in_use_).  On a failure the requests end with its status and their
  // bytes return to the budget.
  int start_group(int kind, int cls, const std::vector<long long> &take, std::string &err) {
    auto gp = std::make_unique<Group>();
    Group &g = *gp;
    g.kind = kind;
    g.cls = cls;
    size_t est = 0;
    for (long long id : take) est += reqs_[id]->bytes;
    // with size classes, smaller classes get higher stream priority: where a
    // larger group's kernel ends, the device starts their waiting kernels first
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) least = greatest = 0;
    const int prio = kind == SFFG_REQ_MINIMIZE && opts_.sffg_serve_classes ? std::max(greatest, least - (6 - std::min(cls, 6)))
                                                                          : least;
    if (cudaStreamCreateWithPriority(&g.stream, cudaStreamNonBlocking, prio) != cudaSuccess ||
        cudaEventCreateWithFlags(&g.ev, cudaEventDisableTiming) != cudaSuccess) {
      for (long long id : take) fail_request(id, SFFG_ECUDA);
      in_use_ -= std::min(in_use_, est);
      release(g);
      err = "stream creation failed";
      return SFFG_ECUDA;
    }
    const int rc = form(g, {}, take, est, err);
    if (rc) {
      for (long long id : take) fail_request(id, rc);
      in_use_ -= std::min(in_use_, est);
      release(g);
      return rc;
    }
    groups_.push_back(std::move(gp));
    groups_started++;
    return SFFG_OK;
  }

  // (Re)builds group g's batch: the carried systems (ids with their
  // exported state, taken from the old batch) and then the new requests.
  // reserved: the bytes in_use_ holds for the new requests; the group then
  // holds the estimate of all its systems, or the batch's measured size if
  // larger.
  int form(Group &g, const std::vector<std::pair<long long, Batch::CgCarry>> &carried,
           const std::vector<long long> &take, size_t reserved, std::string &err) {
    const double t0 = now_ms();
    const int rc = form_batch(g, carried, take, reserved, err);
    form_ms += now_ms() - t0;
    return rc;
  }

  int form_batch(Group &g, const std::vector<std::pair<long long, Batch::CgCarry>> &carried,
                 const std::vector<long long> &take, size_t reserved, std::string &err) {
    std::vector<HostSystem> hs_carried;
    std::vector<std::vector<double>> x0_carried;
    std::unique_ptr<Batch> old = std::move(g.batch);
    if (old) {
      for (size_t k = 0; k < carried.size(); k++) {
        const int s = index_of(g, carried[k].first);
        hs_carried.push_back(old->host_system(s));
        x0_carried.push_back(old->initial_coords(s));
      }
    }
    auto nb = std::make_unique<Batch>(opts_);
    if (old) nb->adopt_split(*old);
    in_use_ -= g.bytes;
    g.bytes = 0;
    old.reset();  // its memory goes back before the new batch takes its own
    std::vector<long long> ids;
    for (size_t k = 0; k < carried.size(); k++) {
      const int s = nb->add_host_system(std::move(hs_carried[k]), x0_carried[k].data());
      if (s < 0) {
        err = nb->last_error;
        return s;
      }
      ids.push_back(carried[k].first);
    }
    for (long long id : take) {
      Request &r = *reqs_[id];
      const int s = nb->add_host_system(std::move(r.hs), r.x.data());
      if (s < 0) {
        err = nb->last_error;
        return s;
      }
      nb->set_noise_key(s, r.key);
      ids.push_back(id);
    }
    int rc = nb->finalize();
    if (rc) {
      err = nb->last_error;
      return rc;
    }
    if (g.kind == SFFG_REQ_MINIMIZE) {
      std::vector<int> maxit;
      std::vector<double> rms;
      for (long long id : ids) {
        maxit.push_back(reqs_[id]->nsteps);
        rms.push_back(reqs_[id]->rmsgrad);
      }
      if ((rc = nb->cg_begin(maxit, rms, 1.0, g.stream))) {
        err = nb->last_error;
        return rc;
      }
      for (size_t k = 0; k < carried.size(); k++)
        if ((rc = nb->cg_import(static_cast<int>(k), carried[k].second, g.stream))) {
          err = nb->last_error;
          return rc;
        }
    } else if ((rc = nb->md_begin(true, nullptr, nullptr, g.stream))) {
      err = nb->last_error;
      return rc;
    }
    size_t est = 0;
    for (long long id : ids) est += reqs_[id]->bytes;
    in_use_ -= reserved;
    g.bytes = std::max(est, nb->device_bytes());
    in_use_ += g.bytes;
    g.batch = std::move(nb);
    g.ids = ids;
    g.finished.assign(ids.size(), false);
    g.first = true;
    return SFFG_OK;
  }

  static int index_of(const Group &g, long long id) {
    for (size_t s = 0; s < g.ids.size(); s++)
      if (g.ids[s] == id) return static_cast<int>(s);
    return -1;
  }

  // Moves group g's running systems and its joiners into a new batch (g is
  // idle, at a turn that is a multiple of nsnb).
  int join(Group &g, std::string &err) {
    std::vector<std::pair<long long, Batch::CgCarry>> carried;
    for (size_t s = 0; s < g.ids.size(); s++) {
      if (g.finished[s]) continue;
      carried.emplace_back(g.ids[s], Batch::CgCarry());
      const int rc = g.batch->cg_export(static_cast<int>(s), carried.back().second, g.stream);
      if (rc) {
        err = g.batch->last_error;
        return rc;
      }
    }
    std::vector<long long> take;
    take.swap(g.joiners);
    joins++;
    joined += static_cast<long long>(take.size());
    const size_t est = g.joiner_bytes;
    g.joiner_bytes = 0;
    const int rc = form(g, carried, take, est, err);
    if (rc) {
      // the group's old batch is gone: its running requests and the
      // joiners end with the failure's status, and collect() drops it
      for (auto &c : carried) fail_request(c.first, rc);
      for (long long id : take) fail_request(id, rc);
      g.batch.reset();
      g.ids.clear();
      g.finished.clear();
      in_use_ -= std::min(in_use_, g.bytes + est);
      g.bytes = 0;
    }
    return rc;
  }

  void fail_request(long long id, int status) {
    Request &r = *reqs_[id];
    if (r.done) return;
    r.status = status;
    r.energy = std::nan("");
    r.t_done = now_ms();
    r.done = true;
  }

  int launch(Group &g, int turns, std::string &err) {
    int rc = SFFG_OK;
    if (!g.batch) return SFFG_OK;
    if (g.kind == SFFG_REQ_MINIMIZE) {
      const int nsnb = std::max(1, opts_.nsnb);
      if (!g.joiners.empty()) {
        if (g.nrunning() == 0 || g.batch->cg_turn() % nsnb == 0) {
          if ((rc = join(g, err))) return rc;
        } else {
          // run up to the next turn that is a multiple of nsnb
          turns = std::min(turns, nsnb - g.batch->cg_turn() % nsnb);
        }
      }
      if (g.nrunning() == 0) return SFFG_OK;
      rc = g.batch->cg_turns(turns, g.first, g.stream);
    } else {
      // up to the end of the running system with the fewest steps left, so
      // that every system runs exactly its own number of steps
      int k = turns;
      for (size_t s = 0; s < g.ids.size(); s++)
        if (!g.finished[s]) k = std::min(k, reqs_[g.ids[s]]->nsteps - g.turns);
      if (k <= 0) return SFFG_OK;
      rc = g.batch->md_steps(g.turns, k, nullptr, nullptr, g.stream);
      g.turns += k;
    }
    if (rc) {
      err = g.batch->last_error;
      return rc;
    }
    g.first = false;
    if (cudaEventRecord(g.ev, g.stream) != cudaSuccess) {
      err = "event record failed";
      return SFFG_ECUDA;
    }
    g.in_flight = true;
    return SFFG_OK;
  }

  // Takes the results of systems that ended and retires finished groups
  // (those not waiting for joiners).  A request whose coordinates turned
  // non-finite ends at once with SFFG_ENONFINITE; the others in its group go
  // on unaffected.
  int collect(std::string &err) {
    for (size_t gi = 0; gi < groups_.size();) {
      Group &g = *groups_[gi];
      if (g.in_flight) {
        gi++;
        continue;
      }
      if (!g.batch) {  // a join that failed
        release(g);
        groups_.erase(groups_.begin() + gi);
        continue;
      }
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
      if (g.kind == SFFG_REQ_MINIMIZE) {
        int na = 0;
        std::vector<int> st;
        std::vector<double> en;
        int rc = g.batch->cg_poll(&na, &st, &en, g.stream);
        if (rc) {
          err = g.batch->last_error;
          return rc;
        }
        for (int s = 0; s < nsys; s++)
          if (!g.finished[s] && (st[s] != 0 || na == 0)) finish(g, s, st[s] != 0 ? st[s] : -3, en[s]);
      } else {
        std::vector<double> ene;
        for (int s = 0; s < nsys; s++) {
          if (g.finished[s]) continue;
          const Request &r = *reqs_[g.ids[s]];
          if (g.turns >= r.nsteps) {
            if (ene.empty()) g.batch->get_all_energies(ene, g.stream);
            g.batch->set_active(s, false, g.stream);
            finish(g, s, r.nsteps, ene[13 * s]);
          }
        }
      }
      if (g.nrunning() == 0 && g.joiners.empty()) {
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
    if (g.ev) cudaEventDestroy(g.ev);
    if (g.stream) cudaStreamDestroy(g.stream);
    g.ev = nullptr;
    g.stream = nullptr;
  }

  Options opts_;
  size_t budget_, in_use_ = 0;
  int max_groups_;
  long long next_id_ = 1;
  std::deque<long long> pending_;
  std::map<long long, std::unique_ptr<Request>> reqs_;
  std::vector<std::unique_ptr<Group>> groups_;
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

extern "C" int sffg_server_counts(const sffg_server *s, long long *groups_started, long long *joins,
                                  long long *joined, double *form_ms) {
  if (!s) return SFFG_EINVAL;
  if (form_ms) *form_ms = s->impl->form_ms;
  if (groups_started) *groups_started = s->impl->groups_started;
  if (joins) *joins = s->impl->joins;
  if (joined) *joined = s->impl->joined;
  return SFFG_OK;
}

extern "C" const char *sffg_server_error(const sffg_server *s) { return s ? s->err.c_str() : ""; }

extern "C" int sffg_server_destroy(sffg_server *s) {
  if (!s) return SFFG_EINVAL;
  delete s->impl;
  delete s;
  return SFFG_OK;
}
