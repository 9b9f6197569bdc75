// Batch engine: device memory, uploads, list builds, the evaluation
// pipeline, device-resident md() and conjgrad().
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>

#include <nvtx3/nvToolsExt.h>

#include "engine.h"
#include "gbneck_tables.h"
#include "kernels_aux.cuh"
#include "lists.cuh"
#include "passes.h"

namespace sffg {

namespace {

template <class T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    release();
    n = count;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(&p, count * sizeof(T));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  size_t bytes() const { return n * sizeof(T); }
};


// NVTX range over a host-side scope: evaluations, list builds, md and
// minimiser turns show as named ranges in Nsight Systems or under ncu
// --nvtx (free when no tool is attached).
struct Range {
  explicit Range(const char *name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
};

}  // namespace

struct DeviceState {
  cudaStream_t stream = nullptr;
  // the bonded FP64 terms run on a side stream, beside the list upkeep and
  // the FP32 pair passes (fork after the pack, join before the gather)
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  // a queued list build's counters (pinned) and the event after their copy
  int *list_host = nullptr;
  cudaEvent_t list_ev = nullptr;
  // md replay snapshot
  DBuf<double> ck_x, ck_v, ck_accel, ck_tscal;
  DBuf<long long> ck_ekin_last;
  int nsm = 0;
  cudaEvent_t tune_ev[3][2] = {};  // pass timing while the work split is tuned
  // per slot
  DBuf<float4> pos_hi, pos_lo, gbpar;
  DBuf<int> param, slot_atom;
  DBuf<float> q32, reff32, rinv2, sumda32;
  DBuf<double> rborn64, q64, alpha, beta, gamma, reff64, psi64, chainfac;
  DBuf<double2> rinv64;  // 1 / (rborn - offset), 1 / rborn
  DBuf<long long> acc_sumi, acc_sd, acc_fx, acc_fy, acc_fz;
  // per tile
  DBuf<unsigned> tile_valid;
  DBuf<int> tile_sys;
  DBuf<float4> box_lo, box_hi;
  DBuf<int> excl_tile_start, excl_tile_j, excl_tile_idx;
  DBuf<unsigned> excl_masks;
  // per system
  DBuf<int> sys_active, sys_lj_off, sys_ntypes, sys_tile_end, sys_has_frozen, nonfinite;
  DBuf<int> sys_natom, sys_atom_off;
  DBuf<float2> lj;
  DBuf<double2> lj64;  // the same table in FP64 (close pairs)
  DBuf<float2> sys_born;  // (rgbmax + Fsmax)^2, polynomial-tail flag (DevTables::sys_born)
  DBuf<float> sys_gbb2;   // (rgbmax + Fsmax + skin)^2: lists B and C
  DBuf<long long> energy;
  DBuf<double> etot;
  // per atom
  DBuf<double> x, grad, v, accel, minv, sqrmass;
  DBuf<int> atom_slot, atom_sys, atom_frozen;
  // bonded
  DBuf<int2> bond_atoms;
  DBuf<double2> bond_par, angle_par;
  DBuf<int4> angle_atoms, dih_atoms, p14_atoms;
  DBuf<double4_32a> dih_par, p14_par;
  // pair lists (lists.cuh) and work counters: 0 candidates, 1 overflow,
  // 2 chunks of list A, 3 chunks of list B, 4 rebuild flag of lists B and
  // C, 5..7 queues of passes 1, 2 and 3, 10 chunks of list C
  DBuf<int2> cand;
  DBuf<int4> cand_n, cand_off;
  DBuf<unsigned> colA, colB, colC, colE, colK;
  DBuf<int> cand_start, cand_count, chunksA, chunksB, chunksC, chunk0A, chunk0B, chunk0C;
  DBuf<int> chunkA_i, entA_slot, chunkB_i, entB_slot, chunkC_i, entC_slot;
  DBuf<unsigned> entA_col, entA_exc, entA_close, entB_col, entC_col;
  DBuf<float4> xb;
  DBuf<int> counters;
  DBuf<unsigned> step;  // md step number (the Philox counter of the noise)
  DBuf<unsigned long long> sys_key;  // per system: noise key
  DBuf<int> tile_flagB;              // per tile: entries of lists B and C to be remade
  DBuf<double> cons_w, cons_x0;      // per atom: restraint weight (0: none), reference position
  // CUDA graphs of an evaluation and of an md step without a list rebuild,
  // with the list-buffer pointers they were captured against
  cudaGraphExec_t g_eval = nullptr, g_step = nullptr;
  std::vector<const void *> sig_eval, sig_step;
  long long launches_eval = 0, launches_step = 0;
  // model tables
  DBuf<float> neck_pos, neck_val;
  // dynamics
  DBuf<double> tscal, noise, rndf;
  // RATTLE (option rattle = 1 or 2): the constrained bonds of every system
  // by level (k_rattle), the coordinates before each drift, and a status
  // word per system
  DBuf<int2> rat_atoms;
  DBuf<double> rat_req, xold;
  DBuf<int> rat_level, rat_sys_level, rat_status;
  DBuf<long long> ekin, ekin_last;  // the step's kinetic sum, and the last finished step's
  // minimisation
  DBuf<double> cg_w;
  DBuf<CgState> cg_state;
  DBuf<int> cg_nactive;
  // per-pass timing: a ring of event pairs, read back lazily so that
  // timing never stalls the host between evaluations
  static constexpr int kRing = 64;
  cudaEvent_t events[kRing][3][2] = {};
  long long ev_head = 0, ev_tail = 0;  // recorded / collected evaluations
  double pass_ms[3] = {0, 0, 0};
  long long timed_evals = 0;

  ~DeviceState() {
    for (auto &pe : tune_ev)
      for (auto &e : pe)
        if (e) cudaEventDestroy(e);
    if (g_eval) cudaGraphExecDestroy(g_eval);
    if (g_step) cudaGraphExecDestroy(g_step);
    for (auto &ring : events)
      for (auto &pe : ring)
        for (auto &e : pe)
          if (e) cudaEventDestroy(e);
    if (fork_ev) cudaEventDestroy(fork_ev);
    if (list_ev) cudaEventDestroy(list_ev);
    if (list_host) cudaFreeHost(list_host);
    ck_x.release(); ck_v.release(); ck_accel.release(); ck_tscal.release(); ck_ekin_last.release();
    if (join_ev) cudaEventDestroy(join_ev);
    if (side) cudaStreamDestroy(side);
    if (stream) cudaStreamDestroy(stream);
    // DBuf members release in their own destructors? they are PODs: free here
    auto rel = [](auto &b) { b.release(); };
    rel(pos_hi); rel(pos_lo); rel(gbpar); rel(param); rel(slot_atom); rel(q32); rel(reff32);
    rel(rinv2); rel(sumda32); rel(rborn64); rel(rinv64); rel(q64); rel(alpha); rel(beta); rel(gamma);
    rel(reff64); rel(psi64); rel(chainfac); rel(acc_sumi); rel(acc_sd); rel(acc_fx); rel(acc_fy);
    rel(acc_fz); rel(tile_valid); rel(tile_sys); rel(box_lo); rel(box_hi); rel(excl_tile_start);
    rel(excl_tile_j); rel(excl_tile_idx); rel(excl_masks); rel(sys_active); rel(sys_lj_off);
    rel(sys_ntypes); rel(sys_tile_end); rel(sys_has_frozen); rel(nonfinite); rel(sys_natom);
    rel(sys_atom_off); rel(lj); rel(lj64); rel(sys_born); rel(sys_gbb2); rel(energy); rel(etot); rel(x); rel(grad); rel(v); rel(accel);
    rel(minv); rel(sqrmass); rel(atom_slot); rel(atom_sys); rel(atom_frozen); rel(bond_atoms);
    rel(bond_par); rel(angle_par); rel(angle_atoms); rel(dih_atoms); rel(p14_atoms); rel(dih_par);
    rel(p14_par); rel(cand); rel(cand_n); rel(cand_off); rel(colA); rel(colB); rel(colC); rel(colE);
    rel(cand_start); rel(cand_count); rel(chunksA); rel(chunksB); rel(chunksC); rel(chunk0A);
    rel(chunk0B); rel(chunk0C); rel(chunkA_i); rel(entA_slot); rel(chunkB_i); rel(entB_slot);
    rel(chunkC_i); rel(entC_slot); rel(entA_col); rel(entA_exc); rel(entB_col); rel(entC_col);
    rel(colK); rel(entA_close);
    rel(xb); rel(counters); rel(step); rel(cg_nactive); rel(sys_key); rel(tile_flagB); rel(cons_w); rel(cons_x0); rel(neck_pos); rel(neck_val); rel(tscal);
    rel(noise); rel(rndf); rel(rat_atoms); rel(rat_req); rel(xold); rel(rat_level); rel(rat_sys_level);
    rel(rat_status); rel(ekin); rel(ekin_last); rel(cg_w); rel(cg_state);
  }
};

#define SFFG_CK(call)                                                               \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      last_error = std::string(#call) + ": " + cudaGetErrorString(e_);              \
      return SFFG_ECUDA;                                                            \
    }                                                                               \
  } while (0)

// Settles a queued list build first (see Batch::settle).
#define SFFG_SETTLE(stream)                      \
  do {                                           \
    const int settle_rc_ = settle(stream);       \
    if (settle_rc_ != SFFG_OK) return settle_rc_; \
  } while (0)

Batch::Batch(const Options &opts) : opts_(opts), mp_(model_from_options(opts)) {}

Batch::~Batch() = default;

int Batch::add_system(PARMSTRUCT_T *prm, const int *frozen, const double *x, bool mutate_prm) {
  if (finalized_) {
    last_error = "add_system after finalize";
    return SFFG_ESTATE;
  }
  if (!prm || !x || prm->Natom <= 0) {
    last_error = "add_system: null topology or coordinates";
    return SFFG_EINVAL;
  }
  HostSystem hs;
  ModelParams mp;
  build_host_system(prm, frozen, opts_, mutate_prm, hs, mp);
  return add_host_system(std::move(hs), x);
}

int Batch::add_host_system(HostSystem hs, const double *x) {
  if (finalized_) {
    last_error = "add_system after finalize";
    return SFFG_ESTATE;
  }
  SystemInfo si;
  si.natom = hs.natom;
  si.atom_off = natom_total_;
  si.fsmax = hs.fsmax;
  si.frozen = hs.frozen;
  si.mass = hs.mass;
  si.ntypes = hs.ntypes;
  for (int f : hs.frozen) si.has_frozen |= f != 0;
  for (auto &d : hs.dihedrals) {
    const bool usual = !(std::fabs(d.phase - 3.142) > 0.01 && std::fabs(d.phase) > 0.01);
    const int m = static_cast<int>(std::fabs(d.pn));
    if (usual && (m < 1 || m > 6)) {
      last_error = "bad value for Pn in a dihedral";
      return SFFG_EINVAL;
    }
  }
  si.noise_key = sys_.size();
  natom_total_ += hs.natom;
  x0_.emplace_back(x, x + 3 * hs.natom);
  host_.push_back(std::move(hs));
  sys_.push_back(std::move(si));
  return static_cast<int>(sys_.size()) - 1;
}

namespace {

// Squared list-B cutoff: rgbmax + Fsmax + skin.
double list_b_cut2(const ModelParams &mp, double fsmax) {
  const double c = mp.rgbmax + fsmax + kListSkin;
  return c * c;
}

// Tile order: recursive balanced bisection of the atoms along the longest
// extent of each group, the first part holding a whole number of 32-atom
// tiles (about half).  Leaves are the tiles: compact boxes (about 9.5 A
// across at protein-like densities, against 16 x 14 x 11 A for runs of a
// Morton order), so far fewer tile pairs fall within a cutoff.  The one
// short tile, if natom is not a multiple of 32, is the last.
void bisect_tiles(const double *x, int *idx, int cnt) {
  if (cnt <= 32) return;
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int k = 0; k < cnt; k++)
    for (int d = 0; d < 3; d++) {
      const double v = x[3 * idx[k] + d];
      if (!std::isfinite(v)) continue;
      lo[d] = std::min(lo[d], v);
      hi[d] = std::max(hi[d], v);
    }
  int ax = 0;
  for (int d = 1; d < 3; d++)
    if (hi[d] - lo[d] > hi[ax] - lo[ax]) ax = d;
  const int nleft = ((cnt / 32 + 1) / 2) * 32;
  auto key = [&](int a) {
    const double v = x[3 * a + ax];
    return std::isfinite(v) ? v : 0.0;  // a strict weak order even for NaN input
  };
  std::nth_element(idx, idx + nleft, idx + cnt, [&](int a, int b) {
    const double xa = key(a), xb = key(b);
    return xa < xb || (xa == xb && a < b);
  });
  bisect_tiles(x, idx, nleft);
  bisect_tiles(x, idx + nleft, cnt - nleft);
}

}  // namespace

int Batch::finalize() {
  if (finalized_) return SFFG_OK;
  if (sys_.empty()) {
    last_error = "finalize: no systems";
    return SFFG_EINVAL;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    last_error = "no CUDA device";
    return SFFG_ENODEV;
  }
  d_.reset(new DeviceState());
  SFFG_CK(cudaStreamCreateWithFlags(&d_->stream, cudaStreamNonBlocking));
  SFFG_CK(cudaStreamCreateWithFlags(&d_->side, cudaStreamNonBlocking));
  SFFG_CK(cudaEventCreateWithFlags(&d_->fork_ev, cudaEventDisableTiming));
  SFFG_CK(cudaEventCreateWithFlags(&d_->join_ev, cudaEventDisableTiming));
  SFFG_CK(cudaDeviceGetAttribute(&d_->nsm, cudaDevAttrMultiProcessorCount, dev));
  // slot and tile layout
  int slot = 0, tile = 0;
  for (auto &s : sys_) {
    s.slot_off = slot;
    s.tile_off = tile;
    s.ntile = (s.natom + 31) / 32;
    slot += s.ntile * 32;
    tile += s.ntile;
  }
  nslot_ = slot;
  ntile_ = tile;
  const int rc = upload();
  if (rc) return rc;
  finalized_ = true;
  return SFFG_OK;
}

int Batch::upload() {
  DeviceState &d = *d_;
  const int nsys = num_systems();
  std::vector<int> slot_atom(nslot_, -1), param(nslot_, 0), tile_sys(ntile_, 0);
  std::vector<unsigned> tile_valid(ntile_, 0u);
  std::vector<float> q32(nslot_, 0.f);
  std::vector<float4> gbpar(nslot_, make_float4(1.f, 0.f, 1.f, 0.f));
  std::vector<double> rb64(nslot_, 1.0), q64(nslot_, 0.0), al(nslot_, 0.0), be(nslot_, 0.0), ga(nslot_, 0.0);
  std::vector<double2> rinv64(nslot_, make_double2(1.0, 1.0));
  std::vector<int> atom_slot(natom_total_), atom_sys(natom_total_), atom_frozen(natom_total_);
  std::vector<double> x(3 * static_cast<size_t>(natom_total_)), minv(3 * static_cast<size_t>(natom_total_)),
      sqrmass(3 * static_cast<size_t>(natom_total_));
  std::vector<int> sys_tile_end(nsys), sys_has_frozen(nsys), sys_ntypes(nsys), sys_lj_off(nsys),
      sys_natom(nsys), sys_atom_off(nsys);
  std::vector<float2> lj, sys_born(nsys);
  std::vector<float> sys_gbb2(nsys);
  std::vector<double2> lj64;
  std::map<std::vector<double>, int> lj_dedupe;
  std::vector<int> excl_tile_start(ntile_ + 1, 0);
  std::vector<std::vector<std::pair<int, int>>> excl_by_tile(ntile_);
  std::vector<unsigned> excl_masks;
  std::vector<int2> bond_atoms;
  std::vector<double2> bond_par, angle_par;
  std::vector<int4> angle_atoms, dih_atoms, p14_atoms;
  std::vector<double4_32a> dih_par, p14_par;
  const double off = mp_.gboffset;
  for (int s = 0; s < nsys; s++) {
    const SystemInfo &si = sys_[s];
    const HostSystem &hs = host_[s];
    const std::vector<double> &xs = x0_[s];
    const int n = si.natom;
    // spatial order: tiles from a balanced bisection of the initial
    // coordinates
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    bisect_tiles(xs.data(), order.data(), n);
    std::vector<int> local_slot(n);
    for (int k = 0; k < n; k++) local_slot[order[k]] = k;
    double smax = 0.0;  // largest |s| = |fs (rborn - offset)| of the system's atoms
    for (int i = 0; i < n; i++) {
      const int sl = si.slot_off + local_slot[i];
      const int a = si.atom_off + i;
      slot_atom[sl] = a;
      atom_slot[a] = sl;
      atom_sys[a] = s;
      atom_frozen[a] = hs.frozen[i];
      const double rho = hs.rborn[i] - off, sd = hs.fs[i] * rho;
      const float sf = static_cast<float>(sd);
      const float scorr = sf != 0.0f ? static_cast<float>(3.0 * (sd - static_cast<double>(sf)) / sf) : 0.0f;
      gbpar[sl] = make_float4(static_cast<float>(rho), sf, static_cast<float>(hs.rborn[i]), scorr);
      smax = std::max(smax, std::fabs(sd));
      param[sl] = (hs.type[i] & 0xffff) | (hs.neck[i] << 16) | (hs.frozen[i] ? (1 << 24) : 0);
      q32[sl] = static_cast<float>(hs.q[i]);
      q64[sl] = hs.q[i];
      rb64[sl] = hs.rborn[i];
      rinv64[sl] = make_double2(1.0 / (hs.rborn[i] - off), 1.0 / hs.rborn[i]);
      al[sl] = hs.alpha[i];
      be[sl] = hs.beta[i];
      ga[sl] = hs.gamma[i];
      for (int k = 0; k < 3; k++) {
        x[3 * static_cast<size_t>(a) + k] = xs[3 * i + k];
        minv[3 * static_cast<size_t>(a) + k] = 1.0 / hs.mass[i];
        sqrmass[3 * static_cast<size_t>(a) + k] = 1.0 / std::sqrt(1.0 / hs.mass[i]);
      }
    }
    for (int t = 0; t < si.ntile; t++) {
      const int T = si.tile_off + t;
      tile_sys[T] = s;
      const int cnt = std::min(32, n - 32 * t);
      tile_valid[T] = cnt >= 32 ? 0xffffffffu : ((1u << cnt) - 1u);
    }
    sys_tile_end[s] = si.tile_off + si.ntile;
    sys_has_frozen[s] = si.has_frozen;
    sys_ntypes[s] = hs.ntypes;
    // a tail pair has q = (rgbmax - d + s_j) / rgbmax <= 2 |s_j| / rgbmax
    const double rc = mp_.rgbmax + si.fsmax;
    sys_born[s] = make_float2(static_cast<float>(rc * rc), 2.0 * smax <= 0.3 * mp_.rgbmax * 0.999 ? 1.0f : 0.0f);
    if (sys_born[s].y == 0.0f) tail_poly_all_ = false;
    sys_gbb2[s] = static_cast<float>(std::min(list_b_cut2(mp_, si.fsmax), 1e30));
    sys_natom[s] = n;
    sys_atom_off[s] = si.atom_off;
    {
      std::vector<double> keyv(hs.lj_a64);
      keyv.insert(keyv.end(), hs.lj_b64.begin(), hs.lj_b64.end());
      keyv.push_back(static_cast<double>(hs.ntypes));
      auto it = lj_dedupe.find(keyv);
      if (it == lj_dedupe.end()) {
        const int o = static_cast<int>(lj.size());
        for (size_t k = 0; k < hs.lj_a.size(); k++) {
          lj.push_back(make_float2(hs.lj_a[k], hs.lj_b[k]));
          lj64.push_back(make_double2(hs.lj_a64[k], hs.lj_b64[k]));
        }
        it = lj_dedupe.emplace(keyv, o).first;
      }
      sys_lj_off[s] = it->second;
    }
    // exclusion masks by tile pair: row = lane of the lower tile's atom
    std::map<std::pair<int, int>, int> pair_idx;
    for (auto &e : hs.excl) {
      int si1 = si.slot_off + local_slot[e.first], si2 = si.slot_off + local_slot[e.second];
      int t1 = si1 >> 5, t2 = si2 >> 5, l1 = si1 & 31, l2 = si2 & 31;
      if (t1 > t2 || (t1 == t2 && l1 > l2)) {
        std::swap(t1, t2);
        std::swap(l1, l2);
      }
      auto key2 = std::make_pair(t1, t2);
      auto it = pair_idx.find(key2);
      if (it == pair_idx.end()) {
        const int idx = static_cast<int>(excl_masks.size() / 32);
        excl_masks.resize(excl_masks.size() + 32, 0u);
        it = pair_idx.emplace(key2, idx).first;
        excl_by_tile[t1].push_back({t2, idx});
      }
      excl_masks[static_cast<size_t>(it->second) * 32 + l1] |= 1u << l2;
    }
    const int ao = si.atom_off;
    for (auto &b : hs.bonds) {
      bond_atoms.push_back(make_int2(ao + b.a, ao + b.b));
      bond_par.push_back(make_double2(b.rk, b.req));
    }
    for (auto &a : hs.angles) {
      angle_atoms.push_back(make_int4(ao + a.a, ao + a.b, ao + a.c, 0));
      angle_par.push_back(make_double2(a.tk, a.teq));
    }
    for (auto &t : hs.dihedrals) {
      dih_atoms.push_back(make_int4(ao + t.a, ao + t.b, ao + t.c, ao + t.d));
      dih_par.push_back(make_double4_32a(t.pk, t.pn, t.phase, 0.0));
    }
    for (auto &p : hs.pairs14) {
      p14_atoms.push_back(make_int4(ao + p.a, ao + p.b, p.pow10, 0));
      // q_i * (q_j * scee), the reference's cgi * cgj (eff.c:1123-1125)
      p14_par.push_back(make_double4_32a(hs.q[p.a] * (hs.q[p.b] * p.scee), p.c12, p.c6, p.scnb));
    }
  }
  std::vector<int> excl_tile_j, excl_tile_idx;
  for (int T = 0; T < ntile_; T++) {
    excl_tile_start[T] = static_cast<int>(excl_tile_j.size());
    for (auto &e : excl_by_tile[T]) {
      excl_tile_j.push_back(e.first);
      excl_tile_idx.push_back(e.second);
    }
  }
  excl_tile_start[ntile_] = static_cast<int>(excl_tile_j.size());
  // candidate tile pairs: every tile pair of a system could be one
  long long cap = 0;
  for (auto &sy : sys_) cap += static_cast<long long>(sy.ntile) * (sy.ntile + 1) / 2;
  if (cap > (1LL << 31) / 32 - 64) {
    last_error = "batch too large for one pair list";
    return SFFG_ENOMEM;
  }
  auto up = [&](auto &buf, const auto &vec) -> cudaError_t {
    cudaError_t e = buf.alloc(vec.size());
    if (e != cudaSuccess || vec.empty()) return e;
    return cudaMemcpy(buf.p, vec.data(), vec.size() * sizeof(vec[0]), cudaMemcpyHostToDevice);
  };
  SFFG_CK(up(d.slot_atom, slot_atom));
  SFFG_CK(up(d.param, param));
  SFFG_CK(up(d.q32, q32));
  SFFG_CK(up(d.gbpar, gbpar));
  SFFG_CK(up(d.rborn64, rb64));
  SFFG_CK(up(d.rinv64, rinv64));
  SFFG_CK(up(d.q64, q64));
  SFFG_CK(up(d.alpha, al));
  SFFG_CK(up(d.beta, be));
  SFFG_CK(up(d.gamma, ga));
  SFFG_CK(up(d.tile_sys, tile_sys));
  SFFG_CK(up(d.tile_valid, tile_valid));
  SFFG_CK(up(d.sys_tile_end, sys_tile_end));
  SFFG_CK(up(d.sys_has_frozen, sys_has_frozen));
  SFFG_CK(up(d.sys_ntypes, sys_ntypes));
  SFFG_CK(up(d.sys_born, sys_born));
  SFFG_CK(up(d.sys_gbb2, sys_gbb2));
  SFFG_CK(up(d.sys_lj_off, sys_lj_off));
  SFFG_CK(up(d.sys_natom, sys_natom));
  SFFG_CK(up(d.sys_atom_off, sys_atom_off));
  SFFG_CK(up(d.lj, lj));
  SFFG_CK(up(d.lj64, lj64));
  SFFG_CK(up(d.excl_tile_start, excl_tile_start));
  SFFG_CK(up(d.excl_tile_j, excl_tile_j));
  SFFG_CK(up(d.excl_tile_idx, excl_tile_idx));
  SFFG_CK(up(d.excl_masks, excl_masks));
  SFFG_CK(up(d.atom_slot, atom_slot));
  SFFG_CK(up(d.atom_sys, atom_sys));
  SFFG_CK(up(d.atom_frozen, atom_frozen));
  SFFG_CK(up(d.x, x));
  SFFG_CK(up(d.minv, minv));
  SFFG_CK(up(d.sqrmass, sqrmass));
  SFFG_CK(up(d.bond_atoms, bond_atoms));
  SFFG_CK(up(d.bond_par, bond_par));
  SFFG_CK(up(d.angle_atoms, angle_atoms));
  SFFG_CK(up(d.angle_par, angle_par));
  SFFG_CK(up(d.dih_atoms, dih_atoms));
  SFFG_CK(up(d.dih_par, dih_par));
  SFFG_CK(up(d.p14_atoms, p14_atoms));
  SFFG_CK(up(d.p14_par, p14_par));
  std::vector<float> npos(441), nval(441);
  for (int i = 0; i < 441; i++) {
    npos[i] = static_cast<float>(sffg_neck_max_pos[i]);
    nval[i] = static_cast<float>(sffg_neck_max_val[i]);
  }
  SFFG_CK(up(d.neck_pos, npos));
  SFFG_CK(up(d.neck_val, nval));
  std::vector<int> ones(nsys, 1);
  SFFG_CK(up(d.sys_active, ones));
  SFFG_CK(d.nonfinite.alloc(nsys));
  SFFG_CK(d.pos_hi.alloc(nslot_));
  SFFG_CK(d.pos_lo.alloc(nslot_));
  SFFG_CK(d.reff32.alloc(nslot_));
  SFFG_CK(d.rinv2.alloc(nslot_));
  SFFG_CK(d.sumda32.alloc(nslot_));
  SFFG_CK(d.reff64.alloc(nslot_));
  SFFG_CK(d.psi64.alloc(nslot_));
  SFFG_CK(d.chainfac.alloc(nslot_));
  SFFG_CK(d.acc_sumi.alloc(nslot_));
  SFFG_CK(d.acc_sd.alloc(nslot_));
  SFFG_CK(d.acc_fx.alloc(nslot_));
  SFFG_CK(d.acc_fy.alloc(nslot_));
  SFFG_CK(d.acc_fz.alloc(nslot_));
  SFFG_CK(d.box_lo.alloc(ntile_));
  SFFG_CK(d.box_hi.alloc(ntile_));
  static_assert(E_NSLOTS == kEnergySlots, "energy slots");
  SFFG_CK(d.energy.alloc(static_cast<size_t>(nsys) * kEnergySlots));
  SFFG_CK(d.etot.alloc(nsys));
  SFFG_CK(d.grad.alloc(3 * static_cast<size_t>(natom_total_)));
  SFFG_CK(d.v.alloc(3 * static_cast<size_t>(natom_total_)));
  SFFG_CK(d.accel.alloc(3 * static_cast<size_t>(natom_total_)));
  SFFG_CK(cudaMemset(d.v.p, 0, d.v.bytes()));
  SFFG_CK(cudaMemset(d.accel.p, 0, d.accel.bytes()));
  SFFG_CK(cudaMemset(d.nonfinite.p, 0, d.nonfinite.bytes()));
  cand_max_ = cap;
  SFFG_CK(d.cand_start.alloc(ntile_));
  SFFG_CK(d.cand_count.alloc(ntile_));
  SFFG_CK(d.chunksA.alloc(ntile_));
  SFFG_CK(d.chunksB.alloc(ntile_));
  SFFG_CK(d.chunk0A.alloc(ntile_));
  SFFG_CK(d.chunk0B.alloc(ntile_));
  SFFG_CK(d.chunksC.alloc(ntile_));
  SFFG_CK(d.chunk0C.alloc(ntile_));
  SFFG_CK(d.xb.alloc(nslot_));
  SFFG_CK(d.counters.alloc(16));
  SFFG_CK(d.step.alloc(1));
  {
    // positional restraints, per atom
    bool any = false;
    std::vector<double> w(natom_total_, 0.0), xr(3 * static_cast<size_t>(natom_total_), 0.0);
    for (int s = 0; s < nsys; s++) {
      const SystemInfo &si = sys_[s];
      if (si.constrained.empty()) continue;
      for (int i = 0; i < si.natom; i++)
        if (si.constrained[i]) {
          w[si.atom_off + i] = opts_.wcons;
          any = any || opts_.wcons != 0.0;
        }
      std::copy(si.x0.begin(), si.x0.end(), xr.begin() + 3 * static_cast<size_t>(si.atom_off));
    }
    if (any) {
      SFFG_CK(up(d.cons_w, w));
      SFFG_CK(up(d.cons_x0, xr));
    }
  }
  SFFG_CK(d.tile_flagB.alloc(ntile_));
  SFFG_CK(cudaMemset(d.tile_flagB.p, 0, d.tile_flagB.bytes()));
  {
    std::vector<unsigned long long> keys(nsys);
    for (int s = 0; s < nsys; s++) keys[s] = sys_[s].noise_key;
    SFFG_CK(up(d.sys_key, keys));
  }
  SFFG_CK(cudaMemset(d.step.p, 0, sizeof(unsigned)));
  SFFG_CK(cudaMemset(d.counters.p, 0, d.counters.bytes()));
  SFFG_CK(d.tscal.alloc(nsys));
  SFFG_CK(d.ekin.alloc(nsys));
  SFFG_CK(d.ekin_last.alloc(nsys));
  {
    // kinetic degrees of freedom per system: 3N minus frozen, minus one per
    // RATTLE constraint (sff.c:2142-2146)
    std::vector<double> rndf(nsys);
    for (int s = 0; s < nsys; s++) {
      int nf = 0;
      for (int f : sys_[s].frozen) nf += f != 0;
      rndf[s] = 3.0 * sys_[s].natom - 3.0 * nf - rattle_bonds(s);
    }
    SFFG_CK(up(d.rndf, rndf));
  }
  if (opts_.irattle) {
    // level schedule of each system's constrained bonds: a bond's level is
    // one more than the highest level of the earlier bonds sharing an atom
    // with it; the bonds then go level by level, in the reference's order
    // within a level
    std::vector<int2> atoms;
    std::vector<double> req;
    std::vector<int> level_start, sys_level(nsys + 1);
    for (int s = 0; s < nsys; s++) {
      const HostSystem &hs = host_[s];
      const int nb = rattle_bonds(s), ao = 3 * sys_[s].atom_off;
      std::vector<int> last(hs.natom, 0), lev(nb);
      int nlev = 0;
      for (int k = 0; k < nb; k++) {
        const HostSystem::Bond &b = hs.rattle_bonds[k];
        const int l = std::max(last[b.a], last[b.b]);
        lev[k] = l;
        last[b.a] = last[b.b] = l + 1;
        nlev = std::max(nlev, l + 1);
      }
      std::vector<int> start(nlev + 1, 0);
      for (int k = 0; k < nb; k++) start[lev[k] + 1]++;
      for (int l = 0; l < nlev; l++) start[l + 1] += start[l];
      const int base = static_cast<int>(atoms.size());
      sys_level[s] = static_cast<int>(level_start.size());
      for (int l = 0; l < nlev; l++) level_start.push_back(base + start[l]);
      atoms.resize(base + nb);
      req.resize(base + nb);
      for (int k = 0; k < nb; k++) {
        const HostSystem::Bond &b = hs.rattle_bonds[k];
        const int at = base + start[lev[k]]++;
        atoms[at] = make_int2(ao + 3 * b.a, ao + 3 * b.b);
        req[at] = b.req;
      }
    }
    sys_level[nsys] = static_cast<int>(level_start.size());
    level_start.push_back(static_cast<int>(atoms.size()));
    SFFG_CK(up(d.rat_atoms, atoms));
    SFFG_CK(up(d.rat_req, req));
    SFFG_CK(up(d.rat_level, level_start));
    SFFG_CK(up(d.rat_sys_level, sys_level));
    SFFG_CK(d.rat_status.alloc(nsys));
    SFFG_CK(cudaMemset(d.rat_status.p, 0, d.rat_status.bytes()));
    SFFG_CK(d.xold.alloc(3 * static_cast<size_t>(natom_total_)));
  }
  std::vector<double> onesd(nsys, 1.0);
  SFFG_CK(cudaMemcpy(d.tscal.p, onesd.data(), nsys * sizeof(double), cudaMemcpyHostToDevice));
  {
    const bool neck = mp_.gb == 7 || mp_.gb == 8;
    occ_[0] = born_blocks_per_sm(neck, tail_poly_all_);
    occ_[1] = gbpair_blocks_per_sm(mp_.kappa != 0.0);
    occ_[2] = chain_blocks_per_sm(neck, tail_poly_all_);
    for (int p = 0; p < 3; p++) {
      cfg_[p].claim = 4;
      cfg_[p].blocks = occ_[p] * d.nsm;
    }
  }
  return SFFG_OK;
}

size_t Batch::device_bytes() const {
  if (!d_) return 0;
  const DeviceState &d = *d_;
  size_t b = 0;
  b += d.pos_hi.bytes() + d.pos_lo.bytes() + d.gbpar.bytes() + d.param.bytes() + d.slot_atom.bytes();
  b += d.q32.bytes() + d.reff32.bytes() + d.rinv2.bytes() + d.sumda32.bytes() + d.rborn64.bytes();
  b += d.q64.bytes() + d.alpha.bytes() + d.beta.bytes() + d.gamma.bytes() + d.reff64.bytes();
  b += d.psi64.bytes() + d.chainfac.bytes() + d.acc_sumi.bytes() + d.acc_sd.bytes() + d.acc_fx.bytes();
  b += d.acc_fy.bytes() + d.acc_fz.bytes() + d.x.bytes();
  b += d.cand.bytes() + d.cand_n.bytes() + d.cand_off.bytes() + d.colA.bytes() + d.colB.bytes() + d.colC.bytes() + d.colE.bytes();
  b += d.chunkA_i.bytes() + d.entA_slot.bytes() + d.entA_col.bytes() + d.entA_exc.bytes();
  b += d.chunkB_i.bytes() + d.entB_slot.bytes() + d.entB_col.bytes() + d.xb.bytes();
  b += d.chunkC_i.bytes() + d.entC_slot.bytes() + d.entC_col.bytes();
  b += d.colK.bytes() + d.entA_close.bytes();
  b += d.grad.bytes() + d.v.bytes() + d.accel.bytes() + d.minv.bytes() + d.sqrmass.bytes();
  b += d.excl_masks.bytes() + d.cg_w.bytes() + d.noise.bytes();
  b += d.bond_par.bytes() + d.angle_par.bytes() + d.dih_par.bytes() + d.p14_par.bytes();
  return b;
}

double *Batch::d_coords() { return d_ ? d_->x.p : nullptr; }
double *Batch::d_grad() { return d_ ? d_->grad.p : nullptr; }
void *Batch::default_stream() { return d_ ? d_->stream : nullptr; }

// NULL selects the legacy default stream, as documented in sffg.h.
static cudaStream_t pick(DeviceState &d, void *stream) {
  (void)d;
  return stream ? static_cast<cudaStream_t>(stream) : cudaStreamLegacy;
}

int Batch::set_coords(int s, const double *x, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_ || s < 0 || s >= num_systems()) return SFFG_EINVAL;
  const SystemInfo &si = sys_[s];
  cudaStream_t st = pick(*d_, stream);
  SFFG_CK(cudaMemcpyAsync(d_->x.p + 3 * static_cast<size_t>(si.atom_off), x, 3 * sizeof(double) * si.natom,
                          cudaMemcpyHostToDevice, st));
  SFFG_CK(cudaMemsetAsync(d_->nonfinite.p + s, 0, sizeof(int), st));
  return SFFG_OK;
}

static int copy_out(Batch &b, DeviceState &d, double *dev, int s, double *host, int per_atom,
                    void *stream, std::string &err) {
  const SystemInfo &si = b.system(s);
  cudaStream_t st = pick(d, stream);
  cudaError_t e = cudaMemcpyAsync(host, dev + static_cast<size_t>(per_atom) * si.atom_off,
                                  per_atom * sizeof(double) * si.natom, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    err = cudaGetErrorString(e);
    return SFFG_ECUDA;
  }
  return SFFG_OK;
}

int Batch::get_coords(int s, double *x, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_ || s < 0 || s >= num_systems()) return SFFG_EINVAL;
  return copy_out(*this, *d_, d_->x.p, s, x, 3, stream, last_error);
}

int Batch::get_grad(int s, double *g, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_ || s < 0 || s >= num_systems()) return SFFG_EINVAL;
  return copy_out(*this, *d_, d_->grad.p, s, g, 3, stream, last_error);
}

int Batch::set_velocities(int s, const double *v, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_ || s < 0 || s >= num_systems()) return SFFG_EINVAL;
  const SystemInfo &si = sys_[s];
  SFFG_CK(cudaMemcpyAsync(d_->v.p + 3 * static_cast<size_t>(si.atom_off), v, 3 * sizeof(double) * si.natom,
                          cudaMemcpyHostToDevice, pick(*d_, stream)));
  return SFFG_OK;
}

int Batch::get_velocities(int s, double *v, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_ || s < 0 || s >= num_systems()) return SFFG_EINVAL;
  return copy_out(*this, *d_, d_->v.p, s, v, 3, stream, last_error);
}

int Batch::get_reff(int s, double *reff, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_ || s < 0 || s >= num_systems()) return SFFG_EINVAL;
  const SystemInfo &si = sys_[s];
  std::vector<double> r(static_cast<size_t>(si.ntile) * 32);
  cudaStream_t st = pick(*d_, stream);
  SFFG_CK(cudaMemcpyAsync(r.data(), d_->reff64.p + si.slot_off, r.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  std::vector<int> sa(r.size());
  SFFG_CK(cudaMemcpyAsync(sa.data(), d_->slot_atom.p + si.slot_off, sa.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaStreamSynchronize(st));
  for (size_t k = 0; k < r.size(); k++)
    if (sa[k] >= 0) reff[sa[k] - si.atom_off] = r[k];
  return SFFG_OK;
}

static void ene_from_fixed(const long long *e, double *ene) {
  const double k = 1.0 / kEnergyScale;
  for (int i = 0; i < 13; i++) ene[i] = 0.0;
  ene[1] = e[E_EVDW] * k;
  ene[2] = e[E_EEL] * k;
  ene[3] = e[E_BOND] * k;
  ene[4] = e[E_ANGLE] * k;
  ene[5] = e[E_DIHED] * k;
  ene[7] = e[E_ENB14] * k;
  ene[8] = e[E_EEL14] * k;
  ene[9] = e[E_CONS] * k;
  ene[10] = e[E_EGB] * k;
  for (int i = 1; i <= 12; i++) ene[0] += ene[i];
}

int Batch::get_energy(int s, double *ene, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_ || s < 0 || s >= num_systems()) return SFFG_EINVAL;
  long long e[kEnergySlots];
  cudaStream_t st = pick(*d_, stream);
  SFFG_CK(cudaMemcpyAsync(e, d_->energy.p + kEnergySlots * s, sizeof(e), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaStreamSynchronize(st));
  ene_from_fixed(e, ene);
  return SFFG_OK;
}

int Batch::get_energy_grad(int s, double *ene, double *g, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_ || s < 0 || s >= num_systems()) return SFFG_EINVAL;
  const SystemInfo &si = sys_[s];
  long long e[kEnergySlots];
  cudaStream_t st = pick(*d_, stream);
  SFFG_CK(cudaMemcpyAsync(g, d_->grad.p + 3 * static_cast<size_t>(si.atom_off), 3 * sizeof(double) * si.natom,
                          cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaMemcpyAsync(e, d_->energy.p + kEnergySlots * s, sizeof(e), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaStreamSynchronize(st));
  ene_from_fixed(e, ene);
  return SFFG_OK;
}

int Batch::set_all_coords(const double *x, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_) return SFFG_ESTATE;
  cudaStream_t st = pick(*d_, stream);
  SFFG_CK(cudaMemcpyAsync(d_->x.p, x, 3 * sizeof(double) * natom_total_, cudaMemcpyHostToDevice, st));
  SFFG_CK(cudaMemsetAsync(d_->nonfinite.p, 0, d_->nonfinite.bytes(), st));
  return SFFG_OK;
}

namespace {
constexpr char kStateMagic[8] = {'S', 'F', 'F', 'G', 'M', 'D', '1', 0};
}

int Batch::save_state(const char *path, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_) return SFFG_ESTATE;
  DeviceState &d = *d_;
  cudaStream_t st = pick(d, stream);
  const size_t n3 = 3 * static_cast<size_t>(natom_total_), nsys = num_systems();
  std::vector<double> buf(3 * n3 + nsys);
  SFFG_CK(cudaMemcpyAsync(buf.data(), d.x.p, n3 * sizeof(double), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaMemcpyAsync(buf.data() + n3, d.v.p, n3 * sizeof(double), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaMemcpyAsync(buf.data() + 2 * n3, d.accel.p, n3 * sizeof(double), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaMemcpyAsync(buf.data() + 3 * n3, d.tscal.p, nsys * sizeof(double), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaStreamSynchronize(st));
  FILE *fp = std::fopen(path, "wb");
  if (!fp) {
    last_error = std::string("save_state: cannot open ") + path;
    return SFFG_EINVAL;
  }
  const long long hdr[2] = {natom_total_, static_cast<long long>(nsys)};
  bool ok = std::fwrite(kStateMagic, 1, 8, fp) == 8 && std::fwrite(hdr, sizeof(hdr), 1, fp) == 1 &&
            std::fwrite(buf.data(), sizeof(double), buf.size(), fp) == buf.size();
  ok = (std::fclose(fp) == 0) && ok;
  if (!ok) {
    last_error = std::string("save_state: write failed: ") + path;
    return SFFG_EINVAL;
  }
  return SFFG_OK;
}

int Batch::load_state(const char *path, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_) return SFFG_ESTATE;
  DeviceState &d = *d_;
  cudaStream_t st = pick(d, stream);
  const size_t n3 = 3 * static_cast<size_t>(natom_total_), nsys = num_systems();
  FILE *fp = std::fopen(path, "rb");
  if (!fp) {
    last_error = std::string("load_state: cannot open ") + path;
    return SFFG_EINVAL;
  }
  char magic[8] = {};
  long long hdr[2] = {0, 0};
  std::vector<double> buf(3 * n3 + nsys);
  bool ok = std::fread(magic, 1, 8, fp) == 8 && std::memcmp(magic, kStateMagic, 8) == 0 &&
            std::fread(hdr, sizeof(hdr), 1, fp) == 1 && hdr[0] == natom_total_ &&
            hdr[1] == static_cast<long long>(nsys) && std::fread(buf.data(), sizeof(double), buf.size(), fp) == buf.size();
  std::fclose(fp);
  if (!ok) {
    last_error = std::string("load_state: not a state of this batch: ") + path;
    return SFFG_EINVAL;
  }
  SFFG_CK(cudaMemcpyAsync(d.x.p, buf.data(), n3 * sizeof(double), cudaMemcpyHostToDevice, st));
  SFFG_CK(cudaMemcpyAsync(d.v.p, buf.data() + n3, n3 * sizeof(double), cudaMemcpyHostToDevice, st));
  SFFG_CK(cudaMemcpyAsync(d.accel.p, buf.data() + 2 * n3, n3 * sizeof(double), cudaMemcpyHostToDevice, st));
  SFFG_CK(cudaMemcpyAsync(d.tscal.p, buf.data() + 3 * n3, nsys * sizeof(double), cudaMemcpyHostToDevice, st));
  SFFG_CK(cudaMemsetAsync(d.ekin.p, 0, d.ekin.bytes(), st));
  SFFG_CK(cudaMemsetAsync(d.nonfinite.p, 0, d.nonfinite.bytes(), st));
  SFFG_CK(cudaStreamSynchronize(st));  // the staging buffer goes out of scope
  return run_eval(true, stream);
}

int Batch::system_status(std::vector<int> &status, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_) return SFFG_ESTATE;
  const int nsys = num_systems();
  std::vector<int> bad(nsys);
  cudaStream_t st = pick(*d_, stream);
  std::vector<int> rat(nsys, 0);
  SFFG_CK(cudaMemcpyAsync(bad.data(), d_->nonfinite.p, nsys * sizeof(int), cudaMemcpyDeviceToHost, st));
  if (d_->rat_status.p)
    SFFG_CK(cudaMemcpyAsync(rat.data(), d_->rat_status.p, nsys * sizeof(int), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaStreamSynchronize(st));
  status.resize(nsys);
  for (int s = 0; s < nsys; s++) status[s] = bad[s] ? SFFG_ENONFINITE : rat[s] ? SFFG_ECONSTRAINT : SFFG_OK;
  return SFFG_OK;
}

int Batch::set_all_active(const std::vector<int> &on, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_ || static_cast<int>(on.size()) != num_systems()) return SFFG_EINVAL;
  note_active(on);
  SFFG_CK(cudaMemcpyAsync(d_->sys_active.p, ones_.data(), ones_.size() * sizeof(int), cudaMemcpyHostToDevice,
                          pick(*d_, stream)));
  return SFFG_OK;
}

int Batch::get_all_energy_grad(std::vector<double> &out, double *grad, void *stream, std::vector<int> *status) {
  SFFG_SETTLE(stream);
  if (!finalized_) return SFFG_ESTATE;
  const int nsys = num_systems();
  std::vector<long long> e(kEnergySlots * static_cast<size_t>(nsys));
  std::vector<int> bad(status ? nsys : 0);
  cudaStream_t st = pick(*d_, stream);
  SFFG_CK(cudaMemcpyAsync(grad, d_->grad.p, 3 * sizeof(double) * natom_total_, cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaMemcpyAsync(e.data(), d_->energy.p, e.size() * sizeof(long long), cudaMemcpyDeviceToHost, st));
  if (status)
    SFFG_CK(cudaMemcpyAsync(bad.data(), d_->nonfinite.p, nsys * sizeof(int), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaStreamSynchronize(st));
  out.resize(13 * static_cast<size_t>(nsys));
  for (int s = 0; s < nsys; s++) ene_from_fixed(&e[kEnergySlots * s], &out[13 * s]);
  if (status) {
    status->resize(nsys);
    for (int s = 0; s < nsys; s++) (*status)[s] = bad[s] ? SFFG_ENONFINITE : SFFG_OK;
  }
  return SFFG_OK;
}

int Batch::get_all_energies(std::vector<double> &out, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_) return SFFG_ESTATE;
  const int nsys = num_systems();
  std::vector<long long> e(kEnergySlots * static_cast<size_t>(nsys));
  cudaStream_t st = pick(*d_, stream);
  SFFG_CK(cudaMemcpyAsync(e.data(), d_->energy.p, e.size() * sizeof(long long), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaStreamSynchronize(st));
  out.resize(13 * static_cast<size_t>(nsys));
  for (int s = 0; s < nsys; s++) ene_from_fixed(&e[kEnergySlots * s], &out[13 * s]);
  return SFFG_OK;
}

DevTables make_tables(DeviceState &d, const ModelParams &mp, int queue) {
  DevTables t;
  t.pos_hi = d.pos_hi.p;
  t.pos_lo = d.pos_lo.p;
  t.gbpar = d.gbpar.p;
  t.param = d.param.p;
  t.reff32 = d.reff32.p;
  t.rinv2 = d.rinv2.p;
  t.sumda32 = d.sumda32.p;
  t.tile_sys = d.tile_sys.p;
  t.box_lo = d.box_lo.p;
  t.box_hi = d.box_hi.p;
  t.sys_active = d.sys_active.p;
  t.sys_lj_off = d.sys_lj_off.p;
  t.sys_ntypes = d.sys_ntypes.p;
  t.sys_born = d.sys_born.p;
  t.lj = d.lj.p;
  t.lj64 = d.lj64.p;
  t.lj_n = static_cast<int>(d.lj.n);
  t.nslot = static_cast<int>(d.pos_hi.n);
  t.ntile = static_cast<int>(d.tile_sys.n);
  t.la.chunk_i = d.chunkA_i.p;
  t.la.slot = d.entA_slot.p;
  t.la.col = d.entA_col.p;
  t.la.exc = d.entA_exc.p;
  t.la.close = d.entA_close.p;
  t.la.nchunk = d.counters.p + 2;
  t.lb.chunk_i = d.chunkB_i.p;
  t.lb.slot = d.entB_slot.p;
  t.lb.col = d.entB_col.p;
  t.lb.exc = nullptr;
  t.lb.close = nullptr;
  t.lb.nchunk = d.counters.p + 3;
  t.lc.chunk_i = d.chunkC_i.p;
  t.lc.slot = d.entC_slot.p;
  t.lc.col = d.entC_col.p;
  t.lc.exc = nullptr;
  t.lc.close = nullptr;
  t.lc.nchunk = d.counters.p + 10;
  t.counter = d.counters.p + queue;
  t.acc_sumi = d.acc_sumi.p;
  t.acc_sd = d.acc_sd.p;
  t.acc_fx = d.acc_fx.p;
  t.acc_fy = d.acc_fy.p;
  t.acc_fz = d.acc_fz.p;
  t.energy = d.energy.p;
  t.born.rgbmax = static_cast<float>(mp.rgbmax);
  t.born.rgbmax1i = static_cast<float>(1.0 / mp.rgbmax);
  t.born.rgbmax2i = static_cast<float>(1.0 / (mp.rgbmax * mp.rgbmax));
  t.born.cutoff2 = 0.0f;  // per system: sys_born
  t.pair.kappa_s = static_cast<float>(mp.kappa * kKscale);
  t.pair.inv_epsext = static_cast<float>(1.0 / mp.epsext);
  t.pair.dielfac0 = static_cast<float>(1.0 - 1.0 / mp.epsext);
  t.neck_scale = static_cast<float>(mp.gbneckscale);
  t.neck_pos = d.neck_pos.p;
  t.neck_val = d.neck_val.p;
  return t;
}

namespace {

template <class T>
cudaError_t ensure(DBuf<T> &b, size_t n) {
  if (b.n >= n) return cudaSuccess;
  return b.alloc(std::max(n, b.n + b.n / 4));
}

}  // namespace

ListArgs Batch::list_args() {
  DeviceState &d = *d_;
  ListArgs a;
  a.pos_hi = d.pos_hi.p;
  a.pos_lo = d.pos_lo.p;
  a.box_lo = d.box_lo.p;
  a.box_hi = d.box_hi.p;
  a.x = d.x.p;
  a.slot_atom = d.slot_atom.p;
  a.param = d.param.p;
  a.tile_valid = d.tile_valid.p;
  a.tile_sys = d.tile_sys.p;
  a.sys_tile_end = d.sys_tile_end.p;
  a.sys_active = d.sys_active.p;
  a.excl_tile_start = d.excl_tile_start.p;
  a.excl_tile_j = d.excl_tile_j.p;
  a.excl_tile_idx = d.excl_tile_idx.p;
  a.excl_masks = d.excl_masks.p;
  a.ntile = ntile_;
  a.cut2f = static_cast<float>(mp_.cut * mp_.cut);
  a.cut2 = mp_.cut * mp_.cut;
  a.sys_gbb2 = d.sys_gbb2.p;
  a.cand = d.cand.p;
  a.cand_cap = static_cast<int>(d.cand.n);
  a.ent_cap = static_cast<int>(std::min<size_t>(d.entA_slot.n / 32, 0x7fffffff));
  a.ncand = d.counters.p + 0;
  a.overflow = d.counters.p + 1;
  a.chunks_needed = d.counters.p + 12;
  a.cand_start = d.cand_start.p;
  a.cand_count = d.cand_count.p;
  a.colA = d.colA.p;
  a.colB = d.colB.p;
  a.colC = d.colC.p;
  a.colK = d.colK.p;
  a.colE = d.colE.p;
  a.gbpar = d.gbpar.p;
  a.cand_n = d.cand_n.p;
  a.cand_off = d.cand_off.p;
  a.chunksA = d.chunksA.p;
  a.chunksB = d.chunksB.p;
  a.chunk0A = d.chunk0A.p;
  a.chunk0B = d.chunk0B.p;
  a.chunksC = d.chunksC.p;
  a.chunk0C = d.chunk0C.p;
  a.nchunkA = d.counters.p + 2;
  a.nchunkB = d.counters.p + 3;
  a.nchunkC = d.counters.p + 10;
  a.chunkA_i = d.chunkA_i.p;
  a.entA_slot = d.entA_slot.p;
  a.entA_col = d.entA_col.p;
  a.entA_exc = d.entA_exc.p;
  a.entA_close = d.entA_close.p;
  a.close2f = (kClose + 1.0f) * (kClose + 1.0f);
  a.chunkB_i = d.chunkB_i.p;
  a.entB_slot = d.entB_slot.p;
  a.entB_col = d.entB_col.p;
  a.chunkC_i = d.chunkC_i.p;
  a.entC_slot = d.entC_slot.p;
  a.entC_col = d.entC_col.p;
  a.flagB = d.counters.p + 4;
  a.tile_flagB = d.tile_flagB.p;
  a.xb = d.xb.p;
  return a;
}

// The pair lists from the current coordinates (lists.cuh, stages 1-6).
// Synchronous form: the host reads two counts back (candidates, chunks) to
// size the stores exactly; the first build, and any build asked to, takes
// it.  Queued form (build_lists_queued), while queued_builds_ is set: no
// host round trip.
int Batch::build_lists(void *stream) {
  Range range("sffg list build");
  DeviceState &d = *d_;
  cudaStream_t st = pick(d, stream);
  if (queued_builds_ && sized_ && !force_sync_build_) return build_lists_queued(st);
  force_sync_build_ = false;
  const int tile_blocks = (ntile_ * 32 + 255) / 256;
  if (d.cand.n == 0) SFFG_CK(d.cand.alloc(static_cast<size_t>(std::min<long long>(cand_max_, 64LL * ntile_ + 1024))));
  int c[2] = {0, 0};
  for (int attempt = 0;; attempt++) {
    SFFG_CK(cudaMemsetAsync(d.counters.p, 0, 2 * sizeof(int), st));
    k_list_candidates<<<tile_blocks, 256, 0, st>>>(list_args());
    SFFG_CK(cudaGetLastError());
    launches_++;
    SFFG_CK(cudaMemcpyAsync(c, d.counters.p, sizeof(c), cudaMemcpyDeviceToHost, st));
    SFFG_CK(cudaStreamSynchronize(st));
    // the store keeps at least 25% headroom (the queued builds' margin):
    // below it, it is grown to 150% of the count and the stage runs again
    const long long keep = std::min<long long>(cand_max_, c[0] + c[0] / 4 + 512);
    if (!c[1] && static_cast<long long>(d.cand.n) >= keep) break;
    if (attempt >= 3) {
      last_error = "pair list build did not fit";
      return SFFG_ENOMEM;
    }
    SFFG_CK(d.cand.alloc(static_cast<size_t>(std::min<long long>(cand_max_, c[0] + c[0] / 2 + 1024))));
  }
  ncand_ = c[0];
  // the column stores hold as many candidates as the candidate store
  const size_t nc = std::max<size_t>(1, d.cand.n);
  SFFG_CK(ensure(d.colA, nc * 32));
  SFFG_CK(ensure(d.colB, nc * 32));
  SFFG_CK(ensure(d.colC, nc * 32));
  SFFG_CK(ensure(d.colK, nc * 32));
  SFFG_CK(ensure(d.colE, nc * 32));
  SFFG_CK(ensure(d.cand_n, nc));
  SFFG_CK(ensure(d.cand_off, nc));
  const int cand_blocks = static_cast<int>(std::min<long long>((static_cast<long long>(nc) * 32 + 255) / 256, 16LL * d.nsm));
  {
    ListArgs a = list_args();
    a.ent_cap = 0x7fffffff;  // the entry stores are sized below, from the count
    k_list_columns<false><<<cand_blocks, 256, 0, st>>>(a);
    k_list_offsets<false><<<tile_blocks, 256, 0, st>>>(a);
    k_list_scan<false><<<1, 1024, 0, st>>>(a);
    SFFG_CK(cudaGetLastError());
    launches_ += 3;
  }
  int nch = 0;
  SFFG_CK(cudaMemcpyAsync(&nch, d.counters.p + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaStreamSynchronize(st));
  // lists B and C are subsets of list A: the same capacity serves all
  // three, also when B and C are remade later; 25% headroom at least
  // (below it, 50%), the queued builds' margin
  const size_t keep_ne = static_cast<size_t>(nch + nch / 4 + 32) * 32;
  const size_t ne = d.entA_slot.n >= keep_ne ? d.entA_slot.n : static_cast<size_t>(nch + nch / 2 + 64) * 32;
  SFFG_CK(ensure(d.entA_slot, ne));
  SFFG_CK(ensure(d.entA_col, ne));
  SFFG_CK(ensure(d.entA_exc, ne));
  SFFG_CK(ensure(d.entA_close, ne));
  SFFG_CK(ensure(d.entB_slot, ne));
  SFFG_CK(ensure(d.entB_col, ne));
  SFFG_CK(ensure(d.chunkA_i, ne / 32));
  SFFG_CK(ensure(d.chunkB_i, ne / 32));
  SFFG_CK(ensure(d.entC_slot, ne));
  SFFG_CK(ensure(d.entC_col, ne));
  SFFG_CK(ensure(d.chunkC_i, ne / 32));
  {
    const ListArgs a = list_args();
    k_list_fill<false><<<cand_blocks, 256, 0, st>>>(a);
    k_list_pad<false><<<tile_blocks, 256, 0, st>>>(a);
    k_list_done<<<(a.ntile + 255) / 256, 256, 0, st>>>(a.flagB, a.tile_flagB, a.ntile);
    SFFG_CK(cudaGetLastError());
    launches_ += 3;
  }
  have_list_ = true;
  list_builds_++;
  last_ncand_ = ncand_;
  last_nch_ = nch;
  sized_ = true;
  return SFFG_OK;
}

// The queued form: the stores keep 50% headroom over the last known counts
// (growing them here if need be), all six stages launch at once, and the
// stages check the stores' capacities themselves (lists.cuh): a store too
// small sets the overflow flag, and the lists come out empty.  The counters
// then go to pinned host memory behind an event; resolve_list_check() reads
// them.  Callers that queue a build check it before trusting the results
// (eval_checked, md_steps).
int Batch::build_lists_queued(cudaStream_t st) {
  DeviceState &d = *d_;
  const int tile_blocks = (ntile_ * 32 + 255) / 256;
  // grown (to 150% of the last count) only once the headroom falls below
  // 25%: a store that moves frees the old one, which waits for the device,
  // and every captured graph must be captured again
  const long long keep_cand = std::min<long long>(cand_max_, last_ncand_ + last_ncand_ / 4 + 512);
  if (static_cast<long long>(d.cand.n) < keep_cand)
    SFFG_CK(d.cand.alloc(static_cast<size_t>(std::min<long long>(cand_max_, last_ncand_ + last_ncand_ / 2 + 1024))));
  const size_t nc = std::max<size_t>(1, d.cand.n);
  // the column stores hold as many candidates as the candidate store
  SFFG_CK(ensure(d.colA, nc * 32));
  SFFG_CK(ensure(d.colB, nc * 32));
  SFFG_CK(ensure(d.colC, nc * 32));
  SFFG_CK(ensure(d.colK, nc * 32));
  SFFG_CK(ensure(d.colE, nc * 32));
  SFFG_CK(ensure(d.cand_n, nc));
  SFFG_CK(ensure(d.cand_off, nc));
  const size_t keep_ne = static_cast<size_t>(last_nch_ + last_nch_ / 4 + 32) * 32;
  const size_t ne = d.entA_slot.n >= keep_ne ? d.entA_slot.n : static_cast<size_t>(last_nch_ + last_nch_ / 2 + 64) * 32;
  SFFG_CK(ensure(d.entA_slot, ne));
  SFFG_CK(ensure(d.entA_col, ne));
  SFFG_CK(ensure(d.entA_exc, ne));
  SFFG_CK(ensure(d.entA_close, ne));
  SFFG_CK(ensure(d.entB_slot, ne));
  SFFG_CK(ensure(d.entB_col, ne));
  SFFG_CK(ensure(d.chunkA_i, ne / 32));
  SFFG_CK(ensure(d.chunkB_i, ne / 32));
  SFFG_CK(ensure(d.entC_slot, ne));
  SFFG_CK(ensure(d.entC_col, ne));
  SFFG_CK(ensure(d.chunkC_i, ne / 32));
  if (!d.list_ev) SFFG_CK(cudaEventCreateWithFlags(&d.list_ev, cudaEventDisableTiming));
  if (!d.list_host) SFFG_CK(cudaHostAlloc(reinterpret_cast<void **>(&d.list_host), 16 * sizeof(int), cudaHostAllocDefault));
  // the smallest store of each kind sets the capacity the stages check
  ListArgs a = list_args();
  a.cand_cap = static_cast<int>(std::min({d.cand.n, d.cand_n.n, d.cand_off.n, d.colA.n / 32, d.colB.n / 32,
                                          d.colC.n / 32, d.colK.n / 32, d.colE.n / 32}));
  a.ent_cap = static_cast<int>(std::min({d.entA_slot.n, d.entA_col.n, d.entA_exc.n, d.entA_close.n, d.entB_slot.n,
                                         d.entB_col.n, d.entC_slot.n, d.entC_col.n, d.chunkA_i.n * 32,
                                         d.chunkB_i.n * 32, d.chunkC_i.n * 32}) / 32);
  const int cand_blocks = static_cast<int>(std::min<long long>((static_cast<long long>(nc) * 32 + 255) / 256, 16LL * d.nsm));
  SFFG_CK(cudaMemsetAsync(d.counters.p, 0, 2 * sizeof(int), st));
  k_list_candidates<<<tile_blocks, 256, 0, st>>>(a);
  launch_pdl(k_list_columns<false>, cand_blocks, 256, st, a);
  launch_pdl(k_list_offsets<false>, tile_blocks, 256, st, a);
  launch_pdl(k_list_scan<false>, 1, 1024, st, a);
  launch_pdl(k_list_fill<false>, cand_blocks, 256, st, a);
  launch_pdl(k_list_pad<false>, tile_blocks, 256, st, a);
  launch_pdl(k_list_done, (a.ntile + 255) / 256, 256, st, a.flagB, a.tile_flagB, a.ntile);
  SFFG_CK(cudaGetLastError());
  launches_ += 7;
  SFFG_CK(cudaMemcpyAsync(d.list_host, d.counters.p, 16 * sizeof(int), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaEventRecord(d.list_ev, st));
  list_check_pending_ = true;
  have_list_ = true;
  list_builds_++;
  return SFFG_OK;
}

// Reads the counters of the last queued list build (waiting for them if
// need be): overflowed when a store was too small.  The counts seen update
// the ones the next queued build sizes its stores from.
std::atomic<long long> g_list_overflows{0};

int Batch::resolve_list_check(bool *overflowed) {
  *overflowed = false;
  if (!list_check_pending_) return SFFG_OK;
  DeviceState &d = *d_;
  SFFG_CK(cudaEventSynchronize(d.list_ev));
  list_check_pending_ = false;
  const int *c = d.list_host;
  *overflowed = c[1] != 0;
  if (*overflowed) g_list_overflows++;
  // counters[0]: candidates wanted (also when they did not fit); [12]: the
  // chunks list A needed (written when the candidates fitted)
  last_ncand_ = std::max<long long>(c[0], *overflowed ? last_ncand_ : 0);
  if (!*overflowed) ncand_ = c[0];
  last_nch_ = std::max<long long>(c[12], *overflowed ? last_nch_ : 0);
  return SFFG_OK;
}

// Settles a queued list build: when it overflowed (its lists came out
// empty), md steps taken since its snapshot are replayed from the snapshot
// with a synchronous build; otherwise the snapshot is dropped.
int Batch::settle_md(cudaStream_t st) {
  DeviceState &d = *d_;
  bool ovf = false;
  int rc = resolve_list_check(&ovf);
  if (rc) return rc;
  if (!ovf) {
    md_ckpt_valid_ = false;
    return SFFG_OK;
  }
  if (!md_ckpt_valid_) {
    // no snapshot (cannot happen: queued builds come from eval_checked,
    // which resolves its own, or md_steps, which takes one): rebuild next
    have_list_ = false;
    return SFFG_OK;
  }
  const size_t n3 = 3 * static_cast<size_t>(natom_total_);
  SFFG_CK(cudaMemcpyAsync(d.x.p, d.ck_x.p, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
  SFFG_CK(cudaMemcpyAsync(d.v.p, d.ck_v.p, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
  SFFG_CK(cudaMemcpyAsync(d.accel.p, d.ck_accel.p, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
  SFFG_CK(cudaMemcpyAsync(d.tscal.p, d.ck_tscal.p, d.tscal.bytes(), cudaMemcpyDeviceToDevice, st));
  SFFG_CK(cudaMemcpyAsync(d.ekin_last.p, d.ck_ekin_last.p, d.ekin_last.bytes(), cudaMemcpyDeviceToDevice, st));
  const int from = md_ckpt_step_, nsteps = md_ckpt_steps_;
  md_ckpt_valid_ = false;
  force_sync_build_ = true;
  rc = md_steps(from, nsteps, nullptr, nullptr, st, true);
  force_sync_build_ = false;
  return rc;
}

int Batch::settle(void *stream) {
  if (!list_check_pending_ && !md_ckpt_valid_) return SFFG_OK;
  if (!d_) return SFFG_OK;
  return settle_md(pick(*d_, stream));
}

// The pinned counter buffer, its event and the md snapshot of queued list
// builds, made once before the first such build (a pinned allocation takes
// milliseconds and must not fall inside a step).
int Batch::prepare_queued_builds() {
  DeviceState &d = *d_;
  if (!d.list_ev) SFFG_CK(cudaEventCreateWithFlags(&d.list_ev, cudaEventDisableTiming));
  if (!d.list_host) SFFG_CK(cudaHostAlloc(reinterpret_cast<void **>(&d.list_host), 16 * sizeof(int), cudaHostAllocDefault));
  const size_t n3 = 3 * static_cast<size_t>(natom_total_);
  if (d.ck_x.n < n3) {
    SFFG_CK(d.ck_x.alloc(n3));
    SFFG_CK(d.ck_v.alloc(n3));
    SFFG_CK(d.ck_accel.alloc(n3));
  }
  if (d.ck_tscal.n < d.tscal.n) SFFG_CK(d.ck_tscal.alloc(d.tscal.n));
  if (d.ck_ekin_last.n < d.ekin_last.n) SFFG_CK(d.ck_ekin_last.alloc(d.ekin_last.n));
  return SFFG_OK;
}

int Batch::eval_checked(bool rebuild, void *stream) {
  int rc = settle(stream);
  if (rc) return rc;
  if (!rebuild || !sized_ || !finalized_) return eval(rebuild, stream);
  if ((rc = prepare_queued_builds())) return rc;
  queued_builds_ = true;
  rc = eval(true, stream);
  queued_builds_ = false;
  if (rc) return rc;
  bool ovf = false;
  if ((rc = resolve_list_check(&ovf))) return rc;
  if (ovf) {  // a store was too small: again, with the stores sized exactly
    force_sync_build_ = true;
    rc = eval(true, stream);
    force_sync_build_ = false;
  }
  return rc;
}

// Remakes list B from list A when k_pack found an atom that moved too far
// since list B was made; every launch returns at once otherwise.
void Batch::rebuild_list_b(void *stream) {
  DeviceState &d = *d_;
  cudaStream_t st = pick(d, stream);
  const int tile_blocks = (ntile_ * 32 + 255) / 256;
  const int cand_blocks = 16 * d.nsm;  // grid-stride over the candidates (fixed, for graph capture)
  const ListArgs a = list_args();
  launch_pdl(k_list_columns<true>, cand_blocks, 256, st, a);
  launch_pdl(k_list_offsets<true>, tile_blocks, 256, st, a);
  launch_pdl(k_list_scan<true>, 1, 1024, st, a);
  launch_pdl(k_list_fill<true>, cand_blocks, 256, st, a);
  launch_pdl(k_list_pad<true>, tile_blocks, 256, st, a);
  launch_pdl(k_list_done, (a.ntile + 255) / 256, 256, st, a.flagB, a.tile_flagB, a.ntile);
  launches_ += 6;
}

int Batch::eval(bool rebuild, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_) {
    last_error = "eval before finalize";
    return SFFG_ESTATE;
  }
  return run_eval(rebuild || !have_list_, stream);
}

// The list buffers a captured graph depends on (they move when a list
// outgrows its store).
std::vector<const void *> Batch::list_sig() const {
  const DeviceState &d = *d_;
  return {d.cand.p, d.cand_n.p, d.cand_off.p, d.colA.p, d.colB.p, d.colC.p, d.colE.p, d.chunkA_i.p,
          d.entA_slot.p, d.entA_col.p, d.entA_exc.p, d.chunkB_i.p, d.entB_slot.p, d.entB_col.p, d.chunkC_i.p,
          d.colK.p, d.entA_close.p, d.entC_slot.p,
          d.entC_col.p};
}

bool Batch::graphs_ok() const { return opts_.sffg_graph && !profile_ && have_list_; }

// Captures body() (launches on the batch's private stream) into exec,
// recording how many kernels one replay launches.
int Batch::capture(cudaGraphExec_t &exec, std::vector<const void *> &sig, long long &nlaunch,
                   const std::function<int(cudaStream_t)> &body) {
  DeviceState &d = *d_;
  if (exec && sig == list_sig()) return SFFG_OK;
  if (exec) {
    cudaGraphExecDestroy(exec);
    exec = nullptr;
  }
  const long long l0 = launches_;
  const long long e0 = timers().nevals;
  cudaGraph_t g = nullptr;
  SFFG_CK(cudaStreamBeginCapture(d.stream, cudaStreamCaptureModeThreadLocal));
  const int rc = body(d.stream);
  const cudaError_t ec = cudaStreamEndCapture(d.stream, &g);
  nlaunch = launches_ - l0;
  launches_ = l0;
  timers().nevals = e0;
  if (rc != SFFG_OK || ec != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    if (rc != SFFG_OK) return rc;
    last_error = std::string("graph capture: ") + cudaGetErrorString(ec);
    return SFFG_ECUDA;
  }
  const cudaError_t ei = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  if (ei != cudaSuccess) {
    exec = nullptr;
    last_error = std::string("graph instantiate: ") + cudaGetErrorString(ei);
    return SFFG_ECUDA;
  }
  sig = list_sig();
  return SFFG_OK;
}

// The autotuner of the work split: for each pair pass, how many work
// items a warp claims per grab of the queue and how many blocks run per SM.
// Every candidate runs whole evaluations (twice; best of the two counts)
// with the passes timed by events; each pass keeps its fastest candidate.
// Results do not depend on the split (fixed-point sums), so tuning changes
// speed only.  Batches under kTuneMinAtoms atoms keep the defaults.
int Batch::ensure_tuned(cudaStream_t st) {
  constexpr int kTuneMinAtoms = 20000;
  if (tuned_ || !have_list_ || profile_ || !opts_.sffg_tune || natom_total_ < kTuneMinAtoms) return SFFG_OK;
  DeviceState &d = *d_;
  tuned_ = true;
  for (auto &pe : d.tune_ev)
    for (auto &e : pe)
      if (!e) SFFG_CK(cudaEventCreate(&e));
  struct Cand {
    int claim, level;
  };
  std::vector<Cand> cands;
  for (int claim : {1, 2, 4, 8})
    for (int level = 0; level < 2; level++) cands.push_back({claim, level});
  double best[3] = {1e30, 1e30, 1e30};
  PassCfg pick_cfg[3] = {cfg_[0], cfg_[1], cfg_[2]};
  tuning_ = true;
  const long long l0 = launches_, e0 = timers().nevals;
  int rc = SFFG_OK;
  for (int round = 0; round < 2 && rc == SFFG_OK; round++)
    for (const Cand &c : cands) {
      for (int p = 0; p < 3; p++) {
        cfg_[p].claim = c.claim;
        cfg_[p].blocks = std::max(1, occ_[p] - c.level) * d.nsm;
      }
      if ((rc = run_eval_direct(false, st))) break;
      if (cudaStreamSynchronize(st) != cudaSuccess) {
        rc = SFFG_ECUDA;
        break;
      }
      for (int p = 0; p < 3; p++) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, d.tune_ev[p][0], d.tune_ev[p][1]);
        if (ms < best[p]) {
          best[p] = ms;
          pick_cfg[p] = cfg_[p];
        }
      }
    }
  tuning_ = false;
  launches_ = l0;
  timers().nevals = e0;
  for (int p = 0; p < 3; p++) cfg_[p] = pick_cfg[p];
  return rc;
}

int Batch::tuned_split(int pass, int *claim, int *blocks) const {
  if (pass < 0 || pass > 2) return SFFG_EINVAL;
  *claim = cfg_[pass].claim;
  *blocks = cfg_[pass].blocks;
  return SFFG_OK;
}

// One evaluation; without a list rebuild it replays a captured graph (one
// launch instead of ~20) unless graphs are off or pass timing is on.
int Batch::run_eval(bool rebuild, void *stream) {
  Range range("sffg evaluation");
  DeviceState &d = *d_;
  cudaStream_t st = pick(d, stream);
  if (!rebuild) {
    const int rc = ensure_tuned(st);
    if (rc) return rc;
  }
  if (rebuild || !graphs_ok()) return run_eval_direct(rebuild, st);
  int rc = capture(d.g_eval, d.sig_eval, d.launches_eval,
                   [&](cudaStream_t cs) { return run_eval_direct(false, cs); });
  if (rc) return rc;
  SFFG_CK(cudaGraphLaunch(d.g_eval, st));
  launches_ += d.launches_eval;
  timers().nevals++;
  return SFFG_OK;
}

int Batch::run_eval_direct(bool rebuild, void *stream) {
  DeviceState &d = *d_;
  cudaStream_t st = pick(d, stream);
  const int nsys = num_systems();
  // k_pack also clears the pass queues' counters and the energy slots
  SFFG_CK(launch_pdl(k_pack, (nslot_ + 255) / 256, 256, st, d.x.p, d.slot_atom.p, d.q32.p, d.tile_valid.p, nslot_,
                     d.pos_hi.p, d.pos_lo.p, d.box_lo.p, d.box_hi.p, d.acc_sumi.p, d.acc_fx.p, d.acc_fy.p,
                     d.acc_fz.p, d.nonfinite.p, d.tile_sys.p, d.xb.p, kListMove * kListMove, d.counters.p + 4,
                     d.tile_flagB.p, d.counters.p + 5, d.energy.p, static_cast<int>(d.energy.n)));
  SFFG_CK(cudaGetLastError());
  // bonded and 1-4 terms (FP64) on the side stream: they need only x and the
  // zeroed accumulators, and keep the FP64 units busy while the list upkeep
  // and the FP32 pair passes run
  SFFG_CK(cudaEventRecord(d.fork_ev, st));
  SFFG_CK(cudaStreamWaitEvent(d.side, d.fork_ev, 0));
  const cudaStream_t bs = d.side;
  BondedArgs ba;
  ba.natom = natom_total_;
  ba.x = d.x.p;
  ba.atom_slot = d.atom_slot.p;
  ba.atom_sys = d.atom_sys.p;
  ba.acc_fx = d.acc_fx.p;
  ba.acc_fy = d.acc_fy.p;
  ba.acc_fz = d.acc_fz.p;
  ba.energy = d.energy.p;
  ba.sys_active = d.sys_active.p;
  auto blocks = [](size_t n) { return static_cast<int>((n + 127) / 128); };
  if (d.bond_atoms.n) k_bonds<<<blocks(d.bond_atoms.n), 128, 0, bs>>>(ba, d.bond_atoms.p, d.bond_par.p, static_cast<int>(d.bond_atoms.n));
  if (d.angle_atoms.n) k_angles<<<blocks(d.angle_atoms.n), 128, 0, bs>>>(ba, d.angle_atoms.p, d.angle_par.p, static_cast<int>(d.angle_atoms.n));
  if (d.dih_atoms.n) k_dihedrals<<<blocks(d.dih_atoms.n), 128, 0, bs>>>(ba, d.dih_atoms.p, d.dih_par.p, static_cast<int>(d.dih_atoms.n));
  if (d.p14_atoms.n) k_pairs14<<<blocks(d.p14_atoms.n), 128, 0, bs>>>(ba, d.p14_atoms.p, d.p14_par.p, static_cast<int>(d.p14_atoms.n));
  if (d.cons_w.n) {
    k_restraints<<<blocks(d.cons_w.n), 128, 0, bs>>>(ba, d.cons_w.p, d.cons_x0.p, static_cast<int>(d.cons_w.n));
    launches_++;
  }
  SFFG_CK(cudaGetLastError());
  SFFG_CK(cudaEventRecord(d.join_ev, bs));
  if (rebuild) {
    const int rc = build_lists(st);
    if (rc) return rc;
  } else {
    rebuild_list_b(st);
    SFFG_CK(cudaGetLastError());
  }
  // pass 1
  const bool neck = mp_.gb == 7 || mp_.gb == 8;
  const int ring = static_cast<int>(d.ev_head % DeviceState::kRing);
  if (profile_) {
    if (d.ev_head - d.ev_tail >= DeviceState::kRing) collect_pass_times(d, 1);
    SFFG_CK(cudaEventRecord(d.events[ring][0][0], st));
  }
  {
    DevTables t = make_tables(d, mp_, 5);
    t.claim = cfg_[0].claim;
    if (tuning_) SFFG_CK(cudaEventRecord(d.tune_ev[0][0], st));
    {
      Range range("pass 1 Born radii");
      launch_born(neck, tail_poly_all_, cfg_[0].blocks, st, t);
    }
    if (tuning_) SFFG_CK(cudaEventRecord(d.tune_ev[0][1], st));
    SFFG_CK(cudaGetLastError());
  }
  if (profile_) SFFG_CK(cudaEventRecord(d.events[ring][0][1], st));
  // Born radii, diagonal terms
  {
    FinishArgs f;
    f.acc_sumi = d.acc_sumi.p;
    f.acc_sd = d.acc_sd.p;
    f.energy = d.energy.p;
    f.slot_atom = d.slot_atom.p;
    f.tile_sys = d.tile_sys.p;
    f.sys_active = d.sys_active.p;
    f.param = d.param.p;
    f.rborn64 = d.rborn64.p;
    f.rinv64 = d.rinv64.p;
    f.q64 = d.q64.p;
    f.alpha = d.alpha.p;
    f.beta = d.beta.p;
    f.gamma = d.gamma.p;
    f.reff64 = d.reff64.p;
    f.psi64 = d.psi64.p;
    f.chainfac = d.chainfac.p;
    f.reff32 = d.reff32.p;
    f.rinv2 = d.rinv2.p;
    f.nslot = nslot_;
    f.gb = mp_.gb;
    f.gboffset = mp_.gboffset;
    f.kappa = mp_.kappa;
    f.epsext = mp_.epsext;
    launch_pdl(k_born_finish, (nslot_ + 255) / 256, 256, st, f);
    SFFG_CK(cudaGetLastError());
  }
  // pass 2
  if (profile_) SFFG_CK(cudaEventRecord(d.events[ring][1][0], st));
  {
    DevTables t = make_tables(d, mp_, 6);
    t.claim = cfg_[1].claim;
    t.lj_shared = opts_.sffg_lj_shared != 0;
    if (tuning_) SFFG_CK(cudaEventRecord(d.tune_ev[1][0], st));
    {
      Range range("pass 2 GB Coulomb LJ");
      launch_gbpair(mp_.kappa != 0.0, cfg_[1].blocks, st, t);
    }
    if (tuning_) SFFG_CK(cudaEventRecord(d.tune_ev[1][1], st));
    SFFG_CK(cudaGetLastError());
  }
  if (profile_) SFFG_CK(cudaEventRecord(d.events[ring][1][1], st));
  launch_pdl(k_chain_prep, (nslot_ + 255) / 256, 256, st, d.acc_sd.p, d.chainfac.p, d.param.p, d.slot_atom.p,
                                                     d.sumda32.p, nslot_);
  // pass 3
  if (profile_) SFFG_CK(cudaEventRecord(d.events[ring][2][0], st));
  {
    DevTables t = make_tables(d, mp_, 7);
    t.claim = cfg_[2].claim;
    if (tuning_) SFFG_CK(cudaEventRecord(d.tune_ev[2][0], st));
    {
      Range range("pass 3 chain rule");
      launch_chain(neck, tail_poly_all_, cfg_[2].blocks, st, t);
    }
    if (tuning_) SFFG_CK(cudaEventRecord(d.tune_ev[2][1], st));
    SFFG_CK(cudaGetLastError());
  }
  if (profile_) {
    SFFG_CK(cudaEventRecord(d.events[ring][2][1], st));
    d.ev_head++;
  }
  SFFG_CK(cudaStreamWaitEvent(st, d.join_ev, 0));
  // natom_total_ >= nsys: the gather's threads also cover the totals
  launch_pdl(k_gather_grad, (natom_total_ + 255) / 256, 256, st, d.acc_fx.p, d.acc_fy.p, d.acc_fz.p, d.atom_slot.p,
                                                            d.atom_frozen.p, d.atom_sys.p, d.sys_active.p,
                                                            d.grad.p, natom_total_, d.energy.p, d.etot.p, nsys);
  SFFG_CK(cudaGetLastError());
  // pack, four bonded kinds (when present), three pair kernels, Born finish,
  // chain prep, gather with the energy totals
  launches_ += 8 + (d.bond_atoms.n > 0) + (d.angle_atoms.n > 0) + (d.dih_atoms.n > 0) + (d.p14_atoms.n > 0);
  timers().nevals++;
  return SFFG_OK;
}

long long Batch::num_pairs(int s) {
  if (settle(nullptr) != SFFG_OK) return -1;
  // Count the pairs of system s on list A (the reference's list; a
  // diagnostic path, synchronous).
  if (!finalized_ || !have_list_) return -1;
  DeviceState &d = *d_;
  int nch = 0;
  if (cudaMemcpy(&nch, d.counters.p + 2, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  std::vector<int> owner(nch);
  std::vector<unsigned> col(static_cast<size_t>(nch) * 32);
  std::vector<int> tsys(ntile_);
  if (nch > 0) {
    cudaMemcpy(owner.data(), d.chunkA_i.p, owner.size() * sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(col.data(), d.entA_col.p, col.size() * sizeof(unsigned), cudaMemcpyDeviceToHost);
  }
  cudaMemcpy(tsys.data(), d.tile_sys.p, tsys.size() * sizeof(int), cudaMemcpyDeviceToHost);
  long long n = 0;
  for (int k = 0; k < nch; k++) {
    if (tsys[owner[k]] != s) continue;
    for (int l = 0; l < 32; l++) n += __builtin_popcount(col[static_cast<size_t>(k) * 32 + l]);
  }
  return n;
}

// Reads back up to max_evals of the oldest recorded evaluations (all when
// max_evals < 0).
void Batch::collect_pass_times(DeviceState &d, long long max_evals) {
  long long n = 0;
  while (d.ev_tail < d.ev_head && (max_evals < 0 || n < max_evals)) {
    const int r = static_cast<int>(d.ev_tail % DeviceState::kRing);
    for (int k = 0; k < 3; k++) {
      float ms = 0.f;
      if (cudaEventSynchronize(d.events[r][k][1]) == cudaSuccess &&
          cudaEventElapsedTime(&ms, d.events[r][k][0], d.events[r][k][1]) == cudaSuccess)
        d.pass_ms[k] += ms;
    }
    d.timed_evals++;
    d.ev_tail++;
    n++;
  }
}

int Batch::set_profiling(bool on) {
  if (!finalized_) return SFFG_ESTATE;
  DeviceState &d = *d_;
  if (on && !d.events[0][0][0]) {
    for (auto &ring : d.events)
      for (auto &pe : ring)
        for (auto &e : pe) SFFG_CK(cudaEventCreate(&e));
  }
  profile_ = on;
  return SFFG_OK;
}

int Batch::kernel_times(double ms[3], long long *nevals) {
  if (!finalized_) return SFFG_ESTATE;
  DeviceState &d = *d_;
  collect_pass_times(d, -1);
  for (int k = 0; k < 3; k++) {
    ms[k] = d.pass_ms[k];
    d.pass_ms[k] = 0.0;
  }
  if (nevals) *nevals = d.timed_evals;
  d.timed_evals = 0;
  return SFFG_OK;
}

// ------------------------------------------------------------------ md

// End of an md step: kinetic energy, the Berendsen factor of the next step
// (apply) and the Philox step counter.
// The step's kinetic sum moves to ekin_last and ekin is cleared for the
// next step's kick.
__global__ void k_md_tscal(long long *ekin, long long *ekin_last, double *tscal, double *ekin_out, int nsys,
                           double ekin0_per_dof, const double *rndf, double dttp, double c_ave_factor, int apply,
                           unsigned *step) {
  pdl_wait();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) ++*step;
  if (s >= nsys) return;
  const long long e = ekin[s];
  ekin_last[s] = e;
  ekin[s] = 0;
  double ek = 0.5 * static_cast<double>(e) * (1.0 / 4294967296.0) * c_ave_factor;
  if (ekin_out) ekin_out[s] = ek;
  if (apply) {
    const double ekin0 = ekin0_per_dof * rndf[s];
    tscal[s] = ek > 0.01 ? sqrt(1. + dttp * (ekin0 / ek - 1.)) : 1.0;
  }
}

static void md_args(Batch &b, DeviceState &d, const Options &o, int natom_total, MdArgs &a, double &c_ave) {
  const double boltz2 = 9.93595e-4;
  const double dtx = o.dt * 20.455, dt5 = 0.5 * dtx, gammai = o.gamma_ln / 20.455;
  a.x = d.x.p;
  a.v = d.v.p;
  a.accel = d.accel.p;
  a.grad = d.grad.p;
  a.minv = d.minv.p;
  a.sqrmass = d.sqrmass.p;
  a.atom_frozen = d.atom_frozen.p;
  a.atom_sys = d.atom_sys.p;
  a.sys_active = d.sys_active.p;
  a.noise = nullptr;
  a.tscal = d.tscal.p;
  a.ekin = d.ekin.p;
  a.n3 = 3 * natom_total;
  a.dtx = dtx;
  a.dt5 = dt5;
  a.c_explic = 1.0 - gammai * dt5;
  a.c_implic = 1.0 / (1.0 + gammai * dt5);
  a.sdfac = std::sqrt(4.0 * gammai * boltz2 * o.temp0 / dtx);
  a.vlimit = o.vlimit;
  a.gammai = gammai;
  a.seed = o.sffg_seed;
  a.step = d.step.p;
  a.sys_atom_off = d.sys_atom_off.p;
  a.sys_key = d.sys_key.p;
  a.xold = o.irattle ? d.xold.p : nullptr;
  c_ave = gammai > 0.0 ? 1.0 + gammai * dt5 : 1.0;
  (void)b;
}

// Uploads one step's worth of reference-stream draws (coordinate order,
// frozen atoms skipped) for every system.
static int upload_noise(Batch &b, DeviceState &d, Batch::NoiseFn noise, void *ctx, cudaStream_t st,
                        std::vector<double> &h) {
  const int nsys = b.num_systems();
  const size_t n3 = 3 * static_cast<size_t>(b.total_atoms());
  if (d.noise.n != n3 && d.noise.alloc(n3) != cudaSuccess) return SFFG_ENOMEM;
  h.assign(n3, 0.0);
  std::vector<double> draws;
  for (int s = 0; s < nsys; s++) {
    const SystemInfo &si = b.system(s);
    int cnt = 0;
    for (int i = 0; i < 3 * si.natom; i++) cnt += si.frozen[i / 3] ? 0 : 1;
    draws.resize(cnt);
    noise(ctx, s, cnt, draws.data());
    int k = 0;
    for (int i = 0; i < 3 * si.natom; i++)
      if (!si.frozen[i / 3]) h[3 * static_cast<size_t>(si.atom_off) + i] = draws[k++];
  }
  cudaError_t e = cudaMemcpyAsync(d.noise.p, h.data(), n3 * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // h is reused by the next step
  return e == cudaSuccess ? SFFG_OK : SFFG_ECUDA;
}

int Batch::md_begin(bool rebuild, NoiseFn noise, void *noise_ctx, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_) return SFFG_ESTATE;
  DeviceState &d = *d_;
  cudaStream_t st = pick(d, stream);
  MdArgs a;
  double c_ave;
  md_args(*this, d, opts_, natom_total_, a, c_ave);
  int rc = run_eval(rebuild || !have_list_, st);
  if (rc) return rc;
  std::vector<double> h;
  if (noise && a.gammai != 0.0) {
    if ((rc = upload_noise(*this, d, noise, noise_ctx, st, h))) return rc;
    a.noise = d.noise.p;
  }
  if ((rc = prepare_queued_builds())) return rc;
  SFFG_CK(cudaMemsetAsync(d.ekin.p, 0, d.ekin.bytes(), st));
  SFFG_CK(cudaMemsetAsync(d.step.p, 0, sizeof(unsigned), st));
  const int nb = (a.n3 + 255) / 256;
  k_md_kick<<<nb, 256, 0, st>>>(a, 1);
  SFFG_CK(cudaGetLastError());
  // the kinetic sum of the first kick is not a step's: each step's kick
  // starts from zero (k_md_tscal clears it afterwards)
  SFFG_CK(cudaMemcpyAsync(d.ekin_last.p, d.ekin.p, d.ekin.bytes(), cudaMemcpyDeviceToDevice, st));
  SFFG_CK(cudaMemsetAsync(d.ekin.p, 0, d.ekin.bytes(), st));
  launches_++;
  return SFFG_OK;
}

int Batch::md_com_remove(void *stream) {
  if (!finalized_) return SFFG_ESTATE;
  const int rc = settle(stream);
  if (rc) return rc;
  return md_com_remove_direct(pick(*d_, stream));
}

int Batch::md_com_remove_direct(cudaStream_t st) {
  DeviceState &d = *d_;
  k_com_remove<<<num_systems(), kComThreads, 0, st>>>(d.x.p, d.v.p, d.minv.p, d.sys_atom_off.p, d.sys_natom.p,
                                                      d.sys_active.p, opts_.gamma_ln == 0.0 || opts_.hcp != 0);
  SFFG_CK(cudaGetLastError());
  launches_++;
  return SFFG_OK;
}

int Batch::md_steps(int step0, int k, NoiseFn noise, void *noise_ctx, void *stream, bool com_at_end) {
  Range range("sffg md steps");
  if (!finalized_) return SFFG_ESTATE;
  DeviceState &d = *d_;
  cudaStream_t st = pick(d, stream);
  const int nsys = num_systems();
  MdArgs a;
  double c_ave;
  md_args(*this, d, opts_, natom_total_, a, c_ave);
  const double boltz2 = 9.93595e-4;
  std::vector<double> h;
  const int nb = (a.n3 + 255) / 256;
  int rc = SFFG_OK;
  // the step counter holds the number of the next step
  step_host_ = static_cast<unsigned>(step0 + 1);
  SFFG_CK(cudaMemcpyAsync(d.step.p, &step_host_, sizeof(unsigned), cudaMemcpyHostToDevice, st));
  // one step after the drift: evaluation, kick, kinetic energy, counter
  RattleArgs ra;
  if (opts_.irattle) {
    ra.x = d.x.p;
    ra.v = d.v.p;
    ra.xold = d.xold.p;
    ra.minv = d.minv.p;
    ra.atoms = d.rat_atoms.p;
    ra.req = d.rat_req.p;
    ra.level = d.rat_level.p;
    ra.sys_level = d.rat_sys_level.p;
    ra.sys_active = d.sys_active.p;
    ra.status = d.rat_status.p;
    ra.dt = a.dtx;
  }
  auto step_body = [&](cudaStream_t s, bool rebuild, bool capturing) -> int {
    launch_pdl(k_md_drift, nb, 256, s, a);
    if (opts_.irattle) {
      // the reference keeps the position tolerance in single precision
      ra.eps = static_cast<double>(static_cast<float>(0.0000001));
      launch_pdl(k_rattle<false>, nsys, kRattleThreads, s, ra);
      launches_++;
    }
    int r = capturing ? run_eval_direct(false, s) : run_eval(rebuild, s);
    if (r) return r;
    if (noise && a.gammai != 0.0) {
      if ((r = upload_noise(*this, d, noise, noise_ctx, s, h))) return r;
      a.noise = d.noise.p;
    }
    launch_pdl(k_md_kick, nb, 256, s, a, 0);
    if (opts_.irattle) {
      ra.eps = 0.0000001 / a.dtx;
      launch_pdl(k_rattle<true>, nsys, kRattleThreads, s, ra);
      launch_pdl(k_md_ekin, nb, 256, s, a);
      launches_ += 2;
    }
    launch_pdl(k_md_tscal, (nsys + 127) / 128, 128, s, d.ekin.p, d.ekin_last.p, d.tscal.p,
               static_cast<double *>(nullptr), nsys,
               boltz2 * opts_.temp0, static_cast<const double *>(d.rndf.p), opts_.dt / opts_.tautp, c_ave,
               a.gammai == 0.0, d.step.p);
    launches_ += 3;  // drift, kick, tscal
    SFFG_CK(cudaGetLastError());
    return SFFG_OK;
  };
  // a queued list build that has finished by now is checked without waiting
  if (list_check_pending_ && cudaEventQuery(d.list_ev) == cudaSuccess && (rc = settle_md(st))) return rc;
  for (int i = 1; i <= k; i++) {
    const int nstep = step0 + i;
    const bool rebuild = opts_.nsnb > 0 && nstep % opts_.nsnb == 0;
    // centre-of-mass motion removal every nscm steps (sff.c:2346-2351)
    const bool com = opts_.nscm > 0 && nstep % opts_.nscm == 0 && (i < k || com_at_end);
    if (rebuild && !noise && sized_ && !force_sync_build_) {
      // a rebuild step without host round trips: the previous queued build
      // is settled first, then the state this step starts from is kept, so
      // that if this build's stores prove too small the steps from here can
      // be replayed (settle_md)
      if ((rc = settle_md(st))) break;
      const size_t n3 = 3 * static_cast<size_t>(natom_total_);
      if (d.ck_x.n < n3) {
        SFFG_CK(d.ck_x.alloc(n3));
        SFFG_CK(d.ck_v.alloc(n3));
        SFFG_CK(d.ck_accel.alloc(n3));
      }
      if (d.ck_tscal.n < d.tscal.n) SFFG_CK(d.ck_tscal.alloc(d.tscal.n));
      if (d.ck_ekin_last.n < d.ekin_last.n) SFFG_CK(d.ck_ekin_last.alloc(d.ekin_last.n));
      SFFG_CK(cudaMemcpyAsync(d.ck_x.p, d.x.p, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
      SFFG_CK(cudaMemcpyAsync(d.ck_v.p, d.v.p, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
      SFFG_CK(cudaMemcpyAsync(d.ck_accel.p, d.accel.p, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
      SFFG_CK(cudaMemcpyAsync(d.ck_tscal.p, d.tscal.p, d.tscal.bytes(), cudaMemcpyDeviceToDevice, st));
      SFFG_CK(cudaMemcpyAsync(d.ck_ekin_last.p, d.ekin_last.p, d.ekin_last.bytes(), cudaMemcpyDeviceToDevice, st));
      md_ckpt_valid_ = true;
      md_ckpt_step_ = nstep - 1;
      md_ckpt_steps_ = 0;
      queued_builds_ = true;
      rc = step_body(st, true, false);
      queued_builds_ = false;
      if (rc) break;
    } else if (!rebuild && !noise && !com && graphs_ok()) {
      if ((rc = ensure_tuned(st))) break;
      if ((rc = capture(d.g_step, d.sig_step, d.launches_step, [&](cudaStream_t cs) { return step_body(cs, false, true); })))
        break;
      SFFG_CK(cudaGraphLaunch(d.g_step, st));
      launches_ += d.launches_step;
      timers().nevals++;
    } else if ((rc = step_body(st, rebuild, false))) {
      break;
    }
    if (md_ckpt_valid_) md_ckpt_steps_++;
    if (com && (rc = md_com_remove_direct(st))) break;
  }
  return rc;
}

int Batch::md_kinetic(std::vector<double> &ekin, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_) return SFFG_ESTATE;
  DeviceState &d = *d_;
  cudaStream_t st = pick(d, stream);
  const int nsys = num_systems();
  std::vector<long long> e(nsys);
  SFFG_CK(cudaMemcpyAsync(e.data(), d.ekin_last.p, nsys * sizeof(long long), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaStreamSynchronize(st));
  const double dt5 = 0.5 * opts_.dt * 20.455, gammai = opts_.gamma_ln / 20.455;
  const double c_ave = gammai > 0.0 ? 1.0 + gammai * dt5 : 1.0;
  ekin.resize(nsys);
  for (int s = 0; s < nsys; s++) ekin[s] = 0.5 * static_cast<double>(e[s]) * (1.0 / 4294967296.0) * c_ave;
  return SFFG_OK;
}

int Batch::md_set_tscal(const std::vector<double> &tscal, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_ || static_cast<int>(tscal.size()) != num_systems()) return SFFG_EINVAL;
  SFFG_CK(cudaMemcpyAsync(d_->tscal.p, tscal.data(), tscal.size() * sizeof(double), cudaMemcpyHostToDevice,
                          pick(*d_, stream)));
  return SFFG_OK;
}

// ------------------------------------------------------------------ conjgrad

namespace {

constexpr int kCgThreads = 256;

// Sum of a value over the block; every thread receives the total.
__device__ double block_sum(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  for (int k = 0; k < kCgThreads / 32; k++) t += red[k];
  return t;
}

__device__ double block_max(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(kFull, v, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double t = red[0];
  for (int k = 1; k < kCgThreads / 32; k++) t = fmax(t, red[k]);
  return t;
}

struct CgArgs {
  CgState *state;
  double *x, *g, *w;
  const double *etot;
  const int *sys_natom, *sys_atom_off;
  int *sys_active;
  int *nactive;
};

// Runs one system's copy of the reference's conjgrad() (conjgrad.c:75-263)
// from just after an evaluation up to the next evaluation request (label
// L10) or to its end (L100).  Every thread follows the same scalar control
// flow; vector loops and dot products are spread over the block.
__global__ void __launch_bounds__(kCgThreads) k_cg_post(CgArgs a) {
  pdl_wait();
  const int s = blockIdx.x;
  if (!a.sys_active[s]) return;
  __shared__ double red[kCgThreads / 32];
  CgState st = a.state[s];
  const int n = 3 * a.sys_natom[s];
  const size_t off = 3 * static_cast<size_t>(a.sys_atom_off[s]);
  double *x = a.x + off, *g = a.g + off, *w = a.w + 6 * off;
  double *wd = w, *rsdx = w + n, *rsdg = w + 2 * n, *wginit = w + 3 * n, *xopt = w + 4 * n, *gopt = w + 5 * n;
  const int maxlin = 10, mxfcon = 4;
  double f = a.etot[s];
  st.f = f;
  int label = st.niter >= 2 ? 30 : 20;
  for (int guard = 0; guard < 1000; guard++) {
    switch (label) {
      case 20:
        for (int i = threadIdx.x; i < n; i += kCgThreads) wd[i] = -g[i];
        st.iterrs = 0;
        if (st.iterc > 0) { label = 40; break; }
        // fall through
      case 30: {
        double pg = 0.0, ps = 0.0;
        for (int i = threadIdx.x; i < n; i += kCgThreads) {
          pg += wd[i] * g[i];
          ps += g[i] * g[i];
        }
        st.gnew = block_sum(pg, red);
        st.sum = block_sum(ps, red);
        bool take = false;
        if (st.niter == 1) {
          st.fmin = f;
          take = true;
        } else {
          st.fch = f - st.fmin;
          if (st.fch < 0.0 || (st.fch == 0.0 && st.gnew / st.gmin >= -1.0)) {
            st.fmin = f;
            take = true;
          }
        }
        if (take) {
          st.gsqrd = st.sum;
          st.nfopt = st.niter;
          for (int i = threadIdx.x; i < n; i += kCgThreads) {
            xopt[i] = x[i];
            gopt[i] = g[i];
          }
          if (st.sum <= st.dgrad) { label = 100; break; }
        }
        if (st.niter == st.maxiter + 1) { st.ier = -3; label = 100; break; }
        if (st.niter > 1) { label = 60; break; }
        st.dfpr = st.dfpred;
        st.stmin = st.dfpred / st.gsqrd;
      }
        // fall through
      case 40: {
        ++st.iterc;
        st.finit = f;
        double pg = 0.0;
        for (int i = threadIdx.x; i < n; i += kCgThreads) {
          wginit[i] = g[i];
          pg += wd[i] * g[i];
        }
        st.ginit = block_sum(pg, red);
        if (st.ginit >= 0.0) { st.ier = -2; label = 90; break; }
        st.gmin = st.ginit;
        st.sbound = -1.0;
        st.nfbeg = st.niter;
        st.iretry = -1;
        {
          const double q = fabs(st.dfpr / st.ginit);
          st.stepch = st.stmin <= q ? st.stmin : q;
        }
        st.stmin = 0.0;
      }
        // fall through
      case 50: {
        st.step = st.stmin + st.stepch;
        double pw = 0.0;
        for (int i = threadIdx.x; i < n; i += kCgThreads) {
          x[i] = xopt[i] + st.stepch * wd[i];
          pw = fmax(pw, fabs(x[i] - xopt[i]));
        }
        const double work = block_max(pw, red);
        if (work > 0.0) { label = 10; break; }
        if (st.niter > st.nfbeg + 1) st.ier = -1;
        if (fabs(st.gmin / st.ginit) > 0.2) st.ier = -1;
        label = 90;
        break;
      }
      case 60: {
        const double work = (st.fch + st.fch) / st.stepch - st.gnew - st.gmin;
        st.ddspln = (st.gnew - st.gmin) / st.stepch;
        if (st.niter > st.nfopt) st.sbound = st.step;
        if (st.niter <= st.nfopt) {
          if (st.gmin * st.gnew <= 0.0) st.sbound = st.stmin;
          st.stmin = st.step;
          st.gmin = st.gnew;
          st.stepch = -st.stepch;
        }
        if (st.fch != 0.0) st.ddspln += (work + work) / st.stepch;
        if (st.gmin == 0.0) { label = 90; break; }
        if (st.niter > st.nfbeg + 1) {
          if (fabs(st.gmin / st.ginit) <= 0.2) { label = 90; break; }
          if (st.niter >= st.nfopt + maxlin) { st.ier = -1; label = 90; break; }
        }
      }
        // fall through
      case 70: {
        st.stepch = (st.sbound - st.stmin) * 0.5;
        if (st.sbound < -0.5) st.stepch = st.stmin * 9.0;
        const double gspln = st.gmin + st.stepch * st.ddspln;
        if (st.gmin * gspln < 0.0) st.stepch = st.stepch * st.gmin / (st.gmin - gspln);
        label = 50;
        break;
      }
      case 80: {
        double pg = 0.0;
        for (int i = threadIdx.x; i < n; i += kCgThreads) pg += g[i] * wginit[i];
        st.sum = block_sum(pg, red);
        st.beta = (st.gsqrd - st.sum) / (st.gmin - st.ginit);
        if (fabs(st.beta * st.gmin) > st.gsqrd * 0.2) {
          ++st.iretry;
          if (st.iretry <= 0) {
            if (st.niter >= st.nfopt + maxlin) { st.ier = -1; label = 90; break; }
            label = 70;
            break;
          }
        }
        if (f < st.finit) st.iterfm = st.iterc;
        if (st.iterc >= st.iterfm + mxfcon) { st.ier = -4; label = 100; break; }
        st.dfpr = st.stmin * st.ginit;
        if (st.iretry > 0) { label = 20; break; }
        if (st.iterrs != 0 && st.iterc - st.iterrs < n && fabs(st.sum) < st.gsqrd * 0.2) {
          double pga = 0.0, pgs = 0.0;
          for (int i = threadIdx.x; i < n; i += kCgThreads) {
            pga += g[i] * rsdg[i];
            pgs += g[i] * rsdx[i];
          }
          st.gama = block_sum(pga, red) / st.gamden;
          const double gs = block_sum(pgs, red);
          if (fabs(st.beta * st.gmin + st.gama * gs) < st.gsqrd * 0.2) {
            __syncthreads();
            for (int i = threadIdx.x; i < n; i += kCgThreads) wd[i] = -g[i] + st.beta * wd[i] + st.gama * rsdx[i];
            __syncthreads();
            label = 40;
            break;
          }
        }
        st.gamden = st.gmin - st.ginit;
        for (int i = threadIdx.x; i < n; i += kCgThreads) {
          rsdx[i] = wd[i];
          rsdg[i] = g[i] - wginit[i];
          wd[i] = -g[i] + st.beta * wd[i];
        }
        __syncthreads();
        st.iterrs = st.iterc;
        label = 40;
        break;
      }
      case 90:
        if (st.niter != st.nfopt) {
          f = st.fmin;
          for (int i = threadIdx.x; i < n; i += kCgThreads) {
            x[i] = xopt[i];
            g[i] = gopt[i];
          }
          __syncthreads();
        }
        if (st.ier == 0) { label = 80; break; }
        label = 100;
        break;
      case 10:
        // request the next evaluation (the reference's L10)
        ++st.niter;
        guard = 1 << 30;
        break;
      case 100:
        st.done = 1;
        st.ret = st.ier == 0 ? st.niter : st.ier;
        guard = 1 << 30;
        break;
      default:
        st.done = 1;
        st.ret = -99;
        guard = 1 << 30;
        break;
    }
  }
  st.f = f;
  __syncthreads();
  if (threadIdx.x == 0) {
    a.state[s] = st;
    if (st.done) {
      a.sys_active[s] = 0;
      atomicSub(a.nactive, 1);
    }
  }
}

}  // namespace

// Batched conjgrad in pieces: cg_begin sets every system's state machine
// at its start; cg_turns launches n turns (evaluation + state-machine step)
// without waiting; cg_poll reads the states back; cg_end restores the
// active flags.  cg() runs them to completion.
int Batch::cg_begin(int maxiter, double rmsgrad, double dfpred, void *stream) {
  SFFG_SETTLE(stream);
  return cg_begin(std::vector<int>(num_systems(), maxiter), std::vector<double>(num_systems(), rmsgrad), dfpred,
                  stream);
}

int Batch::cg_begin(const std::vector<int> &maxiter, const std::vector<double> &rmsgrad, double dfpred,
                    void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_) return SFFG_ESTATE;
  if (static_cast<int>(maxiter.size()) != num_systems() || static_cast<int>(rmsgrad.size()) != num_systems()) {
    last_error = "cg_begin: one maxiter and rmsgrad per system";
    return SFFG_EINVAL;
  }
  DeviceState &d = *d_;
  cudaStream_t st = pick(d, stream);
  const int nsys = num_systems();
  SFFG_CK(d.cg_w.alloc(6 * 3 * static_cast<size_t>(natom_total_)));
  SFFG_CK(d.cg_state.alloc(nsys));
  SFFG_CK(d.cg_nactive.alloc(1));
  std::vector<CgState> init(nsys);
  for (int s = 0; s < nsys; s++) {
    CgState c;
    std::memset(&c, 0, sizeof(c));
    c.niter = 1;  // the reference's first ++niter at L10
    c.maxiter = maxiter[s];
    c.dgrad = rmsgrad[s] * rmsgrad[s] * 3.0 * sys_[s].natom;
    c.dfpred = dfpred;
    init[s] = c;
  }
  cg_host_.assign(init.begin(), init.end());
  SFFG_CK(cudaMemcpyAsync(d.cg_state.p, cg_host_.data(), nsys * sizeof(CgState), cudaMemcpyHostToDevice, st));
  note_active(std::vector<int>(nsys, 1));
  SFFG_CK(cudaMemcpyAsync(d.sys_active.p, ones_.data(), nsys * sizeof(int), cudaMemcpyHostToDevice, st));
  cg_list_builds_ = list_builds_;
  cg_nsys_ = nsys;
  SFFG_CK(cudaMemcpyAsync(d.cg_nactive.p, &cg_nsys_, sizeof(int), cudaMemcpyHostToDevice, st));
  cg_turn_ = 0;
  cg_maxiter_ = *std::max_element(maxiter.begin(), maxiter.end());
  return SFFG_OK;
}

int Batch::cg_turns(int n, bool first_rebuild, void *stream, const std::function<int(int)> &after_eval) {
  SFFG_SETTLE(stream);
  Range range("sffg conjgrad turns");
  DeviceState &d = *d_;
  cudaStream_t st = pick(d, stream);
  CgArgs a;
  a.state = d.cg_state.p;
  a.x = d.x.p;
  a.g = d.grad.p;
  a.w = d.cg_w.p;
  a.etot = d.etot.p;
  a.sys_natom = d.sys_natom.p;
  a.sys_atom_off = d.sys_atom_off.p;
  a.sys_active = d.sys_active.p;
  a.nactive = d.cg_nactive.p;
  for (int k = 0; k < n && cg_turn_ <= cg_maxiter_; k++, cg_turn_++) {
    const int turn = cg_turn_;
    // every active system is at evaluation turn+1, so iter = turn for all
    const bool rebuild = (turn == 0 && first_rebuild) || (turn > 0 && opts_.nsnb > 0 && turn % opts_.nsnb == 0);
    int rc = run_eval(rebuild || !have_list_, st);
    if (rc) return rc;
    if (after_eval && (rc = after_eval(turn))) return rc;
    k_cg_post<<<num_systems(), kCgThreads, 0, st>>>(a);
    SFFG_CK(cudaGetLastError());
    launches_++;
  }
  return SFFG_OK;
}

int Batch::cg_poll(int *nactive, std::vector<int> *status, std::vector<double> *energy, void *stream) {
  SFFG_SETTLE(stream);
  DeviceState &d = *d_;
  cudaStream_t st = pick(d, stream);
  const int nsys = num_systems();
  int na = 0;
  SFFG_CK(cudaMemcpyAsync(&na, d.cg_nactive.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  if (status || energy)
    SFFG_CK(cudaMemcpyAsync(cg_host_.data(), d.cg_state.p, nsys * sizeof(CgState), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaStreamSynchronize(st));
  if (cg_turn_ > cg_maxiter_) na = 0;  // every turn ran
  if (nactive) *nactive = na;
  if (status) {
    status->resize(nsys);
    for (int s = 0; s < nsys; s++) (*status)[s] = cg_host_[s].done ? cg_host_[s].ret : (na ? 0 : -3);
  }
  if (energy) {
    energy->resize(nsys);
    for (int s = 0; s < nsys; s++) (*energy)[s] = cg_host_[s].f;
  }
  return SFFG_OK;
}

int Batch::cg_export(int sys, CgCarry &c, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_ || sys < 0 || sys >= num_systems() || !d_->cg_state.p) return SFFG_ESTATE;
  DeviceState &d = *d_;
  cudaStream_t st = pick(d, stream);
  const size_t n = 3 * static_cast<size_t>(sys_[sys].natom), off = 3 * static_cast<size_t>(sys_[sys].atom_off);
  c.x.resize(n);
  c.g.resize(n);
  c.w.resize(6 * n);
  SFFG_CK(cudaMemcpyAsync(&c.st, d.cg_state.p + sys, sizeof(CgState), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaMemcpyAsync(c.x.data(), d.x.p + off, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaMemcpyAsync(c.g.data(), d.grad.p + off, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaMemcpyAsync(c.w.data(), d.cg_w.p + 6 * off, 6 * n * sizeof(double), cudaMemcpyDeviceToHost, st));
  SFFG_CK(cudaStreamSynchronize(st));
  return SFFG_OK;
}

int Batch::cg_import(int sys, const CgCarry &c, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_ || sys < 0 || sys >= num_systems() || !d_->cg_state.p || cg_turn_ != 0) return SFFG_ESTATE;
  const size_t n = 3 * static_cast<size_t>(sys_[sys].natom), off = 3 * static_cast<size_t>(sys_[sys].atom_off);
  if (c.x.size() != n || c.g.size() != n || c.w.size() != 6 * n) {
    last_error = "cg_import: state of another system size";
    return SFFG_EINVAL;
  }
  DeviceState &d = *d_;
  cudaStream_t st = pick(d, stream);
  cg_host_[sys] = c.st;
  SFFG_CK(cudaMemcpyAsync(d.cg_state.p + sys, &cg_host_[sys], sizeof(CgState), cudaMemcpyHostToDevice, st));
  SFFG_CK(cudaMemcpyAsync(d.x.p + off, c.x.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
  SFFG_CK(cudaMemcpyAsync(d.grad.p + off, c.g.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
  SFFG_CK(cudaMemcpyAsync(d.cg_w.p + 6 * off, c.w.data(), 6 * n * sizeof(double), cudaMemcpyHostToDevice, st));
  // the host vectors may go once this returns
  SFFG_CK(cudaStreamSynchronize(st));
  return SFFG_OK;
}

void Batch::adopt_split(const Batch &from) {
  if (!from.tuned_) return;
  for (int p = 0; p < 3; p++) cfg_[p] = from.cfg_[p];
  tuned_ = true;
}

int Batch::set_restraints(int sys, const int *constrained, const double *x0) {
  if (finalized_ || sys < 0 || sys >= num_systems() || !constrained || !x0) return SFFG_EINVAL;
  SystemInfo &si = sys_[sys];
  si.constrained.assign(constrained, constrained + si.natom);
  si.x0.assign(x0, x0 + 3 * static_cast<size_t>(si.natom));
  return SFFG_OK;
}

int Batch::set_noise_key(int sys, unsigned long long key) {
  if (finalized_ || sys < 0 || sys >= num_systems()) return SFFG_ESTATE;
  sys_[sys].noise_key = key;
  return SFFG_OK;
}

// List builds leave out inactive systems, so a system switched back on
// needs a rebuild before its next evaluation.
void Batch::note_active(const std::vector<int> &on) {
  ones_.resize(num_systems(), 1);
  for (size_t s = 0; s < on.size(); s++) {
    if (on[s] && !ones_[s]) have_list_ = false;
    ones_[s] = on[s];
  }
}

int Batch::set_active(int sys, bool on, void *stream) {
  SFFG_SETTLE(stream);
  if (!finalized_ || sys < 0 || sys >= num_systems()) return SFFG_EINVAL;
  DeviceState &d = *d_;
  ones_.resize(num_systems(), 1);
  if (on && !ones_[sys]) have_list_ = false;
  ones_[sys] = on ? 1 : 0;
  SFFG_CK(cudaMemcpyAsync(d.sys_active.p + sys, &ones_[sys], sizeof(int), cudaMemcpyHostToDevice, pick(d, stream)));
  return SFFG_OK;
}

int Batch::cg_end(void *stream) {
  SFFG_SETTLE(stream);
  DeviceState &d = *d_;
  cudaStream_t st = pick(d, stream);
  // a system the minimiser switched off on the device misses the list
  // rebuilds made after it ended
  if (num_systems() > 1 && list_builds_ != cg_list_builds_) have_list_ = false;
  note_active(std::vector<int>(num_systems(), 1));
  SFFG_CK(cudaMemcpyAsync(d.sys_active.p, ones_.data(), ones_.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  SFFG_CK(cudaStreamSynchronize(st));
  return SFFG_OK;
}

int Batch::cg(int maxiter, double rmsgrad, double dfpred, bool first_rebuild, std::vector<int> &status,
              std::vector<double> &energy, void *stream, const std::function<int(int)> &after_eval) {
  int rc = cg_begin(maxiter, rmsgrad, dfpred, stream);
  if (rc) return rc;
  bool first = first_rebuild;
  while (true) {
    if ((rc = cg_turns(8, first, stream, after_eval))) break;
    first = false;
    int na = 0;
    if ((rc = cg_poll(&na, nullptr, nullptr, stream))) break;
    if (na <= 0) break;
  }
  const int rc2 = cg_poll(nullptr, &status, &energy, stream);
  const int rc3 = cg_end(stream);
  return rc ? rc : (rc2 ? rc2 : rc3);
}

}  // namespace sffg

// The first failed bounds check of a build with -DSFFG_CHECKED (a
// CheckCode), 0 when none failed, -1 in the normal build.
extern "C" long long sffg_list_overflows(void) { return sffg::g_list_overflows.load(); }

extern "C" int sffg_checked_code(void) {
#ifdef SFFG_CHECKED
  int c = 0;
  cudaMemcpyFromSymbol(&c, sffg::g_check_code, sizeof(int));
  const int codes[4] = {c, sffg::pass1_check_code(), sffg::pass2_check_code(), sffg::pass3_check_code()};
  for (int k : codes)
    if (k) return k;
  return 0;
#else
  return -1;
#endif
}
