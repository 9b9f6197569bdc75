// Device kernels of the generalized-Born path (sm_103a).
//
// The three pair passes of the reference's egb() (src/sff/eff.c:1566-1733,
// 1770-2066, 2131-2405) run over compacted pair-list chunks (lists.cuh): a
// chunk is an i-tile of 32 atoms and 32 packed j-atoms with a column mask
// each.  A warp owns one chunk at a time: lane l holds i-atom l in
// registers; the 32 j-atoms are staged in shared memory and read by
// broadcast, so at step s every lane pairs its i-atom with j-atom s.  Both
// directions of each unordered pair are handled in one visit (Newton's
// third law); the j-side partial sums, spread over the 32 lanes, are folded
// with a shuffle transpose-reduction every few steps.  Per chunk the FP32
// partial sums are converted to 64-bit fixed point, so the totals do not
// depend on how chunks are scheduled.
#pragma once

#include <cstdint>

#include "gbmath.cuh"

namespace sffg {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kEnergySlots = 9;  // fixed-point energy terms per system (EnergySlot)

// One compacted pair list (built by lists.cuh).
struct ChunkList {
  const int *chunk_i;   // i-tile of each chunk
  const int *slot;      // 32 j slots per chunk
  const unsigned *col;  // per entry, bit i: the pair with lane i of the i-tile is listed
  const unsigned *exc;  // per entry, bit i: the pair is excluded from Coulomb/LJ (cutoff list)
  const int *nchunk;
};

struct DevTables {
  // per slot
  const float4 *pos_hi;   // x, y, z (high part), q
  const float4 *pos_lo;   // x, y, z (low part), 0
  const float4 *gbpar;    // rho = rborn - offset, s = fs * rho, rborn, 3 (s - fl(s)) / fl(s)
  const int *param;       // LJ type | neck index << 16 | frozen << 24
  const float *reff32;    // effective Born radius (pass 2)
  const float *rinv2;     // sqrt(log2(e)/4) / reff (pass 2)
  const float *sumda32;   // chain-rule weight (pass 3)
  // per tile
  const int *tile_sys;
  // per system
  const int *sys_active;
  const int *sys_lj_off;
  const int *sys_ntypes;
  const float2 *lj;       // (A, B) per type pair, per system blocks
  int lj_n;               // entries of lj
  bool lj_shared;         // pass 2 may stage lj in shared memory
  int nslot, ntile;       // extents, for the checked build
  // lists: la (r < cut) for pass 2; lb and lc (r < rgbmax + Fsmax + skin,
  // lc the pairs within near-field range) for passes 1 and 3
  ChunkList la, lb, lc;
  int *counter;
  int claim;  // work items a warp takes per grab of the queue (tuned)
  // accumulators
  long long *acc_sumi, *acc_sd, *acc_fx, *acc_fy, *acc_fz;
  long long *energy;       // nsys * kEnergySlots
  // model
  BornConst born;
  PairConst pair;
  float neck_scale;
  const float *neck_pos, *neck_val;  // 441 each
};

// ---- checked build ---------------------------------------------------------
// With -DSFFG_CHECKED every indirect index of the kernels (list entries,
// tiles, table rows, atoms of bonded terms) is tested against its array's
// extent; a failed test records a code in the translation unit's error word
// (the first failure wins), the access goes to element 0 instead, and the
// kernel runs on: an out-of-range index is reported, never dereferenced,
// and nothing traps.  sffg_checked_code() reads the word.  Without the
// option the checks compile to nothing.
enum CheckCode { kCheckSlot = 1, kCheckTile = 2, kCheckLj = 3, kCheckNeck = 4, kCheckAtom = 5 };
#ifdef SFFG_CHECKED
static __device__ int g_check_code;
__device__ __forceinline__ int checked_index(int i, int n, int code) {
  if (static_cast<unsigned>(i) >= static_cast<unsigned>(n)) {
    atomicCAS(&g_check_code, 0, code);
    return 0;
  }
  return i;
}
#define SFFG_IDX(i, n, code) ::sffg::checked_index((i), (n), (code))
#else
#define SFFG_IDX(i, n, code) (i)
#endif

__device__ __forceinline__ long long to_fixed(float v, float scale) {
  return __float2ll_rn(v * scale);
}

// Steps per group of the pair loops: j-side partial sums are kept in
// registers for a group of steps, then folded across the warp.  Fewer steps
// per group keep the unrolled loop body (and the instruction-cache
// footprint) small at the cost of more shuffles per step; measured best:
// 4 for all three passes (with pass 2 at 3 blocks per SM; at 2 blocks per
// SM, 8 was better for it).
#ifndef SFFG_GROUP_BORN
#define SFFG_GROUP_BORN 4
#endif
#ifndef SFFG_GROUP_PAIR
#define SFFG_GROUP_PAIR 4
#endif
constexpr int kGroup = SFFG_GROUP_BORN;
constexpr int kGroupPair = SFFG_GROUP_PAIR;

constexpr int ilog2(int k) { return k == 8 ? 3 : k == 4 ? 2 : k == 2 ? 1 : 0; }

// Sum of v[e] over the 32 lanes for e = 0..K-1, delivered to lane K*g + e
// (zero in the other lanes): log2(K) transposing shuffle stages (each lane
// keeps half of its values and sends the other half across), then a plain
// butterfly over the remaining lane bits.  After the transposing stages
// lane L holds element L >> (5 - log2 K).
template <int K>
__device__ __forceinline__ float reduce_to_lane(const float (&v)[K], int g, int lane) {
  static_assert(K == 2 || K == 4 || K == 8, "group of 2, 4 or 8 steps");
  constexpr int kLog2 = ilog2(K);
  float a[K];
#pragma unroll
  for (int k = 0; k < K; k++) a[k] = v[k];
  int m = K, dist = 16;
#pragma unroll
  for (int st = 0; st < kLog2; st++) {
    const bool b = lane & dist;
    m >>= 1;
#pragma unroll
    for (int k = 0; k < m; k++) {
      const float send = b ? a[k] : a[k + m];
      const float keep = b ? a[k + m] : a[k];
      a[k] = keep + __shfl_xor_sync(kFull, send, dist);
    }
    dist >>= 1;
  }
  float c = a[0];
#pragma unroll
  for (int d = 16 >> kLog2; d > 0; d >>= 1) c += __shfl_xor_sync(kFull, c, d);
  const float r = __shfl_sync(kFull, c, (lane & (K - 1)) << (5 - kLog2));
  return (lane >> kLog2) == g ? r : 0.0f;
}

__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// Programmatic dependent launch: a kernel launched with the programmatic
// stream-serialization attribute (launch_pdl) may be scheduled while the
// kernel before it on the stream drains; it waits here, before reading
// anything that kernel wrote, until that grid has completed and its writes
// are visible.  A kernel launched without the attribute passes at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ void atomic_add_ll(long long *p, long long v) {
  if (v != 0) atomicAdd(reinterpret_cast<unsigned long long *>(p), static_cast<unsigned long long>(v));
}

// Claims the next `claim` work items of the queue for this warp.
__device__ __forceinline__ int claim_chunk(int *counter, int lane, int claim) {
  int base = 0;
  if (lane == 0) base = atomicAdd(counter, claim);
  return __shfl_sync(kFull, base, 0);
}

// Both directions of the descreening of one pair of list B (value, or for
// DERIV the derivative / dij): vi is atom i descreened by sphere j, vj the
// converse.  List B holds no pair within near-field range, so only the far
// field (evaluated for every lane), the rgbmax tail (evaluated when any
// lane of the warp needs it) and the zero beyond rgbmax + s remain; the
// branches are warp-uniform.
template <bool DERIV>
__device__ __forceinline__ void descreen_pair(const BornConst &c, bool in, float dij, float d1, float s_i,
                                              float s_j, float &vi, float &vj) {
  vi = DERIV ? far_deriv(d1, s_j) : far_term(d1, s_j);
  vj = DERIV ? far_deriv(d1, s_i) : far_term(d1, s_i);
  const bool ti = dij > c.rgbmax - s_j, tj = dij > c.rgbmax - s_i;
  if (__any_sync(kFull, in && (ti || tj))) {
    const float qi = tail_closed<DERIV>(c, dij, d1, s_j);
    const float qj = tail_closed<DERIV>(c, dij, d1, s_i);
    vi = ti ? qi : vi;
    vj = tj ? qj : vj;
  }
  // beyond rgbmax + s the term is zero; with a negative s (GBneck2 screens
  // sulfur with fs < 0) that range starts below rgbmax - s
  vi = dij > c.rgbmax + s_j ? 0.0f : vi;
  vj = dij > c.rgbmax + s_i ? 0.0f : vj;
}

// Stages the j-entries of chunk k in shared memory: lane l loads entry l.
// Returns this lane's j slot (padding entries point at a real slot of the
// i-tile and have an empty column).
__device__ __forceinline__ int chunk_entry(const ChunkList &L, int k, int lane, unsigned &col, int nslot) {
  const size_t e = static_cast<size_t>(k) * 32 + lane;
  col = L.col[e];
  return SFFG_IDX(L.slot[e], nslot, kCheckSlot);
}

// ------------------------------------------------------------ list C chunks
// List C holds the pairs close enough for the near-field forms; its chunks
// are sparse (~13% of the 32 x 32 bits set), so a warp walks the set bits
// of a chunk 32 pairs at a time, one pair per lane, and evaluates the whole
// ladder of the reference for both directions.  Lane t then collects, in
// pair order, the terms of i-atom t and of j-entry t (a fixed order, so the
// sums are deterministic).
//
// Passes 1 and 3 take the chunks of lists B and C from one work queue, the
// list C chunks spread evenly among the others: near-field chunks are
// latency-bound (long dependent chains, little work), far-field chunks
// throughput-bound, and mixing them keeps every SM issuing.

// Work item m of the merged queue: true and the list C chunk k, or false
// and the list B chunk k.
__device__ __forceinline__ bool merged_item(int m, int nB, int nC, int &k) {
  const long long n = static_cast<long long>(nB) + nC;
  const int c0 = static_cast<int>(static_cast<long long>(m) * nC / n);
  const int c1 = static_cast<int>(static_cast<long long>(m + 1) * nC / n);
  k = c1 > c0 ? c0 : m - c0;
  return c1 > c0;
}



// Pair p of the chunk (0 <= p < total): its j-entry and i-lane, from the
// exclusive prefix counts s_pre of set bits per entry.
__device__ __forceinline__ void near_pair(const int *s_pre, const unsigned *s_col, int p, int &il, int &jl) {
  int j = 0;
#pragma unroll
  for (int b = 16; b > 0; b >>= 1)
    if (s_pre[j + b] <= p) j += b;
  jl = j;
  // position of set bit number r (from 0) of the entry's column
  unsigned m = s_col[j];
  int r = p - s_pre[j], pos = 0;
#pragma unroll
  for (int b = 16; b > 0; b >>= 1) {
    const int c = __popc(m & ((1u << b) - 1u));
    if (c <= r) {
      r -= c;
      m >>= b;
      pos += b;
    }
  }
  il = pos;
}

// Stages chunk k of list C: j-entries in shared memory, their bit counts'
// exclusive prefix; returns the chunk's pair count.
__device__ __forceinline__ int near_stage(const DevTables &t, int k, int lane, float4 *hj, float4 *lj,
                                          float4 *gj, int *pj, unsigned *cj, int *pre, int &sj, unsigned &col,
                                          bool sda) {
  const size_t e = static_cast<size_t>(k) * 32 + lane;
  col = t.lc.col[e];
  sj = SFFG_IDX(t.lc.slot[e], t.nslot, kCheckSlot);
  float4 l = t.pos_lo[sj];
  if (sda) l.w = t.sumda32[sj];
  hj[lane] = t.pos_hi[sj];
  lj[lane] = l;
  gj[lane] = t.gbpar[sj];
  pj[lane] = t.param[sj];
  cj[lane] = col;
  const int c = __popc(col);
  int incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += v;
  }
  pre[lane] = incl - c;
  __syncwarp();
  return __shfl_sync(kFull, incl, 31);
}

// ------------------------------------------------------------------ pass 1
// Born-radius descreening sums (src/sff/eff.c:1566-1709): both directions
// of every pair within rgbmax + Fsmax, over lists B and C.
template <bool NECK>
__global__ void __launch_bounds__(256, 3) k_born(const DevTables t) {
  __shared__ float4 sm_hi[8][32], sm_lo[8][32], sm_gb[8][32];  // j entries of the chunk
  __shared__ float4 si_hi[8][32], si_lo[8][32], si_gb[8][32];  // the i-tile
  __shared__ unsigned sm_col[8][32];
  __shared__ int sm_par[8][32], si_par[8][32], s_pre[8][32];
  __shared__ float s_npos[NECK ? 441 : 1], s_nval[NECK ? 441 : 1];
  if (NECK) {  // static tables: staged before the wait
    for (int i = threadIdx.x; i < 441; i += blockDim.x) {
      s_npos[i] = t.neck_pos[i];
      s_nval[i] = t.neck_val[i];
    }
    __syncthreads();
  }
  pdl_wait();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nB = *t.lb.nchunk, nC = *t.lc.nchunk, nitem = nB + nC;
  const float FB = 1099511627776.0f;
  int cur_I = -1;
  float xi = 0, yi = 0, zi = 0, xli = 0, yli = 0, zli = 0, si = 0, rbi = 0, sci = 0;
  int nki = 0;
  long long sumi64 = 0;

  // list B chunk k: lanes hold the i-tile, steps walk the 32 j-entries
  auto far_chunk = [&](int k) {
    unsigned mycol;
    const int sj = chunk_entry(t.lb, k, lane, mycol, t.nslot);
    sm_hi[w][lane] = t.pos_hi[sj];
    sm_lo[w][lane] = t.pos_lo[sj];
    {
      // far chunks never read the radius rho in gbpar.x: it carries the
      // entry's column mask, one shared read per step fewer
      float4 gq = t.gbpar[sj];
      gq.x = __uint_as_float(mycol);
      sm_gb[w][lane] = gq;
    }
    if (NECK) sm_par[w][lane] = t.param[sj];
    const unsigned cols = __ballot_sync(kFull, mycol != 0u);
    __syncwarp();
    float acc_i = 0.0f, acc_j = 0.0f;
#pragma unroll 1
    for (int g = 0; g < 32 / kGroup; g++) {
      float aj[kGroup];
#pragma unroll
      for (int s = 0; s < kGroup; s++) {
        const int j = g * kGroup + s;
        aj[s] = 0.0f;
        if (!((cols >> j) & 1u)) continue;  // padding entry
        const float4 h = sm_hi[w][j], l = sm_lo[w][j], gp = sm_gb[w][j];
        const float dx = (xi - h.x) + (xli - l.x);
        const float dy = (yi - h.y) + (yli - l.y);
        const float dz = (zi - h.z) + (zli - l.z);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const bool in = ((__float_as_uint(gp.x) >> lane) & 1u) && r2 <= t.born.cutoff2;
        if (!__any_sync(kFull, in)) continue;  // every lane out of range
        const float dij1i = rsqrt_nr(r2);
        const float dij = r2 * dij1i;
        float ti, tj;
        descreen_pair<false>(t.born, in, dij, dij1i, si, gp.y, ti, tj);
        ti = fmaf(ti, gp.w, ti);
        tj = fmaf(tj, sci, tj);
        if (NECK) {
          const bool nk = in && dij < rbi + gp.z + 6.8f;
          if (__any_sync(kFull, nk)) {
            const int nkj = (sm_par[w][j] >> 16) & 0xff;
            const float a = neck_term(dij, s_npos[SFFG_IDX(nki * 21 + nkj, 441, kCheckNeck)], s_nval[SFFG_IDX(nki * 21 + nkj, 441, kCheckNeck)], t.neck_scale);
            const float b = neck_term(dij, s_npos[SFFG_IDX(nkj * 21 + nki, 441, kCheckNeck)], s_nval[SFFG_IDX(nkj * 21 + nki, 441, kCheckNeck)], t.neck_scale);
            ti += nk ? a : 0.0f;
            tj += nk ? b : 0.0f;
          }
        }
        acc_i += in ? ti : 0.0f;
        aj[s] = in ? tj : 0.0f;
      }
      acc_j += reduce_to_lane(aj, g, lane);
    }
    sumi64 += to_fixed(acc_i, FB);
    if (mycol) atomic_add_ll(&t.acc_sumi[sj], to_fixed(acc_j, FB));
    __syncwarp();
  };

  // list C chunk k: 32 compacted pairs per round, one per lane
  auto near_chunk = [&](int k) {
    int sj;
    unsigned mycol;
    const int total =
        near_stage(t, k, lane, sm_hi[w], sm_lo[w], sm_gb[w], sm_par[w], sm_col[w], s_pre[w], sj, mycol, false);
    float acc_i = 0.0f, acc_j = 0.0f;
    for (int b0 = 0; b0 < total; b0 += 32) {
      const int p = b0 + lane;
      float ti = 0.0f, tj = 0.0f;
      int il = 0, jl = 0;
      if (p < total) {
        near_pair(s_pre[w], sm_col[w], p, il, jl);
        const float4 hi = si_hi[w][il], li = si_lo[w][il], gi = si_gb[w][il];
        const float4 h = sm_hi[w][jl], l = sm_lo[w][jl], gp = sm_gb[w][jl];
        const float dx = (hi.x - h.x) + (li.x - l.x);
        const float dy = (hi.y - h.y) + (li.y - l.y);
        const float dz = (hi.z - h.z) + (li.z - l.z);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        if (r2 <= t.born.cutoff2) {
          const float d1 = rsqrt_nr(r2);
          const float dij = r2 * d1;
          ti = descreen(t.born, dij, r2, d1, gi.x, gp.y);
          tj = descreen(t.born, dij, r2, d1, gp.x, gi.y);
          ti = fmaf(ti, gp.w, ti);
          tj = fmaf(tj, gi.w, tj);
          if (NECK && dij < gi.z + gp.z + 6.8f) {
            const int nkp = (si_par[w][il] >> 16) & 0xff, nkj = (sm_par[w][jl] >> 16) & 0xff;
            ti += neck_term(dij, s_npos[SFFG_IDX(nkp * 21 + nkj, 441, kCheckNeck)], s_nval[SFFG_IDX(nkp * 21 + nkj, 441, kCheckNeck)], t.neck_scale);
            tj += neck_term(dij, s_npos[SFFG_IDX(nkj * 21 + nkp, 441, kCheckNeck)], s_nval[SFFG_IDX(nkj * 21 + nkp, 441, kCheckNeck)], t.neck_scale);
          }
        }
      }
      const int n = min(32, total - b0);
      for (int q = 0; q < n; q++) {
        const float a = __shfl_sync(kFull, ti, q), c = __shfl_sync(kFull, tj, q);
        const int iq = __shfl_sync(kFull, il, q), jq = __shfl_sync(kFull, jl, q);
        acc_i += iq == lane ? a : 0.0f;
        acc_j += jq == lane ? c : 0.0f;
      }
    }
    sumi64 += to_fixed(acc_i, FB);
    if (mycol) atomic_add_ll(&t.acc_sumi[sj], to_fixed(acc_j, FB));
    __syncwarp();
  };

  for (;;) {
    const int base = claim_chunk(t.counter, lane, t.claim);
    if (base >= nitem) break;
    const int end = min(base + t.claim, nitem);
    for (int m = base; m < end; m++) {
      int k;
      const bool nr = merged_item(m, nB, nC, k);
      const int I = SFFG_IDX(nr ? t.lc.chunk_i[k] : t.lb.chunk_i[k], t.ntile, kCheckTile);
      if (!t.sys_active[t.tile_sys[I]]) continue;
      if (I != cur_I) {
        if (cur_I >= 0) atomic_add_ll(&t.acc_sumi[cur_I * 32 + lane], sumi64);
        cur_I = I;
        sumi64 = 0;
        const int sl = I * 32 + lane;
        const float4 h = t.pos_hi[sl], l = t.pos_lo[sl], g = t.gbpar[sl];
        const int pr = t.param[sl];
        xi = h.x; yi = h.y; zi = h.z; xli = l.x; yli = l.y; zli = l.z;
        si = g.y; rbi = g.z; sci = g.w;
        nki = (pr >> 16) & 0xff;
        si_hi[w][lane] = h;
        si_lo[w][lane] = l;
        si_gb[w][lane] = g;
        si_par[w][lane] = pr;
      }
      if (nr) near_chunk(k);
      else far_chunk(k);
    }
  }
  if (cur_I >= 0) atomic_add_ll(&t.acc_sumi[cur_I * 32 + lane], sumi64);
}

// ------------------------------------------------------------------ pass 2
// GB + Coulomb + Lennard-Jones pair energies, dE/dr and sumdeijda
// (src/sff/eff.c:1902-2063) over list A.
// Lennard-Jones tables of up to this many (A, B) entries (all systems of the
// batch together) are read from shared memory in pass 2.
constexpr int kLjShared = 4096;

template <bool KAPPA, bool LJS>
__global__ void __launch_bounds__(256, 3) k_gbpair(const DevTables t) {
  // j-entries of the chunk: position (hi, lo + Born radius) and
  // (1/R_j^2 / 4, Lennard-Jones row offset type_j * ntypes, column mask,
  // exclusion mask), three 16-byte reads per step
  __shared__ float4 sm_hi[8][32], sm_lo[8][32];
  __shared__ uint4 sm_aux[8][32];
  __shared__ float2 s_lj[LJS ? kLjShared : 1];
  if (LJS) {  // a static table: staged before the wait
    for (int i = threadIdx.x; i < t.lj_n; i += blockDim.x) s_lj[i] = t.lj[i];
    __syncthreads();
  }
  pdl_wait();
  const float2 *const lj_all = LJS ? s_lj : t.lj;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nchunk = *t.la.nchunk;
  int cur_I = -1, cur_sys = -1;
  float xi = 0, yi = 0, zi = 0, xli = 0, yli = 0, zli = 0, qi = 0, ri = 1, rvi = 0;
  int ti = 0, nt = 1;
  const float2 *lj = lj_all;
  long long fx64 = 0, fy64 = 0, fz64 = 0, sd64 = 0, ep64 = 0, ee64 = 0, ev64 = 0;
  const float FS = 4294967296.0f;
  auto flush_i = [&]() {
    const int sl = cur_I * 32 + lane;
    atomic_add_ll(&t.acc_fx[sl], fx64);
    atomic_add_ll(&t.acc_fy[sl], fy64);
    atomic_add_ll(&t.acc_fz[sl], fz64);
    atomic_add_ll(&t.acc_sd[sl], sd64);
  };
  auto flush_e = [&]() {
    long long a = warp_sum_ll(ep64), b = warp_sum_ll(ee64), c = warp_sum_ll(ev64);
    if (lane == 0) {
      atomic_add_ll(&t.energy[cur_sys * kEnergySlots + 0], -a);
      atomic_add_ll(&t.energy[cur_sys * kEnergySlots + 1], b);
      atomic_add_ll(&t.energy[cur_sys * kEnergySlots + 2], c);
    }
    ep64 = ee64 = ev64 = 0;
  };
  for (;;) {
    const int base = claim_chunk(t.counter, lane, t.claim);
    if (base >= nchunk) break;
    const int end = min(base + t.claim, nchunk);
    for (int k = base; k < end; k++) {
      const int I = SFFG_IDX(t.la.chunk_i[k], t.ntile, kCheckTile);
      const int sys = t.tile_sys[I];
      if (!t.sys_active[sys]) continue;
      if (sys != cur_sys) {
        if (cur_sys >= 0) flush_e();
        cur_sys = sys;
        lj = lj_all + t.sys_lj_off[sys];
        nt = t.sys_ntypes[sys];
      }
      if (I != cur_I) {
        if (cur_I >= 0) flush_i();
        cur_I = I;
        fx64 = fy64 = fz64 = sd64 = 0;
        const int sl = I * 32 + lane;
        const float4 h = t.pos_hi[sl], l = t.pos_lo[sl];
        xi = h.x; yi = h.y; zi = h.z; qi = h.w; xli = l.x; yli = l.y; zli = l.z;
        ri = t.reff32[sl];
        rvi = t.rinv2[sl];
        ti = t.param[sl] & 0xffff;
      }
      unsigned mycol;
      const int sj = chunk_entry(t.la, k, lane, mycol, t.nslot);
      {
        float4 l = t.pos_lo[sj];
        l.w = t.reff32[sj];
        sm_hi[w][lane] = t.pos_hi[sj];
        sm_lo[w][lane] = l;
        sm_aux[w][lane] = make_uint4(__float_as_uint(t.rinv2[sj]), (t.param[sj] & 0xffff) * nt, mycol,
                                     t.la.exc[static_cast<size_t>(k) * 32 + lane]);
      }
      const unsigned cols = __ballot_sync(kFull, mycol != 0u);
      __syncwarp();
      float fix = 0, fiy = 0, fiz = 0, sdi = 0, ep = 0, ee = 0, ev = 0;
      float jx = 0, jy = 0, jz = 0, jsd = 0;
#pragma unroll 1
      for (int g = 0; g < 32 / kGroupPair; g++) {
        float ax[kGroupPair], ay[kGroupPair], az[kGroupPair], as[kGroupPair];
#pragma unroll
        for (int s = 0; s < kGroupPair; s++) {
          const int j = g * kGroupPair + s;
          ax[s] = ay[s] = az[s] = as[s] = 0.0f;
          if (!((cols >> j) & 1u)) continue;  // padding entry
          const float4 h = sm_hi[w][j], l = sm_lo[w][j];
          const uint4 au = sm_aux[w][j];
          const float dx = (xi - h.x) + (xli - l.x);
          const float dy = (yi - h.y) + (yli - l.y);
          const float dz = (zi - h.z) + (zli - l.z);
          const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          const bool in = (au.z >> lane) & 1u;
          const bool coul = in && !((au.w >> lane) & 1u);
          // row type_j: the lanes' i types fall in one row of the symmetric table
#ifdef SFFG_CHECKED
          const float2 ab = lj_all[SFFG_IDX(static_cast<int>(lj - lj_all) + static_cast<int>(au.y) + ti, t.lj_n,
                                            kCheckLj)];
#else
          const float2 ab = lj[au.y + ti];
#endif
          // a lane off the list gets zero charge and coefficients (and r2 = 1:
          // the self pair of a diagonal tile has r2 = 0), hence zero terms
          const float qq = in ? qi * h.w : 0.0f;
          const PairOut o = gb_pair<KAPPA>(t.pair, in ? r2 : 1.0f, qq, coul ? qq : 0.0f, ri, l.w, rvi,
                                           __uint_as_float(au.x), coul ? ab.x : 0.0f, coul ? ab.y : 0.0f);
          const float de = o.de;
          fix = fmaf(de, dx, fix);
          fiy = fmaf(de, dy, fiy);
          fiz = fmaf(de, dz, fiz);
          ax[s] = -de * dx;
          ay[s] = -de * dy;
          az[s] = -de * dz;
          sdi += o.sd_i;
          as[s] = o.sd_j;
          ep += o.epol;
          ee += o.eel;
          ev += o.evdw;
        }
        jx += reduce_to_lane(ax, g, lane);
        jy += reduce_to_lane(ay, g, lane);
        jz += reduce_to_lane(az, g, lane);
        jsd += reduce_to_lane(as, g, lane);
      }
      fx64 += to_fixed(fix, FS);
      fy64 += to_fixed(fiy, FS);
      fz64 += to_fixed(fiz, FS);
      sd64 += to_fixed(sdi, FS);
      ep64 += to_fixed(ep, FS);
      ee64 += to_fixed(ee, FS);
      ev64 += to_fixed(ev, FS);
      if (mycol) {
        atomic_add_ll(&t.acc_fx[sj], to_fixed(jx, FS));
        atomic_add_ll(&t.acc_fy[sj], to_fixed(jy, FS));
        atomic_add_ll(&t.acc_fz[sj], to_fixed(jz, FS));
        atomic_add_ll(&t.acc_sd[sj], to_fixed(jsd, FS));
      }
      __syncwarp();
    }
  }
  if (cur_I >= 0) flush_i();
  if (cur_sys >= 0) flush_e();
}

// ------------------------------------------------------------------ pass 3
// Chain rule through the Born radii (src/sff/eff.c:2241-2395) over lists B
// and C: for each pair within rgbmax + Fsmax, g = sumda_i d_ij +
// sumda_j d_ji, f_i -= g r_ij, f_j += g r_ij.
template <bool NECK>
__global__ void __launch_bounds__(256, 3) k_chain(const DevTables t) {
  __shared__ float4 sm_hi[8][32], sm_lo[8][32], sm_gb[8][32];  // j entries (lo.w = sumda)
  __shared__ float4 si_hi[8][32], si_lo[8][32], si_gb[8][32];  // the i-tile (lo.w = sumda)
  __shared__ unsigned sm_col[8][32];
  __shared__ int sm_par[8][32], si_par[8][32], s_pre[8][32];
  __shared__ float s_npos[NECK ? 441 : 1], s_nval[NECK ? 441 : 1];
  if (NECK) {  // static tables: staged before the wait
    for (int i = threadIdx.x; i < 441; i += blockDim.x) {
      s_npos[i] = t.neck_pos[i];
      s_nval[i] = t.neck_val[i];
    }
    __syncthreads();
  }
  pdl_wait();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nB = *t.lb.nchunk, nC = *t.lc.nchunk, nitem = nB + nC;
  const float FS = 4294967296.0f;
  int cur_I = -1;
  float xi = 0, yi = 0, zi = 0, xli = 0, yli = 0, zli = 0, si = 0, rbi = 0, sci = 0, sdai = 0;
  int nki = 0;
  long long fx64 = 0, fy64 = 0, fz64 = 0;
  auto flush_i = [&]() {
    const int sl = cur_I * 32 + lane;
    atomic_add_ll(&t.acc_fx[sl], fx64);
    atomic_add_ll(&t.acc_fy[sl], fy64);
    atomic_add_ll(&t.acc_fz[sl], fz64);
  };
  auto add_j = [&](int sj, float jx, float jy, float jz) {
    atomic_add_ll(&t.acc_fx[sj], to_fixed(jx, FS));
    atomic_add_ll(&t.acc_fy[sj], to_fixed(jy, FS));
    atomic_add_ll(&t.acc_fz[sj], to_fixed(jz, FS));
  };

  auto far_chunk = [&](int k) {
    unsigned mycol;
    const int sj = chunk_entry(t.lb, k, lane, mycol, t.nslot);
    {
      float4 l = t.pos_lo[sj];
      l.w = t.sumda32[sj];
      sm_hi[w][lane] = t.pos_hi[sj];
      sm_lo[w][lane] = l;
      float4 gq = t.gbpar[sj];
      gq.x = __uint_as_float(mycol);  // the column mask, as in pass 1
      sm_gb[w][lane] = gq;
      if (NECK) sm_par[w][lane] = t.param[sj];
    }
    const unsigned cols = __ballot_sync(kFull, mycol != 0u);
    __syncwarp();
    float fix = 0, fiy = 0, fiz = 0, jx = 0, jy = 0, jz = 0;
#pragma unroll 1
    for (int g = 0; g < 32 / kGroup; g++) {
      float ax[kGroup], ay[kGroup], az[kGroup];
#pragma unroll
      for (int s = 0; s < kGroup; s++) {
        const int j = g * kGroup + s;
        ax[s] = ay[s] = az[s] = 0.0f;
        if (!((cols >> j) & 1u)) continue;
        const float4 h = sm_hi[w][j], l = sm_lo[w][j], gp = sm_gb[w][j];
        const float dx = (xi - h.x) + (xli - l.x);
        const float dy = (yi - h.y) + (yli - l.y);
        const float dz = (zi - h.z) + (zli - l.z);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const bool in = ((__float_as_uint(gp.x) >> lane) & 1u) && r2 <= t.born.cutoff2;
        if (!__any_sync(kFull, in)) continue;
        // the hardware rsqrt alone: pass 3 only shapes the forces, whose RMS
        // error against FP64 it leaves at 4.70e-6 (to 3 digits) for -2% time
        const float dij1i = rsqrt_fast(r2);
        const float dij = r2 * dij1i;
        float di, dj;
        descreen_pair<true>(t.born, in, dij, dij1i, si, gp.y, di, dj);
        di = fmaf(di, gp.w, di);
        dj = fmaf(dj, sci, dj);
        if (NECK) {
          const bool nk = in && dij < rbi + gp.z + 6.8f;
          if (__any_sync(kFull, nk)) {
            const int nkj = (sm_par[w][j] >> 16) & 0xff;
            const float a = neck_deriv(dij, s_npos[SFFG_IDX(nki * 21 + nkj, 441, kCheckNeck)], s_nval[SFFG_IDX(nki * 21 + nkj, 441, kCheckNeck)], t.neck_scale);
            const float b = neck_deriv(dij, s_npos[SFFG_IDX(nkj * 21 + nki, 441, kCheckNeck)], s_nval[SFFG_IDX(nkj * 21 + nki, 441, kCheckNeck)], t.neck_scale);
            di += nk ? a : 0.0f;
            dj += nk ? b : 0.0f;
          }
        }
        const float gg = in ? fmaf(sdai, di, l.w * dj) : 0.0f;
        fix = fmaf(-gg, dx, fix);
        fiy = fmaf(-gg, dy, fiy);
        fiz = fmaf(-gg, dz, fiz);
        ax[s] = gg * dx;
        ay[s] = gg * dy;
        az[s] = gg * dz;
      }
      jx += reduce_to_lane(ax, g, lane);
      jy += reduce_to_lane(ay, g, lane);
      jz += reduce_to_lane(az, g, lane);
    }
    fx64 += to_fixed(fix, FS);
    fy64 += to_fixed(fiy, FS);
    fz64 += to_fixed(fiz, FS);
    if (mycol) add_j(sj, jx, jy, jz);
    __syncwarp();
  };

  auto near_chunk = [&](int k) {
    int sj;
    unsigned mycol;
    const int total =
        near_stage(t, k, lane, sm_hi[w], sm_lo[w], sm_gb[w], sm_par[w], sm_col[w], s_pre[w], sj, mycol, true);
    float fix = 0, fiy = 0, fiz = 0, jx = 0, jy = 0, jz = 0;
    for (int b0 = 0; b0 < total; b0 += 32) {
      const int p = b0 + lane;
      float gx = 0.0f, gy = 0.0f, gz = 0.0f;
      int il = 0, jl = 0;
      if (p < total) {
        near_pair(s_pre[w], sm_col[w], p, il, jl);
        const float4 hi = si_hi[w][il], li = si_lo[w][il], gi = si_gb[w][il];
        const float4 h = sm_hi[w][jl], l = sm_lo[w][jl], gp = sm_gb[w][jl];
        const float dx = (hi.x - h.x) + (li.x - l.x);
        const float dy = (hi.y - h.y) + (li.y - l.y);
        const float dz = (hi.z - h.z) + (li.z - l.z);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        if (r2 <= t.born.cutoff2) {
          const float d1 = rsqrt_nr(r2);
          const float dij = r2 * d1;
          float di = descreen_deriv(t.born, dij, r2, d1, gi.x, gp.y);
          float dj = descreen_deriv(t.born, dij, r2, d1, gp.x, gi.y);
          di = fmaf(di, gp.w, di);
          dj = fmaf(dj, gi.w, dj);
          if (NECK && dij < gi.z + gp.z + 6.8f) {
            const int nkp = (si_par[w][il] >> 16) & 0xff, nkj = (sm_par[w][jl] >> 16) & 0xff;
            di += neck_deriv(dij, s_npos[SFFG_IDX(nkp * 21 + nkj, 441, kCheckNeck)], s_nval[SFFG_IDX(nkp * 21 + nkj, 441, kCheckNeck)], t.neck_scale);
            dj += neck_deriv(dij, s_npos[SFFG_IDX(nkj * 21 + nkp, 441, kCheckNeck)], s_nval[SFFG_IDX(nkj * 21 + nkp, 441, kCheckNeck)], t.neck_scale);
          }
          const float gg = fmaf(li.w, di, l.w * dj);
          gx = gg * dx;
          gy = gg * dy;
          gz = gg * dz;
        }
      }
      const int n = min(32, total - b0);
      for (int q = 0; q < n; q++) {
        const float ax = __shfl_sync(kFull, gx, q), ay = __shfl_sync(kFull, gy, q),
                    az = __shfl_sync(kFull, gz, q);
        const int iq = __shfl_sync(kFull, il, q), jq = __shfl_sync(kFull, jl, q);
        const bool mi = iq == lane, mj = jq == lane;
        fix -= mi ? ax : 0.0f;
        fiy -= mi ? ay : 0.0f;
        fiz -= mi ? az : 0.0f;
        jx += mj ? ax : 0.0f;
        jy += mj ? ay : 0.0f;
        jz += mj ? az : 0.0f;
      }
    }
    fx64 += to_fixed(fix, FS);
    fy64 += to_fixed(fiy, FS);
    fz64 += to_fixed(fiz, FS);
    if (mycol) add_j(sj, jx, jy, jz);
    __syncwarp();
  };

  for (;;) {
    const int base = claim_chunk(t.counter, lane, t.claim);
    if (base >= nitem) break;
    const int end = min(base + t.claim, nitem);
    for (int m = base; m < end; m++) {
      int k;
      const bool nr = merged_item(m, nB, nC, k);
      const int I = SFFG_IDX(nr ? t.lc.chunk_i[k] : t.lb.chunk_i[k], t.ntile, kCheckTile);
      if (!t.sys_active[t.tile_sys[I]]) continue;
      if (I != cur_I) {
        if (cur_I >= 0) flush_i();
        cur_I = I;
        fx64 = fy64 = fz64 = 0;
        const int sl = I * 32 + lane;
        const float4 h = t.pos_hi[sl], g = t.gbpar[sl];
        float4 l = t.pos_lo[sl];
        const int pr = t.param[sl];
        xi = h.x; yi = h.y; zi = h.z; xli = l.x; yli = l.y; zli = l.z;
        si = g.y; rbi = g.z; sci = g.w;
        sdai = t.sumda32[sl];
        nki = (pr >> 16) & 0xff;
        l.w = sdai;
        si_hi[w][lane] = h;
        si_lo[w][lane] = l;
        si_gb[w][lane] = g;
        si_par[w][lane] = pr;
      }
      if (nr) near_chunk(k);
      else far_chunk(k);
    }
  }
  if (cur_I >= 0) flush_i();
}

}  // namespace sffg
