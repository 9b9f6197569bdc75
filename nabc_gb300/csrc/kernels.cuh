// Device kernels of the generalized-Born path (sm_103a).
//
// The three pair passes of the reference's egb() (src/sff/eff.c:1566-1733,
// 1770-2066, 2131-2405) run over compacted pair-list chunks (lists.cuh): a
// chunk is an i-tile of 32 atoms and 32 packed j-atoms with a column mask
// each.  A warp owns one chunk at a time: lane l holds i-atom l in
// registers; the far-field chunks are walked in a rotation (lane l meets
// j-entry (l + s) mod 32 at step s, the entry's j-side sums moving one lane
// per step), the near-field chunks pair by pair.  Both directions of each
// unordered pair are handled in one visit (Newton's third law).  Per chunk
// the FP32 partial sums are converted to 64-bit fixed point, so the totals
// do not depend on how chunks are scheduled.
#pragma once

#include <cstdint>
#include <type_traits>

#include "gbmath.cuh"
#include "pack2.cuh"

namespace sffg {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kEnergySlots = 9;  // fixed-point energy terms per system (EnergySlot)
// Non-excluded pairs closer than this (in A, at the list build) take their
// Coulomb and Lennard-Jones terms in FP64: their forces reach 1e3-1e5
// kcal/mol/A, where FP32 rounding alone is ~1e-7 of them.
constexpr float kClose = 2.5f;

// One compacted pair list (built by lists.cuh).
struct ChunkList {
  const int *chunk_i;   // i-tile of each chunk
  const int *slot;      // 32 j slots per chunk
  const unsigned *col;  // per entry, bit i: the pair with lane i of the i-tile is listed
  const unsigned *exc;  // per entry, bit i: the pair is excluded from Coulomb/LJ (cutoff list)
  const unsigned *close;  // per entry, bit i: a close pair, Coulomb/LJ in FP64 (cutoff list)
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
  const float4 *box_lo, *box_hi;  // bounding boxes (their centres are the tiles' reference points)
  // per system
  const int *sys_active;
  const int *sys_lj_off;
  const int *sys_ntypes;
  // (rgbmax + Fsmax)^2 with the system's own Fsmax (the reference skips a
  // pair beyond it, eff.c:1649), and 1 where every rgbmax tail of the
  // system has q = (rgbmax - d + s) / rgbmax <= 0.3, so that the polynomial
  // form alone serves (passes 1 and 3)
  const float2 *sys_born;
  const float2 *lj;       // (A, B) per type pair, per system blocks
  const double2 *lj64;    // the same table in FP64 (close pairs)
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

// ------------------------------------------------------ rotation schedule
// Far-field chunks (lists A, B and T) are walked in a rotation: lane l holds
// i-atom l of the chunk's i-tile; at step s (0..31) it takes j-entry
// (l + s) mod 32, so every step the warp evaluates 32 different pairs and
// each entry meets each lane once.  The entry data sit twice in shared
// memory (entries 0..31, then again), so lane l's read at step s is element
// l + s with the step as an immediate offset.  An entry's j-side sums travel
// with it: after each step every lane hands them to lane l - 1, which meets
// that entry next; after 32 steps lane e holds entry e's sums.  The column
// masks are transposed once per chunk so that bit s of a lane's mask word is
// its pair at step s.  Coordinates are taken relative to a reference point
// of the i-tile: the i-atom's exactly (high + low parts), the entry's as one
// FP32 value.

// 32 x 32 bit-matrix transpose over the warp: lane l returns the word whose
// bit e is bit l of lane e's x.
__device__ __forceinline__ unsigned warp_transpose_bits(unsigned x, int lane) {
  unsigned m = 0x0000ffffu;
#pragma unroll
  for (int j = 16; j != 0; j >>= 1, m ^= m << j) {
    const unsigned y = __shfl_xor_sync(kFull, x, j);
    x = (lane & j) ? ((x & ~m) | ((y >> j) & m)) : ((x & m) | ((y << j) & ~m));
  }
  return x;
}

// Lane l's pair at step s of the rotation schedule: bit s of the result is
// bit l of entry (l + s) mod 32's column word col (held by that lane).
__device__ __forceinline__ unsigned rotation_mask(unsigned col, int lane) {
  const unsigned t = warp_transpose_bits(col, lane);
  return __funnelshift_r(t, t, lane);
}

// (hi + lo) - c for coordinates split into FP32 high and low parts and a
// reference point c: the exact difference hi - c (two-sum) plus lo.  d gets
// the rounded value; e the remainder (|e| <= half an ulp of d).
__device__ __forceinline__ void rel_coord(float hi, float lo, float c, float &d, float &e) {
  const float s = hi - c;
  const float hv = s + c;
  const float err = (hi - hv) + ((hv - s) - c);  // hi - c = s + err exactly
  const float t = err + lo;
  d = s + t;
  e = (s - d) + t;
}

// Reference point of tile I: its bounding box's centre rounded to 1/256 A.
__device__ __forceinline__ float3 tile_ref(const float4 *box_lo, const float4 *box_hi, int I) {
  const float4 a = box_lo[I], b = box_hi[I];
  const float cx = rintf((a.x + b.x) * 128.0f) * (1.0f / 256.0f);
  const float cy = rintf((a.y + b.y) * 128.0f) * (1.0f / 256.0f);
  const float cz = rintf((a.z + b.z) * 128.0f) * (1.0f / 256.0f);
  // a tile without a finite atom has an empty (inverted) box: centre 0
  return make_float3(isfinite(cx) ? cx : 0.0f, isfinite(cy) ? cy : 0.0f, isfinite(cz) ? cz : 0.0f);
}

__device__ __forceinline__ float ex2_ftz(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ float rsqrt_ftz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
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
// and the list B chunk k (the list C chunks spread evenly among the others).
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

// Far-field descreening term of a sphere of radius s (s2 = s^2) at
// 1/dij^2 = d2i (the Taylor form of eff.c:1674-1681), and its derivative
// over dij (eff.c:2299-2307): far_term / far_deriv with s^2 and 1/dij^2
// supplied.
__device__ __forceinline__ float far_term2(float d2i, float s, float s2) {
  const float tmpsd = s2 * d2i;
  const float dumbo = fmaf(tmpsd, fmaf(tmpsd, fmaf(tmpsd, fmaf(tmpsd, kTDD, kTD), kTC), kTB), kTA) + kTAlo;
  return s * tmpsd * d2i * dumbo;
}

__device__ __forceinline__ float far_deriv2(float d2i, float s, float s2) {
  const float tmpsd = s2 * d2i;
  const float dumbo = fmaf(tmpsd, fmaf(tmpsd, fmaf(tmpsd, fmaf(tmpsd, kTHH, kTH), kTG), kTF), kTE) + kTElo;
  return tmpsd * s * d2i * d2i * dumbo;
}

// r^2 given to a lane whose pair is not on the list: every far-field,
// tail and neck term of it is an exact zero.
constexpr float kOffList = 1.0e30f;

// POLY: every system of the batch takes the polynomial rgbmax tail
// (2 max|s| <= 0.3 rgbmax); the logarithmic form is then left out of the
// code, which keeps it out of the hot loop's registers.
template <bool NECK, bool POLY>
__global__ void __launch_bounds__(256, 3) k_born(const DevTables t) {
  // far-field chunks (list B): per warp the entries twice, (x, y, z
  // relative to the i-tile's reference point, s) and (s correction, s^2,
  // rborn, neck index)
  __shared__ float4 sm_a[8][64], sm_b[8][64];
  // near-field chunks (list C)
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
  const float rgbmax = t.born.rgbmax;
  const int next = (lane + 1) & 31;
  int cur_I = -1;
  float3 cref = make_float3(0.f, 0.f, 0.f);
  float xi = 0, yi = 0, zi = 0, xil = 0, yil = 0, zil = 0, si = 0, si2 = 0, rbi = 0, sci = 0;
  int nki = 0;
  // the i-tile's system: (rgbmax + Fsmax)^2 over its own atoms, and whether
  // its rgbmax tails take the polynomial form
  float cut2 = 0.0f;
  bool tpoly = false;
  long long sumi64 = 0;

  // list B chunk k, rotation schedule
  auto far_chunk = [&](int k) {
    const size_t e = static_cast<size_t>(k) * 32 + lane;
    const unsigned mycol = t.lb.col[e];
    const int sj = SFFG_IDX(t.lb.slot[e], t.nslot, kCheckSlot);
    {
      const float4 h = t.pos_hi[sj], l = t.pos_lo[sj], g = t.gbpar[sj];
      float dx, dy, dz, ex, ey, ez;
      rel_coord(h.x, l.x, cref.x, dx, ex);
      rel_coord(h.y, l.y, cref.y, dy, ey);
      rel_coord(h.z, l.z, cref.z, dz, ez);
      const float4 a = make_float4(dx, dy, dz, g.y);
      const float4 b = make_float4(g.w, g.y * g.y, g.z, NECK ? __int_as_float((t.param[sj] >> 16) & 0xff) : 0.0f);
      sm_a[w][lane] = a;
      sm_a[w][lane + 32] = a;
      sm_b[w][lane] = b;
      sm_b[w][lane + 32] = b;
    }
    const unsigned m_in = rotation_mask(mycol, lane);
    __syncwarp();
    float acc_i = 0.0f, aj = 0.0f;
#pragma unroll 1
    for (int g = 0; g < 32; g += 4) {
      const unsigned gin = m_in >> g;
      const float4 *pa = &sm_a[w][lane + g];
      const float4 *pb = &sm_b[w][lane + g];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const float4 a = pa[u];
        const bool in = (gin >> u) & 1u;
        const float dx = (xi - a.x) + xil;
        const float dy = (yi - a.y) + yil;
        const float dz = (zi - a.z) + zil;
        float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        // off the list, or beyond rgbmax + Fsmax, where the reference skips
        // the pair (eff.c:1649)
        r2 = in && r2 <= cut2 ? r2 : kOffList;
        const float d1 = rsqrt_nr(r2);
        const float d2i = d1 * d1;
        const float cj = pb[u].x;
        // both directions as packed pairs: (sphere j on atom i, sphere i on
        // atom j)
        const f2 S = pk(a.w, si);
        float ti, tj;
        upk(far_term_x2(d2i, S, pk(pb[u].y, si2)), ti, tj);
        const float dij = r2 * d1;
        {
          // the smooth tail for dij > rgbmax - s, zero beyond rgbmax + s
          // (with a negative s, GBneck2's sulfur, that range starts below);
          // nearly every step of a chunk has some tail pair, so it is
          // evaluated throughout
          const bool qi_ = dij > rgbmax - a.w, qj_ = dij > rgbmax - si;
          float vi, vj;
          if (POLY || tpoly) {
            upk(tail_x2<false>(t.born, dij, d1, S), vi, vj);
          } else {
            vi = tail_closed<false>(t.born, dij, d1, a.w);
            vj = tail_closed<false>(t.born, dij, d1, si);
          }
          ti = qi_ ? vi : ti;
          tj = qj_ ? vj : tj;
          ti = dij > rgbmax + a.w ? 0.0f : ti;
          tj = dij > rgbmax + si ? 0.0f : tj;
        }
        ti = fmaf(ti, cj, ti);
        tj = fmaf(tj, sci, tj);
        if (NECK) {
          const float4 b = pb[u];
          const bool nk = dij < rbi + b.z + 6.8f;
          if (__any_sync(kFull, nk)) {
            const int nkj = __float_as_int(b.w);
            const int ij = SFFG_IDX(nki * 21 + nkj, 441, kCheckNeck), ji = SFFG_IDX(nkj * 21 + nki, 441, kCheckNeck);
            const float na = neck_term(dij, s_npos[ij], s_nval[ij], t.neck_scale);
            const float nb = neck_term(dij, s_npos[ji], s_nval[ji], t.neck_scale);
            // the reference adds the neck term only to pairs it has not
            // skipped as beyond rgbmax + s (eff.c:1663-1664, 1699-1707)
            ti += nk && dij <= rgbmax + a.w ? na : 0.0f;
            tj += nk && dij <= rgbmax + si ? nb : 0.0f;
          }
        }
        acc_i += ti;
        aj = __shfl_sync(kFull, aj + tj, next);
      }
    }
    sumi64 += to_fixed(acc_i, FB);
    if (mycol) atomic_add_ll(&t.acc_sumi[sj], to_fixed(aj, FB));
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
        if (r2 <= cut2) {
          const float d1 = rsqrt_nr(r2);
          const float dij = r2 * d1;
          ti = descreen<!POLY>(t.born, dij, r2, d1, gi.x, gp.y);
          tj = descreen<!POLY>(t.born, dij, r2, d1, gp.x, gi.y);
          ti = fmaf(ti, gp.w, ti);
          tj = fmaf(tj, gi.w, tj);
          if (NECK && dij < gi.z + gp.z + 6.8f) {
            const int nkp = (si_par[w][il] >> 16) & 0xff, nkj = (sm_par[w][jl] >> 16) & 0xff;
            if (dij <= t.born.rgbmax + gp.y)
              ti += neck_term(dij, s_npos[SFFG_IDX(nkp * 21 + nkj, 441, kCheckNeck)], s_nval[SFFG_IDX(nkp * 21 + nkj, 441, kCheckNeck)], t.neck_scale);
            if (dij <= t.born.rgbmax + gi.y)
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
      const int sys = t.tile_sys[I];
      if (!t.sys_active[sys]) continue;
      if (I != cur_I) {
        const float2 sb = t.sys_born[sys];
        cut2 = sb.x;
        tpoly = sb.y != 0.0f;
        if (cur_I >= 0) atomic_add_ll(&t.acc_sumi[cur_I * 32 + lane], sumi64);
        cur_I = I;
        sumi64 = 0;
        const int sl = I * 32 + lane;
        const float4 h = t.pos_hi[sl], l = t.pos_lo[sl], g = t.gbpar[sl];
        const int pr = t.param[sl];
        cref = tile_ref(t.box_lo, t.box_hi, I);
        rel_coord(h.x, l.x, cref.x, xi, xil);
        rel_coord(h.y, l.y, cref.y, yi, yil);
        rel_coord(h.z, l.z, cref.z, zi, zil);
        si = g.y; si2 = g.y * g.y; rbi = g.z; sci = g.w;
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
//
// Rotation schedule: lane l holds i-atom l of the chunk's i-tile; at step s
// (0..31) it takes j-entry (l + s) mod 32, so every step the warp evaluates
// 32 different pairs and each entry meets each lane once.  The entry data
// sit twice in shared memory (entries 0..31, then again), so lane l's read
// at step s is element l + s with the step as an immediate offset.  An
// entry's j-side sums travel with it: after each step every lane hands its
// j-side partials to lane l - 1, which meets that entry next; after 32
// steps lane e holds entry e's sums.  The column masks are transposed once
// per chunk so that bit s of a lane's mask word is its pair at step s.
// Lennard-Jones tables of up to this many (A, B) entries (all systems of the
// batch together) are read from shared memory in pass 2.
constexpr int kLjShared = 4096;

template <bool KAPPA, bool LJS>
__global__ void __launch_bounds__(256, 3) k_gbpair(const DevTables t) {
  // per warp, the chunk's 32 entries twice: (x, y, z relative to the i-tile's
  // reference point, q), (R, sqrt(log2 e / 4) / R, Lennard-Jones row) and,
  // for chunks with close pairs, (the low parts of x, y, z, the slot)
  __shared__ float4 sm_a[8][64];
  __shared__ float4 sm_b[8][64];
  __shared__ float4 sm_e[8][64];
  // the batch's Lennard-Jones table and, after it, one zero entry (the
  // coefficients of an excluded pair)
  __shared__ float2 s_lj[LJS ? kLjShared + 1 : 1];
  if (LJS) {  // a static table: staged before the wait
    for (int i = threadIdx.x; i < t.lj_n; i += blockDim.x) s_lj[i] = t.lj[i];
    if (threadIdx.x == 0) s_lj[t.lj_n] = make_float2(0.0f, 0.0f);
    __syncthreads();
  }
  pdl_wait();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nchunk = *t.la.nchunk;
  const int zero_lj = t.lj_n;
  const int next = (lane + 1) & 31;
  int cur_I = -1, cur_sys = -1;
  float3 cref = make_float3(0.f, 0.f, 0.f);
  float xi = 0, yi = 0, zi = 0, xil = 0, yil = 0, zil = 0, qi = 0, ri = 1, rvi = 0;
  int lj_i = 0, lj_full_i = 0, nt = 1;
  const float2 *lj = t.lj;
  long long fx64 = 0, fy64 = 0, fz64 = 0, sd64 = 0, ep64 = 0, ee64 = 0, ev64 = 0;
  const float FS = 4294967296.0f;
  const double FSD = 4294967296.0;
  // kappa = 0: dielfac is a constant, applied once per chunk to the GB
  // energy and the sumdeijda sums (the 1/2 of eff.c's temp5 with it)
  const float dielfac = t.pair.dielfac0;
  const float ep_scale = KAPPA ? 1.0f : dielfac, sd_scale = KAPPA ? 0.5f : 0.5f * dielfac;
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
  // Coulomb and Lennard-Jones of a close pair in FP64 (eff.c:2004-2025),
  // from the exact relative coordinates (i: high + low parts; entry: its
  // rounded value and remainder), added to the fixed-point sums directly
  auto close_pair = [&](const float4 &a, const float4 &b, const float4 &e) {
    const double dx = (static_cast<double>(xi) - a.x) + (static_cast<double>(xil) - e.x);
    const double dy = (static_cast<double>(yi) - a.y) + (static_cast<double>(yil) - e.y);
    const double dz = (static_cast<double>(zi) - a.z) + (static_cast<double>(zil) - e.z);
    const double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
    double rinv = rsqrt_ftz(static_cast<float>(r2));
    rinv = rinv * fma(-0.5 * r2 * rinv, rinv, 1.5);  // two Newton steps: FP64 accuracy
    rinv = rinv * fma(-0.5 * r2 * rinv, rinv, 1.5);
    const double r2inv = rinv * rinv;
    const double2 ab = t.lj64[__float_as_int(b.z) + lj_full_i];
    const double eel = static_cast<double>(qi) * a.w * rinv;
    const double r6inv = r2inv * r2inv * r2inv;
    const double f6 = ab.y * r6inv, f12 = ab.x * (r6inv * r6inv);
    const double de = -(12.0 * f12 - 6.0 * f6 + eel) * r2inv;
    const long long gx = __double2ll_rn(de * dx * FSD), gy = __double2ll_rn(de * dy * FSD),
                    gz = __double2ll_rn(de * dz * FSD);
    fx64 += gx;
    fy64 += gy;
    fz64 += gz;
    const int sj = __float_as_int(e.w);
    atomic_add_ll(&t.acc_fx[sj], -gx);
    atomic_add_ll(&t.acc_fy[sj], -gy);
    atomic_add_ll(&t.acc_fz[sj], -gz);
    ee64 += __double2ll_rn(eel * FSD);
    ev64 += __double2ll_rn((f12 - f6) * FSD);
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
        nt = t.sys_ntypes[sys];
        lj = t.lj + t.sys_lj_off[sys];
      }
      if (I != cur_I) {
        if (cur_I >= 0) flush_i();
        cur_I = I;
        fx64 = fy64 = fz64 = sd64 = 0;
        const int sl = I * 32 + lane;
        cref = tile_ref(t.box_lo, t.box_hi, I);
        const float4 h = t.pos_hi[sl], l = t.pos_lo[sl];
        rel_coord(h.x, l.x, cref.x, xi, xil);
        rel_coord(h.y, l.y, cref.y, yi, yil);
        rel_coord(h.z, l.z, cref.z, zi, zil);
        qi = h.w;
        ri = t.reff32[sl];
        rvi = t.rinv2[sl];
        const int ti = t.param[sl] & 0xffff;
        lj_full_i = t.sys_lj_off[sys] + ti;
        lj_i = LJS ? lj_full_i : ti;
      }
      // stage the chunk's entries (lane e: entry e), twice
      const size_t e = static_cast<size_t>(k) * 32 + lane;
      const unsigned mycol = t.la.col[e];
      const unsigned myexc = t.la.exc[e];
      const unsigned myclose = t.la.close[e];
      const int sj = SFFG_IDX(t.la.slot[e], t.nslot, kCheckSlot);
      const bool any_close = __any_sync(kFull, myclose != 0u);
      {
        const float4 h = t.pos_hi[sj], l = t.pos_lo[sj];
        float dx, dy, dz, ex, ey, ez;
        rel_coord(h.x, l.x, cref.x, dx, ex);
        rel_coord(h.y, l.y, cref.y, dy, ey);
        rel_coord(h.z, l.z, cref.z, dz, ez);
        const float4 a = make_float4(dx, dy, dz, h.w);
        const float4 b = make_float4(t.reff32[sj], t.rinv2[sj], __int_as_float((t.param[sj] & 0xffff) * nt), 0.0f);
        sm_a[w][lane] = a;
        sm_a[w][lane + 32] = a;
        sm_b[w][lane] = b;
        sm_b[w][lane + 32] = b;
        if (any_close) {
          const float4 c = make_float4(ex, ey, ez, __int_as_float(sj));
          sm_e[w][lane] = c;
          sm_e[w][lane + 32] = c;
        }
      }
      const unsigned m_in = rotation_mask(mycol, lane);
      const unsigned m_coul = __any_sync(kFull, myexc != 0u) ? m_in & ~rotation_mask(myexc, lane) : m_in;
      // pairs that were within kClose + 1 A at the list build (not excluded)
      const unsigned m_close = any_close ? rotation_mask(myclose, lane) : 0u;
      __syncwarp();
      float fix = 0, fiy = 0, fiz = 0, sdi = 0, ep = 0, ee = 0, ev = 0;
      float jx = 0, jy = 0, jz = 0, jsd = 0;  // j-side sums of the entry this lane meets
      // the 32 steps of the rotation; CLOSE: the chunk holds pairs that may
      // be closer than kClose now, whose Coulomb and Lennard-Jones terms
      // then go to close_pair (FP64) instead of the FP32 sums
      auto steps = [&](auto close_tag) {
        constexpr bool CLOSE = decltype(close_tag)::value;
#pragma unroll 1
        for (int g = 0; g < 32; g += 8) {
          const unsigned gin = m_in >> g, gcoul = m_coul >> g, gclose = m_close >> g;
          const float4 *pa = &sm_a[w][lane + g];
          const float4 *pb = &sm_b[w][lane + g];
#pragma unroll
          for (int u = 0; u < 8; u++) {
            const float4 a = pa[u], b = pb[u];
            const bool in = (gin >> u) & 1u;
            bool coul = (gcoul >> u) & 1u;
            const float dx = (xi - a.x) + xil;
            const float dy = (yi - a.y) + yil;
            const float dz = (zi - a.z) + zil;
            // a lane off the list gets r2 = 1 and zero charges and
            // coefficients (the self pair of a diagonal tile has r2 = 0), so
            // its terms are exact zeros
            const float r2 = in ? fmaf(dx, dx, fmaf(dy, dy, dz * dz)) : 1.0f;
            bool cl = false;
            if (CLOSE) {
              cl = ((gclose >> u) & 1u) && r2 < kClose * kClose;
              coul = coul && !cl;
            }
            const float qij = qi * a.w;
            const float qq = in ? qij : 0.0f;
            const float qc = coul ? qij : 0.0f;
            float lja, ljb;
            if (LJS) {
              const float2 ab = s_lj[SFFG_IDX(coul ? __float_as_int(b.z) + lj_i : zero_lj, t.lj_n + 1, kCheckLj)];
              lja = ab.x;
              ljb = ab.y;
            } else {
#ifdef SFFG_CHECKED
              const float2 ab = t.lj[SFFG_IDX(static_cast<int>(lj - t.lj) + __float_as_int(b.z) + lj_i, t.lj_n,
                                              kCheckLj)];
#else
              const float2 ab = lj[__float_as_int(b.z) + lj_i];
#endif
              lja = coul ? ab.x : 0.0f;
              ljb = coul ? ab.y : 0.0f;
            }
            // generalized Born (eff.c:1924-1987)
            const float rb2 = ri * b.x;
            const float efac = ex2_ftz(-r2 * (rvi * b.y));
            const float f2 = fmaf(rb2, efac, r2);
            const float fgbi = rsqrt_ftz(f2);
            const float temp4 = fgbi * fgbi * fgbi;
            float de, temp5;
            if (KAPPA) {
              const float fgbk = -t.pair.kappa_s * (f2 * fgbi);
              const float expmkf = expf(fgbk) * t.pair.inv_epsext;
              const float dfac = 1.0f - expmkf;
              const float temp6 = qq * temp4 * (dfac + fgbk * expmkf);
              ep = fmaf(qq * dfac, fgbi, ep);
              de = temp6 * fmaf(-0.25f, efac, 1.0f);
              temp5 = efac * temp6 * fmaf(0.25f, r2, rb2);
            } else {
              // dielfac factored out of temp6 (into de below, and into the
              // energy and sumdeijda scales)
              const float temp6 = qq * temp4;
              ep = fmaf(qq, fgbi, ep);
              de = dielfac * (temp6 * fmaf(-0.25f, efac, 1.0f));
              temp5 = efac * temp6 * fmaf(0.25f, r2, rb2);
            }
            sdi += temp5;
            // Coulomb and Lennard-Jones (eff.c:2004-2025), zero for excluded
            // and close pairs
            const float rinv = rsqrt_ftz(r2);
            const float r2inv = rinv * rinv;
            const float eel = qc * rinv;
            const float r6inv = r2inv * r2inv * r2inv;
            const float f6 = ljb * r6inv;
            const float f12 = lja * (r6inv * r6inv);
            ee += eel;
            ev += f12 - f6;
            de = fmaf(-fmaf(12.0f, f12, fmaf(-6.0f, f6, eel)), r2inv, de);
            fix = fmaf(de, dx, fix);
            fiy = fmaf(de, dy, fiy);
            fiz = fmaf(de, dz, fiz);
            jx = fmaf(-de, dx, jx);
            jy = fmaf(-de, dy, jy);
            jz = fmaf(-de, dz, jz);
            jsd += temp5;
            if (CLOSE) {
              if (__any_sync(kFull, cl)) {
                if (cl) close_pair(a, b, sm_e[w][lane + g + u]);
              }
            }
            // hand the entry's sums to the lane that meets it next
            jx = __shfl_sync(kFull, jx, next);
            jy = __shfl_sync(kFull, jy, next);
            jz = __shfl_sync(kFull, jz, next);
            jsd = __shfl_sync(kFull, jsd, next);
          }
        }
      };
      if (any_close) steps(std::true_type());
      else steps(std::false_type());
      fx64 += to_fixed(fix, FS);
      fy64 += to_fixed(fiy, FS);
      fz64 += to_fixed(fiz, FS);
      sd64 += to_fixed(sdi * (sd_scale * ri), FS);
      ep64 += to_fixed(ep * ep_scale, FS);
      ee64 += to_fixed(ee, FS);
      ev64 += to_fixed(ev, FS);
      // after 32 hand-overs lane e holds entry e's sums
      if (mycol) {
        atomic_add_ll(&t.acc_fx[sj], to_fixed(jx, FS));
        atomic_add_ll(&t.acc_fy[sj], to_fixed(jy, FS));
        atomic_add_ll(&t.acc_fz[sj], to_fixed(jz, FS));
        atomic_add_ll(&t.acc_sd[sj], to_fixed(jsd * (sd_scale * sm_b[w][lane].x), FS));
      }
      __syncwarp();
    }
  }
  if (cur_I >= 0) flush_i();
  if (cur_sys >= 0) flush_e();
}

// ------------------------------------------------------------------ pass 3
// Chain rule through the Born radii (src/sff/eff.c:2241-2395) over lists
// B and C: for each pair within rgbmax + Fsmax, g = sumda_i d_ij +
// sumda_j d_ji, f_i -= g r_ij, f_j += g r_ij.
template <bool NECK, bool POLY>
__global__ void __launch_bounds__(256, 3) k_chain(const DevTables t) {
  // far-field chunks (list B): per warp the entries twice, (x, y, z
  // relative to the i-tile's reference point, s) and (s correction, s^2,
  // sumda, rborn); the neck index apart
  __shared__ float4 sm_a[8][64], sm_b[8][64];
  __shared__ int sm_nk[NECK ? 8 : 1][64];
  // near-field chunks (list C)
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
  const float rgbmax = t.born.rgbmax;
  const int next = (lane + 1) & 31;
  int cur_I = -1;
  float3 cref = make_float3(0.f, 0.f, 0.f);
  float xi = 0, yi = 0, zi = 0, xil = 0, yil = 0, zil = 0, si = 0, si2 = 0, rbi = 0, sci = 0, sdai = 0;
  int nki = 0;
  // the i-tile's system: (rgbmax + Fsmax)^2 over its own atoms, and whether
  // its rgbmax tails take the polynomial form
  float cut2 = 0.0f;
  bool tpoly = false;
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

  // list B chunk k, rotation schedule
  auto far_chunk = [&](int k) {
    const size_t e = static_cast<size_t>(k) * 32 + lane;
    const unsigned mycol = t.lb.col[e];
    const int sj = SFFG_IDX(t.lb.slot[e], t.nslot, kCheckSlot);
    {
      const float4 h = t.pos_hi[sj], l = t.pos_lo[sj], g = t.gbpar[sj];
      float dx, dy, dz, ex, ey, ez;
      rel_coord(h.x, l.x, cref.x, dx, ex);
      rel_coord(h.y, l.y, cref.y, dy, ey);
      rel_coord(h.z, l.z, cref.z, dz, ez);
      const float4 a = make_float4(dx, dy, dz, g.y);
      const float4 b = make_float4(g.w, g.y * g.y, t.sumda32[sj], g.z);
      sm_a[w][lane] = a;
      sm_a[w][lane + 32] = a;
      sm_b[w][lane] = b;
      sm_b[w][lane + 32] = b;
      if (NECK) {
        const int nk = (t.param[sj] >> 16) & 0xff;
        sm_nk[NECK ? w : 0][lane] = nk;
        sm_nk[NECK ? w : 0][lane + 32] = nk;
      }
    }
    const unsigned m_in = rotation_mask(mycol, lane);
    __syncwarp();
    float fix = 0, fiy = 0, fiz = 0, jx = 0, jy = 0, jz = 0;
#pragma unroll 1
    for (int g = 0; g < 32; g += 4) {
      const unsigned gin = m_in >> g;
      const float4 *pa = &sm_a[w][lane + g];
      const float4 *pb = &sm_b[w][lane + g];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const float4 a = pa[u];
        const float4 b = pb[u];
        const bool in = (gin >> u) & 1u;
        const float dx = (xi - a.x) + xil;
        const float dy = (yi - a.y) + yil;
        const float dz = (zi - a.z) + zil;
        float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        // off the list, or beyond rgbmax + Fsmax, where the reference skips
        // the pair (eff.c:2263)
        r2 = in && r2 <= cut2 ? r2 : kOffList;
        // the hardware rsqrt alone: pass 3 only shapes the forces
        const float d1 = rsqrt_ftz(r2);
        const float d2i = d1 * d1;
        const f2 S = pk(a.w, si);
        float di, dj;
        upk(far_deriv_x2(d2i, S, pk(b.y, si2)), di, dj);
        const float dij = r2 * d1;
        {
          const bool qi_ = dij > rgbmax - a.w, qj_ = dij > rgbmax - si;
          float vi, vj;
          if (POLY || tpoly) {
            upk(tail_x2<true>(t.born, dij, d1, S), vi, vj);
          } else {
            vi = tail_closed<true>(t.born, dij, d1, a.w);
            vj = tail_closed<true>(t.born, dij, d1, si);
          }
          di = qi_ ? vi : di;
          dj = qj_ ? vj : dj;
          di = dij > rgbmax + a.w ? 0.0f : di;
          dj = dij > rgbmax + si ? 0.0f : dj;
        }
        di = fmaf(di, b.x, di);
        dj = fmaf(dj, sci, dj);
        if (NECK) {
          const bool nk = dij < rbi + b.w + 6.8f;
          if (__any_sync(kFull, nk)) {
            const int nkj = sm_nk[NECK ? w : 0][lane + g + u];
            const int ij = SFFG_IDX(nki * 21 + nkj, 441, kCheckNeck), ji = SFFG_IDX(nkj * 21 + nki, 441, kCheckNeck);
            const float na = neck_deriv(dij, s_npos[ij], s_nval[ij], t.neck_scale);
            const float nb = neck_deriv(dij, s_npos[ji], s_nval[ji], t.neck_scale);
            // only for pairs within rgbmax + s (eff.c:2288-2289, 2330-2345)
            di += nk && dij <= rgbmax + a.w ? na : 0.0f;
            dj += nk && dij <= rgbmax + si ? nb : 0.0f;
          }
        }
        const float gg = fmaf(sdai, di, b.z * dj);
        fix = fmaf(-gg, dx, fix);
        fiy = fmaf(-gg, dy, fiy);
        fiz = fmaf(-gg, dz, fiz);
        jx = __shfl_sync(kFull, fmaf(gg, dx, jx), next);
        jy = __shfl_sync(kFull, fmaf(gg, dy, jy), next);
        jz = __shfl_sync(kFull, fmaf(gg, dz, jz), next);
      }
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
        if (r2 <= cut2) {
          const float d1 = rsqrt_nr(r2);
          const float dij = r2 * d1;
          float di = descreen_deriv<!POLY>(t.born, dij, r2, d1, gi.x, gp.y);
          float dj = descreen_deriv<!POLY>(t.born, dij, r2, d1, gp.x, gi.y);
          di = fmaf(di, gp.w, di);
          dj = fmaf(dj, gi.w, dj);
          if (NECK && dij < gi.z + gp.z + 6.8f) {
            const int nkp = (si_par[w][il] >> 16) & 0xff, nkj = (sm_par[w][jl] >> 16) & 0xff;
            if (dij <= t.born.rgbmax + gp.y)
              di += neck_deriv(dij, s_npos[SFFG_IDX(nkp * 21 + nkj, 441, kCheckNeck)], s_nval[SFFG_IDX(nkp * 21 + nkj, 441, kCheckNeck)], t.neck_scale);
            if (dij <= t.born.rgbmax + gi.y)
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
      const int sys = t.tile_sys[I];
      if (!t.sys_active[sys]) continue;
      if (I != cur_I) {
        const float2 sb = t.sys_born[sys];
        cut2 = sb.x;
        tpoly = sb.y != 0.0f;
        if (cur_I >= 0) flush_i();
        cur_I = I;
        fx64 = fy64 = fz64 = 0;
        const int sl = I * 32 + lane;
        const float4 h = t.pos_hi[sl], g = t.gbpar[sl];
        float4 l = t.pos_lo[sl];
        const int pr = t.param[sl];
        cref = tile_ref(t.box_lo, t.box_hi, I);
        rel_coord(h.x, l.x, cref.x, xi, xil);
        rel_coord(h.y, l.y, cref.y, yi, yil);
        rel_coord(h.z, l.z, cref.z, zi, zil);
        si = g.y; si2 = g.y * g.y; rbi = g.z; sci = g.w;
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
