// Device kernels of the generalized-Born path (sm_103a).
//
// The three pair passes of the reference's egb() (src/sff/eff.c:1566-1733,
// 1770-2066, 2131-2405) run over a list of 32x32 atom-tile pairs.  A warp
// owns one tile pair at a time: lane l holds i-atom l of the i-tile in
// registers; the 32 j-atoms are staged in shared memory and read by
// broadcast, so at step s every lane pairs its i-atom with j-atom s.  Both
// directions of each unordered pair are handled in one visit (Newton's
// third law); the j-side partial sums, spread over the 32 lanes, are folded
// with a shuffle transpose-reduction every 8 steps.  Per tile pair the FP32
// partial sums are converted to 64-bit fixed point, so the totals do not
// depend on how tile pairs are scheduled.
#pragma once

#include <cstdint>

#include "gbmath.cuh"

namespace sffg {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kChunk = 4;  // tile pairs a warp claims per work-queue grab

// Work item: i-tile, j-tile (j >= i), index of the in-list bit mask (-1:
// every valid pair is on the list) and of the exclusion bit mask (-1: none).
using Item = int4;

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
  const unsigned *tile_valid;
  const int *tile_sys;
  const float4 *box_lo, *box_hi;
  // per system
  const int *sys_active;
  const int *sys_lj_off;
  const int *sys_ntypes;
  const float2 *lj;       // (A, B) per type pair, per system blocks
  // lists
  const Item *items;
  const int *nitems;
  const unsigned *masks;
  const unsigned *excl_masks;
  int *counter;
  // accumulators
  long long *acc_sumi, *acc_sd, *acc_fx, *acc_fy, *acc_fz;
  long long *energy;       // nsys * E_NSLOTS
  // model
  BornConst born;
  PairConst pair;
  float neck_scale;
  const float *neck_pos, *neck_val;  // 441 each
};

__device__ __forceinline__ long long to_fixed(float v, float scale) {
  return __float2ll_rn(v * scale);
}

// Sum of v[e] over the 32 lanes for e = 0..7, delivered to lane 8*g + e
// (zero in the other lanes).
__device__ __forceinline__ float reduce8_to_lane(const float (&v)[8], int g, int lane) {
  const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
  float a[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    float send = b4 ? v[k] : v[k + 4];
    float keep = b4 ? v[k + 4] : v[k];
    a[k] = keep + __shfl_xor_sync(kFull, send, 16);
  }
  float b[2];
#pragma unroll
  for (int k = 0; k < 2; k++) {
    float send = b3 ? a[k] : a[k + 2];
    float keep = b3 ? a[k + 2] : a[k];
    b[k] = keep + __shfl_xor_sync(kFull, send, 8);
  }
  float send = b2 ? b[0] : b[1];
  float keep = b2 ? b[1] : b[0];
  float c = keep + __shfl_xor_sync(kFull, send, 4);
  c += __shfl_xor_sync(kFull, c, 2);
  c += __shfl_xor_sync(kFull, c, 1);
  float r = __shfl_sync(kFull, c, (lane & 7) << 2);
  return ((lane >> 3) == g) ? r : 0.0f;
}

__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

__device__ __forceinline__ void atomic_add_ll(long long *p, long long v) {
  if (v != 0) atomicAdd(reinterpret_cast<unsigned long long *>(p), static_cast<unsigned long long>(v));
}

// Claims the next chunk of the work queue for this warp.
__device__ __forceinline__ int claim_chunk(int *counter, int lane) {
  int base = 0;
  if (lane == 0) base = atomicAdd(counter, kChunk);
  return __shfl_sync(kFull, base, 0);
}

// Rows of the in-list mask for this lane's i-atom against the j-tile.
__device__ __forceinline__ unsigned row_mask(const DevTables &t, const Item &it, int lane) {
  const unsigned vI = t.tile_valid[it.x];
  unsigned row = it.z < 0 ? t.tile_valid[it.y] : t.masks[static_cast<size_t>(it.z) * 32 + lane];
  if (!((vI >> lane) & 1u)) row = 0u;
  if (it.x == it.y) row &= lane < 31 ? (kFull << (lane + 1)) : 0u;
  return row;
}

// Squared distance between two tiles' bounding boxes.
__device__ __forceinline__ float box_dist2(const DevTables &t, int I, int J) {
  const float4 al = t.box_lo[I], ah = t.box_hi[I], bl = t.box_lo[J], bh = t.box_hi[J];
  float dx = fmaxf(0.0f, fmaxf(al.x - bh.x, bl.x - ah.x));
  float dy = fmaxf(0.0f, fmaxf(al.y - bh.y, bl.y - ah.y));
  float dz = fmaxf(0.0f, fmaxf(al.z - bh.z, bl.z - ah.z));
  return dx * dx + dy * dy + dz * dz;
}

// ------------------------------------------------------------------ pass 1
// Born-radius descreening sums (src/sff/eff.c:1566-1709): both directions
// of every listed pair within rgbmax + Fsmax.
template <bool NECK>
__global__ void __launch_bounds__(256, 2) k_born(const DevTables t) {
  __shared__ float4 sm_hi[8][32], sm_lo[8][32], sm_gb[8][32];
  __shared__ int sm_par[8][32];
  __shared__ float s_npos[NECK ? 441 : 1], s_nval[NECK ? 441 : 1];
  if (NECK) {
    for (int i = threadIdx.x; i < 441; i += blockDim.x) {
      s_npos[i] = t.neck_pos[i];
      s_nval[i] = t.neck_val[i];
    }
    __syncthreads();
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nitems = *t.nitems;
  const float cut2 = t.born.cutoff2 * 1.0001f + 1e-3f;
  int cur_I = -1;
  float xi = 0, yi = 0, zi = 0, xli = 0, yli = 0, zli = 0, rhoi = 1, si = 0, rbi = 0, sci = 0;
  int nki = 0;
  long long sumi64 = 0;
  for (;;) {
    const int base = claim_chunk(t.counter, lane);
    if (base >= nitems) break;
    const int end = min(base + kChunk, nitems);
    for (int k = base; k < end; k++) {
      const Item it = t.items[k];
      const int I = it.x, J = it.y;
      if (!t.sys_active[t.tile_sys[I]]) continue;
      if (box_dist2(t, I, J) > cut2) continue;
      if (I != cur_I) {
        if (cur_I >= 0) atomic_add_ll(&t.acc_sumi[cur_I * 32 + lane], sumi64);
        cur_I = I;
        sumi64 = 0;
        const int sl = I * 32 + lane;
        const float4 h = t.pos_hi[sl], l = t.pos_lo[sl], g = t.gbpar[sl];
        xi = h.x; yi = h.y; zi = h.z; xli = l.x; yli = l.y; zli = l.z;
        rhoi = g.x; si = g.y; rbi = g.z; sci = g.w;
        nki = (t.param[sl] >> 16) & 0xff;
      }
      const int sj = J * 32 + lane;
      sm_hi[w][lane] = t.pos_hi[sj];
      sm_lo[w][lane] = t.pos_lo[sj];
      sm_gb[w][lane] = t.gbpar[sj];
      if (NECK) sm_par[w][lane] = t.param[sj];
      const unsigned row = row_mask(t, it, lane);
      const unsigned cols = __reduce_or_sync(kFull, row);
      __syncwarp();
      float acc_i = 0.0f, acc_j = 0.0f;
#pragma unroll 1
      for (int g = 0; g < 4; g++) {
        float aj[8];
#pragma unroll
        for (int s = 0; s < 8; s++) {
          const int j = g * 8 + s;
          aj[s] = 0.0f;
          if (!((cols >> j) & 1u)) continue;  // j listed for no lane
          const float4 h = sm_hi[w][j], l = sm_lo[w][j], gp = sm_gb[w][j];
          const float dx = (xi - h.x) + (xli - l.x);
          const float dy = (yi - h.y) + (yli - l.y);
          const float dz = (zi - h.z) + (zli - l.z);
          const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          const bool in = ((row >> j) & 1u) && r2 <= t.born.cutoff2;
          if (!__any_sync(kFull, in)) continue;  // every lane out of range
          const float dij1i = rsqrt_nr(r2);
          const float dij = r2 * dij1i;
          float ti = descreen(t.born, dij, r2, dij1i, rhoi, gp.y);
          float tj = descreen(t.born, dij, r2, dij1i, gp.x, si);
          ti = fmaf(ti, gp.w, ti);
          tj = fmaf(tj, sci, tj);
          if (NECK) {
            if (dij < rbi + gp.z + 6.8f) {
              const int nkj = (sm_par[w][j] >> 16) & 0xff;
              ti += neck_term(dij, s_npos[nki * 21 + nkj], s_nval[nki * 21 + nkj], t.neck_scale);
              tj += neck_term(dij, s_npos[nkj * 21 + nki], s_nval[nkj * 21 + nki], t.neck_scale);
            }
          }
          acc_i += in ? ti : 0.0f;
          aj[s] = in ? tj : 0.0f;
        }
        acc_j += reduce8_to_lane(aj, g, lane);
      }
      sumi64 += to_fixed(acc_i, 1099511627776.0f);
      if ((t.tile_valid[J] >> lane) & 1u) atomic_add_ll(&t.acc_sumi[sj], to_fixed(acc_j, 1099511627776.0f));
      __syncwarp();
    }
  }
  if (cur_I >= 0) atomic_add_ll(&t.acc_sumi[cur_I * 32 + lane], sumi64);
}

// ------------------------------------------------------------------ pass 2
// GB + Coulomb + Lennard-Jones pair energies, dE/dr and sumdeijda
// (src/sff/eff.c:1902-2063).
template <bool KAPPA>
__global__ void __launch_bounds__(256, 2) k_gbpair(const DevTables t) {
  __shared__ float4 sm_hi[8][32], sm_lo[8][32];
  __shared__ float2 sm_aux[8][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nitems = *t.nitems;
  int cur_I = -1, cur_sys = -1;
  float xi = 0, yi = 0, zi = 0, xli = 0, yli = 0, zli = 0, qi = 0, ri = 1, rvi = 0;
  int ti = 0, nt = 1;
  const float2 *lj = t.lj;
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
      atomic_add_ll(&t.energy[cur_sys * 8 + 0], -a);
      atomic_add_ll(&t.energy[cur_sys * 8 + 1], b);
      atomic_add_ll(&t.energy[cur_sys * 8 + 2], c);
    }
    ep64 = ee64 = ev64 = 0;
  };
  for (;;) {
    const int base = claim_chunk(t.counter, lane);
    if (base >= nitems) break;
    const int end = min(base + kChunk, nitems);
    for (int k = base; k < end; k++) {
      const Item it = t.items[k];
      const int I = it.x, J = it.y;
      const int sys = t.tile_sys[I];
      if (!t.sys_active[sys]) continue;
      if (sys != cur_sys) {
        if (cur_sys >= 0) flush_e();
        cur_sys = sys;
        lj = t.lj + t.sys_lj_off[sys];
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
        ti = (t.param[sl] & 0xffff) * nt;
      }
      const int sj = J * 32 + lane;
      {
        float4 l = t.pos_lo[sj];
        l.w = t.reff32[sj];
        sm_hi[w][lane] = t.pos_hi[sj];
        sm_lo[w][lane] = l;
        sm_aux[w][lane] = make_float2(t.rinv2[sj], __int_as_float(t.param[sj] & 0xffff));
      }
      const unsigned row = row_mask(t, it, lane);
      const unsigned cols = __reduce_or_sync(kFull, row);
      const unsigned exr = it.w < 0 ? 0u : t.excl_masks[static_cast<size_t>(it.w) * 32 + lane];
      __syncwarp();
      float fix = 0, fiy = 0, fiz = 0, sdi = 0, ep = 0, ee = 0, ev = 0;
      float jx = 0, jy = 0, jz = 0, jsd = 0;
#pragma unroll 1
      for (int g = 0; g < 4; g++) {
        float ax[8], ay[8], az[8], as[8];
#pragma unroll
        for (int s = 0; s < 8; s++) {
          const int j = g * 8 + s;
          ax[s] = ay[s] = az[s] = as[s] = 0.0f;
          if (!((cols >> j) & 1u)) continue;  // j listed for no lane
          const float4 h = sm_hi[w][j], l = sm_lo[w][j];
          const float2 au = sm_aux[w][j];
          const float dx = (xi - h.x) + (xli - l.x);
          const float dy = (yi - h.y) + (yli - l.y);
          const float dz = (zi - h.z) + (zli - l.z);
          const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          const bool in = (row >> j) & 1u;
          const bool coul = !((exr >> j) & 1u);
          const float2 ab = lj[ti + __float_as_int(au.y)];
          const PairOut o = gb_pair<KAPPA>(t.pair, r2, qi * h.w, ri, l.w, rvi, au.x, coul, ab.x, ab.y);
          const float de = in ? o.de : 0.0f;
          fix = fmaf(de, dx, fix);
          fiy = fmaf(de, dy, fiy);
          fiz = fmaf(de, dz, fiz);
          ax[s] = -de * dx;
          ay[s] = -de * dy;
          az[s] = -de * dz;
          sdi += in ? o.sd_i : 0.0f;
          as[s] = in ? o.sd_j : 0.0f;
          ep += in ? o.epol : 0.0f;
          ee += in ? o.eel : 0.0f;
          ev += in ? o.evdw : 0.0f;
        }
        jx += reduce8_to_lane(ax, g, lane);
        jy += reduce8_to_lane(ay, g, lane);
        jz += reduce8_to_lane(az, g, lane);
        jsd += reduce8_to_lane(as, g, lane);
      }
      fx64 += to_fixed(fix, FS);
      fy64 += to_fixed(fiy, FS);
      fz64 += to_fixed(fiz, FS);
      sd64 += to_fixed(sdi, FS);
      ep64 += to_fixed(ep, FS);
      ee64 += to_fixed(ee, FS);
      ev64 += to_fixed(ev, FS);
      if ((t.tile_valid[J] >> lane) & 1u) {
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
// Chain rule through the Born radii (src/sff/eff.c:2241-2395): for each
// listed pair, g = sumda_i d_ij + sumda_j d_ji, f_i -= g r_ij, f_j += g r_ij.
template <bool NECK>
__global__ void __launch_bounds__(256, 2) k_chain(const DevTables t) {
  __shared__ float4 sm_hi[8][32], sm_lo[8][32], sm_gb[8][32];
  __shared__ int sm_par[8][32];
  __shared__ float s_npos[NECK ? 441 : 1], s_nval[NECK ? 441 : 1];
  if (NECK) {
    for (int i = threadIdx.x; i < 441; i += blockDim.x) {
      s_npos[i] = t.neck_pos[i];
      s_nval[i] = t.neck_val[i];
    }
    __syncthreads();
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nitems = *t.nitems;
  const float cut2 = t.born.cutoff2 * 1.0001f + 1e-3f;
  const float FS = 4294967296.0f;
  int cur_I = -1;
  float xi = 0, yi = 0, zi = 0, xli = 0, yli = 0, zli = 0, rhoi = 1, si = 0, rbi = 0, sci = 0, sdai = 0;
  int nki = 0;
  long long fx64 = 0, fy64 = 0, fz64 = 0;
  auto flush_i = [&]() {
    const int sl = cur_I * 32 + lane;
    atomic_add_ll(&t.acc_fx[sl], fx64);
    atomic_add_ll(&t.acc_fy[sl], fy64);
    atomic_add_ll(&t.acc_fz[sl], fz64);
  };
  for (;;) {
    const int base = claim_chunk(t.counter, lane);
    if (base >= nitems) break;
    const int end = min(base + kChunk, nitems);
    for (int k = base; k < end; k++) {
      const Item it = t.items[k];
      const int I = it.x, J = it.y;
      if (!t.sys_active[t.tile_sys[I]]) continue;
      if (box_dist2(t, I, J) > cut2) continue;
      if (I != cur_I) {
        if (cur_I >= 0) flush_i();
        cur_I = I;
        fx64 = fy64 = fz64 = 0;
        const int sl = I * 32 + lane;
        const float4 h = t.pos_hi[sl], l = t.pos_lo[sl], g = t.gbpar[sl];
        xi = h.x; yi = h.y; zi = h.z; xli = l.x; yli = l.y; zli = l.z;
        rhoi = g.x; si = g.y; rbi = g.z; sci = g.w;
        sdai = t.sumda32[sl];
        nki = (t.param[sl] >> 16) & 0xff;
      }
      const int sj = J * 32 + lane;
      {
        float4 l = t.pos_lo[sj];
        l.w = t.sumda32[sj];
        sm_hi[w][lane] = t.pos_hi[sj];
        sm_lo[w][lane] = l;
        sm_gb[w][lane] = t.gbpar[sj];
        if (NECK) sm_par[w][lane] = t.param[sj];
      }
      const unsigned row = row_mask(t, it, lane);
      const unsigned cols = __reduce_or_sync(kFull, row);
      __syncwarp();
      float fix = 0, fiy = 0, fiz = 0, jx = 0, jy = 0, jz = 0;
#pragma unroll 1
      for (int g = 0; g < 4; g++) {
        float ax[8], ay[8], az[8];
#pragma unroll
        for (int s = 0; s < 8; s++) {
          const int j = g * 8 + s;
          ax[s] = ay[s] = az[s] = 0.0f;
          if (!((cols >> j) & 1u)) continue;
          const float4 h = sm_hi[w][j], l = sm_lo[w][j], gp = sm_gb[w][j];
          const float dx = (xi - h.x) + (xli - l.x);
          const float dy = (yi - h.y) + (yli - l.y);
          const float dz = (zi - h.z) + (zli - l.z);
          const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          const bool in = ((row >> j) & 1u) && r2 <= t.born.cutoff2;
          if (!__any_sync(kFull, in)) continue;
          const float dij1i = rsqrt_nr(r2);
          const float dij = r2 * dij1i;
          float di = descreen_deriv(t.born, dij, r2, dij1i, rhoi, gp.y);
          float dj = descreen_deriv(t.born, dij, r2, dij1i, gp.x, si);
          di = fmaf(di, gp.w, di);
          dj = fmaf(dj, sci, dj);
          if (NECK) {
            if (dij < rbi + gp.z + 6.8f) {
              const int nkj = (sm_par[w][j] >> 16) & 0xff;
              di += neck_deriv(dij, s_npos[nki * 21 + nkj], s_nval[nki * 21 + nkj], t.neck_scale);
              dj += neck_deriv(dij, s_npos[nkj * 21 + nki], s_nval[nkj * 21 + nki], t.neck_scale);
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
        jx += reduce8_to_lane(ax, g, lane);
        jy += reduce8_to_lane(ay, g, lane);
        jz += reduce8_to_lane(az, g, lane);
      }
      fx64 += to_fixed(fix, FS);
      fy64 += to_fixed(fiy, FS);
      fz64 += to_fixed(fiz, FS);
      if ((t.tile_valid[J] >> lane) & 1u) {
        atomic_add_ll(&t.acc_fx[sj], to_fixed(jx, FS));
        atomic_add_ll(&t.acc_fy[sj], to_fixed(jy, FS));
        atomic_add_ll(&t.acc_fz[sj], to_fixed(jz, FS));
      }
      __syncwarp();
    }
  }
  if (cur_I >= 0) flush_i();
}

}  // namespace sffg
