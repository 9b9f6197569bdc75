// Pair lists: the reference's neighbour list (src/sff/nblist.c:813-1240,
// pairs with r < cut at build time, excluded pairs included, pairs of two
// frozen atoms left out, nblist.c:726-746) stored as compacted chunks.
//
// For every i-tile (32 slots) the j-atoms of tiles J >= I that pair with at
// least one of its atoms are packed, 32 per chunk, each with a column mask
// (bit i: the pair with lane i of the i-tile is listed) and, for the cutoff
// list, an exclusion column mask.  A warp of a pair pass takes one chunk:
// its lanes hold the i-tile, its steps walk the 32 packed j-atoms.  Packing
// j-atoms instead of whole 32-atom tiles keeps ~50-60% of the lane-steps
// busy at protein densities, against ~20-35% for tile pairs.
//
// Three lists share one build:
//   list A, pairs with r < cut: pass 2 (GB + Coulomb + LJ) -- exactly the
//           reference's list, rebuilt every nsnb evaluations; its entries
//           also mark the non-excluded pairs closer than kClose + 1 A, whose
//           Coulomb and Lennard-Jones terms pass 2 takes in FP64 once they
//           are closer than kClose;
//   lists B and C, the pairs of list A with r < rgbmax + Fsmax + skin:
//           passes 1 and 3 (Born radii and chain rule), which the reference
//           runs over list A skipping pairs beyond rgbmax + Fsmax at every
//           evaluation.  List C holds the pairs close enough to need the
//           near-field forms of the descreening integral (r < 4 max(s_i,
//           s_j) + skin), list B all others, so the main kernels of passes 1
//           and 3 carry no near-field code.  The entries of a tile are
//           remade from list A (on the device, with no host round trip) as
//           soon as one of its atoms has moved more than skin / 3 since its
//           last remake, so every pair of list A within rgbmax + Fsmax now
//           is on B or C, and no pair of list B has come within
//           4 max(s_i, s_j).  (Splitting list B at rgbmax - Fsmax into pairs
//           that never reach the smooth rgbmax tail and pairs that can was
//           tried: half of list B's j-atoms have pairs on both sides, so the
//           two lists held 1.5 times the lane-steps of one, 27% of them
//           busy in the tail list, which needs the tail form throughout.)
//
// Build stages (one launch each):
//   1 candidates   warp per i-tile: tile pairs (I, J >= I) whose bounding
//                  boxes are within cut
//   2 columns      warp per candidate: column masks of both lists and the
//                  exclusion columns; entry counts
//   3 offsets      warp per i-tile: entry offsets of each candidate within
//                  the i-tile, chunks per i-tile
//   4 scan         one block: first chunk of every i-tile, chunk totals
//   5 fill         warp per candidate: the entries
//   6 pad          warp per i-tile: padding entries and chunk owners
// Stages 2-6 also run in "lists B and C only" mode when the displacement
// check (in k_pack) fires for some tile; each of those launches returns at
// once unless a flag is set, and only the tile pairs with a flagged tile
// get new columns (the others keep theirs), and only flagged tiles take new
// reference positions.  Since a tile pair's columns were made, each of its
// atoms has moved at most 2 x skin/3 from there (skin/3 from its reference
// position, which was at most skin/3 away then) and the flagged tile's
// atoms at most skin/3, so the pair distance has changed by less than the
// skin: no pair within rgbmax + Fsmax is ever missing, none of list B is
// in near-field range; and a system's lists, with the rounding of its
// sums, depend on its own atoms only.
#pragma once

#include "kernels.cuh"

namespace sffg {

constexpr float kListSkin = 0.8f;  // margin of lists B and C, in Angstrom
constexpr float kListMove = kListSkin / 3.0f;  // displacement that remakes a tile's entries

struct ListArgs {
  const float4 *pos_hi, *pos_lo, *box_lo, *box_hi;
  const double *x;
  const float4 *gbpar;  // per slot: .y = screened radius s
  const int *slot_atom, *param;
  const unsigned *tile_valid;
  const int *tile_sys, *sys_tile_end, *sys_active;
  const int *excl_tile_start;  // per tile: range into excl_tile_j / excl_tile_idx
  const int *excl_tile_j, *excl_tile_idx;
  const unsigned *excl_masks;  // per tile pair with exclusions: 32 rows (bit = j lane)
  int ntile;
  float cut2f;   // cut^2 (list A), FP32
  double cut2;   // cut^2, exact FP64 decision for borderline pairs
  const float *sys_gbb2;  // per system (rgbmax + Fsmax + skin)^2, its own Fsmax (lists B and C)
  float close2f; // (kClose + 1 A)^2: list A's possibly close pairs
  // candidates
  int2 *cand;
  int cand_cap;  // candidates the store holds (the column arrays hold as many)
  int ent_cap;   // list chunks each entry store holds
  // overflow: set when a store is too small (the candidates, or the entries
  // of list A); every later stage then returns at once and the chunk counts
  // are zero, so the passes read nothing past a store.  chunks_needed: the
  // chunks list A needed.
  int *ncand, *overflow, *chunks_needed;
  int *cand_start, *cand_count;  // per i-tile
  unsigned *colA, *colB, *colC, *colE, *colK;  // per candidate x 32 lanes
  int4 *cand_n;                  // entries of (A, B, C) per candidate
  int4 *cand_off;                // their offsets within the i-tile
  int *chunksA, *chunksB, *chunksC;  // per i-tile
  int *chunk0A, *chunk0B, *chunk0C;  // first chunk of each i-tile
  int *nchunkA, *nchunkB, *nchunkC;
  // the lists
  int *chunkA_i, *entA_slot;
  unsigned *entA_col, *entA_exc, *entA_close;
  int *chunkB_i, *entB_slot;
  unsigned *entB_col;
  int *chunkC_i, *entC_slot;
  unsigned *entC_col;
  // rebuild flag of lists B and C (set by the displacement check) and the
  // positions they were made from
  int *flagB;        // some tile needs its entries of lists B and C remade
  int *tile_flagB;   // per tile: an atom of it moved more than kListMove
  float4 *xb;
};

// ---- stage 1 -------------------------------------------------------------
__global__ void k_list_candidates(const ListArgs a) {
  pdl_wait();
  const int lane = threadIdx.x & 31;
  const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (I >= a.ntile) return;
  const int sys = a.tile_sys[I];
  if (!a.sys_active[sys]) {
    if (lane == 0) {
      a.cand_start[I] = 0;
      a.cand_count[I] = 0;
    }
    return;
  }
  const int jend = a.sys_tile_end[sys];
  const float4 il = a.box_lo[I], ih = a.box_hi[I];
  const float lim = a.cut2f * 1.0001f + 1e-3f;
  auto near = [&](int J) {
    if (J >= jend) return false;
    const float4 bl = a.box_lo[J], bh = a.box_hi[J];
    const float dx = fmaxf(0.0f, fmaxf(il.x - bh.x, bl.x - ih.x));
    const float dy = fmaxf(0.0f, fmaxf(il.y - bh.y, bl.y - ih.y));
    const float dz = fmaxf(0.0f, fmaxf(il.z - bh.z, bl.z - ih.z));
    return dx * dx + dy * dy + dz * dz < lim;
  };
  int cnt = 0;
  for (int J0 = I; J0 < jend; J0 += 32) cnt += __popc(__ballot_sync(kFull, near(J0 + lane)));
  int base = 0;
  if (lane == 0) base = atomicAdd(a.ncand, cnt);
  base = __shfl_sync(kFull, base, 0);
  if (base + cnt > a.cand_cap) {  // the host grows the store and runs this stage again
    if (lane == 0) {
      atomicExch(a.overflow, 1);
      a.cand_start[I] = 0;
      a.cand_count[I] = 0;
    }
    return;
  }
  int k = base;
  for (int J0 = I; J0 < jend; J0 += 32) {
    const bool c = near(J0 + lane);
    const unsigned bal = __ballot_sync(kFull, c);
    if (c) a.cand[k + __popc(bal & ((1u << lane) - 1u))] = make_int2(I, J0 + lane);
    k += __popc(bal);
  }
  if (lane == 0) {
    a.cand_start[I] = base;
    a.cand_count[I] = cnt;
  }
}

// ---- stage 2 -------------------------------------------------------------
// Lane l takes j-atom l of tile J and walks the 32 atoms of tile I.
// list A: r^2 < cut^2, decided in FP64 from the double coordinates when
// the FP32 distance is within 1e-5 of the cutoff, as the reference decides
// (nblist.c:726-746); upper triangle within a tile; no pair of two frozen
// atoms.  Lists B and C: list A pairs with r^2 < (rgbmax + Fsmax +
// skin)^2, on C when r < 4 max(s_i, s_j) + skin, else on B.
// GB_ONLY: list A stays as built; lists B and C are remade from its
// columns.
template <bool GB_ONLY>
__global__ void k_list_columns(const ListArgs a) {
  pdl_wait();
  __shared__ float4 s_hi[8][32], s_lo[8][32];
  __shared__ float s_s[8][32];
  __shared__ int s_atom[8][32];
  __shared__ unsigned s_ex[8][32];
  if ((GB_ONLY && !*a.flagB) || *a.overflow) return;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int ncand = min(*a.ncand, a.cand_cap), nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < ncand; c += nwarps) {
  const int2 p = a.cand[c];
  const int I = p.x, J = p.y;
  if (GB_ONLY && !a.tile_flagB[I] && !a.tile_flagB[J]) {
    // both tiles stayed within kListMove of their reference positions: the
    // pairs keep their lists, only the counts are needed again
    const size_t e = static_cast<size_t>(c) * 32 + lane;
    const int nA = __popc(__ballot_sync(kFull, a.colA[e] != 0u)), nB = __popc(__ballot_sync(kFull, a.colB[e] != 0u));
    const int nC = __popc(__ballot_sync(kFull, a.colC[e] != 0u));
    if (lane == 0) a.cand_n[c] = make_int4(nA, nB, nC, 0);
    continue;
  }
  const int si = I * 32 + lane, sj = J * 32 + lane;
  s_hi[w][lane] = a.pos_hi[si];
  s_lo[w][lane] = a.pos_lo[si];
  s_atom[w][lane] = a.slot_atom[si];
  s_s[w][lane] = a.gbpar[si].y;
  const unsigned vI = a.tile_valid[I];
  const unsigned frzI = __ballot_sync(kFull, (a.param[si] >> 24) & 1);
  const float4 hj = a.pos_hi[sj], lj = a.pos_lo[sj];
  const bool vj = (a.tile_valid[J] >> lane) & 1u;
  const bool frzj = (a.param[sj] >> 24) & 1;
  const int aj = a.slot_atom[sj];
  const float sjs = a.gbpar[sj].y;
  // exclusion rows of this tile pair, if it has any: the lanes search the
  // i-tile's list of excluded tile partners together, then stage the rows
  unsigned exrow = 0u;
  if (!GB_ONLY) {
    const int e0 = a.excl_tile_start[I], e1 = a.excl_tile_start[I + 1];
    int ex = -1;
    for (int e = e0; e < e1; e += 32) {
      const bool hit = e + lane < e1 && a.excl_tile_j[e + lane] == J;
      const unsigned bal = __ballot_sync(kFull, hit);
      if (bal) {
        ex = a.excl_tile_idx[e + __ffs(bal) - 1];
        break;
      }
    }
    if (ex >= 0) exrow = a.excl_masks[static_cast<size_t>(ex) * 32 + lane];
  }
  s_ex[w][lane] = exrow;
  const bool has_ex = __any_sync(kFull, exrow != 0u);
  __syncwarp();
  const unsigned prevA = GB_ONLY ? a.colA[static_cast<size_t>(c) * 32 + lane] : 0u;
  unsigned colA = 0, colB = 0, colC = 0, colE = 0, colK = 0;
  const float gbb = a.sys_gbb2[a.tile_sys[I]] * 1.0001f + 1e-3f;
  // rows to test (warp-uniform): every valid i-atom, or for a remake only
  // those with a list-A pair in this tile pair
  unsigned rows = prevA;
  if (GB_ONLY) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rows |= __shfl_xor_sync(kFull, rows, o);
  } else {
    rows = ~0u;
  }
  rows &= vI;
  for (; rows; rows &= rows - 1u) {
    const int i = __ffs(rows) - 1;
    const float4 hi = s_hi[w][i], li = s_lo[w][i];
    const float dx = (hi.x - hj.x) + (li.x - lj.x);
    const float dy = (hi.y - hj.y) + (li.y - lj.y);
    const float dz = (hi.z - hj.z) + (li.z - lj.z);
    const float r2 = dx * dx + dy * dy + dz * dz;
    bool in;
    if (GB_ONLY) {
      in = (prevA >> i) & 1u;
    } else {
      if (!vj) {
        in = false;
      } else if (r2 < a.cut2f * 0.99999f) {
        in = true;
      } else if (r2 > a.cut2f * 1.00001f) {
        in = false;
      } else {  // borderline: decide exactly as the reference does, in FP64
        const int ai = s_atom[w][i];
        const double ddx = a.x[3 * ai] - a.x[3 * aj], ddy = a.x[3 * ai + 1] - a.x[3 * aj + 1],
                     ddz = a.x[3 * ai + 2] - a.x[3 * aj + 2];
        in = ddx * ddx + ddy * ddy + ddz * ddz < a.cut2;
      }
      in = in && vj && !(I == J && i >= lane) && !(((frzI >> i) & 1u) && frzj);
      const unsigned exb = has_ex ? (s_ex[w][i] >> lane) & 1u : 0u;
      colE |= exb << i;
      // a non-excluded pair this close may come within kClose before the
      // next build; pass 2 checks those pairs' distance at every evaluation
      colK |= static_cast<unsigned>(in && !exb && r2 < a.close2f) << i;
    }
    const float nr = 4.0f * fmaxf(s_s[w][i], sjs) + kListSkin;
    const bool gb = in && r2 < gbb, near = r2 < nr * nr * 1.0001f;
    colA |= static_cast<unsigned>(in) << i;
    colB |= static_cast<unsigned>(gb && !near) << i;
    colC |= static_cast<unsigned>(gb && near) << i;
  }
  const size_t e = static_cast<size_t>(c) * 32 + lane;
  if (!GB_ONLY) {
    a.colA[e] = colA;
    a.colE[e] = colE;
    a.colK[e] = colK;
  }
  a.colB[e] = colB;
  a.colC[e] = colC;
  const int nA = __popc(__ballot_sync(kFull, colA != 0u)), nB = __popc(__ballot_sync(kFull, colB != 0u));
  const int nC = __popc(__ballot_sync(kFull, colC != 0u));
  if (lane == 0) a.cand_n[c] = make_int4(nA, nB, nC, 0);
  __syncwarp();  // the staged i-tile is rewritten by the next candidate
  }
}

// ---- stage 3 -------------------------------------------------------------
template <bool GB_ONLY>
__global__ void k_list_offsets(const ListArgs a) {
  pdl_wait();
  if ((GB_ONLY && !*a.flagB) || *a.overflow) return;
  const int lane = threadIdx.x & 31;
  const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (I >= a.ntile) return;
  const int c0 = a.cand_start[I], n = a.cand_count[I];
  int runA = 0, runB = 0, runC = 0;
  for (int k0 = 0; k0 < n; k0 += 32) {
    const int k = k0 + lane;
    const int4 v = k < n ? a.cand_n[c0 + k] : make_int4(0, 0, 0, 0);
    int sA = v.x, sB = v.y, sC = v.z;  // inclusive warp scans
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int tA = __shfl_up_sync(kFull, sA, o), tB = __shfl_up_sync(kFull, sB, o),
                tC = __shfl_up_sync(kFull, sC, o);
      if (lane >= o) {
        sA += tA;
        sB += tB;
        sC += tC;
      }
    }
    if (k < n) {
      int4 off = make_int4(runA + sA - v.x, runB + sB - v.y, runC + sC - v.z, 0);
      if (GB_ONLY) off.x = a.cand_off[c0 + k].x;
      a.cand_off[c0 + k] = off;
    }
    runA += __shfl_sync(kFull, sA, 31);
    runB += __shfl_sync(kFull, sB, 31);
    runC += __shfl_sync(kFull, sC, 31);
  }
  if (lane == 0) {
    if (!GB_ONLY) a.chunksA[I] = (runA + 31) >> 5;
    a.chunksB[I] = (runB + 31) >> 5;
    a.chunksC[I] = (runC + 31) >> 5;
  }
}

// ---- stage 4 -------------------------------------------------------------
// Exclusive scan of chunks per i-tile, one block of 1024 threads.
template <bool GB_ONLY>
__global__ void __launch_bounds__(1024) k_list_scan(const ListArgs a) {
  pdl_wait();
  __shared__ int s_a[1024], s_b[1024], s_c[1024];
  if (GB_ONLY && !*a.flagB) return;
  const int t = threadIdx.x, n = a.ntile;
  if (*a.overflow) {  // a store was too small: empty lists
    if (t == 0) {
      *a.nchunkA = 0;
      *a.nchunkB = 0;
      *a.nchunkC = 0;
    }
    return;
  }
  const int per = (n + 1023) / 1024, lo = min(n, t * per), hi = min(n, lo + per);
  int sa = 0, sb = 0, sc = 0;
  for (int i = lo; i < hi; i++) {
    if (!GB_ONLY) sa += a.chunksA[i];
    sb += a.chunksB[i];
    sc += a.chunksC[i];
  }
  s_a[t] = sa;
  s_b[t] = sb;
  s_c[t] = sc;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {  // inclusive Hillis-Steele scan
    const int va = t >= o ? s_a[t - o] : 0, vb = t >= o ? s_b[t - o] : 0, vc = t >= o ? s_c[t - o] : 0;
    __syncthreads();
    s_a[t] += va;
    s_b[t] += vb;
    s_c[t] += vc;
    __syncthreads();
  }
  int ra = s_a[t] - sa, rb = s_b[t] - sb, rc = s_c[t] - sc;
  for (int i = lo; i < hi; i++) {
    if (!GB_ONLY) {
      a.chunk0A[i] = ra;
      ra += a.chunksA[i];
    }
    a.chunk0B[i] = rb;
    rb += a.chunksB[i];
    a.chunk0C[i] = rc;
    rc += a.chunksC[i];
  }
  if (t == 1023) {
    // list A's entries must fit their store (B and C hold subsets of them)
    const bool fits = GB_ONLY || static_cast<long long>(s_a[1023]) <= a.ent_cap;
    if (!GB_ONLY) {
      *a.chunks_needed = s_a[1023];
      if (!fits) atomicExch(a.overflow, 1);
      *a.nchunkA = fits ? s_a[1023] : 0;
    }
    *a.nchunkB = fits ? s_b[1023] : 0;
    *a.nchunkC = fits ? s_c[1023] : 0;
  }
}

// ---- stage 5 -------------------------------------------------------------
template <bool GB_ONLY>
__global__ void k_list_fill(const ListArgs a) {
  pdl_wait();
  if ((GB_ONLY && !*a.flagB) || *a.overflow) return;
  const int lane = threadIdx.x & 31;
  const int ncand = min(*a.ncand, a.cand_cap), nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < ncand; c += nwarps) {
  const int2 p = a.cand[c];
  const int4 off = a.cand_off[c];
  const size_t e = static_cast<size_t>(c) * 32 + lane;
  const unsigned lt = (1u << lane) - 1u;
  if (!GB_ONLY) {
    const unsigned col = a.colA[e];
    const unsigned bal = __ballot_sync(kFull, col != 0u);
    if (col) {
      const size_t pos = static_cast<size_t>(a.chunk0A[p.x]) * 32 + off.x + __popc(bal & lt);
      a.entA_slot[pos] = p.y * 32 + lane;
      a.entA_col[pos] = col;
      a.entA_exc[pos] = a.colE[e];
      a.entA_close[pos] = a.colK[e];
    }
  }
  {
    const unsigned col = a.colB[e];
    const unsigned bal = __ballot_sync(kFull, col != 0u);
    if (col) {
      const size_t pos = static_cast<size_t>(a.chunk0B[p.x]) * 32 + off.y + __popc(bal & lt);
      a.entB_slot[pos] = p.y * 32 + lane;
      a.entB_col[pos] = col;
    }
  }
  {
    const unsigned col = a.colC[e];
    const unsigned bal = __ballot_sync(kFull, col != 0u);
    if (col) {
      const size_t pos = static_cast<size_t>(a.chunk0C[p.x]) * 32 + off.z + __popc(bal & lt);
      a.entC_slot[pos] = p.y * 32 + lane;
      a.entC_col[pos] = col;
    }
  }
  }
}

// ---- stage 6 -------------------------------------------------------------
// Padding entries after each i-tile's last entry, and the owner of every
// chunk.  A padding entry points at the i-tile's own first slot with an
// empty column, so the passes load harmless data for it.
template <bool GB_ONLY>
__global__ void k_list_pad(const ListArgs a) {
  pdl_wait();
  if ((GB_ONLY && !*a.flagB) || *a.overflow) return;
  const int lane = threadIdx.x & 31;
  const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (I >= a.ntile) return;
  const int c0 = a.cand_start[I], n = a.cand_count[I];
  int tot[3] = {0, 0, 0};
  if (n > 0) {
    const int4 lo = a.cand_off[c0 + n - 1], ln = a.cand_n[c0 + n - 1];
    tot[0] = lo.x + ln.x;
    tot[1] = lo.y + ln.y;
    tot[2] = lo.z + ln.z;
  }
  for (int list = GB_ONLY ? 1 : 0; list < 3; list++) {
    const int ch0 = list == 0 ? a.chunk0A[I] : list == 1 ? a.chunk0B[I] : a.chunk0C[I];
    const int nch = list == 0 ? a.chunksA[I] : list == 1 ? a.chunksB[I] : a.chunksC[I];
    int *slot = list == 0 ? a.entA_slot : list == 1 ? a.entB_slot : a.entC_slot;
    unsigned *col = list == 0 ? a.entA_col : list == 1 ? a.entB_col : a.entC_col;
    int *owner = list == 0 ? a.chunkA_i : list == 1 ? a.chunkB_i : a.chunkC_i;
    const int end = nch * 32;
    for (int k = tot[list] + lane; k < end; k += 32) {
      const size_t pos = static_cast<size_t>(ch0) * 32 + k;
      slot[pos] = I * 32;
      col[pos] = 0u;
      if (list == 0) {
        a.entA_exc[pos] = 0u;
        a.entA_close[pos] = 0u;
      }
    }
    for (int k = lane; k < nch; k += 32) owner[ch0 + k] = I;
  }
  // lists B and C now reflect the current positions of the tiles remade
  if (!GB_ONLY || a.tile_flagB[I]) a.xb[I * 32 + lane] = a.pos_hi[I * 32 + lane];
}

// Clears the list-B flag after a (re)build; launched last.
__global__ void k_list_done(int *flagB, int *tile_flagB, int ntile) {
  pdl_wait();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) *flagB = 0;
  if (s < ntile) tile_flagB[s] = 0;
}

}  // namespace sffg
