// Per-atom, per-tile, list-building, bonded and integrator kernels.
#pragma once

#include <cstdint>

#include "kernels.cuh"

namespace sffg {

constexpr double kLog2eQuarterSqrt = 0.60056120439322491;  // sqrt(log2(e) / 4)
constexpr double kKscale = 0.73;                           // src/sff/eff.c:1368

// ------------------------------------------------------------ packing
// Splits the FP64 coordinates of every slot into FP32 high/low parts,
// computes each tile's bounding box, and clears the per-slot accumulators.
// One warp per tile.  Padding slots sit far away with zero charge.
__global__ void k_pack(const double *__restrict__ x, const int *__restrict__ slot_atom,
                       const float *__restrict__ q32, const unsigned *__restrict__ tile_valid,
                       int nslot, float4 *pos_hi, float4 *pos_lo, float4 *box_lo, float4 *box_hi,
                       long long *acc_sumi, long long *acc_fx, long long *acc_fy, long long *acc_fz,
                       int *nonfinite_sys, const int *tile_sys, const float4 *xb, float xb_lim2,
                       int *flagB, int *tile_flagB, int *queue_counters, long long *energy, int nenergy) {
  pdl_wait();
  {
    // the evaluation's fresh sums: pass work-queue counters and energy slots
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nthr = gridDim.x * blockDim.x;
    if (tid < 5) queue_counters[tid] = 0;
    for (int i = tid; i < nenergy; i += nthr) energy[i] = 0;
  }
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  if (slot - lane >= nslot) return;  // whole warp beyond the last tile
  const int tile = slot >> 5;
  const int a = slot < nslot ? slot_atom[slot] : -1;
  float4 hi, lo;
  float bx0 = 3e38f, by0 = 3e38f, bz0 = 3e38f, bx1 = -3e38f, by1 = -3e38f, bz1 = -3e38f;
  bool bad = false;
  if (a >= 0) {
    const double X = x[3 * a], Y = x[3 * a + 1], Z = x[3 * a + 2];
    bad = !(isfinite(X) && isfinite(Y) && isfinite(Z));
    const float hx = static_cast<float>(X), hy = static_cast<float>(Y), hz = static_cast<float>(Z);
    hi = make_float4(hx, hy, hz, q32[slot]);
    lo = make_float4(static_cast<float>(X - hx), static_cast<float>(Y - hy), static_cast<float>(Z - hz), 0.f);
    // a tile's entries of lists B and C stay valid while none of its atoms
    // has moved more than sqrt(xb_lim2) since they were made (a NaN also
    // asks for a remake)
    const float4 q = xb[slot];
    const float mx = hx - q.x, my = hy - q.y, mz = hz - q.z;
    if (!(mx * mx + my * my + mz * mz <= xb_lim2)) {
      *flagB = 1;
      tile_flagB[tile] = 1;
    }
    if (!bad) {
      bx0 = bx1 = hx;
      by0 = by1 = hy;
      bz0 = bz1 = hz;
    }
  } else {
    hi = make_float4(1.0e6f + 16.0f * lane, 1.0e6f, 1.0e6f, 0.f);
    lo = make_float4(0.f, 0.f, 0.f, 0.f);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    bx0 = fminf(bx0, __shfl_xor_sync(kFull, bx0, o));
    by0 = fminf(by0, __shfl_xor_sync(kFull, by0, o));
    bz0 = fminf(bz0, __shfl_xor_sync(kFull, bz0, o));
    bx1 = fmaxf(bx1, __shfl_xor_sync(kFull, bx1, o));
    by1 = fmaxf(by1, __shfl_xor_sync(kFull, by1, o));
    bz1 = fmaxf(bz1, __shfl_xor_sync(kFull, bz1, o));
  }
  const unsigned anybad = __ballot_sync(kFull, bad);
  if (slot >= nslot) return;
  pos_hi[slot] = hi;
  pos_lo[slot] = lo;
  acc_sumi[slot] = 0;
  acc_fx[slot] = 0;
  acc_fy[slot] = 0;
  acc_fz[slot] = 0;
  if (lane == 0) {
    box_lo[tile] = make_float4(bx0, by0, bz0, 0.f);
    box_hi[tile] = make_float4(bx1, by1, bz1, 0.f);
    if (anybad) nonfinite_sys[tile_sys[tile]] = 1;
  }
  (void)tile_valid;
}

// ------------------------------------------------------------ Born radii
// Effective Born radii from the descreening sums (src/sff/eff.c:1710-1727),
// the diagonal self energy and its sumdeijda seed (eff.c:1884-1893).  FP64.
struct FinishArgs {
  const long long *acc_sumi;
  long long *acc_sd;
  long long *energy;
  const int *slot_atom, *tile_sys, *sys_active, *param;
  const double *rborn64, *q64, *alpha, *beta, *gamma;
  const double2 *rinv64;  // per slot: 1 / (rborn - offset), 1 / rborn
  double *reff64, *psi64, *chainfac;
  float *reff32, *rinv2;
  int nslot, gb;
  double gboffset, kappa, epsext;
};

__global__ void k_born_finish(const FinishArgs a) {
  pdl_wait();
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  if (slot - lane >= a.nslot) return;
  const int sys = a.tile_sys[slot >> 5];
  double ediag = 0.0;
  if (slot < a.nslot) {
    const int at = a.slot_atom[slot];
    if (at >= 0 && a.sys_active[sys]) {
      // one FP64 division per atom (the reciprocal radii are static; GB300's
      // FP64 divisions are slow): inv = 1 / reff
      const double rb = a.rborn64[slot], ri = rb - a.gboffset;
      const double2 ir = a.rinv64[slot];
      const double sumi = -static_cast<double>(a.acc_sumi[slot]) * (1.0 / 1099511627776.0);
      double reff, inv, psi = 0.0, fac = 1.0;
      if (a.gb == 1) {
        inv = ir.x + sumi;
        reff = 1.0 / inv;
        if (reff < 0.0) {
          reff = 30.0;
          inv = 1.0 / 30.0;
        }
      } else {
        psi = -ri * sumi;
        const double al = a.alpha[slot], be = a.beta[slot], ga = a.gamma[slot];
        const double th = tanh((al - be * psi + ga * psi * psi) * psi);
        inv = ir.x - th * ir.y;
        reff = 1.0 / inv;
        fac = (al - 2.0 * be * psi + 3.0 * ga * psi * psi) * (1.0 - th * th) * (ri * ir.y);
      }
      a.reff64[slot] = reff;
      a.psi64[slot] = psi;
      a.chainfac[slot] = fac;
      a.reff32[slot] = static_cast<float>(reff);
      a.rinv2[slot] = static_cast<float>(kLog2eQuarterSqrt * inv);
      double sd = 0.0;
      if (!((a.param[slot] >> 24) & 1)) {
        const double qi = a.q64[slot];
        const double expmkf = (a.kappa != 0.0 ? exp(-kKscale * a.kappa * reff) : 1.0) / a.epsext;
        const double dielfac = 1.0 - expmkf, qi2h = 0.5 * qi * qi, qid2h = qi2h * dielfac;
        ediag = -qid2h * inv;
        sd = qid2h - kKscale * a.kappa * qi2h * expmkf * reff;
      }
      a.acc_sd[slot] = __double2ll_rn(sd * 4294967296.0);
    } else {
      a.reff32[slot] = 1.0f;
      a.rinv2[slot] = 0.0f;
      a.acc_sd[slot] = 0;
    }
  }
  // a tile never straddles systems, so the warp shares sys
  const long long e = warp_sum_ll(__double2ll_rn(ediag * 4294967296.0));
  if (lane == 0 && slot < a.nslot) atomic_add_ll(&a.energy[sys * kEnergySlots + 0], e);
}

// Chain-rule weight of each atom for pass 3 (src/sff/eff.c:2211-2231).
__global__ void k_chain_prep(const long long *acc_sd, const double *chainfac, const int *param,
                             const int *slot_atom, float *sumda32, int nslot) {
  pdl_wait();
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= nslot) return;
  double v = 0.0;
  if (slot_atom[slot] >= 0 && !((param[slot] >> 24) & 1))
    v = static_cast<double>(acc_sd[slot]) * (1.0 / 4294967296.0) * chainfac[slot];
  sumda32[slot] = static_cast<float>(v);
}

// ------------------------------------------------------------ bonded terms
// FP64, one thread per term, forces scattered in fixed point.  Terms are
// stored with batch-global atom indices, grouped by system.
struct BondedArgs {
  int natom;  // atoms of the batch, for the checked build
  const double *x;
  const int *atom_slot;
  const int *atom_sys;
  long long *acc_fx, *acc_fy, *acc_fz;
  long long *energy;
  const int *sys_active;
};

__device__ __forceinline__ void add_force(const BondedArgs &a, int atom, double gx, double gy, double gz) {
  const int s = a.atom_slot[atom];
  atomic_add_ll(&a.acc_fx[s], __double2ll_rn(gx * 4294967296.0));
  atomic_add_ll(&a.acc_fy[s], __double2ll_rn(gy * 4294967296.0));
  atomic_add_ll(&a.acc_fz[s], __double2ll_rn(gz * 4294967296.0));
}

// Adds each lane's energy into its system's slot; a warp whose lanes share
// one system uses a single atomic.
__device__ __forceinline__ void add_energy(const BondedArgs &a, int sys, int slot, double e) {
  const long long v = __double2ll_rn(e * 4294967296.0);
  const int s0 = __shfl_sync(kFull, sys, 0);
  if (__all_sync(kFull, sys == s0 || sys < 0)) {
    const long long t = warp_sum_ll(sys >= 0 ? v : 0);
    if ((threadIdx.x & 31) == 0 && s0 >= 0) atomic_add_ll(&a.energy[s0 * kEnergySlots + slot], t);
  } else if (sys >= 0) {
    atomic_add_ll(&a.energy[sys * kEnergySlots + slot], v);
  }
}

// Harmonic bonds: src/sff/eff.c:116-154.
__global__ void k_bonds(const BondedArgs a, const int2 *atoms, const double2 *par, int n) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int sys = -1;
  double e = 0.0;
  if (i < n) {
    const int p = SFFG_IDX(atoms[i].x, a.natom, kCheckAtom), q = SFFG_IDX(atoms[i].y, a.natom, kCheckAtom);
    sys = a.atom_sys[p];
    if (!a.sys_active[sys]) {
      sys = -1;
    } else {
      const double rx = a.x[3 * p] - a.x[3 * q], ry = a.x[3 * p + 1] - a.x[3 * q + 1], rz = a.x[3 * p + 2] - a.x[3 * q + 2];
      const double r = sqrt(rx * rx + ry * ry + rz * rz);
      const double db = r - par[i].y;
      double df = par[i].x * db;
      e = df * db;
      df *= 2.0 / r;
      add_force(a, p, rx * df, ry * df, rz * df);
      add_force(a, q, -rx * df, -ry * df, -rz * df);
    }
  }
  add_energy(a, sys, E_BOND, e);
}

// Harmonic angles: src/sff/eff.c:216-300.
__global__ void k_angles(const BondedArgs a, const int4 *atoms, const double2 *par, int n) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int sys = -1;
  double e = 0.0;
  if (i < n) {
    const int p = SFFG_IDX(atoms[i].x, a.natom, kCheckAtom), q = SFFG_IDX(atoms[i].y, a.natom, kCheckAtom),
              r = SFFG_IDX(atoms[i].z, a.natom, kCheckAtom);
    sys = a.atom_sys[p];
    if (!a.sys_active[sys]) {
      sys = -1;
    } else {
      const double dxi = a.x[3 * p] - a.x[3 * q], dyi = a.x[3 * p + 1] - a.x[3 * q + 1], dzi = a.x[3 * p + 2] - a.x[3 * q + 2];
      const double dxj = a.x[3 * r] - a.x[3 * q], dyj = a.x[3 * r + 1] - a.x[3 * q + 1], dzj = a.x[3 * r + 2] - a.x[3 * q + 2];
      const double ri = sqrt(dxi * dxi + dyi * dyi + dzi * dzi), rj = sqrt(dxj * dxj + dyj * dyj + dzj * dzj);
      const double rir = 1.0 / ri, rjr = 1.0 / rj;
      const double uxi = dxi * rir, uyi = dyi * rir, uzi = dzi * rir, uxj = dxj * rjr, uyj = dyj * rjr, uzj = dzj * rjr;
      double cst = uxi * uxj + uyi * uyj + uzi * uzj;
      cst = fmin(1.0, fmax(-1.0, cst));
      const double at = acos(cst), da = at - par[i].y;
      double df = da * par[i].x;
      e = df * da;
      df = df + df;
      double sn = sin(at);
      if (sn > 0 && sn < 1.e-3) sn = 1.e-3;
      else if (sn < 0 && sn > -1.e-3) sn = -1.e-3;
      df = -df / sn;
      const double xa = df * rir * (uxj - cst * uxi), xc = df * rjr * (uxi - cst * uxj);
      const double ya = df * rir * (uyj - cst * uyi), yc = df * rjr * (uyi - cst * uyj);
      const double za = df * rir * (uzj - cst * uzi), zc = df * rjr * (uzi - cst * uzj);
      add_force(a, p, xa, ya, za);
      add_force(a, r, xc, yc, zc);
      add_force(a, q, -(xa + xc), -(ya + yc), -(za + zc));
    }
  }
  add_energy(a, sys, E_ANGLE, e);
}

// Cosine dihedrals: src/sff/eff.c:373-618 (one expanded term per thread).
__global__ void k_dihedrals(const BondedArgs a, const int4 *atoms, const double4_32a *par, int n) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int sys = -1;
  double e = 0.0;
  if (i < n) {
    const int p = SFFG_IDX(atoms[i].x, a.natom, kCheckAtom), q = SFFG_IDX(atoms[i].y, a.natom, kCheckAtom),
              r = SFFG_IDX(atoms[i].z, a.natom, kCheckAtom), w = SFFG_IDX(atoms[i].w, a.natom, kCheckAtom);
    sys = a.atom_sys[p];
    if (!a.sys_active[sys]) {
      sys = -1;
    } else {
      const double pk = par[i].x, pn = par[i].y, phase = par[i].z;
      const double *x = a.x;
      const double ax = x[3 * q] - x[3 * p], ay = x[3 * q + 1] - x[3 * p + 1], az = x[3 * q + 2] - x[3 * p + 2];
      const double bx = x[3 * r] - x[3 * q], by = x[3 * r + 1] - x[3 * q + 1], bz = x[3 * r + 2] - x[3 * q + 2];
      const double cx = x[3 * w] - x[3 * r], cy = x[3 * w + 1] - x[3 * r + 1], cz = x[3 * w + 2] - x[3 * r + 2];
      const double ab = ax * bx + ay * by + az * bz, bc = bx * cx + by * cy + bz * cz, ac = ax * cx + ay * cy + az * cz;
      const double aa = ax * ax + ay * ay + az * az, bb = bx * bx + by * by + bz * bz, cc = cx * cx + cy * cy + cz * cz;
      const double uu = aa * bb - ab * ab, vv = bb * cc - bc * bc, uv = ab * bc - ac * bb;
      const double den = uu == 0.0 ? 0.0 : 1.0 / sqrt(uu * vv);
      const double co = uv * den, co1 = 0.5 * co * den;
      const double a0x = -bc * bx + bb * cx, a0y = -bc * by + bb * cy, a0z = -bc * bz + bb * cz;
      const double b0x = ab * cx + bc * ax - 2. * ac * bx, b0y = ab * cy + bc * ay - 2. * ac * by, b0z = ab * cz + bc * az - 2. * ac * bz;
      const double c0x = ab * bx - bb * ax, c0y = ab * by - bb * ay, c0z = ab * bz - bb * az;
      const double a1x = 2. * uu * (-cc * bx + bc * cx), a1y = 2. * uu * (-cc * by + bc * cy), a1z = 2. * uu * (-cc * bz + bc * cz);
      const double b1x = 2. * uu * (bb * cx - bc * bx), b1y = 2. * uu * (bb * cy - bc * by), b1z = 2. * uu * (bb * cz - bc * bz);
      const double a2x = -2. * vv * (bb * ax - ab * bx), a2y = -2. * vv * (bb * ay - ab * by), a2z = -2. * vv * (bb * az - ab * bz);
      const double b2x = 2. * vv * (aa * bx - ab * ax), b2y = 2. * vv * (aa * by - ab * ay), b2z = 2. * vv * (aa * bz - ab * az);
      double df;
      if (fabs(phase - 3.142) > 0.01 && fabs(phase) > 0.01) {
        const double c = fmin(1.0, fmax(-1.0, co));
        double phi = acos(c);
        const double ux = ay * bz - az * by, uy = az * bx - ax * bz, uz = ax * by - ay * bx;
        const double vx = by * cz - bz * cy, vy = bz * cx - bx * cz, vz = bx * cy - by * cx;
        const double sx = uy * vz - uz * vy, sy = uz * vx - ux * vz, sz = ux * vy - uy * vx;
        if (sx * bx + sy * by + sz * bz < 0.0) phi = -phi;
        const double delta = pn * phi - phase;
        e = pk * (1.0 + cos(delta));
        const double yy = sin(phi);
        if (fabs(yy) > 0.001) df = pk * pn * sin(delta) / yy;
        else if (phi > -1.0 && phi < 1.0) df = pk * pn * sin(delta) * 1000.;
        else df = -pk * pn * sin(delta) * 1000.;
      } else {
        const double sg = fabs(phase - 3.142) < 0.01 ? -1.0 : 1.0, c2 = co * co;
        switch (static_cast<int>(fabs(pn))) {
          case 1: e = pk * (1.0 + sg * co); df = sg * pk; break;
          case 2: e = pk * (1.0 + sg * (2. * c2 - 1.)); df = sg * pk * 4. * co; break;
          case 3: e = pk * (1.0 + sg * co * (4. * c2 - 3.)); df = sg * pk * (12. * c2 - 3.); break;
          case 4: e = pk * (1.0 + sg * (8. * c2 * (c2 - 1.) + 1.)); df = sg * pk * co * (32. * c2 - 16.); break;
          case 5: e = pk * (1.0 + sg * (16. * c2 * c2 * co - 20. * c2 * co + 5. * co)); df = sg * pk * (80. * c2 * c2 - 60. * c2 + 5.); break;
          case 6: e = pk * (1.0 + sg * (32. * c2 * c2 * c2 - 48. * c2 * c2 + 18. * c2 - 1.)); df = sg * pk * co * (192. * c2 * c2 - 192. * c2 + 36.); break;
          default: e = 0.0; df = 0.0;  // rejected on the host
        }
      }
      add_force(a, p, df * (a0x - a2x * co1) * den, df * (a0y - a2y * co1) * den, df * (a0z - a2z * co1) * den);
      add_force(a, q, df * (-a0x - b0x - (a1x - a2x - b2x) * co1) * den, df * (-a0y - b0y - (a1y - a2y - b2y) * co1) * den,
                df * (-a0z - b0z - (a1z - a2z - b2z) * co1) * den);
      add_force(a, r, df * (b0x - c0x - (-a1x - b1x + b2x) * co1) * den, df * (b0y - c0y - (-a1y - b1y + b2y) * co1) * den,
                df * (b0z - c0z - (-a1z - b1z + b2z) * co1) * den);
      add_force(a, w, df * (c0x - b1x * co1) * den, df * (c0y - b1y * co1) * den, df * (c0z - b1z * co1) * den);
    }
  }
  add_energy(a, sys, E_DIHED, e);
}

// Scaled 1-4 Coulomb and Lennard-Jones (nbond with N14 = 1, diel = C;
// src/sff/eff.c:1212-1310).  atoms = (i, j, 10-12 flag, 0);
// par = (q_i q_j scee, c12, c6, scnb).
__global__ void k_pairs14(const BondedArgs a, const int4 *atoms, const double4_32a *par, int n) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int sys = -1;
  double eel = 0.0, evdw = 0.0;
  if (i < n) {
    const int p = SFFG_IDX(atoms[i].x, a.natom, kCheckAtom), q = SFFG_IDX(atoms[i].y, a.natom, kCheckAtom);
    sys = a.atom_sys[p];
    if (!a.sys_active[sys]) {
      sys = -1;
    } else {
      const double xij = a.x[3 * p] - a.x[3 * q], yij = a.x[3 * p + 1] - a.x[3 * q + 1], zij = a.x[3 * p + 2] - a.x[3 * q + 2];
      const double r2 = xij * xij + yij * yij + zij * zij, r2inv = 1.0 / r2, r = sqrt(r2), rinv = r * r2inv;
      const double rs = par[i].x * rinv, scnb = par[i].w;
      eel = rs;
      double df;
      if (atoms[i].z == 0) {
        const double r6 = r2inv * r2inv * r2inv, f2 = par[i].z * r6, f1 = par[i].y * r6 * r6;
        evdw = (f1 - f2) * scnb;
        df = (-rs + (6.0 * f2 - 12.0 * f1) * scnb) * rinv;
      } else {
        const double r10 = r2inv * r2inv * r2inv * r2inv * r2inv, f2 = par[i].z * r10, f1 = par[i].y * r10 * r2inv;
        evdw = (f1 - f2) * scnb;
        df = (-rs + (10.0 * f2 - 12.0 * f1) * scnb) * rinv;
      }
      df *= rinv;
      add_force(a, p, df * xij, df * yij, df * zij);
      add_force(a, q, -df * xij, -df * yij, -df * zij);
    }
  }
  add_energy(a, sys, E_EEL14, eel);
  add_energy(a, sys, E_ENB14, evdw);
}

// Fixed-point forces -> FP64 gradient in the caller's atom order; frozen
// atoms get zero (src/sff/eff.c:2826-2834).
// Harmonic positional restraints (src/sff/eff.c:17-80, econs):
// wcons |x - x0|^2 for every constrained atom; w[atom] = wcons or 0.
__global__ void k_restraints(const BondedArgs a, const double *w, const double *x0, int natom) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int sys = -1;
  double e = 0.0;
  if (i < natom && w[i] != 0.0) {
    sys = a.atom_sys[i];
    if (!a.sys_active[sys]) {
      sys = -1;
    } else {
      const double rx = a.x[3 * i] - x0[3 * i], ry = a.x[3 * i + 1] - x0[3 * i + 1],
                   rz = a.x[3 * i + 2] - x0[3 * i + 2];
      e = w[i] * (rx * rx + ry * ry + rz * rz);
      add_force(a, i, 2. * w[i] * rx, 2. * w[i] * ry, 2. * w[i] * rz);
    }
  }
  add_energy(a, sys, E_CONS, e);
}

// Centre-of-mass motion removal of md (src/sff/com.c:10-47 and 53-147,
// called every nscm steps at sff.c:2347-2351): one block per system moves
// the centre of mass to the origin and, with also_v, removes the
// centre-of-mass velocity and the rigid rotation (angular momentum over the
// inertia tensor, both scaled by 1e-3 as the reference does).
constexpr int kComThreads = 256;

__device__ double block_sum(double v, double *sh) {
  const int t = threadIdx.x;
  sh[t] = v;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (t < o) sh[t] += sh[t + o];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kComThreads) k_com_remove(double *x, double *v, const double *minv,
                                                             const int *sys_atom_off, const int *sys_natom,
                                                             const int *sys_active, int also_v) {
  pdl_wait();
  __shared__ double sh[kComThreads];
  const int s = blockIdx.x;
  if (!sys_active[s]) return;
  const int a0 = sys_atom_off[s], n = sys_natom[s];
  double m = 0, mx = 0, my = 0, mz = 0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int i = 3 * (a0 + k);
    const double mi = 1. / minv[i];
    m += mi;
    mx += x[i] * mi;
    my += x[i + 1] * mi;
    mz += x[i + 2] * mi;
  }
  const double mt = block_sum(m, sh);
  const double xs = block_sum(mx, sh) / mt, ys = block_sum(my, sh) / mt, zs = block_sum(mz, sh) / mt;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int i = 3 * (a0 + k);
    x[i] -= xs;
    x[i + 1] -= ys;
    x[i + 2] -= zs;
  }
  if (!also_v) return;
  __syncthreads();
  double px = 0, py = 0, pz = 0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int i = 3 * (a0 + k);
    const double mi = 1. / minv[i];
    px += v[i] * mi;
    py += v[i + 1] * mi;
    pz += v[i + 2] * mi;
  }
  const double vx = block_sum(px, sh) / mt, vy = block_sum(py, sh) / mt, vz = block_sum(pz, sh) / mt;
  constexpr double kScale = 1.e-3;
  double l[3] = {0, 0, 0}, in[6] = {0, 0, 0, 0, 0, 0};  // xx xy xz yy yz zz
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int i = 3 * (a0 + k);
    v[i] -= vx;
    v[i + 1] -= vy;
    v[i + 2] -= vz;
    const double mi = 1. / minv[i], X = x[i], Y = x[i + 1], Z = x[i + 2];
    l[0] += kScale * (Y * v[i + 2] - Z * v[i + 1]) * mi;
    l[1] += kScale * (Z * v[i] - X * v[i + 2]) * mi;
    l[2] += kScale * (X * v[i + 1] - Y * v[i]) * mi;
    in[0] += X * X * mi;
    in[1] += X * Y * mi;
    in[2] += X * Z * mi;
    in[3] += Y * Y * mi;
    in[4] += Y * Z * mi;
    in[5] += Z * Z * mi;
  }
  double L[3], M[6];
  for (int c = 0; c < 3; c++) L[c] = block_sum(l[c], sh);
  for (int c = 0; c < 6; c++) M[c] = block_sum(in[c], sh);
  // inertia tensor and its inverse by cofactors (com.c:107-118, 150-175)
  const double I0 = (M[3] + M[5]) * kScale, I1 = -M[1] * kScale, I2 = -M[2] * kScale;
  const double I4 = (M[0] + M[5]) * kScale, I5 = -M[4] * kScale, I8 = (M[0] + M[3]) * kScale;
  const double c0 = I4 * I8 - I5 * I5, c1 = I1 * I8 - I5 * I2, c2 = I1 * I5 - I4 * I2;
  const double c4 = I0 * I8 - I2 * I2, c5 = I0 * I5 - I1 * I2, c8 = I0 * I4 - I1 * I1;
  const double det = I0 * c0 - I1 * c1 + I2 * c2;
  // the symmetric inverse: [c0 -c1 c2; -c1 c4 -c5; c2 -c5 c8] / det
  const double ox = (c0 * L[0] - c1 * L[1] + c2 * L[2]) / det;
  const double oy = (-c1 * L[0] + c4 * L[1] - c5 * L[2]) / det;
  const double oz = (c2 * L[0] - c5 * L[1] + c8 * L[2]) / det;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int i = 3 * (a0 + k);
    const double X = x[i], Y = x[i + 1], Z = x[i + 2];
    v[i] = v[i] - oy * Z + oz * Y;
    v[i + 1] = v[i + 1] - oz * X + ox * Z;
    v[i + 2] = v[i + 2] - ox * Y + oy * X;
  }
}

// Total energy of system s from the fixed-point slots, summed in the
// reference's ene[1..12] order (src/sff/eff.c:2871-2874).
__device__ __forceinline__ double energy_total(const long long *energy, int s) {
  const double k = 1.0 / 4294967296.0;
  const long long *e = energy + s * kEnergySlots;
  double ene[13] = {0};
  ene[1] = e[E_EVDW] * k;
  ene[2] = e[E_EEL] * k;
  ene[3] = e[E_BOND] * k;
  ene[4] = e[E_ANGLE] * k;
  ene[5] = e[E_DIHED] * k;
  ene[7] = e[E_ENB14] * k;
  ene[8] = e[E_EEL14] * k;
  ene[9] = e[E_CONS] * k;
  ene[10] = e[E_EGB] * k;
  double t = 0.0;
  for (int i = 1; i <= 12; i++) t += ene[i];
  return t;
}

// The gradient of every atom and, on the first nsys threads, every
// system's total energy.
__global__ void k_gather_grad(const long long *acc_fx, const long long *acc_fy, const long long *acc_fz,
                              const int *atom_slot, const int *atom_frozen, const int *atom_sys,
                              const int *sys_active, double *grad, int natom, const long long *energy,
                              double *etot, int nsys) {
  pdl_wait();
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a < nsys) etot[a] = energy_total(energy, a);
  if (a >= natom || !sys_active[atom_sys[a]]) return;
  const int s = atom_slot[a];
  const double k = 1.0 / 4294967296.0;
  const bool fz = atom_frozen[a];
  grad[3 * a] = fz ? 0.0 : static_cast<double>(acc_fx[s]) * k;
  grad[3 * a + 1] = fz ? 0.0 : static_cast<double>(acc_fy[s]) * k;
  grad[3 * a + 2] = fz ? 0.0 : static_cast<double>(acc_fz[s]) * k;
}

// ------------------------------------------------------------ dynamics
// Counter-based normal deviates for device-side Langevin noise: Philox4x32
// (Salmon et al., SC'11, 10 rounds) feeding a Box-Muller transform.
__device__ __forceinline__ uint4 philox4x32(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    const unsigned hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const unsigned hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}

// Unit Gaussian from two uniform 32-bit words (Box-Muller, in FP32: the
// Langevin noise needs no more, and FP64 transcendentals are slow here).
__device__ __forceinline__ double normal_from(unsigned a, unsigned b) {
  const float u1 = (static_cast<float>(a >> 8) + 1.0f) * (1.0f / 16777216.0f);  // (0, 1]
  const float u2 = static_cast<float>(b >> 8) * (1.0f / 16777216.0f);           // [0, 1)
  return static_cast<double>(sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2));
}

struct MdArgs {
  double *x, *v, *accel;
  const double *grad, *minv, *sqrmass;
  const int *atom_frozen, *atom_sys, *sys_active;
  const double *noise;  // reference-stream draws (per coordinate) or null
  double *tscal;        // per system (Berendsen)
  long long *ekin;      // per system, fixed point 2^32
  int n3;
  double dtx, dt5, c_explic, c_implic, sdfac, vlimit, gammai;
  unsigned long long seed;
  const unsigned *step;  // Philox counter: the step number (advanced by k_md_tscal)
  // per system: first atom and noise key; the noise of a coordinate depends
  // on (system key, coordinate index within the system, step) only, so a
  // system draws the same noise alone or in any batch
  const int *sys_atom_off;
  const unsigned long long *sys_key;
  // RATTLE (null without): the coordinates before the drift, kept for the
  // position sweeps; with it the kick leaves the kinetic energy to k_md_ekin,
  // which runs after the velocity sweeps
  double *xold;
};

// First half of a step (src/sff/sff.c:2243-2248): half-kick and drift.
__global__ void k_md_drift(const MdArgs a) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n3) return;
  const int sys = a.atom_sys[i / 3];
  if (!a.sys_active[sys]) return;
  double v = a.v[i];
  v = a.gammai == 0.0 ? (v + a.accel[i]) * a.tscal[sys] : a.c_explic * v + a.accel[i];
  v = fmin(a.vlimit, fmax(-a.vlimit, v));
  a.v[i] = v;
  if (a.xold) a.xold[i] = a.x[i];
  a.x[i] += v * a.dtx;
}

// Force kick after the new gradient (src/sff/sff.c:2262-2276) and the
// kinetic energy (2294-2306).  init = 1 only sets the accelerations of the
// first force evaluation (2197-2215).
__global__ void k_md_kick(const MdArgs a, int init) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int sys = -1;
  double ek = 0.0;
  if (i < a.n3) {
    const int at = i / 3;
    sys = a.atom_sys[at];
    if (!a.sys_active[sys]) {
      sys = -1;
    } else {
      const double g = a.grad[i], minv = a.minv[i];
      double v = a.v[i];
      if (a.gammai == 0.0) {
        const double acc = -g * minv * a.dt5;
        a.accel[i] = acc;
        if (!init) v = (v + acc) * a.tscal[sys];
      } else if (!a.atom_frozen[at]) {
        double z;
        if (a.noise) {
          z = a.noise[i];
        } else {
          const unsigned long long key = a.sys_key[sys];
          const unsigned il = static_cast<unsigned>(i - 3 * a.sys_atom_off[sys]);
          const uint4 r = philox4x32(make_uint4(il, *a.step, static_cast<unsigned>(key), static_cast<unsigned>(key >> 32)),
                                     make_uint2(static_cast<unsigned>(a.seed), static_cast<unsigned>(a.seed >> 32)));
          z = normal_from(r.x, r.y);
        }
        const double sd = a.sdfac * a.sqrmass[i];
        const double acc = (-g + sd * z) * minv * a.dt5;
        a.accel[i] = acc;
        if (!init) v = (v + acc) * a.c_implic;
      } else if (init) {
        a.accel[i] = 0.0;
      }
      a.v[i] = v;
      ek = v * v / minv;
    }
  }
  if (a.xold && !init) return;  // k_md_ekin sums it after the velocity sweeps
  // kinetic energy per system, fixed point; warps of one system use one atomic
  const long long t = __double2ll_rn(ek * 4294967296.0);
  const int s0 = __shfl_sync(kFull, sys, 0);
  if (__all_sync(kFull, sys == s0 || sys < 0)) {
    const long long tt = warp_sum_ll(sys >= 0 ? t : 0);
    if ((threadIdx.x & 31) == 0 && s0 >= 0) atomic_add_ll(&a.ekin[s0], tt);
  } else if (sys >= 0) {
    atomic_add_ll(&a.ekin[sys], t);
  }
}

// Kinetic energy per system after RATTLE's velocity sweeps (sff.c:2294-2306),
// summed as k_md_kick sums it.
__global__ void k_md_ekin(const MdArgs a) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int sys = -1;
  double ek = 0.0;
  if (i < a.n3) {
    sys = a.atom_sys[i / 3];
    if (!a.sys_active[sys]) {
      sys = -1;
    } else {
      const double v = a.v[i];
      ek = v * v / a.minv[i];
    }
  }
  const long long t = __double2ll_rn(ek * 4294967296.0);
  const int s0 = __shfl_sync(kFull, sys, 0);
  if (__all_sync(kFull, sys == s0 || sys < 0)) {
    const long long tt = warp_sum_ll(sys >= 0 ? t : 0);
    if ((threadIdx.x & 31) == 0 && s0 >= 0) atomic_add_ll(&a.ekin[s0], tt);
  } else if (sys >= 0) {
    atomic_add_ll(&a.ekin[sys], t);
  }
}

// ------------------------------------------------------------------ RATTLE
// Bond-length constraints (src/sff/rattle.c, after TINKER): Gauss-Seidel
// sweeps over the constrained bonds in the topology's order until no bond
// needs a correction.  One block per system.  The bonds of a system are
// grouped by level: a bond's level is one more than the highest level of
// the earlier bonds (in the reference's order) that share an atom with it,
// so the bonds of one level share no atom and run in parallel, and every
// atom sees its corrections in the reference's order: the sweeps give the
// sequential loop's values bit for bit.  The arithmetic is written with
// round-to-nearest intrinsics in the reference's order of operations (no
// contraction into FMA).  A system whose sweeps reach the reference's limit
// (1,000, an error there) gets its status word set and its loop ends.
struct RattleArgs {
  double *x, *v;
  const double *xold, *minv;
  const int2 *atoms;      // coordinate offsets (3 * atom) of each bond's two atoms
  const double *req;      // bond lengths
  const int *level;       // start of each level's bonds (levels of all systems, then the end)
  const int *sys_level;   // per system: its first level (nsys + 1 entries)
  const int *sys_active;
  int *status;            // per system: 1 once a sweep loop hit its limit
  double dt;              // time step (the integrator's units)
  double eps;             // tolerance: positions (float) 1e-7, velocities 1e-7 / dt
};

constexpr int kRattleThreads = 128;

// One bond of the position sweep (rattle.c:55-97); true if it was corrected.
__device__ __forceinline__ bool rattle_bond_pos(const RattleArgs &a, int k) {
  const int2 ab = a.atoms[k];
  const int i = ab.x, j = ab.y;
  double *x = a.x, *v = a.v;
  const double xr = __dsub_rn(x[j], x[i]), yr = __dsub_rn(x[j + 1], x[i + 1]), zr = __dsub_rn(x[j + 2], x[i + 2]);
  const double dist2 = __dadd_rn(__dadd_rn(__dmul_rn(xr, xr), __dmul_rn(yr, yr)), __dmul_rn(zr, zr));
  const double req = a.req[k];
  const double delta = __dsub_rn(__dmul_rn(req, req), dist2);
  if (!(fabs(delta) > a.eps)) return false;
  const double xo = __dsub_rn(a.xold[j], a.xold[i]), yo = __dsub_rn(a.xold[j + 1], a.xold[i + 1]),
               zo = __dsub_rn(a.xold[j + 2], a.xold[i + 2]);
  const double dot = __dadd_rn(__dadd_rn(__dmul_rn(xr, xo), __dmul_rn(yr, yo)), __dmul_rn(zr, zo));
  double ra = a.minv[i], rb = a.minv[j];
  const double term = __ddiv_rn(__dmul_rn(1.2, delta), __dmul_rn(__dmul_rn(2.0, __dadd_rn(ra, rb)), dot));
  const double tx = __dmul_rn(xo, term), ty = __dmul_rn(yo, term), tz = __dmul_rn(zo, term);
  x[i] = __dsub_rn(x[i], __dmul_rn(tx, ra));
  x[i + 1] = __dsub_rn(x[i + 1], __dmul_rn(ty, ra));
  x[i + 2] = __dsub_rn(x[i + 2], __dmul_rn(tz, ra));
  x[j] = __dadd_rn(x[j], __dmul_rn(tx, rb));
  x[j + 1] = __dadd_rn(x[j + 1], __dmul_rn(ty, rb));
  x[j + 2] = __dadd_rn(x[j + 2], __dmul_rn(tz, rb));
  ra = __ddiv_rn(ra, a.dt);
  rb = __ddiv_rn(rb, a.dt);
  v[i] = __dsub_rn(v[i], __dmul_rn(tx, ra));
  v[i + 1] = __dsub_rn(v[i + 1], __dmul_rn(ty, ra));
  v[i + 2] = __dsub_rn(v[i + 2], __dmul_rn(tz, ra));
  v[j] = __dadd_rn(v[j], __dmul_rn(tx, rb));
  v[j + 1] = __dadd_rn(v[j + 1], __dmul_rn(ty, rb));
  v[j + 2] = __dadd_rn(v[j + 2], __dmul_rn(tz, rb));
  return true;
}

// One bond of the velocity sweep (rattle2, rattle.c:137-172).
__device__ __forceinline__ bool rattle_bond_vel(const RattleArgs &a, int k) {
  const int2 ab = a.atoms[k];
  const int i = ab.x, j = ab.y;
  const double *x = a.x;
  double *v = a.v;
  const double xr = __dsub_rn(x[j], x[i]), yr = __dsub_rn(x[j + 1], x[i + 1]), zr = __dsub_rn(x[j + 2], x[i + 2]);
  const double xv = __dsub_rn(v[j], v[i]), yv = __dsub_rn(v[j + 1], v[i + 1]), zv = __dsub_rn(v[j + 2], v[i + 2]);
  const double dot = __dadd_rn(__dadd_rn(__dmul_rn(xr, xv), __dmul_rn(yr, yv)), __dmul_rn(zr, zv));
  const double ra = a.minv[i], rb = a.minv[j], req = a.req[k];
  const double term = __ddiv_rn(__dmul_rn(-dot, 1.2), __dmul_rn(__dmul_rn(__dadd_rn(ra, rb), req), req));
  if (!(fabs(term) > a.eps)) return false;
  const double tx = __dmul_rn(xr, term), ty = __dmul_rn(yr, term), tz = __dmul_rn(zr, term);
  v[i] = __dsub_rn(v[i], __dmul_rn(tx, ra));
  v[i + 1] = __dsub_rn(v[i + 1], __dmul_rn(ty, ra));
  v[i + 2] = __dsub_rn(v[i + 2], __dmul_rn(tz, ra));
  v[j] = __dadd_rn(v[j], __dmul_rn(tx, rb));
  v[j + 1] = __dadd_rn(v[j + 1], __dmul_rn(ty, rb));
  v[j + 2] = __dadd_rn(v[j + 2], __dmul_rn(tz, rb));
  return true;
}

// VEL = false: rattle() on the positions (and the velocities with them);
// VEL = true: rattle2() on the velocities.
template <bool VEL>
__global__ void __launch_bounds__(kRattleThreads) k_rattle(const RattleArgs a) {
  pdl_wait();
  const int s = blockIdx.x;
  if (!a.sys_active[s]) return;
  const int l0 = a.sys_level[s], l1 = a.sys_level[s + 1];
  if (l0 == l1) return;
  __shared__ int s_done;
  int niter = 0;
  bool done = false;
  while (!done && niter < 1000) {
    niter++;
    if (threadIdx.x == 0) s_done = 1;
    __syncthreads();
    for (int L = l0; L < l1; L++) {
      const int k1 = a.level[L + 1];
      for (int k = a.level[L] + static_cast<int>(threadIdx.x); k < k1; k += kRattleThreads)
        if (VEL ? rattle_bond_vel(a, k) : rattle_bond_pos(a, k)) s_done = 0;
      __syncthreads();
    }
    done = s_done != 0;
    __syncthreads();
  }
  if (niter >= 999 && threadIdx.x == 0) a.status[s] = 1;
}

}  // namespace sffg
