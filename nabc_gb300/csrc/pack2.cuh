// Packed FP32 pairs (sm_100 and later): two single-precision values in one
// 64-bit register pair, operated on by the f32x2 instructions, each half
// rounded exactly as the scalar instruction rounds it.
//
// The far-field chunks of passes 1 and 3 evaluate both directions of a pair
// -- sphere j descreening atom i and sphere i descreening atom j -- with the
// same operations on different screened radii; done as pairs, the two
// directions take one instruction each instead of two.
#pragma once

#include "gbmath.cuh"

namespace sffg {

struct f2 {
  unsigned long long v;
};

__device__ __forceinline__ f2 pk(float a, float b) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
  return r;
}

__device__ __forceinline__ f2 splat(float a) { return pk(a, a); }

__device__ __forceinline__ void upk(f2 p, float &a, float &b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(p.v));
}

__device__ __forceinline__ f2 add2(f2 a, f2 b) {
  f2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}

__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
  f2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}

__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
  f2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}

__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
  f2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}

// far_term2 and far_deriv2 (passes 1 and 3) for s = (s_j, s_i) and
// s2 = (s_j^2, s_i^2): the same operations in the same order.
__device__ __forceinline__ f2 far_term_x2(float d2i, f2 s, f2 s2) {
  const f2 D = splat(d2i);
  const f2 tmpsd = mul2(s2, D);
  f2 dumbo = fma2(tmpsd, splat(kTDD), splat(kTD));
  dumbo = fma2(tmpsd, dumbo, splat(kTC));
  dumbo = fma2(tmpsd, dumbo, splat(kTB));
  dumbo = fma2(tmpsd, dumbo, splat(kTA));
  dumbo = add2(dumbo, splat(kTAlo));
  return mul2(mul2(mul2(s, tmpsd), D), dumbo);
}

__device__ __forceinline__ f2 far_deriv_x2(float d2i, f2 s, f2 s2) {
  const f2 D = splat(d2i);
  const f2 tmpsd = mul2(s2, D);
  f2 dumbo = fma2(tmpsd, splat(kTHH), splat(kTH));
  dumbo = fma2(tmpsd, dumbo, splat(kTG));
  dumbo = fma2(tmpsd, dumbo, splat(kTF));
  dumbo = fma2(tmpsd, dumbo, splat(kTE));
  dumbo = add2(dumbo, splat(kTElo));
  return mul2(mul2(mul2(mul2(tmpsd, s), D), D), dumbo);
}

// tail_closed<DERIV> (gbmath.cuh) of both directions for s = (s_j, s_i),
// valid while q <= 0.3 in both halves (the caller checks; q above that, a
// small rgbmax, takes the scalar form).  The series polynomial is carried
// negated, so that -(q^3 p) is one product, rounded as the scalar form
// rounds q^3 p.
template <bool DERIV>
__device__ __forceinline__ f2 tail_x2(const BornConst &c, float d, float d1, f2 s) {
  constexpr float kTailPolyNeg[9] = {-3.333333334e-01f, -2.499999724e-01f, -2.000024300e-01f,
                                     -1.665848892e-01f, -1.442217029e-01f, -1.123967482e-01f,
                                     -1.778587994e-01f, 9.662055524e-02f, -3.680403911e-01f};
  const f2 a = sub2(splat(d), s), w = sub2(splat(c.rgbmax), a);
  const f2 q = mul2(w, splat(c.rgbmax1i));
  f2 p = splat(kTailPolyNeg[8]);
#pragma unroll
  for (int k = 7; k >= 0; k--) p = fma2(p, q, splat(kTailPolyNeg[k]));
  float ax, ay;
  upk(a, ax, ay);
  float yx, yy;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yx) : "f"(ax));
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yy) : "f"(ay));
  // one Newton step, as rcp_fast: y + y (1 - a y)
  const f2 y = pk(yx, yy);
  const f2 one = splat(1.0f);
  const f2 ra = fma2(y, fma2(sub2(splat(0.0f), a), y, one), y);
  const f2 q2 = mul2(q, q);
  const f2 F = fma2(mul2(s, ra), q2, mul2(mul2(q2, q), p));
  if (!DERIV) return mul2(mul2(splat(0.25f), splat(d1)), F);
  const f2 rr = mul2(ra, splat(c.rgbmax1i));
  const f2 two_s = mul2(splat(2.0f), s);
  const f2 dF = mul2(mul2(w, fma2(a, sub2(two_s, w), mul2(s, w))), mul2(rr, rr));
  const float d13 = 0.25f * d1 * d1 * d1;
  return mul2(splat(d13), fma2(splat(d), dF, F));
}

}  // namespace sffg
