// UnsharpMaskFilter's point-wise step on the device (edges.rs:440-448), shared
// by the stand-alone kernels (unsharp.cu) and the two-pass z kernel, which
// applies it to the blur as it stores it.
#pragma once

#include <cuda_runtime.h>

#include "internal.hpp"

namespace itkg {

// The reference's sequence in f64 (edges.rs:440-448).
__device__ __noinline__ inline double unsharp_f64(double o, double b, double amount, double threshold) {
  const double e = __dsub_rn(o, b);
  return fabs(e) > threshold ? __dadd_rn(o, __dmul_rn(amount, e)) : o;
}

// Error-free sum: s + t == a + b exactly, s = RN(a + b) (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& t) {
  s = __fadd_rn(a, b);
  const float a1 = __fsub_rn(s, b);
  const float b1 = __fsub_rn(s, a1);
  t = __fadd_rn(__fsub_rn(a, a1), __fsub_rn(b, b1));
}

// RN32 of the reference's f64 result for f32 o, b, from f32 arithmetic.
// Returns false when it cannot decide (the caller takes the f64 sequence).
//   e* = o - b exactly as eh + el (TwoSum).  eh == 0 means e = 0 exactly.
//   The threshold test on e = RN64(e*) is decided from |eh| unless |eh| lies
//   within 2^-20 of the threshold (|e* - eh| <= 2^-24 |eh|).
//   p = amount * e* as ph + pl (ph + t = ah eh exactly by FMA; the dropped
//   terms al el and r e* are below 2^-47 |p|), and o + p as sh + s2 with
//   sh + s1 = o + ph exactly (TwoSum), s2 = s1 + pl rounded.  sh + s2 is
//   within 2^-43 (|o| + |ph|) of o + amount e*, and the reference's three f64
//   roundings move v at most 2^-50 (|o| + |ph|) from it, so v lies within
//   delta = 2^-40 (|o| + |ph|) of sh + s2.  Round-to-nearest is monotonic:
//   when sh + (s2 + delta) and sh + (s2 - delta), bounds rounded outward,
//   round to the same f32, RN32(v) is that f32.
//   Otherwise v is within delta of a tie (amount 0.5 adds one bit, so this is
//   common on real data).  When amount is an f32 and every step is exact --
//   ah el, t + ah el and s1 + that sum without error, and e* and amount e*
//   span at most 53 bits (their low parts within 2^-29 of the high ones) --
//   the reference's e, p and v were exact as well (v, near an f32 tie, spans
//   at most 50 bits), and RN32(sh + s2) rounds the same exact value.
//   Magnitude guards keep every step clear of overflow and of underflow below
//   delta; zero results always fall back (delta separates the bounds), which
//   also leaves the signs of zero to the f64 sequence.
__device__ __forceinline__ bool unsharp_fast_f32(float o, float b, const UnsharpConsts& k, float& out) {
  if (!(fmaxf(fabsf(o), fabsf(b)) < 0x1p90f)) return false;  // NaN, inf, huge
  float eh, el;
  two_sum(o, -b, eh, el);
  if (eh == 0.0f) {  // e = 0: |e| > threshold only for a negative threshold
    // o + amount * 0 with IEEE signed-zero rules (the same in f32 and f64)
    out = k.thr_neg ? __fadd_rn(o, __fmul_rn(k.ah, eh)) : o;
    return true;
  }
  const float ae = fabsf(eh);
  bool pass;
  if (ae > k.thr_up) pass = true;
  else if (ae < k.thr_dn) pass = false;
  else return false;
  if (!pass) {
    out = o;
    return true;
  }
  const float ph = __fmul_rn(k.ah, eh);
  const float t = __fmaf_rn(k.ah, eh, -ph);
  const float pl = __fadd_rn(t, __fadd_rn(__fmul_rn(k.ah, el), __fmul_rn(k.al, eh)));
  float sh, s1;
  two_sum(o, ph, sh, s1);
  const float s2 = __fadd_rn(s1, pl);
  const float scale = __fadd_ru(fabsf(o), fabsf(ph));
  if (!(scale >= 0x1p-80f) || !(fabsf(ph) < 0x1p100f) || ae < 0x1p-60f) return false;
  const float delta = __fmul_rn(scale, 0x1p-40f);
  const float hi = __fadd_rn(sh, __fadd_ru(s2, delta));
  const float lo = __fadd_rn(sh, __fadd_rd(s2, -delta));
  if (hi == lo) {
    out = hi;
    return true;
  }
  if (k.a_exact && (el == 0.0f || fabsf(el) >= __fmul_rn(ae, 0x1p-29f))) {
    const float c = __fmul_rn(k.ah, el);
    const float ce = __fmaf_rn(k.ah, el, -c);
    float p2, p2e, s2x, s2e;
    two_sum(t, c, p2, p2e);
    two_sum(s1, p2, s2x, s2e);
    if (ce == 0.0f && p2e == 0.0f && s2e == 0.0f && (p2 == 0.0f || fabsf(p2) >= __fmul_rn(fabsf(ph), 0x1p-29f))) {
      out = __fadd_rn(sh, s2x);
      return true;
    }
  }
  return false;
}

// u8 pixels (o, b in 0..255): u8::from_f64 (round half away from zero, clamp
// to [0, 255]) of the reference's f64 result, from f32 arithmetic; false when
// undecided.  e = o - b is exact, the threshold test on the integer |e| is
// exact (k.u8_min_pass), and v lies within delta of sh + s2 as for f32 pixels;
// from_f64 is monotonic, so equal conversions of the outward-rounded bounds
// decide it.  At an exact tie (amount 0.5 and an odd e) the bounds straddle a
// half-integer; when amount is an f32 and ah e and o + ah e are exact in f32
// (t == 0, s1 == 0), the reference's f64 steps were exact too and the tie is
// converted as the reference converts it.
__device__ __forceinline__ uint8_t u8_from_f32(float v) {
  return (uint8_t)fminf(fmaxf(roundf(v), 0.0f), 255.0f);
}

__device__ __forceinline__ bool unsharp_fast_u8(uint8_t ob, uint8_t bb, const UnsharpConsts& k, uint8_t& out) {
  const float o = (float)ob, e = __fsub_rn(o, (float)bb);
  if (!(fabsf(e) >= k.u8_min_pass) || e == 0.0f) {  // v = o (o + amount 0 = o for e = 0)
    out = ob;
    return true;
  }
  const float ph = __fmul_rn(k.ah, e);
  const float t = __fmaf_rn(k.ah, e, -ph);
  const float pl = __fadd_rn(t, __fmul_rn(k.al, e));
  float sh, s1;
  two_sum(o, ph, sh, s1);
  const float s2 = __fadd_rn(s1, pl);
  const float delta = __fmul_rn(__fadd_ru(o, fabsf(ph)), 0x1p-40f);
  const uint8_t qh = u8_from_f32(__fadd_ru(sh, __fadd_ru(s2, delta)));
  const uint8_t ql = u8_from_f32(__fadd_rd(sh, __fadd_rd(s2, -delta)));
  if (qh == ql) {
    out = qh;
    return true;
  }
  if (k.a_exact && t == 0.0f && s1 == 0.0f) {
    out = u8_from_f32(sh);
    return true;
  }
  return false;
}

// FMA rounding (k.cheap, k.fast): o + amount e by one f32 FMA with e = o - b
// rounded to f32 -- within a few f32 ulps of the reference -- and the
// threshold test still decided as the reference decides it (in f64 when
// |o - b| lies within 2^-20 of the threshold, or is NaN).
__device__ __forceinline__ float unsharp_cheap_f32(float o, float b, const UnsharpConsts& k) {
  const float eh = __fsub_rn(o, b);
  const float ae = fabsf(eh);
  if (ae > k.thr_up) return __fmaf_rn(k.ah, eh, o);
  if (ae < k.thr_dn || eh == 0.0f) return o;  // e = 0 passes only a negative threshold: o + amount 0 = o
  return __double2float_rn(unsharp_f64((double)o, (double)b, k.amount, k.threshold));
}

__device__ __forceinline__ float unsharp_f32(float o, float b, const UnsharpConsts& k) {
  if (k.cheap && k.fast) return unsharp_cheap_f32(o, b, k);
  float q;
  if (!k.fast || !unsharp_fast_f32(o, b, k, q))
    q = __double2float_rn(unsharp_f64((double)o, (double)b, k.amount, k.threshold));
  return q;
}

// Reference rounding, one quad: the exact f32 test per voxel, f64 where it
// cannot decide.  Out of line, so that a caller unrolled over many steps
// carries one copy.
__device__ __noinline__ inline float4 unsharp_quad_exact(float4 o, float b0, float b1, float b2, float b3,
                                                         const UnsharpConsts& k) {
  const float ov[4] = {o.x, o.y, o.z, o.w}, bv[4] = {b0, b1, b2, b3};
  float r[4];
#pragma unroll
  for (int c = 0; c < 4; ++c)
    if (!k.fast || !unsharp_fast_f32(ov[c], bv[c], k, r[c]))
      r[c] = __double2float_rn(unsharp_f64((double)ov[c], (double)bv[c], k.amount, k.threshold));
  return make_float4(r[0], r[1], r[2], r[3]);
}

}  // namespace itkg
