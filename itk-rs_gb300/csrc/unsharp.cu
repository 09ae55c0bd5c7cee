// UnsharpMaskFilter (src/filters/edges.rs:374-452): the point-wise step after
// the blur.  For every requested voxel the reference computes, in f64 with
// each operation rounded:
//   e = orig - blur;  v = |e| > threshold ? orig + amount * e : orig
// and converts v with P::from_f64 (f32: round to nearest; u8: round half away
// from zero, clamp to [0, 255], NaN -> 0).  Vector pixels follow
// pixel.rs:93-98: to_f64 reads the first component and from_f64 fills every
// component.  The blur itself is the convolve_axis family's
// (itkg_separable_generate_region) with the filter's own kernel.
//
// f64 arithmetic runs at a small fraction of the f32 rate on this GPU, so the
// f32 kernel gets the reference's result from f32 arithmetic and falls back to
// the f64 sequence only for voxels it cannot decide (see unsharp_fast_f32).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "internal.hpp"

namespace itkg {
namespace {

constexpr int kT = 256;

// amount and threshold as the f32 path uses them (built on the host)
struct UnsharpConsts {
  double amount, threshold;  // the reference's values (the f64 sequence)
  float ah, al;              // amount = ah + al + r, |r| <= 2^-48 |amount|
  float thr_up, thr_dn;      // |e| > thr_up: the test passes; |e| < thr_dn: it fails
  int thr_neg;               // threshold < 0 (the test for e = 0)
  int a_exact;               // amount == ah exactly
  int fast;                  // 0: every voxel takes the f64 sequence
};

__device__ __forceinline__ uint8_t u8_of(double v) {
  double r = round(v);
  r = fmin(fmax(r, 0.0), 255.0);
  return (uint8_t)r;
}

// The reference's sequence in f64 (edges.rs:440-448).
__device__ __noinline__ double unsharp_f64(double o, double b, double amount, double threshold) {
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
//   terms al el and r e* are below 2^-47 |p|), s = o + p as rh + rl (TwoSum).
//   |rh + rl - (o + amount e*)| <= 2^-43.5 (|o| + |ph|), and the reference's
//   three f64 roundings move v at most 2^-50 (|o| + |ph|) from o + amount e*;
//   delta = 2^-40 (|o| + |ph|) bounds both.  RN32(v) = rh whenever
//   |rl| + delta is below half the gap from rh to its nearer neighbour.
//   Near a tie (e.g. amount 0.5 adds one bit) that test fails, but when
//   amount is an f32 and el == 0, o + amount e* = sh + s1 + t; if s1 + t
//   also sums exactly, rh + rl is the exact value, every f64 step of the
//   reference was exact too (e*, ah eh and the result need at most 48 bits),
//   and both round it to f32 the same way, ties to even included.
//   Magnitude guards keep every step clear of overflow and underflow.
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
  if (ae < 0x1p-60f) return false;
  const float ph = __fmul_rn(k.ah, eh);
  const float t = __fmaf_rn(k.ah, eh, -ph);
  const float cross = __fadd_rn(__fmul_rn(k.ah, el), __fmul_rn(k.al, eh));
  const float pl = __fadd_rn(t, cross);
  float sh, s1, s2, s2e, rh, rl;
  two_sum(o, ph, sh, s1);
  two_sum(s1, pl, s2, s2e);
  two_sum(sh, s2, rh, rl);
  const float arh = fabsf(rh);
  if (!(arh >= 0x1p-60f) || !(fabsf(ph) < 0x1p100f)) return false;
  const float delta = __fmul_rn(__fadd_ru(fabsf(o), fabsf(ph)), 0x1p-40f);
  const float pow2 = __uint_as_float(__float_as_uint(arh) & 0x7f800000u);  // 2^exponent(rh)
  // half the gap to the nearer neighbour: ulp / 2, or ulp / 4 at a power of two
  const float half = arh == pow2 ? __fmul_rn(pow2, 0x1p-25f) : __fmul_rn(pow2, 0x1p-24f);
  if (!(__fadd_ru(fabsf(rl), delta) < half) && !(k.a_exact && el == 0.0f && s2e == 0.0f)) return false;
  out = rh;
  return true;
}

template <typename Tp>
__global__ void __launch_bounds__(kT) k_unsharp(const char* in, int64_t ip0, int64_t ip1, int64_t ip2, const char* blur,
                                                 int64_t bp0, int64_t bp1, int64_t bp2, char* out, int64_t op0,
                                                 int64_t op1, int64_t op2, int64_t m0, int64_t m1, int64_t m2,
                                                 int comps, const UnsharpConsts k) {
  const int64_t x = (int64_t)blockIdx.x * kT + threadIdx.x;
  if (x >= m0) return;
  for (int64_t z = blockIdx.z; z < m2; z += gridDim.z)
    for (int64_t y = blockIdx.y; y < m1; y += gridDim.y) {
      const Tp o = *reinterpret_cast<const Tp*>(in + x * ip0 + y * ip1 + z * ip2);
      const Tp b = *reinterpret_cast<const Tp*>(blur + x * bp0 + y * bp1 + z * bp2);
      char* const dst = out + x * op0 + y * op1 + z * op2;
      if constexpr (sizeof(Tp) == 1) {
        const uint8_t q = u8_of(unsharp_f64((double)o, (double)b, k.amount, k.threshold));
        for (int c = 0; c < comps; ++c) reinterpret_cast<uint8_t*>(dst)[c] = q;
      } else {
        float q;
        if (!k.fast || !unsharp_fast_f32(o, b, k, q))
          q = __double2float_rn(unsharp_f64((double)o, (double)b, k.amount, k.threshold));
        for (int c = 0; c < comps; ++c) reinterpret_cast<float*>(dst)[c] = q;
      }
    }
}

// The f32 constants of the fast path for `amount` and `threshold`.
UnsharpConsts make_consts(double amount, double threshold) {
  UnsharpConsts k{};
  k.amount = amount;
  k.threshold = threshold;
  const double aa = std::fabs(amount);
  k.fast = (aa <= 0x1p30 && (amount == 0.0 || aa >= 0x1p-30)) ? 1 : 0;  // false for NaN
  k.ah = (float)amount;
  k.al = (float)(amount - (double)k.ah);
  k.a_exact = (double)k.ah == amount ? 1 : 0;
  k.thr_neg = threshold < 0.0 ? 1 : 0;
  if (std::isnan(threshold)) {  // |e| > NaN never holds
    k.thr_up = INFINITY;
    k.thr_dn = INFINITY;
  } else if (threshold <= 0.0) {  // every e != 0 passes
    k.thr_up = -1.0f;
    k.thr_dn = -1.0f;
  } else {
    const double up = threshold * (1.0 + 0x1p-20), dn = threshold * (1.0 - 0x1p-20);
    float fu = (float)up, fd = (float)dn;
    if ((double)fu < up) fu = std::nextafter(fu, INFINITY);
    if ((double)fd > dn) fd = std::nextafter(fd, 0.0f);
    if (threshold < 0x1p-100) {  // |eh| <= 2^-100 is left undecided
      fu = std::max(fu, 0x1p-100f);
      fd = 0.0f;
    }
    k.thr_up = fu;
    k.thr_dn = fd;
  }
  return k;
}

}  // namespace

// in / blur / out: the first requested voxel of each image and their pitches
// (bytes); m: the requested size; comps: components per pixel.
itkg_status launch_unsharp(int dtype, int comps, const void* in, const int64_t* ip, const void* blur,
                           const int64_t* bp, void* out, const int64_t* op, const int64_t* m, double amount,
                           double threshold, void* stream) {
  if (m[0] * m[1] * m[2] == 0) return ITKG_SUCCESS;
  const dim3 gr((unsigned)((m[0] + kT - 1) / kT), (unsigned)std::min<int64_t>(m[1], 65535),
                (unsigned)std::min<int64_t>(m[2], 65535));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const char* ic = static_cast<const char*>(in);
  const char* bc = static_cast<const char*>(blur);
  char* oc = static_cast<char*>(out);
  const UnsharpConsts k = make_consts(amount, threshold);
  if (dtype == ITKG_U8)
    k_unsharp<uint8_t><<<gr, kT, 0, s>>>(ic, ip[0], ip[1], ip[2], bc, bp[0], bp[1], bp[2], oc, op[0], op[1], op[2],
                                         m[0], m[1], m[2], comps, k);
  else
    k_unsharp<float><<<gr, kT, 0, s>>>(ic, ip[0], ip[1], ip[2], bc, bp[0], bp[1], bp[2], oc, op[0], op[1], op[2],
                                       m[0], m[1], m[2], comps, k);
  note_launch("unsharp");
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "unsharp launch: %s", cudaGetErrorString(e));
  return ITKG_SUCCESS;
}

}  // namespace itkg
