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
// f64 arithmetic runs at a small fraction of the f32 rate on this GPU, so in
// reference rounding the f32 kernel gets the reference's result from f32
// arithmetic and falls back to the f64 sequence only for voxels it cannot
// decide (unsharp_fast_f32); FMA rounding takes one f32 FMA per voxel
// (unsharp_cheap_f32), and in 3-D the two-pass z kernel applies it as it
// stores the blur.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "internal.hpp"
#include "unsharp.cuh"

namespace itkg {
namespace {

constexpr int kT = 256;

__device__ __forceinline__ uint8_t u8_of(double v) {
  double r = round(v);
  r = fmin(fmax(r, 0.0), 255.0);
  return (uint8_t)r;
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
        uint8_t q;
        if (!k.fast || !unsharp_fast_u8(o, b, k, q)) q = u8_of(unsharp_f64((double)o, (double)b, k.amount, k.threshold));
        for (int c = 0; c < comps; ++c) reinterpret_cast<uint8_t*>(dst)[c] = q;
      } else {
        const float q = unsharp_f32(o, b, k);
        for (int c = 0; c < comps; ++c) reinterpret_cast<float*>(dst)[c] = q;
      }
    }
}


// Scalar f32 rows of 16-byte aligned quads (x pitch 4, width a multiple of 4,
// 16-byte aligned rows): thread i of the grid takes quads i, i + grid, ... of
// the rows x quads space, streaming loads and stores.  I: the index type
// (32-bit when the voxel count allows, for cheaper divisions).
//
// Voxels the f32 test cannot decide (a few in a thousand on smooth data) are
// not computed in place: in f64 a warp would stall on every one of them.  The
// block appends (quad index * 4 + lane) to its own segment of `defer`
// (kDeferCap entries; its count in defer_n[block]) and k_unsharp_deferred
// finishes them afterwards, a handful of f64 sequences per block.  Entries
// past the segment's capacity are computed in place.
constexpr int kQT = 256;
constexpr int kDeferCap = 2048;

template <typename I>
__device__ __forceinline__ void quad_addr(I i, I nq, I m1, int64_t p1, int64_t p2, int64_t& off, I& qx) {
  const I row = i / nq;
  qx = i - row * nq;
  const I z = row / m1;
  const I y = row - z * m1;
  off = (int64_t)y * p1 + (int64_t)z * p2;
}

template <typename I>
__global__ void __launch_bounds__(kQT) k_unsharp_quads(const char* in, int64_t ip1, int64_t ip2, const char* blur,
                                                        int64_t bp1, int64_t bp2, char* out, int64_t op1, int64_t op2,
                                                        I nq, I m1, I total, const UnsharpConsts k, I* defer,
                                                        uint32_t* defer_n) {
  __shared__ uint32_t n_def;
  if (threadIdx.x == 0) n_def = 0;
  __syncthreads();
  I* const seg = defer + (size_t)blockIdx.x * kDeferCap;
  // two quads per step (i and i + stride), their loads issued together
  const I stride = (I)gridDim.x * kQT;
  for (I i0 = (I)blockIdx.x * kQT + threadIdx.x; i0 < total; i0 += 2 * stride) {
    float4 o[2], b[2];
    int64_t ooff[2];
    I qxs[2];
    bool live[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const I i = i0 + (I)h * stride;
      live[h] = i < total;
      if (!live[h]) continue;
      const I row = i / nq;
      const I qx = i - row * nq;
      const I z = row / m1;
      const I y = row - z * m1;
      qxs[h] = qx;
      ooff[h] = (int64_t)y * op1 + (int64_t)z * op2;
      o[h] = __ldcs(reinterpret_cast<const float4*>(in + (int64_t)y * ip1 + (int64_t)z * ip2) + qx);
      b[h] = __ldcs(reinterpret_cast<const float4*>(blur + (int64_t)y * bp1 + (int64_t)z * bp2) + qx);
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (!live[h]) continue;
      const I i = i0 + (I)h * stride;
      const float ov[4] = {o[h].x, o[h].y, o[h].z, o[h].w}, bv[4] = {b[h].x, b[h].y, b[h].z, b[h].w};
      float r[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        if (k.cheap) {
          r[c] = unsharp_cheap_f32(ov[c], bv[c], k);
        } else if (!unsharp_fast_f32(ov[c], bv[c], k, r[c])) {
          const uint32_t slot = atomicAdd(&n_def, 1u);
          if (slot < kDeferCap) {
            seg[slot] = i * 4 + (I)c;
            r[c] = ov[c];  // overwritten by k_unsharp_deferred
          } else {
            r[c] = __double2float_rn(unsharp_f64((double)ov[c], (double)bv[c], k.amount, k.threshold));
          }
        }
      }
      __stcs(reinterpret_cast<float4*>(out + ooff[h]) + qxs[h], make_float4(r[0], r[1], r[2], r[3]));
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) defer_n[blockIdx.x] = min(n_def, (uint32_t)kDeferCap);
}

// The voxels k_unsharp_quads deferred: block b takes segment b.
template <typename I>
__global__ void __launch_bounds__(kQT) k_unsharp_deferred(const char* in, int64_t ip1, int64_t ip2, const char* blur,
                                                           int64_t bp1, int64_t bp2, char* out, int64_t op1,
                                                           int64_t op2, I nq, I m1, const UnsharpConsts k,
                                                           const I* defer, const uint32_t* defer_n) {
  const uint32_t n = defer_n[blockIdx.x];
  const I* const seg = defer + (size_t)blockIdx.x * kDeferCap;
  for (uint32_t j = threadIdx.x; j < n; j += kQT) {
    const I e = seg[j];
    const I i = e >> 2;
    const int c = (int)(e & 3);
    int64_t off;
    I qx;
    quad_addr(i, nq, m1, ip1, ip2, off, qx);
    const float o = reinterpret_cast<const float*>(in + off)[4 * (int64_t)qx + c];
    quad_addr(i, nq, m1, bp1, bp2, off, qx);
    const float b = reinterpret_cast<const float*>(blur + off)[4 * (int64_t)qx + c];
    quad_addr(i, nq, m1, op1, op2, off, qx);
    reinterpret_cast<float*>(out + off)[4 * (int64_t)qx + c] =
        __double2float_rn(unsharp_f64((double)o, (double)b, k.amount, k.threshold));
  }
}

// Scalar u8 rows of 4-byte aligned quads (x pitch 1, width a multiple of 4):
// four voxels per thread from 4-byte loads; undecided voxels in f64 in place
// (none on smooth data).
__global__ void __launch_bounds__(kQT) k_unsharp_u8_quads(const char* in, int64_t ip1, int64_t ip2, const char* blur,
                                                           int64_t bp1, int64_t bp2, char* out, int64_t op1,
                                                           int64_t op2, uint32_t nq, uint32_t m1, uint32_t total,
                                                           const UnsharpConsts k) {
  for (uint32_t i = blockIdx.x * kQT + threadIdx.x; i < total; i += gridDim.x * kQT) {
    const uint32_t row = i / nq;
    const uint32_t qx = i - row * nq;
    const uint32_t z = row / m1;
    const uint32_t y = row - z * m1;
    const uchar4 o = reinterpret_cast<const uchar4*>(in + (int64_t)y * ip1 + (int64_t)z * ip2)[qx];
    const uchar4 b = reinterpret_cast<const uchar4*>(blur + (int64_t)y * bp1 + (int64_t)z * bp2)[qx];
    const uint8_t ov[4] = {o.x, o.y, o.z, o.w}, bv[4] = {b.x, b.y, b.z, b.w};
    uint8_t r[4];
#pragma unroll
    for (int c = 0; c < 4; ++c)
      if (!k.fast || !unsharp_fast_u8(ov[c], bv[c], k, r[c]))
        r[c] = u8_of(unsharp_f64((double)ov[c], (double)bv[c], k.amount, k.threshold));
    reinterpret_cast<uchar4*>(out + (int64_t)y * op1 + (int64_t)z * op2)[qx] = make_uchar4(r[0], r[1], r[2], r[3]);
  }
}

template <typename I>
itkg_status launch_quads(const char* ic, const int64_t* ip, const char* bc, const int64_t* bp, char* oc,
                         const int64_t* op, const int64_t* m, uint64_t total, unsigned blocks, const UnsharpConsts& k,
                         cudaStream_t s) {
  void* scratch = nullptr;
  const size_t list_bytes = (size_t)blocks * kDeferCap * sizeof(I);
  itkg_status st = scratch_alloc(&scratch, list_bytes + (size_t)blocks * sizeof(uint32_t), s);
  if (st != ITKG_SUCCESS) return st;
  I* const defer = static_cast<I*>(scratch);
  uint32_t* const defer_n = reinterpret_cast<uint32_t*>(static_cast<char*>(scratch) + list_bytes);
  k_unsharp_quads<I><<<blocks, kQT, 0, s>>>(ic, ip[1], ip[2], bc, bp[1], bp[2], oc, op[1], op[2], (I)(m[0] / 4),
                                            (I)m[1], (I)total, k, defer, defer_n);
  note_launch("unsharp");
  k_unsharp_deferred<I><<<blocks, kQT, 0, s>>>(ic, ip[1], ip[2], bc, bp[1], bp[2], oc, op[1], op[2], (I)(m[0] / 4),
                                               (I)m[1], k, defer, defer_n);
  note_launch("unsharp_deferred");
  scratch_free(scratch, s);
  return ITKG_SUCCESS;
}

}  // namespace

// The f32 constants of the fast path for `amount` and `threshold`.
UnsharpConsts unsharp_consts(double amount, double threshold, bool cheap) {
  UnsharpConsts k{};
  k.cheap = cheap ? 1 : 0;
  k.amount = amount;
  k.threshold = threshold;
  const double aa = std::fabs(amount);
  k.fast = (aa <= 0x1p30 && (amount == 0.0 || aa >= 0x1p-30)) ? 1 : 0;  // false for NaN
  k.ah = (float)amount;
  k.al = (float)(amount - (double)k.ah);
  k.a_exact = (double)k.ah == amount ? 1 : 0;
  k.thr_neg = threshold < 0.0 ? 1 : 0;
  // |e| > threshold for an integer |e| <= 255: |e| >= floor(threshold) + 1
  if (std::isnan(threshold)) k.u8_min_pass = INFINITY;
  else if (threshold < 0.0) k.u8_min_pass = 0.0f;
  else k.u8_min_pass = threshold >= 256.0 ? 256.0f : (float)(std::floor(threshold) + 1.0);
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

// in / blur / out: the first requested voxel of each image and their pitches
// (bytes); m: the requested size; comps: components per pixel.
itkg_status launch_unsharp(int dtype, int comps, const void* in, const int64_t* ip, const void* blur,
                           const int64_t* bp, void* out, const int64_t* op, const int64_t* m, double amount,
                           double threshold, int rounding, void* stream) {
  if (m[0] * m[1] * m[2] == 0) return ITKG_SUCCESS;
  const dim3 gr((unsigned)((m[0] + kT - 1) / kT), (unsigned)std::min<int64_t>(m[1], 65535),
                (unsigned)std::min<int64_t>(m[2], 65535));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const char* ic = static_cast<const char*>(in);
  const char* bc = static_cast<const char*>(blur);
  char* oc = static_cast<char*>(out);
  const UnsharpConsts k = unsharp_consts(amount, threshold, rounding == ITKG_ROUND_FMA);
  auto a16 = [](const void* p, int64_t p1, int64_t p2) {
    return ((uintptr_t)p % 16) == 0 && p1 % 16 == 0 && p2 % 16 == 0;
  };
  const bool quads = dtype == ITKG_F32 && k.fast && comps == 1 && ip[0] == 4 && bp[0] == 4 && op[0] == 4 && m[0] % 4 == 0 &&
                     m[0] / 4 <= UINT32_MAX && m[1] <= UINT32_MAX && a16(in, ip[1], ip[2]) &&
                     a16(blur, bp[1], bp[2]) && a16(out, op[1], op[2]);
  if (quads) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t total = (uint64_t)(m[0] / 4) * (uint64_t)m[1] * (uint64_t)m[2];
    // one full wave of resident blocks (each thread takes two quads per step)
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_unsharp_quads<uint32_t>, kQT, 0);
    const uint64_t blocks =
        std::min<uint64_t>((total + 2 * kQT - 1) / (2 * kQT), (uint64_t)std::max(sms, 1) * std::max(per_sm, 1));
    // quad indices * 4 + 3 must fit the index type
    const itkg_status st = 4 * (total + (uint64_t)blocks * kQT) < UINT32_MAX
                               ? launch_quads<uint32_t>(ic, ip, bc, bp, oc, op, m, total, (unsigned)blocks, k, s)
                               : launch_quads<uint64_t>(ic, ip, bc, bp, oc, op, m, total, (unsigned)blocks, k, s);
    if (st != ITKG_SUCCESS) return st;
  } else if (dtype == ITKG_U8 && comps == 1 && ip[0] == 1 && bp[0] == 1 && op[0] == 1 && m[0] % 4 == 0 &&
             (uint64_t)(m[0] / 4) * (uint64_t)m[1] * (uint64_t)m[2] + (uint64_t)kQT * 65536 < UINT32_MAX &&
             ((uintptr_t)in % 4) == 0 && ((uintptr_t)blur % 4) == 0 && ((uintptr_t)out % 4) == 0 &&
             ip[1] % 4 == 0 && ip[2] % 4 == 0 && bp[1] % 4 == 0 && bp[2] % 4 == 0 && op[1] % 4 == 0 &&
             op[2] % 4 == 0) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t total = (uint32_t)((m[0] / 4) * m[1] * m[2]);
    const uint32_t blocks = std::min<uint32_t>((total + kQT - 1) / kQT, (uint32_t)std::max(sms, 1) * 8);
    k_unsharp_u8_quads<<<blocks, kQT, 0, s>>>(ic, ip[1], ip[2], bc, bp[1], bp[2], oc, op[1], op[2],
                                             (uint32_t)(m[0] / 4), (uint32_t)m[1], total, k);
    note_launch("unsharp_u8");
  } else if (dtype == ITKG_U8) {
    k_unsharp<uint8_t><<<gr, kT, 0, s>>>(ic, ip[0], ip[1], ip[2], bc, bp[0], bp[1], bp[2], oc, op[0], op[1], op[2],
                                         m[0], m[1], m[2], comps, k);
    note_launch("unsharp");
  } else {
    k_unsharp<float><<<gr, kT, 0, s>>>(ic, ip[0], ip[1], ip[2], bc, bp[0], bp[1], bp[2], oc, op[0], op[1], op[2],
                                       m[0], m[1], m[2], comps, k);
    note_launch("unsharp");
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "unsharp launch: %s", cudaGetErrorString(e));
  return ITKG_SUCCESS;
}

}  // namespace itkg
