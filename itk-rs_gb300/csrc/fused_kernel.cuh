// Fused 3-D Gaussian kernels (templates).  Included by the translation units
// that instantiate them per input element type (fused.cu, fused_in16.cu,
// fused_in8.cu); see fused.cu for the design.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <mutex>
#include <vector>

#include "f32x2.cuh"
#include "internal.hpp"
#include "pixel.cuh"

#include <type_traits>

namespace itkg {
namespace fusedk {

constexpr int kMaxFusedR = 12;
constexpr int kMaxFusedK = 2 * kMaxFusedR + 1;

// What a fused launch computes.
//   kFwd  y = G x stored (or converted) into dst;
//   kDot  <ybar, G x> summed per CTA into partials[blockIdx.x] (nothing stored;
//         with derivative weights on one axis this is one term of dL/dsigma);
//   kAdj  dst (+)= G^T x for the whole image: the halo outside the image is
//         zero (not replicated) and the edge outputs of every pass add the
//         clamped taps back, sum_{d<r} P[r-1-d] v[edge -/+ d] (P = prefix sums
//         of the weights).
enum FusedMode { kFwd = 0, kDot = 1, kAdj = 2 };

struct Fused3DArgs {
  const char* src;
  char* dst;
  int64_t src_pitch[3];  // bytes
  int64_t dst_pitch[3];
  int32_t src_origin[3];
  int32_t dst_origin[3];
  int32_t req_lo[3];  // requested region, inclusive bounds
  int32_t req_hi[3];
  int32_t lo[3];  // gather bounds (image bounds within the input buffer), inclusive
  int32_t hi[3];
  int32_t ntx, nty;  // tiles along x and y
  int64_t units;     // ntx * nty * nz_requested
  int32_t out_dtype;
  int32_t pad_;
  unsigned int* fault;  // device fault word, set when a bounded wait gives up
  long long wait_limit; // clock cycles a wait on a tile load may take
  // kDot: ybar (f32) at the output positions, and one f64 partial per CTA
  const char* ybar;
  int64_t ybar_pitch[3];
  int32_t ybar_origin[3];
  int32_t accumulate;  // kAdj: dst += result
  double* partials;
  float wx[kMaxFusedK];
  float wy[kMaxFusedK];
  float wz[kMaxFusedK];
  f2_t wx2[kMaxFusedK];  // {w, w} pairs for the packed passes
  f2_t wy2[kMaxFusedK];
  f2_t wz2[kMaxFusedK];
  float px[kMaxFusedK];  // kAdj: prefix sums of the weights
  float py[kMaxFusedK];
  float pz[kMaxFusedK];
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void cp_async4(uint32_t saddr, const void* g) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(saddr), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_test_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up after `limit` clock cycles (by default 2^31, about a
// second) and reports false.  With a limit below kWaitSpinBelow the wait polls
// without suspending (a try_wait may suspend the thread for a while by
// itself), so that a short limit set for a test is kept to.
constexpr long long kWaitDefault = 1ll << 31;
constexpr long long kWaitSpinBelow = 1ll << 16;
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long limit = kWaitDefault) {
  if (mbar_test_wait(bar, parity)) return true;
  const long long t0 = clock64();
  if (limit < kWaitSpinBelow) {
    while (!mbar_test_wait(bar, parity))
      if (clock64() - t0 > limit) return false;
    return true;
  }
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Tile shape per radius and input element type.
template <int RX, int RY, int RZ, typename Tin>
struct Cfg3 {
  static constexpr int KX = 2 * RX + 1, KY = 2 * RY + 1, KZ = 2 * RZ + 1;
  static constexpr int ESZ = (int)sizeof(Tin);       // input element bytes
  static constexpr int NT = 256;                    // threads per CTA
  static constexpr int NW = NT / 32;
  static constexpr int TX = 32;                     // one lane per output column
  static constexpr int MY = RZ <= 8 ? 4 : 2;        // rows per thread (y pass, z ring)
  static constexpr int MY2 = MY / 2;                // packed row pairs
  static constexpr int TY = NW * MY;
  static constexpr int MX = 8;                      // x outputs per x-pass task
  static constexpr int AE = 16 / ESZ;               // elements per 16 bytes (TMA x alignment)
  static constexpr int XA = (RX + AE - 1) / AE * AE;  // x halo rounded up to 16 bytes
  static constexpr int BW = TX + 2 * XA;            // staged tile width (elements)
  static constexpr int IH = TY + 2 * RY;            // staged tile height
  static constexpr int OFF = (XA - RX) % 4;         // window misalignment
  static constexpr int WB = XA - RX - OFF;          // aligned window start (col)
  static constexpr int WIN = (MX + 2 * RX + OFF + 3) / 4 * 4;  // x-pass window (elements)
  static constexpr int S = 4;                       // slices in flight
  static constexpr int BOX = IH * BW * ESZ;         // bytes of one tile load
  static constexpr int STAGE = (BOX + 127) / 128 * 128;  // bytes per stage (128-byte multiple)
  static constexpr int NLD = (IH * BW + NT - 1) / NT;  // gather elements per thread (f32 gather)
  static constexpr size_t SMEM = (size_t)S * STAGE + sizeof(float) * 2 * IH * TX + 128;
  static constexpr int MINB = 2;
  static_assert(WB + TX - MX + WIN <= BW, "x window stays inside the staged row");
  static_assert(TX % MX == 0, "x segments");
};

// Four consecutive staged elements -> f32 (exact conversions; the reference's
// UnaryFilter(|p| p as f32), examples/blur_png.rs:35).
__device__ __forceinline__ void load4(const float* p, float* v) {
  const float4 f = *reinterpret_cast<const float4*>(p);
  v[0] = f.x, v[1] = f.y, v[2] = f.z, v[3] = f.w;
}
__device__ __forceinline__ void load4(const int16_t* p, float* v) {
  const uint2 u = *reinterpret_cast<const uint2*>(p);
  v[0] = (float)(int16_t)(u.x & 0xffffu), v[1] = (float)(int16_t)(u.x >> 16);
  v[2] = (float)(int16_t)(u.y & 0xffffu), v[3] = (float)(int16_t)(u.y >> 16);
}
__device__ __forceinline__ void load4(const uint8_t* p, float* v) {
  const uint32_t u = *reinterpret_cast<const uint32_t*>(p);
  v[0] = (float)(u & 0xffu), v[1] = (float)((u >> 8) & 0xffu);
  v[2] = (float)((u >> 16) & 0xffu), v[3] = (float)(u >> 24);
}
__device__ __forceinline__ void load4(const __nv_bfloat16* p, float* v) {
  const uint2 u = *reinterpret_cast<const uint2*>(p);
  v[0] = __uint_as_float(u.x << 16), v[1] = __uint_as_float(u.x & 0xffff0000u);
  v[2] = __uint_as_float(u.y << 16), v[3] = __uint_as_float(u.y & 0xffff0000u);
}
__device__ __forceinline__ void load4(const __half* p, float* v) {
  const uint2 u = *reinterpret_cast<const uint2*>(p);
  v[0] = __half2float(__ushort_as_half((unsigned short)(u.x & 0xffffu)));
  v[1] = __half2float(__ushort_as_half((unsigned short)(u.x >> 16)));
  v[2] = __half2float(__ushort_as_half((unsigned short)(u.y & 0xffffu)));
  v[3] = __half2float(__ushort_as_half((unsigned short)(u.y >> 16)));
}

// z pass for phase P: push the packed y-filtered values into every ring slot,
// then hand back the completed slot (P + 1) mod KZ and clear it.
template <int P, int KZ, int MY2, bool REF>
__device__ __forceinline__ void push_phase(f2_t (&acc)[MY2][KZ], const f2_t (&yv)[MY2],
                                           const Fused3DArgs& a, f2_t (&done)[MY2], bool push) {
#pragma unroll
  for (int k = 0; k < KZ && push; ++k) {
    const int slot = (P - k + KZ) % KZ;
#pragma unroll
    for (int m = 0; m < MY2; ++m) {
      if constexpr (REF) {
        float a0, a1, v0, v1;
        unpack2(acc[m][slot], a0, a1);
        unpack2(yv[m], v0, v1);
        acc[m][slot] = pack2(__fadd_rn(a0, __fmul_rn(v0, a.wz[k])), __fadd_rn(a1, __fmul_rn(v1, a.wz[k])));
      } else {
        acc[m][slot] = fma2(yv[m], a.wz2[k], acc[m][slot]);
      }
    }
  }
  constexpr int D = (P + 1) % KZ;
#pragma unroll
  for (int m = 0; m < MY2; ++m) {
    done[m] = acc[m][D];
    acc[m][D] = 0ull;
  }
}

#define ITKG_PUSH_CASE(N)                                                   \
  case N:                                                                   \
    if constexpr (N < KZ) push_phase<N, KZ, MY2, REF>(acc, yv, a, done, do_push);    \
    break;

// The fused filter over units [u_begin, u_end) of one request `a` (a unit is
// one output slice of one (x, y) tile).  Returns false if a bounded wait gave
// up (the device fault word is then set).
template <int RX, int RY, int RZ, bool REF, bool TMA, typename Tin, int MODE = kFwd>
__device__ __forceinline__ bool fused_range(const Fused3DArgs& a, const CUtensorMap* tmap,
                                            int64_t u_begin, int64_t u_end, unsigned char* const stage0,
                                            uint32_t bbase, uint32_t& phase_bits) {
  using C = Cfg3<RX, RY, RZ, Tin>;
  constexpr int KX = C::KX, KY = C::KY, KZ = C::KZ, TX = C::TX, TY = C::TY, MY = C::MY,
                MY2 = C::MY2, MX = C::MX, BW = C::BW, IH = C::IH, XA = C::XA, S = C::S,
                NLD = C::NLD, NT = C::NT, WIN = C::WIN, WB = C::WB, OFF = C::OFF;
  static_assert(KZ <= 25, "phase switch covers KZ <= 25");
  float* const xs = reinterpret_cast<float*>(stage0 + S * C::STAGE);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nzr = a.req_hi[2] - a.req_lo[2] + 1;
  const uint32_t sbase = smem_u32(stage0);
  double dot_acc = 0.0;  // kDot: this thread's share of <ybar, G x> (f32 runs of 8 slices folded in)
  float dot_f = 0.0f;
  int dot_n = 0;

  for (int64_t u = u_begin; u < u_end;) {
    const int64_t tile = u / nzr;
    const int zs = (int)(u % nzr);
    const int64_t zrem = zs + (u_end - u);
    const int ze = zrem < nzr ? (int)zrem : nzr;
    u += ze - zs;
    const int z0 = a.req_lo[2] + zs, z1 = a.req_lo[2] + ze;  // outputs [z0, z1)
    const int tx0 = a.req_lo[0] + (int)(tile % a.ntx) * TX;
    const int ty0 = a.req_lo[1] + (int)(tile / a.ntx) * TY;
    const int gx0 = tx0 - XA, gy0 = ty0 - RY;  // image coords of stage element (0, 0)
    const bool edge = gx0 < a.lo[0] || gx0 + BW - 1 > a.hi[0] || gy0 < a.lo[1] || gy0 + IH - 1 > a.hi[1];
    // kAdj: does this tile hold an edge column / row of the image?
    const bool xedge = (a.lo[0] >= tx0 && a.lo[0] < tx0 + TX) || (a.hi[0] >= tx0 && a.hi[0] < tx0 + TX);
    const bool yedge = (a.lo[1] >= ty0 && a.lo[1] < ty0 + TY) || (a.hi[1] >= ty0 && a.hi[1] < ty0 + TY);
    (void)xedge;
    (void)yedge;

    // cp.async path: gather offsets of this thread's share (clamped x, y).
    int32_t goff[TMA ? 1 : NLD];
    if constexpr (!TMA) {
#pragma unroll
      for (int i = 0; i < NLD; ++i) {
        const int e = tid + i * NT;
        const int gx = clampi(gx0 + e % BW, a.lo[0], a.hi[0]);
        const int gy = clampi(gy0 + e / BW, a.lo[1], a.hi[1]);
        goff[i] = (int32_t)((gx - a.src_origin[0]) * a.src_pitch[0] +
                            (gy - a.src_origin[1]) * a.src_pitch[1]);
      }
    }
    auto issue = [&](int s, int st) {
      if constexpr (TMA) {
        if (tid == 0) {
          asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
          const uint32_t bar = bbase + 8 * st;
          mbar_expect_tx(bar, (uint32_t)C::BOX);  // bytes of one box
          tma_load_3d(sbase + (uint32_t)(st * C::STAGE), tmap, gx0 - a.src_origin[0],
                      gy0 - a.src_origin[1], s - a.src_origin[2], bar);
        }
      } else {
        const char* base = a.src + (int64_t)(s - a.src_origin[2]) * a.src_pitch[2];
        const uint32_t sb = sbase + (uint32_t)(st * C::STAGE);
#pragma unroll
        for (int i = 0; i < NLD; ++i) {
          const int e = tid + i * NT;
          if (i < NLD - 1 || e < IH * BW) cp_async4(sb + (uint32_t)e * 4u, base + goff[i]);
        }
        cp_async_commit();
      }
    };

    const int jb = z0 - RZ, je = z1 - 1 + RZ;
    const int s_first = max(jb, a.lo[2]), s_last = min(je, a.hi[2]);
    for (int q = 0; q < S; ++q) {
      if (s_first + q <= s_last) issue(s_first + q, q);
      else if (!TMA) cp_async_commit();
    }

    f2_t acc[MY2][KZ];
#pragma unroll
    for (int m = 0; m < MY2; ++m)
#pragma unroll
      for (int q = 0; q < KZ; ++q) acc[m][q] = 0ull;
    f2_t yv[MY2];
#pragma unroll
    for (int m = 0; m < MY2; ++m) yv[m] = 0ull;
    f2_t acc_lo[MY2], acc_hi[MY2];  // kAdj: z-edge folds of outputs lo and hi
#pragma unroll
    for (int m = 0; m < MY2; ++m) acc_lo[m] = acc_hi[m] = 0ull;

    // Output addressing for this thread's column and rows.
    const int col_x = tx0 + lane;
    const int row_y0 = ty0 + warp * MY;
    const bool col_ok = col_x <= a.req_hi[0];
    int nrows_ok = a.req_hi[1] - row_y0 + 1;
    nrows_ok = nrows_ok < 0 ? 0 : (nrows_ok > MY ? MY : nrows_ok);
    char* const obase = a.dst + (int64_t)(col_x - a.dst_origin[0]) * a.dst_pitch[0] +
                        (int64_t)(row_y0 - a.dst_origin[1]) * a.dst_pitch[1];
    const int64_t opy = a.dst_pitch[1];

    // Stage slice s (already issued into stage st) and run its x pass into
    // xbuf.  Returns false if the bounded wait on the tile load gave up.
    auto stage_and_xpass = [&](int st, float* xbuf) -> bool {
      Tin* const tile = reinterpret_cast<Tin*>(stage0 + st * C::STAGE);
      if constexpr (TMA) {
        const bool ok = mbar_wait(bbase + 8 * st, (phase_bits >> st) & 1u, a.wait_limit);
        phase_bits ^= 1u << st;
        if (MODE != kAdj && edge) {
          // Replicate the image's edge values into the halo: first the
          // columns left of lo / right of hi (nl, nr of them), then whole
          // rows above / below (nt, nb of them).  Sources are in-image
          // columns and rows, which these loops never write.  Each thread
          // timed its own wait: the CTA agrees on the outcome at this
          // barrier, so that every thread leaves here or none does.
          if (!__syncthreads_and(ok)) return false;
          const int nl = max(0, a.lo[0] - gx0), nr = max(0, gx0 + BW - 1 - a.hi[0]);
          const int ncol = nl + nr;
          for (int e = tid; e < ncol * IH; e += NT) {
            const int r = e / ncol, i = e % ncol;
            const int c = i < nl ? i : BW - 1 - (i - nl);
            tile[r * BW + c] = tile[r * BW + clampi(gx0 + c, a.lo[0], a.hi[0]) - gx0];
          }
          __syncthreads();
          const int nt = max(0, a.lo[1] - gy0), nb = max(0, gy0 + IH - 1 - a.hi[1]);
          for (int e = tid; e < (nt + nb) * BW; e += NT) {
            const int i = e / BW, c = e % BW;
            const int r = i < nt ? i : IH - 1 - (i - nt);
            tile[r * BW + c] = tile[(clampi(gy0 + r, a.lo[1], a.hi[1]) - gy0) * BW + c];
          }
          __syncthreads();
        }
        if (!ok) return false;  // no barrier here: the caller's __syncthreads_or sees it
      } else {
        cp_async_wait<S - 1>();
        __syncthreads();
      }
      constexpr int SEGS = TX / MX;
      for (int t = tid; t < IH * SEGS; t += NT) {
        const int row = t / SEGS, x0 = (t % SEGS) * MX;
        float v[WIN];
        const Tin* src = tile + row * BW + x0 + WB;
#pragma unroll
        for (int q = 0; q < WIN / 4; ++q) load4(src + 4 * q, v + 4 * q);
        float o[MX];
        if constexpr (REF) {
#pragma unroll
          for (int m = 0; m < MX; ++m) {
            float ax = 0.0f;
#pragma unroll
            for (int k = 0; k < KX; ++k) ax = tap<true>(ax, v[m + k + OFF], a.wx[k]);
            o[m] = ax;
          }
        } else {
          // even/odd aligned pairs of the window: E[i] = (v[2i], v[2i+1]), O[i] = (v[2i+1], v[2i+2])
          f2_t E[WIN / 2], O[WIN / 2 - 1];
#pragma unroll
          for (int i = 0; i < WIN / 2; ++i) E[i] = pack2(v[2 * i], v[2 * i + 1]);
#pragma unroll
          for (int i = 0; i < WIN / 2 - 1; ++i) O[i] = pack2(v[2 * i + 1], v[2 * i + 2]);
#pragma unroll
          for (int m = 0; m < MX / 2; ++m) {
            f2_t ax = 0ull;
#pragma unroll
            for (int k = 0; k < KX; ++k) {
              const int q = 2 * m + k + OFF;
              ax = fma2((q & 1) ? O[(q - 1) / 2] : E[q / 2], a.wx2[k], ax);
            }
            unpack2(ax, o[2 * m], o[2 * m + 1]);
          }
          if constexpr (MODE == kAdj) {
            if (xedge) {  // the taps the forward clamped onto the edge columns
#pragma unroll
              for (int m = 0; m < MX; ++m) {
                const int X = tx0 + x0 + m;
                if (X == a.lo[0])
#pragma unroll
                  for (int d = 0; d < RX; ++d) o[m] = fmaf(a.px[RX - 1 - d], v[m + RX + d + OFF], o[m]);
                if (X == a.hi[0])
#pragma unroll
                  for (int d = 0; d < RX; ++d) o[m] = fmaf(a.px[RX - 1 - d], v[m + RX - d + OFF], o[m]);
              }
            }
          }
        }
        float4* dst4 = reinterpret_cast<float4*>(xbuf + row * TX + x0);
#pragma unroll
        for (int q = 0; q < MX / 4; ++q)
          dst4[q] = make_float4(o[4 * q], o[4 * q + 1], o[4 * q + 2], o[4 * q + 3]);
      }
      return true;
    };
    // A tile load did not complete in time: record it, let every issued load
    // land (the one given up on included, whose phase bit was already
    // flipped; default bound), and leave.
#define ITKG_ON_TIMEOUT(CONS_NOW)                                                  \
  do {                                                                             \
    if (tid == 0) {                                                                \
      atomicExch(a.fault, 1u);                                                     \
      if (TMA)                                                                     \
        for (int q_ = 0; q_ < S; ++q_) {                                           \
          const int sq_ = ((CONS_NOW) + q_) % S;                                   \
          if (s_first + (CONS_NOW) + q_ <= s_last)                                 \
            mbar_wait(bbase + 8 * sq_, ((phase_bits >> sq_) & 1u) ^ (q_ == 0 ? 1u : 0u)); \
        }                                                                          \
    }                                                                              \
  } while (0)

    // Pipeline: the x pass of slice s + 1 runs in the same barrier interval
    // as the y pass of slice s (double-buffered x-filtered tile).
    if (s_first <= s_last) {
      const bool ok = stage_and_xpass(0, xs);
      if (__syncthreads_or(!ok)) {
        ITKG_ON_TIMEOUT(0);
        return false;
      }
    }
    int prev_s = INT_MIN;
    int cons = 0;  // slices consumed by the y pass so far
    int p = 0;     // phase (j - jb) mod KZ
    for (int j = jb; j <= je; ++j) {
      const int s = clampi(j, a.lo[2], a.hi[2]);
      if (s != prev_s) {
        prev_s = s;
        const int st = cons % S;
        if (cons > 0) {
          // x pass of s (previous interval) visible; y pass of s - 1 done
          __syncthreads();
        }
        {
          const int sn = s_first + cons + S;
          if (sn <= s_last) issue(sn, st);
          else if (!TMA) cp_async_commit();
        }
        const float* xcur = xs + (cons & 1) * IH * TX;
        if (s + 1 <= s_last) {
          const bool ok = stage_and_xpass((cons + 1) % S, xs + ((cons + 1) & 1) * IH * TX);
          if (__syncthreads_or(!ok)) {
            ITKG_ON_TIMEOUT(cons + 1);
            return false;
          }
        }
        ++cons;
        // ---- y pass: xcur -> yv (registers, packed in row pairs) ----
        float w[MY + 2 * RY];
#pragma unroll
        for (int i = 0; i < MY + 2 * RY; ++i) w[i] = xcur[(warp * MY + i) * TX + lane];
        if constexpr (REF) {
#pragma unroll
          for (int m = 0; m < MY2; ++m) {
            float y0 = 0.0f, y1 = 0.0f;
#pragma unroll
            for (int k = 0; k < KY; ++k) {
              y0 = tap<true>(y0, w[2 * m + k], a.wy[k]);
              y1 = tap<true>(y1, w[2 * m + 1 + k], a.wy[k]);
            }
            yv[m] = pack2(y0, y1);
          }
        } else {
          constexpr int NWIN = MY + 2 * RY;
          f2_t E[NWIN / 2], O[NWIN / 2];
#pragma unroll
          for (int i = 0; i < NWIN / 2; ++i) E[i] = pack2(w[2 * i], w[2 * i + 1]);
#pragma unroll
          for (int i = 0; i + 1 < NWIN / 2; ++i) O[i] = pack2(w[2 * i + 1], w[2 * i + 2]);
#pragma unroll
          for (int m = 0; m < MY2; ++m) {
            f2_t ay = 0ull;
#pragma unroll
            for (int k = 0; k < KY; ++k) {
              const int q = 2 * m + k;
              ay = fma2((q & 1) ? O[(q - 1) / 2] : E[q / 2], a.wy2[k], ay);
            }
            yv[m] = ay;
          }
          if constexpr (MODE == kAdj) {
            if (yedge) {  // the taps the forward clamped onto the edge rows
              float yl[MY];
#pragma unroll
              for (int m = 0; m < MY2; ++m) unpack2(yv[m], yl[2 * m], yl[2 * m + 1]);
#pragma unroll
              for (int m = 0; m < MY; ++m) {
                const int Y = ty0 + warp * MY + m;
                if (Y == a.lo[1])
#pragma unroll
                  for (int d = 0; d < RY; ++d) yl[m] = fmaf(a.py[RY - 1 - d], w[m + RY + d], yl[m]);
                if (Y == a.hi[1])
#pragma unroll
                  for (int d = 0; d < RY; ++d) yl[m] = fmaf(a.py[RY - 1 - d], w[m + RY - d], yl[m]);
              }
#pragma unroll
              for (int m = 0; m < MY2; ++m) yv[m] = pack2(yl[2 * m], yl[2 * m + 1]);
            }
          }
        }
      }
      // ---- z pass: push slice j into the ring, pop output z = j - RZ ----
      const bool do_push = MODE != kAdj || (j >= a.lo[2] && j <= a.hi[2]);
      if constexpr (MODE == kAdj) {
        // only in-image slices fold (j outside the image carries the clamped
        // slice's values, which the adjoint must not count again)
        const int dl = j - a.lo[2], dh = a.hi[2] - j;
        if (do_push && dl < RZ) {
          const f2_t wp = pack2(a.pz[RZ - 1 - dl], a.pz[RZ - 1 - dl]);
#pragma unroll
          for (int m = 0; m < MY2; ++m) acc_lo[m] = fma2(yv[m], wp, acc_lo[m]);
        }
        if (do_push && dh < RZ) {
          const f2_t wp = pack2(a.pz[RZ - 1 - dh], a.pz[RZ - 1 - dh]);
#pragma unroll
          for (int m = 0; m < MY2; ++m) acc_hi[m] = fma2(yv[m], wp, acc_hi[m]);
        }
      }
      f2_t done[MY2];
      switch (p) {
        ITKG_PUSH_CASE(0) ITKG_PUSH_CASE(1) ITKG_PUSH_CASE(2) ITKG_PUSH_CASE(3)
        ITKG_PUSH_CASE(4) ITKG_PUSH_CASE(5) ITKG_PUSH_CASE(6) ITKG_PUSH_CASE(7)
        ITKG_PUSH_CASE(8) ITKG_PUSH_CASE(9) ITKG_PUSH_CASE(10) ITKG_PUSH_CASE(11)
        ITKG_PUSH_CASE(12) ITKG_PUSH_CASE(13) ITKG_PUSH_CASE(14) ITKG_PUSH_CASE(15)
        ITKG_PUSH_CASE(16) ITKG_PUSH_CASE(17) ITKG_PUSH_CASE(18) ITKG_PUSH_CASE(19)
        ITKG_PUSH_CASE(20) ITKG_PUSH_CASE(21) ITKG_PUSH_CASE(22) ITKG_PUSH_CASE(23)
        ITKG_PUSH_CASE(24)
        default: break;
      }
      p = p + 1 == KZ ? 0 : p + 1;
      const int z = j - RZ;
      if (z >= z0 && col_ok) {
        if constexpr (MODE == kAdj) {
          if (z == a.lo[2])
#pragma unroll
            for (int m = 0; m < MY2; ++m) done[m] = add2(done[m], acc_lo[m]);
          if (z == a.hi[2])
#pragma unroll
            for (int m = 0; m < MY2; ++m) done[m] = add2(done[m], acc_hi[m]);
        }
        float vals[MY];
#pragma unroll
        for (int m = 0; m < MY2; ++m) unpack2(done[m], vals[2 * m], vals[2 * m + 1]);
        if constexpr (MODE == kDot) {
          const char* yrow = a.ybar + (int64_t)(col_x - a.ybar_origin[0]) * a.ybar_pitch[0] +
                             (int64_t)(row_y0 - a.ybar_origin[1]) * a.ybar_pitch[1] +
                             (int64_t)(z - a.ybar_origin[2]) * a.ybar_pitch[2];
          float sl = 0.0f;
#pragma unroll
          for (int m = 0; m < MY; ++m)
            if (m < nrows_ok) sl = fmaf(vals[m], *reinterpret_cast<const float*>(yrow + m * a.ybar_pitch[1]), sl);
          dot_f += sl;
          if (++dot_n == 8) {
            dot_acc += (double)dot_f;
            dot_f = 0.0f;
            dot_n = 0;
          }
        } else if constexpr (MODE == kAdj) {
          char* orow = obase + (int64_t)(z - a.dst_origin[2]) * a.dst_pitch[2];
#pragma unroll
          for (int m = 0; m < MY; ++m)
            if (m < nrows_ok) {
              float* q = reinterpret_cast<float*>(orow + m * opy);
              *q = a.accumulate ? *q + vals[m] : vals[m];
            }
        } else {
        char* orow = obase + (int64_t)(z - a.dst_origin[2]) * a.dst_pitch[2];
        if (a.out_dtype == ITKG_F32) {
#pragma unroll
          for (int m = 0; m < MY; ++m)
            if (m < nrows_ok) __stcs(reinterpret_cast<float*>(orow + m * opy), vals[m]);
        } else {
#pragma unroll
          for (int m = 0; m < MY; ++m) {
            if (m >= nrows_ok) continue;
            char* q = orow + m * opy;
            if (a.out_dtype == ITKG_BF16) *reinterpret_cast<__nv_bfloat16*>(q) = from_f32<__nv_bfloat16>(vals[m]);
            else if (a.out_dtype == ITKG_F16) *reinterpret_cast<__half*>(q) = from_f32<__half>(vals[m]);
            else *reinterpret_cast<uint8_t*>(q) = from_f32<uint8_t>(vals[m]);
          }
        }
        }
      }
    }
    if constexpr (!TMA) cp_async_wait<0>();
    __syncthreads();
  }
#undef ITKG_ON_TIMEOUT
  if constexpr (MODE == kDot) {
    dot_acc += (double)dot_f;
    // block sum of dot_acc -> partials[blockIdx.x] (fixed order)
    __shared__ double red[NT / 32];
    for (int off = 16; off > 0; off >>= 1) dot_acc += __shfl_down_sync(0xffffffffu, dot_acc, off);
    if (lane == 0) red[warp] = dot_acc;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < NT / 32; ++w) t += red[w];
      a.partials[blockIdx.x] = t;
    }
  }
  return true;
}

// Shared-memory set-up common to the single- and multi-request kernels.
#define ITKG_FUSED_PROLOGUE                                                              \
  using C = Cfg3<RX, RY, RZ, Tin>;                                                       \
  extern __shared__ __align__(128) unsigned char smem[];                                 \
  __shared__ __align__(8) uint64_t mbar[C::S];                                           \
  /* TMA destinations must be 128-byte aligned: offset by an index so the compiler */    \
  /* keeps shared-memory addressing. */                                                  \
  unsigned char* const stage0 = smem + ((128u - (smem_u32(smem) & 127u)) & 127u);        \
  const uint32_t bbase = smem_u32(mbar);                                                 \
  if (TMA) {                                                                             \
    if (threadIdx.x == 0) {                                                              \
      for (int i = 0; i < C::S; ++i) mbar_init(bbase + 8 * i, 1);                        \
      asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");               \
    }                                                                                    \
    __syncthreads();                                                                     \
  }                                                                                      \
  uint32_t phase_bits = 0;

template <int RX, int RY, int RZ, bool REF, bool TMA, typename Tin>
__global__ void __launch_bounds__(Cfg3<RX, RY, RZ, Tin>::NT, Cfg3<RX, RY, RZ, Tin>::MINB)
    k_fused3d(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ Fused3DArgs a) {
  ITKG_FUSED_PROLOGUE
  const int64_t u_begin = a.units * blockIdx.x / gridDim.x;
  const int64_t u_end = a.units * (blockIdx.x + 1) / gridDim.x;
  fused_range<RX, RY, RZ, REF, TMA, Tin>(a, &tmap, u_begin, u_end, stage0, bbase, phase_bits);
}

// VJP launches (f32 input, TMA tile loads, FMA rounding): kDot or kAdj.
template <int RX, int RY, int RZ, int MODE>
__global__ void __launch_bounds__(Cfg3<RX, RY, RZ, float>::NT, Cfg3<RX, RY, RZ, float>::MINB)
    k_fused3d_vjp(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ Fused3DArgs a) {
  using Tin = float;
  constexpr bool TMA = true;
  ITKG_FUSED_PROLOGUE
  const int64_t u_begin = a.units * blockIdx.x / gridDim.x;
  const int64_t u_end = a.units * (blockIdx.x + 1) / gridDim.x;
  fused_range<RX, RY, RZ, false, true, float, MODE>(a, &tmap, u_begin, u_end, stage0, bbase, phase_bits);
}

// One request of a multi-request launch; its units are [unit_begin, unit_begin + a.units).
struct FusedItem {
  Fused3DArgs a;
  int64_t unit_begin;
  int64_t pad_[7];
};

struct Entry {
  int rx, ry, rz, dtype;
  void (*fn[2][2])(const CUtensorMap, const Fused3DArgs);  // [ref][tma]
  void (*multi[2][2])(const FusedItem*, const CUtensorMap*, int, int64_t);
  void (*vjp[2])(const CUtensorMap, const Fused3DArgs);  // [0] kDot, [1] kAdj (f32 only)
  size_t smem;
  int tx, ty, nt, xa, bw, ih, ae;
};

// Persistent multi-request launch: the CTAs split the union of all requests'
// units evenly; a CTA copies each request's arguments to shared memory as it
// reaches it and runs the same fused filter on its share.
template <int RX, int RY, int RZ, bool REF, bool TMA, typename Tin>
__global__ void __launch_bounds__(Cfg3<RX, RY, RZ, Tin>::NT, Cfg3<RX, RY, RZ, Tin>::MINB)
    k_fused3d_multi(const FusedItem* __restrict__ items, const CUtensorMap* __restrict__ maps,
                        int nitems, int64_t total_units) {
  ITKG_FUSED_PROLOGUE
  __shared__ __align__(16) Fused3DArgs sa;
  int64_t u = total_units * blockIdx.x / gridDim.x;
  const int64_t u_end = total_units * (blockIdx.x + 1) / gridDim.x;
  int it = 0;
  while (it + 1 < nitems && items[it + 1].unit_begin <= u) ++it;
  while (u < u_end && it < nitems) {
    __syncthreads();  // previous request's arguments no longer in use
    {
      const uint32_t* srcw = reinterpret_cast<const uint32_t*>(&items[it].a);
      uint32_t* dstw = reinterpret_cast<uint32_t*>(&sa);
      for (int i = threadIdx.x; i < (int)(sizeof(Fused3DArgs) / 4); i += C::NT) dstw[i] = srcw[i];
    }
    __syncthreads();
    const int64_t ib = items[it].unit_begin;
    const int64_t e = min(u_end, ib + sa.units);
    if (!fused_range<RX, RY, RZ, REF, TMA, Tin>(sa, &maps[it], u - ib, e - ib, stage0, bbase, phase_bits))
      return;
    u = e;
    ++it;
  }
}
#undef ITKG_FUSED_PROLOGUE

// ---- dispatch table -----------------------------------------------------------
using KernelFn = void (*)(const CUtensorMap, const Fused3DArgs);
using MultiFn = void (*)(const FusedItem*, const CUtensorMap*, int, int64_t);

template <typename T> constexpr int dtype_of();
template <> constexpr int dtype_of<float>() { return ITKG_F32; }
template <> constexpr int dtype_of<int16_t>() { return ITKG_I16; }
template <> constexpr int dtype_of<uint8_t>() { return ITKG_U8; }
template <> constexpr int dtype_of<__nv_bfloat16>() { return ITKG_BF16; }
template <> constexpr int dtype_of<__half>() { return ITKG_F16; }

// Kernels of one radius triple and input type; the f32 cp.async gather
// variants exist only for f32 input (other types need TMA).
template <int RX, int RY, int RZ, typename Tin>
Entry make_entry() {
  using C = Cfg3<RX, RY, RZ, Tin>;
  Entry e{RX, RY, RZ, dtype_of<Tin>(), {}, {}, {}, C::SMEM, C::TX, C::TY, C::NT, C::XA, C::BW, C::IH, C::AE};
  e.fn[0][1] = k_fused3d<RX, RY, RZ, false, true, Tin>;
  e.fn[1][1] = k_fused3d<RX, RY, RZ, true, true, Tin>;
  e.multi[0][1] = k_fused3d_multi<RX, RY, RZ, false, true, Tin>;
  e.multi[1][1] = k_fused3d_multi<RX, RY, RZ, true, true, Tin>;
  if constexpr (std::is_same<Tin, float>::value) {
    e.fn[0][0] = k_fused3d<RX, RY, RZ, false, false, Tin>;
    e.fn[1][0] = k_fused3d<RX, RY, RZ, true, false, Tin>;
    e.multi[0][0] = k_fused3d_multi<RX, RY, RZ, false, false, Tin>;
    e.multi[1][0] = k_fused3d_multi<RX, RY, RZ, true, false, Tin>;
    e.vjp[0] = k_fused3d_vjp<RX, RY, RZ, kDot>;
    // the adjoint's edge-fold registers spill beyond radius 6: per-axis there
    if constexpr (RX <= 6 && RY <= 6 && RZ <= 6) e.vjp[1] = k_fused3d_vjp<RX, RY, RZ, kAdj>;
  }
  return e;
}

// The radius triples every input type is built for.
#define ITKG_FUSED_TABLE(T)                                                            \
  {make_entry<1, 1, 1, T>(), make_entry<2, 2, 2, T>(), make_entry<3, 3, 3, T>(),       \
   make_entry<4, 4, 4, T>(), make_entry<5, 5, 5, T>(), make_entry<6, 6, 6, T>(),       \
   make_entry<7, 7, 7, T>(), make_entry<8, 8, 8, T>(), make_entry<7, 7, 2, T>()}

}  // namespace fusedk

// Per input type tables (fused.cu, fused_in16.cu, fused_in8.cu).
const fusedk::Entry* fused_entries_f32(int* n);
const fusedk::Entry* fused_entries_i16(int* n);
const fusedk::Entry* fused_entries_bf16(int* n);
const fusedk::Entry* fused_entries_f16(int* n);
const fusedk::Entry* fused_entries_u8(int* n);

}  // namespace itkg
