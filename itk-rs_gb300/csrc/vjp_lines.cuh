// Tiled per-axis passes of the VJP for large radii (13 <= r <= 24, where the
// two-pass VJP kernels do not apply): the dual-number forward pass
//   (v, dv) -> (G v, G dv + G' v)           (clamp boundary, as the forward)
// and the adjoint pass
//   xbar[i] = sum_k w[k] ybar[i - r + k] (+ the folded edge taps at i = 0, n - 1)
// along one axis, with the semantics of k_dual_axis / k_adjoint_axis in vjp.cu.
//
// A CTA owns a tile of kLines lines x kLen outputs along the pass axis.  Lines
// run along x for passes along y and z (the tile's loads and stores are then
// coalesced 128-byte rows) and along y for passes along x.  The CTA stages the
// tile's kLen + 2r input positions of every line in shared memory once (clamped
// to the image for the dual pass, zero outside it for the adjoint), then each
// thread filters kRun consecutive outputs of one line, reading each of the
// kRun + 2r staged values its outputs reach once (push form, accumulators in
// registers).  Each input value is read from global memory (kLen + 2r) / kLen
// times instead of once per tap and output run.  The accumulators are packed
// pairs of adjacent outputs, so one fma.rn.f32x2 adds a staged value to two
// outputs (each lane's sum is the scalar fmaf chain's, bit for bit).
#pragma once

#include <cuda_runtime.h>

#include "f32x2.cuh"
#include "internal.hpp"

namespace itkg {
namespace vjplines {

constexpr int kMinR = 13, kMaxR = 24;
constexpr int kLines = 32;                 // lines per tile (one warp across them)
constexpr int kRun = 16;                   // outputs per thread
constexpr int kLen = 64;                   // outputs per line and tile
constexpr int kSegs = kLen / kRun;         // threads per line
constexpr int kThreads = kLines * kSegs;   // 128

struct LineTaps {
  float w[2 * kMaxR + 1];
  float aux[2 * kMaxR + 1];  // dw/dsigma (dual pass) or the prefix sums P (adjoint pass)
  // tap pairs of an output pair (j, j + 1) and the staged value j + d:
  // wp[d] = (w[d], w[d - 1]), ap[d] = (aux[d], aux[d - 1]), for 1 <= d <= 2r
  f2_t wp[2 * kMaxR + 1];
  f2_t ap[2 * kMaxR + 1];
};

// Host: fills the tap pairs from w and aux (k = 0 .. 2r).
inline void line_taps_pairs(LineTaps* T, int r) {
  for (int d = 1; d <= 2 * r; ++d) {
    T->wp[d] = pack2_host(T->w[d], T->w[d - 1]);
    T->ap[d] = pack2_host(T->aux[d], T->aux[d - 1]);
  }
}

struct LineGeom {
  int32_t n;           // image size along the pass axis
  int32_t nlines;      // image size along the lines' axis
  int32_t nother;      // image size along the third axis
  int32_t tiles_line;  // tiles along the lines' axis
  int32_t tiles_pass;  // tiles along the pass axis
  int32_t pad_;
};

template <int R, bool AX0>
struct LineCfg {
  static constexpr int K = 2 * R + 1;
  static constexpr int NP = kLen + 2 * R;  // staged positions per line
  static constexpr int WIN = kRun + 2 * R;
  // staged element (line l, position p): l * LS + p * PS (floats).  Passes
  // along y / z: one 32-float row per position, the warp's threads on
  // consecutive lines.  Passes along x: one row per line, padded to an odd
  // number of floats so the warp's threads (one line each) hit distinct banks.
  static constexpr int PP = NP | 1;
  static constexpr int LS = AX0 ? PP : 1;
  static constexpr int PS = AX0 ? 1 : kLines;
  static constexpr int ARRAY = AX0 ? kLines * PP : NP * kLines;  // floats per staged array
};

__device__ __forceinline__ int clamp_i(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Byte offset of (line l, pass position p, other o) in an image with `pitch`.
template <bool AX0>
__device__ __forceinline__ int64_t line_off(const int64_t* pitch, int axis, int64_t l, int64_t p, int64_t o) {
  if constexpr (AX0) return p * pitch[0] + l * pitch[1] + o * pitch[2];
  return axis == 1 ? l * pitch[0] + p * pitch[1] + o * pitch[2] : l * pitch[0] + o * pitch[1] + p * pitch[2];
}

// One 4-byte asynchronous copy global -> shared; with zero set, the shared
// word is filled with zeros and nothing is read.
__device__ __forceinline__ void cp4(float* dst, const void* src, bool zero) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(zero ? 0 : 4) : "memory");
}

// Stage one array's tile: positions p0 - R .. p0 + kLen + R - 1 of lines
// l0 .. l0 + kLines - 1.  CLAMP: positions clamped to [0, n) (dual pass), else
// zero outside (adjoint); lines beyond the image read zero.  `base` points at
// the tile's (line 0, position 0, other o); lp / pp: byte pitches of the lines'
// axis and of the pass axis.  Asynchronous copies: the caller waits
// (cp.async.wait_all) and synchronises the block before reading.
template <int R, bool AX0, bool CLAMP>
__device__ __forceinline__ void stage_tile(float* s, const char* base, int64_t lp, int64_t pp, const LineGeom& g,
                                           int l0, int p0) {
  using C = LineCfg<R, AX0>;
  // positions p0 - R .. p0 + kLen + R - 1 all inside the image: no clamping
  const bool interior = p0 - R >= 0 && p0 + kLen + R <= g.n;
  if constexpr (AX0) {
    // thread pi stages position pi of every line (consecutive threads on
    // consecutive x): its position, clamp and in-image test are fixed, and
    // its source steps by one line pitch
    static_assert(C::NP <= kThreads, "one position per thread and line");
    const int pi = threadIdx.x;
    if (pi < C::NP) {
      int p = p0 - R + pi;
      bool pin = true;
      if (!interior) {
        if (CLAMP) p = clamp_i(p, 0, g.n - 1);
        pin = p >= 0 && p < g.n;
      }
      const int nl = min(kLines, g.nlines - l0);  // lines of the tile inside the image (>= 1)
      const char* src = base + (int64_t)(pin ? p : 0) * pp + (int64_t)l0 * lp;
      float* dst = s + pi;
#pragma unroll 4
      for (int li = 0; li < kLines; ++li, src += lp, dst += C::PP) {
        const bool in = pin && li < nl;
        cp4(dst, in ? src : base, !in);
      }
    }
  } else {
    // this thread's line is fixed (kThreads is a multiple of kLines); its
    // positions step by kThreads / kLines
    constexpr int STEP = kThreads / kLines;
    const int li = threadIdx.x % kLines;
    const int l = l0 + li;
    const bool lin = l < g.nlines;
    const char* const col = base + (int64_t)(lin ? l : 0) * lp;
    const int pi0 = threadIdx.x / kLines;
    if (interior && lin) {
      const char* q = col + (int64_t)(p0 - R + pi0) * pp;
      const int64_t dq = (int64_t)STEP * pp;
#pragma unroll 4
      for (int pi = pi0; pi < C::NP; pi += STEP, q += dq) cp4(s + pi * kLines + li, q, false);
    } else {
#pragma unroll 4
      for (int pi = pi0; pi < C::NP; pi += STEP) {
        int p = p0 - R + pi;
        if (CLAMP) p = clamp_i(p, 0, g.n - 1);
        const bool in = lin && p >= 0 && p < g.n;
        cp4(s + pi * kLines + li, in ? col + (int64_t)p * pp : base, !in);
      }
    }
  }
}

__device__ __forceinline__ void stage_wait() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();
}

// Byte pitches of the lines' and the pass axes, and the offset of other o.
template <bool AX0>
__device__ __forceinline__ void tile_pitches(const int64_t* pitch, int axis, int o, int64_t* lp, int64_t* pp,
                                             int64_t* oo) {
  if constexpr (AX0) {
    *lp = pitch[1], *pp = pitch[0], *oo = (int64_t)o * pitch[2];
  } else {
    // (selects, not pitch[axis]: a runtime index into the kernel parameters
    // would copy them to local memory)
    *lp = pitch[0];
    *pp = axis == 1 ? pitch[1] : pitch[2];
    *oo = (int64_t)o * (axis == 1 ? pitch[2] : pitch[1]);
  }
}

// Push-form filtering of one line's window: staged value q (positions
// p0 + seg kRun - R + q) is read from shared memory once and added, times the
// tap weight, to every output j of the thread's run that it reaches (tap
// k = q - j), so each output still sums its taps in ascending order.  acc[h]
// packs outputs 2h and 2h + 1: where both taps exist (1 <= q - 2h <= 2R) one
// packed fma adds the value to both, at q - 2h = 0 (2R + 1) only the first
// (second) output takes it.  W2 adds T.aux's taps into acc2 the same way (the
// dual pass's G' of the same values).
template <int R, bool AX0, bool W2>
__device__ __forceinline__ void filter_run(const float* s, int li, int seg, const LineTaps& T,
                                           f2_t (&acc)[kRun / 2], f2_t (&acc2)[kRun / 2]) {
  using C = LineCfg<R, AX0>;
  constexpr int K = C::K;
  const float* const p = s + li * C::LS + seg * kRun * C::PS;
#pragma unroll
  for (int q = 0; q < C::WIN; ++q) {
    const float x = p[q * C::PS];
    const f2_t xx = pack2(x, x);
#pragma unroll
    for (int h = 0; h < kRun / 2; ++h) {
      const int d = q - 2 * h;  // output 2h takes tap d, output 2h + 1 tap d - 1
      if (d >= 1 && d < K) {
        acc[h] = fma2(xx, T.wp[d], acc[h]);
        if constexpr (W2) acc2[h] = fma2(xx, T.ap[d], acc2[h]);
      } else if (d == 0 || d == K) {
        float lo, hi;
        unpack2(acc[h], lo, hi);
        if (d == 0) lo = fmaf(T.w[0], x, lo);
        else hi = fmaf(T.w[K - 1], x, hi);
        acc[h] = pack2(lo, hi);
        if constexpr (W2) {
          unpack2(acc2[h], lo, hi);
          if (d == 0) lo = fmaf(T.aux[0], x, lo);
          else hi = fmaf(T.aux[K - 1], x, hi);
          acc2[h] = pack2(lo, hi);
        }
      }
    }
  }
}

// The run's outputs as scalars.
__device__ __forceinline__ void unpack_run(const f2_t (&a)[kRun / 2], float (&v)[kRun]) {
#pragma unroll
  for (int h = 0; h < kRun / 2; ++h) unpack2(a[h], v[2 * h], v[2 * h + 1]);
}

// Tile index -> (first line, first pass position, other).
__device__ __forceinline__ void tile_of(const LineGeom& g, int64_t t, int* l0, int* p0, int* o) {
  const int64_t per_o = (int64_t)g.tiles_line * g.tiles_pass;
  *o = (int)(t / per_o);
  const int64_t r = t - (int64_t)(*o) * per_o;
  *p0 = (int)(r / g.tiles_line) * kLen;
  *l0 = (int)(r % g.tiles_line) * kLines;
}

// Passes along x write their results through shared memory (one row of kLen
// outputs per line, padded to an odd stride), so that the global stores and
// the accumulating loads run along x; passes along y and z store directly
// (the warp's threads are consecutive x).
constexpr int kOutPitch = kLen + 1;

// Writes (or, with ACC, adds) this thread's run to `out`, and with dout its
// second run.  `s` is a free shared buffer of 2 kLines kOutPitch floats (AX0).
template <bool AX0>
__device__ __forceinline__ void store_runs(const VjpAxisArgs& a, const LineGeom& g, float* s, int l0, int p0,
                                           int o, int li, int seg, const float (&v)[kRun],
                                           const float (&dv)[kRun], bool two, bool acc) {
  char* const ob = reinterpret_cast<char*>(a.out);
  char* const db = reinterpret_cast<char*>(a.dout);
  if constexpr (AX0) {
#pragma unroll
    for (int j = 0; j < kRun; ++j) {
      s[li * kOutPitch + seg * kRun + j] = v[j];
      if (two) s[(kLines + li) * kOutPitch + seg * kRun + j] = dv[j];
    }
    __syncthreads();
    // thread t writes position t % kLen of lines t / kLen, + kThreads / kLen, ...
    static_assert(kThreads % kLen == 0, "whole rows per step");
    constexpr int LSTEP = kThreads / kLen;
    const int pj = threadIdx.x % kLen;
    const int p = p0 + pj;
    if (p < g.n) {
      const int nl = min(kLines, g.nlines - l0);  // lines of the tile inside the image
      int lj = threadIdx.x / kLen;
      int64_t off = line_off<true>(a.out_pitch, 0, l0 + lj, p, o);
      const int64_t step = (int64_t)LSTEP * a.out_pitch[1];
      for (; lj < nl; lj += LSTEP, off += step) {
        float* const po = reinterpret_cast<float*>(ob + off);
        const float r = s[lj * kOutPitch + pj];
        *po = acc ? *po + r : r;
        if (two) *reinterpret_cast<float*>(db + off) = s[(kLines + lj) * kOutPitch + pj];
      }
    }
  } else {
    const int l = l0 + li;
    if (l >= g.nlines) return;
    int64_t lp, pp, oo;
    tile_pitches<false>(a.out_pitch, a.axis, o, &lp, &pp, &oo);
    char* const ol = ob + (int64_t)l * lp + oo;
    char* const dl = db + (ol - ob);
#pragma unroll
    for (int j = 0; j < kRun; ++j) {
      const int p = p0 + seg * kRun + j;
      if (p >= g.n) continue;
      const int64_t off = (int64_t)p * pp;
      float* const po = reinterpret_cast<float*>(ol + off);
      *po = acc ? *po + v[j] : v[j];
      if (two) *reinterpret_cast<float*>(dl + off) = dv[j];
    }
  }
}

// The dual pass: out = G in, dout = G din + G' in (din may be NULL).
template <int R, bool AX0>
__global__ void __launch_bounds__(kThreads) k_line_dual(const VjpAxisArgs a, const LineTaps T, const LineGeom g) {
  using C = LineCfg<R, AX0>;
  extern __shared__ float smem[];
  float* const sx = smem;
  float* const sd = smem + C::ARRAY;
  int l0, p0, o;
  tile_of(g, blockIdx.x, &l0, &p0, &o);
  const bool has_d = a.din != nullptr;
  int64_t lp, pp, oo;
  tile_pitches<AX0>(a.in_pitch, a.axis, o, &lp, &pp, &oo);
  stage_tile<R, AX0, true>(sx, reinterpret_cast<const char*>(a.in) + oo, lp, pp, g, l0, p0);
  if (has_d) stage_tile<R, AX0, true>(sd, reinterpret_cast<const char*>(a.din) + oo, lp, pp, g, l0, p0);
  stage_wait();
  const int li = threadIdx.x % kLines, seg = threadIdx.x / kLines;
  f2_t v2[kRun / 2], d2[kRun / 2];
#pragma unroll
  for (int h = 0; h < kRun / 2; ++h) v2[h] = 0ull, d2[h] = 0ull;
  filter_run<R, AX0, true>(sx, li, seg, T, v2, d2);
  if (has_d) filter_run<R, AX0, false>(sd, li, seg, T, d2, d2);
  float v[kRun], dv[kRun];
  unpack_run(v2, v);
  unpack_run(d2, dv);
  if constexpr (AX0) __syncthreads();  // the staged input is free for the output rows
  store_runs<AX0>(a, g, smem, l0, p0, o, li, seg, v, dv, true, false);
}

// The adjoint pass: out (+)= G^T in, with the taps the forward clamped onto
// the edge voxels folded back at positions 0 and n - 1.
template <int R, bool AX0>
__global__ void __launch_bounds__(kThreads) k_line_adjoint(const VjpAxisArgs a, const LineTaps T, const LineGeom g) {
  using C = LineCfg<R, AX0>;
  extern __shared__ float smem[];
  int l0, p0, o;
  tile_of(g, blockIdx.x, &l0, &p0, &o);
  int64_t lp, pp, oo;
  tile_pitches<AX0>(a.in_pitch, a.axis, o, &lp, &pp, &oo);
  stage_tile<R, AX0, false>(smem, reinterpret_cast<const char*>(a.in) + oo, lp, pp, g, l0, p0);
  stage_wait();
  const int li = threadIdx.x % kLines, seg = threadIdx.x / kLines;
  f2_t a2[kRun / 2];
#pragma unroll
  for (int h = 0; h < kRun / 2; ++h) a2[h] = 0ull;
  filter_run<R, AX0, false>(smem, li, seg, T, a2, a2);
  float acc[kRun];
  unpack_run(a2, acc);
  // the edge folds (rare: only the tiles holding position 0 or n - 1)
  if (l0 + li < g.nlines && (p0 == 0 || p0 + kLen >= g.n)) {
    const float* const sl = smem + li * C::LS;
    auto at = [&](int q) { return sl[(q - (p0 - R)) * C::PS]; };
#pragma unroll
    for (int j = 0; j < kRun; ++j) {
      const int p = p0 + seg * kRun + j;
      if (p == 0)
        for (int d = 0; d < R && d < g.n; ++d) acc[j] = fmaf(T.aux[R - 1 - d], at(d), acc[j]);
      if (p == g.n - 1)
        for (int d = 0; d < R && d < g.n; ++d) acc[j] = fmaf(T.aux[R - 1 - d], at(g.n - 1 - d), acc[j]);
    }
  }
  if constexpr (AX0) __syncthreads();
  store_runs<AX0>(a, g, smem, l0, p0, o, li, seg, acc, acc, false, a.accumulate != 0);
}

// Host: the tile grid of a pass.  False when the image does not fit the int32
// tile arithmetic.
inline bool line_geom(const VjpAxisArgs& a, LineGeom* g, int64_t* ntiles) {
  const int axis = a.axis;
  const int laxis = axis == 0 ? 1 : 0;
  const int oaxis = 3 - axis - laxis;
  const int64_t n = a.size[axis], nl = a.size[laxis], no = a.size[oaxis];
  if (n < 1 || nl < 1 || no < 1 || n > INT32_MAX / 2 || nl > INT32_MAX / 2 || no > INT32_MAX) return false;
  g->n = (int32_t)n;
  g->nlines = (int32_t)nl;
  g->nother = (int32_t)no;
  g->tiles_line = (int32_t)((nl + kLines - 1) / kLines);
  g->tiles_pass = (int32_t)((n + kLen - 1) / kLen);
  g->pad_ = 0;
  *ntiles = (int64_t)g->tiles_line * g->tiles_pass * no;
  return *ntiles <= INT32_MAX;
}

}  // namespace vjplines
}  // namespace itkg
