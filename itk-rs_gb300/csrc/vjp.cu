// Vector-Jacobian product of the Gaussian (not in the reference, which has no
// derivative): per-axis adjoint and dual-number passes, and the f64 reductions.
//
// Forward along one axis (conv.rs:11-41, whole image [0, n)):
//   y[o] = sum_k w[k] x[clamp(o + k - r, 0, n - 1)]
// Adjoint:  xbar[i] = sum_{o,k : clamp(o+k-r) = i} w[k] ybar[o].  Because the
// f32 weights are exactly symmetric (w[k] = w[2r-k], gaussian.rs:31-35 squares
// the offset), this is
//   xbar[i] = sum_k w[k] ybar[i - r + k]          (ybar zero outside [0, n))
//           + [i == 0]   sum_{d<r} ybar[d] P[r-1-d]
//           + [i == n-1] sum_{d<r} ybar[n-1-d] P[r-1-d]
// with P[m] = w[0] + ... + w[m]: the two end terms fold back the taps the
// forward clamped onto the edge voxels.
// sigma derivative: forward-mode dual numbers through the passes,
//   (v, dv) -> (G v, G dv + G' v),   G' = d/dsigma of the pass (same radius),
// so after the last pass dv = dy/dsigma and dL/dsigma = <ybar, dv>.
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.hpp"
#include "pixel.cuh"

namespace itkg {
namespace {

constexpr int kThreads = 256;

struct Taps {
  float w[kMaxVjpTaps];
  float aux[kMaxVjpTaps];  // dw/dsigma (dual pass) or prefix sums P (adjoint pass)
};

// v[i] for a runtime i by selects: indexing a kernel parameter's array with a
// runtime index would copy the parameters to local memory.
__host__ __device__ __forceinline__ int64_t pick3(const int64_t (&v)[kMaxDim], int i) {
  return i == 0 ? v[0] : (i == 1 ? v[1] : v[2]);
}

__device__ __forceinline__ const char* px(const void* base, const int64_t* pitch, int64_t x,
                                          int64_t y, int64_t z) {
  return static_cast<const char*>(base) + x * pitch[0] + y * pitch[1] + z * pitch[2];
}

// One adjoint pass along `axis` over the whole image (accumulate: out += result).
__global__ void __launch_bounds__(kThreads) k_adjoint_axis(const VjpAxisArgs a, const Taps T) {
  const int64_t t = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (t >= a.size[0]) return;
  const int64_t nrows = a.size[1] * a.size[2];
  const int r = a.radius, K = 2 * r + 1;
  const int axis = a.axis;
  const int64_t n = pick3(a.size, axis);
  const int64_t ap = pick3(a.in_pitch, axis);
  for (int64_t row = blockIdx.y; row < nrows; row += gridDim.y) {
    const int64_t y = row % a.size[1], z = row / a.size[1];
    const int64_t i = axis == 0 ? t : (axis == 1 ? y : z);
    const char* base = px(a.in, a.in_pitch, axis == 0 ? 0 : t, axis == 1 ? 0 : y, axis == 2 ? 0 : z);
    float acc = 0.0f;
    for (int k = 0; k < K; ++k) {
      const int64_t s = i - r + k;
      if (s >= 0 && s < n) acc = fmaf(T.w[k], *reinterpret_cast<const float*>(base + s * ap), acc);
    }
    if (i == 0)
      for (int d = 0; d < r && d < n; ++d)
        acc = fmaf(T.aux[r - 1 - d], *reinterpret_cast<const float*>(base + d * ap), acc);
    if (i == n - 1)
      for (int d = 0; d < r && d < n; ++d)
        acc = fmaf(T.aux[r - 1 - d], *reinterpret_cast<const float*>(base + (n - 1 - d) * ap), acc);
    float* o = reinterpret_cast<float*>(const_cast<char*>(px(a.out, a.out_pitch, t, y, z)));
    *o = a.accumulate ? *o + acc : acc;
  }
}

// One dual pass: (v, dv) -> (G v, G dv + G' v) along `axis` (clamp boundary).
__global__ void __launch_bounds__(kThreads) k_dual_axis(const VjpAxisArgs a, const Taps T) {
  const int64_t t = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (t >= a.size[0]) return;
  const int64_t nrows = a.size[1] * a.size[2];
  const int r = a.radius, K = 2 * r + 1;
  const int axis = a.axis;
  const int64_t n = pick3(a.size, axis);
  const int64_t ap = pick3(a.in_pitch, axis);
  for (int64_t row = blockIdx.y; row < nrows; row += gridDim.y) {
    const int64_t y = row % a.size[1], z = row / a.size[1];
    const int64_t i = axis == 0 ? t : (axis == 1 ? y : z);
    const int64_t bx = axis == 0 ? 0 : t, by = axis == 1 ? 0 : y, bz = axis == 2 ? 0 : z;
    const char* vb = px(a.in, a.in_pitch, bx, by, bz);
    const char* db = a.din ? px(a.din, a.in_pitch, bx, by, bz) : nullptr;
    float v = 0.0f, dv = 0.0f;
    for (int k = 0; k < K; ++k) {
      int64_t s = i + k - r;
      s = s < 0 ? 0 : (s >= n ? n - 1 : s);
      const float xv = *reinterpret_cast<const float*>(vb + s * ap);
      v = fmaf(T.w[k], xv, v);
      dv = fmaf(T.aux[k], xv, dv);
      if (db) dv = fmaf(T.w[k], *reinterpret_cast<const float*>(db + s * ap), dv);
    }
    *reinterpret_cast<float*>(const_cast<char*>(px(a.out, a.out_pitch, t, y, z))) = v;
    *reinterpret_cast<float*>(const_cast<char*>(px(a.dout, a.out_pitch, t, y, z))) = dv;
  }
}

// The same two passes with the radius a template parameter (R <= 12: taps
// unrolled, weights read from the parameter bank; radii 13 .. 24 take the tiled
// passes of vjp_lines.cuh) and RUN outputs per thread
// along a marching axis -- y for passes along x and y, z for passes along z.
// Along y and z the RUN outputs share one register window of K + RUN - 1
// loads; along x the taps' offsets (and, for the adjoint, which taps fall
// inside the image) are computed once per thread.
constexpr int kMaxSmallVjpR = 12;

template <int R, int RUN, bool AX0>
__global__ void __launch_bounds__(kThreads, 2) k_adjoint_small(const VjpAxisArgs a, const Taps T) {
  constexpr int K = 2 * R + 1;
  const int64_t x = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (x >= a.size[0]) return;
  const int axis = AX0 ? 0 : a.axis;
  const int md = axis == 2 ? 2 : 1, od = axis == 2 ? 1 : 2;
  const int64_t n = pick3(a.size, axis), mn = pick3(a.size, md), on = pick3(a.size, od);
  const int64_t ap = pick3(a.in_pitch, axis);
  const char* const ix = reinterpret_cast<const char*>(a.in) + x * a.in_pitch[0];
  char* const ox = reinterpret_cast<char*>(a.out) + x * a.out_pitch[0];
  for (int64_t o = blockIdx.z; o < on; o += gridDim.z) {
    const char* const io = ix + o * pick3(a.in_pitch, od);
    char* const oo = ox + o * pick3(a.out_pitch, od);
    for (int64_t mb = (int64_t)blockIdx.y * RUN; mb < mn; mb += (int64_t)gridDim.y * RUN) {
      const int nv = (int)(mn - mb < RUN ? mn - mb : RUN);
      float acc[RUN];
      if constexpr (AX0) {
        // taps along x: offset and whether the tap lies in [0, n), shared by the RUN rows
        const char* rows[RUN];
#pragma unroll
        for (int r = 0; r < RUN; ++r) {
          acc[r] = 0.0f;
          rows[r] = io + (mb + (r < nv ? r : 0)) * pick3(a.in_pitch, md);
        }
#pragma unroll
        for (int k = 0; k < K; ++k) {
          const int64_t sx = x - R + k;
          if (sx >= 0 && sx < n) {
            const int64_t off = (sx - x) * ap;
#pragma unroll
            for (int r = 0; r < RUN; ++r)
              acc[r] = fmaf(T.w[k], __ldg(reinterpret_cast<const float*>(rows[r] + off)), acc[r]);
          }
        }
      } else {
        float v[K + RUN - 1];  // ybar at mb - R .. mb + RUN - 1 + R, zero outside the image
#pragma unroll
        for (int j = 0; j < K + RUN - 1; ++j) {
          const int64_t s = mb - R + j;
          v[j] = (s >= 0 && s < n) ? __ldg(reinterpret_cast<const float*>(io + s * ap)) : 0.0f;
        }
#pragma unroll
        for (int r = 0; r < RUN; ++r) {
          acc[r] = 0.0f;
#pragma unroll
          for (int k = 0; k < K; ++k) acc[r] = fmaf(T.w[k], v[r + k], acc[r]);
        }
      }
#pragma unroll
      for (int r = 0; r < RUN; ++r) {
        if (r >= nv) break;
        const int64_t m = mb + r;
        const int64_t i = AX0 ? x : m;  // position along the pass axis
        float res = acc[r];
        if (i == 0 || i == n - 1) {  // the taps the forward clamped onto the edge voxels
          const char* const line = AX0 ? io + m * pick3(a.in_pitch, md) - x * ap : io;
          if (i == 0)
            for (int d = 0; d < R && d < n; ++d)
              res = fmaf(T.aux[R - 1 - d], *reinterpret_cast<const float*>(line + d * ap), res);
          if (i == n - 1)
            for (int d = 0; d < R && d < n; ++d)
              res = fmaf(T.aux[R - 1 - d], *reinterpret_cast<const float*>(line + (n - 1 - d) * ap), res);
        }
        float* const po = reinterpret_cast<float*>(oo + m * pick3(a.out_pitch, md));
        *po = a.accumulate ? *po + res : res;
      }
    }
  }
}

template <int R, int RUN, bool AX0>
__global__ void __launch_bounds__(kThreads, 2) k_dual_small(const VjpAxisArgs a, const Taps T) {
  constexpr int K = 2 * R + 1;
  const int64_t x = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (x >= a.size[0]) return;
  const int axis = AX0 ? 0 : a.axis;
  const int md = axis == 2 ? 2 : 1, od = axis == 2 ? 1 : 2;
  const int64_t n = pick3(a.size, axis), mn = pick3(a.size, md), on = pick3(a.size, od);
  const int64_t ap = pick3(a.in_pitch, axis);
  const bool has_d = a.din != nullptr;
  const int64_t dbase = has_d ? reinterpret_cast<const char*>(a.din) - reinterpret_cast<const char*>(a.in) : 0;
  const char* const ix = reinterpret_cast<const char*>(a.in) + x * a.in_pitch[0];
  const int64_t oxo = x * a.out_pitch[0];
  for (int64_t o = blockIdx.z; o < on; o += gridDim.z) {
    const char* const io = ix + o * pick3(a.in_pitch, od);
    const int64_t oo = oxo + o * pick3(a.out_pitch, od);
    for (int64_t mb = (int64_t)blockIdx.y * RUN; mb < mn; mb += (int64_t)gridDim.y * RUN) {
      const int nv = (int)(mn - mb < RUN ? mn - mb : RUN);
      float v[RUN], dv[RUN];
      if constexpr (AX0) {
        // clamped taps along x, shared by the RUN rows
        const char* rows[RUN];
#pragma unroll
        for (int r = 0; r < RUN; ++r) {
          v[r] = 0.0f;
          dv[r] = 0.0f;
          rows[r] = io + (mb + (r < nv ? r : 0)) * pick3(a.in_pitch, md);
        }
#pragma unroll
        for (int k = 0; k < K; ++k) {
          int64_t sx = x + k - R;
          sx = sx < 0 ? 0 : (sx >= n ? n - 1 : sx);
          const int64_t off = (sx - x) * ap;
#pragma unroll
          for (int r = 0; r < RUN; ++r) {
            const float xv = __ldg(reinterpret_cast<const float*>(rows[r] + off));
            v[r] = fmaf(T.w[k], xv, v[r]);
            dv[r] = fmaf(T.aux[k], xv, dv[r]);
            if (has_d) dv[r] = fmaf(T.w[k], __ldg(reinterpret_cast<const float*>(rows[r] + dbase + off)), dv[r]);
          }
        }
      } else {
        // positions mb - R .. mb + RUN - 1 + R clamped to [0, n - 1] and, beyond the
        // last valid output's taps, to its last tap
        const int64_t top = mb + nv - 1 + R < n - 1 ? mb + nv - 1 + R : n - 1;
        float w[K + RUN - 1], dw[K + RUN - 1];
#pragma unroll
        for (int j = 0; j < K + RUN - 1; ++j) {
          int64_t s = mb - R + j;
          s = s < 0 ? 0 : (s > top ? top : s);
          w[j] = __ldg(reinterpret_cast<const float*>(io + s * ap));
          dw[j] = has_d ? __ldg(reinterpret_cast<const float*>(io + dbase + s * ap)) : 0.0f;
        }
#pragma unroll
        for (int r = 0; r < RUN; ++r) {
          v[r] = 0.0f;
          dv[r] = 0.0f;
#pragma unroll
          for (int k = 0; k < K; ++k) {
            v[r] = fmaf(T.w[k], w[r + k], v[r]);
            dv[r] = fmaf(T.aux[k], w[r + k], dv[r]);
            if (has_d) dv[r] = fmaf(T.w[k], dw[r + k], dv[r]);
          }
        }
      }
#pragma unroll
      for (int r = 0; r < RUN; ++r) {
        if (r >= nv) break;
        const int64_t off = oo + (mb + r) * pick3(a.out_pitch, md);
        *reinterpret_cast<float*>(reinterpret_cast<char*>(a.out) + off) = v[r];
        *reinterpret_cast<float*>(reinterpret_cast<char*>(a.dout) + off) = dv[r];
      }
    }
  }
}

using VjpFn = void (*)(const VjpAxisArgs, const Taps);
constexpr int kAdjRun = 4, kDualRun = 2;
struct VjpPair {
  VjpFn ax0, ax12;  // passes along x; along y or z
};
template <int R>
constexpr VjpPair adj_fn() { return {k_adjoint_small<R, kAdjRun, true>, k_adjoint_small<R, kAdjRun, false>}; }
template <int R>
constexpr VjpPair dual_fn() { return {k_dual_small<R, kDualRun, true>, k_dual_small<R, kDualRun, false>}; }
#define ITKG_VJP_TABLE(F) \
  {{nullptr, nullptr}, F<1>(), F<2>(), F<3>(), F<4>(), F<5>(), F<6>(), F<7>(), F<8>(), F<9>(), F<10>(), F<11>(), F<12>()}
const VjpPair kAdjSmall[kMaxSmallVjpR + 1] = ITKG_VJP_TABLE(adj_fn);
const VjpPair kDualSmall[kMaxSmallVjpR + 1] = ITKG_VJP_TABLE(dual_fn);
#undef ITKG_VJP_TABLE

dim3 grid_small(const VjpAxisArgs& a, int run) {
  const int md = a.axis == 2 ? 2 : 1, od = a.axis == 2 ? 1 : 2;
  const int64_t gx = (a.size[0] + kThreads - 1) / kThreads;
  const int64_t gy = (pick3(a.size, md) + run - 1) / run;
  return dim3((unsigned)gx, (unsigned)(gy < 65535 ? gy : 65535), (unsigned)(pick3(a.size, od) < 65535 ? pick3(a.size, od) : 65535));
}

// Per-block f64 partial sums of sum(p * q) over a pitched image: each thread
// sums its products in f32 runs of 16 and folds each run into f64 (an f64
// operation per element would hold this GPU's slow FP64 pipe for longer than
// the loads take).
__global__ void __launch_bounds__(kThreads) k_dot_partials(const DotArgs d, double* partials) {
  const int64_t nx = d.size[0], nxy = d.size[0] * d.size[1];
  const int64_t n = nxy * d.size[2];
  double s = 0.0;
  float f = 0.0f;
  int run = 0;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads) {
    const int64_t x = i % nx, y = (i / nx) % d.size[1], z = i / nxy;
    const float a = *reinterpret_cast<const float*>(px(d.p, d.p_pitch, x, y, z));
    const float b = *reinterpret_cast<const float*>(px(d.q, d.q_pitch, x, y, z));
    f = fmaf(a, b, f);
    if (++run == 16) {
      s += (double)f;
      f = 0.0f;
      run = 0;
    }
  }
  s += (double)f;
  __shared__ double red[kThreads];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

// Squared-error loss against a target t, per voxel: d = y - t,
// ybar = 2 d (written densely), and per-block f64 partials of sum d^2 and of
// sum ybar * dy (the sigma gradient).  partials: [nblocks] loss, [nblocks] sigma.
// Block b takes a contiguous run of the image's rows (x lines); a thread sums
// its voxels' products in f32 for up to 8 rows at a time and folds them into
// f64 (f64 arithmetic on this GPU is scarce; the f32 runs keep each partial's
// relative error near 1e-7).
__global__ void __launch_bounds__(kThreads) k_sqerr(const float* __restrict__ y,
                                                     const float* __restrict__ dy, const DotArgs t,
                                                     float* __restrict__ ybar, double* partials) {
  const int64_t nx = t.size[0], ny = t.size[1];
  const int64_t rows = ny * t.size[2];
  const int64_t r0 = rows * blockIdx.x / gridDim.x, r1 = rows * (blockIdx.x + 1) / gridDim.x;
  double sl = 0.0, ss = 0.0;
  float fl = 0.0f, fs = 0.0f;
  int run = 0;
  for (int64_t row = r0; row < r1; ++row) {
    const int64_t yy = row % ny, z = row / ny;
    const char* const trow = reinterpret_cast<const char*>(t.q) + yy * t.q_pitch[1] + z * t.q_pitch[2];
    const int64_t base = row * nx;
    for (int64_t x = threadIdx.x; x < nx; x += kThreads) {
      const float tv = *reinterpret_cast<const float*>(trow + x * t.q_pitch[0]);
      const float d = y[base + x] - tv;
      const float g = 2.0f * d;
      ybar[base + x] = g;
      fl = fmaf(d, d, fl);
      if (dy) fs = fmaf(g, dy[base + x], fs);
    }
    if (++run == 8) {
      sl += (double)fl;
      ss += (double)fs;
      fl = fs = 0.0f;
      run = 0;
    }
  }
  sl += (double)fl;
  ss += (double)fs;
  __shared__ double red[2][kThreads];
  red[0][threadIdx.x] = sl;
  red[1][threadIdx.x] = ss;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      red[0][threadIdx.x] += red[0][threadIdx.x + w];
      red[1][threadIdx.x] += red[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = red[0][0];
    partials[gridDim.x + blockIdx.x] = red[1][0];
  }
}

// The same over dense images whose rows are whole quads (the target too): a
// grid-stride loop over the volume's quads, four quads per thread in flight,
// the f32 runs folded into f64 every 8 quads.  A fixed grid makes the partials
// deterministic.
__global__ void __launch_bounds__(kThreads) k_sqerr_q(const float4* __restrict__ y, const float4* __restrict__ dy,
                                                        const float4* __restrict__ t, float4* __restrict__ ybar,
                                                        int64_t nq, double* partials) {
  constexpr int U = 4;
  double sl = 0.0, ss = 0.0;
  const int64_t stride = (int64_t)gridDim.x * kThreads;
  for (int64_t i0 = (int64_t)blockIdx.x * kThreads + threadIdx.x; i0 < nq; i0 += U * stride) {
    float4 yv[U], tv[U], dv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = i0 + u * stride;
      if (i < nq) {
        yv[u] = __ldcs(y + i);
        tv[u] = __ldg(t + i);
        dv[u] = dy ? __ldcs(dy + i) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
    }
    float fl = 0.0f, fs = 0.0f;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = i0 + u * stride;
      if (i >= nq) break;
      const float4 d = make_float4(yv[u].x - tv[u].x, yv[u].y - tv[u].y, yv[u].z - tv[u].z, yv[u].w - tv[u].w);
      const float4 g = make_float4(2.0f * d.x, 2.0f * d.y, 2.0f * d.z, 2.0f * d.w);
      __stcs(ybar + i, g);
      fl = fmaf(d.x, d.x, fl);
      fl = fmaf(d.y, d.y, fl);
      fl = fmaf(d.z, d.z, fl);
      fl = fmaf(d.w, d.w, fl);
      fs = fmaf(g.x, dv[u].x, fs);
      fs = fmaf(g.y, dv[u].y, fs);
      fs = fmaf(g.z, dv[u].z, fs);
      fs = fmaf(g.w, dv[u].w, fs);
    }
    sl += (double)fl;
    ss += (double)fs;
  }
  __shared__ double red[2][kThreads];
  red[0][threadIdx.x] = sl;
  red[1][threadIdx.x] = ss;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      red[0][threadIdx.x] += red[0][threadIdx.x + w];
      red[1][threadIdx.x] += red[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = red[0][0];
    partials[gridDim.x + blockIdx.x] = red[1][0];
  }
}

// Fixed-order final sum of the partials (deterministic).
__global__ void k_sum_partials(const double* partials, int n, double* out, int accumulate) {
  __shared__ double red[kThreads];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += kThreads) s += partials[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = accumulate ? *out + red[0] : red[0];
}

dim3 grid_for(const VjpAxisArgs& a) {
  const int64_t gx = (a.size[0] + kThreads - 1) / kThreads;
  const int64_t rows = a.size[1] * a.size[2];
  return dim3((unsigned)gx, (unsigned)(rows < 65535 ? rows : 65535), 1);
}

Taps make_taps(const float* w, const float* second, int K) {
  Taps T;
  for (int k = 0; k < kMaxVjpTaps; ++k) {
    T.w[k] = k < K ? w[k] : 0.0f;
    T.aux[k] = k < K ? second[k] : 0.0f;
  }
  return T;
}

itkg_status launched(const char* name) {
  note_launch(name);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "%s launch: %s", name, cudaGetErrorString(e));
  return ITKG_SUCCESS;
}

}  // namespace

itkg_status launch_adjoint_axis(const VjpAxisArgs& a, const float* w, const float* prefix,
                                void* stream) {
  if (2 * a.radius + 1 > kMaxVjpTaps)
    return set_error(ITKG_ERROR_UNSUPPORTED, "VJP radius %d exceeds %d", a.radius, (kMaxVjpTaps - 1) / 2);
  {
    const itkg_status st = launch_line_adjoint(a, w, prefix, stream);
    if (st != ITKG_ERROR_UNSUPPORTED) return st;
  }
  const Taps T = make_taps(w, prefix, 2 * a.radius + 1);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (a.radius >= 1 && a.radius <= kMaxSmallVjpR && a.size[0] <= INT32_MAX) {
    const VjpFn fn = a.axis == 0 ? kAdjSmall[a.radius].ax0 : kAdjSmall[a.radius].ax12;
    fn<<<grid_small(a, kAdjRun), kThreads, 0, s>>>(a, T);
    return launched("adjoint_axis_f32");
  }
  k_adjoint_axis<<<grid_for(a), kThreads, 0, s>>>(a, T);
  return launched("adjoint_axis_f32");
}

itkg_status launch_dual_axis(const VjpAxisArgs& a, const float* w, const float* dw, void* stream) {
  if (2 * a.radius + 1 > kMaxVjpTaps)
    return set_error(ITKG_ERROR_UNSUPPORTED, "VJP radius %d exceeds %d", a.radius, (kMaxVjpTaps - 1) / 2);
  {
    const itkg_status st = launch_line_dual(a, w, dw, stream);
    if (st != ITKG_ERROR_UNSUPPORTED) return st;
  }
  const Taps T = make_taps(w, dw, 2 * a.radius + 1);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (a.radius >= 1 && a.radius <= kMaxSmallVjpR && a.size[0] <= INT32_MAX) {
    const VjpFn fn = a.axis == 0 ? kDualSmall[a.radius].ax0 : kDualSmall[a.radius].ax12;
    fn<<<grid_small(a, kDualRun), kThreads, 0, s>>>(a, T);
    return launched("dual_axis_f32");
  }
  k_dual_axis<<<grid_for(a), kThreads, 0, s>>>(a, T);
  return launched("dual_axis_f32");
}

int dot_partial_blocks(int64_t n) {
  const int64_t b = (n + kThreads * 8 - 1) / (kThreads * 8);
  return (int)(b < 1 ? 1 : (b > 2048 ? 2048 : b));
}

itkg_status launch_sqerr(const float* y, const float* dy, const DotArgs& t, float* ybar,
                         double* partials, int nblocks, double* loss_out, double* sigma_out,
                         bool accumulate_loss, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t nx = t.size[0], ny = t.size[1];
  const bool quads = nx % 4 == 0 && t.q_pitch[0] == 4 && t.q_pitch[1] == 4 * nx && t.q_pitch[2] == 4 * nx * ny &&
                     (((uintptr_t)y | (uintptr_t)dy | (uintptr_t)t.q | (uintptr_t)ybar) & 15) == 0;
  // the quad kernel: about 16 quads per thread (fewer, longer-running blocks)
  const int64_t nq = nx / 4 * ny * t.size[2];
  const int nb = quads ? (int)std::max<int64_t>(1, std::min<int64_t>(nblocks, (nq + kThreads * 16 - 1) / (kThreads * 16)))
                       : nblocks;
  if (quads)
    k_sqerr_q<<<nb, kThreads, 0, s>>>(reinterpret_cast<const float4*>(y), reinterpret_cast<const float4*>(dy),
                                      reinterpret_cast<const float4*>(t.q), reinterpret_cast<float4*>(ybar), nq,
                                      partials);
  else
    k_sqerr<<<nb, kThreads, 0, s>>>(y, dy, t, ybar, partials);
  itkg_status st = launched("sqerr_partials_f64");
  if (st != ITKG_SUCCESS) return st;
  k_sum_partials<<<1, kThreads, 0, s>>>(partials, nb, loss_out, accumulate_loss ? 1 : 0);
  if ((st = launched("sum_partials_f64")) != ITKG_SUCCESS) return st;
  if (!sigma_out) return ITKG_SUCCESS;
  k_sum_partials<<<1, kThreads, 0, s>>>(partials + nb, nb, sigma_out, 0);
  return launched("sum_partials_f64");
}

itkg_status launch_sum_partials(const double* partials, int n, double* out, bool accumulate,
                                void* stream) {
  k_sum_partials<<<1, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(partials, n, out,
                                                                        accumulate ? 1 : 0);
  return launched("sum_partials_f64");
}

itkg_status launch_dot(const DotArgs& d, double* partials, int nblocks, double* out,
                       bool accumulate, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_dot_partials<<<nblocks, kThreads, 0, s>>>(d, partials);
  itkg_status st = launched("dot_partials_f64");
  if (st != ITKG_SUCCESS) return st;
  k_sum_partials<<<1, kThreads, 0, s>>>(partials, nblocks, out, accumulate ? 1 : 0);
  return launched("sum_partials_f64");
}

}  // namespace itkg
