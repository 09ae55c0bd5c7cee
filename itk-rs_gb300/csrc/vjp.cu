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

#include "internal.hpp"
#include "pixel.cuh"

namespace itkg {
namespace {

constexpr int kThreads = 256;

struct Taps {
  float w[kMaxVjpTaps];
  float aux[kMaxVjpTaps];  // dw/dsigma (dual pass) or prefix sums P (adjoint pass)
};

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
  const int64_t n = a.size[axis];
  const int64_t ap = a.in_pitch[axis];
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
  const int64_t n = a.size[axis];
  const int64_t ap = a.in_pitch[axis];
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

// Per-block f64 partial sums of sum(p * q) over a pitched image.
__global__ void __launch_bounds__(kThreads) k_dot_partials(const DotArgs d, double* partials) {
  const int64_t nx = d.size[0], nxy = d.size[0] * d.size[1];
  const int64_t n = nxy * d.size[2];
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads) {
    const int64_t x = i % nx, y = (i / nx) % d.size[1], z = i / nxy;
    const float a = *reinterpret_cast<const float*>(px(d.p, d.p_pitch, x, y, z));
    const float b = *reinterpret_cast<const float*>(px(d.q, d.q_pitch, x, y, z));
    s += (double)a * (double)b;
  }
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
__global__ void __launch_bounds__(kThreads) k_sqerr(const float* __restrict__ y,
                                                     const float* __restrict__ dy, const DotArgs t,
                                                     float* __restrict__ ybar, double* partials) {
  const int64_t nx = t.size[0], nxy = t.size[0] * t.size[1];
  const int64_t n = nxy * t.size[2];
  double sl = 0.0, ss = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads) {
    const int64_t x = i % nx, yy = (i / nx) % t.size[1], z = i / nxy;
    const float tv = *reinterpret_cast<const float*>(px(t.q, t.q_pitch, x, yy, z));
    const float d = y[i] - tv;
    const float g = 2.0f * d;
    ybar[i] = g;
    sl += (double)d * (double)d;
    if (dy) ss += (double)g * (double)dy[i];
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
  k_adjoint_axis<<<grid_for(a), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      a, make_taps(w, prefix, 2 * a.radius + 1));
  return launched("adjoint_axis_f32");
}

itkg_status launch_dual_axis(const VjpAxisArgs& a, const float* w, const float* dw, void* stream) {
  if (2 * a.radius + 1 > kMaxVjpTaps)
    return set_error(ITKG_ERROR_UNSUPPORTED, "VJP radius %d exceeds %d", a.radius, (kMaxVjpTaps - 1) / 2);
  k_dual_axis<<<grid_for(a), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      a, make_taps(w, dw, 2 * a.radius + 1));
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
  k_sqerr<<<nblocks, kThreads, 0, s>>>(y, dy, t, ybar, partials);
  itkg_status st = launched("sqerr_partials_f64");
  if (st != ITKG_SUCCESS) return st;
  k_sum_partials<<<1, kThreads, 0, s>>>(partials, nblocks, loss_out, accumulate_loss ? 1 : 0);
  if ((st = launched("sum_partials_f64")) != ITKG_SUCCESS) return st;
  if (!sigma_out) return ITKG_SUCCESS;
  k_sum_partials<<<1, kThreads, 0, s>>>(partials + nblocks, nblocks, sigma_out, 0);
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
