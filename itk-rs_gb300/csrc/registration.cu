// The in-crate Gaussian callers that iterate around it:
//   DemonsRegistrationFilter / DiffeomorphicDemonsRegistrationFilter
//     (src/filters/registration_methods.rs:39-100, 126-148): the demons force
//     update of a 2-D displacement field, then (diffeomorphic) GaussianFilter
//     on each displacement component;
//   N4BiasFieldCorrectionFilter (src/filters/bias_correction.rs:45-83): per
//     iteration the log image, its GaussianFilter smoothing, the corrected
//     image exp(log - smoothed) and a mean-absolute-change convergence test.
// This file holds the point-wise kernels; the Gaussian is the library's own
// generate_region, called by the entry points in abi.cpp.
//
// Arithmetic follows the reference operation by operation in f64 with every
// product, sum, quotient and square root rounded separately (__dmul_rn,
// __dadd_rn, __ddiv_rn, __dsqrt_rn: IEEE results, identical to the
// reference's on any host).  N4's ln and exp are the device's f64 log and exp,
// whose last bit may differ from the host libm's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "internal.hpp"

namespace itkg {
namespace {

constexpr int kT = 256;

// Rust's `f64 as i64` (saturating, NaN -> 0).
__device__ __forceinline__ long long sat_i64(double v) {
  if (v != v) return 0;
  if (v >= 9.2233720368547758e18) return LLONG_MAX;
  if (v <= -9.2233720368547758e18) return LLONG_MIN;
  return (long long)v;
}

// One demons iteration (registration_methods.rs:58-90) over the w x h fixed
// region, pixel i = y * w + x.  fixed / moving: f32 rows at the given pitches
// (elements); the moving image's region is mw x mh at (mox, moy), the fixed
// region's index (ox, oy).  A warped index whose flat offset (computed as the
// reference's Image::flat_index does, image.rs:111-120, with wrapping usize
// arithmetic) falls outside the moving buffer is where the reference panics:
// the kernel sets *err and leaves that pixel's displacement unchanged.
__global__ void __launch_bounds__(kT) k_demons_step(const float* __restrict__ fixed, int64_t fp, int64_t w, int64_t h,
                                                     int64_t ox, int64_t oy, const float* __restrict__ moving, int64_t mp,
                                                     int64_t mw, int64_t mh, int64_t mox, int64_t moy,
                                                     const double* __restrict__ dxi, const double* __restrict__ dyi,
                                                     double* __restrict__ dxo, double* __restrict__ dyo, double max_step,
                                                     unsigned int* err) {
  const int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x;
  if (i >= w * h) return;
  const int64_t y = i / w, x = i - y * w;
  const double dx0 = dxi[i], dy0 = dyi[i];
  const double wx = __dadd_rn((double)x, dx0);
  const double wy = __dadd_rn((double)y, dy0);
  const unsigned long long xi = (unsigned long long)ox + (unsigned long long)sat_i64(round(wx));
  const unsigned long long yi = (unsigned long long)oy + (unsigned long long)sat_i64(round(wy));
  const unsigned long long lx = xi - (unsigned long long)mox, ly = yi - (unsigned long long)moy;
  const unsigned long long flat = lx + ly * (unsigned long long)mw;
  if (flat >= (unsigned long long)(mw * mh)) {
    atomicExch(err, 1u);
    dxo[i] = dx0;
    dyo[i] = dy0;
    return;
  }
  const int64_t fy = (int64_t)(flat / (unsigned long long)mw), fx = (int64_t)(flat % (unsigned long long)mw);
  const double m_val = (double)moving[fy * mp + fx];
  const double f_val = (double)fixed[y * fp + x];
  // gradient of fixed, central differences clamped to its region
  const int64_t xp = x + 1 < w ? x + 1 : w - 1, xm = x - 1 > 0 ? x - 1 : 0;
  const int64_t yp = y + 1 < h ? y + 1 : h - 1, ym = y - 1 > 0 ? y - 1 : 0;
  const double gx = __dmul_rn(__dadd_rn((double)fixed[y * fp + xp], -(double)fixed[y * fp + xm]), 0.5);
  const double gy = __dmul_rn(__dadd_rn((double)fixed[yp * fp + x], -(double)fixed[ym * fp + x]), 0.5);
  const double diff = __dadd_rn(f_val, -m_val);
  const double denom =
      __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(gx, gx), __dmul_rn(gy, gy)), __dmul_rn(diff, diff)), 1e-6);
  const double step = __ddiv_rn(diff, denom);
  const double sx = __dmul_rn(step, gx), sy = __dmul_rn(step, gy);
  const double norm = __dsqrt_rn(__dadd_rn(__dmul_rn(sx, sx), __dmul_rn(sy, sy)));
  const double scale = norm > max_step ? __ddiv_rn(max_step, norm) : 1.0;
  dxo[i] = __dadd_rn(dx0, __dmul_rn(sx, scale));
  dyo[i] = __dadd_rn(dy0, __dmul_rn(sy, scale));
}

// f64 displacement -> f32 (`as f32`, round to nearest): interleaved
// VecPixel<f32, 2> rows at pitch op (pixels), or two planar images (rows at
// pitch pp floats) when planar != 0.
__global__ void __launch_bounds__(kT) k_demons_to_f32(const double* __restrict__ dx, const double* __restrict__ dy,
                                                       int64_t w, int64_t h, float* __restrict__ out, int64_t op,
                                                       float* __restrict__ px, float* __restrict__ py, int64_t pp,
                                                       int planar) {
  const int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x;
  if (i >= w * h) return;
  const int64_t y = i / w, x = i - y * w;
  const float fx = __double2float_rn(dx[i]), fy = __double2float_rn(dy[i]);
  if (planar) {
    px[y * pp + x] = fx;
    py[y * pp + x] = fy;
  } else {
    *reinterpret_cast<float2*>(out + 2 * (y * op + x)) = make_float2(fx, fy);
  }
}

// two planar f32 images (rows at pitch sp) -> interleaved VecPixel<f32, 2>
__global__ void __launch_bounds__(kT) k_interleave2(const float* __restrict__ a, const float* __restrict__ b, int64_t sp,
                                                     int64_t w, int64_t h, float* __restrict__ out, int64_t op) {
  const int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x;
  if (i >= w * h) return;
  const int64_t y = i / w, x = i - y * w;
  *reinterpret_cast<float2*>(out + 2 * (y * op + x)) = make_float2(a[y * sp + x], b[y * sp + x]);
}

// N4: corrected = (p as f64).max(1e-6) (bias_correction.rs:51)
__global__ void __launch_bounds__(kT) k_n4_init(const float* __restrict__ in, int64_t ip, int64_t w, int64_t h,
                                                 double* __restrict__ corr) {
  const int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x;
  if (i >= w * h) return;
  const int64_t y = i / w, x = i - y * w;
  corr[i] = fmax((double)in[y * ip + x], 1e-6);
}

// N4: log_data = ln(corrected) (f64, kept) and its f32 image (:55, :64)
__global__ void __launch_bounds__(kT) k_n4_log(const double* __restrict__ corr, int64_t n, double* __restrict__ ld,
                                                float* __restrict__ lf) {
  const int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x;
  if (i >= n) return;
  const double l = log(corr[i]);
  ld[i] = l;
  lf[i] = __double2float_rn(l);
}

// N4: corrected = exp(l - s).max(1e-6) (:71-74) and per-block sums of
// |corrected - prev| (:77), summed by a fixed-order reduction afterwards
__global__ void __launch_bounds__(kT) k_n4_update(const double* __restrict__ ld, const float* __restrict__ sm,
                                                   int64_t n, double* __restrict__ corr, double* __restrict__ partials) {
  __shared__ double red[kT / 32];
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT) {
    const double prev = corr[i];
    const double c = fmax(exp(__dadd_rn(ld[i], -(double)sm[i])), 1e-6);
    corr[i] = c;
    acc = __dadd_rn(acc, fabs(__dadd_rn(c, -prev)));
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < kT / 32; ++k) t += red[k];
    partials[blockIdx.x] = t;
  }
}

// N4: output = corrected as f32 (:80)
__global__ void __launch_bounds__(kT) k_n4_store(const double* __restrict__ corr, int64_t w, int64_t h,
                                                  float* __restrict__ out, int64_t op) {
  const int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x;
  if (i >= w * h) return;
  const int64_t y = i / w, x = i - y * w;
  out[y * op + x] = __double2float_rn(corr[i]);
}

unsigned blocks_for(int64_t n) { return (unsigned)((n + kT - 1) / kT); }

itkg_status launched(const char* name) {
  note_launch(name);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "%s launch: %s", name, cudaGetErrorString(e));
  return ITKG_SUCCESS;
}

}  // namespace

itkg_status launch_demons_step(const DemonsGeom& g, const double* dxi, const double* dyi, double* dxo, double* dyo,
                               double max_step, unsigned int* err, void* stream) {
  const int64_t n = g.w * g.h;
  if (n == 0) return ITKG_SUCCESS;
  k_demons_step<<<blocks_for(n), kT, 0, static_cast<cudaStream_t>(stream)>>>(
      g.fixed, g.fp, g.w, g.h, g.ox, g.oy, g.moving, g.mp, g.mw, g.mh, g.mox, g.moy, dxi, dyi, dxo, dyo, max_step,
      err);
  return launched("demons_step_f64");
}

itkg_status launch_demons_to_f32(const double* dx, const double* dy, int64_t w, int64_t h, float* out, int64_t op,
                                 float* px, float* py, int64_t pp, void* stream) {
  if (w * h == 0) return ITKG_SUCCESS;
  k_demons_to_f32<<<blocks_for(w * h), kT, 0, static_cast<cudaStream_t>(stream)>>>(dx, dy, w, h, out, op, px, py, pp,
                                                                                     px != nullptr ? 1 : 0);
  return launched("demons_to_f32");
}

itkg_status launch_interleave2(const float* a, const float* b, int64_t sp, int64_t w, int64_t h, float* out, int64_t op,
                               void* stream) {
  if (w * h == 0) return ITKG_SUCCESS;
  k_interleave2<<<blocks_for(w * h), kT, 0, static_cast<cudaStream_t>(stream)>>>(a, b, sp, w, h, out, op);
  return launched("interleave2");
}

itkg_status launch_n4_init(const float* in, int64_t ip, int64_t w, int64_t h, double* corr, void* stream) {
  k_n4_init<<<blocks_for(w * h), kT, 0, static_cast<cudaStream_t>(stream)>>>(in, ip, w, h, corr);
  return launched("n4_init");
}

itkg_status launch_n4_log(const double* corr, int64_t n, double* ld, float* lf, void* stream) {
  k_n4_log<<<blocks_for(n), kT, 0, static_cast<cudaStream_t>(stream)>>>(corr, n, ld, lf);
  return launched("n4_log_f64");
}

int n4_blocks(int64_t n) {
  const int64_t b = (n + kT * 8 - 1) / (kT * 8);
  return (int)std::min<int64_t>(std::max<int64_t>(b, 1), 1024);
}

itkg_status launch_n4_update(const double* ld, const float* sm, int64_t n, double* corr, double* partials, int blocks,
                             void* stream) {
  k_n4_update<<<blocks, kT, 0, static_cast<cudaStream_t>(stream)>>>(ld, sm, n, corr, partials);
  return launched("n4_update_f64");
}

itkg_status launch_n4_store(const double* corr, int64_t w, int64_t h, float* out, int64_t op, void* stream) {
  k_n4_store<<<blocks_for(w * h), kT, 0, static_cast<cudaStream_t>(stream)>>>(corr, w, h, out, op);
  return launched("n4_store");
}

}  // namespace itkg
