// Region geometry, descriptor validation and CUDA error mapping shared by the
// C-ABI translation units (abi.cpp, vjp_host.cpp, batch.cpp).
//   kernel_radius            src/filters/gaussian.rs:24-27
//   build_kernel             src/filters/gaussian.rs:29-40
//   padded / clipped         src/image.rs:28-64
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "internal.hpp"

namespace itkg {

inline itkg_status cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return ITKG_SUCCESS;
  cudaGetLastError();  // clear sticky-free errors
  if (e == cudaErrorMemoryAllocation)
    return set_error(ITKG_ERROR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
    return set_error(ITKG_ERROR_NO_DEVICE, "%s: %s", what, cudaGetErrorString(e));
  return set_error(ITKG_ERROR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define ITKG_CUDA(call)                                   \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_status(e_, #call); \
  } while (0)

#define ITKG_TRY(expr)                        \
  do {                                        \
    itkg_status s_ = (expr);                  \
    if (s_ != ITKG_SUCCESS) return s_;        \
  } while (0)


inline uint64_t kernel_radius(double sigma, double spacing) {
  const double c = std::ceil(3.0 * (sigma / spacing));
  if (!(c > 0.0)) return 0;  // NaN and non-positive saturate to 0
  if (c >= 18446744073709551615.0) return UINT64_MAX;
  return (uint64_t)c;
}

inline void build_kernel(double sigma_px, uint64_t radius, double* out) {
  const uint64_t len = 2 * radius + 1;
  for (uint64_t i = 0; i < len; ++i) {
    const double x = (double)i - (double)radius;
    const double t = x / sigma_px;
    out[i] = std::exp(-0.5 * (t * t));
  }
  double sum = 0.0;
  for (uint64_t i = 0; i < len; ++i) sum += out[i];
  for (uint64_t i = 0; i < len; ++i) out[i] /= sum;
}

inline itkg_region padded(const itkg_region& r, int D, const uint64_t* radii) {
  itkg_region o = r;
  for (int d = 0; d < D; ++d) {
    o.index[d] -= (int64_t)radii[d];
    o.size[d] += 2 * radii[d];
  }
  return o;
}

inline itkg_region clipped(const itkg_region& r, int D, const itkg_region& b) {
  itkg_region o = r;
  for (int d = 0; d < D; ++d) {
    const int64_t se = r.index[d] + (int64_t)r.size[d];
    const int64_t be = b.index[d] + (int64_t)b.size[d];
    const int64_t s = std::max(r.index[d], b.index[d]);
    const int64_t e = std::min(se, be);
    o.index[d] = s;
    o.size[d] = e > s ? (uint64_t)(e - s) : 0;
  }
  return o;
}

inline uint64_t region_len(const itkg_region& r, int D) {
  uint64_t n = 1;
  for (int d = 0; d < D; ++d) n *= r.size[d];
  return n;
}

inline bool region_contains(const itkg_region& outer, const itkg_region& inner, int D) {
  for (int d = 0; d < D; ++d) {
    if (inner.size[d] == 0) return true;
    if (inner.index[d] < outer.index[d]) return false;
    if (inner.index[d] + (int64_t)inner.size[d] > outer.index[d] + (int64_t)outer.size[d])
      return false;
  }
  return true;
}

// Fill unused trailing axes so kernels can treat every image as 3-D.
inline itkg_region full3(const itkg_region& r, int D) {
  itkg_region o = r;
  for (int d = D; d < kMaxDim; ++d) {
    o.index[d] = 0;
    o.size[d] = 1;
  }
  return o;
}

inline itkg_status validate_image(const itkg_image* im, const char* name) {
  if (!im) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s is NULL", name);
  if (im->dim < 1 || im->dim > kMaxDim)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s: dim %d not in 1..3", name, im->dim);
  if (dtype_size(im->dtype) == 0)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s: unknown dtype %d", name, im->dtype);
  if (im->components < 1 || im->components > 3)
    return set_error(ITKG_ERROR_UNSUPPORTED, "%s: components must be 1, 2 or 3", name);
  if (im->location != ITKG_DEVICE && im->location != ITKG_HOST)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s: unknown location", name);
  const int64_t pb = (int64_t)im->components * dtype_size(im->dtype);
  if (im->pitch[0] != pb)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s: pitch[0]=%lld must equal the pixel size %lld",
                     name, (long long)im->pitch[0], (long long)pb);
  for (int d = 1; d < im->dim; ++d)
    if (im->pitch[d] <= 0 || im->pitch[d] % dtype_size(im->dtype) != 0)
      return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s: pitch[%d] invalid", name, d);
  if (!im->data && region_len(im->region, im->dim) != 0)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s: data is NULL", name);
  return ITKG_SUCCESS;
}

// The smoothing filters take scalar pixels, VecPixel<_, 3> and VecPixel<_, 2>
// (2-D displacement fields, DisplacementFieldToBSplineFilter).
inline itkg_status filter_components(const itkg_image* im, const char* name) {
  if (im->components < 1 || im->components > 3)
    return set_error(ITKG_ERROR_UNSUPPORTED, "%s: components must be 1, 2 or 3", name);
  return ITKG_SUCCESS;
}

// Normalised device view of an image (3-D, pitches for unused axes = 0).
inline void origin_pitch(const itkg_image& im, int64_t* origin, int64_t* pitch) {
  for (int d = 0; d < kMaxDim; ++d) {
    origin[d] = d < im.dim ? im.region.index[d] : 0;
    pitch[d] = d < im.dim ? im.pitch[d] : 0;
  }
}

// Dense layout with rows and slices padded to `align` bytes.
inline void dense_layout(itkg_image* im, int align) {
  const int64_t pb = (int64_t)im->components * dtype_size(im->dtype);
  im->pitch[0] = pb;
  int64_t row = (int64_t)im->region.size[0] * pb;
  if (align > 1) row = (row + align - 1) / align * align;
  if (row == 0) row = align > 1 ? align : pb;
  im->pitch[1] = row;
  im->pitch[2] = row * (int64_t)(im->dim >= 2 ? std::max<uint64_t>(im->region.size[1], 1) : 1);
  for (int d = im->dim; d < kMaxDim; ++d) im->pitch[d] = d == 1 ? row : im->pitch[d];
}

inline size_t image_bytes(const itkg_image& im) {
  if (region_len(im.region, im.dim) == 0) return 0;
  size_t last = 0;
  for (int d = 0; d < im.dim; ++d) last += (size_t)(im.region.size[d] - 1) * (size_t)im.pitch[d];
  return last + (size_t)im.pitch[0];
}

// Copy `reg` between two images (any locations) with 2-D copies per slice, or

}  // namespace itkg
