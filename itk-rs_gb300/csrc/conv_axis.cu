// Per-axis separable pass: the general path of GaussianFilter::generate_region
// (src/filters/gaussian.rs:74-88) that runs one convolve_axis
// (src/filters/conv.rs:11-41) per axis through an f32 scratch buffer.  It
// covers every dimension, dtype, component count and radius up to 384, and is
// the fallback when no fused kernel fits.
//
// One thread computes one output component; threads run along axis 0 so loads
// and stores coalesce for every pass (for axes 1 and 2 each tap is a row-wide
// coalesced load).  The tap loop is the reference's: ascending k, clamp to the
// source extent on `axis`, acc starting at zero.
#include <cuda_runtime.h>

#include "internal.hpp"
#include "pixel.cuh"

namespace itkg {
namespace {

constexpr int kThreads = 256;

template <typename Tin, typename Tout, bool REF>
__global__ void __launch_bounds__(kThreads)
    k_conv_axis_f32(const AxisArgs a, const AxisWeightsF32 W) {
  const int64_t rowlen = a.out_size[0] * a.comps;
  const int64_t t = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (t >= rowlen) return;
  const int c = (int)(t % a.comps);
  const int64_t x = t / a.comps + a.out_index[0];
  const int64_t nrows = a.out_size[1] * a.out_size[2];
  const int axis = a.axis;
  const int K = 2 * a.radius + 1;
  for (int64_t row = blockIdx.y; row < nrows; row += gridDim.y) {
    const int64_t y = row % a.out_size[1] + a.out_index[1];
    const int64_t z = row / a.out_size[1] + a.out_index[2];
    const char* sb = static_cast<const char*>(a.src) + c * (int64_t)sizeof(Tin);
    int64_t oa;
    if (axis == 0) {
      oa = x;
      sb += (y - a.src_origin[1]) * a.src_pitch[1] + (z - a.src_origin[2]) * a.src_pitch[2];
    } else if (axis == 1) {
      oa = y;
      sb += (x - a.src_origin[0]) * a.src_pitch[0] + (z - a.src_origin[2]) * a.src_pitch[2];
    } else {
      oa = z;
      sb += (x - a.src_origin[0]) * a.src_pitch[0] + (y - a.src_origin[1]) * a.src_pitch[1];
    }
    const int64_t ap = a.src_pitch[axis];
    const int64_t ao = a.src_origin[axis];
    float acc = 0.0f;
    for (int k = 0; k < K; ++k) {
      int64_t s = oa + k - a.radius;
      s = s < a.lo ? a.lo : s;
      s = s > a.hi ? a.hi : s;
      const float v = to_f32(*reinterpret_cast<const Tin*>(sb + (s - ao) * ap));
      acc = tap<REF>(acc, v, W.w[k]);
    }
    char* db = static_cast<char*>(a.dst) + c * (int64_t)sizeof(Tout) +
               (x - a.dst_origin[0]) * a.dst_pitch[0] + (y - a.dst_origin[1]) * a.dst_pitch[1] +
               (z - a.dst_origin[2]) * a.dst_pitch[2];
    *reinterpret_cast<Tout*>(db) = from_f32<Tout>(acc);
  }
}

// GaussianFilter<Image<u8>>: NumericPixel for u8 (src/pixel.rs:430-435).  Each
// tap is round(x as f64 * w).clamp(0, 255) as u8 and the accumulator is a u8
// with wrapping adds.  The per-tap products are tabulated once per block:
// lut[k][v] for all 256 values of v, computed in f64 exactly as the reference
// does (an f64 product and round-half-away-from-zero are exact operations), so
// the pass itself is table lookups and byte adds.
__global__ void __launch_bounds__(kThreads)
    k_conv_axis_u8(const AxisArgs a, const AxisWeightsF64 W) {
  extern __shared__ uint8_t lut[];
  const int K = 2 * a.radius + 1;
  for (int i = threadIdx.x; i < K * 256; i += kThreads) {
    const int k = i >> 8, v = i & 255;
    double p = round((double)v * W.w[k]);
    p = p < 0.0 ? 0.0 : (p > 255.0 ? 255.0 : p);
    lut[i] = (uint8_t)p;
  }
  __syncthreads();
  const int64_t rowlen = a.out_size[0] * a.comps;
  const int64_t t = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (t >= rowlen) return;
  const int c = (int)(t % a.comps);
  const int64_t x = t / a.comps + a.out_index[0];
  const int64_t nrows = a.out_size[1] * a.out_size[2];
  const int axis = a.axis;
  for (int64_t row = blockIdx.y; row < nrows; row += gridDim.y) {
    const int64_t y = row % a.out_size[1] + a.out_index[1];
    const int64_t z = row / a.out_size[1] + a.out_index[2];
    const uint8_t* sb = static_cast<const uint8_t*>(a.src) + c;
    int64_t oa;
    if (axis == 0) {
      oa = x;
      sb += (y - a.src_origin[1]) * a.src_pitch[1] + (z - a.src_origin[2]) * a.src_pitch[2];
    } else if (axis == 1) {
      oa = y;
      sb += (x - a.src_origin[0]) * a.src_pitch[0] + (z - a.src_origin[2]) * a.src_pitch[2];
    } else {
      oa = z;
      sb += (x - a.src_origin[0]) * a.src_pitch[0] + (y - a.src_origin[1]) * a.src_pitch[1];
    }
    const int64_t ap = a.src_pitch[axis];
    const int64_t ao = a.src_origin[axis];
    uint8_t acc = 0;
    for (int k = 0; k < K; ++k) {
      int64_t s = oa + k - a.radius;
      s = s < a.lo ? a.lo : s;
      s = s > a.hi ? a.hi : s;
      acc = (uint8_t)(acc + lut[(k << 8) | sb[(s - ao) * ap]]);
    }
    uint8_t* db = static_cast<uint8_t*>(a.dst) + c + (x - a.dst_origin[0]) * a.dst_pitch[0] +
                  (y - a.dst_origin[1]) * a.dst_pitch[1] + (z - a.dst_origin[2]) * a.dst_pitch[2];
    *db = acc;
  }
}

dim3 grid_for(const AxisArgs& a) {
  const int64_t rowlen = a.out_size[0] * a.comps;
  const int64_t nrows = a.out_size[1] * a.out_size[2];
  const int64_t gx = (rowlen + kThreads - 1) / kThreads;
  int64_t gy = nrows < 65535 ? nrows : 65535;
  return dim3((unsigned)gx, (unsigned)gy, 1);
}

template <typename Tin, typename Tout>
itkg_status launch_typed(const AxisArgs& a, const AxisWeightsF32& W, int rounding,
                         cudaStream_t s) {
  dim3 grid = grid_for(a);
  if (rounding == ITKG_ROUND_REFERENCE) {
    k_conv_axis_f32<Tin, Tout, true><<<grid, kThreads, 0, s>>>(a, W);
    note_launch("conv_axis_f32_ref");
  } else {
    k_conv_axis_f32<Tin, Tout, false><<<grid, kThreads, 0, s>>>(a, W);
    note_launch("conv_axis_f32_fma");
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "conv_axis launch: %s", cudaGetErrorString(e));
  return ITKG_SUCCESS;
}

template <typename Tin>
itkg_status launch_in(const AxisArgs& a, const AxisWeightsF32& W, int out_dtype, int rounding,
                      cudaStream_t s) {
  switch (out_dtype) {
    case ITKG_F32: return launch_typed<Tin, float>(a, W, rounding, s);
    case ITKG_BF16: return launch_typed<Tin, __nv_bfloat16>(a, W, rounding, s);
    case ITKG_F16: return launch_typed<Tin, __half>(a, W, rounding, s);
    case ITKG_U8: return launch_typed<Tin, uint8_t>(a, W, rounding, s);
    default: return set_error(ITKG_ERROR_UNSUPPORTED, "output dtype %d not supported", out_dtype);
  }
}

}  // namespace

itkg_status launch_conv_axis_f32(const AxisArgs& a, const float* w, int in_dtype, int out_dtype,
                                 int rounding, void* stream) {
  const int K = 2 * a.radius + 1;
  if (K > kMaxParamTaps)
    return set_error(ITKG_ERROR_UNSUPPORTED, "radius %d exceeds the per-axis limit %d", a.radius,
                     (kMaxParamTaps - 1) / 2);
  if (a.out_size[0] * a.out_size[1] * a.out_size[2] == 0) return ITKG_SUCCESS;
  AxisWeightsF32 W;
  for (int k = 0; k < K; ++k) W.w[k] = w[k];
  for (int k = K; k < kMaxParamTaps; ++k) W.w[k] = 0.0f;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (in_dtype) {
    case ITKG_F32: return launch_in<float>(a, W, out_dtype, rounding, s);
    case ITKG_I16: return launch_in<int16_t>(a, W, out_dtype, rounding, s);
    case ITKG_U8: return launch_in<uint8_t>(a, W, out_dtype, rounding, s);
    case ITKG_BF16: return launch_in<__nv_bfloat16>(a, W, out_dtype, rounding, s);
    case ITKG_F16: return launch_in<__half>(a, W, out_dtype, rounding, s);
    default: return set_error(ITKG_ERROR_UNSUPPORTED, "input dtype %d not supported", in_dtype);
  }
}

itkg_status launch_conv_axis_u8(const AxisArgs& a, const double* w, void* stream) {
  const int K = 2 * a.radius + 1;
  if (a.radius > kMaxU8Radius)
    return set_error(ITKG_ERROR_UNSUPPORTED, "u8 pixel arithmetic supports radius <= %d",
                     kMaxU8Radius);
  if (a.out_size[0] * a.out_size[1] * a.out_size[2] == 0) return ITKG_SUCCESS;
  AxisWeightsF64 W;
  for (int k = 0; k < K; ++k) W.w[k] = w[k];
  for (int k = K; k < kMaxParamTaps / 2; ++k) W.w[k] = 0.0;
  const size_t smem = (size_t)K * 256;
  cudaFuncSetAttribute(k_conv_axis_u8, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       256 * (2 * kMaxU8Radius + 1));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_conv_axis_u8<<<grid_for(a), kThreads, smem, s>>>(a, W);
  note_launch("conv_axis_u8_pixel");
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "conv_axis_u8 launch: %s", cudaGetErrorString(e));
  return ITKG_SUCCESS;
}

}  // namespace itkg
