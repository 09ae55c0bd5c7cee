// Pixel load/store conversions shared by every kernel.
//
// Loads convert the storage type exactly to f32: this is the reference's
// UnaryFilter(|p| p as f32) placed in front of GaussianFilter<f32>
// (examples/blur_png.rs:35-36).  Stores convert f32 to the storage type:
// bf16/f16 round to nearest even; u8 follows the reference's
// |p: f32| p.round().clamp(0.0, 255.0) as u8 (examples/blur_png.rs:37), where
// round is half away from zero and NaN maps to 0 (Rust's saturating cast).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cstdint>

namespace itkg {

__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(int16_t v) { return (float)v; }
__device__ __forceinline__ float to_f32(uint8_t v) { return (float)v; }
__device__ __forceinline__ float to_f32(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float to_f32(__half v) { return __half2float(v); }

template <typename T>
__device__ __forceinline__ T from_f32(float v);

template <>
__device__ __forceinline__ float from_f32<float>(float v) { return v; }
template <>
__device__ __forceinline__ __nv_bfloat16 from_f32<__nv_bfloat16>(float v) {
  return __float2bfloat16_rn(v);
}
template <>
__device__ __forceinline__ __half from_f32<__half>(float v) { return __float2half_rn(v); }
template <>
__device__ __forceinline__ uint8_t from_f32<uint8_t>(float v) {
  float r = roundf(v);  // half away from zero, like Rust's f32::round
  if (r != r) return 0;
  r = fminf(fmaxf(r, 0.0f), 255.0f);
  return (uint8_t)r;
}

// One reference tap: acc + x * w with separate rounding (conv.rs:35 through
// pixel.rs:418), or a fused multiply-add.
template <bool REF>
__device__ __forceinline__ float tap(float acc, float x, float w) {
  if constexpr (REF) {
    return __fadd_rn(acc, __fmul_rn(x, w));
  } else {
    return fmaf(x, w, acc);
  }
}

}  // namespace itkg
