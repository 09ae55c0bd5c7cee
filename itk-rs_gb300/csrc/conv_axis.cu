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

#include <algorithm>
#include <cstdint>
#include <type_traits>

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
// with wrapping adds.  The per-tap products are tabulated once per pass by
// k_u8_lut: lut[k][v] for all 256 values of v, computed in f64 exactly as the
// reference does (an f64 product and round-half-away-from-zero are exact
// operations); each block copies the table into shared memory, so the pass
// itself is table lookups and byte adds.
__global__ void __launch_bounds__(kThreads) k_u8_lut(const AxisWeightsF64 W, int K, uint8_t* lut) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= K * 256) return;
  const int k = i >> 8, v = i & 255;
  double p = round((double)v * W.w[k]);
  p = p < 0.0 ? 0.0 : (p > 255.0 ? 255.0 : p);
  lut[i] = (uint8_t)p;
}

__global__ void __launch_bounds__(kThreads)
    k_conv_axis_u8(const AxisArgs a, const uint32_t* glut) {
  extern __shared__ uint8_t lut[];
  const int K = 2 * a.radius + 1;
  for (int i = threadIdx.x; i < K * 64; i += kThreads) reinterpret_cast<uint32_t*>(lut)[i] = glut[i];
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

// f32 -> f32 passes with radius <= 12 (every intermediate pass of the per-axis
// path, and the binomial blur's rounds): the radius is a template parameter
// (taps unrolled, weights read from the parameter bank) and each thread makes
// kRun outputs along a marching axis -- y for passes along x and y, z for
// passes along z.  Along y and z the kRun outputs share one register window of
// K + kRun - 1 loads; along x each of the kRun rows takes its K taps from the
// cache lines its warp already loaded.  Same arithmetic as k_conv_axis_f32: ascending taps from
// zero, clamp to [lo, hi] on `axis`.
template <int R>
constexpr int run_of() { return R <= 2 ? 8 : 4; }
constexpr int kMaxSmallR = 12;

template <int R, bool REF>
__global__ void __launch_bounds__(kThreads, R <= 4 ? 4 : 2)
    k_conv_axis_small(const AxisArgs a, const AxisWeightsF32 W) {
  constexpr int K = 2 * R + 1;
  constexpr int kRun = run_of<R>();
  const int64_t rowlen = a.out_size[0] * a.comps;
  const int64_t t = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (t >= rowlen) return;
  const int c = (int)(t % a.comps);
  const int64_t x = t / a.comps + a.out_index[0];
  const int axis = a.axis;
  const int md = axis == 2 ? 2 : 1;  // marching axis
  const int od = axis == 2 ? 1 : 2;  // the remaining axis
  const int64_t m0 = a.out_index[md], mn = a.out_size[md];
  const int64_t o0 = a.out_index[od], on = a.out_size[od];
  const char* const sx = static_cast<const char*>(a.src) + c * 4 + (x - a.src_origin[0]) * a.src_pitch[0];
  char* const dx = static_cast<char*>(a.dst) + c * 4 + (x - a.dst_origin[0]) * a.dst_pitch[0];
  const int64_t spm = a.src_pitch[md], spo = a.src_pitch[od];
  const int64_t dpm = a.dst_pitch[md], dpo = a.dst_pitch[od];
  // passes along x: the clamped tap offsets of this column
  int32_t xo[K];  // (clamped tap - x) * pitch: within +-R pixels
  if (axis == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      int64_t s = x + k - R;
      s = s < a.lo ? a.lo : (s > a.hi ? a.hi : s);
      xo[k] = (int32_t)((s - x) * a.src_pitch[0]);
    }
  }
  for (int64_t o = o0 + blockIdx.z; o < o0 + on; o += gridDim.z) {
    const char* const so = sx + (o - a.src_origin[od]) * spo;
    char* const dso = dx + (o - a.dst_origin[od]) * dpo;
    for (int64_t mb = m0 + (int64_t)blockIdx.y * kRun; mb < m0 + mn; mb += (int64_t)gridDim.y * kRun) {
      const int nv = (int)(m0 + mn - mb < kRun ? m0 + mn - mb : kRun);  // valid outputs of the run
      float acc[kRun];
      if (axis == 0) {
#pragma unroll
        for (int r = 0; r < kRun; ++r) {
          acc[r] = 0.0f;
          if (r < nv) {
            const char* const row = so + (mb + r - a.src_origin[md]) * spm;
#pragma unroll
            for (int k = 0; k < K; ++k) acc[r] = tap<REF>(acc[r], __ldg(reinterpret_cast<const float*>(row + xo[k])), W.w[k]);
          }
        }
      } else {
        // window over the marching axis: positions mb - R .. mb + kRun - 1 + R, clamped
        // to [lo, hi] and, beyond the last valid output's taps, to its last tap
        const int64_t top = mb + nv - 1 + R < a.hi ? mb + nv - 1 + R : a.hi;
        float v[K + kRun - 1];
#pragma unroll
        for (int j = 0; j < K + kRun - 1; ++j) {
          int64_t s = mb - R + j;
          s = s < a.lo ? a.lo : (s > top ? top : s);
          v[j] = __ldg(reinterpret_cast<const float*>(so + (s - a.src_origin[md]) * spm));
        }
#pragma unroll
        for (int r = 0; r < kRun; ++r) {
          acc[r] = 0.0f;
#pragma unroll
          for (int k = 0; k < K; ++k) acc[r] = tap<REF>(acc[r], v[r + k], W.w[k]);
        }
      }
#pragma unroll
      for (int r = 0; r < kRun; ++r)
        if (r < nv) *reinterpret_cast<float*>(dso + (mb + r - a.dst_origin[md]) * dpm) = acc[r];
    }
  }
}

using SmallFn = void (*)(const AxisArgs, const AxisWeightsF32);
template <int R>
constexpr SmallFn small_fn(bool ref) {
  return ref ? k_conv_axis_small<R, true> : k_conv_axis_small<R, false>;
}
SmallFn small_table(int r, bool ref) {
  static const SmallFn t[kMaxSmallR + 1][2] = {
      {nullptr, nullptr},
      {small_fn<1>(false), small_fn<1>(true)},   {small_fn<2>(false), small_fn<2>(true)},
      {small_fn<3>(false), small_fn<3>(true)},   {small_fn<4>(false), small_fn<4>(true)},
      {small_fn<5>(false), small_fn<5>(true)},   {small_fn<6>(false), small_fn<6>(true)},
      {small_fn<7>(false), small_fn<7>(true)},   {small_fn<8>(false), small_fn<8>(true)},
      {small_fn<9>(false), small_fn<9>(true)},   {small_fn<10>(false), small_fn<10>(true)},
      {small_fn<11>(false), small_fn<11>(true)}, {small_fn<12>(false), small_fn<12>(true)}};
  return (r >= 1 && r <= kMaxSmallR) ? t[r][ref ? 1 : 0] : nullptr;
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
  if constexpr (std::is_same<Tin, float>::value && std::is_same<Tout, float>::value) {
    const SmallFn fn = small_table(a.radius, rounding == ITKG_ROUND_REFERENCE);
    if (fn) {
      const int md = a.axis == 2 ? 2 : 1, od = a.axis == 2 ? 1 : 2;
      const int64_t gx = (a.out_size[0] * a.comps + kThreads - 1) / kThreads;
      const int run = a.radius <= 2 ? 8 : 4;
      const int64_t gy = std::min<int64_t>((a.out_size[md] + run - 1) / run, 65535);
      const int64_t gz = std::min<int64_t>(a.out_size[od], 65535);
      if (gx <= INT32_MAX) {
        fn<<<dim3((unsigned)gx, (unsigned)gy, (unsigned)gz), kThreads, 0, s>>>(a, W);
        note_launch(rounding == ITKG_ROUND_REFERENCE ? "conv_axis_f32_ref" : "conv_axis_f32_fma");
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "conv_axis launch: %s", cudaGetErrorString(e));
        return ITKG_SUCCESS;
      }
    }
  }
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

// Scalar u8 images (x pitch 1): four consecutive x outputs per thread, so the
// tap positions (and, on x, the loaded window of 4 + 2r pixels) are shared.
// The u8 adds wrap, so their order does not change the result.
__global__ void __launch_bounds__(kThreads)
    k_conv_axis_u8_x4(const AxisArgs a, const uint32_t* glut) {
  extern __shared__ uint8_t lut[];
  const int K = 2 * a.radius + 1;
  for (int i = threadIdx.x; i < K * 64; i += kThreads) reinterpret_cast<uint32_t*>(lut)[i] = glut[i];
  __syncthreads();
  const int64_t t = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const int64_t x = a.out_index[0] + 4 * t;
  const int64_t xe = a.out_index[0] + a.out_size[0];
  if (x >= xe) return;
  const int n = xe - x < 4 ? (int)(xe - x) : 4;
  const int64_t nrows = a.out_size[1] * a.out_size[2];
  const int axis = a.axis;
  for (int64_t row = blockIdx.y; row < nrows; row += gridDim.y) {
    const int64_t y = row % a.out_size[1] + a.out_index[1];
    const int64_t z = row / a.out_size[1] + a.out_index[2];
    uint32_t acc[4] = {0, 0, 0, 0};
    const uint8_t* const src = static_cast<const uint8_t*>(a.src);
    if (axis == 0) {
      const uint8_t* sb = src + (y - a.src_origin[1]) * a.src_pitch[1] + (z - a.src_origin[2]) * a.src_pitch[2];
      for (int i = 0; i < K + n - 1; ++i) {  // window position x - r + i: the taps of outputs x .. x + n - 1
        int64_t s = x - a.radius + i;
        s = s < a.lo ? a.lo : (s > a.hi ? a.hi : s);
        const uint32_t v = sb[s - a.src_origin[0]];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int k = i - j;
          if (k >= 0 && k < K) acc[j] += lut[(k << 8) | v];
        }
      }
    } else {
      const int64_t oa = axis == 1 ? y : z;
      const uint8_t* sb = src + (x - a.src_origin[0]) +
                          (axis == 1 ? (z - a.src_origin[2]) * a.src_pitch[2] : (y - a.src_origin[1]) * a.src_pitch[1]);
      const int64_t ap = a.src_pitch[axis];
      const int64_t ao = a.src_origin[axis];
      for (int k = 0; k < K; ++k) {
        int64_t s = oa + k - a.radius;
        s = s < a.lo ? a.lo : (s > a.hi ? a.hi : s);
        const uint8_t* p = sb + (s - ao) * ap;
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (j < n) acc[j] += lut[(k << 8) | p[j]];
      }
    }
    uint8_t* db = static_cast<uint8_t*>(a.dst) + (x - a.dst_origin[0]) + (y - a.dst_origin[1]) * a.dst_pitch[1] +
                  (z - a.dst_origin[2]) * a.dst_pitch[2];
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (j < n) db[j] = (uint8_t)acc[j];
  }
}

itkg_status launch_conv_axis_u8(const AxisArgs& a, const double* w, void* stream, void* lut_buf) {
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
  // The table (K * 256 bytes: a whole number of uint32 words) lives in the
  // caller's buffer when one is given, else in stream-ordered scratch.
  void* glut = lut_buf;
  if (!glut) {
    const itkg_status st = scratch_alloc(&glut, smem, s);
    if (st != ITKG_SUCCESS) return st;
  }
  k_u8_lut<<<(unsigned)((K * 256 + kThreads - 1) / kThreads), kThreads, 0, s>>>(W, K, static_cast<uint8_t*>(glut));
  note_launch("u8_lut");
  // a few dozen rows per block, so that copying the table is a small part of a block's work
  const bool x4 = a.comps == 1 && a.src_pitch[0] == 1 && a.dst_pitch[0] == 1;
  dim3 grid = grid_for(a);
  if (x4) grid.x = (unsigned)(((a.out_size[0] + 3) / 4 + kThreads - 1) / kThreads);
  grid.y = (unsigned)std::min<int64_t>((int64_t)grid.y, std::max<int64_t>(1, 4096 / (int64_t)grid.x));
  if (x4) {
    cudaFuncSetAttribute(k_conv_axis_u8_x4, cudaFuncAttributeMaxDynamicSharedMemorySize, 256 * (2 * kMaxU8Radius + 1));
    k_conv_axis_u8_x4<<<grid, kThreads, smem, s>>>(a, static_cast<const uint32_t*>(glut));
  } else {
    k_conv_axis_u8<<<grid, kThreads, smem, s>>>(a, static_cast<const uint32_t*>(glut));
  }
  note_launch("conv_axis_u8_pixel");
  if (!lut_buf) scratch_free(glut, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "conv_axis_u8 launch: %s", cudaGetErrorString(e));
  return ITKG_SUCCESS;
}

}  // namespace itkg
