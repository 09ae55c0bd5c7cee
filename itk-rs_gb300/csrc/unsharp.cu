// UnsharpMaskFilter (src/filters/edges.rs:374-452): the point-wise step after
// the blur.  For every requested voxel, in f64 with each operation rounded in
// the reference's order:
//   edge = orig - blur;  out = |edge| > threshold ? orig + amount * edge : orig
// converted with P::from_f64 (f32: round to nearest; u8: round half away from
// zero, clamp to [0, 255], NaN -> 0).  Vector pixels follow pixel.rs:93-98:
// to_f64 reads the first component and from_f64 fills every component.  The
// blur itself is the convolve_axis family's (itkg_separable_generate_region)
// with the filter's own kernel.
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.hpp"

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
                                                 int comps, double amount, double threshold) {
  const int64_t x = (int64_t)blockIdx.x * kT + threadIdx.x;
  if (x >= m0) return;
  for (int64_t z = blockIdx.z; z < m2; z += gridDim.z)
    for (int64_t y = blockIdx.y; y < m1; y += gridDim.y) {
      const double orig = (double)*reinterpret_cast<const Tp*>(in + x * ip0 + y * ip1 + z * ip2);
      const double bl = (double)*reinterpret_cast<const Tp*>(blur + x * bp0 + y * bp1 + z * bp2);
      const double edge = __dsub_rn(orig, bl);
      const double v = fabs(edge) > threshold ? __dadd_rn(orig, __dmul_rn(amount, edge)) : orig;
      char* const o = out + x * op0 + y * op1 + z * op2;
      if constexpr (sizeof(Tp) == 1) {
        const uint8_t q = u8_of(v);
        for (int c = 0; c < comps; ++c) reinterpret_cast<uint8_t*>(o)[c] = q;
      } else {
        const float q = __double2float_rn(v);
        for (int c = 0; c < comps; ++c) reinterpret_cast<float*>(o)[c] = q;
      }
    }
}

}  // namespace

// in / blur / out: the first requested voxel of each image and their pitches
// (bytes); m: the requested size; comps: components per pixel.
itkg_status launch_unsharp(int dtype, int comps, const void* in, const int64_t* ip, const void* blur,
                           const int64_t* bp, void* out, const int64_t* op, const int64_t* m, double amount,
                           double threshold, void* stream) {
  if (m[0] * m[1] * m[2] == 0) return ITKG_SUCCESS;
  const dim3 gr((unsigned)((m[0] + kT - 1) / kT), (unsigned)std::min<int64_t>(m[1], 65535),
                (unsigned)std::min<int64_t>(m[2], 65535));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const char* ic = static_cast<const char*>(in);
  const char* bc = static_cast<const char*>(blur);
  char* oc = static_cast<char*>(out);
  if (dtype == ITKG_U8)
    k_unsharp<uint8_t><<<gr, kT, 0, s>>>(ic, ip[0], ip[1], ip[2], bc, bp[0], bp[1], bp[2], oc, op[0], op[1], op[2],
                                         m[0], m[1], m[2], comps, amount, threshold);
  else
    k_unsharp<float><<<gr, kT, 0, s>>>(ic, ip[0], ip[1], ip[2], bc, bp[0], bp[1], bp[2], oc, op[0], op[1], op[2],
                                       m[0], m[1], m[2], comps, amount, threshold);
  note_launch("unsharp");
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "unsharp launch: %s", cudaGetErrorString(e));
  return ITKG_SUCCESS;
}

}  // namespace itkg
