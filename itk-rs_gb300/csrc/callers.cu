// BSplineDownsampleFilter's subsampling (src/filters/spatial.rs:1155-1166):
// output voxel i of the downsampled region takes the smoothed voxel at
// index + 2 (i - index) on every axis.  Pixels are copied as bytes.
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.hpp"

namespace itkg {
namespace {

constexpr int kT = 256;

__global__ void __launch_bounds__(kT) k_subsample2(const char* src, int64_t sp0, int64_t sp1, int64_t sp2, char* dst,
                                                    int64_t dp0, int64_t dp1, int64_t dp2, int64_t m0, int64_t m1,
                                                    int64_t m2, int elem) {
  const int64_t x = (int64_t)blockIdx.x * kT + threadIdx.x;
  if (x >= m0) return;
  for (int64_t z = blockIdx.z; z < m2; z += gridDim.z)
    for (int64_t y = blockIdx.y; y < m1; y += gridDim.y) {
      const char* s = src + 2 * (x * sp0 + y * sp1 + z * sp2);
      char* d = dst + x * dp0 + y * dp1 + z * dp2;
      if (elem == 4) {
        *reinterpret_cast<uint32_t*>(d) = *reinterpret_cast<const uint32_t*>(s);
      } else {
        for (int b = 0; b < elem; ++b) d[b] = s[b];
      }
    }
}

}  // namespace

// src: the smoothed voxel at the region's index, dst: the output voxel there;
// pitches in bytes; m: the downsampled size (unused axes 1); elem: pixel bytes.
itkg_status launch_subsample2(const void* src, const int64_t* sp, void* dst, const int64_t* dp, const int64_t* m,
                              int elem, void* stream) {
  if (m[0] * m[1] * m[2] == 0) return ITKG_SUCCESS;
  const dim3 gr((unsigned)((m[0] + kT - 1) / kT), (unsigned)std::min<int64_t>(m[1], 65535),
                (unsigned)std::min<int64_t>(m[2], 65535));
  k_subsample2<<<gr, kT, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const char*>(src), sp[0], sp[1], sp[2],
                                                                 static_cast<char*>(dst), dp[0], dp[1], dp[2], m[0],
                                                                 m[1], m[2], elem);
  note_launch("subsample2");
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "subsample launch: %s", cudaGetErrorString(e));
  return ITKG_SUCCESS;
}

}  // namespace itkg
