// RecursiveGaussianFilter / RecursiveGaussianAxisFilter
// (src/filters/recursive_gaussian.rs): the Young & van Vliet 3rd-order IIR
// approximation of the Gaussian.  The reference converts the whole largest
// region to f64 (P::to_f64), runs on every line along each axis a causal then
// an anticausal pass in place (recursive_gaussian.rs:56-130), and converts the
// requested region back (P::from_f64).  Here:
//   k_rec_load   the largest region -> a dense f64 scratch image
//   k_rec_lines  one thread per line: the causal pass, then the anticausal pass
//   k_rec_store  the requested region -> the output (f32: round to nearest; u8:
//                round half away from zero, clamp to [0, 255], NaN -> 0)
// Reference rounding rounds every product and sum separately in the
// reference's order, bit for bit; FMA rounding uses fused multiply-adds (f64
// throughout either way: an f32 recursion drifts past 1e-5 of the reference
// once sigma reaches a few pixels).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "internal.hpp"
#include "pixel.cuh"

namespace itkg {
namespace {

constexpr int kT = 256;

struct RecGeom {
  int64_t n[3];        // largest region size (1 on missing axes)
  int64_t lo[3];       // largest region index
};

template <typename Tin, typename T>
__global__ void __launch_bounds__(kT) k_rec_load(const char* src, int64_t so0, int64_t so1, int64_t so2,
                                                  int64_t sp0, int64_t sp1, int64_t sp2, RecGeom g, T* d) {
  const int64_t x = (int64_t)blockIdx.x * kT + threadIdx.x;
  if (x >= g.n[0]) return;
  for (int64_t z = blockIdx.z; z < g.n[2]; z += gridDim.z)
    for (int64_t y = blockIdx.y; y < g.n[1]; y += gridDim.y) {
      const char* p = src + (g.lo[0] + x - so0) * sp0 + (g.lo[1] + y - so1) * sp1 + (g.lo[2] + z - so2) * sp2;
      const float v = to_f32(*reinterpret_cast<const Tin*>(p));  // exact for every input type
      d[(z * g.n[1] + y) * g.n[0] + x] = (T)v;
    }
}

// v = B x + a1 y[-1] + a2 y[-2] + a3 y[-3]
template <bool REF>
__device__ __forceinline__ double rec_step(double x, double y1, double y2, double y3, double B, double a1,
                                           double a2, double a3) {
  if constexpr (REF) {
    // (((B x) + a1 y1) + a2 y2) + a3 y3, each product and sum rounded (recursive_gaussian.rs:63)
    double v = __dadd_rn(__dmul_rn(B, x), __dmul_rn(a1, y1));
    v = __dadd_rn(v, __dmul_rn(a2, y2));
    return __dadd_rn(v, __dmul_rn(a3, y3));
  } else {
    return fma(a3, y3, fma(a2, y2, fma(a1, y1, __dmul_rn(B, x))));
  }
}

// One line per thread.  axis 0: lines are rows (stride 1); axis 1: stride n0;
// axis 2: stride n0 n1.
template <typename T, bool REF>
__global__ void __launch_bounds__(kT) k_rec_lines(T* d, RecGeom g, int axis, T B, T a1, T a2, T a3) {
  const int64_t L = (int64_t)blockIdx.x * kT + threadIdx.x;
  const int64_t n0 = g.n[0], n1 = g.n[1], n2 = g.n[2];
  int64_t nlines, base, s, n;
  if (axis == 0) {
    nlines = n1 * n2;
    base = L * n0;
    s = 1;
    n = n0;
  } else if (axis == 1) {
    nlines = n0 * n2;
    base = (L / n0) * n0 * n1 + L % n0;
    s = n0;
    n = n1;
  } else {
    nlines = n0 * n1;
    base = L;
    s = n0 * n1;
    n = n2;
  }
  if (L >= nlines) return;
  T* const p = d + base;
  T y1 = p[0], y2 = y1, y3 = y1;  // steady state of the first sample
  for (int64_t i = 0; i < n; ++i) {
    const T v = rec_step<REF>(p[i * s], y1, y2, y3, B, a1, a2, a3);
    y3 = y2;
    y2 = y1;
    y1 = v;
    p[i * s] = v;
  }
  y1 = p[(n - 1) * s];
  y2 = y1;
  y3 = y1;
  for (int64_t i = n - 1; i >= 0; --i) {
    const T v = rec_step<REF>(p[i * s], y1, y2, y3, B, a1, a2, a3);
    y3 = y2;
    y2 = y1;
    y1 = v;
    p[i * s] = v;
  }
}

__device__ __forceinline__ float out_f32(double v) { return __double2float_rn(v); }
__device__ __forceinline__ uint8_t out_u8_of(double v) {  // round half away from zero, clamp, NaN -> 0
  double r = round(v);
  r = fmin(fmax(r, 0.0), 255.0);
  return (uint8_t)r;
}

template <typename T, int OUT>
__global__ void __launch_bounds__(kT) k_rec_store(const T* d, RecGeom g, int64_t r0, int64_t r1, int64_t r2,
                                                   int64_t m0, int64_t m1, int64_t m2, char* dst, int64_t do0,
                                                   int64_t do1, int64_t do2, int64_t dp0, int64_t dp1, int64_t dp2) {
  const int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x;
  if (i >= m0) return;
  for (int64_t k = blockIdx.z; k < m2; k += gridDim.z)
    for (int64_t j = blockIdx.y; j < m1; j += gridDim.y) {
      const int64_t x = r0 + i, y = r1 + j, z = r2 + k;  // absolute
      const T v = d[((z - g.lo[2]) * g.n[1] + (y - g.lo[1])) * g.n[0] + (x - g.lo[0])];
      char* p = dst + (x - do0) * dp0 + (y - do1) * dp1 + (z - do2) * dp2;
      if (OUT == ITKG_U8) *reinterpret_cast<uint8_t*>(p) = out_u8_of((double)v);
      else *reinterpret_cast<float*>(p) = out_f32(v);
    }
}

// The derivative users (edges.rs:686-950): stencils on the smoothed image `s`
// (a dense image of the requested region, m0 x m1 x m2, in the input's pixel
// type), clamped to that region, in f64 with every operation rounded in the
// reference's order.  kind: 0 gradient magnitude, 1 Laplacian, 2 derivative
// (axis, order), 3 gradient (one f32 component per axis), 4 2-D Hessian
// (f32 components h00, h11, h01).
template <typename Tp>
__device__ __forceinline__ double sval(const Tp* s, int64_t m0, int64_t m1, int64_t x, int64_t y, int64_t z) {
  return (double)s[(z * m1 + y) * m0 + x];
}

template <typename Tp>
__global__ void __launch_bounds__(kT) k_rec_deriv(const Tp* s, int64_t m0, int64_t m1, int64_t m2, int D, int kind,
                                                   int axis, int order, double h0, double h1, double h2, char* dst,
                                                   int64_t dp0, int64_t dp1, int64_t dp2, int out_u8) {
  const int64_t x = (int64_t)blockIdx.x * kT + threadIdx.x;
  if (x >= m0) return;
  const int64_t m[3] = {m0, m1, m2};
  const double h[3] = {h0, h1, h2};
  for (int64_t z = blockIdx.z; z < m2; z += gridDim.z)
    for (int64_t y = blockIdx.y; y < m1; y += gridDim.y) {
      const int64_t p[3] = {x, y, z};
      // s at p with coordinate a moved by off, clamped to the region
      auto get = [&](int a, int off) {
        int64_t q[3] = {p[0], p[1], p[2]};
        q[a] = q[a] + off < 0 ? 0 : (q[a] + off >= m[a] ? m[a] - 1 : q[a] + off);
        return sval(s, m0, m1, q[0], q[1], q[2]);
      };
      auto first = [&](int a) {  // (s[+1] - s[-1]) / (2 h)
        return __ddiv_rn(__dsub_rn(get(a, 1), get(a, -1)), __dmul_rn(2.0, h[a]));
      };
      auto second = [&](int a) {  // ((s[+1] - 2 s[0]) + s[-1]) / (h h)
        return __ddiv_rn(__dadd_rn(__dsub_rn(get(a, 1), __dmul_rn(2.0, get(a, 0))), get(a, -1)),
                         __dmul_rn(h[a], h[a]));
      };
      char* const o = dst + x * dp0 + y * dp1 + z * dp2;
      if (kind <= 2) {
        double v = 0.0;
        if (kind == 0) {
          for (int a = 0; a < D; ++a) {
            const double d = first(a);
            v = __dadd_rn(v, __dmul_rn(d, d));
          }
          v = __dsqrt_rn(v);
        } else if (kind == 1) {
          for (int a = 0; a < D; ++a) v = __dadd_rn(v, second(a));
        } else {
          v = order == 1 ? first(axis) : (order == 2 ? second(axis) : 0.0);
        }
        if (out_u8) *reinterpret_cast<uint8_t*>(o) = out_u8_of(v);
        else *reinterpret_cast<float*>(o) = __double2float_rn(v);
      } else if (kind == 3) {
        for (int a = 0; a < D; ++a) reinterpret_cast<float*>(o)[a] = __double2float_rn(first(a));
      } else {
        const double h00 = second(0), h11 = second(1);
        auto g2 = [&](int dx, int dy) {
          const int64_t xi = x + dx < 0 ? 0 : (x + dx >= m0 ? m0 - 1 : x + dx);
          const int64_t yi = y + dy < 0 ? 0 : (y + dy >= m1 ? m1 - 1 : y + dy);
          return sval(s, m0, m1, xi, yi, z);
        };
        const double num = __dadd_rn(__dsub_rn(__dsub_rn(g2(1, 1), g2(1, -1)), g2(-1, 1)), g2(-1, -1));
        const double h01 = __ddiv_rn(num, __dmul_rn(__dmul_rn(4.0, h0), h1));
        float* const f = reinterpret_cast<float*>(o);
        f[0] = __double2float_rn(h00);
        f[1] = __double2float_rn(h11);
        f[2] = __double2float_rn(h01);
      }
    }
}

// DifferenceOfGaussiansFilter (edges.rs:995-1006): s1 - s2 in f64, converted.
template <typename Tp>
__global__ void __launch_bounds__(kT) k_rec_sub(const Tp* s1, const Tp* s2, int64_t m0, int64_t m1, int64_t m2,
                                                 char* dst, int64_t dp0, int64_t dp1, int64_t dp2, int out_u8) {
  const int64_t x = (int64_t)blockIdx.x * kT + threadIdx.x;
  if (x >= m0) return;
  for (int64_t z = blockIdx.z; z < m2; z += gridDim.z)
    for (int64_t y = blockIdx.y; y < m1; y += gridDim.y) {
      const int64_t i = (z * m1 + y) * m0 + x;
      const double v = __dsub_rn((double)s1[i], (double)s2[i]);
      char* const o = dst + x * dp0 + y * dp1 + z * dp2;
      if (out_u8) *reinterpret_cast<uint8_t*>(o) = out_u8_of(v);
      else *reinterpret_cast<float*>(o) = __double2float_rn(v);
    }
}

// ZeroCrossingFilter (edges.rs:480-514) over the Laplacian image `l` (dense,
// the requested region): 1 where center * neighbour < 0 (f64; exact for f32
// and u8 values) for a neighbour along some axis, clamped to the region;
// else 0, in the pixel type.
template <typename Tp>
__global__ void __launch_bounds__(kT) k_rec_zero(const Tp* l, int64_t m0, int64_t m1, int64_t m2, int D, char* dst,
                                                  int64_t dp0, int64_t dp1, int64_t dp2, int out_u8) {
  const int64_t x = (int64_t)blockIdx.x * kT + threadIdx.x;
  if (x >= m0) return;
  const int64_t m[3] = {m0, m1, m2};
  for (int64_t z = blockIdx.z; z < m2; z += gridDim.z)
    for (int64_t y = blockIdx.y; y < m1; y += gridDim.y) {
      const int64_t p[3] = {x, y, z};
      const double c = sval(l, m0, m1, x, y, z);
      bool zc = false;
      for (int a = 0; a < D && !zc; ++a)
        for (int off = -1; off <= 1 && !zc; off += 2) {
          int64_t q[3] = {p[0], p[1], p[2]};
          q[a] = q[a] + off < 0 ? 0 : (q[a] + off >= m[a] ? m[a] - 1 : q[a] + off);
          zc = __dmul_rn(c, sval(l, m0, m1, q[0], q[1], q[2])) < 0.0;
        }
      char* const o = dst + x * dp0 + y * dp1 + z * dp2;
      if (out_u8) *reinterpret_cast<uint8_t*>(o) = zc ? 1 : 0;
      else *reinterpret_cast<float*>(o) = zc ? 1.0f : 0.0f;
    }
}

dim3 grid3(int64_t n0, int64_t n1, int64_t n2) {
  return dim3((unsigned)((n0 + kT - 1) / kT), (unsigned)std::min<int64_t>(std::max<int64_t>(n1, 1), 65535),
              (unsigned)std::min<int64_t>(std::max<int64_t>(n2, 1), 65535));
}

}  // namespace

// Host-side Young & van Vliet coefficients (recursive_gaussian.rs:33-49), f64,
// every operation in the reference's order.
void yvv_coeffs(double sigma, double out[4]) {
  if (!(sigma > 0.5)) sigma = 0.5;  // sigma.max(0.5); f64::max takes 0.5 over NaN
  const double q = sigma >= 2.5 ? 0.98711 * sigma - 0.96330 : 3.97156 - 4.14554 * std::sqrt(1.0 - 0.26891 * sigma);
  const double q2 = q * q;
  const double q3 = q2 * q;
  const double b0 = 1.57825 + 2.44413 * q + 1.4281 * q2 + 0.422205 * q3;
  const double b1 = 2.44413 * q + 2.85619 * q2 + 1.26661 * q3;
  const double b2 = -(1.4281 * q2 + 1.26661 * q3);
  const double b3 = 0.422205 * q3;
  out[0] = 1.0 - (b1 + b2 + b3) / b0;
  out[1] = b1 / b0;
  out[2] = b2 / b0;
  out[3] = b3 / b0;
}

itkg_status launch_recursive(const itkg_image& in, const itkg_region& largest, const itkg_region& requested,
                             double sigma, int axis, int rounding, const itkg_image& out, void* stream) {
  const int D = in.dim;
  const bool ref = rounding == ITKG_ROUND_REFERENCE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  RecGeom g;
  for (int d = 0; d < 3; ++d) {
    g.n[d] = d < D ? (int64_t)largest.size[d] : 1;
    g.lo[d] = d < D ? largest.index[d] : 0;
  }
  const int64_t total = g.n[0] * g.n[1] * g.n[2];
  if (total == 0) return ITKG_SUCCESS;
  double* buf = nullptr;
  {
    const itkg_status sa = scratch_alloc(reinterpret_cast<void**>(&buf), (size_t)total * sizeof(double), stream);
    if (sa != ITKG_SUCCESS) return sa;
  }
  int64_t so[3] = {0, 0, 0}, sp[3] = {0, 0, 0}, dof[3] = {0, 0, 0}, dp[3] = {0, 0, 0};
  for (int d = 0; d < 3; ++d) {
    so[d] = d < D ? in.region.index[d] : 0;
    sp[d] = in.pitch[d];
    dof[d] = d < D ? out.region.index[d] : 0;
    dp[d] = out.pitch[d];
  }
  const char* src = static_cast<const char*>(in.data);
  itkg_status st = ITKG_SUCCESS;
  {  // load the largest region as f64
    const dim3 gr = grid3(g.n[0], g.n[1], g.n[2]);
    switch (in.dtype) {
      case ITKG_F32: k_rec_load<float, double><<<gr, kT, 0, s>>>(src, so[0], so[1], so[2], sp[0], sp[1], sp[2], g, buf); break;
      case ITKG_I16: k_rec_load<int16_t, double><<<gr, kT, 0, s>>>(src, so[0], so[1], so[2], sp[0], sp[1], sp[2], g, buf); break;
      case ITKG_U8: k_rec_load<uint8_t, double><<<gr, kT, 0, s>>>(src, so[0], so[1], so[2], sp[0], sp[1], sp[2], g, buf); break;
      case ITKG_BF16: k_rec_load<__nv_bfloat16, double><<<gr, kT, 0, s>>>(src, so[0], so[1], so[2], sp[0], sp[1], sp[2], g, buf); break;
      case ITKG_F16: k_rec_load<__half, double><<<gr, kT, 0, s>>>(src, so[0], so[1], so[2], sp[0], sp[1], sp[2], g, buf); break;
      default: st = set_error(ITKG_ERROR_UNSUPPORTED, "input dtype %d not supported", in.dtype);
    }
    if (st == ITKG_SUCCESS) note_launch("recursive_load");
  }
  // lines, axis by axis (lines of length <= 1 are left alone, recursive_gaussian.rs:98-100)
  for (int a = 0; a < D && st == ITKG_SUCCESS; ++a) {
    if (axis >= 0 && a != axis) continue;
    if (g.n[a] <= 1) continue;
    double c[4];
    yvv_coeffs(sigma / in.spacing[a], c);
    const unsigned blocks = (unsigned)((total / g.n[a] + kT - 1) / kT);
    if (ref) k_rec_lines<double, true><<<blocks, kT, 0, s>>>(buf, g, a, c[0], c[1], c[2], c[3]);
    else k_rec_lines<double, false><<<blocks, kT, 0, s>>>(buf, g, a, c[0], c[1], c[2], c[3]);
    note_launch(ref ? "recursive_lines_f64" : "recursive_lines_f64_fma");
  }
  if (st == ITKG_SUCCESS) {  // the requested region, converted
    int64_t r[3] = {0, 0, 0}, m[3] = {1, 1, 1};
    for (int d = 0; d < D; ++d) r[d] = requested.index[d], m[d] = (int64_t)requested.size[d];
    const dim3 gr = grid3(m[0], m[1], m[2]);
    char* dst = static_cast<char*>(out.data);
    if (out.dtype == ITKG_U8)
      k_rec_store<double, ITKG_U8><<<gr, kT, 0, s>>>(buf, g, r[0], r[1], r[2], m[0], m[1], m[2], dst, dof[0], dof[1],
                                                     dof[2], dp[0], dp[1], dp[2]);
    else
      k_rec_store<double, ITKG_F32><<<gr, kT, 0, s>>>(buf, g, r[0], r[1], r[2], m[0], m[1], m[2], dst, dof[0], dof[1],
                                                      dof[2], dp[0], dp[1], dp[2]);
    note_launch("recursive_store");
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) st = set_error(ITKG_ERROR_CUDA, "recursive gaussian launch: %s", cudaGetErrorString(e));
  }
  scratch_free(buf, stream);
  if (st == ITKG_SUCCESS) set_last_kernel(ref ? "recursive_lines_f64" : "recursive_lines_f64_fma");
  return st;
}

itkg_status launch_recursive_derivative(const itkg_image& in, const itkg_region& largest,
                                        const itkg_region& requested, double sigma, double sigma2, int kind,
                                        int axis, int order, int rounding, const itkg_image& out, void* stream) {
  const int D = in.dim;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the smoothed image: RecursiveGaussianFilter::generate_region(requested) in the input's pixel type
  itkg_image sm;
  std::memset(&sm, 0, sizeof sm);
  sm.dim = D;
  sm.dtype = in.dtype;
  sm.components = 1;
  sm.location = ITKG_DEVICE;
  sm.region = requested;
  int64_t m[3] = {1, 1, 1};
  for (int d = 0; d < D; ++d) m[d] = (int64_t)requested.size[d], sm.spacing[d] = in.spacing[d];
  const int64_t esz = in.dtype == ITKG_U8 ? 1 : 4;
  sm.pitch[0] = esz;
  sm.pitch[1] = esz * m[0];
  sm.pitch[2] = esz * m[0] * m[1];
  const bool dog = kind == 5;
  const size_t sm_bytes = (size_t)(esz * m[0] * m[1] * m[2]);
  void* buf = nullptr;
  void* buf2 = nullptr;
  {
    itkg_status sa = scratch_alloc(&buf, sm_bytes, stream);
    if (sa == ITKG_SUCCESS && dog) sa = scratch_alloc(&buf2, sm_bytes, stream);
    if (sa != ITKG_SUCCESS) {
      scratch_free(buf, stream);
      return sa;
    }
  }
  sm.data = buf;
  itkg_status st = launch_recursive(in, largest, requested, sigma, -1, rounding, sm, stream);
  if (st == ITKG_SUCCESS && dog) {  // the second smoothing, then s1 - s2
    itkg_image sm2 = sm;
    sm2.data = buf2;
    st = launch_recursive(in, largest, requested, sigma2, -1, rounding, sm2, stream);
    if (st == ITKG_SUCCESS) {
      int64_t dp[3] = {0, 0, 0};
      for (int d = 0; d < 3; ++d) dp[d] = d < D ? out.pitch[d] : 0;
      char* dst = static_cast<char*>(out.data);
      for (int d = 0; d < D; ++d) dst += (requested.index[d] - out.region.index[d]) * out.pitch[d];
      const dim3 gr = grid3(m[0], m[1], m[2]);
      const int u8 = out.dtype == ITKG_U8 ? 1 : 0;
      if (in.dtype == ITKG_U8)
        k_rec_sub<uint8_t><<<gr, kT, 0, s>>>(static_cast<const uint8_t*>(buf), static_cast<const uint8_t*>(buf2), m[0],
                                             m[1], m[2], dst, dp[0], dp[1], dp[2], u8);
      else
        k_rec_sub<float><<<gr, kT, 0, s>>>(static_cast<const float*>(buf), static_cast<const float*>(buf2), m[0], m[1],
                                           m[2], dst, dp[0], dp[1], dp[2], u8);
      note_launch("recursive_difference");
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) st = set_error(ITKG_ERROR_CUDA, "recursive difference launch: %s", cudaGetErrorString(e));
    }
    scratch_free(buf, stream);
    scratch_free(buf2, stream);
    if (st == ITKG_SUCCESS) set_last_kernel("recursive_difference");
    return st;
  }
  if (st == ITKG_SUCCESS) {
    double h[3] = {1.0, 1.0, 1.0};
    for (int d = 0; d < D; ++d) h[d] = in.spacing[d];
    int64_t dp[3] = {0, 0, 0};
    for (int d = 0; d < 3; ++d) dp[d] = d < D ? out.pitch[d] : 0;
    char* dst = static_cast<char*>(out.data);
    for (int d = 0; d < D; ++d) dst += (requested.index[d] - out.region.index[d]) * out.pitch[d];
    const dim3 gr = grid3(m[0], m[1], m[2]);
    const int u8 = out.dtype == ITKG_U8 ? 1 : 0;
    // ZeroCrossingBasedEdgeDetectionFilter (edges.rs:1045-1052): the Laplacian
    // (kind 1) into a dense scratch image in the pixel type, then zero crossings
    const bool zero = kind == 6;
    void* lap = nullptr;
    if (zero) st = scratch_alloc(&lap, sm_bytes, stream);
    if (st == ITKG_SUCCESS) {
      char* const d1 = zero ? static_cast<char*>(lap) : dst;
      const int64_t p1[3] = {zero ? esz : dp[0], zero ? esz * m[0] : dp[1], zero ? esz * m[0] * m[1] : dp[2]};
      const int k1 = zero ? 1 : kind;
      if (in.dtype == ITKG_U8)
        k_rec_deriv<uint8_t><<<gr, kT, 0, s>>>(static_cast<const uint8_t*>(buf), m[0], m[1], m[2], D, k1, axis, order,
                                               h[0], h[1], h[2], d1, p1[0], p1[1], p1[2], u8);
      else
        k_rec_deriv<float><<<gr, kT, 0, s>>>(static_cast<const float*>(buf), m[0], m[1], m[2], D, k1, axis, order,
                                             h[0], h[1], h[2], d1, p1[0], p1[1], p1[2], u8);
      note_launch("recursive_derivative");
      if (zero) {
        if (in.dtype == ITKG_U8)
          k_rec_zero<uint8_t><<<gr, kT, 0, s>>>(static_cast<const uint8_t*>(lap), m[0], m[1], m[2], D, dst, dp[0],
                                                dp[1], dp[2], u8);
        else
          k_rec_zero<float><<<gr, kT, 0, s>>>(static_cast<const float*>(lap), m[0], m[1], m[2], D, dst, dp[0], dp[1],
                                              dp[2], u8);
        note_launch("recursive_zero_crossing");
      }
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) st = set_error(ITKG_ERROR_CUDA, "recursive derivative launch: %s", cudaGetErrorString(e));
    }
    scratch_free(lap, stream);
  }
  scratch_free(buf, stream);
  if (st == ITKG_SUCCESS) set_last_kernel(kind == 6 ? "recursive_zero_crossing" : "recursive_derivative");
  return st;
}

}  // namespace itkg
