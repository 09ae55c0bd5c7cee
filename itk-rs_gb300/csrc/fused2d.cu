// Fused 2-D Gaussian forward: both passes of GaussianFilter::generate_region
// (src/filters/gaussian.rs:74-88) for Image<f32, 2> and
// Image<VecPixel<f32, 3>, 2> in one kernel.
//
// A CTA owns TXW output columns of the requested region and a range of output
// rows [y0, y1); it marches the input rows j = y0 - RY .. y1 - 1 + RY (clamped
// to the image, the reference's clamp-to-edge on axis 1, conv.rs:31-33):
//   1. the row segment (TXW + 2XA pixels, clamped on x) is gathered by
//      cp.async into a ring of S row stages in shared memory, de-interleaving
//      the components into C planar rows;
//   2. x pass: each thread filters 4 consecutive pixels of one component from
//      a register window;
//   3. y pass, "push" form: the thread adds w[k] * v to its ring of KY
//      accumulators (pairs of pixels in f32x2 registers); the ring slot is a
//      compile-time function of j mod KY.  Output row j - RY pops out after
//      row j has been pushed and is stored with the component interleaving of
//      the output image.
// Reference rounding: scalar acc = acc + x * w in ascending tap order from zero
// per pass, f32 intermediate -- bit-identical to the reference.  FMA rounding:
// packed f32x2 FMAs.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <mutex>
#include <vector>

#include "f32x2.cuh"
#include "internal.hpp"
#include "pixel.cuh"

namespace itkg {
namespace {

constexpr int kMax2DR = 12;
constexpr int kMax2DK = 2 * kMax2DR + 1;

struct Fused2DArgs {
  const char* src;
  char* dst;
  int64_t src_pitch[2];  // bytes (pixel, row)
  int64_t dst_pitch[2];
  int32_t src_origin[2];
  int32_t dst_origin[2];
  int32_t req_lo[2], req_hi[2];  // inclusive
  int32_t lo[2], hi[2];          // gather bounds (image within buffer), inclusive
  int32_t ntx;                   // tiles along x
  int32_t out_dtype;
  int32_t out_esz;               // bytes of one output component
  int32_t pad_;
  int64_t units;                 // slices * ntx * requested rows
  int64_t slice_units;           // ntx * requested rows
  int64_t src_slice, dst_slice;  // bytes between slices (a 3-D image with a 1-tap z kernel)
  float wx[kMax2DK], wy[kMax2DK];
  f2_t wx2[kMax2DK], wy2[kMax2DK];
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cpa4(uint32_t s, const void* g) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(g) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cpa_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
__device__ __forceinline__ int clampi2(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

template <int RX, int RY, int C>
struct Cfg2 {
  static constexpr int KX = 2 * RX + 1, KY = 2 * RY + 1;
  static constexpr int TPC = 32;               // threads (one warp) per component plane
  static constexpr int NT = TPC * C;
  static constexpr int MXP = 4;                // pixels per thread
  static constexpr int TXW = TPC * MXP;        // output columns per tile
  static constexpr int XA = (RX + 3) / 4 * 4;  // halo rounded to 16 bytes
  static constexpr int PW = TXW + 2 * XA;      // staged plane row width (floats)
  static constexpr int OFF = (XA - RX) % 4;
  static constexpr int WB = XA - RX - OFF;
  static constexpr int WIN = (MXP + 2 * RX + OFF + 3) / 4 * 4;
  static constexpr int S = 4;                  // rows in flight
  static constexpr int ROW = C * PW;           // floats per staged row
  static constexpr int NLD = (ROW + NT - 1) / NT;
  static constexpr size_t SMEM = sizeof(float) * (size_t)S * ROW;
  static_assert(WB + TXW - MXP + WIN <= PW, "window inside the staged row");
};

template <int P, int KY, bool REF>
__device__ __forceinline__ void push2(f2_t (&acc)[2][KY], const f2_t (&xv)[2], const Fused2DArgs& a,
                                      f2_t (&done)[2]) {
#pragma unroll
  for (int k = 0; k < KY; ++k) {
    const int slot = (P - k + KY) % KY;
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      if constexpr (REF) {
        float a0, a1, v0, v1;
        unpack2(acc[m][slot], a0, a1);
        unpack2(xv[m], v0, v1);
        acc[m][slot] = pack2(__fadd_rn(a0, __fmul_rn(v0, a.wy[k])), __fadd_rn(a1, __fmul_rn(v1, a.wy[k])));
      } else {
        acc[m][slot] = fma2(xv[m], a.wy2[k], acc[m][slot]);
      }
    }
  }
  constexpr int D = (P + 1) % KY;
#pragma unroll
  for (int m = 0; m < 2; ++m) {
    done[m] = acc[m][D];
    acc[m][D] = 0ull;
  }
}

#define ITKG_PUSH2(N) \
  case N:             \
    if constexpr (N < KY) push2<N, KY, REF>(acc, xv, a, done); \
    break;

template <int RX, int RY, int C, bool REF>
__global__ void __launch_bounds__(Cfg2<RX, RY, C>::NT) k_fused2d(const Fused2DArgs a) {
  using G = Cfg2<RX, RY, C>;
  constexpr int KX = G::KX, KY = G::KY, TPC = G::TPC, MXP = G::MXP, TXW = G::TXW, XA = G::XA,
                PW = G::PW, OFF = G::OFF, WB = G::WB, WIN = G::WIN, S = G::S, ROW = G::ROW,
                NLD = G::NLD, NT = G::NT;
  extern __shared__ __align__(16) float rows[];
  const int tid = threadIdx.x;
  const int comp = tid / TPC, lt = tid % TPC;
  const int nyr = a.req_hi[1] - a.req_lo[1] + 1;
  const int64_t u_begin = a.units * blockIdx.x / gridDim.x;
  const int64_t u_end = a.units * (blockIdx.x + 1) / gridDim.x;
  const uint32_t sbase = smem_addr(rows);

  for (int64_t u = u_begin; u < u_end;) {
    const int64_t zq = u / a.slice_units;
    const int64_t uu = u - zq * a.slice_units;
    const char* const srcz = a.src + zq * a.src_slice;
    char* const dstz = a.dst + zq * a.dst_slice;
    const int64_t tile = uu / nyr;
    const int ys = (int)(uu % nyr);
    const int64_t yrem = ys + (u_end - u);
    const int ye = yrem < nyr ? (int)yrem : nyr;
    u += ye - ys;
    const int y0 = a.req_lo[1] + ys, y1 = a.req_lo[1] + ye;
    const int tx0 = a.req_lo[0] + (int)tile * TXW;
    const int gx0 = tx0 - XA;

    // gather offsets (pixel x clamped; component c of pixel -> plane c)
    int32_t goff[NLD];
    uint32_t soff[NLD];
#pragma unroll
    for (int i = 0; i < NLD; ++i) {
      const int e = tid + i * NT;
      const int c = e / PW, col = e % PW;
      const int gx = clampi2(gx0 + col, a.lo[0], a.hi[0]);
      goff[i] = (int32_t)((gx - a.src_origin[0]) * a.src_pitch[0] + c * 4);
      soff[i] = (uint32_t)(e * 4);
    }
    auto issue = [&](int row, int st) {
      const char* base = srcz + (int64_t)(row - a.src_origin[1]) * a.src_pitch[1];
      const uint32_t sb = sbase + (uint32_t)(st * ROW * 4);
#pragma unroll
      for (int i = 0; i < NLD; ++i)
        if (i < NLD - 1 || tid + i * NT < ROW) cpa4(sb + soff[i], base + goff[i]);
      cpa_commit();
    };
    const int jb = y0 - RY, je = y1 - 1 + RY;
    const int r_first = max(jb, a.lo[1]), r_last = min(je, a.hi[1]);
    for (int q = 0; q < S - 1; ++q) {
      if (r_first + q <= r_last) issue(r_first + q, q);
      else cpa_commit();
    }

    f2_t acc[2][KY];
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
      for (int q = 0; q < KY; ++q) acc[m][q] = 0ull;
    f2_t xv[2] = {0ull, 0ull};

    const int px0 = tx0 + lt * MXP;  // first output pixel of this thread
    int npx = a.req_hi[0] - px0 + 1;
    npx = npx < 0 ? 0 : (npx > MXP ? MXP : npx);
    char* const obase = dstz + (int64_t)(px0 - a.dst_origin[0]) * a.dst_pitch[0] + comp * a.out_esz;
    int prev = INT_MIN, cons = 0, p = 0;
    for (int j = jb; j <= je; ++j) {
      const int rr = clampi2(j, a.lo[1], a.hi[1]);
      if (rr != prev) {
        prev = rr;
        cpa_wait<S - 2>();
        __syncthreads();  // row rr visible; stage of the previous row free
        {
          const int rn = r_first + cons + S - 1;
          if (rn <= r_last) issue(rn, (cons + S - 1) % S);
          else cpa_commit();
        }
        const float* plane = rows + (cons % S) * ROW + comp * PW;
        ++cons;
        float v[WIN];
        const float* src = plane + lt * MXP + WB;
#pragma unroll
        for (int q = 0; q < WIN / 4; ++q) {
          const float4 f = *reinterpret_cast<const float4*>(src + 4 * q);
          v[4 * q] = f.x, v[4 * q + 1] = f.y, v[4 * q + 2] = f.z, v[4 * q + 3] = f.w;
        }
        if constexpr (REF) {
          float o[MXP];
#pragma unroll
          for (int m = 0; m < MXP; ++m) {
            float ax = 0.0f;
#pragma unroll
            for (int k = 0; k < KX; ++k) ax = tap<true>(ax, v[m + k + OFF], a.wx[k]);
            o[m] = ax;
          }
          xv[0] = pack2(o[0], o[1]);
          xv[1] = pack2(o[2], o[3]);
        } else {
          f2_t E[WIN / 2], O[WIN / 2 - 1];
#pragma unroll
          for (int i = 0; i < WIN / 2; ++i) E[i] = pack2(v[2 * i], v[2 * i + 1]);
#pragma unroll
          for (int i = 0; i < WIN / 2 - 1; ++i) O[i] = pack2(v[2 * i + 1], v[2 * i + 2]);
#pragma unroll
          for (int m = 0; m < 2; ++m) {
            f2_t ax = 0ull;
#pragma unroll
            for (int k = 0; k < KX; ++k) {
              const int q = 2 * m + k + OFF;
              ax = fma2((q & 1) ? O[(q - 1) / 2] : E[q / 2], a.wx2[k], ax);
            }
            xv[m] = ax;
          }
        }
      }
      f2_t done[2];
      switch (p) {
        ITKG_PUSH2(0) ITKG_PUSH2(1) ITKG_PUSH2(2) ITKG_PUSH2(3) ITKG_PUSH2(4) ITKG_PUSH2(5)
        ITKG_PUSH2(6) ITKG_PUSH2(7) ITKG_PUSH2(8) ITKG_PUSH2(9) ITKG_PUSH2(10) ITKG_PUSH2(11)
        ITKG_PUSH2(12) ITKG_PUSH2(13) ITKG_PUSH2(14) ITKG_PUSH2(15) ITKG_PUSH2(16) ITKG_PUSH2(17)
        ITKG_PUSH2(18) ITKG_PUSH2(19) ITKG_PUSH2(20) ITKG_PUSH2(21) ITKG_PUSH2(22) ITKG_PUSH2(23)
        ITKG_PUSH2(24)
        default: break;
      }
      p = p + 1 == KY ? 0 : p + 1;
      const int y = j - RY;
      if (y >= y0 && npx > 0) {
        float vals[4];
        unpack2(done[0], vals[0], vals[1]);
        unpack2(done[1], vals[2], vals[3]);
        char* orow = obase + (int64_t)(y - a.dst_origin[1]) * a.dst_pitch[1];
#pragma unroll
        for (int m = 0; m < MXP; ++m) {
          if (m >= npx) break;
          char* q = orow + m * a.dst_pitch[0];
          switch (a.out_dtype) {
            case ITKG_F32: *reinterpret_cast<float*>(q) = vals[m]; break;
            case ITKG_BF16: *reinterpret_cast<__nv_bfloat16*>(q) = from_f32<__nv_bfloat16>(vals[m]); break;
            case ITKG_F16: *reinterpret_cast<__half*>(q) = from_f32<__half>(vals[m]); break;
            default: *reinterpret_cast<uint8_t*>(q) = from_f32<uint8_t>(vals[m]); break;
          }
        }
      }
    }
    cpa_wait<0>();
    __syncthreads();
  }
}

using Fn2 = void (*)(const Fused2DArgs);
struct Entry2 {
  int r, comps;
  Fn2 fn[2];  // [ref]
  size_t smem;
  int nt, txw, ky;
};

template <int R, int C>
Entry2 make2() {
  using G = Cfg2<R, R, C>;
  return Entry2{R, C, {k_fused2d<R, R, C, false>, k_fused2d<R, R, C, true>}, G::SMEM, G::NT, G::TXW, G::KY};
}

const Entry2 kTable2[] = {
    make2<1, 1>(), make2<2, 1>(), make2<3, 1>(), make2<4, 1>(), make2<5, 1>(), make2<6, 1>(),
    make2<7, 1>(), make2<8, 1>(), make2<1, 3>(), make2<2, 3>(), make2<3, 3>(), make2<4, 3>(),
    make2<5, 3>(), make2<6, 3>(), make2<7, 3>(), make2<8, 3>(), make2<9, 1>(), make2<10, 1>(),
    make2<11, 1>(), make2<12, 1>(), make2<9, 3>(), make2<10, 3>(), make2<11, 3>(), make2<12, 3>(),
};

struct Occ2 {
  Fn2 fn;
  int dev, blocks;
};
std::mutex g_occ2_mu;
std::vector<Occ2> g_occ2;

itkg_status resident2(const Entry2& e, Fn2 fn, int* out) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(err));
  {
    std::lock_guard<std::mutex> lk(g_occ2_mu);
    for (const Occ2& o : g_occ2)
      if (o.fn == fn && o.dev == dev) {
        *out = o.blocks;
        return ITKG_SUCCESS;
      }
  }
  err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e.smem);
  if (err != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(err));
  int per_sm = 0, sms = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, e.nt, e.smem);
  if (err != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "occupancy: %s", cudaGetErrorString(err));
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  std::lock_guard<std::mutex> lk(g_occ2_mu);
  g_occ2.push_back({fn, dev, std::max(1, per_sm) * sms});
  *out = g_occ2.back().blocks;
  return ITKG_SUCCESS;
}

bool fits32(int64_t v) { return v >= INT_MIN && v <= INT_MAX; }

}  // namespace

itkg_status launch_fused2d(const FusedGeom& g, const float* const w[kMaxDim], void* stream, bool dry_run) {
  // 2-D, or 3-D with the 1-tap kernel [1] on z (each slice filtered alone)
  const bool slices = g.dim == 3 && g.radius[2] == 0 && w[2] && w[2][0] == 1.0f;
  if (g.u8pix) return ITKG_ERROR_UNSUPPORTED;
  {
    // The tile kernel for launches of up to 6 M output floats (measured on
    // 64^2 .. 4096^2 images, 1 and 3 components, sigma 1.5 and 4: it is up to
    // 2x faster there, where the row-marching kernel waits for its rows one
    // after another); the row-marching kernel beyond, where the tile halos
    // (up to 1.75x the x-pass work) cost more than its waits.
    const int force = kernel2d_override();
    const int64_t floats = g.req_size[0] * g.req_size[1] * (slices ? g.req_size[2] : 1) * g.comps;
    if (force == 1 || (force == 0 && floats <= (6ll << 20))) {
      const itkg_status st = launch_tile2d(g, w, stream, dry_run);
      if (st != ITKG_ERROR_UNSUPPORTED || force == 1) return st;
    }
  }
  if ((g.dim != 2 && !slices) || g.in_dtype != ITKG_F32 || g.out_dtype == ITKG_I16) return ITKG_ERROR_UNSUPPORTED;
  if (g.radius[0] != g.radius[1] || g.radius[0] < 1) return ITKG_ERROR_UNSUPPORTED;
  const Entry2* e = nullptr;
  for (const Entry2& t : kTable2)
    if (t.r == g.radius[0] && t.comps == g.comps) e = &t;
  if (!e) return ITKG_ERROR_UNSUPPORTED;
  for (int d = 0; d < 2; ++d)
    if (!fits32(g.lo[d]) || !fits32(g.hi[d]) || !fits32(g.src_origin[d]) || !fits32(g.dst_origin[d]) ||
        !fits32(g.req_index[d] + g.req_size[d]) || !fits32(g.req_index[d] - 64))
      return ITKG_ERROR_UNSUPPORTED;
  if (!fits32((g.hi[0] - g.src_origin[0] + 1) * g.src_pitch[0])) return ITKG_ERROR_UNSUPPORTED;
  if (g.src_pitch[0] != 4 * g.comps || ((uintptr_t)g.src & 3) || (g.src_pitch[1] & 3) ||
      (slices && (g.src_pitch[2] & 3)))
    return ITKG_ERROR_UNSUPPORTED;
  if (dry_run) return ITKG_SUCCESS;

  Fused2DArgs a;
  std::memset(&a, 0, sizeof a);
  a.src = static_cast<const char*>(g.src);
  a.dst = static_cast<char*>(g.dst);
  int64_t nz = 1;
  if (slices) {  // start at the first requested slice
    nz = g.req_size[2];
    a.src += (g.req_index[2] - g.src_origin[2]) * g.src_pitch[2];
    a.dst += (g.req_index[2] - g.dst_origin[2]) * g.dst_pitch[2];
    a.src_slice = g.src_pitch[2];
    a.dst_slice = g.dst_pitch[2];
  }
  for (int d = 0; d < 2; ++d) {
    a.src_pitch[d] = g.src_pitch[d];
    a.dst_pitch[d] = g.dst_pitch[d];
    a.src_origin[d] = (int32_t)g.src_origin[d];
    a.dst_origin[d] = (int32_t)g.dst_origin[d];
    a.req_lo[d] = (int32_t)g.req_index[d];
    a.req_hi[d] = (int32_t)(g.req_index[d] + g.req_size[d] - 1);
    // gather bounds: image bounds within the input buffer (see fused.cu)
    a.lo[d] = (int32_t)std::max<int64_t>(g.lo[d], g.src_origin[d]);
    a.hi[d] = (int32_t)std::min<int64_t>(g.hi[d], g.src_origin[d] + g.src_size[d] - 1);
  }
  a.ntx = (int32_t)((g.req_size[0] + e->txw - 1) / e->txw);
  a.slice_units = (int64_t)a.ntx * g.req_size[1];
  a.units = a.slice_units * nz;
  a.out_dtype = g.out_dtype;
  a.out_esz = dtype_size(g.out_dtype);
  for (int k = 0; k < 2 * e->r + 1; ++k) {
    a.wx[k] = w[0][k];
    a.wy[k] = w[1][k];
    a.wx2[k] = splat2_host(w[0][k]);
    a.wy2[k] = splat2_host(w[1][k]);
  }
  const bool ref = g.rounding == ITKG_ROUND_REFERENCE;
  Fn2 fn = e->fn[ref ? 1 : 0];
  int resident = 0;
  {
    const itkg_status st = resident2(*e, fn, &resident);
    if (st != ITKG_SUCCESS) return st;
  }
  // Rows per CTA: as few as fill half the SMs' thread slots.  Small images are
  // latency-bound, so short row runs (and their extra halo rows) win; large
  // images get long runs over a single resident wave.
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t target = std::max<int64_t>(1, (int64_t)sms * (1024 / e->nt));
  const int64_t grid = std::min<int64_t>({resident, target, a.units});
  fn<<<(unsigned)grid, e->nt, e->smem, static_cast<cudaStream_t>(stream)>>>(a);
  note_launch(ref ? "fused2d_f32_ref" : "fused2d_f32_fma");
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "fused2d launch: %s", cudaGetErrorString(err));
  return ITKG_SUCCESS;
}

}  // namespace itkg
