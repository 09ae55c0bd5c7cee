// Fused 3-D Gaussian forward: all three separable passes of
// GaussianFilter::generate_region (src/filters/gaussian.rs:74-88) in one
// kernel, so each input voxel is read from HBM once and each output voxel is
// written once.
//
// Decomposition.  A CTA owns an output tile of TX x TY columns (x, y) and a
// range of output slices [z0, z1).  It marches through the input slices
// j = z0 - RZ .. z1 - 1 + RZ (clamped to the image on z, which is the
// reference's clamp-to-edge on axis 2, conv.rs:31-33):
//   1. the (TX + 2RX) x (TY + 2RY) input tile of slice j is staged in shared
//      memory by cp.async, S slices ahead; x and y coordinates are clamped to
//      the image bounds as the tile is gathered, so the halo already holds the
//      reference's edge replication;
//   2. x pass: shared tile -> shared x-filtered tile (TY + 2RY rows);
//   3. y pass: each thread filters MY consecutive rows of one column from a
//      register window;
//   4. z pass, "push" form: slice j contributes w[k] * v to the outputs
//      z = j + RZ - k; each thread keeps a ring of KZ accumulators per owned
//      column in registers (rows paired into f32x2 registers), the ring slot
//      being a compile-time function of the phase j mod KZ, selected by a
//      switch.  The accumulator of output z receives its taps in ascending k
//      (ascending j), starting from zero, so with reference rounding the
//      result is bit-identical to the reference's sequence
//      acc = 0; acc = acc + x * w (conv.rs:26-36); the intermediates of every
//      pass are f32 values exactly as the reference stores them.
// Slices clamped at the z ends are filtered once and pushed repeatedly.
//
// Work balance.  The (tile, z) units of the request are split evenly over a
// grid of (SMs x resident CTAs) CTAs; a CTA's share is one or two z-segments.
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

constexpr int kMaxFusedR = 8;
constexpr int kMaxFusedK = 2 * kMaxFusedR + 1;

struct Fused3DArgs {
  const char* src;
  char* dst;
  int64_t src_pitch[3];  // bytes
  int64_t dst_pitch[3];
  int32_t src_origin[3];
  int32_t dst_origin[3];
  int32_t req_lo[3];  // requested region, inclusive bounds
  int32_t req_hi[3];
  int32_t lo[3];  // gather bounds (image bounds within the input buffer), inclusive
  int32_t hi[3];
  int32_t ntx, nty;  // tiles along x and y
  int64_t units;     // ntx * nty * nz_requested
  int32_t out_dtype;
  int32_t pad_;
  float wx[kMaxFusedK];
  float wy[kMaxFusedK];
  f2_t wz2[kMaxFusedK];  // {w, w} pairs for the packed z pass
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void cp_async4(uint32_t saddr, const void* g) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(saddr), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Tile shape per radius.
template <int RX, int RY, int RZ>
struct Cfg3 {
  static constexpr int KX = 2 * RX + 1, KY = 2 * RY + 1, KZ = 2 * RZ + 1;
  static constexpr int NT = 256;                  // threads per CTA
  static constexpr int NW = NT / 32;
  static constexpr int TX = 32;                   // one lane per output column
  static constexpr int MY = 4;                    // rows per thread (y pass, z ring)
  static constexpr int MY2 = MY / 2;              // packed row pairs
  static constexpr int TY = NW * MY;
  static constexpr int MX = 4;                    // x outputs per x-pass task
  static constexpr int IW = TX + 2 * RX;          // staged tile width
  static constexpr int IH = TY + 2 * RY;          // staged tile height
  static constexpr int WIN = ((MX + 2 * RX) + 3) / 4 * 4;  // x-pass window, float4 multiple
  static constexpr int IWP = ((TX - MX + WIN) + 3) / 4 * 4;  // row stride (floats)
  static constexpr int S = 4;                     // slices in flight
  static constexpr int NLD = (IH * IW + NT - 1) / NT;
  static constexpr int STAGE = IH * IWP;          // floats per stage
  static constexpr size_t SMEM = sizeof(float) * (size_t)(S * STAGE + IH * TX);
  static constexpr int MINB = 2;
};

// z pass for phase P: push the packed y-filtered values into every ring slot,
// then hand back the completed slot (P + 1) mod KZ and clear it.
template <int P, int KZ, int MY2, bool REF>
__device__ __forceinline__ void push_phase(f2_t (&acc)[MY2][KZ], const f2_t (&yv)[MY2],
                                           const Fused3DArgs& a, f2_t (&done)[MY2]) {
#pragma unroll
  for (int k = 0; k < KZ; ++k) {
    const int slot = (P - k + KZ) % KZ;
#pragma unroll
    for (int m = 0; m < MY2; ++m) acc[m][slot] = tap2<REF>(acc[m][slot], yv[m], a.wz2[k]);
  }
  constexpr int D = (P + 1) % KZ;
#pragma unroll
  for (int m = 0; m < MY2; ++m) {
    done[m] = acc[m][D];
    acc[m][D] = 0ull;
  }
}

#define ITKG_PUSH_CASE(N)                                          \
  case N:                                                          \
    if constexpr (N < KZ) push_phase<N, KZ, MY2, REF>(acc, yv, a, done); \
    break;

template <int RX, int RY, int RZ, bool REF>
__global__ void __launch_bounds__(Cfg3<RX, RY, RZ>::NT, Cfg3<RX, RY, RZ>::MINB)
    k_fused3d_f32(const Fused3DArgs a) {
  using C = Cfg3<RX, RY, RZ>;
  constexpr int KX = C::KX, KY = C::KY, KZ = C::KZ, TX = C::TX, TY = C::TY, MY = C::MY,
                MY2 = C::MY2, MX = C::MX, IW = C::IW, IH = C::IH, IWP = C::IWP, S = C::S,
                NLD = C::NLD, NT = C::NT;
  static_assert(KZ <= 17, "phase switch covers KZ <= 17");
  extern __shared__ __align__(16) float smem[];
  float* const stage0 = smem;
  float* const xs = smem + S * C::STAGE;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nzr = a.req_hi[2] - a.req_lo[2] + 1;
  const int64_t u_begin = a.units * blockIdx.x / gridDim.x;
  const int64_t u_end = a.units * (blockIdx.x + 1) / gridDim.x;
  const uint32_t sbase = smem_u32(stage0);

  for (int64_t u = u_begin; u < u_end;) {
    const int64_t tile = u / nzr;
    const int zs = (int)(u % nzr);
    const int64_t zrem = zs + (u_end - u);
    const int ze = zrem < nzr ? (int)zrem : nzr;
    u += ze - zs;
    const int z0 = a.req_lo[2] + zs, z1 = a.req_lo[2] + ze;  // outputs [z0, z1)
    const int tx0 = a.req_lo[0] + (int)(tile % a.ntx) * TX;
    const int ty0 = a.req_lo[1] + (int)(tile / a.ntx) * TY;

    // Gather offsets of this thread's share of the staged tile (clamped x, y).
    int32_t goff[NLD];
#pragma unroll
    for (int i = 0; i < NLD; ++i) {
      const int e = tid + i * NT;
      const int row = e / IW, col = e % IW;
      const int gx = clampi(tx0 - RX + col, a.lo[0], a.hi[0]);
      const int gy = clampi(ty0 - RY + row, a.lo[1], a.hi[1]);
      goff[i] = (int32_t)((gx - a.src_origin[0]) * a.src_pitch[0] +
                          (gy - a.src_origin[1]) * a.src_pitch[1]);
    }

    const int jb = z0 - RZ, je = z1 - 1 + RZ;
    const int s_first = max(jb, a.lo[2]), s_last = min(je, a.hi[2]);
#define ITKG_ISSUE(S_, ST_)                                                               \
  do {                                                                                    \
    const char* base_ = a.src + (int64_t)((S_) - a.src_origin[2]) * a.src_pitch[2];       \
    const uint32_t sb_ = sbase + (uint32_t)((ST_) * C::STAGE * 4);                        \
    _Pragma("unroll") for (int i = 0; i < NLD; ++i) {                                     \
      const int e_ = tid + i * NT;                                                        \
      if (i < NLD - 1 || e_ < IH * IW)                                                    \
        cp_async4(sb_ + (uint32_t)(((e_ / IW) * IWP + e_ % IW) * 4), base_ + goff[i]);    \
    }                                                                                     \
  } while (0)
#pragma unroll
    for (int q = 0; q < S; ++q) {
      if (s_first + q <= s_last) ITKG_ISSUE(s_first + q, q);
      cp_async_commit();
    }

    f2_t acc[MY2][KZ];
#pragma unroll
    for (int m = 0; m < MY2; ++m)
#pragma unroll
      for (int q = 0; q < KZ; ++q) acc[m][q] = 0ull;
    f2_t yv[MY2];
#pragma unroll
    for (int m = 0; m < MY2; ++m) yv[m] = 0ull;

    // Output addressing for this thread's column and rows.
    const int col_x = tx0 + lane;
    const int row_y0 = ty0 + warp * MY;
    const bool col_ok = col_x <= a.req_hi[0];
    int nrows_ok = a.req_hi[1] - row_y0 + 1;
    nrows_ok = nrows_ok < 0 ? 0 : (nrows_ok > MY ? MY : nrows_ok);
    char* const obase = a.dst + (int64_t)(col_x - a.dst_origin[0]) * a.dst_pitch[0] +
                        (int64_t)(row_y0 - a.dst_origin[1]) * a.dst_pitch[1];
    const int64_t opy = a.dst_pitch[1];

    int prev_s = INT_MIN;
    int cons = 0;
    int p = 0;  // phase (j - jb) mod KZ
    for (int j = jb; j <= je; ++j) {
      const int s = clampi(j, a.lo[2], a.hi[2]);
      if (s != prev_s) {
        prev_s = s;
        const int st = cons % S;
        cp_async_wait<S - 1>();
        __syncthreads();
        // ---- x pass: stage -> xs ----
        const float* tile = stage0 + st * C::STAGE;
        constexpr int SEGS = TX / MX;
        for (int t = tid; t < IH * SEGS; t += NT) {
          const int row = t / SEGS, x0 = (t % SEGS) * MX;
          float v[C::WIN];
          const float4* src4 = reinterpret_cast<const float4*>(tile + row * IWP + x0);
#pragma unroll
          for (int q = 0; q < C::WIN / 4; ++q) {
            const float4 f = src4[q];
            v[4 * q + 0] = f.x;
            v[4 * q + 1] = f.y;
            v[4 * q + 2] = f.z;
            v[4 * q + 3] = f.w;
          }
          float o[MX];
#pragma unroll
          for (int m = 0; m < MX; ++m) {
            float ax = 0.0f;
#pragma unroll
            for (int k = 0; k < KX; ++k) ax = tap<REF>(ax, v[m + k], a.wx[k]);
            o[m] = ax;
          }
          *reinterpret_cast<float4*>(xs + row * TX + x0) = make_float4(o[0], o[1], o[2], o[3]);
        }
        __syncthreads();
        {
          const int sn = s_first + cons + S;
          if (sn <= s_last) ITKG_ISSUE(sn, st);
          cp_async_commit();
        }
        ++cons;
        // ---- y pass: xs -> yv (registers, packed in row pairs) ----
        float w[MY + 2 * RY];
#pragma unroll
        for (int i = 0; i < MY + 2 * RY; ++i) w[i] = xs[(warp * MY + i) * TX + lane];
#pragma unroll
        for (int m = 0; m < MY2; ++m) {
          float y0 = 0.0f, y1 = 0.0f;
#pragma unroll
          for (int k = 0; k < KY; ++k) {
            y0 = tap<REF>(y0, w[2 * m + k], a.wy[k]);
            y1 = tap<REF>(y1, w[2 * m + 1 + k], a.wy[k]);
          }
          yv[m] = pack2(y0, y1);
        }
      }
      // ---- z pass: push slice j into the ring, pop output z = j - RZ ----
      f2_t done[MY2];
      switch (p) {
        ITKG_PUSH_CASE(0) ITKG_PUSH_CASE(1) ITKG_PUSH_CASE(2) ITKG_PUSH_CASE(3)
        ITKG_PUSH_CASE(4) ITKG_PUSH_CASE(5) ITKG_PUSH_CASE(6) ITKG_PUSH_CASE(7)
        ITKG_PUSH_CASE(8) ITKG_PUSH_CASE(9) ITKG_PUSH_CASE(10) ITKG_PUSH_CASE(11)
        ITKG_PUSH_CASE(12) ITKG_PUSH_CASE(13) ITKG_PUSH_CASE(14) ITKG_PUSH_CASE(15)
        ITKG_PUSH_CASE(16)
        default: break;
      }
      p = p + 1 == KZ ? 0 : p + 1;
      const int z = j - RZ;
      if (z >= z0 && col_ok) {
        char* orow = obase + (int64_t)(z - a.dst_origin[2]) * a.dst_pitch[2];
        float vals[MY];
#pragma unroll
        for (int m = 0; m < MY2; ++m) unpack2(done[m], vals[2 * m], vals[2 * m + 1]);
        if (a.out_dtype == ITKG_F32) {
#pragma unroll
          for (int m = 0; m < MY; ++m)
            if (m < nrows_ok) __stcs(reinterpret_cast<float*>(orow + m * opy), vals[m]);
        } else {
#pragma unroll
          for (int m = 0; m < MY; ++m) {
            if (m >= nrows_ok) continue;
            char* q = orow + m * opy;
            if (a.out_dtype == ITKG_BF16) *reinterpret_cast<__nv_bfloat16*>(q) = from_f32<__nv_bfloat16>(vals[m]);
            else if (a.out_dtype == ITKG_F16) *reinterpret_cast<__half*>(q) = from_f32<__half>(vals[m]);
            else *reinterpret_cast<uint8_t*>(q) = from_f32<uint8_t>(vals[m]);
          }
        }
      }
    }
#undef ITKG_ISSUE
    cp_async_wait<0>();
    __syncthreads();
  }
}

// ---- dispatch table -----------------------------------------------------------
using KernelFn = void (*)(const Fused3DArgs);

struct Entry {
  int rx, ry, rz;
  KernelFn ref, fma;
  size_t smem;
  int tx, ty, nt;
};

template <int RX, int RY, int RZ>
Entry make_entry() {
  using C = Cfg3<RX, RY, RZ>;
  return Entry{RX, RY, RZ, k_fused3d_f32<RX, RY, RZ, true>, k_fused3d_f32<RX, RY, RZ, false>,
               C::SMEM, C::TX, C::TY, C::NT};
}

const Entry kTable[] = {
    make_entry<1, 1, 1>(), make_entry<2, 2, 2>(), make_entry<3, 3, 3>(), make_entry<4, 4, 4>(),
    make_entry<5, 5, 5>(), make_entry<6, 6, 6>(), make_entry<7, 7, 7>(), make_entry<8, 8, 8>(),
    make_entry<7, 7, 2>(),
};

const Entry* find_entry(int rx, int ry, int rz) {
  for (const Entry& e : kTable)
    if (e.rx == rx && e.ry == ry && e.rz == rz) return &e;
  return nullptr;
}

struct Occ {
  KernelFn fn;
  int dev;
  int blocks;
};
std::mutex g_occ_mu;
std::vector<Occ> g_occ;

itkg_status resident_ctas(KernelFn fn, size_t smem, int nt, int* out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "cudaGetDevice failed");
  {
    std::lock_guard<std::mutex> lk(g_occ_mu);
    for (const Occ& o : g_occ)
      if (o.fn == fn && o.dev == dev) {
        *out = o.blocks;
        return ITKG_SUCCESS;
      }
  }
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(e));
  int per_sm = 0, sms = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, nt, smem);
  if (e != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "occupancy: %s", cudaGetErrorString(e));
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "SM count: %s", cudaGetErrorString(e));
  const int blocks = std::max(1, per_sm) * sms;
  std::lock_guard<std::mutex> lk(g_occ_mu);
  g_occ.push_back({fn, dev, blocks});
  *out = blocks;
  return ITKG_SUCCESS;
}

bool fits_i32(int64_t v) { return v >= INT_MIN && v <= INT_MAX; }

}  // namespace

itkg_status launch_fused(const FusedGeom& g, const float* const w[kMaxDim], void* stream,
                         bool dry_run) {
  if (g.dim != 3 || g.comps != 1 || g.in_dtype != ITKG_F32) return ITKG_ERROR_UNSUPPORTED;
  if (g.out_dtype == ITKG_I16) return ITKG_ERROR_UNSUPPORTED;
  const Entry* e = find_entry(g.radius[0], g.radius[1], g.radius[2]);
  if (!e) return ITKG_ERROR_UNSUPPORTED;
  // 32-bit in-slice offsets and coordinates
  for (int d = 0; d < 3; ++d)
    if (!fits_i32(g.lo[d]) || !fits_i32(g.hi[d]) || !fits_i32(g.src_origin[d]) ||
        !fits_i32(g.dst_origin[d]) || !fits_i32(g.req_index[d] + g.req_size[d]))
      return ITKG_ERROR_UNSUPPORTED;
  const int64_t span = (g.hi[0] - g.src_origin[0] + 1) * g.src_pitch[0] +
                       (g.hi[1] - g.src_origin[1] + 1) * g.src_pitch[1];
  if (!fits_i32(span)) return ITKG_ERROR_UNSUPPORTED;
  if (g.src_pitch[0] != 4) return ITKG_ERROR_UNSUPPORTED;
  if (((uintptr_t)g.src & 3) || (g.src_pitch[1] & 3) || (g.src_pitch[2] & 3)) return ITKG_ERROR_UNSUPPORTED;
  if (dry_run) return ITKG_SUCCESS;

  Fused3DArgs a;
  std::memset(&a, 0, sizeof a);
  a.src = static_cast<const char*>(g.src);
  a.dst = static_cast<char*>(g.dst);
  for (int d = 0; d < 3; ++d) {
    a.src_pitch[d] = g.src_pitch[d];
    a.dst_pitch[d] = g.dst_pitch[d];
    a.src_origin[d] = (int32_t)g.src_origin[d];
    a.dst_origin[d] = (int32_t)g.dst_origin[d];
    a.req_lo[d] = (int32_t)g.req_index[d];
    a.req_hi[d] = (int32_t)(g.req_index[d] + g.req_size[d] - 1);
    // Gather bounds: the image bounds intersected with the input buffer.  Every
    // coordinate that feeds a stored output clamps identically under both
    // (the buffer covers input_region_for_output(requested)); tile columns
    // beyond the request only feed outputs that are never stored, and the
    // intersection keeps their loads inside the buffer.
    a.lo[d] = (int32_t)std::max<int64_t>(g.lo[d], g.src_origin[d]);
    a.hi[d] = (int32_t)std::min<int64_t>(g.hi[d], g.src_origin[d] + g.src_size[d] - 1);
  }
  a.ntx = (int32_t)((g.req_size[0] + e->tx - 1) / e->tx);
  a.nty = (int32_t)((g.req_size[1] + e->ty - 1) / e->ty);
  a.units = (int64_t)a.ntx * a.nty * g.req_size[2];
  a.out_dtype = g.out_dtype;
  for (int k = 0; k < 2 * e->rx + 1; ++k) a.wx[k] = w[0][k];
  for (int k = 0; k < 2 * e->ry + 1; ++k) a.wy[k] = w[1][k];
  for (int k = 0; k < 2 * e->rz + 1; ++k) a.wz2[k] = splat2_host(w[2][k]);
  KernelFn fn = g.rounding == ITKG_ROUND_REFERENCE ? e->ref : e->fma;
  int resident = 0;
  {
    const itkg_status st = resident_ctas(fn, e->smem, e->nt, &resident);
    if (st != ITKG_SUCCESS) return st;
  }
  const int64_t grid = std::min<int64_t>(a.units, resident);
  fn<<<(unsigned)grid, e->nt, e->smem, static_cast<cudaStream_t>(stream)>>>(a);
  note_launch(g.rounding == ITKG_ROUND_REFERENCE ? "fused3d_f32_ref" : "fused3d_f32_fma");
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "fused3d launch: %s", cudaGetErrorString(err));
  return ITKG_SUCCESS;
}

}  // namespace itkg
