// Tiled 2-D Gaussian forward: both passes of GaussianFilter::generate_region
// (src/filters/gaussian.rs:74-88) for Image<f32, 2>, Image<VecPixel<f32, 2>, 2>
// and Image<VecPixel<f32, 3>, 2> (and every slice of a 3-D image whose z kernel is
// the 1-tap [1], SliceBySliceFilter), one CTA per 64 x 32 output tile:
//   1. the tile's (64 + 2r) x (32 + 2r) input pixels, rows and columns clamped
//      to the image (the reference's clamp-to-edge, conv.rs:31-33), arrive by
//      4-byte cp.async all at once, de-interleaved into C planar tiles;
//   2. x pass: each item filters 4 consecutive pixels of one staged row of one
//      component from a register window (16-byte shared loads) into the
//      x-filtered tile (all 32 + 2r rows: the halo rows are what the y taps of
//      the tile's edge rows read, clamped rows included);
//   3. y pass: each item filters 8 consecutive rows of one column of one
//      component from a register window, and stores them.
// Every load of the CTA is in flight at once, so a tile costs about one memory
// round trip plus its arithmetic: the row-marching kernel (fused2d.cu) waits
// for its rows one after another, which is what small images pay for.
// Reference rounding: scalar acc = acc + x * w in ascending tap order from zero
// per pass, f32 intermediate -- bit-identical to the reference.  FMA rounding:
// fmaf in the same order.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "internal.hpp"
#include "pixel.cuh"

namespace itkg {
namespace {

constexpr int kT2MaxR = 12;
constexpr int kT2MaxK = 2 * kT2MaxR + 1;
constexpr int kTW = 64, kTH = 32;  // output tile (pixels x rows)
constexpr int kT2Threads = 256;
constexpr int kYRun = 8;           // rows per y-pass item

struct Tile2DArgs {
  const char* src;
  char* dst;
  int64_t src_pitch[2];  // bytes (pixel, row)
  int64_t dst_pitch[2];
  int64_t src_slice, dst_slice;  // bytes between slices (SliceBySliceFilter over a 3-D image)
  int32_t src_origin[2];
  int32_t dst_origin[2];
  int32_t req_lo[2], req_hi[2];  // inclusive
  int32_t lo[2], hi[2];          // gather bounds (the image within the buffer), inclusive
  int32_t ntx, nty;              // tiles per slice along x and y
  int32_t out_dtype;
  int32_t out_esz;
  float wx[kT2MaxK], wy[kT2MaxK];
};

template <int R, int C>
struct T2Cfg {
  static constexpr int K = 2 * R + 1;
  static constexpr int IW = kTW + 2 * R;          // staged row (pixels)
  static constexpr int IWP = (IW + 3) / 4 * 4;    // 16-byte aligned staged rows
  static constexpr int IH = kTH + 2 * R;          // staged rows
  static constexpr int WIN = (4 + 2 * R + 3) / 4 * 4;  // x window, whole float4s
  static constexpr int IN = C * IH * IWP;         // staged floats
  static constexpr int XF = C * IH * kTW;         // x-filtered floats
  static constexpr size_t SMEM = sizeof(float) * (size_t)(IN + XF);
  static_assert(WIN <= IWP, "x window inside a staged row");
};

__device__ __forceinline__ void cp4(float* dst, const void* src) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}

// One tile t of the launch described by `a` (weights wx / wy in registers).
template <int R, int C, bool REF>
__device__ __forceinline__ void tile2d_body(const Tile2DArgs& a, const float (&wx)[2 * R + 1],
                                            const float (&wy)[2 * R + 1], int64_t t, float* sm) {
  using G = T2Cfg<R, C>;
  constexpr int K = G::K, IW = G::IW, IWP = G::IWP, IH = G::IH, WIN = G::WIN;
  float* const sin = sm;             // [C][IH][IWP]
  float* const sxf = sm + G::IN;     // [C][IH][kTW]
  const int64_t per_slice = (int64_t)a.ntx * a.nty;
  const int64_t zq = t / per_slice;
  const int ti = (int)(t - zq * per_slice);
  const int tx0 = a.req_lo[0] + (ti % a.ntx) * kTW;
  const int ty0 = a.req_lo[1] + (ti / a.ntx) * kTH;
  const char* const srcz = a.src + zq * a.src_slice;

  // 1. stage the clamped input tile; components fastest, so a warp reads
  //    consecutive floats of an interleaved row
  for (int e = threadIdx.x; e < IH * IW * C; e += kT2Threads) {
    const int c = C == 1 ? 0 : e % C;
    const int pe = C == 1 ? e : e / C;
    const int col = pe % IW, row = pe / IW;
    const int gx = min(max(tx0 - R + col, a.lo[0]), a.hi[0]);
    const int gy = min(max(ty0 - R + row, a.lo[1]), a.hi[1]);
    const char* p = srcz + (int64_t)(gx - a.src_origin[0]) * a.src_pitch[0] +
                    (int64_t)(gy - a.src_origin[1]) * a.src_pitch[1] + c * 4;
    cp4(sin + (c * IH + row) * IWP + col, p);
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();

  // 2. x pass: items (component, staged row, quad of output columns)
  for (int it = threadIdx.x; it < C * IH * (kTW / 4); it += kT2Threads) {
    const int q = it % (kTW / 4);
    const int cr = it / (kTW / 4);  // c * IH + row
    const float* const src = sin + cr * IWP + 4 * q;
    float v[WIN];
#pragma unroll
    for (int i = 0; i < WIN / 4; ++i) {
      const float4 f = *reinterpret_cast<const float4*>(src + 4 * i);
      v[4 * i] = f.x, v[4 * i + 1] = f.y, v[4 * i + 2] = f.z, v[4 * i + 3] = f.w;
    }
    float o[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      float acc = 0.0f;
#pragma unroll
      for (int k = 0; k < K; ++k) acc = REF ? tap<true>(acc, v[m + k], wx[k]) : fmaf(v[m + k], wx[k], acc);
      o[m] = acc;
    }
    *reinterpret_cast<float4*>(sxf + cr * kTW + 4 * q) = make_float4(o[0], o[1], o[2], o[3]);
  }
  __syncthreads();

  // 3. y pass: items (component, output column, run of kYRun rows)
  char* const dstz = a.dst + zq * a.dst_slice;
  for (int it = threadIdx.x; it < C * kTW * (kTH / kYRun); it += kT2Threads) {
    const int x = it % kTW;
    const int rest = it / kTW;
    const int c = rest % C;
    const int run = rest / C;
    const int gx = tx0 + x;
    const int gy0 = ty0 + run * kYRun;
    if (gx > a.req_hi[0] || gy0 > a.req_hi[1]) continue;
    const float* const col = sxf + (c * IH + run * kYRun) * kTW + x;
    float v[kYRun + 2 * R];
#pragma unroll
    for (int j = 0; j < kYRun + 2 * R; ++j) v[j] = col[j * kTW];
    char* const ob = dstz + (int64_t)(gx - a.dst_origin[0]) * a.dst_pitch[0] + (int64_t)c * a.out_esz +
                     (int64_t)(gy0 - a.dst_origin[1]) * a.dst_pitch[1];
#pragma unroll
    for (int m = 0; m < kYRun; ++m) {
      if (gy0 + m > a.req_hi[1]) break;
      float acc = 0.0f;
#pragma unroll
      for (int k = 0; k < K; ++k) acc = REF ? tap<true>(acc, v[m + k], wy[k]) : fmaf(v[m + k], wy[k], acc);
      char* const q = ob + (int64_t)m * a.dst_pitch[1];
      switch (a.out_dtype) {
        case ITKG_F32: *reinterpret_cast<float*>(q) = acc; break;
        case ITKG_BF16: *reinterpret_cast<__nv_bfloat16*>(q) = from_f32<__nv_bfloat16>(acc); break;
        case ITKG_F16: *reinterpret_cast<__half*>(q) = from_f32<__half>(acc); break;
        default: *reinterpret_cast<uint8_t*>(q) = from_f32<uint8_t>(acc); break;
      }
    }
  }
}

template <int R, int C, bool REF>
__global__ void __launch_bounds__(kT2Threads) k_tile2d(const Tile2DArgs a) {
  extern __shared__ __align__(16) float sm[];
  float wx[2 * R + 1], wy[2 * R + 1];
#pragma unroll
  for (int k = 0; k < 2 * R + 1; ++k) wx[k] = a.wx[k], wy[k] = a.wy[k];
  tile2d_body<R, C, REF>(a, wx, wy, blockIdx.x, sm);
}

// Many requests of one class (radius, components, rounding) in one launch:
// request q owns the CTAs [starts[q], starts[q + 1]); each CTA copies its
// request's arguments to shared memory and its weights to registers.
template <int R, int C, bool REF>
__global__ void __launch_bounds__(kT2Threads) k_tile2d_multi(const Tile2DArgs* reqs, const int32_t* starts, int nreq) {
  extern __shared__ __align__(16) float sm[];
  __shared__ Tile2DArgs sa;
  __shared__ int sq;
  if (threadIdx.x == 0) {
    int lo = 0, hi = nreq - 1;  // the last q with starts[q] <= blockIdx.x
    while (lo < hi) {
      const int mid = (lo + hi + 1) / 2;
      if (starts[mid] <= (int)blockIdx.x) lo = mid;
      else hi = mid - 1;
    }
    sq = lo;
  }
  __syncthreads();
  const int q = sq;
  {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(reqs + q);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&sa);
    for (int i = threadIdx.x; i < (int)(sizeof(Tile2DArgs) / 4); i += kT2Threads) dst[i] = src[i];
  }
  __syncthreads();
  float wx[2 * R + 1], wy[2 * R + 1];
#pragma unroll
  for (int k = 0; k < 2 * R + 1; ++k) wx[k] = sa.wx[k], wy[k] = sa.wy[k];
  tile2d_body<R, C, REF>(sa, wx, wy, (int64_t)blockIdx.x - starts[q], sm);
}

using FnT2 = void (*)(const Tile2DArgs);
using FnT2M = void (*)(const Tile2DArgs*, const int32_t*, int);
struct EntryT2 {
  int r, comps;
  FnT2 fn[2];    // [ref]
  FnT2M multi[2];
  size_t smem;
};
template <int R, int C>
EntryT2 make_t2() {
  return EntryT2{R, C, {k_tile2d<R, C, false>, k_tile2d<R, C, true>},
                 {k_tile2d_multi<R, C, false>, k_tile2d_multi<R, C, true>}, T2Cfg<R, C>::SMEM};
}
const EntryT2 kTableT2[] = {
    make_t2<1, 1>(),  make_t2<2, 1>(),  make_t2<3, 1>(),  make_t2<4, 1>(),  make_t2<5, 1>(),  make_t2<6, 1>(),
    make_t2<7, 1>(),  make_t2<8, 1>(),  make_t2<9, 1>(),  make_t2<10, 1>(), make_t2<11, 1>(), make_t2<12, 1>(),
    make_t2<1, 3>(),  make_t2<2, 3>(),  make_t2<3, 3>(),  make_t2<4, 3>(),  make_t2<5, 3>(),  make_t2<6, 3>(),
    make_t2<7, 3>(),  make_t2<8, 3>(),  make_t2<9, 3>(),  make_t2<10, 3>(), make_t2<11, 3>(), make_t2<12, 3>(),
    // VecPixel<f32, 2> (displacement fields)
    make_t2<1, 2>(),  make_t2<2, 2>(),  make_t2<3, 2>(),  make_t2<4, 2>(),  make_t2<5, 2>(),  make_t2<6, 2>(),
    make_t2<7, 2>(),  make_t2<8, 2>(),  make_t2<9, 2>(),  make_t2<10, 2>(), make_t2<11, 2>(), make_t2<12, 2>(),
};

bool fits32t(int64_t v) { return v >= INT_MIN && v <= INT_MAX; }

// cudaFuncSetAttribute once per kernel and device
std::mutex g_t2_mu;
std::vector<std::pair<const void*, int>> g_t2_ready;
itkg_status prepare_t2(const void* fn, size_t smem) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(err));
  std::lock_guard<std::mutex> lk(g_t2_mu);
  for (const auto& r : g_t2_ready)
    if (r.first == fn && r.second == dev) return ITKG_SUCCESS;
  err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(err));
  g_t2_ready.push_back({fn, dev});
  return ITKG_SUCCESS;
}

// The launch arguments of one request, its table entry and tile count;
// ITKG_ERROR_UNSUPPORTED (no error set) when the tile kernel does not cover it.
itkg_status build_t2(const FusedGeom& g, const float* const w[kMaxDim], Tile2DArgs* out, const EntryT2** entry,
                     int64_t* ntiles) {
  const bool slices = g.dim == 3 && g.radius[2] == 0 && w[2] && w[2][0] == 1.0f;
  if (g.u8pix) return ITKG_ERROR_UNSUPPORTED;
  if ((g.dim != 2 && !slices) || g.in_dtype != ITKG_F32 || g.out_dtype == ITKG_I16) return ITKG_ERROR_UNSUPPORTED;
  if (g.radius[0] != g.radius[1] || g.radius[0] < 1) return ITKG_ERROR_UNSUPPORTED;
  const EntryT2* e = nullptr;
  for (const EntryT2& t : kTableT2)
    if (t.r == g.radius[0] && t.comps == g.comps) e = &t;
  if (!e) return ITKG_ERROR_UNSUPPORTED;
  for (int d = 0; d < 2; ++d)
    if (!fits32t(g.lo[d]) || !fits32t(g.hi[d]) || !fits32t(g.src_origin[d]) || !fits32t(g.dst_origin[d]) ||
        !fits32t(g.req_index[d] + g.req_size[d] + kTH) || !fits32t(g.req_index[d] - 64))
      return ITKG_ERROR_UNSUPPORTED;
  if (g.src_pitch[0] != 4 * g.comps || ((uintptr_t)g.src & 3) || (g.src_pitch[1] & 3) ||
      (slices && (g.src_pitch[2] & 3)))
    return ITKG_ERROR_UNSUPPORTED;
  const int64_t nz = slices ? g.req_size[2] : 1;
  const int64_t ntx = (g.req_size[0] + kTW - 1) / kTW, nty = (g.req_size[1] + kTH - 1) / kTH;
  if (ntx * nty * nz > INT_MAX) return ITKG_ERROR_UNSUPPORTED;
  Tile2DArgs& a = *out;
  std::memset(&a, 0, sizeof a);
  a.src = static_cast<const char*>(g.src);
  a.dst = static_cast<char*>(g.dst);
  if (slices) {  // start at the first requested slice
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
    a.lo[d] = (int32_t)std::max<int64_t>(g.lo[d], g.src_origin[d]);
    a.hi[d] = (int32_t)std::min<int64_t>(g.hi[d], g.src_origin[d] + g.src_size[d] - 1);
  }
  a.ntx = (int32_t)ntx;
  a.nty = (int32_t)nty;
  a.out_dtype = g.out_dtype;
  a.out_esz = dtype_size(g.out_dtype);
  for (int k = 0; k < 2 * e->r + 1; ++k) a.wx[k] = w[0][k], a.wy[k] = w[1][k];
  *entry = e;
  *ntiles = ntx * nty * nz;
  return ITKG_SUCCESS;
}

}  // namespace

itkg_status launch_tile2d(const FusedGeom& g, const float* const w[kMaxDim], void* stream, bool dry_run) {
  Tile2DArgs a;
  const EntryT2* e = nullptr;
  int64_t ntiles = 0;
  {
    const itkg_status st = build_t2(g, w, &a, &e, &ntiles);
    if (st != ITKG_SUCCESS) return st;
  }
  if (dry_run) return ITKG_SUCCESS;
  const bool ref = g.rounding == ITKG_ROUND_REFERENCE;
  const FnT2 fn = e->fn[ref ? 1 : 0];
  {
    const itkg_status pst = prepare_t2(reinterpret_cast<const void*>(fn), e->smem);
    if (pst != ITKG_SUCCESS) return pst;
  }
  fn<<<(unsigned)ntiles, kT2Threads, e->smem, static_cast<cudaStream_t>(stream)>>>(a);
  const cudaError_t err = cudaGetLastError();
  note_launch(ref ? "tile2d_f32_ref" : "tile2d_f32_fma");
  if (err != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "tile2d launch: %s", cudaGetErrorString(err));
  return ITKG_SUCCESS;
}

// Multi-request launches: the requests grouped by kernel class, one launch per
// class with the requests' arguments and CTA ranges in device tables.
struct Tile2DMultiGroup {
  const EntryT2* e = nullptr;
  bool ref = false;
  std::vector<Tile2DArgs> reqs;
  std::vector<int32_t> starts;  // CTA ranges, starts.back() = CTAs in all
  Tile2DArgs* d_reqs = nullptr;
  int32_t* d_starts = nullptr;
  double work = 0.0;
};
struct Tile2DMultiPlan {
  std::vector<Tile2DMultiGroup> groups;
};

itkg_status tile2d_multi_prepare(const std::vector<FusedGeom>& geoms,
                                 const std::vector<std::vector<std::vector<float>>>& weights,
                                 Tile2DMultiPlan** out, std::vector<std::string>* lines) {
  Tile2DMultiPlan* plan = new Tile2DMultiPlan();
  *out = plan;
  for (size_t i = 0; i < geoms.size(); ++i) {
    const FusedGeom& g = geoms[i];
    const float* w[kMaxDim] = {nullptr, nullptr, nullptr};
    for (int d = 0; d < g.dim && d < (int)weights[i].size(); ++d) w[d] = weights[i][d].data();
    Tile2DArgs a;
    const EntryT2* e = nullptr;
    int64_t ntiles = 0;
    const itkg_status st = build_t2(g, w, &a, &e, &ntiles);
    if (st != ITKG_SUCCESS) return st == ITKG_ERROR_UNSUPPORTED ? set_error(st, "no tile kernel for 2-D item %zu", i) : st;
    const bool ref = g.rounding == ITKG_ROUND_REFERENCE;
    Tile2DMultiGroup* grp = nullptr;
    for (Tile2DMultiGroup& q : plan->groups)
      if (q.e == e && q.ref == ref) grp = &q;
    if (!grp) {
      plan->groups.push_back(Tile2DMultiGroup());
      grp = &plan->groups.back();
      grp->e = e;
      grp->ref = ref;
      grp->starts.push_back(0);
    }
    if ((int64_t)grp->starts.back() + ntiles > INT_MAX) return set_error(ITKG_ERROR_UNSUPPORTED, "too many tiles");
    grp->reqs.push_back(a);
    grp->starts.push_back(grp->starts.back() + (int32_t)ntiles);
    grp->work += (double)g.req_size[0] * g.req_size[1] * g.comps * (double)(2 * e->r + 1 + 4);
  }
  for (Tile2DMultiGroup& q : plan->groups) {
    cudaError_t err = cudaMalloc(&q.d_reqs, sizeof(Tile2DArgs) * q.reqs.size());
    if (err == cudaSuccess) err = cudaMalloc(&q.d_starts, sizeof(int32_t) * q.starts.size());
    if (err == cudaSuccess)
      err = cudaMemcpy(q.d_reqs, q.reqs.data(), sizeof(Tile2DArgs) * q.reqs.size(), cudaMemcpyHostToDevice);
    if (err == cudaSuccess)
      err = cudaMemcpy(q.d_starts, q.starts.data(), sizeof(int32_t) * q.starts.size(), cudaMemcpyHostToDevice);
    if (err != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "tile2d multi tables: %s", cudaGetErrorString(err));
    const itkg_status pst = prepare_t2(reinterpret_cast<const void*>(q.e->multi[q.ref ? 1 : 0]), q.e->smem);
    if (pst != ITKG_SUCCESS) return pst;
    if (lines)
      lines->push_back(std::string(q.ref ? "tile2d_f32_ref" : "tile2d_f32_fma") + " multi-request launch: r=" +
                       std::to_string(q.e->r) + ", " + std::to_string(q.e->comps) + " components, " +
                       std::to_string(q.reqs.size()) + " requests, " + std::to_string(q.starts.back()) + " CTAs");
  }
  return ITKG_SUCCESS;
}

int tile2d_multi_groups(const Tile2DMultiPlan* plan) { return plan ? (int)plan->groups.size() : 0; }

double tile2d_multi_work(const Tile2DMultiPlan* plan, int group) { return plan->groups[group].work; }

itkg_status tile2d_multi_launch(const Tile2DMultiPlan* plan, int group, void* stream) {
  const Tile2DMultiGroup& q = plan->groups[group];
  const FnT2M fn = q.e->multi[q.ref ? 1 : 0];
  fn<<<(unsigned)q.starts.back(), kT2Threads, q.e->smem, static_cast<cudaStream_t>(stream)>>>(
      q.d_reqs, q.d_starts, (int)q.reqs.size());
  note_launch(q.ref ? "tile2d_multi_f32_ref" : "tile2d_multi_f32_fma");
  const cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "tile2d multi launch: %s", cudaGetErrorString(err));
  return ITKG_SUCCESS;
}

void tile2d_multi_free(Tile2DMultiPlan* plan) {
  if (!plan) return;
  for (Tile2DMultiGroup& q : plan->groups) {
    if (q.d_reqs) cudaFree(q.d_reqs);
    if (q.d_starts) cudaFree(q.d_starts);
  }
  delete plan;
}

}  // namespace itkg
