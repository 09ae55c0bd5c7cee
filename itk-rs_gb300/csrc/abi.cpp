// C-ABI implementation: validation, region geometry, host staging and kernel
// dispatch for GaussianFilter::generate_region and stream_full.
//
// Region geometry follows the reference exactly:
//   kernel_radius            src/filters/gaussian.rs:24-27
//   build_kernel             src/filters/gaussian.rs:29-40
//   input_region_for_output  src/filters/gaussian.rs:52-57
//   generate_region passes   src/filters/gaussian.rs:59-91
//   padded_per_axis/clipped  src/image.rs:28-64
//   split_region             src/region_splitter.rs:17-48
//   stream_full              src/source.rs:81-98
#include <cuda_runtime.h>

#include <array>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "geom.hpp"
#include "internal.hpp"

namespace itkg {

namespace {
thread_local std::string t_error;
thread_local std::string t_kernel;
}  // namespace

itkg_status set_error(itkg_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_error = buf;
  return st;
}

void set_last_kernel(const char* name) { t_kernel = name; }

namespace {
std::atomic<uint64_t> g_launches{0};
}  // namespace

void note_launch(const char* name) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  t_kernel = name;
}

void note_launches(uint64_t n, const char* name) {
  g_launches.fetch_add(n, std::memory_order_relaxed);
  t_kernel = name;
}

// ---- scratch: one memory pool per device, never trimmed --------------------
namespace {
std::mutex g_pool_mu;
std::vector<cudaMemPool_t> g_pools;  // indexed by device
}  // namespace

static itkg_status device_pool(cudaMemPool_t* out) {
  int dev = 0;
  ITKG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_pool_mu);
  if ((int)g_pools.size() <= dev) g_pools.resize(dev + 1, nullptr);
  if (!g_pools[dev]) {
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof props);
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool;
    ITKG_CUDA(cudaMemPoolCreate(&pool, &props));
    uint64_t thr = UINT64_MAX;
    ITKG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
    g_pools[dev] = pool;
  }
  *out = g_pools[dev];
  return ITKG_SUCCESS;
}

namespace {
std::atomic<uint64_t> g_scratch_allocs{0};
std::atomic<int64_t> g_fail_after{-1};  // allocations to grant before an injected failure; -1: none
std::atomic<long long> g_wait_limit{1ll << 31};
}  // namespace

long long wait_limit_cycles() { return g_wait_limit.load(std::memory_order_relaxed); }
std::atomic<int> g_kernel2d{0};
int kernel2d_override() { return g_kernel2d.load(std::memory_order_relaxed); }

itkg_status scratch_alloc(void** p, size_t bytes, void* stream) {
  int64_t f = g_fail_after.load(std::memory_order_relaxed);
  while (f >= 0 && !g_fail_after.compare_exchange_weak(f, f - 1, std::memory_order_relaxed)) {
  }
  if (f == 0) return set_error(ITKG_ERROR_OUT_OF_MEMORY, "device scratch allocation failed (injected)");
  g_scratch_allocs.fetch_add(1, std::memory_order_relaxed);
  cudaMemPool_t pool;
  ITKG_TRY(device_pool(&pool));
  if (bytes == 0) bytes = 256;
  ITKG_CUDA(cudaMallocFromPoolAsync(p, bytes, pool, static_cast<cudaStream_t>(stream)));
  return ITKG_SUCCESS;
}

void scratch_free(void* p, void* stream) {
  if (p) cudaFreeAsync(p, static_cast<cudaStream_t>(stream));
}

// Copy `reg` between two images (any locations) with 2-D copies per slice, or
// one copy when both sides are contiguous over the region.
static itkg_status copy_region(const itkg_image& dst, const itkg_image& src, const itkg_region& reg0,
                               cudaStream_t s) {
  const int D = src.dim;
  const itkg_region reg = full3(reg0, D);
  if (region_len(reg, D) == 0) return ITKG_SUCCESS;
  int64_t so[3], sp[3], dof[3], dp[3];
  origin_pitch(src, so, sp);
  origin_pitch(dst, dof, dp);
  const size_t pb = (size_t)src.pitch[0];
  const size_t width = (size_t)reg.size[0] * pb;
  auto sptr = [&](int64_t y, int64_t z) {
    return static_cast<const char*>(src.data) + (reg.index[0] - so[0]) * sp[0] +
           (y - so[1]) * sp[1] + (z - so[2]) * sp[2];
  };
  auto dptr = [&](int64_t y, int64_t z) {
    return static_cast<char*>(dst.data) + (reg.index[0] - dof[0]) * dp[0] + (y - dof[1]) * dp[1] +
           (z - dof[2]) * dp[2];
  };
  const uint64_t ny = reg.size[1], nz = reg.size[2];
  // whole region contiguous on both sides?
  const bool rows_dense = (D < 2 || ((size_t)sp[1] == width && (size_t)dp[1] == width));
  const bool slices_dense =
      (D < 3 || ((size_t)sp[2] == width * ny && (size_t)dp[2] == width * ny));
  if (rows_dense && slices_dense) {
    ITKG_CUDA(cudaMemcpyAsync(dptr(reg.index[1], reg.index[2]), sptr(reg.index[1], reg.index[2]),
                              width * ny * nz, cudaMemcpyDefault, s));
    return ITKG_SUCCESS;
  }
  for (uint64_t z = 0; z < nz; ++z) {
    const int64_t az = reg.index[2] + (int64_t)z;
    const size_t spitch = D >= 2 ? (size_t)sp[1] : width;
    const size_t dpitch = D >= 2 ? (size_t)dp[1] : width;
    ITKG_CUDA(cudaMemcpy2DAsync(dptr(reg.index[1], az), dpitch, sptr(reg.index[1], az), spitch,
                                width, ny, cudaMemcpyDefault, s));
  }
  return ITKG_SUCCESS;
}

// What a call convolves with: the Gaussian of sigma (radius and kernel per axis
// from the spacing, gaussian.rs:24-40), or explicit f64 kernels per axis applied
// in `reps` rounds of one pass per axis (the convolve_axis family: mean.rs,
// binomial_blur.rs).
struct KernelSpec {
  bool gaussian = true;
  double sigma = 0.0;
  uint64_t radius[kMaxDim] = {0, 0, 0};
  const double* w[kMaxDim] = {nullptr, nullptr, nullptr};
  uint64_t reps = 1;
};

struct Plan {
  int D = 0;
  uint64_t radii[kMaxDim] = {0, 0, 0};
  std::vector<double> w64[kMaxDim];
  std::vector<float> w32[kMaxDim];
  uint64_t reps = 1;       // rounds of one pass per axis
  bool symmetric = true;   // every f32 kernel reads the same backwards
  itkg_region in_reg;
};

static itkg_status make_plan(const itkg_image& in, const itkg_region& requested, const itkg_region& largest,
                             const KernelSpec& ks, Plan* p) {
  const int D = in.dim;
  p->D = D;
  p->reps = ks.gaussian ? 1 : ks.reps;
  uint64_t pad[kMaxDim] = {0, 0, 0};
  for (int d = 0; d < D; ++d) {
    const uint64_t r = ks.gaussian ? kernel_radius(ks.sigma, in.spacing[d]) : ks.radius[d];
    if (r > (1u << 20))
      return ks.gaussian ? set_error(ITKG_ERROR_INVALID_ARGUMENT,
                                     "kernel radius %llu on axis %d (sigma=%g, spacing=%g) is not allocatable",
                                     (unsigned long long)r, d, ks.sigma, in.spacing[d])
                         : set_error(ITKG_ERROR_INVALID_ARGUMENT, "kernel radius %llu on axis %d is not allocatable",
                                     (unsigned long long)r, d);
    p->radii[d] = r;
    p->w64[d].resize(2 * r + 1);
    if (ks.gaussian) build_kernel(ks.sigma / in.spacing[d], r, p->w64[d].data());
    else std::copy(ks.w[d], ks.w[d] + 2 * r + 1, p->w64[d].begin());
    p->w32[d].resize(2 * r + 1);
    for (size_t k = 0; k < p->w64[d].size(); ++k) p->w32[d][k] = (float)p->w64[d][k];
    for (size_t k = 0; k < p->w32[d].size(); ++k)
      if (std::memcmp(&p->w32[d][k], &p->w32[d][2 * r - k], sizeof(float)) != 0) p->symmetric = false;
    pad[d] = r * p->reps;
  }
  p->in_reg = clipped(padded(requested, D, pad), D, largest);
  return ITKG_SUCCESS;
}

// ---- per-axis execution (one pass per axis and round, through scratch) -------
// Pass (rep, axis) writes `requested` padded by (reps - rep - 1) kernel radii on
// every axis and one more on the axes after `axis`, clipped to the bounds; the
// last pass writes `requested` (binomial_blur.rs:63-87; with one round these
// are the Gaussian's intermediate regions, gaussian.rs:79-85).  Zero rounds
// copy `requested` (through one pass of the 1-tap kernel [1] when the output
// type differs from the input's).
static itkg_status run_per_axis(const itkg_image& in, const itkg_region& largest,
                                const itkg_region& requested, const itkg_gaussian_params& prm,
                                const Plan& plan, const itkg_image& out, cudaStream_t s) {
  const int D = in.dim;
  const bool u8pix = prm.arithmetic == ITKG_ARITH_PIXEL_U8;
  const int scratch_dtype = u8pix ? ITKG_U8 : ITKG_F32;
  static const double kOne64 = 1.0;
  static const float kOne32 = 1.0f;
  const uint64_t reps = plan.reps;
  if (reps == 0 && in.dtype == out.dtype) {  // the reference returns the crop itself
    ITKG_TRY(copy_region(out, in, requested, s));
    set_last_kernel("copy");
    return ITKG_SUCCESS;
  }
  int npass = reps == 0 ? 1 : (int)std::min<uint64_t>(reps * (uint64_t)D, (uint64_t)INT32_MAX);
  // One round whose last axes have the 1-tap kernel [1] (SliceBySliceFilter's z):
  // those passes would copy their input, and after a real pass no value is -0
  // (every sum starts at +0), so they are left out; the last real pass writes
  // `requested` to the output.
  if (reps == 1)
    while (npass > 1 && plan.radii[npass - 1] == 0 && plan.w64[npass - 1].size() == 1 &&
           plan.w64[npass - 1][0] == 1.0)
      --npass;
  auto region_of = [&](int p) {
    if (p + 1 == npass) return requested;
    const uint64_t rep = (uint64_t)(p / D), remaining = reps - rep - 1;
    const int axis = p % D;
    uint64_t pad[kMaxDim] = {0, 0, 0};
    for (int d = 0; d < D; ++d) pad[d] = (d > axis ? remaining + 1 : remaining) * plan.radii[d];
    return clipped(padded(requested, D, pad), D, largest);
  };
  size_t max_bytes = 0;
  for (int p = 0; p + 1 < npass; ++p)
    max_bytes = std::max(max_bytes, (size_t)region_len(region_of(p), D) * (size_t)in.components *
                                        dtype_size(scratch_dtype));
  void* bufs[2] = {nullptr, nullptr};
  if (npass > 1) {
    ITKG_TRY(scratch_alloc(&bufs[0], max_bytes, s));
    if (npass > 2) {
      itkg_status st = scratch_alloc(&bufs[1], max_bytes, s);
      if (st != ITKG_SUCCESS) {
        scratch_free(bufs[0], s);
        return st;
      }
    }
  }
  itkg_image cur = in;
  itkg_status st = ITKG_SUCCESS;
  for (int p = 0; p < npass && st == ITKG_SUCCESS; ++p) {
    const int a = reps == 0 ? 0 : p % D;
    const itkg_region reg = region_of(p);
    itkg_image nxt;
    if (p + 1 < npass) {
      std::memset(&nxt, 0, sizeof nxt);
      nxt.dim = D;
      nxt.dtype = scratch_dtype;
      nxt.components = in.components;
      nxt.region = reg;
      dense_layout(&nxt, 1);
      nxt.data = bufs[p & 1];
    } else {
      nxt = out;
    }
    AxisArgs args;
    std::memset(&args, 0, sizeof args);
    args.src = cur.data;
    args.dst = nxt.data;
    origin_pitch(cur, args.src_origin, args.src_pitch);
    origin_pitch(nxt, args.dst_origin, args.dst_pitch);
    const itkg_region o3 = full3(reg, D);
    for (int d = 0; d < kMaxDim; ++d) {
      args.out_index[d] = o3.index[d];
      args.out_size[d] = (int64_t)o3.size[d];
    }
    args.lo = largest.index[a];
    args.hi = largest.index[a] + (int64_t)largest.size[a] - 1;
    args.axis = a;
    args.radius = reps == 0 ? 0 : (int32_t)plan.radii[a];
    args.comps = in.components;
    if (u8pix) {
      st = launch_conv_axis_u8(args, reps == 0 ? &kOne64 : plan.w64[a].data(), s);
    } else {
      const int in_dt = p == 0 ? in.dtype : ITKG_F32;
      const int out_dt = p + 1 < npass ? ITKG_F32 : out.dtype;
      st = launch_conv_axis_f32(args, reps == 0 ? &kOne32 : plan.w32[a].data(), in_dt, out_dt, prm.rounding, s);
    }
    cur = nxt;
  }
  scratch_free(bufs[0], s);
  scratch_free(bufs[1], s);
  if (st == ITKG_SUCCESS) set_last_kernel(u8pix ? "per_axis_u8_pixel" : prm.rounding == ITKG_ROUND_REFERENCE ? "per_axis_f32_ref" : "per_axis_f32_fma");
  return st;
}

static itkg_status check_params(const itkg_gaussian_params* prm) {
  if (!prm) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "params is NULL");
  if (prm->arithmetic != ITKG_ARITH_F32 && prm->arithmetic != ITKG_ARITH_PIXEL_U8)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "unknown arithmetic %d", prm->arithmetic);
  if (prm->rounding != ITKG_ROUND_REFERENCE && prm->rounding != ITKG_ROUND_FMA)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "unknown rounding %d", prm->rounding);
  if (prm->algorithm < ITKG_ALGO_AUTO || prm->algorithm > ITKG_ALGO_ONE_TRIP)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "unknown algorithm %d", prm->algorithm);
  if (prm->reserved != 0) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "reserved must be 0");
  return ITKG_SUCCESS;
}

// Device-resident input and output.
static void make_fused_geom(const itkg_image& in, const itkg_region& largest,
                            const itkg_region& requested, const itkg_gaussian_params& prm,
                            const Plan& plan, const itkg_image& out, FusedGeom* gp) {
  const int D = in.dim;
  FusedGeom& g = *gp;
  {
    std::memset(&g, 0, sizeof g);
    g.src = in.data;
    g.dst = out.data;
    origin_pitch(in, g.src_origin, g.src_pitch);
    origin_pitch(out, g.dst_origin, g.dst_pitch);
    const itkg_region r3 = full3(requested, D);
    const itkg_region l3 = full3(largest, D);
    const itkg_region b3 = full3(in.region, D);
    for (int d = 0; d < kMaxDim; ++d) {
      g.src_size[d] = (int64_t)b3.size[d];
      g.req_index[d] = r3.index[d];
      g.req_size[d] = (int64_t)r3.size[d];
      g.lo[d] = l3.index[d];
      g.hi[d] = l3.index[d] + (int64_t)l3.size[d] - 1;
      g.radius[d] = d < D ? (int32_t)plan.radii[d] : 0;
    }
    g.dim = D;
    g.comps = in.components;
    g.in_dtype = in.dtype;
    g.out_dtype = out.dtype;
    g.rounding = prm.rounding;
    g.u8pix = prm.arithmetic == ITKG_ARITH_PIXEL_U8 ? 1 : 0;
  }
}

static itkg_status generate_device(const itkg_image& in, const itkg_region& largest,
                                   const itkg_region& requested, const itkg_gaussian_params& prm,
                                   const Plan& plan, const itkg_image& out, cudaStream_t s);

// Several rounds of symmetric kernels (the binomial blur): round k is one
// single-round call -- x, y and z passes in the two-pass, fused or per-axis
// kernels, whichever fits, as for the Gaussian -- that writes `requested`
// padded by (reps - k - 1) radii (clipped) into f32 scratch.  Inside a round
// those kernels write exactly the intermediate regions of passes (k, x),
// (k, y), (k, z) of the per-axis schedule (binomial_blur.rs:63-87) and round
// each pass to f32, so the result is the schedule's.
static itkg_status run_rounds(const itkg_image& in, const itkg_region& largest,
                              const itkg_region& requested, const itkg_gaussian_params& prm,
                              const Plan& plan, const itkg_image& out, cudaStream_t s) {
  const int D = in.dim;
  const uint64_t reps = plan.reps;
  Plan one = plan;
  one.reps = 1;
  auto round_region = [&](uint64_t k) {
    if (k + 1 == reps) return requested;
    uint64_t pad[kMaxDim] = {0, 0, 0};
    for (int d = 0; d < D; ++d) pad[d] = (reps - k - 1) * plan.radii[d];
    return clipped(padded(requested, D, pad), D, largest);
  };
  itkg_image bufs[2];
  void* mem[2] = {nullptr, nullptr};
  size_t bytes = 0;
  for (int i = 0; i < 2; ++i) {
    std::memset(&bufs[i], 0, sizeof bufs[i]);
    bufs[i].dim = D;
    bufs[i].dtype = ITKG_F32;
    bufs[i].components = in.components;
    bufs[i].location = ITKG_DEVICE;
    for (int d = 0; d < D; ++d) bufs[i].spacing[d] = in.spacing[d];
  }
  {
    itkg_image probe = bufs[0];
    probe.region = round_region(0);  // the largest round region
    dense_layout(&probe, 16);
    bytes = image_bytes(probe);
  }
  itkg_status st = scratch_alloc(&mem[0], bytes, s);
  if (st == ITKG_SUCCESS && reps > 2) st = scratch_alloc(&mem[1], bytes, s);
  itkg_image cur = in;
  for (uint64_t k = 0; k < reps && st == ITKG_SUCCESS; ++k) {
    const itkg_region rk = round_region(k);
    itkg_image nxt = out;
    if (k + 1 < reps) {
      nxt = bufs[k & 1];
      nxt.region = rk;
      dense_layout(&nxt, 16);
      nxt.data = mem[k & 1];
    }
    st = generate_device(cur, largest, rk, prm, one, nxt, s);
    cur = nxt;
  }
  scratch_free(mem[0], s);
  scratch_free(mem[1], s);
  return st;
}

static itkg_status generate_device(const itkg_image& in, const itkg_region& largest,
                                   const itkg_region& requested, const itkg_gaussian_params& prm,
                                   const Plan& plan, const itkg_image& out, cudaStream_t s) {
  const int D = in.dim;
  // The single-launch kernels run one round of a kernel that reads the same
  // backwards (their y and z passes index the weights by distance from the centre).
  if (!plan.symmetric || plan.reps == 0 ||
      (plan.reps > 1 && (prm.algorithm == ITKG_ALGO_PER_AXIS || prm.arithmetic == ITKG_ARITH_PIXEL_U8))) {
    if (prm.algorithm == ITKG_ALGO_FUSED || prm.algorithm == ITKG_ALGO_TWO_PASS || prm.algorithm == ITKG_ALGO_ONE_TRIP)
      return set_error(ITKG_ERROR_UNSUPPORTED,
                       "asymmetric kernels, zero rounds and u8 pixel arithmetic over several rounds run per axis only");
    return run_per_axis(in, largest, requested, prm, plan, out, s);
  }
  if (plan.reps > 1) return run_rounds(in, largest, requested, prm, plan, out, s);
  // u8 pixel arithmetic: the two-pass kernels when every tap has an f32
  // constant that reproduces its u8 products, else the per-axis passes
  if (prm.arithmetic == ITKG_ARITH_PIXEL_U8 && D == 3 &&
      (prm.algorithm == ITKG_ALGO_AUTO || prm.algorithm == ITKG_ALGO_TWO_PASS)) {
    FusedGeom g;
    make_fused_geom(in, largest, requested, prm, plan, out, &g);
    std::vector<float> c[kMaxDim];
    bool ok = true;
    for (int d = 0; d < D && ok; ++d) {
      c[d].resize(plan.w64[d].size());
      ok = u8_pixel_tap_consts(plan.w64[d].data(), (int)plan.w64[d].size(), c[d].data());
    }
    if (ok) {
      const float* w[kMaxDim] = {c[0].data(), c[1].data(), c[2].data()};
      if (launch_two_pass(g, w, s, /*dry_run=*/true) == ITKG_SUCCESS) return launch_two_pass(g, w, s, false);
    }
    if (prm.algorithm == ITKG_ALGO_TWO_PASS)
      return set_error(ITKG_ERROR_UNSUPPORTED, "the two-pass kernels do not cover this geometry");
  }
  if (prm.arithmetic != ITKG_ARITH_PIXEL_U8 && prm.algorithm != ITKG_ALGO_PER_AXIS) {
    FusedGeom g;
    make_fused_geom(in, largest, requested, prm, plan, out, &g);
    const float* w[kMaxDim] = {nullptr, nullptr, nullptr};
    for (int d = 0; d < D; ++d) w[d] = plan.w32[d].data();
    if (prm.algorithm == ITKG_ALGO_ONE_TRIP) {
      if (launch_one_trip(g, w, s, /*dry_run=*/true) == ITKG_SUCCESS) return launch_one_trip(g, w, s, false);
      return set_error(ITKG_ERROR_UNSUPPORTED, "the one-trip kernel does not cover this geometry");
    }
    if (prm.algorithm == ITKG_ALGO_AUTO || prm.algorithm == ITKG_ALGO_TWO_PASS) {
      if (launch_two_pass(g, w, s, /*dry_run=*/true) == ITKG_SUCCESS) return launch_two_pass(g, w, s, false);
      if (prm.algorithm == ITKG_ALGO_TWO_PASS)
        return set_error(ITKG_ERROR_UNSUPPORTED, "the two-pass kernels do not cover this geometry");
    }
    // 3-D with the 1-tap kernel [1] on z (SliceBySliceFilter): the 2-D kernel over every slice
    if (D == 3 && plan.radii[2] == 0 && plan.w64[2].size() == 1 && plan.w64[2][0] == 1.0 &&
        launch_fused2d(g, w, s, /*dry_run=*/true) == ITKG_SUCCESS)
      return launch_fused2d(g, w, s, false);
    itkg_status st = launch_fused(g, w, s, /*dry_run=*/true);
    if (st == ITKG_SUCCESS) return launch_fused(g, w, s, false);
    if (prm.algorithm == ITKG_ALGO_FUSED)
      return set_error(ITKG_ERROR_UNSUPPORTED, "no fused kernel covers this geometry");
  }
  return run_per_axis(in, largest, requested, prm, plan, out, s);
}

itkg_status tile2d_geom_for(const itkg_image& in, const itkg_region& largest, const itkg_region& requested,
                            const itkg_gaussian_params& prm, const itkg_image& out, FusedGeom* g,
                            std::vector<std::vector<float>>* weights) {
  if (prm.arithmetic == ITKG_ARITH_PIXEL_U8 || prm.algorithm == ITKG_ALGO_PER_AXIS) return ITKG_ERROR_UNSUPPORTED;
  const int D = in.dim;
  if (D != 2) return ITKG_ERROR_UNSUPPORTED;
  if (out.dim != D || out.components != in.components || region_len(requested, D) == 0 ||
      !region_contains(largest, requested, D) || !region_contains(out.region, requested, D))
    return ITKG_ERROR_UNSUPPORTED;
  Plan plan;
  KernelSpec ks;
  ks.sigma = prm.sigma;
  if (make_plan(in, requested, largest, ks, &plan) != ITKG_SUCCESS) return ITKG_ERROR_UNSUPPORTED;
  if (!plan.symmetric || !region_contains(in.region, plan.in_reg, D)) return ITKG_ERROR_UNSUPPORTED;
  make_fused_geom(in, largest, requested, prm, plan, out, g);
  const float* w[kMaxDim] = {nullptr, nullptr, nullptr};
  for (int d = 0; d < D; ++d) w[d] = plan.w32[d].data();
  if (launch_tile2d(*g, w, nullptr, /*dry_run=*/true) != ITKG_SUCCESS) return ITKG_ERROR_UNSUPPORTED;
  weights->assign(plan.w32, plan.w32 + D);
  return ITKG_SUCCESS;
}

itkg_status fused_geom_for(const itkg_image& in, const itkg_region& largest,
                           const itkg_region& requested, const itkg_gaussian_params& prm,
                           const itkg_image& out, FusedGeom* g,
                           std::vector<std::vector<float>>* weights) {
  if (prm.arithmetic == ITKG_ARITH_PIXEL_U8 || prm.algorithm == ITKG_ALGO_PER_AXIS)
    return ITKG_ERROR_UNSUPPORTED;
  const int D = in.dim;
  if (D != 3) return ITKG_ERROR_UNSUPPORTED;  // the multi-request kernels are 3-D
  if (out.dim != D || out.components != in.components || region_len(requested, D) == 0 ||
      !region_contains(largest, requested, D) || !region_contains(out.region, requested, D))
    return ITKG_ERROR_UNSUPPORTED;
  Plan plan;
  KernelSpec ks;
  ks.sigma = prm.sigma;
  if (make_plan(in, requested, largest, ks, &plan) != ITKG_SUCCESS) return ITKG_ERROR_UNSUPPORTED;
  if (!region_contains(in.region, plan.in_reg, D)) return ITKG_ERROR_UNSUPPORTED;
  make_fused_geom(in, largest, requested, prm, plan, out, g);
  const float* w[kMaxDim] = {nullptr, nullptr, nullptr};
  for (int d = 0; d < D; ++d) w[d] = plan.w32[d].data();
  if (launch_fused(*g, w, nullptr, /*dry_run=*/true) != ITKG_SUCCESS) return ITKG_ERROR_UNSUPPORTED;
  weights->assign(plan.w32, plan.w32 + D);
  return ITKG_SUCCESS;
}

// ---- host buffers: pipelined staging ---------------------------------------
// Helper streams of the current device for the staged host-buffer path, per
// host thread (created on a thread's first staged call, never destroyed), so
// that staged calls from several threads run side by side.
static itkg_status staging_streams(cudaStream_t out[3]) {
  thread_local std::vector<std::array<cudaStream_t, 3>> per_dev;
  int dev = 0;
  ITKG_CUDA(cudaGetDevice(&dev));
  if ((int)per_dev.size() <= dev) per_dev.resize(dev + 1, {nullptr, nullptr, nullptr});
  for (int i = 0; i < 3; ++i) {
    if (!per_dev[dev][i]) ITKG_CUDA(cudaStreamCreateWithFlags(&per_dev[dev][i], cudaStreamNonBlocking));
    out[i] = per_dev[dev][i];
  }
  return ITKG_SUCCESS;
}

// Timing-free events for the staged path, per thread and device, created once
// and reused: a call records each of its events once and ends with a stream
// synchronize that covers every stream it recorded on.
static itkg_status staging_event(size_t idx, cudaEvent_t* e) {
  thread_local std::vector<std::vector<cudaEvent_t>> per_dev;
  int dev = 0;
  ITKG_CUDA(cudaGetDevice(&dev));
  if ((int)per_dev.size() <= dev) per_dev.resize(dev + 1);
  std::vector<cudaEvent_t>& pool = per_dev[dev];
  while (pool.size() <= idx) {
    cudaEvent_t ne = nullptr;
    ITKG_CUDA(cudaEventCreateWithFlags(&ne, cudaEventDisableTiming));
    pool.push_back(ne);
  }
  *e = pool[idx];
  return ITKG_SUCCESS;
}

// Copies the kernels' fault word into a per-thread pinned word on stream s, so
// that a call which synchronises s anyway reads it with no second synchronous
// copy.  *word is valid once s has been synchronised.
static itkg_status fault_word_async(cudaStream_t s, const unsigned int** word) {
  thread_local unsigned int* pinned = nullptr;
  if (!pinned) ITKG_CUDA(cudaMallocHost(reinterpret_cast<void**>(&pinned), sizeof(unsigned int)));
  unsigned int* dev_word = nullptr;
  ITKG_TRY(device_fault_word(&dev_word));
  ITKG_CUDA(cudaMemcpyAsync(pinned, dev_word, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
  *word = pinned;
  return ITKG_SUCCESS;
}

// After the synchronize: a kernel that gave up on a bounded wait makes the call
// fail (and the fault word is cleared) instead of returning an incomplete result.
static itkg_status check_fault_word(const unsigned int* word) {
  if (!word || *word == 0) return ITKG_SUCCESS;
  unsigned int fault = 0;
  ITKG_TRY(fused_fault_flag(&fault, true));
  return set_error(ITKG_ERROR_TIMEOUT, "a kernel gave up waiting for a tile load");
}

// Slabs along axis D-1 for a host-buffer call: about 4 MiB of output each, at
// most 8, and at least 2 kernel lengths thick (1 = no pipelining).
static int staging_pieces(const itkg_image& out, const itkg_region& requested, int D) {
  const uint64_t n_last = requested.size[D - 1];
  const uint64_t bytes = region_len(requested, D) * (uint64_t)out.pitch[0];
  uint64_t p = bytes / (4ull << 20);
  if (p > 8) p = 8;
  if (p > n_last / 8) p = n_last / 8;
  return p < 2 ? 1 : (int)p;
}

// Host-buffer call in `pieces` slabs along axis D-1 (the split of stream_full,
// source.rs:81-98): slab k's new input slices are copied to the device on
// copy stream A, the slab is filtered on stream B once they have landed, and
// its output is copied back on stream C -- so host-to-device copies, filtering
// and device-to-host copies of different slabs overlap.  The result is the
// whole-request result (every slab clamps to the largest region).
static itkg_status generate_staged(const itkg_image* input, const itkg_region* largest,
                                   const itkg_region* requested, const KernelSpec& ks,
                                   const itkg_gaussian_params* prm, const Plan& plan, const itkg_image* output,
                                   int pieces, cudaStream_t s) {
  const int D = input->dim, L = D - 1;
  const bool host_in = input->location == ITKG_HOST;
  const bool host_out = output->location == ITKG_HOST;
  cudaStream_t hs[3];
  ITKG_TRY(staging_streams(hs));
  itkg_image din = *input, dout = *output;
  void* pin = nullptr;
  void* pout = nullptr;
  itkg_status st = ITKG_SUCCESS;
  if (host_in) {
    din.location = ITKG_DEVICE;
    din.region = plan.in_reg;
    dense_layout(&din, 16);
    st = scratch_alloc(&pin, image_bytes(din), s);
    din.data = pin;
  }
  if (st == ITKG_SUCCESS && host_out) {
    dout.location = ITKG_DEVICE;
    dout.region = *requested;
    dense_layout(&dout, 16);
    st = scratch_alloc(&pout, image_bytes(dout), s);
    dout.data = pout;
  }
  size_t n_events = 0;
  auto event = [&](cudaStream_t on, cudaEvent_t* e) -> itkg_status {
    ITKG_TRY(staging_event(n_events++, e));
    ITKG_CUDA(cudaEventRecord(*e, on));
    return ITKG_SUCCESS;
  };
  cudaEvent_t e0 = nullptr;
  if (st == ITKG_SUCCESS) st = event(s, &e0);  // prior work on s, and the scratch
  for (int i = 0; i < 3 && st == ITKG_SUCCESS; ++i) st = cuda_status(cudaStreamWaitEvent(hs[i], e0, 0), "wait");
  const uint64_t n_last = requested->size[L];
  int64_t copied_to = plan.in_reg.index[L];  // input slices below this are on the device
  for (int k = 0; k < pieces && st == ITKG_SUCCESS; ++k) {
    itkg_region rk = *requested;
    rk.index[L] = requested->index[L] + (int64_t)(n_last * k / pieces);
    rk.size[L] = n_last * (k + 1) / pieces - n_last * k / pieces;
    Plan pk;
    st = make_plan(din, rk, *largest, ks, &pk);
    if (st != ITKG_SUCCESS) break;
    cudaEvent_t ein = nullptr, eout = nullptr;
    if (host_in) {
      const int64_t end = pk.in_reg.index[L] + (int64_t)pk.in_reg.size[L];
      if (end > copied_to) {
        itkg_region cr = plan.in_reg;
        cr.index[L] = copied_to;
        cr.size[L] = (uint64_t)(end - copied_to);
        st = copy_region(din, *input, cr, hs[0]);
        copied_to = end;
      }
      if (st == ITKG_SUCCESS) st = event(hs[0], &ein);
      if (st == ITKG_SUCCESS) st = cuda_status(cudaStreamWaitEvent(hs[1], ein, 0), "wait");
    }
    if (st == ITKG_SUCCESS) st = generate_device(din, *largest, rk, *prm, pk, dout, hs[1]);
    if (st == ITKG_SUCCESS && host_out) {
      st = event(hs[1], &eout);
      if (st == ITKG_SUCCESS) st = cuda_status(cudaStreamWaitEvent(hs[2], eout, 0), "wait");
      if (st == ITKG_SUCCESS) st = copy_region(*output, dout, rk, hs[2]);
    }
  }
  // join: s waits for all three helper streams, then frees the scratch
  for (int i = 0; i < 3; ++i) {
    cudaEvent_t ej = nullptr;
    if (event(hs[i], &ej) == ITKG_SUCCESS) cudaStreamWaitEvent(s, ej, 0);
  }
  scratch_free(pin, s);
  scratch_free(pout, s);
  const unsigned int* fw = nullptr;
  if (st == ITKG_SUCCESS) st = fault_word_async(s, &fw);
  const cudaError_t es = cudaStreamSynchronize(s);
  if (st != ITKG_SUCCESS) return st;
  if (es != cudaSuccess) return cuda_status(es, "cudaStreamSynchronize");
  return check_fault_word(fw);
}

// ks: the kernels (NULL: the Gaussian of prm->sigma); prm: arithmetic,
// rounding and algorithm.
static itkg_status generate_region(const itkg_image* input, const itkg_region* largest,
                                   const itkg_region* requested, const KernelSpec* ks_in,
                                   const itkg_gaussian_params* prm, const itkg_image* output, cudaStream_t s) {
  ITKG_TRY(validate_image(input, "input"));
  ITKG_TRY(validate_image(output, "output"));
  ITKG_TRY(filter_components(input, "input"));
  ITKG_TRY(filter_components(output, "output"));
  ITKG_TRY(check_params(prm));
  KernelSpec gauss;
  gauss.sigma = prm->sigma;
  const KernelSpec& ks = ks_in ? *ks_in : gauss;
  if (!largest || !requested) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "region is NULL");
  const int D = input->dim;
  if (output->dim != D) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "input/output dim differ");
  if (output->components != input->components)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "input/output components differ");
  if (prm->arithmetic == ITKG_ARITH_PIXEL_U8) {
    if (input->dtype != ITKG_U8 || output->dtype != ITKG_U8)
      return set_error(ITKG_ERROR_INVALID_ARGUMENT, "u8 pixel arithmetic needs u8 input and output");
  } else if (output->dtype == ITKG_I16) {
    return set_error(ITKG_ERROR_UNSUPPORTED, "i16 output is not provided (the reference has no i16 NumericPixel)");
  }
  if (region_len(*requested, D) == 0) return ITKG_SUCCESS;
  if (!region_contains(*largest, *requested, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "requested region lies outside the largest region");
  if (!region_contains(output->region, *requested, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "output buffer does not contain the requested region");
  Plan plan;
  ITKG_TRY(make_plan(*input, *requested, *largest, ks, &plan));
  if (!region_contains(input->region, plan.in_reg, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT,
                     "input buffer does not cover input_region_for_output(requested)");

  const bool host_in = input->location == ITKG_HOST;
  const bool host_out = output->location == ITKG_HOST;
  if (!host_in && !host_out) return generate_device(*input, *largest, *requested, *prm, plan, *output, s);
  const int pieces = staging_pieces(*output, *requested, D);
  if (pieces > 1) return generate_staged(input, largest, requested, ks, prm, plan, output, pieces, s);

  // Stage host buffers through stream-ordered scratch.
  itkg_image din = *input, dout = *output;
  void* pin = nullptr;
  void* pout = nullptr;
  itkg_status st = ITKG_SUCCESS;
  if (host_in) {
    din.location = ITKG_DEVICE;
    din.region = plan.in_reg;
    dense_layout(&din, 16);
    st = scratch_alloc(&pin, image_bytes(din), s);
    if (st == ITKG_SUCCESS) {
      din.data = pin;
      st = copy_region(din, *input, plan.in_reg, s);
    }
  }
  if (st == ITKG_SUCCESS && host_out) {
    dout.location = ITKG_DEVICE;
    dout.region = *requested;
    dense_layout(&dout, 16);
    st = scratch_alloc(&pout, image_bytes(dout), s);
    if (st == ITKG_SUCCESS) dout.data = pout;
  }
  if (st == ITKG_SUCCESS) st = generate_device(din, *largest, *requested, *prm, plan, dout, s);
  if (st == ITKG_SUCCESS && host_out) st = copy_region(*output, dout, *requested, s);
  scratch_free(pin, s);
  scratch_free(pout, s);
  if (st == ITKG_SUCCESS) {
    // The call synchronises anyway: surface a kernel that gave up on a
    // bounded wait instead of returning an incomplete result as success.
    const unsigned int* fw = nullptr;
    ITKG_TRY(fault_word_async(s, &fw));
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e, "cudaStreamSynchronize");
    return check_fault_word(fw);
  }
  // a failed call still returns only once no copy from or to the caller's
  // host buffers is in flight
  cudaStreamSynchronize(s);
  return st;
}

}  // namespace itkg

using namespace itkg;

extern "C" {

int32_t itkg_abi_version(void) { return ITKG_ABI_VERSION; }
const char* itkg_last_error(void) { return t_error.c_str(); }
const char* itkg_last_kernel(void) { return t_kernel.c_str(); }
uint64_t itkg_scratch_alloc_counter(void) { return g_scratch_allocs.load(std::memory_order_relaxed); }
void itkg_debug_fail_scratch_alloc(int64_t after) { g_fail_after.store(after < 0 ? -1 : after); }
void itkg_debug_set_wait_limit(int64_t cycles) { g_wait_limit.store(cycles > 0 ? cycles : (1ll << 31)); }
void itkg_debug_set_2d_kernel(int32_t which) { g_kernel2d.store(which == 1 || which == 2 ? which : 0); }
uint64_t itkg_launch_counter(void) { return g_launches.load(std::memory_order_relaxed); }

uint64_t itkg_kernel_radius(double sigma, double spacing) { return kernel_radius(sigma, spacing); }

itkg_status itkg_build_kernel(double sigma_pixels, uint64_t radius, double* weights_out) {
  if (!weights_out) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "weights_out is NULL");
  if (radius > (1u << 20)) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "radius too large");
  build_kernel(sigma_pixels, radius, weights_out);
  return ITKG_SUCCESS;
}

itkg_status itkg_region_padded_per_axis(const itkg_region* r, int32_t dim, const uint64_t* radii,
                                        itkg_region* out) {
  if (!r || !radii || !out || dim < 1 || dim > kMaxDim)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "bad argument");
  *out = padded(*r, dim, radii);
  return ITKG_SUCCESS;
}

itkg_status itkg_region_clipped_to(const itkg_region* r, int32_t dim, const itkg_region* bounds,
                                   itkg_region* out) {
  if (!r || !bounds || !out || dim < 1 || dim > kMaxDim)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "bad argument");
  *out = clipped(*r, dim, *bounds);
  return ITKG_SUCCESS;
}

itkg_status itkg_gaussian_input_region_for_output(const itkg_region* output_region,
                                                  const itkg_region* largest, int32_t dim,
                                                  const double* spacing, double sigma,
                                                  itkg_region* input_region) {
  if (!output_region || !largest || !spacing || !input_region || dim < 1 || dim > kMaxDim)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "bad argument");
  uint64_t radii[kMaxDim] = {0, 0, 0};
  for (int d = 0; d < dim; ++d) radii[d] = kernel_radius(sigma, spacing[d]);
  *input_region = clipped(padded(*output_region, dim, radii), dim, *largest);
  return ITKG_SUCCESS;
}

itkg_status itkg_split_region(const itkg_region* region, int32_t dim, uint64_t num_pieces,
                              itkg_region* pieces, uint64_t capacity, uint64_t* count) {
  if (!region || !count || dim < 1 || dim > kMaxDim)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "bad argument");
  num_pieces = num_pieces < 1 ? 1 : num_pieces;
  *count = 0;
  if (region_len(*region, dim) == 0) return ITKG_SUCCESS;
  const int slow = dim - 1;
  const uint64_t total = region->size[slow];
  uint64_t actual = std::min(num_pieces, total);
  actual = actual < 1 ? 1 : actual;
  const uint64_t base = total / actual, rem = total % actual;
  int64_t start = region->index[slow];
  for (uint64_t i = 0; i < actual; ++i) {
    const uint64_t sz = base + (i < rem ? 1 : 0);
    if (pieces && i < capacity) {
      pieces[i] = *region;
      pieces[i].index[slow] = start;
      pieces[i].size[slow] = sz;
    }
    start += (int64_t)sz;
  }
  *count = actual;
  return ITKG_SUCCESS;
}

itkg_status itkg_device_count(int32_t* count) {
  if (!count) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "count is NULL");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *count = 0;
    return ITKG_SUCCESS;
  }
  *count = n;
  return ITKG_SUCCESS;
}

itkg_status itkg_set_device(int32_t device) {
  ITKG_CUDA(cudaSetDevice(device));
  return ITKG_SUCCESS;
}

itkg_status itkg_device_alloc(size_t bytes, void** ptr) {
  if (!ptr) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "ptr is NULL");
  ITKG_CUDA(cudaMalloc(ptr, bytes ? bytes : 1));
  return ITKG_SUCCESS;
}

itkg_status itkg_device_free(void* ptr) {
  ITKG_CUDA(cudaFree(ptr));
  return ITKG_SUCCESS;
}

itkg_status itkg_host_alloc_pinned(size_t bytes, void** ptr) {
  if (!ptr) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "ptr is NULL");
  ITKG_CUDA(cudaMallocHost(ptr, bytes ? bytes : 1));
  return ITKG_SUCCESS;
}

itkg_status itkg_host_free_pinned(void* ptr) {
  ITKG_CUDA(cudaFreeHost(ptr));
  return ITKG_SUCCESS;
}

itkg_status itkg_memcpy(void* dst, const void* src, size_t bytes, int32_t kind, void* stream) {
  cudaMemcpyKind k = kind == 0   ? cudaMemcpyHostToDevice
                     : kind == 1 ? cudaMemcpyDeviceToHost
                     : kind == 2 ? cudaMemcpyDeviceToDevice
                                 : cudaMemcpyDefault;
  ITKG_CUDA(cudaMemcpyAsync(dst, src, bytes, k, static_cast<cudaStream_t>(stream)));
  return ITKG_SUCCESS;
}

itkg_status itkg_memset_device(void* dst, int32_t value, size_t bytes, void* stream) {
  ITKG_CUDA(cudaMemsetAsync(dst, value, bytes, static_cast<cudaStream_t>(stream)));
  return ITKG_SUCCESS;
}

itkg_status itkg_device_fault(int32_t clear, uint32_t* flag) {
  if (!flag) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "flag is NULL");
  unsigned int f = 0;
  ITKG_TRY(fused_fault_flag(&f, clear != 0));
  *flag = f;
  return ITKG_SUCCESS;
}

itkg_status itkg_stream_create(void** stream) {
  if (!stream) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "stream is NULL");
  cudaStream_t s = nullptr;
  ITKG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  *stream = s;
  return ITKG_SUCCESS;
}

itkg_status itkg_stream_destroy(void* stream) {
  if (stream) ITKG_CUDA(cudaStreamDestroy(static_cast<cudaStream_t>(stream)));
  return ITKG_SUCCESS;
}

itkg_status itkg_stream_synchronize(void* stream) {
  ITKG_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
  return ITKG_SUCCESS;
}

itkg_status itkg_image_alloc_device(itkg_image* img, int32_t dim, int32_t dtype, int32_t components,
                                    const itkg_region* region, const double* spacing,
                                    const double* origin) {
  if (!img || !region || dim < 1 || dim > kMaxDim || dtype_size(dtype) == 0 || components < 1 ||
      components > 3)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "bad argument");
  std::memset(img, 0, sizeof *img);
  img->dim = dim;
  img->dtype = dtype;
  img->components = components;
  img->location = ITKG_DEVICE;
  img->region = *region;
  for (int d = 0; d < kMaxDim; ++d) {
    img->spacing[d] = spacing ? (d < dim ? spacing[d] : 1.0) : 1.0;
    img->origin[d] = origin ? (d < dim ? origin[d] : 0.0) : 0.0;
  }
  dense_layout(img, 128);
  void* p = nullptr;
  ITKG_CUDA(cudaMalloc(&p, std::max<size_t>(image_bytes(*img), 128)));
  img->data = p;
  return ITKG_SUCCESS;
}

itkg_status itkg_image_free(itkg_image* img) {
  if (!img) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "img is NULL");
  if (img->data) ITKG_CUDA(cudaFree(img->data));
  img->data = nullptr;
  return ITKG_SUCCESS;
}

itkg_status itkg_image_copy_from(itkg_image* dst, const itkg_image* src, void* stream) {
  ITKG_TRY(validate_image(dst, "dst"));
  ITKG_TRY(validate_image(src, "src"));
  if (dst->dim != src->dim || dst->dtype != src->dtype || dst->components != src->components)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "copy_from: images differ in dim, dtype or components");
  if (!region_contains(dst->region, src->region, src->dim))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "copy_from: dst does not contain src's region");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  ITKG_TRY(copy_region(*dst, *src, src->region, s));
  ITKG_CUDA(cudaStreamSynchronize(s));
  return ITKG_SUCCESS;
}

itkg_status itkg_gaussian_generate_region(const itkg_image* input, const itkg_region* largest,
                                          const itkg_region* requested,
                                          const itkg_gaussian_params* params, itkg_image* output,
                                          void* stream) {
  return generate_region(input, largest, requested, nullptr, params, output,
                         static_cast<cudaStream_t>(stream));
}

itkg_status itkg_box_kernel(uint64_t radius, double* weights_out) {
  if (!weights_out) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "weights_out is NULL");
  if (radius > (1u << 20)) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "radius too large");
  const uint64_t len = 2 * radius + 1;  // mean.rs:15-18
  for (uint64_t k = 0; k < len; ++k) weights_out[k] = 1.0 / (double)len;
  return ITKG_SUCCESS;
}

itkg_status itkg_yvv_coeffs(double sigma, double* coeffs_out) {
  if (!coeffs_out) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "coeffs_out is NULL");
  yvv_coeffs(sigma, coeffs_out);
  return ITKG_SUCCESS;
}

itkg_status itkg_recursive_gaussian_generate_region(const itkg_image* input, const itkg_region* largest,
                                                    const itkg_region* requested,
                                                    const itkg_recursive_params* params, itkg_image* output,
                                                    void* stream) {
  ITKG_TRY(validate_image(input, "input"));
  ITKG_TRY(validate_image(output, "output"));
  if (!params) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "params is NULL");
  if (!largest || !requested) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "region is NULL");
  const int D = input->dim;
  if (output->dim != D) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "input/output dim differ");
  if (input->components != 1 || output->components != 1)
    return set_error(ITKG_ERROR_UNSUPPORTED, "the recursive Gaussian takes scalar pixels");
  if (params->rounding != ITKG_ROUND_REFERENCE && params->rounding != ITKG_ROUND_FMA)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "unknown rounding %d", params->rounding);
  if (params->axis < -1 || params->axis >= D)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "axis %d outside [-1, %d]", params->axis, D - 1);
  if (params->reserved[0] != 0 || params->reserved[1] != 0)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "reserved must be 0");
  if (output->dtype != ITKG_F32 && output->dtype != ITKG_U8)
    return set_error(ITKG_ERROR_UNSUPPORTED, "output dtype %d: f32 and u8 are provided", output->dtype);
  if (region_len(*requested, D) == 0) return ITKG_SUCCESS;
  if (!region_contains(*largest, *requested, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "requested region lies outside the largest region");
  if (!region_contains(output->region, *requested, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "output buffer does not contain the requested region");
  // the reference filters the whole largest region (recursive_gaussian.rs:148-150)
  if (!region_contains(input->region, *largest, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "input buffer does not cover the largest region");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool host_in = input->location == ITKG_HOST, host_out = output->location == ITKG_HOST;
  itkg_image din = *input, dout = *output;
  void* pin = nullptr;
  void* pout = nullptr;
  itkg_status st = ITKG_SUCCESS;
  if (host_in) {
    din.location = ITKG_DEVICE;
    din.region = *largest;
    dense_layout(&din, 16);
    st = scratch_alloc(&pin, image_bytes(din), s);
    din.data = pin;
    if (st == ITKG_SUCCESS) st = copy_region(din, *input, *largest, s);
  }
  if (st == ITKG_SUCCESS && host_out) {
    dout.location = ITKG_DEVICE;
    dout.region = *requested;
    dense_layout(&dout, 16);
    st = scratch_alloc(&pout, image_bytes(dout), s);
    dout.data = pout;
  }
  if (st == ITKG_SUCCESS)
    st = launch_recursive(din, *largest, *requested, params->sigma, params->axis, params->rounding, dout, s);
  if (st == ITKG_SUCCESS && host_out) st = copy_region(*output, dout, *requested, s);
  scratch_free(pin, s);
  scratch_free(pout, s);
  if (st == ITKG_SUCCESS && (host_in || host_out)) ITKG_CUDA(cudaStreamSynchronize(s));
  return st;
}

itkg_status itkg_recursive_gaussian_derivative_generate_region(const itkg_image* input, const itkg_region* largest,
                                                               const itkg_region* requested,
                                                               const itkg_recursive_derivative_params* params,
                                                               itkg_image* output, void* stream) {
  ITKG_TRY(validate_image(input, "input"));
  if (!output) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "output is NULL");
  if (!params) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "params is NULL");
  if (!largest || !requested) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "region is NULL");
  const int D = input->dim;
  const int kind = params->kind;
  if (kind < ITKG_REC_GRADIENT_MAGNITUDE || kind > ITKG_REC_ZERO_CROSSING_EDGES)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "unknown kind %d", kind);
  if (kind == ITKG_REC_HESSIAN && D != 2)
    return set_error(ITKG_ERROR_UNSUPPORTED, "the Hessian filter is 2-D (edges.rs:905)");
  if (kind == ITKG_REC_DERIVATIVE && (params->axis < 0 || params->axis >= D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "axis %d outside [0, %d)", params->axis, D);
  if (params->rounding != ITKG_ROUND_REFERENCE && params->rounding != ITKG_ROUND_FMA)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "unknown rounding %d", params->rounding);
  if (params->reserved[0] != 0 || params->reserved[1] != 0)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "reserved must be 0");
  if (input->components != 1 || (input->dtype != ITKG_F32 && input->dtype != ITKG_U8))
    return set_error(ITKG_ERROR_UNSUPPORTED, "the smoothed image is scalar f32 or u8 (its NumericPixel)");
  // the output: the pixel type for the scalar filters, f32 vectors for the gradient and the Hessian
  const bool scalar_out =
      kind <= ITKG_REC_DERIVATIVE || kind == ITKG_REC_DIFFERENCE_OF_GAUSSIANS || kind == ITKG_REC_ZERO_CROSSING_EDGES;
  const int want_dtype = scalar_out ? input->dtype : ITKG_F32;
  const int want_comps = scalar_out ? 1 : (kind == ITKG_REC_GRADIENT ? D : 3);
  if (output->dim != D || output->dtype != want_dtype || output->components != want_comps)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "output must be dim %d, dtype %d, %d component(s)", D, want_dtype,
                     want_comps);
  if (output->location != ITKG_DEVICE && output->location != ITKG_HOST)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "output: unknown location");
  if (output->pitch[0] != (int64_t)want_comps * dtype_size(want_dtype))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "output: pitch[0] must equal the pixel size");
  for (int d = 1; d < D; ++d)
    if (output->pitch[d] <= 0) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "output: pitch[%d] invalid", d);
  if (region_len(*requested, D) == 0) return ITKG_SUCCESS;
  if (!output->data) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "output: data is NULL");
  if (!region_contains(*largest, *requested, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "requested region lies outside the largest region");
  if (!region_contains(output->region, *requested, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "output buffer does not contain the requested region");
  if (!region_contains(input->region, *largest, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "input buffer does not cover the largest region");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool host_in = input->location == ITKG_HOST, host_out = output->location == ITKG_HOST;
  itkg_image din = *input, dout = *output;
  void* pin = nullptr;
  void* pout = nullptr;
  itkg_status st = ITKG_SUCCESS;
  if (host_in) {
    din.location = ITKG_DEVICE;
    din.region = *largest;
    dense_layout(&din, 16);
    st = scratch_alloc(&pin, image_bytes(din), s);
    din.data = pin;
    if (st == ITKG_SUCCESS) st = copy_region(din, *input, *largest, s);
  }
  if (st == ITKG_SUCCESS && host_out) {
    dout.location = ITKG_DEVICE;
    dout.region = *requested;
    dense_layout(&dout, 16);
    st = scratch_alloc(&pout, image_bytes(dout), s);
    dout.data = pout;
  }
  if (st == ITKG_SUCCESS)
    st = launch_recursive_derivative(din, *largest, *requested, params->sigma, params->sigma2, kind, params->axis,
                                     params->order, params->rounding, dout, s);
  if (st == ITKG_SUCCESS && host_out) st = copy_region(*output, dout, *requested, s);
  scratch_free(pin, s);
  scratch_free(pout, s);
  if (st == ITKG_SUCCESS && (host_in || host_out)) ITKG_CUDA(cudaStreamSynchronize(s));
  return st;
}

itkg_status itkg_separable_input_region_for_output(const itkg_region* output_region,
                                                   const itkg_region* largest, int32_t dim,
                                                   const uint64_t* radius, uint64_t repetitions,
                                                   itkg_region* input_region) {
  if (!output_region || !largest || !radius || !input_region || dim < 1 || dim > kMaxDim)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "bad argument");
  uint64_t pad[kMaxDim] = {0, 0, 0};
  for (int d = 0; d < dim; ++d) {
    if (radius[d] > (1u << 20) || repetitions > (1u << 20))
      return set_error(ITKG_ERROR_INVALID_ARGUMENT, "radius or repetitions too large");
    pad[d] = radius[d] * repetitions;
  }
  *input_region = clipped(padded(*output_region, dim, pad), dim, *largest);
  return ITKG_SUCCESS;
}

itkg_status itkg_separable_generate_region(const itkg_image* input, const itkg_region* largest,
                                           const itkg_region* requested,
                                           const itkg_separable_params* params, itkg_image* output,
                                           void* stream) {
  if (!params) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "params is NULL");
  if (!input) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "input is NULL");
  KernelSpec ks;
  ks.gaussian = false;
  ks.reps = params->repetitions;
  if (params->repetitions > (1u << 20))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "repetitions %llu is too large",
                     (unsigned long long)params->repetitions);
  for (int d = 0; d < kMaxDim; ++d) {
    if (d >= input->dim) continue;
    if (params->radius[d] > (1u << 20))
      return set_error(ITKG_ERROR_INVALID_ARGUMENT, "radius %llu on axis %d is too large",
                       (unsigned long long)params->radius[d], d);
    if (!params->weights[d]) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "weights[%d] is NULL", d);
    if (params->radius[d] * params->repetitions > (1u << 20))
      return set_error(ITKG_ERROR_INVALID_ARGUMENT, "radius x repetitions on axis %d is too large", d);
    ks.radius[d] = params->radius[d];
    ks.w[d] = params->weights[d];
  }
  itkg_gaussian_params opts;
  std::memset(&opts, 0, sizeof opts);
  opts.arithmetic = params->arithmetic;
  opts.rounding = params->rounding;
  opts.algorithm = params->algorithm;
  opts.reserved = params->reserved;
  return generate_region(input, largest, requested, &ks, &opts, output, static_cast<cudaStream_t>(stream));
}

itkg_status itkg_unsharp_kernel(double sigma, uint64_t* radius_out, double* weights_out, uint64_t capacity) {
  if (!radius_out) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "radius_out is NULL");
  if (!(sigma > 0.0) || !std::isfinite(sigma))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "sigma must be finite and > 0 (got %g)", sigma);
  // radius = (3.0 * sigma).ceil() as usize (edges.rs:408)
  const double rr = std::ceil(3.0 * sigma);
  if (rr > (double)(1u << 20)) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "sigma %g gives too large a radius", sigma);
  const uint64_t r = (uint64_t)rr;
  *radius_out = r;
  if (!weights_out) return ITKG_SUCCESS;
  if (capacity < 2 * r + 1)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "weights_out holds %llu weights, %llu needed",
                     (unsigned long long)capacity, (unsigned long long)(2 * r + 1));
  // edges.rs:416-424: exp(-(d * d) / (2 sigma sigma)), then divided by the
  // left-to-right f64 sum (this file is compiled without FP contraction).
  const double two_s2 = 2.0 * sigma * sigma;
  for (uint64_t i = 0; i <= 2 * r; ++i) {
    const double d = (double)i - (double)r;
    weights_out[i] = std::exp(-(d * d) / two_s2);
  }
  double sum = 0.0;
  for (uint64_t i = 0; i <= 2 * r; ++i) sum += weights_out[i];
  for (uint64_t i = 0; i <= 2 * r; ++i) weights_out[i] /= sum;
  return ITKG_SUCCESS;
}

itkg_status itkg_unsharp_mask_generate_region(const itkg_image* input, const itkg_region* largest,
                                              const itkg_region* requested, const itkg_unsharp_params* params,
                                              itkg_image* output, void* stream) {
  if (!params) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "params is NULL");
  ITKG_TRY(validate_image(input, "input"));
  ITKG_TRY(validate_image(output, "output"));
  // the point-wise kernels take scalar and 3-component pixels
  const itkg_image* const ims[2] = {input, output};
  for (const itkg_image* im : ims)
    if (im->components != 1 && im->components != 3)
      return set_error(ITKG_ERROR_UNSUPPORTED, "UnsharpMaskFilter: components must be 1 or 3");
  if (!largest || !requested) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "region is NULL");
  if (params->reserved != 0) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "reserved must be 0");
  if (params->rounding != ITKG_ROUND_REFERENCE && params->rounding != ITKG_ROUND_FMA)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "unknown rounding %d", params->rounding);
  if (input->dtype != ITKG_F32 && input->dtype != ITKG_U8)
    return set_error(ITKG_ERROR_UNSUPPORTED, "the pixel type is f32 or u8");
  if (output->dtype != input->dtype || output->components != input->components || output->dim != input->dim)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "output must have the input's dim, dtype and components");
  const int D = input->dim;
  uint64_t r = 0;
  ITKG_TRY(itkg_unsharp_kernel(params->sigma, &r, nullptr, 0));
  std::vector<double> w(2 * r + 1);
  ITKG_TRY(itkg_unsharp_kernel(params->sigma, &r, w.data(), w.size()));
  if (region_len(*requested, D) == 0) return ITKG_SUCCESS;
  if (!region_contains(*largest, *requested, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "requested region lies outside the largest region");
  if (!region_contains(output->region, *requested, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "output buffer does not contain the requested region");
  uint64_t pad[kMaxDim] = {r, r, r};
  const itkg_region in_reg = clipped(padded(*requested, D, pad), D, *largest);
  if (!region_contains(input->region, in_reg, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "input buffer does not cover input_region_for_output(requested)");

  KernelSpec ks;
  ks.gaussian = false;
  ks.reps = 1;
  for (int d = 0; d < D; ++d) {
    ks.radius[d] = r;
    ks.w[d] = w.data();
  }
  itkg_gaussian_params opts;
  std::memset(&opts, 0, sizeof opts);
  opts.arithmetic = input->dtype == ITKG_U8 ? ITKG_ARITH_PIXEL_U8 : ITKG_ARITH_F32;
  opts.rounding = params->rounding;
  opts.algorithm = ITKG_ALGO_AUTO;

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool host_in = input->location == ITKG_HOST, host_out = output->location == ITKG_HOST;
  itkg_image din = *input, dout = *output, blur = *input;
  void* pin = nullptr;
  void* pout = nullptr;
  void* pblur = nullptr;
  itkg_status st = ITKG_SUCCESS;
  if (host_in) {
    din.location = ITKG_DEVICE;
    din.region = in_reg;
    dense_layout(&din, 16);
    st = scratch_alloc(&pin, image_bytes(din), s);
    din.data = pin;
    if (st == ITKG_SUCCESS) st = copy_region(din, *input, in_reg, s);
  }
  if (st == ITKG_SUCCESS && host_out) {
    dout.location = ITKG_DEVICE;
    dout.region = *requested;
    dense_layout(&dout, 16);
    st = scratch_alloc(&pout, image_bytes(dout), s);
    dout.data = pout;
  }
  // 3-D f32: the two-pass blur whose z kernel stores the point-wise step
  // directly (no blur image in memory)
  bool fused = false;
  if (st == ITKG_SUCCESS && D == 3 && input->dtype == ITKG_F32 && input->components == 1) {
    const UnsharpConsts k = unsharp_consts(params->amount, params->threshold, params->rounding == ITKG_ROUND_FMA);
    Plan plan;
    if (k.fast && make_plan(din, *requested, *largest, ks, &plan) == ITKG_SUCCESS && plan.symmetric &&
        plan.reps == 1) {
      FusedGeom g;
      make_fused_geom(din, *largest, *requested, opts, plan, dout, &g);
      const float* wz[kMaxDim] = {plan.w32[0].data(), plan.w32[1].data(), plan.w32[2].data()};
      if (launch_two_pass(g, wz, s, /*dry_run=*/true, &k) == ITKG_SUCCESS) {
        st = launch_two_pass(g, wz, s, false, &k);
        fused = true;
      }
    }
  }
  if (st == ITKG_SUCCESS && !fused) {
    blur.location = ITKG_DEVICE;
    blur.region = *requested;
    dense_layout(&blur, 16);
    st = scratch_alloc(&pblur, image_bytes(blur), s);
    blur.data = pblur;
  }
  if (st == ITKG_SUCCESS && !fused) st = generate_region(&din, largest, requested, &ks, &opts, &blur, s);
  if (st == ITKG_SUCCESS && !fused) {
    auto at = [&](const itkg_image& im) {
      int64_t off = 0;
      for (int d = 0; d < D; ++d) off += (requested->index[d] - im.region.index[d]) * im.pitch[d];
      return static_cast<char*>(im.data) + off;
    };
    int64_t ip[kMaxDim] = {0, 0, 0}, bp[kMaxDim] = {0, 0, 0}, op[kMaxDim] = {0, 0, 0}, m[kMaxDim] = {1, 1, 1};
    for (int d = 0; d < D; ++d) {
      ip[d] = din.pitch[d];
      bp[d] = blur.pitch[d];
      op[d] = dout.pitch[d];
      m[d] = (int64_t)requested->size[d];
    }
    st = launch_unsharp(input->dtype, input->components, at(din), ip, at(blur), bp, at(dout), op, m, params->amount,
                        params->threshold, params->rounding, s);
  }
  if (st == ITKG_SUCCESS && host_out) st = copy_region(*output, dout, *requested, s);
  scratch_free(pblur, s);
  scratch_free(pin, s);
  scratch_free(pout, s);
  if (st == ITKG_SUCCESS && (host_in || host_out)) {
    const unsigned int* fw = nullptr;
    ITKG_TRY(fault_word_async(s, &fw));
    const cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e, "cudaStreamSynchronize");
    return check_fault_word(fw);
  }
  return st;
}

itkg_status itkg_slice_by_slice_generate_region(const itkg_image* input, const itkg_region* requested,
                                               const itkg_gaussian_params* params, itkg_image* output,
                                               void* stream) {
  ITKG_TRY(validate_image(input, "input"));
  ITKG_TRY(check_params(params));
  if (!requested) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "requested is NULL");
  if (input->dim != 3) return set_error(ITKG_ERROR_UNSUPPORTED, "SliceBySliceFilter is 3-D (spatial.rs:1295)");
  // Each z slice of `requested` is a 2-D Image whose region is the request's
  // x-y window (spatial.rs:1317-1323), smoothed by GaussianFilter with the x
  // and y spacing: one round of the 2-D Gaussian's kernels on x and y, the
  // 1-tap kernel [1] on z, clamped to the request itself.
  uint64_t r[kMaxDim] = {0, 0, 0};
  std::vector<double> w[kMaxDim];
  for (int d = 0; d < 2; ++d) {
    r[d] = kernel_radius(params->sigma, input->spacing[d]);
    if (r[d] > (1u << 20))
      return set_error(ITKG_ERROR_INVALID_ARGUMENT, "kernel radius %llu on axis %d is not allocatable",
                       (unsigned long long)r[d], d);
    w[d].resize(2 * r[d] + 1);
    build_kernel(params->sigma / input->spacing[d], r[d], w[d].data());
  }
  w[2].assign(1, 1.0);
  KernelSpec ks;
  ks.gaussian = false;
  ks.reps = 1;
  for (int d = 0; d < 3; ++d) {
    ks.radius[d] = r[d];
    ks.w[d] = w[d].data();
  }
  itkg_gaussian_params opts = *params;
  opts.sigma = 0.0;
  return generate_region(input, requested, requested, &ks, &opts, output, static_cast<cudaStream_t>(stream));
}

itkg_status itkg_bspline_downsample_generate_region(const itkg_image* input, const itkg_region* largest,
                                                    const itkg_gaussian_params* params, itkg_image* output,
                                                    void* stream) {
  ITKG_TRY(validate_image(input, "input"));
  ITKG_TRY(validate_image(output, "output"));
  ITKG_TRY(filter_components(input, "input"));
  ITKG_TRY(filter_components(output, "output"));
  ITKG_TRY(check_params(params));
  if (!largest) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "largest is NULL");
  const int D = input->dim;
  if (output->dim != D || output->components != input->components)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "output must have the input's dim and components");
  // the downsampled largest region (spatial.rs:1142-1147)
  itkg_region half = *largest;
  for (int d = 0; d < D; ++d) half.size[d] = (largest->size[d] + 1) / 2;
  if (region_len(half, D) == 0) return ITKG_SUCCESS;
  if (!region_contains(output->region, half, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "output buffer does not contain the downsampled largest region");
  if (!region_contains(input->region, *largest, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "input buffer does not cover the largest region");
  // GaussianFilter { sigma: 1.0 } over the whole largest region (spatial.rs:1157-1158), in the output's
  // pixel type, into device scratch; then every other voxel
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  itkg_gaussian_params g = *params;
  g.sigma = 1.0;
  itkg_image sm = *output;
  sm.location = ITKG_DEVICE;
  sm.region = *largest;
  dense_layout(&sm, 16);
  void* psm = nullptr;
  ITKG_TRY(scratch_alloc(&psm, image_bytes(sm), s));
  sm.data = psm;
  itkg_status st = generate_region(input, largest, largest, nullptr, &g, &sm, s);
  itkg_image dout = *output;
  void* pout = nullptr;
  const bool host_out = output->location == ITKG_HOST;
  if (st == ITKG_SUCCESS && host_out) {
    dout.location = ITKG_DEVICE;
    dout.region = half;
    dense_layout(&dout, 16);
    st = scratch_alloc(&pout, image_bytes(dout), s);
    dout.data = pout;
  }
  if (st == ITKG_SUCCESS) {
    int64_t sp[kMaxDim] = {0, 0, 0}, dp[kMaxDim] = {0, 0, 0}, m[kMaxDim] = {1, 1, 1};
    char* dst = static_cast<char*>(dout.data);
    for (int d = 0; d < D; ++d) {
      sp[d] = sm.pitch[d];
      dp[d] = dout.pitch[d];
      m[d] = (int64_t)half.size[d];
      dst += (half.index[d] - dout.region.index[d]) * dout.pitch[d];
    }
    st = launch_subsample2(sm.data, sp, dst, dp, m, output->components * dtype_size(output->dtype), s);
  }
  if (st == ITKG_SUCCESS && host_out) st = copy_region(*output, dout, half, s);
  scratch_free(psm, s);
  scratch_free(pout, s);
  if (st == ITKG_SUCCESS && (host_out || input->location == ITKG_HOST)) ITKG_CUDA(cudaStreamSynchronize(s));
  if (st == ITKG_SUCCESS) set_last_kernel("subsample2");
  return st;
}

itkg_status itkg_stream_full(const itkg_image* input, const itkg_region* largest,
                             const itkg_gaussian_params* params, uint64_t num_pieces,
                             itkg_image* output, void* stream) {
  ITKG_TRY(validate_image(input, "input"));
  ITKG_TRY(validate_image(output, "output"));
  ITKG_TRY(filter_components(input, "input"));
  ITKG_TRY(filter_components(output, "output"));
  if (!largest) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "largest is NULL");
  const int D = input->dim;
  if (!region_contains(output->region, *largest, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "output buffer does not contain the largest region");
  uint64_t count = 0;
  ITKG_TRY(itkg_split_region(largest, D, num_pieces, nullptr, 0, &count));
  std::vector<itkg_region> pieces(count);
  ITKG_TRY(itkg_split_region(largest, D, num_pieces, pieces.data(), count, &count));
  for (const itkg_region& p : pieces)
    ITKG_TRY(generate_region(input, largest, &p, nullptr, params, output, static_cast<cudaStream_t>(stream)));
  return ITKG_SUCCESS;
}


// ---- in-crate callers that iterate around the Gaussian -----------------------

namespace {
// A 2-D f32 scalar image on the device for a point-wise kernel: the image
// itself, or a dense copy of `reg` in scratch (*owned) when it is host memory.
itkg_status device_view(const itkg_image& im, const itkg_region& reg, cudaStream_t s, itkg_image* out, void** owned) {
  *out = im;
  *owned = nullptr;
  if (im.location == ITKG_DEVICE) return ITKG_SUCCESS;
  out->location = ITKG_DEVICE;
  out->region = reg;
  dense_layout(out, 16);
  ITKG_TRY(scratch_alloc(owned, image_bytes(*out), s));
  out->data = *owned;
  return copy_region(*out, im, reg, s);
}

const float* first_pixel(const itkg_image& im, const itkg_region& reg) {
  return reinterpret_cast<const float*>(static_cast<const char*>(im.data) +
                                        (reg.index[0] - im.region.index[0]) * im.pitch[0] +
                                        (reg.index[1] - im.region.index[1]) * im.pitch[1]);
}

itkg_status check_f32_2d(const itkg_image* im, const char* name, int comps) {
  ITKG_TRY(validate_image(im, name));
  if (im->dim != 2 || im->dtype != ITKG_F32 || im->components != comps)
    return set_error(ITKG_ERROR_UNSUPPORTED, "%s must be a 2-D f32 image with %d component(s)", name, comps);
  if (im->pitch[1] % 4 != 0) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s: row pitch not a multiple of 4", name);
  return ITKG_SUCCESS;
}
}  // namespace

itkg_status itkg_demons_registration(const itkg_image* fixed, const itkg_image* moving, int32_t iterations,
                                     double max_step_length, int32_t diffeomorphic, double sigma_diff,
                                     itkg_image* displacement, void* stream) {
  ITKG_TRY(check_f32_2d(fixed, "fixed", 1));
  ITKG_TRY(check_f32_2d(moving, "moving", 1));
  ITKG_TRY(check_f32_2d(displacement, "displacement", 2));
  if (iterations < 0) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "iterations < 0");
  const itkg_region freg = fixed->region, mreg = moving->region;
  if (!region_contains(displacement->region, freg, 2))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "displacement buffer does not contain the fixed image's region");
  const int64_t w = (int64_t)freg.size[0], h = (int64_t)freg.size[1], n = w * h;
  if (n == 0) return ITKG_SUCCESS;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  itkg_image fd, md;
  void *pf = nullptr, *pm = nullptr, *pd = nullptr, *pw = nullptr, *pout = nullptr;
  itkg_status st = device_view(*fixed, freg, s, &fd, &pf);
  if (st == ITKG_SUCCESS) st = device_view(*moving, mreg, s, &md, &pm);
  // displacement (x, y) in f64, two generations, and the error word
  const size_t dbytes = (size_t)n * sizeof(double);
  if (st == ITKG_SUCCESS) st = scratch_alloc(&pd, 4 * dbytes + 256, s);
  double* d[4] = {nullptr, nullptr, nullptr, nullptr};
  unsigned int* err = nullptr;
  if (st == ITKG_SUCCESS) {
    for (int k = 0; k < 4; ++k) d[k] = reinterpret_cast<double*>(static_cast<char*>(pd) + k * dbytes);
    err = reinterpret_cast<unsigned int*>(static_cast<char*>(pd) + 4 * dbytes);
    st = cuda_status(cudaMemsetAsync(pd, 0, 4 * dbytes + 256, s), "cudaMemsetAsync");
  }
  DemonsGeom g;
  g.fixed = first_pixel(fd, freg);
  g.fp = fd.pitch[1] / 4;
  g.w = w;
  g.h = h;
  g.ox = freg.index[0];
  g.oy = freg.index[1];
  g.moving = first_pixel(md, mreg);
  g.mp = md.pitch[1] / 4;
  g.mw = (int64_t)mreg.size[0];
  g.mh = (int64_t)mreg.size[1];
  g.mox = mreg.index[0];
  g.moy = mreg.index[1];
  int cur = 0;  // d[cur], d[cur + 1] hold the current field
  for (int it = 0; it < iterations && st == ITKG_SUCCESS; ++it) {
    st = launch_demons_step(g, d[cur], d[cur + 1], d[2 - cur], d[3 - cur], max_step_length, err, s);
    cur = 2 - cur;
  }
  // the output buffer (device, or a dense scratch copy of the fixed region)
  itkg_image dout = *displacement;
  if (st == ITKG_SUCCESS && displacement->location == ITKG_HOST) {
    dout.location = ITKG_DEVICE;
    dout.region = freg;
    dense_layout(&dout, 16);
    st = scratch_alloc(&pout, image_bytes(dout), s);
    dout.data = pout;
  }
  float* const o = const_cast<float*>(first_pixel(dout, freg));
  const int64_t op = dout.pitch[1] / 8;
  if (st == ITKG_SUCCESS && !diffeomorphic) {
    st = launch_demons_to_f32(d[cur], d[cur + 1], w, h, o, op, nullptr, nullptr, 0, s);
  } else if (st == ITKG_SUCCESS) {
    // DiffeomorphicDemonsRegistrationFilter (registration_methods.rs:126-148):
    // GaussianFilter { sigma: sigma_diff } over each component's whole image
    itkg_image comp;
    std::memset(&comp, 0, sizeof comp);
    comp.dim = 2;
    comp.dtype = ITKG_F32;
    comp.components = 1;
    comp.location = ITKG_DEVICE;
    comp.region = freg;
    comp.spacing[0] = fixed->spacing[0];
    comp.spacing[1] = fixed->spacing[1];
    comp.origin[0] = fixed->origin[0];
    comp.origin[1] = fixed->origin[1];
    dense_layout(&comp, 16);
    const size_t cb = image_bytes(comp);
    st = scratch_alloc(&pw, 4 * cb, s);
    if (st == ITKG_SUCCESS) {
      itkg_image raw[2] = {comp, comp}, sm[2] = {comp, comp};
      for (int c = 0; c < 2; ++c) {
        raw[c].data = static_cast<char*>(pw) + c * cb;
        sm[c].data = static_cast<char*>(pw) + (2 + c) * cb;
      }
      // planar components, rows at the dense pitch (w floats rounded up to 16 bytes)
      const int64_t cp = comp.pitch[1] / 4;
      st = launch_demons_to_f32(d[cur], d[cur + 1], w, h, nullptr, 0, static_cast<float*>(raw[0].data),
                                static_cast<float*>(raw[1].data), cp, s);
      itkg_gaussian_params gp;
      std::memset(&gp, 0, sizeof gp);
      gp.sigma = sigma_diff;
      gp.rounding = ITKG_ROUND_REFERENCE;
      for (int c = 0; c < 2 && st == ITKG_SUCCESS; ++c)
        st = generate_region(&raw[c], &freg, &freg, nullptr, &gp, &sm[c], s);
      if (st == ITKG_SUCCESS)
        st = launch_interleave2(static_cast<const float*>(sm[0].data), static_cast<const float*>(sm[1].data), cp, w, h,
                                o, op, s);
    }
  }
  if (st == ITKG_SUCCESS && displacement->location == ITKG_HOST) st = copy_region(*displacement, dout, freg, s);
  unsigned int herr = 0;
  if (st == ITKG_SUCCESS) st = cuda_status(cudaMemcpyAsync(&herr, err, sizeof herr, cudaMemcpyDeviceToHost, s), "copy");
  const cudaError_t es = cudaStreamSynchronize(s);
  scratch_free(pf, s);
  scratch_free(pm, s);
  scratch_free(pd, s);
  scratch_free(pw, s);
  scratch_free(pout, s);
  if (st != ITKG_SUCCESS) return st;
  if (es != cudaSuccess) return cuda_status(es, "cudaStreamSynchronize");
  if (herr)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT,
                     "a warped index left the moving image's buffer (the reference's Image::get_pixel panics here)");
  set_last_kernel(diffeomorphic ? "demons_diffeomorphic_f64" : "demons_step_f64");
  return ITKG_SUCCESS;
}

itkg_status itkg_n4_bias_field_correction(const itkg_image* input, const itkg_region* largest, int32_t iterations,
                                          double sigma, double convergence_threshold, itkg_image* output,
                                          int32_t* iterations_run, void* stream) {
  ITKG_TRY(check_f32_2d(input, "input", 1));
  ITKG_TRY(check_f32_2d(output, "output", 1));
  if (!largest) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "largest is NULL");
  if (iterations < 0) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "iterations < 0");
  if (!region_contains(input->region, *largest, 2))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "input buffer does not cover the largest region");
  if (!region_contains(output->region, *largest, 2))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "output buffer does not contain the largest region");
  if (iterations_run) *iterations_run = 0;
  const int64_t w = (int64_t)largest->size[0], h = (int64_t)largest->size[1], n = w * h;
  if (n == 0) return ITKG_SUCCESS;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  itkg_image in_d;
  void *pin = nullptr, *pbuf = nullptr, *pout = nullptr;
  itkg_status st = device_view(*input, *largest, s, &in_d, &pin);
  // log image and its smoothing as dense f32 images of the largest region
  itkg_image lf;
  std::memset(&lf, 0, sizeof lf);
  lf.dim = 2;
  lf.dtype = ITKG_F32;
  lf.components = 1;
  lf.location = ITKG_DEVICE;
  lf.region = *largest;
  for (int d = 0; d < 2; ++d) {
    lf.spacing[d] = input->spacing[d];
    lf.origin[d] = input->origin[d];
  }
  lf.pitch[0] = 4;
  lf.pitch[1] = 4 * w;
  lf.pitch[2] = 4 * n;
  itkg_image sm = lf;
  const int nb = n4_blocks(n);
  const size_t dbytes = (size_t)n * 8, fbytes = ((size_t)n * 4 + 255) / 256 * 256;
  if (st == ITKG_SUCCESS) st = scratch_alloc(&pbuf, 2 * dbytes + 2 * fbytes + (size_t)(nb + 1) * 8, s);
  double *corr = nullptr, *ld = nullptr, *part = nullptr;
  if (st == ITKG_SUCCESS) {
    char* b = static_cast<char*>(pbuf);
    corr = reinterpret_cast<double*>(b);
    ld = reinterpret_cast<double*>(b + dbytes);
    lf.data = b + 2 * dbytes;
    sm.data = b + 2 * dbytes + fbytes;
    part = reinterpret_cast<double*>(b + 2 * dbytes + 2 * fbytes);
    st = launch_n4_init(first_pixel(in_d, *largest), in_d.pitch[1] / 4, w, h, corr, s);
  }
  itkg_gaussian_params gp;
  std::memset(&gp, 0, sizeof gp);
  gp.sigma = sigma;
  gp.rounding = ITKG_ROUND_REFERENCE;
  int run = 0;
  for (int it = 0; it < iterations && st == ITKG_SUCCESS; ++it) {
    st = launch_n4_log(corr, n, ld, static_cast<float*>(lf.data), s);
    if (st == ITKG_SUCCESS) st = generate_region(&lf, largest, largest, nullptr, &gp, &sm, s);
    if (st == ITKG_SUCCESS) st = launch_n4_update(ld, static_cast<const float*>(sm.data), n, corr, part, nb, s);
    if (st == ITKG_SUCCESS) st = launch_sum_partials(part, nb, part + nb, false, s);
    double total = 0.0;
    if (st == ITKG_SUCCESS) st = cuda_status(cudaMemcpyAsync(&total, part + nb, 8, cudaMemcpyDeviceToHost, s), "copy");
    if (st == ITKG_SUCCESS) st = cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    ++run;
    // convergence (bias_correction.rs:76-78): mean absolute change
    if (st == ITKG_SUCCESS && total / (double)n < convergence_threshold) break;
  }
  itkg_image dout = *output;
  if (st == ITKG_SUCCESS && output->location == ITKG_HOST) {
    dout.location = ITKG_DEVICE;
    dout.region = *largest;
    dense_layout(&dout, 16);
    st = scratch_alloc(&pout, image_bytes(dout), s);
    dout.data = pout;
  }
  if (st == ITKG_SUCCESS)
    st = launch_n4_store(corr, w, h, const_cast<float*>(first_pixel(dout, *largest)), dout.pitch[1] / 4, s);
  if (st == ITKG_SUCCESS && output->location == ITKG_HOST) st = copy_region(*output, dout, *largest, s);
  const cudaError_t es = cudaStreamSynchronize(s);
  scratch_free(pin, s);
  scratch_free(pbuf, s);
  scratch_free(pout, s);
  if (st != ITKG_SUCCESS) return st;
  if (es != cudaSuccess) return cuda_status(es, "cudaStreamSynchronize");
  if (iterations_run) *iterations_run = run;
  set_last_kernel("n4_update_f64");
  return ITKG_SUCCESS;
}

}  // extern "C"
