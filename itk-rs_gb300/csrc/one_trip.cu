// Host side of the one-trip 3-D forward (kernel in one_trip.cuh): which
// requests it takes, the edge coefficients, the cost-balanced split of the
// (tile, slice) units over the resident CTAs, and the launch.  The kernel
// table is filled by one_trip_r*.cu (one translation unit per pair of x-y radii).
#include <algorithm>
#include <climits>

#include "one_trip.cuh"

namespace itkg {
namespace onetrip {

// one_trip_r*.cu: the kernel for (r, rz, ref), or NULL
Fn one_trip_fn_r12(int r, int rz, bool ref);
Fn one_trip_fn_r34(int r, int rz, bool ref);
Fn one_trip_fn_r56(int r, int rz, bool ref);
Fn one_trip_fn_r78(int r, int rz, bool ref);

Fn one_trip_fn(int r, int rz, bool ref) {
  switch (r) {
    case 1: case 2: return one_trip_fn_r12(r, rz, ref);
    case 3: case 4: return one_trip_fn_r34(r, rz, ref);
    case 5: case 6: return one_trip_fn_r56(r, rz, ref);
    case 7: case 8: return one_trip_fn_r78(r, rz, ref);
    default: return nullptr;
  }
}

size_t one_trip_smem(int r) {
  switch (r) {
    case 1: return Cfg<1, 1>::SMEM;
    case 2: return Cfg<2, 1>::SMEM;
    case 3: return Cfg<3, 1>::SMEM;
    case 4: return Cfg<4, 1>::SMEM;
    case 5: return Cfg<5, 1>::SMEM;
    case 6: return Cfg<6, 1>::SMEM;
    case 7: return Cfg<7, 1>::SMEM;
    default: return Cfg<8, 1>::SMEM;
  }
}

int one_trip_box_w(int r) { return kTX + 2 * ((r + 3) / 4 * 4) + 4; }

}  // namespace onetrip

namespace {
bool fits_i32(int64_t v) { return v >= INT_MIN && v <= INT_MAX; }
}  // namespace

itkg_status launch_one_trip(const FusedGeom& g, const float* const w[kMaxDim], void* stream, bool dry_run) {
  using namespace onetrip;
  if (g.dim != 3 || g.comps != 1 || g.in_dtype != ITKG_F32 || g.out_dtype == ITKG_I16 || g.u8pix)
    return ITKG_ERROR_UNSUPPORTED;
  const int R = g.radius[0], RZ = g.radius[2];
  if (g.radius[1] != R || R < 1 || R > kMaxR || RZ < 1 || RZ > kMaxRZ) return ITKG_ERROR_UNSUPPORTED;
  const bool ref = g.rounding == ITKG_ROUND_REFERENCE;
  const Fn fn = one_trip_fn(R, RZ, ref);
  if (!fn) return ITKG_ERROR_UNSUPPORTED;
  if (g.src_pitch[0] != 4) return ITKG_ERROR_UNSUPPORTED;
  // FMA rounding reads zeros outside the input buffer as the halo and adds the
  // clamped taps back at the image's edges: the buffer must lie inside the
  // image on x and y.
  if (!ref)
    for (int d = 0; d < 2; ++d)
      if (g.src_origin[d] < g.lo[d] || g.src_origin[d] + g.src_size[d] - 1 > g.hi[d]) return ITKG_ERROR_UNSUPPORTED;
  // TMA: 16-byte base and pitches; tile columns start 16-byte aligned
  if (((uintptr_t)g.src & 15) || (g.src_pitch[1] & 15) || (g.src_pitch[2] & 15)) return ITKG_ERROR_UNSUPPORTED;
  if (g.src_pitch[1] >= (1ll << 40) || g.src_pitch[2] >= (1ll << 40)) return ITKG_ERROR_UNSUPPORTED;
  if ((((g.req_index[0] - g.src_origin[0]) % 4) + 4) % 4 != 0) return ITKG_ERROR_UNSUPPORTED;
  for (int d = 0; d < 3; ++d)
    if (!fits_i32(g.lo[d]) || !fits_i32(g.hi[d]) || !fits_i32(g.src_origin[d]) || !fits_i32(g.dst_origin[d]) ||
        !fits_i32(g.req_index[d] + g.req_size[d] + 64) || !fits_i32(g.req_index[d] - 64))
      return ITKG_ERROR_UNSUPPORTED;
  const int64_t nx = g.req_size[0], ny = g.req_size[1], nz = g.req_size[2];
  const int64_t ntx = (nx + kTX - 1) / kTX, nty = (ny + kTY - 1) / kTY;
  const int64_t units = ntx * nty * nz;
  if (units > INT_MAX) return ITKG_ERROR_UNSUPPORTED;
  char* const dst0 = static_cast<char*>(g.dst) + (g.req_index[0] - g.dst_origin[0]) * g.dst_pitch[0] +
                     (g.req_index[1] - g.dst_origin[1]) * g.dst_pitch[1] + (g.req_index[2] - g.dst_origin[2]) * g.dst_pitch[2];
  const bool vec = g.out_dtype == ITKG_F32 && g.dst_pitch[0] == 4 && ((uintptr_t)dst0 & 15) == 0 &&
                   (g.dst_pitch[1] & 15) == 0 && (g.dst_pitch[2] & 15) == 0 && nx % 4 == 0;
  if (dry_run) return ITKG_SUCCESS;

  static_assert(sizeof(Args) < 32000, "kernel parameters");
  Args a;
  std::memset(&a, 0, sizeof a);
  CUtensorMap map;
  const size_t smem = one_trip_smem(R);
  int res = 0;
  itkg_status st = encode_input_map(g, one_trip_box_w(R), kTY + 2 * R, &map);
  if (st == ITKG_SUCCESS) st = device_fault_word(&a.fault);
  if (st == ITKG_SUCCESS) st = max_resident_ctas(reinterpret_cast<const void*>(fn), smem, 256, &res);
  if (st != ITKG_SUCCESS) return st;
  a.wait_limit = wait_limit_cycles();
  a.dst = dst0;
  for (int d = 0; d < 3; ++d) {
    a.dst_pitch[d] = g.dst_pitch[d];
    a.src_origin[d] = (int32_t)g.src_origin[d];
    a.lo[d] = (int32_t)std::max<int64_t>(g.lo[d], g.src_origin[d]);
    a.hi[d] = (int32_t)std::min<int64_t>(g.hi[d], g.src_origin[d] + g.src_size[d] - 1);
  }
  a.x0 = (int32_t)g.req_index[0];
  a.y0 = (int32_t)g.req_index[1];
  a.z0 = (int32_t)g.req_index[2];
  a.nx = (int32_t)nx;
  a.ny = (int32_t)ny;
  a.nz = (int32_t)nz;
  a.ntx = (int32_t)ntx;
  a.nty = (int32_t)nty;
  a.out_dtype = g.out_dtype;
  a.vec = vec ? 1 : 0;
  a.units = units;
  const int K = 2 * R + 1, KZ = 2 * RZ + 1;
  for (int k = 0; k < K; ++k) {
    a.wx[k] = w[0][k];
    a.wy[k] = w[1][k];
    a.wx2[k] = splat2_host(w[0][k]);
    a.wy2[k] = splat2_host(w[1][k]);
  }
  for (int k = 0; k < KZ; ++k) {
    a.wz[k] = w[2][k];
    a.wz2[k] = splat2_host(w[2][k]);
  }
  if (!ref) {
    // clamped-tap weights of the first / last tile columns and rows: p[R - d]
    // for an output d < R inside an edge (p[j] = w[0] + ... + w[j-1])
    double p[2 * kMaxR + 2] = {0.0}, q[2 * kMaxR + 2] = {0.0};
    for (int k = 0; k < K; ++k) p[k + 1] = p[k] + w[0][k];
    for (int k = 0; k < K; ++k) q[k + 1] = q[k] + w[1][k];
    auto coef = [&](const double* pp, int64_t d) { return (d >= 0 && d < R) ? (float)pp[R - d] : 0.0f; };
    a.xr0 = std::max(0, a.ntx - 2);
    a.yr0 = std::max(0, a.nty - 2);
    const int64_t tx_r = g.req_index[0] + (int64_t)a.xr0 * kTX;  // first of the last two tile columns
    const int64_t ty_r = g.req_index[1] + (int64_t)a.yr0 * kTY;
    for (int t = 0; t < kTX; t += 2) {
      const float c0 = coef(p, g.req_index[0] + t - a.lo[0]), c1 = coef(p, g.req_index[0] + t + 1 - a.lo[0]);
      a.cxl[t / 2] = pack2_host(c0, c1);
      if (c0 != 0.0f || c1 != 0.0f) a.edge |= 1;
    }
    for (int t = 0; t < 2 * kTX; t += 2) {
      const float c0 = coef(p, a.hi[0] - (tx_r + t)), c1 = coef(p, a.hi[0] - (tx_r + t + 1));
      a.cxr[t / 2] = pack2_host(c0, c1);
      if (c0 != 0.0f || c1 != 0.0f) a.edge |= 2;
    }
    for (int t = 0; t < kTY; ++t) {
      const float c = coef(q, g.req_index[1] + t - a.lo[1]);
      a.cyt[t] = splat2_host(c);
      if (c != 0.0f) a.edge |= 4;
    }
    for (int t = 0; t < 2 * kTY; ++t) {
      const float c = coef(q, a.hi[1] - (ty_r + t));
      a.cyb[t] = splat2_host(c);
      if (c != 0.0f) a.edge |= 8;
    }
  }
  int64_t grid = std::min<int64_t>(units, res);
  a.nsplit = z_split(ntx * nty, nz, RZ, grid, a.split);
  if (a.nsplit > 0) grid = a.nsplit;

  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof cfg);
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = static_cast<cudaStream_t>(stream);
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t err = cudaLaunchKernelEx(&cfg, fn, map, a);
  note_launch(ref ? "one_trip_f32_ref" : "one_trip_f32_fma");
  if (err == cudaSuccess) err = cudaGetLastError();
  if (err != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "one-trip launch: %s", cudaGetErrorString(err));
  return ITKG_SUCCESS;
}

}  // namespace itkg
