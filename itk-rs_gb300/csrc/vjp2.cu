// Host side of the two-kernel-family VJP (kernels in vjp_two_pass.cuh):
// kernel choice, the U / U' scratch images and the launches.
#include <algorithm>
#include <climits>

#include "vjp_two_pass.cuh"

namespace itkg {
namespace vjp2 {
namespace {

using XYVFn = void (*)(const CUtensorMap, const XYVArgs);
using ZAFn = void (*)(const ZAArgs);

struct Entry {
  int r;
  XYVFn xy[2];  // [mode]
  size_t xy_smem[2];
  int bw, ih, tx, ty;
  ZAFn z;
  ZAFn z2;  // both z adjoints in one pass
};

template <int R>
Entry make() {
  using A = CfgXYV<R, kAdjoint>;
  using Dd = CfgXYV<R, kDualDot>;
  return Entry{R, {k_xy_vjp<R, kAdjoint>, k_xy_vjp<R, kDualDot>}, {A::SMEM, Dd::SMEM}, A::BW, A::IH, A::TX, A::TY,
               k_z_adj<R>, k_z_adj2<R>};
}

const Entry kTable[] = {make<1>(), make<2>(), make<3>(),  make<4>(),  make<5>(),  make<6>(),
                        make<7>(), make<8>(), make<9>(), make<10>(), make<11>(), make<12>()};

const Entry* find(int r) {
  for (const Entry& e : kTable)
    if (e.r == r) return &e;
  return nullptr;
}

size_t z_smem(int r) { return (size_t)(2 * r + 1) * 256 * 16; }
size_t z2_smem(int r) { return (size_t)(2 * r + 1) * 256 * 8; }

bool aligned16(const itkg_image& im) {
  return ((uintptr_t)im.data & 15) == 0 && im.pitch[0] == 4 && (im.pitch[1] & 15) == 0 && (im.pitch[2] & 15) == 0;
}

// exclusive prefix sums p[j] = w[0] + ... + w[j-1], j = 0..R
void prefix(const float* w, int R, float* p) {
  double s = 0.0;
  for (int j = 0; j <= R; ++j) {
    p[j] = (float)s;
    if (j < 2 * R + 1) s += w[j];
  }
}

void tap_pairs(const float* w, int R, f2_t* we, f2_t* wo) {
  const int K = 2 * R + 1;
  auto wk = [&](int k) { return (k < 0 || k >= K) ? 0.0f : w[k]; };
  for (int i = 0; i <= R; ++i) {
    we[i] = pack2_host(wk(2 * i), wk(2 * i + 1));
    wo[i] = pack2_host(wk(2 * i - 1), wk(2 * i));
  }
}

}  // namespace
}  // namespace vjp2

itkg_status launch_vjp_two_pass(const VjpTwoPass& v, void* stream, bool dry_run) {
  const itkg_image& x = *v.x;
  const itkg_image& yb = *v.ybar;
  if (x.dim != 3 || x.components != 1 || v.radius[0] != v.radius[1]) return ITKG_ERROR_UNSUPPORTED;
  for (int d = 0; d < 3; ++d)
    if (v.radius[d] < 1 || v.radius[d] > twopass::kMaxR) return ITKG_ERROR_UNSUPPORTED;
  const vjp2::Entry* e = vjp2::find(v.radius[0]);
  const vjp2::Entry* ez = vjp2::find(v.radius[2]);
  if (!e || !ez || !vjp2::aligned16(x) || !vjp2::aligned16(yb)) return ITKG_ERROR_UNSUPPORTED;
  if (v.xbar && (v.xbar->pitch[0] != 4 || ((uintptr_t)v.xbar->data & 3))) return ITKG_ERROR_UNSUPPORTED;
  const int64_t nx = (int64_t)x.region.size[0], ny = (int64_t)x.region.size[1], nz = (int64_t)x.region.size[2];
  for (int d = 0; d < 3; ++d)
    if (x.region.index[d] < INT_MIN / 2 || x.region.index[d] + (int64_t)x.region.size[d] > INT_MAX / 2)
      return ITKG_ERROR_UNSUPPORTED;
  if (nx > INT_MAX / 8 || ny > INT_MAX / 8 || nz > INT_MAX / 8) return ITKG_ERROR_UNSUPPORTED;
  if (dry_run) return ITKG_SUCCESS;

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int R = v.radius[0], RZ = v.radius[2];
  const bool want_s = v.sigma_out != nullptr;
  // U and U' : dense f32, 16-byte rows
  itkg_image u = x;
  u.pitch[0] = 4;
  u.pitch[1] = (nx * 4 + 15) / 16 * 16;
  u.pitch[2] = u.pitch[1] * ny;
  const size_t ubytes = (size_t)u.pitch[2] * (size_t)nz;
  void* pu = nullptr;
  void* pu2 = nullptr;
  void* ppart = nullptr;
  itkg_status st = scratch_alloc(&pu, ubytes, stream);
  if (st == ITKG_SUCCESS && want_s) st = scratch_alloc(&pu2, ubytes, stream);

  // z adjoints
  vjp2::ZAArgs za;
  std::memset(&za, 0, sizeof za);
  za.in = static_cast<const char*>(yb.data);
  for (int d = 0; d < 3; ++d) za.in_pitch[d] = yb.pitch[d], za.out_pitch[d] = u.pitch[d];
  za.nx = (int32_t)nx;
  za.ny = (int32_t)ny;
  za.nz = (int32_t)nz;
  za.nqx = (int32_t)((nx + 3) / 4);
  za.units = ((int64_t)za.nqx * ny + 255) / 256 * nz;
  int res_z = 0, res_xy = 0;
  for (int k = 0; k < 2 * RZ + 1; ++k) za.wz2[k] = splat2_host(v.w[2][k]);
  vjp2::prefix(v.w[2], RZ, za.pz);
  za.out = static_cast<char*>(pu);
  if (want_s) {
    // U and U' in one pass over ybar (two columns per thread, both weight sets)
    for (int k = 0; k < 2 * RZ + 1; ++k) za.wz2d[k] = splat2_host(v.dw[2][k]);
    vjp2::prefix(v.dw[2], RZ, za.pzd);
    za.out2 = static_cast<char*>(pu2);
    za.npx = (int32_t)((nx + 1) / 2);
    za.units = ((int64_t)za.npx * ny + 255) / 256 * nz;
    if (st == ITKG_SUCCESS)
      st = max_resident_ctas(reinterpret_cast<const void*>(ez->z2), vjp2::z2_smem(RZ), 256, &res_z);
    if (st == ITKG_SUCCESS) {
      const int64_t g = std::min<int64_t>(za.units, res_z);
      ez->z2<<<(unsigned)g, 256, vjp2::z2_smem(RZ), s>>>(za);
      note_launch("z_adjoint2_f32");
      const cudaError_t err = cudaGetLastError();
      if (err != cudaSuccess) st = set_error(ITKG_ERROR_CUDA, "z adjoint launch: %s", cudaGetErrorString(err));
    }
  } else {
    if (st == ITKG_SUCCESS)
      st = max_resident_ctas(reinterpret_cast<const void*>(ez->z), vjp2::z_smem(RZ), 256, &res_z);
    if (st == ITKG_SUCCESS) {
      const int64_t g = std::min<int64_t>(za.units, res_z);
      ez->z<<<(unsigned)g, 256, vjp2::z_smem(RZ), s>>>(za);
      note_launch("z_adjoint_f32");
      const cudaError_t err = cudaGetLastError();
      if (err != cudaSuccess) st = set_error(ITKG_ERROR_CUDA, "z adjoint launch: %s", cudaGetErrorString(err));
    }
  }

  // x-y kernels
  vjp2::XYVArgs xa;
  std::memset(&xa, 0, sizeof xa);
  for (int d = 0; d < 3; ++d) {
    xa.src_origin[d] = (int32_t)x.region.index[d];
    xa.lo[d] = (int32_t)x.region.index[d];
    xa.hi[d] = (int32_t)(x.region.index[d] + (int64_t)x.region.size[d] - 1);
  }
  xa.ntx = (int32_t)((nx + e->tx - 1) / e->tx);
  const int64_t nty = (ny + e->ty - 1) / e->ty;
  xa.ns = (int32_t)nz;
  xa.units = (int64_t)xa.ntx * nty * nz;
  vjp2::tap_pairs(v.w[0], R, xa.we, xa.wo);
  vjp2::tap_pairs(v.dw[0], R, xa.dwe, xa.dwo);
  for (int k = 0; k < 2 * R + 1; ++k) xa.wy2[k] = splat2_host(v.w[1][k]), xa.dwy2[k] = splat2_host(v.dw[1][k]);
  vjp2::prefix(v.w[0], R, xa.px);
  vjp2::prefix(v.w[1], R, xa.py);
  vjp2::prefix(v.dw[0], R, xa.pdx);
  vjp2::prefix(v.dw[1], R, xa.pdy);
  if (st == ITKG_SUCCESS) st = device_fault_word(&xa.fault);
  xa.wait_limit = wait_limit_cycles();
  for (int mode = 0; mode < 2 && st == ITKG_SUCCESS; ++mode) {
    if (mode == vjp2::kAdjoint && !v.xbar) continue;
    if (mode == vjp2::kDualDot && !want_s) continue;
    // the TMA source: U for the adjoint, x for the dual-dot pass
    FusedGeom g;
    std::memset(&g, 0, sizeof g);
    const itkg_image& src = mode == vjp2::kAdjoint ? u : x;
    g.src = mode == vjp2::kAdjoint ? pu : x.data;
    g.in_dtype = ITKG_F32;
    for (int d = 0; d < 3; ++d) g.src_size[d] = (int64_t)x.region.size[d], g.src_pitch[d] = src.pitch[d];
    CUtensorMap map;
    st = encode_input_map(g, e->bw, e->ih, &map);
    if (st != ITKG_SUCCESS) break;
    st = max_resident_ctas(reinterpret_cast<const void*>(e->xy[mode]), e->xy_smem[mode], 256, &res_xy);
    if (st != ITKG_SUCCESS) break;
    const int64_t grid = std::min<int64_t>(xa.units, res_xy);
    if (mode == vjp2::kAdjoint) {
      xa.out = static_cast<char*>(v.xbar->data);
      for (int d = 0; d < 3; ++d) xa.out_pitch[d] = v.xbar->pitch[d];
      xa.accumulate = v.acc_x ? 1 : 0;
    } else {
      xa.u = static_cast<const char*>(pu);
      xa.u2 = static_cast<const char*>(pu2);
      for (int d = 0; d < 3; ++d) xa.u_pitch[d] = u.pitch[d];
      st = scratch_alloc(&ppart, sizeof(double) * (size_t)grid, stream);
      if (st != ITKG_SUCCESS) break;
      xa.partials = static_cast<double*>(ppart);
    }
    e->xy[mode]<<<(unsigned)grid, 256, e->xy_smem[mode], s>>>(map, xa);
    note_launch(mode == vjp2::kAdjoint ? "xy_adjoint_f32" : "xy_dual_dot_f32");
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
      st = set_error(ITKG_ERROR_CUDA, "x-y VJP launch: %s", cudaGetErrorString(err));
      break;
    }
    if (mode == vjp2::kDualDot)
      st = launch_sum_partials(xa.partials, (int)grid, v.sigma_out, v.acc_sigma, stream);
  }
  scratch_free(pu, stream);
  scratch_free(pu2, stream);
  scratch_free(ppart, stream);
  return st;
}

}  // namespace itkg
