// Host side of the two-kernel 3-D forward (kernels in two_pass.cuh): kernel
// choice, the intermediate's layout and its z-chunking, and the launches.
// This file holds the f32 x-y pass table; the i16 / u8 / bf16 / f16 x-y pass
// tables are in two_pass_in.cu, the z-pass instantiations in two_pass_z*.cu.
#include <algorithm>
#include <climits>
#include <cmath>

#include "two_pass.cuh"

namespace itkg {
namespace twopass {
namespace {
const XYEntry kXYF32[] = ITKG_XY_TABLE(float, ITKG_F32);
}  // namespace

ZFn z_fn(int r, bool ref, int store, bool ush) {
  if (ush) return z_ush_fn(r, ref);
  if (r < 1 || r > kMaxR) return nullptr;
  const ZFn* row = nullptr;
  switch (store) {
    case kStoreAny: row = ref ? z_row_ref_any() : z_row_fma_any(); break;
    case kStoreF32Quad: row = ref ? z_row_ref_f32q() : z_row_fma_f32q(); break;
    case kStoreBF16Quad: row = ref ? z_row_ref_bf16q() : z_row_fma_bf16q(); break;
    case kStoreF16Quad: row = ref ? z_row_ref_f16q() : z_row_fma_f16q(); break;
    default: return nullptr;
  }
  return row[r - 1];
}

const XYEntry* xy_entries_f32(int* n) {
  *n = (int)(sizeof(kXYF32) / sizeof(kXYF32[0]));
  return kXYF32;
}
}  // namespace twopass

namespace {

using twopass::XYArgs;
using twopass::XYEntry;

// floor(f32 fma(v, c, 0.5)) for v in 0 .. 255, as the u8 pixel-arithmetic
// kernels compute it: v * c is exact in f64 (8 + 24 significant bits) and so
// is the sum with 0.5 when c >= 2^-21 (at most 32 - log2(c) bits); the one
// rounding to f32 is then the conversion.  Below 2^-21, v * c < 2^-13 and the
// f32 result is below 1 whatever its rounding: floor 0.
int u8p_device_value(int v, float c) {
  if (!(c >= 0x1p-21f)) {
    if (c >= 0.0f) return 0;
    return INT_MIN;  // negative constants are never chosen
  }
  const float s = (float)((double)v * (double)c + 0.5);
  return (int)std::floor(s);
}

bool u8p_tap_ok(double w, float c) {
  for (int v = 0; v < 256; ++v) {
    double r = std::round((double)v * w);  // f64 product, half away from zero
    r = r < 0.0 ? 0.0 : (r > 255.0 ? 255.0 : r);
    if (u8p_device_value(v, c) != (int)r) return false;
  }
  return true;
}
using twopass::ZArgs;

// L2 share the intermediate may take; longer z ranges are processed in chunks.
constexpr int64_t kChunkBytes = 72ll << 20;

const XYEntry* find_xy(int r, int dtype) {
  int n = 0;
  const XYEntry* t = nullptr;
  switch (dtype) {
    case ITKG_F32: t = twopass::xy_entries_f32(&n); break;
    case ITKG_I16: t = twopass::xy_entries_i16(&n); break;
    case ITKG_U8: t = twopass::xy_entries_u8(&n); break;
    case ITKG_BF16: t = twopass::xy_entries_bf16(&n); break;
    case ITKG_F16: t = twopass::xy_entries_f16(&n); break;
    default: return nullptr;
  }
  for (int i = 0; i < n; ++i)
    if (t[i].r == r) return &t[i];
  return nullptr;
}

bool fits_i32(int64_t v) { return v >= INT_MIN && v <= INT_MAX; }

// the z kernel's rings: T quads, and for the unsharp store the input quads too
size_t z_smem(int rz, bool ush = false) {
  return (size_t)(2 * rz + 1) * 256 * 16 * twopass::CfgZ<1>::QPT * (ush ? 2 : 1);
}

const char* xy_name(int dtype, bool ref) {
  static const char* names[5][2] = {{"xy_pass_f32_fma", "xy_pass_f32_ref"},
                                    {"xy_pass_i16_fma", "xy_pass_i16_ref"},
                                    {"xy_pass_u8_fma", "xy_pass_u8_ref"},
                                    {"xy_pass_bf16_fma", "xy_pass_bf16_ref"},
                                    {"xy_pass_f16_fma", "xy_pass_f16_ref"}};
  return names[dtype][ref ? 1 : 0];
}

}  // namespace

// Per-CTA unit ranges of the z pass.  Units are (quad block, output slice),
// block-major; a CTA marches each column segment of its range from 2 rz slices
// before the segment's first output, so its cost is its units plus 2 rz per
// segment.  The ranges are cut greedily under the smallest cost budget that
// lets at most `grid` CTAs cover all units (an even split leaves the CTAs whose
// range straddles two blocks about 2 rz slices behind).  Returns the CTA count
// and fills split[0 .. count]; 0 when the units do not fit the table.
int z_split(int64_t qblocks, int64_t nz, int rz, int64_t grid, int32_t* split) {
  if (grid < 1 || grid > twopass::kMaxZSplit || qblocks * nz > INT_MAX) return 0;
  auto cover = [&](int64_t budget, int32_t* out) -> int64_t {
    int64_t blk = 0, zs = 0, n = 0;
    while (blk < qblocks) {
      if (n == grid) return grid + 1;
      if (out) out[n] = (int32_t)(blk * nz + zs);
      ++n;
      int64_t left = budget;
      while (blk < qblocks) {
        const int64_t take = std::min<int64_t>(nz - zs, left - 2 * rz);
        if (take <= 0) break;
        zs += take;
        left -= take + 2 * rz;
        if (zs < nz) break;
        ++blk;
        zs = 0;
      }
    }
    if (out) out[n] = (int32_t)(qblocks * nz);
    return n;
  };
  int64_t lo = 2 * rz + 1, hi = qblocks * (nz + 2 * rz);
  while (lo < hi) {
    const int64_t mid = lo + (hi - lo) / 2;
    if (cover(mid, nullptr) <= grid) hi = mid;
    else lo = mid + 1;
  }
  return (int)cover(lo, split);
}

bool u8_pixel_tap_consts(const double* w, int K, float* c) {
  for (int k = 0; k < K; ++k) {
    const float c0 = (float)w[k];
    bool found = u8p_tap_ok(w[k], c0);
    float best = c0;
    float up = c0, dn = c0;
    for (int d = 1; d <= 64 && !found; ++d) {
      up = std::nextafter(up, 2.0f);
      dn = std::nextafter(dn, -1.0f);
      if (up >= 0.0f && u8p_tap_ok(w[k], up)) found = true, best = up;
      else if (dn >= 0.0f && u8p_tap_ok(w[k], dn)) found = true, best = dn;
    }
    if (!found) return false;
    c[k] = best;
  }
  return true;
}

itkg_status launch_two_pass(const FusedGeom& g, const float* const w[kMaxDim], void* stream, bool dry_run,
                            const UnsharpConsts* ush) {
  const bool u8p = g.u8pix != 0;
  if (g.dim != 3 || g.comps != 1 || g.out_dtype == ITKG_I16) return ITKG_ERROR_UNSUPPORTED;
  if (g.radius[0] != g.radius[1] || g.radius[2] < 1 || g.radius[2] > twopass::kMaxR)
    return ITKG_ERROR_UNSUPPORTED;
  if (u8p && (g.in_dtype != ITKG_U8 || g.out_dtype != ITKG_U8 || ush)) return ITKG_ERROR_UNSUPPORTED;
  const XYEntry* e = nullptr;
  if (u8p) {
    int n = 0;
    const XYEntry* t = twopass::xy_entries_u8p(&n);
    for (int i = 0; i < n; ++i)
      if (t[i].r == g.radius[0]) e = &t[i];
  } else {
    e = find_xy(g.radius[0], g.in_dtype);
  }
  if (!e) return ITKG_ERROR_UNSUPPORTED;
  const int esz = dtype_size(g.in_dtype);
  if (g.src_pitch[0] != esz) return ITKG_ERROR_UNSUPPORTED;
  // FMA rounding reads zeros outside the input buffer as the halo and adds the
  // clamped taps back at the image's edges: the buffer must lie inside the
  // image on x and y.
  if (g.rounding != ITKG_ROUND_REFERENCE && !u8p)
    for (int d = 0; d < 2; ++d)
      if (g.src_origin[d] < g.lo[d] || g.src_origin[d] + g.src_size[d] - 1 > g.hi[d]) return ITKG_ERROR_UNSUPPORTED;
  // TMA: 16-byte base and pitches, 16-byte aligned first tile column
  const int ae = 16 / esz;
  if (((uintptr_t)g.src & 15) || (g.src_pitch[1] & 15) || (g.src_pitch[2] & 15)) return ITKG_ERROR_UNSUPPORTED;
  if (g.src_pitch[1] >= (1ll << 40) || g.src_pitch[2] >= (1ll << 40)) return ITKG_ERROR_UNSUPPORTED;
  if ((((g.req_index[0] - g.src_origin[0]) % ae) + ae) % ae != 0) return ITKG_ERROR_UNSUPPORTED;
  for (int d = 0; d < 3; ++d)
    if (!fits_i32(g.lo[d]) || !fits_i32(g.hi[d]) || !fits_i32(g.src_origin[d]) || !fits_i32(g.dst_origin[d]) ||
        !fits_i32(g.req_index[d] + g.req_size[d] + 64) || !fits_i32(g.req_index[d] - 64))
      return ITKG_ERROR_UNSUPPORTED;
  const int64_t nx = g.req_size[0], ny = g.req_size[1], nz = g.req_size[2];
  if (!fits_i32(nx) || !fits_i32(ny)) return ITKG_ERROR_UNSUPPORTED;
  const int64_t ntx = (nx + twopass::kTileX - 1) / twopass::kTileX;
  const int64_t nty = (ny + e->ty - 1) / e->ty;
  // one store per quad (16 bytes of f32, 8 bytes of bf16 / f16) when every
  // quad of the output is full and aligned
  char* const dst0 = static_cast<char*>(g.dst) + (g.req_index[0] - g.dst_origin[0]) * g.dst_pitch[0] +
                     (g.req_index[1] - g.dst_origin[1]) * g.dst_pitch[1];
  int store = twopass::kStoreAny;
  if (u8p) {
    if (g.dst_pitch[0] == 1 && ((uintptr_t)dst0 & 3) == 0 && g.dst_pitch[1] % 4 == 0 && g.dst_pitch[2] % 4 == 0 &&
        nx % 4 == 0)
      store = twopass::kStoreU8Quad;
  } else {
    const int osz = g.out_dtype == ITKG_F32 ? 4 : (g.out_dtype == ITKG_BF16 || g.out_dtype == ITKG_F16) ? 2 : 0;
    const int64_t qa = 4 * osz;  // bytes per quad
    if (osz && g.dst_pitch[0] == osz && ((uintptr_t)dst0 % qa) == 0 && g.dst_pitch[1] % qa == 0 &&
        g.dst_pitch[2] % qa == 0 && nx % 4 == 0)
      store = g.out_dtype == ITKG_F32    ? twopass::kStoreF32Quad
              : g.out_dtype == ITKG_BF16 ? twopass::kStoreBF16Quad
                                         : twopass::kStoreF16Quad;
  }
  const bool vec = store == twopass::kStoreF32Quad;
  // the unsharp store reads the input's quads at the output's positions (the
  // TMA checks above make them 16-byte aligned for f32 input)
  const char* const src0 = static_cast<const char*>(g.src) + (g.req_index[0] - g.src_origin[0]) * g.src_pitch[0] +
                           (g.req_index[1] - g.src_origin[1]) * g.src_pitch[1];
  // the point-wise step's arithmetic follows the blur's rounding
  if (ush && (!vec || g.in_dtype != ITKG_F32 || (g.rounding == ITKG_ROUND_REFERENCE) == (ush->cheap != 0) ||
              ((uintptr_t)src0 & 15)))
    return ITKG_ERROR_UNSUPPORTED;
  if (dry_run) return ITKG_SUCCESS;

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool ref = u8p || g.rounding == ITKG_ROUND_REFERENCE;  // u8 pixel arithmetic clamps like the reference rounding
  const int rz = g.radius[2];
  // clamp bounds on z: the image within the input buffer
  const int64_t zlo = std::max<int64_t>(g.lo[2], g.src_origin[2]);
  const int64_t zhi = std::min<int64_t>(g.hi[2], g.src_origin[2] + g.src_size[2] - 1);
  const int64_t tile_floats = (int64_t)twopass::kTileX * e->ty;
  const int64_t slice_floats = ntx * nty * tile_floats;  // T is tile-major
  // outputs per chunk: as many as keep the chunk's intermediate within kChunkBytes
  int64_t chunk = nz;
  {
    const int64_t fit = kChunkBytes / (slice_floats * 4) - 2 * rz;
    if (fit >= 2 * rz + 1) chunk = std::min<int64_t>(nz, fit);
  }
  const int64_t t_slices = std::min<int64_t>(chunk + 2 * rz, zhi - zlo + 1);
  float* t = nullptr;
  {
    const itkg_status sa = scratch_alloc(reinterpret_cast<void**>(&t), (size_t)(t_slices * slice_floats * 4), stream);
    if (sa != ITKG_SUCCESS) return sa;
  }

  CUtensorMap map;
  itkg_status st = encode_input_map(g, e->bw, e->ih, &map);
  XYArgs xa;
  ZArgs za;
  std::memset(&xa, 0, sizeof xa);
  std::memset(&za, 0, sizeof za);
  if (st == ITKG_SUCCESS) st = device_fault_word(&xa.fault);
  xa.wait_limit = wait_limit_cycles();
  int res_xy = 0, res_z = 0;
  const twopass::ZFn zfn =
      u8p ? (store == twopass::kStoreU8Quad ? twopass::z_row_u8p_u8q() : twopass::z_row_u8p_any())[rz - 1]
          : twopass::z_fn(rz, ref, store, ush != nullptr);
  const twopass::XYFn xyfn = e->fn[ref ? 1 : 0];
  if (st == ITKG_SUCCESS) st = max_resident_ctas(reinterpret_cast<const void*>(xyfn), e->smem, e->nt, &res_xy);
  if (st == ITKG_SUCCESS)
    st = max_resident_ctas(reinterpret_cast<const void*>(zfn), z_smem(rz, ush != nullptr), 256, &res_z);
  if (st != ITKG_SUCCESS) {
    scratch_free(t, stream);
    return st;
  }

  xa.t = t;
  xa.t_slice = slice_floats;
  for (int d = 0; d < 3; ++d) {
    xa.src_origin[d] = (int32_t)g.src_origin[d];
    xa.lo[d] = (int32_t)std::max<int64_t>(g.lo[d], g.src_origin[d]);
    xa.hi[d] = (int32_t)std::min<int64_t>(g.hi[d], g.src_origin[d] + g.src_size[d] - 1);
  }
  xa.x0 = (int32_t)g.req_index[0];
  xa.y0 = (int32_t)g.req_index[1];
  xa.ntx = (int32_t)ntx;
  const int R = g.radius[0], K = 2 * R + 1;
  for (int k = 0; k < K; ++k) {
    xa.wx[k] = w[0][k], xa.wx2[k] = splat2_host(w[0][k]);
    xa.wy[k] = w[1][k], xa.wy2[k] = splat2_host(w[1][k]);
  }
  {
    auto wk = [&](int k) { return (k < 0 || k >= K) ? 0.0f : w[0][k]; };
    for (int i = 0; i <= R; ++i) {
      xa.we[i] = pack2_host(wk(2 * i), wk(2 * i + 1));
      xa.wo[i] = pack2_host(wk(2 * i - 1), wk(2 * i));
    }
  }
  xa.nty = (int32_t)nty;
  {
    // clamped-tap weights of the first / last tile column and row (FMA rounding)
    double p[twopass::kMaxK + 1] = {0.0};
    for (int k = 0; k < K; ++k) p[k + 1] = p[k] + w[0][k];
    double q[twopass::kMaxK + 1] = {0.0};
    for (int k = 0; k < K; ++k) q[k + 1] = q[k] + w[1][k];
    auto coef = [&](const double* pp, int64_t d) { return (d >= 0 && d < R) ? (float)pp[R - d] : 0.0f; };
    xa.xr0 = std::max(0, xa.ntx - 2);
    xa.yr0 = std::max(0, (int)nty - 2);
    const int64_t tx_r = g.req_index[0] + (int64_t)xa.xr0 * e->tx;  // first of the last two tile columns
    const int64_t ty_r = g.req_index[1] + (int64_t)xa.yr0 * e->ty;
    for (int t = 0; t < twopass::kTileX; ++t) {
      xa.cxl[t] = coef(p, g.req_index[0] + t - xa.lo[0]);
      if (xa.cxl[t] != 0.0f) xa.edge |= 1;
    }
    for (int t = 0; t < 2 * twopass::kTileX; ++t) {
      xa.cxr[t] = coef(p, xa.hi[0] - (tx_r + t));
      if (xa.cxr[t] != 0.0f) xa.edge |= 2;
    }
    for (int t = 0; t < e->ty; ++t) {
      xa.cyt[t] = coef(q, g.req_index[1] + t - xa.lo[1]);
      if (xa.cyt[t] != 0.0f) xa.edge |= 4;
    }
    for (int t = 0; t < 2 * e->ty; ++t) {
      xa.cyb[t] = coef(q, xa.hi[1] - (ty_r + t));
      if (xa.cyb[t] != 0.0f) xa.edge |= 8;
    }
  }
  za.t = t;
  za.t_slice = slice_floats;
  za.nx = (int32_t)nx;
  za.ny = (int32_t)ny;
  za.ntx = (int32_t)ntx;
  za.out_dtype = g.out_dtype;
  za.dst_pitch[0] = g.dst_pitch[0];
  za.dst_pitch[1] = g.dst_pitch[1];
  za.dst_pitch[2] = g.dst_pitch[2];
  za.vec_store = store;
  if (ush) {
    za.ush = *ush;
    za.ush_pitch[0] = g.src_pitch[0];
    za.ush_pitch[1] = g.src_pitch[1];
    za.ush_pitch[2] = g.src_pitch[2];
  }
  for (int k = 0; k < 2 * rz + 1; ++k) za.wz[k] = w[2][k], za.wz2[k] = splat2_host(w[2][k]);
  const int64_t qblocks = ntx * nty * (tile_floats / 4 / twopass::CfgZ<1>::QB);
  za.tile_rows = e->ty;

  for (int64_t c0 = 0; c0 < nz && st == ITKG_SUCCESS; c0 += chunk) {
    const int64_t c1 = std::min<int64_t>(nz, c0 + chunk);  // outputs [z0 + c0, z0 + c1)
    const int64_t oz0 = g.req_index[2] + c0, oz1 = g.req_index[2] + c1 - 1;
    const int64_t s0 = std::max<int64_t>(zlo, oz0 - rz), s1 = std::min<int64_t>(zhi, oz1 + rz);
    xa.s0 = (int32_t)s0;
    xa.ns = (int32_t)(s1 - s0 + 1);
    xa.t_s0 = (int32_t)s0;
    xa.units = (int64_t)xa.ntx * nty * xa.ns;
    const int64_t gxy = std::min<int64_t>(xa.units, res_xy);
    // programmatic dependent launch on both kernels: the x-y CTAs may start
    // while the stream's previous kernel retires (they wait for it before
    // touching global memory), the z CTAs while the x-y CTAs retire
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg;
    std::memset(&cfg, 0, sizeof cfg);
    cfg.gridDim = dim3((unsigned)gxy);
    cfg.blockDim = dim3((unsigned)e->nt);
    cfg.dynamicSmemBytes = e->smem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t err = cudaLaunchKernelEx(&cfg, xyfn, map, xa);
    note_launch(u8p ? "xy_pass_u8_pixel" : xy_name(g.in_dtype, ref));
    if (err == cudaSuccess) err = cudaGetLastError();
    if (err != cudaSuccess) {
      st = set_error(ITKG_ERROR_CUDA, "xy pass launch: %s", cudaGetErrorString(err));
      break;
    }
    za.t_s0 = (int32_t)s0;
    za.t_s1 = (int32_t)s1;
    za.z0 = (int32_t)oz0;
    za.nz = (int32_t)(c1 - c0);
    za.units = qblocks * za.nz;
    za.dst = dst0 + (oz0 - g.dst_origin[2]) * g.dst_pitch[2];
    if (ush) za.ush_src = src0 + (oz0 - g.src_origin[2]) * g.src_pitch[2];
    int64_t gz = std::min<int64_t>(za.units, res_z);
    za.nsplit = z_split(qblocks, za.nz, rz, gz, za.split);
    if (za.nsplit > 0) gz = za.nsplit;
    cfg.gridDim = dim3((unsigned)gz);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = z_smem(rz, ush != nullptr);
    err = cudaLaunchKernelEx(&cfg, zfn, za);
    note_launch(u8p ? "z_pass_u8_pixel"
                    : ush ? (ref ? "z_pass_unsharp_ref" : "z_pass_unsharp_fma")
                          : (ref ? "z_pass_f32_ref" : "z_pass_f32_fma"));
    if (err == cudaSuccess) err = cudaGetLastError();
    if (err != cudaSuccess) st = set_error(ITKG_ERROR_CUDA, "z pass launch: %s", cudaGetErrorString(err));
  }
  scratch_free(t, stream);
  return st;
}

}  // namespace itkg
