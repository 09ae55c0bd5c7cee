// Fused 3-D Gaussian forward: all three separable passes of
// GaussianFilter::generate_region (src/filters/gaussian.rs:74-88) in one
// kernel, so each input voxel is read from HBM once and each output voxel is
// written once.  The kernel templates are in fused_kernel.cuh; this file holds
// the f32 instantiations and the host-side dispatch (kernel choice, TMA
// descriptors, launch geometry, multi-request batches, the fault word).
//
// Decomposition.  A CTA owns an output tile of TX x TY columns (x, y) and a
// range of output slices [z0, z1).  It marches through the input slices
// j = z0 - RZ .. z1 - 1 + RZ (clamped to the image on z, which is the
// reference's clamp-to-edge on axis 2, conv.rs:31-33):
//   1. the (TX + 2XA) x (TY + 2RY) input tile of slice j is staged in shared
//      memory S slices ahead -- by one TMA tile load per slice (an elected
//      thread, mbarrier completion) when the buffer's base and pitches are
//      16-byte multiples, else (f32 only) by a cp.async gather.  Edge tiles
//      replicate the image's edge values into the halo after the load (TMA
//      fills zeros outside the buffer); the gather clamps its coordinates
//      instead.  Either way the halo holds the reference's clamp-to-edge values.
//      i16 / u8 / bf16 / f16 inputs are staged as loaded and converted exactly
//      to f32 as the x pass reads them (the reference's UnaryFilter(p as f32)).
//   2. x pass: shared tile -> shared x-filtered f32 tile (TY + 2RY rows);
//   3. y pass: each thread filters MY consecutive rows of one column from a
//      register window;
//   4. z pass, "push" form: slice j contributes w[k] * v to the outputs
//      z = j + RZ - k; each thread keeps a ring of KZ accumulators per owned
//      column in registers, the ring slot being a compile-time function of
//      the phase j mod KZ, selected by a switch.
// FMA rounding runs the x, y and z passes as packed two-lane f32x2 FMAs.
// Reference rounding runs scalar acc = acc + x * w with separate roundings in
// ascending tap order, starting from zero, on f32 intermediates --
// bit-identical to conv.rs:26-36 pass by pass.  Slices clamped at the z ends
// are filtered once and pushed again.
//
// Work balance.  The (tile, z) units of the request are split evenly over a
// grid of (SMs x resident CTAs) CTAs; a CTA's share is one or two z-segments.
#include <atomic>

#include "fused_kernel.cuh"

namespace itkg {
namespace fusedk {
namespace {
const Entry kTableF32[] = ITKG_FUSED_TABLE(float);
}  // namespace
}  // namespace fusedk

const fusedk::Entry* fused_entries_f32(int* n) {
  *n = (int)(sizeof(fusedk::kTableF32) / sizeof(fusedk::kTableF32[0]));
  return fusedk::kTableF32;
}

namespace {

using fusedk::Entry;
using fusedk::FusedItem;
using fusedk::Fused3DArgs;
using KernelFn = void (*)(const CUtensorMap, const Fused3DArgs);
using MultiFn = void (*)(const FusedItem*, const CUtensorMap*, int, int64_t);

// Fault words, set when a bounded wait gives up: one per host thread (slot =
// the thread's ordinal modulo kFaultSlots), so that a wait given up under one
// thread's call does not fail another thread's call.
constexpr int kFaultSlots = 64;
__device__ unsigned int g_fused_fault_word[kFaultSlots];

std::atomic<int> g_next_fault_slot{0};
int fault_slot() {
  thread_local const int slot = g_next_fault_slot.fetch_add(1, std::memory_order_relaxed) % kFaultSlots;
  return slot;
}

#define ITKG_CUDA_ST(call)                                                            \
  do {                                                                                \
    const cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess)                                                            \
      return set_error(ITKG_ERROR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));     \
  } while (0)

#define ITKG_TRY_ST(expr)              \
  do {                                 \
    const itkg_status s_ = (expr);     \
    if (s_ != ITKG_SUCCESS) return s_; \
  } while (0)

const Entry* find_entry(int rx, int ry, int rz, int dtype) {
  int n = 0;
  const Entry* t = nullptr;
  switch (dtype) {
    case ITKG_F32: t = fused_entries_f32(&n); break;
    case ITKG_I16: t = fused_entries_i16(&n); break;
    case ITKG_U8: t = fused_entries_u8(&n); break;
    case ITKG_BF16: t = fused_entries_bf16(&n); break;
    case ITKG_F16: t = fused_entries_f16(&n); break;
    default: return nullptr;
  }
  for (int i = 0; i < n; ++i)
    if (t[i].rx == rx && t[i].ry == ry && t[i].rz == rz) return &t[i];
  return nullptr;
}

struct Occ {
  const void* fn;
  int dev;
  int blocks;
};
std::mutex g_occ_mu;
std::vector<Occ> g_occ;
std::vector<unsigned int*> g_fault_addr;  // per device

itkg_status resident_ctas(const void* fn, size_t smem, int nt, int* out) {
  int dev = 0;
  ITKG_CUDA_ST(cudaGetDevice(&dev));
  {
    std::lock_guard<std::mutex> lk(g_occ_mu);
    for (const Occ& o : g_occ)
      if (o.fn == fn && o.dev == dev) {
        *out = o.blocks;
        return ITKG_SUCCESS;
      }
  }
  ITKG_CUDA_ST(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0, sms = 0;
  ITKG_CUDA_ST(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, nt, smem));
  ITKG_CUDA_ST(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = std::max(1, per_sm) * sms;
  std::lock_guard<std::mutex> lk(g_occ_mu);
  g_occ.push_back({fn, dev, blocks});
  *out = blocks;
  return ITKG_SUCCESS;
}

// Device address of the fault word on the current device.
itkg_status fault_address(unsigned int** out) {
  int dev = 0;
  ITKG_CUDA_ST(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_occ_mu);
  if ((int)g_fault_addr.size() <= dev) g_fault_addr.resize(dev + 1, nullptr);
  if (!g_fault_addr[dev]) {
    void* p = nullptr;
    ITKG_CUDA_ST(cudaGetSymbolAddress(&p, g_fused_fault_word));
    g_fault_addr[dev] = static_cast<unsigned int*>(p);
  }
  *out = g_fault_addr[dev] + fault_slot();
  return ITKG_SUCCESS;
}

bool fits_i32(int64_t v) { return v >= INT_MIN && v <= INT_MAX; }

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

CUtensorMapDataType tma_type(int dtype) {
  switch (dtype) {
    case ITKG_I16: return CU_TENSOR_MAP_DATA_TYPE_UINT16;  // raw 16-bit copy
    case ITKG_U8: return CU_TENSOR_MAP_DATA_TYPE_UINT8;
    case ITKG_BF16: return CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    case ITKG_F16: return CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    default: return CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  }
}

// TMA applies when the buffer base and pitches are 16-byte multiples and every
// tile's first column (tx0 - XA, relative to the buffer) is 16-byte aligned.
bool tma_ok(const FusedGeom& g, const Entry& e) {
  if (((uintptr_t)g.src & 15) || (g.src_pitch[1] & 15) || (g.src_pitch[2] & 15)) return false;
  if (((g.req_index[0] - g.src_origin[0]) % e.ae + e.ae) % e.ae != 0) return false;
  if (g.src_pitch[1] >= (1ll << 40) || g.src_pitch[2] >= (1ll << 40)) return false;
  return encode_fn() != nullptr;
}

// Kernel arguments and (when TMA applies) the tensor map of one request.
itkg_status build_args(const FusedGeom& g, const float* const w[kMaxDim], const Entry* e,
                       Fused3DArgs* ap, CUtensorMap* mapp, bool* tma) {
  Fused3DArgs& a = *ap;
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
  ITKG_TRY_ST(fault_address(&a.fault));
  a.wait_limit = wait_limit_cycles();
  for (int k = 0; k < 2 * e->rx + 1; ++k) a.wx[k] = w[0][k], a.wx2[k] = splat2_host(w[0][k]);
  for (int k = 0; k < 2 * e->ry + 1; ++k) a.wy[k] = w[1][k], a.wy2[k] = splat2_host(w[1][k]);
  for (int k = 0; k < 2 * e->rz + 1; ++k) a.wz[k] = w[2][k], a.wz2[k] = splat2_host(w[2][k]);

  CUtensorMap& map = *mapp;
  std::memset(&map, 0, sizeof map);
  *tma = tma_ok(g, *e);
  if (*tma) {
    const cuuint64_t dims[3] = {(cuuint64_t)g.src_size[0], (cuuint64_t)g.src_size[1],
                                (cuuint64_t)g.src_size[2]};
    const cuuint64_t strides[2] = {(cuuint64_t)g.src_pitch[1], (cuuint64_t)g.src_pitch[2]};
    const cuuint32_t box[3] = {(cuuint32_t)e->bw, (cuuint32_t)e->ih, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = encode_fn()(&map, tma_type(e->dtype), 3, const_cast<void*>(g.src), dims, strides,
                             box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(ITKG_ERROR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  }
  return ITKG_SUCCESS;
}

const char* kernel_name(int dtype, bool ref, bool tma) {
  static const char* names[5][2][2] = {
      {{"fused3d_f32_fma", "fused3d_f32_fma_tma"}, {"fused3d_f32_ref", "fused3d_f32_ref_tma"}},
      {{"fused3d_i16_fma", "fused3d_i16_fma_tma"}, {"fused3d_i16_ref", "fused3d_i16_ref_tma"}},
      {{"fused3d_u8_fma", "fused3d_u8_fma_tma"}, {"fused3d_u8_ref", "fused3d_u8_ref_tma"}},
      {{"fused3d_bf16_fma", "fused3d_bf16_fma_tma"}, {"fused3d_bf16_ref", "fused3d_bf16_ref_tma"}},
      {{"fused3d_f16_fma", "fused3d_f16_fma_tma"}, {"fused3d_f16_ref", "fused3d_f16_ref_tma"}}};
  return names[dtype][ref ? 1 : 0][tma ? 1 : 0];
}

// Shape checks common to single and multi-request launches.
bool geometry_ok(const FusedGeom& g) {
  if (g.dim != 3 || g.comps != 1 || g.out_dtype == ITKG_I16) return false;
  for (int d = 0; d < 3; ++d)
    if (!fits_i32(g.lo[d]) || !fits_i32(g.hi[d]) || !fits_i32(g.src_origin[d]) ||
        !fits_i32(g.dst_origin[d]) || !fits_i32(g.req_index[d] + g.req_size[d]) ||
        !fits_i32(g.req_index[d] - 64))
      return false;
  const int64_t span = (g.hi[0] - g.src_origin[0] + 1) * g.src_pitch[0] +
                       (g.hi[1] - g.src_origin[1] + 1) * g.src_pitch[1];
  if (!fits_i32(span)) return false;
  if (g.src_pitch[0] != dtype_size(g.in_dtype)) return false;
  return true;
}

}  // namespace

itkg_status max_resident_ctas(const void* fn, size_t smem, int nt, int* out) {
  return resident_ctas(fn, smem, nt, out);
}

itkg_status device_fault_word(unsigned int** out) { return fault_address(out); }

itkg_status encode_input_map(const FusedGeom& g, int box_w, int box_h, void* map_out) {
  if (!encode_fn()) return set_error(ITKG_ERROR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
  CUtensorMap& map = *static_cast<CUtensorMap*>(map_out);
  std::memset(&map, 0, sizeof map);
  const cuuint64_t dims[3] = {(cuuint64_t)g.src_size[0], (cuuint64_t)g.src_size[1], (cuuint64_t)g.src_size[2]};
  const cuuint64_t strides[2] = {(cuuint64_t)g.src_pitch[1], (cuuint64_t)g.src_pitch[2]};
  const cuuint32_t box[3] = {(cuuint32_t)box_w, (cuuint32_t)box_h, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = encode_fn()(&map, tma_type(g.in_dtype), 3, const_cast<void*>(g.src), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(ITKG_ERROR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return ITKG_SUCCESS;
}

itkg_status launch_fused(const FusedGeom& g, const float* const w[kMaxDim], void* stream,
                         bool dry_run) {
  if (g.u8pix) return ITKG_ERROR_UNSUPPORTED;  // u8 pixel arithmetic: two-pass or per-axis only
  if (g.dim == 2) return launch_fused2d(g, w, stream, dry_run);
  if (!geometry_ok(g)) return ITKG_ERROR_UNSUPPORTED;
  const Entry* e = find_entry(g.radius[0], g.radius[1], g.radius[2], g.in_dtype);
  if (!e) return ITKG_ERROR_UNSUPPORTED;
  if (!tma_ok(g, *e)) {
    // the cp.async gather handles f32 with 4-byte aligned rows only
    if (g.in_dtype != ITKG_F32) return ITKG_ERROR_UNSUPPORTED;
    if (((uintptr_t)g.src & 3) || (g.src_pitch[1] & 3) || (g.src_pitch[2] & 3)) return ITKG_ERROR_UNSUPPORTED;
  }
  if (dry_run) return ITKG_SUCCESS;

  Fused3DArgs a;
  CUtensorMap map;
  bool tma = false;
  ITKG_TRY_ST(build_args(g, w, e, &a, &map, &tma));
  const bool ref = g.rounding == ITKG_ROUND_REFERENCE;
  KernelFn fn = e->fn[ref ? 1 : 0][tma ? 1 : 0];
  if (!fn) return set_error(ITKG_ERROR_UNSUPPORTED, "no fused kernel for this input layout");
  int resident = 0;
  ITKG_TRY_ST(resident_ctas(reinterpret_cast<const void*>(fn), e->smem, e->nt, &resident));
  const int64_t grid = std::min<int64_t>(a.units, resident);
  fn<<<(unsigned)grid, e->nt, e->smem, static_cast<cudaStream_t>(stream)>>>(map, a);
  note_launch(kernel_name(g.in_dtype, ref, tma));
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "fused3d launch: %s", cudaGetErrorString(err));
  return ITKG_SUCCESS;
}

itkg_status launch_fused_vjp(int mode, const FusedGeom& g, const float* const w[kMaxDim],
                             const float* const prefix[kMaxDim], const void* ybar,
                             const int64_t* ybar_pitch, const int64_t* ybar_origin, double* partials,
                             int* grid_out, bool accumulate, void* stream, bool dry_run) {
  if (!geometry_ok(g) || g.in_dtype != ITKG_F32 || g.out_dtype != ITKG_F32) return ITKG_ERROR_UNSUPPORTED;
  const Entry* e = find_entry(g.radius[0], g.radius[1], g.radius[2], ITKG_F32);
  if (!e || !e->vjp[mode == fusedk::kAdj ? 1 : 0] || !tma_ok(g, *e)) return ITKG_ERROR_UNSUPPORTED;
  KernelFn fn = e->vjp[mode == fusedk::kAdj ? 1 : 0];
  int resident = 0;
  ITKG_TRY_ST(resident_ctas(reinterpret_cast<const void*>(fn), e->smem, e->nt, &resident));
  const int64_t units = ((g.req_size[0] + e->tx - 1) / e->tx) * ((g.req_size[1] + e->ty - 1) / e->ty) *
                        g.req_size[2];
  if (grid_out) *grid_out = (int)std::min<int64_t>(units, resident);
  if (dry_run) return ITKG_SUCCESS;
  Fused3DArgs a;
  CUtensorMap map;
  bool tma = false;
  ITKG_TRY_ST(build_args(g, w, e, &a, &map, &tma));
  if (!tma) return set_error(ITKG_ERROR_UNSUPPORTED, "fused VJP needs TMA-aligned buffers");
  a.ybar = static_cast<const char*>(ybar);
  for (int d = 0; d < 3; ++d) {
    a.ybar_pitch[d] = ybar_pitch ? ybar_pitch[d] : 0;
    a.ybar_origin[d] = ybar_origin ? (int32_t)ybar_origin[d] : 0;
  }
  a.accumulate = accumulate ? 1 : 0;
  a.partials = partials;
  if (prefix)
    for (int d = 0; d < 3; ++d) {
      float* P = d == 0 ? a.px : (d == 1 ? a.py : a.pz);
      for (int k = 0; k < 2 * g.radius[d] + 1; ++k) P[k] = prefix[d][k];
    }
  // every CTA writes its partial, so the grid is the resident count (or fewer units)
  const int64_t grid = std::min<int64_t>(a.units, resident);
  if (grid_out) *grid_out = (int)grid;
  fn<<<(unsigned)grid, e->nt, e->smem, static_cast<cudaStream_t>(stream)>>>(map, a);
  note_launch(mode == fusedk::kAdj ? "fused3d_adjoint_f32" : "fused3d_dot_f32");
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "fused3d VJP launch: %s", cudaGetErrorString(err));
  return ITKG_SUCCESS;
}

struct FusedMultiGroup {
  const Entry* e;
  bool ref, tma;
  std::vector<FusedItem> items;
  std::vector<CUtensorMap> maps;
  FusedItem* d_items = nullptr;
  CUtensorMap* d_maps = nullptr;
  int64_t total = 0;
  int grid = 0;
};
struct FusedMultiPlan {
  std::vector<FusedMultiGroup> groups;
};

itkg_status fused_multi_prepare(const std::vector<FusedGeom>& geoms,
                                const std::vector<std::vector<std::vector<float>>>& weights,
                                FusedMultiPlan** out, std::vector<std::string>* lines) {
  FusedMultiPlan* plan = new FusedMultiPlan();
  *out = plan;
  for (size_t i = 0; i < geoms.size(); ++i) {
    const FusedGeom& g = geoms[i];
    const Entry* e = find_entry(g.radius[0], g.radius[1], g.radius[2], g.in_dtype);
    if (!e) return set_error(ITKG_ERROR_UNSUPPORTED, "no fused kernel for item %zu", i);
    const float* w[kMaxDim] = {nullptr, nullptr, nullptr};
    for (int d = 0; d < g.dim; ++d) w[d] = weights[i][d].data();
    FusedItem item;
    std::memset(&item, 0, sizeof item);
    CUtensorMap map;
    bool tma = false;
    ITKG_TRY_ST(build_args(g, w, e, &item.a, &map, &tma));
    const bool ref = g.rounding == ITKG_ROUND_REFERENCE;
    if (!e->multi[ref ? 1 : 0][tma ? 1 : 0])
      return set_error(ITKG_ERROR_UNSUPPORTED, "no fused kernel for item %zu's input layout", i);
    FusedMultiGroup* grp = nullptr;
    for (FusedMultiGroup& q : plan->groups)
      if (q.e == e && q.ref == ref && q.tma == tma) grp = &q;
    if (!grp) {
      plan->groups.push_back(FusedMultiGroup());
      grp = &plan->groups.back();
      grp->e = e;
      grp->ref = ref;
      grp->tma = tma;
    }
    item.unit_begin = grp->total;
    grp->total += item.a.units;
    grp->items.push_back(item);
    grp->maps.push_back(map);
  }
  for (FusedMultiGroup& q : plan->groups) {
    ITKG_CUDA_ST(cudaMalloc(&q.d_items, sizeof(FusedItem) * q.items.size()));
    ITKG_CUDA_ST(cudaMalloc(&q.d_maps, sizeof(CUtensorMap) * q.maps.size()));
    ITKG_CUDA_ST(cudaMemcpy(q.d_items, q.items.data(), sizeof(FusedItem) * q.items.size(),
                            cudaMemcpyHostToDevice));
    ITKG_CUDA_ST(cudaMemcpy(q.d_maps, q.maps.data(), sizeof(CUtensorMap) * q.maps.size(),
                            cudaMemcpyHostToDevice));
    MultiFn fn = q.e->multi[q.ref ? 1 : 0][q.tma ? 1 : 0];
    int resident = 0;
    ITKG_TRY_ST(resident_ctas(reinterpret_cast<const void*>(fn), q.e->smem, q.e->nt, &resident));
    q.grid = (int)std::min<int64_t>(q.total, resident);
    if (lines)
      lines->push_back(std::string(kernel_name(q.e->dtype, q.ref, q.tma)) +
                       " multi-request launch: r=(" + std::to_string(q.e->rx) + "," +
                       std::to_string(q.e->ry) + "," + std::to_string(q.e->rz) + "), " +
                       std::to_string(q.items.size()) + " requests, " + std::to_string(q.total) +
                       " units, " + std::to_string(q.grid) + " CTAs");
  }
  return ITKG_SUCCESS;
}

itkg_status fused_multi_launch(const FusedMultiPlan* plan, void* stream) {
  for (const FusedMultiGroup& q : plan->groups) {
    MultiFn fn = q.e->multi[q.ref ? 1 : 0][q.tma ? 1 : 0];
    fn<<<q.grid, q.e->nt, q.e->smem, static_cast<cudaStream_t>(stream)>>>(q.d_items, q.d_maps,
                                                                           (int)q.items.size(), q.total);
    note_launch("fused3d_multi");
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "fused3d multi launch: %s", cudaGetErrorString(err));
  }
  return ITKG_SUCCESS;
}

void fused_multi_free(FusedMultiPlan* plan) {
  if (!plan) return;
  for (FusedMultiGroup& q : plan->groups) {
    if (q.d_items) cudaFree(q.d_items);
    if (q.d_maps) cudaFree(q.d_maps);
  }
  delete plan;
}

itkg_status fused_fault_flag(unsigned int* flag, bool clear) {
  const size_t off = sizeof(unsigned int) * (size_t)fault_slot();
  cudaError_t e = cudaMemcpyFromSymbol(flag, g_fused_fault_word, sizeof(unsigned int), off);
  if (e != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "fault flag: %s", cudaGetErrorString(e));
  if (clear && *flag) {
    const unsigned int zero = 0;
    e = cudaMemcpyToSymbol(g_fused_fault_word, &zero, sizeof zero, off);
    if (e != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "fault flag: %s", cudaGetErrorString(e));
  }
  return ITKG_SUCCESS;
}

}  // namespace itkg
