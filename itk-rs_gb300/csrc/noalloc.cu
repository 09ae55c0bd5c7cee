// itkg_gaussian_generate_region_noalloc: the per-axis Gaussian path with its
// f32 (or u8) intermediates held in a fixed, file-scope device array instead
// of memory allocated per call.
//
// Who needs it: callers that must not allocate device memory while they run --
// for example an application that has handed all device memory to its own
// pool or caching allocator before calling in, or a latency-critical loop
// whose budget cannot absorb an allocation (or the synchronisation a
// cudaMalloc / cudaFree may imply).  They still pass their own input and
// output buffers; this entry point calls no cudaMalloc, cudaFree or other
// allocating routine.
//
// Limits and sharing:
//   - The array holds kNoAllocScratchBytes (32 MiB).  Every GPU on which the
//     library is loaded keeps this array for the life of the process.
//   - A 3-D request needs two intermediates, a 2-D request one, a 1-D request
//     none; each intermediate covers the requested region padded by the kernel
//     radius on the axes not yet filtered, at 4 bytes per component (f32
//     arithmetic) or 1 byte (u8 pixel arithmetic).  u8 pixel arithmetic also
//     keeps its per-tap table, (2r + 1) * 256 bytes for the largest radius r,
//     in the array.  A request that does not fit is rejected with
//     ITKG_ERROR_INVALID_ARGUMENT.
//   - All calls share the one array, which keeps whatever the last call left
//     in it.  Each pass writes every element of its intermediate before the
//     next pass reads it, so no clearing is needed.  Calls whose GPU work
//     overlaps (for example on two streams at once) race on the array and
//     must be serialised by the caller.
//   - The first call on a device that needs the array (any request of two or
//     more dimensions, and every u8 pixel-arithmetic request) looks up the
//     array's device address (one cudaGetSymbolAddress per device, made with
//     that device current).  Make that first call before any stream capture.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "internal.hpp"

namespace itkg {
namespace {

constexpr size_t kNoAllocScratchBytes = 32u << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_addr_mu;
std::vector<void*> g_addr;  // device address of g_noalloc_scratch, per device

// Looks up the array's device address for the current device (cached).  The
// host-side symbol is only a stand-in; kernels must be given this address.
itkg_status scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(ITKG_ERROR_NO_DEVICE, "cudaGetDevice: %s", cudaGetErrorString(e));
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if ((int)g_addr.size() <= dev) g_addr.resize(dev + 1, nullptr);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return set_error(ITKG_ERROR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return ITKG_SUCCESS;
}

uint64_t len(const itkg_region& r, int D) {
  uint64_t n = 1;
  for (int d = 0; d < D; ++d) n *= r.size[d];
  return n;
}

bool contains(const itkg_region& outer, const itkg_region& inner, int D) {
  for (int d = 0; d < D; ++d) {
    if (inner.size[d] == 0) return true;
    if (inner.index[d] < outer.index[d] ||
        inner.index[d] + (int64_t)inner.size[d] > outer.index[d] + (int64_t)outer.size[d])
      return false;
  }
  return true;
}

itkg_status check_device_image(const itkg_image* im, const char* name) {
  if (!im) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s is NULL", name);
  if (im->dim < 1 || im->dim > kMaxDim)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s: dim %d not in 1..3", name, im->dim);
  if (dtype_size(im->dtype) == 0)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s: unknown dtype %d", name, im->dtype);
  if (im->components != 1 && im->components != 3)
    return set_error(ITKG_ERROR_UNSUPPORTED, "%s: components must be 1 or 3", name);
  if (im->location != ITKG_DEVICE)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT,
                     "%s: the no-allocation entry point takes device buffers only", name);
  if (im->pitch[0] != (int64_t)im->components * dtype_size(im->dtype))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s: pitch[0] must equal the pixel size", name);
  for (int d = 1; d < im->dim; ++d)
    if (im->pitch[d] <= 0 || im->pitch[d] % dtype_size(im->dtype) != 0)
      return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s: pitch[%d] invalid", name, d);
  if (!im->data && len(im->region, im->dim) != 0)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s: data is NULL", name);
  return ITKG_SUCCESS;
}

void fill3(const itkg_region& r, int D, int64_t* index, int64_t* size) {
  for (int d = 0; d < kMaxDim; ++d) {
    index[d] = d < D ? r.index[d] : 0;
    size[d] = d < D ? (int64_t)r.size[d] : 1;
  }
}

}  // namespace
}  // namespace itkg

using namespace itkg;

extern "C" itkg_status itkg_gaussian_generate_region_noalloc(
    const itkg_image* input, const itkg_region* largest, const itkg_region* requested,
    const itkg_gaussian_params* params, itkg_image* output, void* stream) {
  itkg_status st = check_device_image(input, "input");
  if (st != ITKG_SUCCESS) return st;
  if ((st = check_device_image(output, "output")) != ITKG_SUCCESS) return st;
  if (!largest || !requested || !params)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "NULL region or params");
  if (params->arithmetic != ITKG_ARITH_F32 && params->arithmetic != ITKG_ARITH_PIXEL_U8)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "unknown arithmetic %d", params->arithmetic);
  if (params->rounding != ITKG_ROUND_REFERENCE && params->rounding != ITKG_ROUND_FMA)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "unknown rounding %d", params->rounding);
  if (params->reserved != 0) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "reserved must be 0");
  const int D = input->dim;
  if (output->dim != D || output->components != input->components)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "input/output dim or components differ");
  const bool u8pix = params->arithmetic == ITKG_ARITH_PIXEL_U8;
  if (u8pix && (input->dtype != ITKG_U8 || output->dtype != ITKG_U8))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "u8 pixel arithmetic needs u8 input and output");
  if (!u8pix && output->dtype == ITKG_I16)
    return set_error(ITKG_ERROR_UNSUPPORTED, "i16 output is not provided");
  if (len(*requested, D) == 0) return ITKG_SUCCESS;
  if (!contains(*largest, *requested, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "requested region lies outside the largest region");
  if (!contains(output->region, *requested, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "output buffer does not contain the requested region");

  // Radii and weights (gaussian.rs:24-40), input region (gaussian.rs:52-57).
  uint64_t radii[kMaxDim] = {0, 0, 0};
  // Host weights on the stack: the call makes no heap allocation either.
  double w64[kMaxDim][kMaxParamTaps];
  float w32[kMaxDim][kMaxParamTaps];
  for (int d = 0; d < D; ++d) {
    radii[d] = itkg_kernel_radius(params->sigma, input->spacing[d]);
    if (radii[d] > (uint64_t)(kMaxParamTaps - 1) / 2)
      return set_error(ITKG_ERROR_INVALID_ARGUMENT, "kernel radius %llu exceeds %d",
                       (unsigned long long)radii[d], (kMaxParamTaps - 1) / 2);
    if ((st = itkg_build_kernel(params->sigma / input->spacing[d], radii[d], w64[d])) != ITKG_SUCCESS)
      return st;
    for (uint64_t k = 0; k < 2 * radii[d] + 1; ++k) w32[d][k] = (float)w64[d][k];
  }
  itkg_region in_reg;
  if ((st = itkg_gaussian_input_region_for_output(requested, largest, D, input->spacing,
                                                  params->sigma, &in_reg)) != ITKG_SUCCESS)
    return st;
  if (!contains(input->region, in_reg, D))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT,
                     "input buffer does not cover input_region_for_output(requested)");

  // Intermediate regions (gaussian.rs:79-85) and their place in the array.
  const int sdt = u8pix ? ITKG_U8 : ITKG_F32;
  const size_t esz = (size_t)input->components * dtype_size(sdt);
  itkg_region regs[kMaxDim];
  size_t bytes[kMaxDim] = {0, 0, 0};
  for (int a = 0; a < D; ++a) {
    if (a + 1 < D) {
      uint64_t rem[kMaxDim] = {0, 0, 0};
      for (int d = a + 1; d < D; ++d) rem[d] = radii[d];
      itkg_region padded;
      itkg_region_padded_per_axis(requested, D, rem, &padded);
      itkg_region_clipped_to(&padded, D, largest, &regs[a]);
      bytes[a] = (size_t)len(regs[a], D) * esz;
    } else {
      regs[a] = *requested;
    }
  }
  // Pass a writes slot a % 2; slot 1 starts at a 256-byte boundary after slot 0.
  // u8 pixel arithmetic also keeps its per-tap table of (2r + 1) * 256 bytes
  // (r the largest radius) in the array, after the slots; every pass rebuilds
  // the table in place before it filters, in order on the caller's stream.
  const size_t slot0 = D > 1 ? bytes[0] : 0;
  const size_t slot1 = D > 2 ? bytes[1] : 0;
  const size_t off1 = (slot0 + 255) / 256 * 256;
  const size_t off_lut = (off1 + slot1 + 255) / 256 * 256;
  uint64_t rmax = 0;
  for (int d = 0; d < D; ++d) rmax = radii[d] > rmax ? radii[d] : rmax;
  const size_t lut_bytes = u8pix ? (size_t)(2 * rmax + 1) * 256 : 0;
  if (u8pix && rmax > (uint64_t)kMaxU8Radius)
    return set_error(ITKG_ERROR_UNSUPPORTED, "u8 pixel arithmetic supports radius <= %d", kMaxU8Radius);
  const size_t need = u8pix ? off_lut + lut_bytes : off1 + slot1;
  if (need > kNoAllocScratchBytes || slot0 > kNoAllocScratchBytes)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT,
                     "intermediates need %zu bytes; the no-allocation scratch holds %zu bytes",
                     need, kNoAllocScratchBytes);
  void* scratch = nullptr;
  if ((D > 1 || u8pix) && (st = scratch_address(&scratch)) != ITKG_SUCCESS) return st;
  char* slots[2] = {static_cast<char*>(scratch), static_cast<char*>(scratch) + off1};
  void* lut = u8pix ? static_cast<void*>(static_cast<char*>(scratch) + off_lut) : nullptr;

  // D passes, each a convolve_axis (conv.rs:11-41).
  const itkg_image* cur = input;
  itkg_image tmp[2];
  for (int a = 0; a < D; ++a) {
    const itkg_image* nxt = output;
    if (a + 1 < D) {
      itkg_image& t = tmp[a & 1];
      std::memset(&t, 0, sizeof t);
      t.dim = D;
      t.dtype = sdt;
      t.components = input->components;
      t.location = ITKG_DEVICE;
      t.region = regs[a];
      t.pitch[0] = (int64_t)esz;
      t.pitch[1] = t.pitch[0] * (int64_t)regs[a].size[0];
      t.pitch[2] = t.pitch[1] * (int64_t)(D >= 2 ? regs[a].size[1] : 1);
      t.data = slots[a & 1];
      nxt = &t;
    }
    AxisArgs args;
    std::memset(&args, 0, sizeof args);
    args.src = cur->data;
    args.dst = nxt->data;
    for (int d = 0; d < kMaxDim; ++d) {
      args.src_origin[d] = d < D ? cur->region.index[d] : 0;
      args.src_pitch[d] = d < D ? cur->pitch[d] : 0;
      args.dst_origin[d] = d < D ? nxt->region.index[d] : 0;
      args.dst_pitch[d] = d < D ? nxt->pitch[d] : 0;
    }
    fill3(regs[a], D, args.out_index, args.out_size);
    args.lo = largest->index[a];
    args.hi = largest->index[a] + (int64_t)largest->size[a] - 1;
    args.axis = a;
    args.radius = (int32_t)radii[a];
    args.comps = input->components;
    if (u8pix) {
      st = launch_conv_axis_u8(args, w64[a], stream, lut);
    } else {
      const int in_dt = a == 0 ? input->dtype : ITKG_F32;
      const int out_dt = a + 1 < D ? ITKG_F32 : output->dtype;
      st = launch_conv_axis_f32(args, w32[a], in_dt, out_dt, params->rounding, stream);
    }
    if (st != ITKG_SUCCESS) return st;
    cur = nxt;
  }
  set_last_kernel(u8pix ? "noalloc_per_axis_u8_pixel" : "noalloc_per_axis_f32");
  return ITKG_SUCCESS;
}
