// Internal declarations shared by the C-ABI layer (abi.cpp) and the CUDA
// translation units.  Nothing here is part of the public ABI.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "itkg.h"

namespace itkg {

constexpr int kMaxDim = ITKG_MAX_DIM;

// Largest tap count the per-axis kernels take by value as a launch parameter
// (r <= 384: 769 f32 weights = 3076 bytes, under the classic 4 KB limit).
constexpr int kMaxParamTaps = 769;
// Largest radius the u8 pixel-arithmetic path supports (LUT of K*256 bytes
// in shared memory, K <= 255).
constexpr int kMaxU8Radius = 127;

// ---- error reporting (thread-local) ----------------------------------------
itkg_status set_error(itkg_status st, const char* fmt, ...);
void set_last_kernel(const char* name);
// Called at every kernel launch: bumps the process-wide launch counter and
// records the kernel name for itkg_last_kernel().
void note_launch(const char* name);

// ---- dtype helpers --------------------------------------------------------
inline int dtype_size(int dt) {
  switch (dt) {
    case ITKG_F32: return 4;
    case ITKG_I16: return 2;
    case ITKG_U8: return 1;
    case ITKG_BF16: return 2;
    case ITKG_F16: return 2;
    default: return 0;
  }
}

// ---- one separable pass over one axis --------------------------------------
// Output voxel o (absolute index, inside out_index/out_size) gets
//   sum_k w[k] * src[o with o[axis] := clamp(o[axis] + k - r, lo, hi)]
// src/dst addresses: base + sum_d (idx[d] - origin[d]) * pitch[d] + c * elem.
struct AxisArgs {
  const void* src;
  void* dst;
  int64_t src_origin[kMaxDim];
  int64_t src_pitch[kMaxDim];  // bytes
  int64_t dst_origin[kMaxDim];
  int64_t dst_pitch[kMaxDim];  // bytes
  int64_t out_index[kMaxDim];
  int64_t out_size[kMaxDim];
  int64_t lo, hi;              // clamp bounds on `axis` (absolute)
  int32_t axis;
  int32_t radius;
  int32_t comps;
  int32_t pad_;
};

struct AxisWeightsF32 {
  float w[kMaxParamTaps];
};

struct AxisWeightsF64 {  // u8 pixel path: exact f64 weights
  double w[kMaxParamTaps / 2];
};

// conv_axis.cu
itkg_status launch_conv_axis_f32(const AxisArgs& a, const float* w, int in_dtype,
                                 int out_dtype, int rounding, void* stream);
// lut_buf: 256-byte aligned device buffer of at least (2 radius + 1) * 256
// bytes for the per-tap table, or NULL to take it from scratch_alloc.  The
// table kernel and the filter kernel run in order on `stream`, so one buffer
// may serve consecutive calls on that stream.
itkg_status launch_conv_axis_u8(const AxisArgs& a, const double* w, void* stream, void* lut_buf = nullptr);

// ---- fused whole-filter kernels ---------------------------------------------
// Geometry shared by every fused launch.  All indices absolute; the clamp
// bounds on every axis are the largest region.
struct FusedGeom {
  const void* src;
  void* dst;
  int64_t src_origin[kMaxDim];
  int64_t src_size[kMaxDim];   // input buffer extent (region size)
  int64_t src_pitch[kMaxDim];  // bytes
  int64_t dst_origin[kMaxDim];
  int64_t dst_pitch[kMaxDim];  // bytes
  int64_t req_index[kMaxDim];  // requested region
  int64_t req_size[kMaxDim];
  int64_t lo[kMaxDim];         // largest region bounds
  int64_t hi[kMaxDim];
  int32_t radius[kMaxDim];
  int32_t dim;
  int32_t comps;
  int32_t in_dtype;
  int32_t out_dtype;
  int32_t rounding;
  int32_t u8pix;  // u8 pixel arithmetic (NumericPixel for u8); only the two-pass kernels take it
};

// two_pass.cu: the f32 constants c[k] of the u8 pixel-arithmetic kernels for
// the f64 taps w[0 .. K): for every v in 0 .. 255, floor(f32 fma(v, c[k], 0.5))
// must equal round(v as f64 * w[k]).clamp(0, 255) (src/pixel.rs:430-435).
// Tries the nearest f32 first, then its neighbours; false if no f32 within 64
// ulps qualifies for some tap (the caller then runs the per-axis passes).
bool u8_pixel_tap_consts(const double* w, int K, float* c);

// fused.cu: returns ITKG_ERROR_UNSUPPORTED (without setting an error) when no
// fused kernel covers the geometry; the caller then uses the per-axis path.
itkg_status launch_fused(const FusedGeom& g, const float* const w[kMaxDim], void* stream,
                         bool dry_run);

// fused2d.cu: the 2-D counterpart (f32 input, 1 or 3 components, radius <= 12).
itkg_status launch_fused2d(const FusedGeom& g, const float* const w[kMaxDim], void* stream,
                           bool dry_run);
// tile2d.cu: the same geometries on 64 x 32 tiles staged at once (small and
// medium images); launch_fused2d chooses between the two.
itkg_status launch_tile2d(const FusedGeom& g, const float* const w[kMaxDim], void* stream, bool dry_run);
// tile2d.cu: many 2-D requests as one tile-kernel launch per kernel class
// (radius, components, rounding); the batch's 2-D items.
struct Tile2DMultiPlan;
itkg_status tile2d_multi_prepare(const std::vector<FusedGeom>& geoms,
                                 const std::vector<std::vector<std::vector<float>>>& weights,
                                 Tile2DMultiPlan** plan, std::vector<std::string>* lines);
int tile2d_multi_groups(const Tile2DMultiPlan* plan);
double tile2d_multi_work(const Tile2DMultiPlan* plan, int group);
itkg_status tile2d_multi_launch(const Tile2DMultiPlan* plan, int group, void* stream);
void tile2d_multi_free(Tile2DMultiPlan* plan);
// abi.cpp: the 2-D geometry and f32 weights of one request for the tile
// kernel (ITKG_ERROR_UNSUPPORTED when it does not apply).
itkg_status tile2d_geom_for(const itkg_image& in, const itkg_region& largest, const itkg_region& requested,
                            const itkg_gaussian_params& prm, const itkg_image& out, FusedGeom* g,
                            std::vector<std::vector<float>>* weights);
// abi.cpp: the 2-D kernel forced by itkg_debug_set_2d_kernel (0: chosen by size,
// 1: the tile kernel, 2: the row-marching kernel).
int kernel2d_override();

// abi.cpp: validates one 3-D request and fills its fused geometry and f32
// weights; ITKG_ERROR_UNSUPPORTED when no multi-request fused kernel covers it.
itkg_status fused_geom_for(const itkg_image& in, const itkg_region& largest,
                           const itkg_region& requested, const itkg_gaussian_params& prm,
                           const itkg_image& out, FusedGeom* g,
                           std::vector<std::vector<float>>* weights);

// fused.cu: many fused requests; requests sharing a kernel run as one
// persistent multi-request launch.  prepare (outside any stream capture)
// builds and uploads the request tables and appends one line per launch to
// `lines`; launch enqueues the launches; free releases the tables.
struct FusedMultiPlan;
itkg_status fused_multi_prepare(const std::vector<FusedGeom>& geoms,
                                const std::vector<std::vector<std::vector<float>>>& weights,
                                FusedMultiPlan** plan, std::vector<std::string>* lines);
itkg_status fused_multi_launch(const FusedMultiPlan* plan, void* stream);
void fused_multi_free(FusedMultiPlan* plan);

// fused.cu: VJP launches over a whole 3-D f32 image (FMA rounding, TMA only).
//   mode 1 (dot): partials[cta] = per-CTA sums of <ybar, G x> with the weights
//                 given (derivative weights on one axis give one term of
//                 dL/dsigma); *grid_out = number of partials written;
//   mode 2 (adjoint): dst (+)= G^T src with prefix sums `prefix` for the folds.
// ITKG_ERROR_UNSUPPORTED (no error set) when no fused kernel applies; dry_run
// only checks (and reports the grid).
itkg_status launch_fused_vjp(int mode, const FusedGeom& g, const float* const w[kMaxDim],
                             const float* const prefix[kMaxDim], const void* ybar,
                             const int64_t* ybar_pitch, const int64_t* ybar_origin, double* partials,
                             int* grid_out, bool accumulate, void* stream, bool dry_run);

// fused.cu helpers shared by the fused kernels' launchers:
//   max_resident_ctas: SMs x resident CTAs of `fn` (cached per device);
//   device_fault_word: address of the fault word on the current device;
//   encode_input_map: 3-D TMA tensor map (CUtensorMap, 128 bytes) over the
//   input buffer of `g` with a box_w x box_h x 1 box.
itkg_status max_resident_ctas(const void* fn, size_t smem, int nt, int* out);
itkg_status device_fault_word(unsigned int** out);
itkg_status encode_input_map(const FusedGeom& g, int box_w, int box_h, void* map_out);

// two_pass.cu: the 3-D forward as an x-y slice kernel plus a z kernel through
// an L2-sized f32 intermediate (rx == ry <= 12, rz <= 12, TMA-aligned input).
// ITKG_ERROR_UNSUPPORTED (no error set) when it does not apply.
// ush: if non-NULL, the z kernel stores UnsharpMaskFilter's point-wise step
// applied to the blur and to the input voxel instead of the blur itself
// (ush->cheap in FMA rounding, not in reference rounding; f32 input and output
// with 16-byte aligned rows of whole quads; else unsupported).
struct UnsharpConsts;
itkg_status launch_two_pass(const FusedGeom& g, const float* const w[kMaxDim], void* stream,
                            bool dry_run, const UnsharpConsts* ush = nullptr);

// two_pass.cu: per-CTA ranges of (block, slice) units, block-major, where a
// CTA's cost is its units plus 2 rz halo slices per block it touches; the
// smallest cost budget that lets at most `grid` CTAs (<= 1024) cover all
// units.  Returns the CTA count and fills split[0 .. count]; 0 if the units do
// not fit the table.
int z_split(int64_t qblocks, int64_t nz, int rz, int64_t grid, int32_t* split);

// one_trip.cu: the 3-D forward in one kernel (x, y and z passes on chip; f32
// input, rx == ry <= 8, rz <= 8, one component, TMA-aligned input).
// ITKG_ERROR_UNSUPPORTED (no error set) when it does not apply.
itkg_status launch_one_trip(const FusedGeom& g, const float* const w[kMaxDim], void* stream, bool dry_run);

// vjp2.cu: the 3-D VJP as z-adjoint and x-y kernels (rx == ry <= 12, rz <= 12,
// f32, whole image, 16-byte aligned rows of x and ybar).  sigma_out is a
// device double (added to with acc_sigma); xbar may be NULL, sigma_out too.
struct VjpTwoPass {
  const itkg_image* x;
  const itkg_image* ybar;
  itkg_image* xbar;
  double* sigma_out;
  bool acc_x, acc_sigma;
  const float* w[kMaxDim];   // weights per axis
  const float* dw[kMaxDim];  // their sigma derivatives
  int radius[kMaxDim];
};
itkg_status launch_vjp_two_pass(const VjpTwoPass& v, void* stream, bool dry_run);

// RecursiveGaussianFilter (recursive.cu): `in` device image covering `largest`,
// `out` device image covering `requested`; axis -1 = every axis.
void yvv_coeffs(double sigma, double out[4]);
itkg_status launch_recursive(const itkg_image& in, const itkg_region& largest, const itkg_region& requested,
                             double sigma, int axis, int rounding, const itkg_image& out, void* stream);
// Its derivative users: smoothing of `requested` in the input's pixel type,
// then the `kind` stencil (0 gradient magnitude, 1 Laplacian, 2 derivative,
// 3 gradient, 4 2-D Hessian; 5 the difference of two smoothings; 6 zero
// crossings of the Laplacian) into `out`.
itkg_status launch_recursive_derivative(const itkg_image& in, const itkg_region& largest,
                                        const itkg_region& requested, double sigma, double sigma2, int kind,
                                        int axis, int order, int rounding, const itkg_image& out, void* stream);

// UnsharpMaskFilter's point-wise step: its amount and threshold as the f32
// test (unsharp.cuh) uses them.
struct UnsharpConsts {
  double amount, threshold;  // the reference's values (the f64 sequence)
  float ah, al;              // amount = ah + al + r, |r| <= 2^-48 |amount|
  float thr_up, thr_dn;      // |e| > thr_up: the test passes; |e| < thr_dn: it fails
  int thr_neg;               // threshold < 0 (the test for e = 0)
  int a_exact;               // amount == ah exactly
  int fast;                  // 0: every voxel takes the f64 sequence
  int cheap;                 // FMA rounding: o + amount e by one f32 FMA
  float u8_min_pass;         // u8 pixels: |e| (an integer) passes the threshold test iff |e| >= this
};

UnsharpConsts unsharp_consts(double amount, double threshold, bool cheap);

// UnsharpMaskFilter's point-wise step (unsharp.cu): in / blur / out point at
// the first requested voxel of each image; pitches in bytes; m the requested
// size (unused axes 1).
itkg_status launch_unsharp(int dtype, int comps, const void* in, const int64_t* ip, const void* blur,
                           const int64_t* bp, void* out, const int64_t* op, const int64_t* m, double amount,
                           double threshold, int rounding, void* stream);

// BSplineDownsampleFilter's subsampling (callers.cu): dst[i] = src[2 i] on
// every axis; pointers at the region's first voxel, pitches in bytes, m the
// downsampled size (unused axes 1), elem the pixel's bytes.
itkg_status launch_subsample2(const void* src, const int64_t* sp, void* dst, const int64_t* dp, const int64_t* m,
                              int elem, void* stream);

// Demons and N4 point-wise kernels (registration.cu).  DemonsGeom: the fixed
// image (f32 rows at pitch fp elements, w x h at index (ox, oy)) and the
// moving image (rows at pitch mp, mw x mh at (mox, moy)), device pointers at
// each region's first pixel.
struct DemonsGeom {
  const float* fixed;
  int64_t fp, w, h, ox, oy;
  const float* moving;
  int64_t mp, mw, mh, mox, moy;
};
itkg_status launch_demons_step(const DemonsGeom& g, const double* dxi, const double* dyi, double* dxo, double* dyo,
                               double max_step, unsigned int* err, void* stream);
// out: interleaved VecPixel<f32, 2> rows at pitch op (pixels), or, with px and
// py non-NULL, two planar f32 images with rows at pitch pp (floats)
itkg_status launch_demons_to_f32(const double* dx, const double* dy, int64_t w, int64_t h, float* out, int64_t op,
                                 float* px, float* py, int64_t pp, void* stream);
itkg_status launch_interleave2(const float* a, const float* b, int64_t sp, int64_t w, int64_t h, float* out, int64_t op,
                               void* stream);
itkg_status launch_n4_init(const float* in, int64_t ip, int64_t w, int64_t h, double* corr, void* stream);
itkg_status launch_n4_log(const double* corr, int64_t n, double* ld, float* lf, void* stream);
int n4_blocks(int64_t n);
itkg_status launch_n4_update(const double* ld, const float* sm, int64_t n, double* corr, double* partials, int blocks,
                             void* stream);
itkg_status launch_n4_store(const double* corr, int64_t w, int64_t h, float* out, int64_t op, void* stream);

// Bumps the launch counter by n (graph replays).
void note_launches(uint64_t n, const char* name);

// Reads (and optionally clears) the fused kernels' device fault word, which a
// kernel sets when a bounded wait on a tile load gives up.
itkg_status fused_fault_flag(unsigned int* flag, bool clear);

// ---- VJP (vjp.cu): whole-image per-axis passes on f32 buffers ---------------
constexpr int kMaxVjpTaps = 385;  // radius <= 192

struct VjpAxisArgs {
  const float* in;   // pass input (v for dual passes)
  const float* din;  // dual passes: incoming derivative (NULL = zero)
  float* out;
  float* dout;       // dual passes: outgoing derivative
  int64_t in_pitch[kMaxDim];   // bytes (shared by in and din)
  int64_t out_pitch[kMaxDim];  // bytes (shared by out and dout)
  int64_t size[kMaxDim];       // image size (unused axes 1)
  int32_t axis;
  int32_t radius;
  int32_t accumulate;  // adjoint pass: out += result
  int32_t pad_;
};

struct DotArgs {  // sum over the image of p * q (two pitched f32 images)
  const float* p;
  const float* q;
  int64_t p_pitch[kMaxDim];
  int64_t q_pitch[kMaxDim];
  int64_t size[kMaxDim];
};

itkg_status launch_adjoint_axis(const VjpAxisArgs& a, const float* w, const float* prefix,
                                void* stream);
itkg_status launch_dual_axis(const VjpAxisArgs& a, const float* w, const float* dw, void* stream);
// vjp_lines_{dual,adj}.cu: the tiled passes for radii 13 .. 24; return
// ITKG_ERROR_UNSUPPORTED (without setting an error) outside that range or when
// the image does not fit their tile arithmetic.
itkg_status launch_line_dual(const VjpAxisArgs& a, const float* w, const float* dw, void* stream);
itkg_status launch_line_adjoint(const VjpAxisArgs& a, const float* w, const float* prefix, void* stream);
int dot_partial_blocks(int64_t n);
// partials: nblocks doubles of scratch; *out (device) = sum, or += with accumulate.
itkg_status launch_dot(const DotArgs& d, double* partials, int nblocks, double* out,
                       bool accumulate, void* stream);
// *out (+)= sum of n f64 partials, in a fixed order.
itkg_status launch_sum_partials(const double* partials, int n, double* out, bool accumulate,
                                void* stream);
// Squared error against t (DotArgs::q / q_pitch / size): ybar = 2 (y - t) into
// a dense buffer; *loss_out (+)= sum (y - t)^2, *sigma_out = sum ybar * dy
// (dy and sigma_out may be NULL: no sigma term).
// partials: 2 * nblocks doubles of scratch.  y, dy, ybar dense f32.
itkg_status launch_sqerr(const float* y, const float* dy, const DotArgs& t, float* ybar,
                         double* partials, int nblocks, double* loss_out, double* sigma_out,
                         bool accumulate_loss, void* stream);

// Clock cycles a kernel's bounded wait on a tile load may take before it
// gives up (abi.cpp; 2^31 unless a test lowered it).
long long wait_limit_cycles();

// ---- device scratch ---------------------------------------------------------
// Stream-ordered scratch from a library-owned memory pool of the current
// device (cudaMallocAsync / cudaFreeAsync on `stream`).
itkg_status scratch_alloc(void** p, size_t bytes, void* stream);
void scratch_free(void* p, void* stream);

}  // namespace itkg
