/*
 * itkg.h -- C ABI of the GB300 (sm_103a) separable Gaussian path.
 *
 * This is the boundary a host binding (Rust `extern "C"`, C++, Python ctypes)
 * calls in place of itk-rs's CPU implementation of GaussianFilter.  Types and
 * functions mirror the reference's pipeline API for that path:
 *
 *   itkg_region      <-> Region<D>                      (src/image.rs:12-15)
 *   itkg_image       <-> Image<P, D> + device residency (src/image.rs:82-87)
 *   itkg_gaussian_*  <-> GaussianFilter<S>               (src/filters/gaussian.rs:13-91)
 *   itkg_stream_full <-> stream_full                     (src/source.rs:81-98)
 *   itkg_split_region<-> split_region                    (src/region_splitter.rs:17-48)
 *
 * Conventions
 *   - Axis 0 is the fastest-varying axis (image.rs:111-120).  `dim` is D (1..3).
 *   - Every call returns an itkg_status; ITKG_SUCCESS is 0.  On failure,
 *     itkg_last_error() returns a message for the calling thread.  Where the
 *     reference panics (a buffer that does not cover the region a filter must
 *     read, capacity overflow for absurd radii) this ABI returns
 *     ITKG_ERROR_INVALID_ARGUMENT instead.
 *   - `stream` is an opaque cudaStream_t (NULL = legacy default stream).
 *     Device work is enqueued on it; calls that touch host buffers synchronise
 *     it before returning.
 *   - No CUDA or framework types appear in signatures: plain pointers, sizes.
 */
#ifndef ITKG_H
#define ITKG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ITKG_ABI_VERSION 1
#define ITKG_MAX_DIM 3

typedef enum itkg_status {
    ITKG_SUCCESS = 0,
    ITKG_ERROR_INVALID_ARGUMENT = 1, /* bad descriptor, region not covered, ... */
    ITKG_ERROR_UNSUPPORTED = 2,      /* dtype / dimension combination not provided */
    ITKG_ERROR_CUDA = 3,             /* CUDA runtime or driver error */
    ITKG_ERROR_OUT_OF_MEMORY = 4,
    ITKG_ERROR_NO_DEVICE = 5,        /* no usable sm_103 device */
    ITKG_ERROR_TIMEOUT = 6           /* a bounded device-side wait expired */
} itkg_status;

/* Storage type of one pixel component. */
typedef enum itkg_dtype {
    ITKG_F32 = 0,
    ITKG_I16 = 1,  /* read path: exact cast to f32 (UnaryFilter(i16 -> f32)) */
    ITKG_U8 = 2,   /* read: cast to f32 (or u8 pixel arithmetic); write: round+clamp */
    ITKG_BF16 = 3, /* storage only; arithmetic is f32 */
    ITKG_F16 = 4   /* storage only; arithmetic is f32 */
} itkg_dtype;

/* Where `itkg_image::data` lives. */
typedef enum itkg_location {
    ITKG_DEVICE = 0, /* device pointer on the current CUDA device */
    ITKG_HOST = 1    /* host pointer (pinned or pageable); staged by the library */
} itkg_location;

/* Pixel arithmetic of the filter. */
typedef enum itkg_arithmetic {
    /* f32 arithmetic: NumericPixel for f32 (src/pixel.rs:416-421) and, per
     * component, VecPixel<f32,3> (src/pixel.rs:479-495).  i16/u8/bf16/f16
     * inputs are converted exactly to f32 on load, which is the reference's
     * UnaryFilter(p as f32) -> GaussianFilter<f32> chain
     * (examples/blur_png.rs:35-37, tests/blur_png.rs:38-40). */
    ITKG_ARITH_F32 = 0,
    /* GaussianFilter<Image<u8>>: per tap round(x as f64 * w).clamp(0,255)
     * as u8, u8 accumulator with wrapping adds (src/pixel.rs:430-435).
     * Requires u8 input and u8 output. */
    ITKG_ARITH_PIXEL_U8 = 1
} itkg_arithmetic;

/* Rounding discipline of the f32 arithmetic. */
typedef enum itkg_rounding {
    /* Bit-exact with the reference: acc = 0; acc = acc + x * (f32)w in
     * ascending tap order, products and sums rounded separately, f32
     * intermediates between passes (src/filters/conv.rs:26-36). */
    ITKG_ROUND_REFERENCE = 0,
    /* acc = fma(x, w, acc) in the same tap order; within 1e-5 normwise
     * relative of the reference (typically ~1e-7). */
    ITKG_ROUND_FMA = 1
} itkg_rounding;

/* Kernel selection. */
typedef enum itkg_algorithm {
    ITKG_ALGO_AUTO = 0,     /* two-pass, else fused, else per-axis: the first that fits */
    ITKG_ALGO_FUSED = 1,    /* one kernel for all passes; ITKG_ERROR_UNSUPPORTED if none fits */
    ITKG_ALGO_PER_AXIS = 2, /* D separate passes through an f32 scratch buffer */
    ITKG_ALGO_TWO_PASS = 3, /* 3-D: an x-y slice kernel and a z kernel through an f32
                               intermediate sized for L2; ITKG_ERROR_UNSUPPORTED if it
                               does not fit (needs rx == ry <= 12, rz <= 12, one component,
                               16-byte aligned input rows) */
    ITKG_ALGO_ONE_TRIP = 4  /* 3-D: one kernel, x, y and z passes on chip, each voxel
                               read from and written to HBM once; ITKG_ERROR_UNSUPPORTED
                               if it does not fit (needs f32 input, rx == ry <= 8,
                               rz <= 8, one component, 16-byte aligned input rows) */
} itkg_algorithm;

/* Region<D> (src/image.rs:12-15): index[d], size[d] for d < dim. */
typedef struct itkg_region {
    int64_t index[ITKG_MAX_DIM];
    uint64_t size[ITKG_MAX_DIM];
} itkg_region;

/* Image<P, D> (src/image.rs:82-87) with an explicit, possibly padded, layout.
 * Pixel (i0, i1, i2) of the buffered region lives at
 *   data + (i0 - region.index[0]) * pitch[0]
 *        + (i1 - region.index[1]) * pitch[1] + (i2 - region.index[2]) * pitch[2]
 * pitch[0] must equal components * sizeof(dtype) (packed pixels). */
typedef struct itkg_image {
    int32_t dim;
    int32_t dtype;      /* itkg_dtype */
    int32_t components; /* 1 = scalar, 3 = VecPixel<_, 3> (interleaved); 2 = VecPixel<f32, 2>
                           (2-D displacement fields and gradient outputs) */
    int32_t location;   /* itkg_location */
    itkg_region region; /* buffered region (BufferedRegion) */
    int64_t pitch[ITKG_MAX_DIM]; /* bytes between neighbours along each axis */
    double spacing[ITKG_MAX_DIM];
    double origin[ITKG_MAX_DIM];
    void *data;
} itkg_image;

/* GaussianFilter { source, sigma } (src/filters/gaussian.rs:13-17) plus the
 * GPU execution choices. Zero-initialised params = reference rounding, f32
 * arithmetic, automatic kernel choice. */
typedef struct itkg_gaussian_params {
    double sigma;       /* standard deviation in physical units */
    int32_t arithmetic; /* itkg_arithmetic */
    int32_t rounding;   /* itkg_rounding */
    int32_t algorithm;  /* itkg_algorithm */
    int32_t reserved;   /* must be 0 */
} itkg_gaussian_params;

/* ---- library ----------------------------------------------------------- */

int32_t itkg_abi_version(void);
/* Message of the last failing call on this thread ("" if none). */
const char *itkg_last_error(void);
/* Name of the kernel the last successful filter call on this thread ran. */
const char *itkg_last_kernel(void);
/* Number of CUDA kernels this library has launched in this process. */
uint64_t itkg_launch_counter(void);

/* ---- diagnostics and fault injection (no counterpart in the reference) ---- */

/* Number of device scratch allocations (stream-ordered allocations from the
 * library's memory pool, made inside filter calls) in this process.
 * itkg_device_alloc and itkg_image_alloc_device are not counted. */
uint64_t itkg_scratch_alloc_counter(void);
/* Test hook: the scratch allocation after the next `after` ones fails with
 * ITKG_ERROR_OUT_OF_MEMORY (once); a negative value cancels. */
void itkg_debug_fail_scratch_alloc(int64_t after);
/* Test hook: a kernel's bounded wait on a tile load gives up after `cycles`
 * clock cycles instead of about 2^31 (values <= 0 restore that default).
 * A wait that gives up sets the calling thread's device fault word (see
 * itkg_device_fault); the kernel still lets its loads land before it exits. */
void itkg_debug_set_wait_limit(int64_t cycles);
/* Test hook: which kernel runs the fused 2-D forward (2-D images and the
 * slices of SliceBySliceFilter): 1 the tile kernel, 2 the row-marching
 * kernel, anything else the library's choice.  Results are the same. */
void itkg_debug_set_2d_kernel(int32_t which);

/* ---- host-side geometry (no device needed) ------------------------------ */

/* GaussianFilter::kernel_radius (gaussian.rs:24-27): ceil(3*sigma/spacing)
 * with Rust's saturating float->usize cast (NaN and negatives give 0). */
uint64_t itkg_kernel_radius(double sigma, double spacing);

/* GaussianFilter::build_kernel (gaussian.rs:29-40): 2*radius+1 f64 weights. */
itkg_status itkg_build_kernel(double sigma_pixels, uint64_t radius, double *weights_out);

/* Region::padded_per_axis (image.rs:28-37). */
itkg_status itkg_region_padded_per_axis(const itkg_region *r, int32_t dim,
                                        const uint64_t *radii, itkg_region *out);
/* Region::clipped_to (image.rs:52-64). */
itkg_status itkg_region_clipped_to(const itkg_region *r, int32_t dim,
                                   const itkg_region *bounds, itkg_region *out);

/* GaussianFilter::input_region_for_output (gaussian.rs:52-57). */
itkg_status itkg_gaussian_input_region_for_output(const itkg_region *output_region,
                                                  const itkg_region *largest, int32_t dim,
                                                  const double *spacing, double sigma,
                                                  itkg_region *input_region);

/* split_region (region_splitter.rs:17-48). Writes at most `capacity` pieces and
 * stores the number of pieces split_region yields in *count. */
itkg_status itkg_split_region(const itkg_region *region, int32_t dim, uint64_t num_pieces,
                              itkg_region *pieces, uint64_t capacity, uint64_t *count);

/* ---- device memory helpers ---------------------------------------------- */

itkg_status itkg_device_count(int32_t *count);
itkg_status itkg_set_device(int32_t device);
itkg_status itkg_device_alloc(size_t bytes, void **ptr);
itkg_status itkg_device_free(void *ptr);
itkg_status itkg_host_alloc_pinned(size_t bytes, void **ptr);
itkg_status itkg_host_free_pinned(void *ptr);
/* kind: 0 host->device, 1 device->host, 2 device->device, 3 default (UVA). */
itkg_status itkg_memcpy(void *dst, const void *src, size_t bytes, int32_t kind, void *stream);
itkg_status itkg_memset_device(void *dst, int32_t value, size_t bytes, void *stream);
itkg_status itkg_stream_synchronize(void *stream);
/* A non-blocking stream on the current device (for callers with no CUDA
 * runtime of their own, e.g. one stream per host thread), and its release. */
itkg_status itkg_stream_create(void **stream);
itkg_status itkg_stream_destroy(void *stream);
/* Device-side fault word of the calling host thread on the current device:
 * non-zero after a kernel launched by this thread gave up a bounded wait on a
 * tile load (the kernel then returned early and its output is incomplete).
 * Each host thread has its own word (64 words; threads beyond the 64th share
 * them), so one thread's timeout does not fail another's calls.  clear != 0
 * resets it. */
itkg_status itkg_device_fault(int32_t clear, uint32_t *flag);

/* Fill *img for a freshly allocated device image of `region`, with rows and
 * slices padded to 128-byte multiples (TMA-friendly), and allocate it. */
itkg_status itkg_image_alloc_device(itkg_image *img, int32_t dim, int32_t dtype,
                                    int32_t components, const itkg_region *region,
                                    const double *spacing, const double *origin);
itkg_status itkg_image_free(itkg_image *img);

/* Image::copy_from (image.rs:133-140): copy src->region into dst, whose
 * buffered region must contain it.  Either side may be host or device; the
 * call returns after the copy completes. */
itkg_status itkg_image_copy_from(itkg_image *dst, const itkg_image *src, void *stream);

/* ---- the filter ----------------------------------------------------------
 * GaussianFilter<S>::generate_region(requested) (gaussian.rs:59-91).
 *   input     the upstream's output: its buffered region must contain
 *             input_region_for_output(requested) (the reference requests
 *             exactly that region from its source, gaussian.rs:71-72)
 *   largest   source.largest_region(): the clamp-to-edge bounds
 *   requested region to produce; must lie inside `largest`
 *   output    buffered region must contain `requested`; only `requested` is
 *             written (stream_full writes pieces in place)
 * Spacing is taken from input->spacing. */
itkg_status itkg_gaussian_generate_region(const itkg_image *input, const itkg_region *largest,
                                          const itkg_region *requested,
                                          const itkg_gaussian_params *params,
                                          itkg_image *output, void *stream);

/* ---- the convolve_axis family ---------------------------------------------
 * The filters that run convolve_axis (conv.rs:11-41) with their own kernels:
 *   MeanFilter { source, radius }        mean.rs:27-84    box kernel of `radius` on every axis
 *   BoxMeanFilterN { source, radii }     mean.rs:103-137  box kernel of radii[d] on axis d
 *   BinomialBlurFilter { source, reps }  binomial_blur.rs:17-89  [1/4, 1/2, 1/4], `reps` rounds
 *   the Gaussian stages of UnsharpMaskFilter (edges.rs:406-430) and
 *   CannyEdgeDetectionFilter (edges.rs:562-577), which build their own kernels.
 * weights[d]: 2 radius[d] + 1 f64 weights of axis d (axes >= dim ignored),
 * each applied as x * (float)w in ascending order like the Gaussian's.
 * repetitions: rounds of one pass per axis (1 for all but the binomial blur;
 * 0 copies `requested`).  Pass (rep, axis) writes `requested` padded by
 * (repetitions - rep - 1) radii on every axis and one more on the axes after
 * `axis` (binomial_blur.rs:63-87); every pass clamps to `largest`.
 * arithmetic, rounding, algorithm: as for the Gaussian.  The single-launch
 * kernels (ITKG_ALGO_TWO_PASS, _FUSED) take one round of kernels that read the
 * same backwards; other calls run per axis (AUTO) or return
 * ITKG_ERROR_UNSUPPORTED (explicit TWO_PASS / FUSED). */
typedef struct itkg_separable_params {
    uint64_t radius[3];
    const double *weights[3];
    uint64_t repetitions;
    int32_t arithmetic;
    int32_t rounding;
    int32_t algorithm;
    int32_t reserved; /* 0 */
} itkg_separable_params;

/* box_kernel (mean.rs:15-18): 2*radius+1 weights of 1 / (2*radius+1). */
itkg_status itkg_box_kernel(uint64_t radius, double *weights_out);

/* input_region_for_output of the family: `output_region` padded by
 * radius[d] * repetitions on axis d, clipped to `largest` (mean.rs:49-57,
 * 120-122; binomial_blur.rs:44-53). */
itkg_status itkg_separable_input_region_for_output(const itkg_region *output_region,
                                                   const itkg_region *largest, int32_t dim,
                                                   const uint64_t *radius, uint64_t repetitions,
                                                   itkg_region *input_region);

/* generate_region of the family (same buffer rules as
 * itkg_gaussian_generate_region; the input buffer must contain
 * itkg_separable_input_region_for_output(requested)). */
itkg_status itkg_separable_generate_region(const itkg_image *input, const itkg_region *largest,
                                           const itkg_region *requested,
                                           const itkg_separable_params *params,
                                           itkg_image *output, void *stream);

/* ---- UnsharpMaskFilter (edges.rs:374-452) ----------------------------------
 * out = |I - blur(I)| > threshold ? I + amount * (I - blur(I)) : I, in f64,
 * converted to the pixel type (f32 `v as f32`; u8 round half away from zero,
 * clamped to [0, 255]).  blur is the convolve_axis family's pass over every
 * axis with one kernel: radius ceil(3 sigma), weights exp(-d^2 / (2 sigma^2))
 * divided by their f64 sum, sigma in pixels on every axis (the reference
 * ignores the spacing here), accumulated in the pixel type like
 * itkg_separable_generate_region.  Vector pixels: the formula reads the first
 * component and writes its result to every component (pixel.rs:93-98).
 * Input and output: same dtype (f32 or u8) and components; the input buffer
 * must contain itkg_separable_input_region_for_output(requested) with that
 * radius and one repetition. */
typedef struct itkg_unsharp_params {
    double sigma;     /* > 0, pixels */
    double amount;    /* UnsharpMaskFilter::new: 0.5 */
    double threshold; /* UnsharpMaskFilter::new: 0.0 */
    int32_t rounding; /* of the blur: itkg_rounding */
    int32_t reserved; /* 0 */
} itkg_unsharp_params;

/* The blur kernel of UnsharpMaskFilter (edges.rs:408, 415-424): *radius_out =
 * ceil(3 sigma); weights_out (may be NULL) receives its 2 * radius + 1 weights. */
itkg_status itkg_unsharp_kernel(double sigma, uint64_t *radius_out, double *weights_out, uint64_t capacity);

itkg_status itkg_unsharp_mask_generate_region(const itkg_image *input, const itkg_region *largest,
                                              const itkg_region *requested, const itkg_unsharp_params *params,
                                              itkg_image *output, void *stream);

/* ---- in-crate callers of GaussianFilter ------------------------------------
 * SliceBySliceFilter { source, sigma } (filters/spatial.rs:1284-1340), 3-D:
 * every z slice of `requested` is smoothed by a 2-D GaussianFilter with the x
 * and y spacing, clamped to the request's x-y window (the reference builds
 * each slice as an Image over that window).  `input` must contain `requested`
 * (the reference asks its source for exactly that region); params as for
 * itkg_gaussian_generate_region. */
itkg_status itkg_slice_by_slice_generate_region(const itkg_image *input, const itkg_region *requested,
                                               const itkg_gaussian_params *params, itkg_image *output,
                                               void *stream);

/* BSplineDownsampleFilter { source } (filters/spatial.rs:1128-1166): GaussianFilter
 * with sigma 1.0 (params->sigma is not read) over the whole largest region,
 * then every other voxel from the region's index: output voxel i is smoothed
 * voxel index + 2 (i - index).  The reference returns the whole downsampled
 * region (size (n + 1) / 2 per axis, same index) whatever is requested, so
 * `output` must contain it and `input` the largest region.  The output's dtype
 * is the smoothed image's (params->arithmetic as for the Gaussian). */
itkg_status itkg_bspline_downsample_generate_region(const itkg_image *input, const itkg_region *largest,
                                                    const itkg_gaussian_params *params, itkg_image *output,
                                                    void *stream);

/* ---- RecursiveGaussianFilter (recursive_gaussian.rs) -----------------------
 * Young & van Vliet 3rd-order IIR Gaussian: RecursiveGaussianFilter (axis -1,
 * every axis; recursive_gaussian.rs:133-181) and RecursiveGaussianAxisFilter
 * (axis 0..dim-1; 183-239).  The whole largest region is filtered (the
 * reference's input_region_for_output is the largest region), so `input` must
 * cover `largest`; `requested` is written to `output`.
 *   sigma     physical units; sigma / spacing per axis, at least 0.5 (:34)
 *   rounding  f64 either way; ITKG_ROUND_REFERENCE: every product and sum
 *             rounded in the reference's order, bit-exact; ITKG_ROUND_FMA:
 *             fused multiply-adds
 * Scalar input of any dtype (converted exactly); output f32 (`v as f32`) or u8
 * (round half away from zero, clamp to [0, 255], pixel.rs:36). */
typedef struct itkg_recursive_params {
    double sigma;
    int32_t axis;
    int32_t rounding;
    int32_t reserved[2]; /* 0 */
} itkg_recursive_params;

/* (B, a1, a2, a3) of recursive_gaussian.rs:33-49 for sigma in pixels. */
itkg_status itkg_yvv_coeffs(double sigma, double *coeffs_out);

itkg_status itkg_recursive_gaussian_generate_region(const itkg_image *input, const itkg_region *largest,
                                                    const itkg_region *requested,
                                                    const itkg_recursive_params *params,
                                                    itkg_image *output, void *stream);

/* The derivative users of RecursiveGaussianFilter (edges.rs:686-950): the
 * smoothed image RecursiveGaussianFilter::generate_region(requested), in the
 * input's pixel type (f32 or u8), then a central-difference stencil clamped to
 * the requested region (the smoothed image is the stencil's whole source),
 * in f64 with every operation rounded in the reference's order.
 *   kind                                  output
 *   ITKG_REC_GRADIENT_MAGNITUDE  (686-722) pixel type, 1 component
 *   ITKG_REC_LAPLACIAN           (730-766) pixel type, 1 component
 *   ITKG_REC_DERIVATIVE          (772-810) pixel type; `axis`, `order` (1, 2; else 0)
 *   ITKG_REC_GRADIENT            (819-878) f32, dim components (VecPixel<f32, D>)
 *   ITKG_REC_HESSIAN             (892-950) 2-D only; f32, 3 components (h00, h11, h01)
 *   ITKG_REC_DIFFERENCE_OF_GAUSSIANS (955-1009) pixel type: s(sigma) - s(sigma2) in f64
 *   ITKG_REC_ZERO_CROSSING_EDGES (1019-1052) pixel type: the Laplacian stencil
 *                                into the pixel type, then 1 where it changes
 *                                sign to a neighbour along an axis, else 0
 * sigma, rounding: as for itkg_recursive_gaussian_generate_region. */
#define ITKG_REC_GRADIENT_MAGNITUDE 0
#define ITKG_REC_LAPLACIAN 1
#define ITKG_REC_DERIVATIVE 2
#define ITKG_REC_GRADIENT 3
#define ITKG_REC_HESSIAN 4
#define ITKG_REC_DIFFERENCE_OF_GAUSSIANS 5 /* (955-1009) smoothing(sigma) - smoothing(sigma2), pixel type */
#define ITKG_REC_ZERO_CROSSING_EDGES 6     /* (1019-1052) ZeroCrossingBasedEdgeDetectionFilter */
typedef struct itkg_recursive_derivative_params {
    double sigma;
    double sigma2; /* ITKG_REC_DIFFERENCE_OF_GAUSSIANS: the second smoothing */
    int32_t kind;
    int32_t axis;
    int32_t order;
    int32_t rounding;
    int32_t reserved[2]; /* 0 */
} itkg_recursive_derivative_params;

itkg_status itkg_recursive_gaussian_derivative_generate_region(const itkg_image *input, const itkg_region *largest,
                                                               const itkg_region *requested,
                                                               const itkg_recursive_derivative_params *params,
                                                               itkg_image *output, void *stream);

/* ---- derivatives (not in the reference: it has no VJP) ---------------------
 * Vector-Jacobian product of GaussianFilter over a whole image: x is the
 * filter input (requested region = largest region = x->region), ybar = dL/dy
 * on the same region.  The forward y = G x is recomputed, never stored.
 *   xbar      if non-NULL: dL/dx = G^T ybar (the exact adjoint of the clamped
 *             separable convolution, edge voxels receiving the clamped taps);
 *             added to xbar's contents with ITKG_VJP_ACCUMULATE_XBAR.
 *   sigma_bar if non-NULL: dL/dsigma = <ybar, dy/dsigma>, summed in f64, the
 *             radius frozen at ceil(3 sigma / spacing) (the derivative of the
 *             sampled, normalised kernel of gaussian.rs:29-40 at fixed r).  A
 *             host pointer (the call synchronises the stream) unless
 *             ITKG_VJP_SIGMA_BAR_ON_DEVICE; added to with ITKG_VJP_ACCUMULATE_SIGMA.
 * Scalar f32 device images; FMA rounding; sigma must be finite and > 0.
 * params->algorithm selects the kernels (3-D): ITKG_ALGO_AUTO / _TWO_PASS: a
 * z-adjoint kernel and x-y kernels (rx == ry <= 12, rz <= 12, 16-byte aligned
 * rows), else as ITKG_ALGO_FUSED: the fused VJP kernels (radii <= 8, the
 * adjoint <= 6), else the per-axis passes; ITKG_ALGO_PER_AXIS: per-axis only. */
#define ITKG_VJP_ACCUMULATE_XBAR 1
#define ITKG_VJP_ACCUMULATE_SIGMA 2
#define ITKG_VJP_SIGMA_BAR_ON_DEVICE 4
itkg_status itkg_gaussian_vjp(const itkg_image *x, const itkg_image *ybar,
                              const itkg_gaussian_params *params, itkg_image *xbar,
                              double *sigma_bar, int32_t flags, void *stream);

/* Multi-scale squared-error loss and its gradient, the scale stack recomputed
 * level by level instead of stored:
 *   L = sum_l sum_v (G_{sigma_l} x - target)^2
 *   loss      (host, may be NULL): L in f64
 *   xbar      (may be NULL): dL/dx = sum_l G_l^T 2 (G_l x - target), overwritten
 *   sigma_bar (may be NULL): nlevels values dL/dsigma_l (radius frozen per level);
 *             host array unless ITKG_VJP_SIGMA_BAR_ON_DEVICE.
 * Scalar f32 device images of one region; synchronises the stream when it
 * returns host values. */
itkg_status itkg_gaussian_scale_stack_loss_vjp(const itkg_image *x, const itkg_image *target,
                                               const double *sigmas, int32_t nlevels,
                                               itkg_image *xbar, double *loss, double *sigma_bar,
                                               int32_t flags, void *stream);

/* ---- batches (not in the reference: it filters one image per call) ---------
 * A batch collects many forward requests (the arguments of
 * itkg_gaussian_generate_region, device buffers only) and VJP requests (the
 * arguments of itkg_gaussian_vjp, sigma_bar a device pointer or NULL),
 * plans them once and replays them as one CUDA graph:
 *   itkg_batch_plan  picks each item's kernel (an autotuner times the fused
 *                    kernel against per-axis passes once per (dtype, size
 *                    bucket, radius) class unless ITKG_BATCH_NO_AUTOTUNE),
 *                    merges fused items into persistent launches and captures
 *                    everything into a graph; it runs each item at least once
 *                    while tuning, so outputs must be writable at plan time;
 *   itkg_batch_run   launches the graph on `stream` (asynchronous).
 * Buffers must stay valid, and at the same addresses, while the batch exists. */
typedef struct itkg_batch itkg_batch;
#define ITKG_BATCH_NO_AUTOTUNE 1
itkg_status itkg_batch_create(itkg_batch **batch);
itkg_status itkg_batch_destroy(itkg_batch *batch);
itkg_status itkg_batch_add(itkg_batch *batch, const itkg_image *input, const itkg_region *largest,
                           const itkg_region *requested, const itkg_gaussian_params *params,
                           itkg_image *output);
itkg_status itkg_batch_add_vjp(itkg_batch *batch, const itkg_image *x, const itkg_image *ybar,
                               const itkg_gaussian_params *params, itkg_image *xbar,
                               double *sigma_bar_device, int32_t flags);
itkg_status itkg_batch_plan(itkg_batch *batch, int32_t flags, void *stream);
itkg_status itkg_batch_run(itkg_batch *batch, void *stream);
/* One line per planned launch (kernel chosen per item); valid until the next call. */
const char *itkg_batch_describe(itkg_batch *batch);

/* No counterpart in the reference.  The same result as
 * itkg_gaussian_generate_region with algorithm ITKG_ALGO_PER_AXIS, for callers
 * that must not allocate device memory during the call -- for example an
 * application that has handed all device memory to its own pool or caching
 * allocator, or a latency-critical loop that cannot absorb an allocation.
 * This entry point calls no cudaMalloc, cudaFree or other allocating routine:
 * the per-axis intermediates live in one fixed 32 MiB device array inside the
 * library (held on every GPU that loads the library until the process exits).
 *   - input and output must be device buffers (ITKG_DEVICE);
 *   - a request that does not fit the 32 MiB fails with
 *     ITKG_ERROR_INVALID_ARGUMENT.  It holds the intermediates: two for D = 3,
 *     one for D = 2, none for D = 1, each the requested region padded by the
 *     radius on the axes not yet filtered, at 4 bytes per component with f32
 *     arithmetic and 1 byte with u8 pixel arithmetic; u8 pixel arithmetic also
 *     keeps its per-tap table there, (2r + 1) * 256 bytes for the largest
 *     radius r;
 *   - all calls share the array; calls whose GPU work overlaps (e.g. on two
 *     streams) race on it and must be serialised by the caller;
 *   - the first call on each device that uses the array (D >= 2, or u8 pixel
 *     arithmetic) looks up the array's device address, so make that first
 *     call before any stream capture.
 * itkg_scratch_alloc_counter() does not move across these calls. */
itkg_status itkg_gaussian_generate_region_noalloc(const itkg_image *input,
                                                  const itkg_region *largest,
                                                  const itkg_region *requested,
                                                  const itkg_gaussian_params *params,
                                                  itkg_image *output, void *stream);

/* DemonsRegistrationFilter::compute (src/filters/registration_methods.rs:39-100)
 * and, with diffeomorphic != 0, DiffeomorphicDemonsRegistrationFilter::compute
 * (registration_methods.rs:126-148; SyNRegistrationMethod::compute, :211-218,
 * is the latter with the sum of its iteration counts): `iterations` demons
 * force updates of a displacement field (in pixels, f64, as the reference
 * keeps it) from 2-D f32 fixed and moving images, each image's buffered region
 * being its largest region; with diffeomorphic != 0 each displacement
 * component is then smoothed by GaussianFilter { sigma: sigma_diff } in
 * reference rounding.  displacement: 2-D f32, 2 components (VecPixel<f32, 2>),
 * containing the fixed region.  A warped index outside the moving buffer,
 * where the reference panics, returns ITKG_ERROR_INVALID_ARGUMENT.  Any buffer
 * may be host or device memory; the call returns after the result is written. */
itkg_status itkg_demons_registration(const itkg_image *fixed, const itkg_image *moving, int32_t iterations,
                                     double max_step_length, int32_t diffeomorphic, double sigma_diff,
                                     itkg_image *displacement, void *stream);

/* N4BiasFieldCorrectionFilter::generate_region (src/filters/bias_correction.rs:45-83;
 * MRIBiasFieldCorrectionFilter, :113-121, is this call with sigma 20): the
 * largest region of a 2-D f32 image, up to `iterations` times: the f64 log of
 * the corrected image, GaussianFilter { sigma } of its f32 image (reference
 * rounding), corrected = max(exp(log - smoothed), 1e-6), stopping when the
 * mean absolute change falls below convergence_threshold; output = corrected
 * as f32 over the largest region.  *iterations_run (may be NULL) receives the
 * number of iterations run.  ln and exp are the device's f64 functions, whose
 * last bit may differ from the host libm's.  Any buffer may be host or device
 * memory; the call returns after the result is written. */
itkg_status itkg_n4_bias_field_correction(const itkg_image *input, const itkg_region *largest, int32_t iterations,
                                          double sigma, double convergence_threshold, itkg_image *output,
                                          int32_t *iterations_run, void *stream);

/* stream_full(&GaussianFilter{input, sigma}, num_pieces) (source.rs:81-98):
 * output (region == largest) is filled piece by piece along axis D-1.  With a
 * host-resident input and output, only one halo-padded input slab and one
 * output slab are resident on the device at a time (out-of-core streaming). */
itkg_status itkg_stream_full(const itkg_image *input, const itkg_region *largest,
                             const itkg_gaussian_params *params, uint64_t num_pieces,
                             itkg_image *output, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* ITKG_H */
