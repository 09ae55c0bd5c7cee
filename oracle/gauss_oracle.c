/*
 * oracle/gauss_oracle.c -- CPU restatement of itk-rs's separable Gaussian path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: only tests/, the smoke
 * check in __graft_entry__.py and bench.py's CPU-baseline leg load it.  The
 * product (itk-rs_gb300/, include/itkg.h) never links, loads or calls it.
 *
 * It restates, in plain C with IEEE arithmetic (compiled with
 * -ffp-contract=off, no fast-math), the reference algorithm:
 *   - src/filters/gaussian.rs:24-27  kernel_radius  r = ceil(3*sigma/spacing) as usize
 *   - src/filters/gaussian.rs:29-40  build_kernel   f64 exp(-0.5*(x/s)^2), normalised by its f64 sum
 *   - src/filters/gaussian.rs:59-91  generate_region: pass order axis 0..D-1, intermediate
 *                                    regions padded on the axes not yet processed
 *   - src/filters/conv.rs:11-41      convolve_axis: taps in ascending k, clamp to the source
 *                                    buffer's extent, acc = zero; acc = acc + x.scale(w)
 *   - src/pixel.rs:416-421           f32 scale: x * (w as f32), separate rounding (no FMA)
 *   - src/pixel.rs:430-435           u8 scale: round(x as f64 * w).clamp(0,255) as u8, u8 add
 *                                    wraps (release build)
 *   - src/pixel.rs:479-495           VecPixel<T,N>: per-component scale and add
 *   - src/image.rs:23-64             Region::padded_per_axis / clipped_to
 *   - src/region_splitter.rs:17-48   split_region along the slowest axis
 *   - src/source.rs:42-58, 81-98     Image leaf crop, stream_full
 * plus an FP64 oracle (same kernel, same clamp, f64 accumulation, no rounding of
 * intermediates) and a multi-threaded timing port that keeps the reference's
 * structure (serial index-vector build, then a parallel loop over output voxels).
 *
 * Parity pinning: the reference ships no golden vectors and cannot be built in
 * this environment (no Rust toolchain).  This restatement is pinned by re-running
 * the reference's own property tests against it (tests/test_oracle.py):
 * gaussian.rs:107-127, tests/pipeline.rs:19-153, tests/blur_png.rs:17-73,
 * image.rs:180-210, region_splitter.rs:354-396.
 *
 * Layout: axis 0 fastest, dense (image.rs:111-120); a pixel of `comps`
 * components is `comps` consecutive scalars.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_MAXD 3

typedef struct {
    int64_t index[ORC_MAXD];
    int64_t size[ORC_MAXD];
} orc_region;

/* ---- Region helpers (image.rs:23-64) ------------------------------------ */

static int64_t region_len(const orc_region *r, int D) {
    int64_t n = 1;
    for (int d = 0; d < D; d++) n *= r->size[d];
    return n;
}

orc_region orc_padded_per_axis(orc_region r, const uint64_t *radii, int D) {
    for (int d = 0; d < D; d++) {
        r.index[d] -= (int64_t)radii[d];
        r.size[d] += 2 * (int64_t)radii[d];
    }
    return r;
}

orc_region orc_clipped_to(orc_region r, orc_region b, int D) {
    for (int d = 0; d < D; d++) {
        int64_t self_end = r.index[d] + r.size[d];
        int64_t b_end = b.index[d] + b.size[d];
        int64_t s = r.index[d] > b.index[d] ? r.index[d] : b.index[d];
        int64_t e = self_end < b_end ? self_end : b_end;
        r.index[d] = s;
        r.size[d] = (e - s) > 0 ? (e - s) : 0;
    }
    return r;
}

/* ---- Kernel (gaussian.rs:24-40) ----------------------------------------- */

/* Rust `f64 as usize` saturates: NaN -> 0, negative -> 0, too big -> MAX. */
uint64_t orc_kernel_radius(double sigma, double spacing) {
    double sigma_px = sigma / spacing;
    double c = ceil(3.0 * sigma_px);
    if (!(c > 0.0)) return 0;            /* NaN or <= 0 */
    if (c >= 18446744073709551615.0) return UINT64_MAX;
    return (uint64_t)c;
}

void orc_build_kernel(double sigma_px, uint64_t radius, double *out) {
    uint64_t len = 2 * radius + 1;
    double sum = 0.0;
    for (uint64_t i = 0; i < len; i++) {
        double x = (double)i - (double)radius;
        double t = x / sigma_px;
        out[i] = exp(-0.5 * (t * t));     /* powi(2) lowers to t*t */
    }
    for (uint64_t i = 0; i < len; i++) sum += out[i];
    for (uint64_t i = 0; i < len; i++) out[i] /= sum;
}

/* ---- flat index (image.rs:111-120) -------------------------------------- */

static inline int64_t flat_index(const orc_region *reg, const int64_t *idx, int D) {
    int64_t off = 0, stride = 1;
    for (int d = 0; d < D; d++) {
        off += (idx[d] - reg->index[d]) * stride;
        stride *= reg->size[d];
    }
    return off;
}

/* Advance idx over `reg` in axis-0-fastest order; returns 0 when wrapped. */
static inline int next_index(const orc_region *reg, int64_t *idx, int D) {
    for (int d = 0; d < D; d++) {
        idx[d]++;
        if (idx[d] < reg->index[d] + reg->size[d]) return 1;
        idx[d] = reg->index[d];
    }
    return 0;
}

/* ---- convolve_axis (conv.rs:11-41), three scalar semantics -------------- */

typedef enum { PIX_F32 = 0, PIX_U8 = 1, PIX_F64 = 2 } pix_kind;

typedef struct {
    const void *src;
    orc_region src_reg;
    int D, comps, axis;
    const double *kernel;
    uint64_t K;
    orc_region req;
    void *out;
    pix_kind kind;
    const int64_t *indices; /* optional precomputed index vector (timing port) */
    int64_t begin, end;     /* voxel range of `req` in iteration order */
} conv_job;

static inline uint8_t u8_scale(uint8_t x, double w) {
    /* (x as f64 * w).round().clamp(0.0, 255.0) as u8 -- pixel.rs:432 */
    double v = round((double)x * w);
    if (v < 0.0) v = 0.0;
    if (v > 255.0) v = 255.0;
    return (uint8_t)v;
}

static void conv_range(const conv_job *j) {
    const int D = j->D, C = j->comps, axis = j->axis;
    const int64_t r = (int64_t)(j->K / 2);
    const int64_t lo = j->src_reg.index[axis];
    const int64_t hi = j->src_reg.index[axis] + j->src_reg.size[axis] - 1;
    int64_t idx[ORC_MAXD];
    /* position of voxel `begin` in iteration order */
    {
        int64_t rem = j->begin;
        for (int d = 0; d < D; d++) {
            idx[d] = j->req.index[d] + rem % j->req.size[d];
            rem /= j->req.size[d];
        }
    }
    for (int64_t v = j->begin; v < j->end; v++) {
        int64_t o[ORC_MAXD];
        if (j->indices) {
            for (int d = 0; d < D; d++) o[d] = j->indices[v * D + d];
        } else {
            for (int d = 0; d < D; d++) o[d] = idx[d];
        }
        for (int c = 0; c < C; c++) {
            float accf = 0.0f;
            uint8_t accu = 0;
            double accd = 0.0;
            for (uint64_t k = 0; k < j->K; k++) {
                int64_t s[ORC_MAXD];
                for (int d = 0; d < D; d++) s[d] = o[d];
                int64_t t = o[axis] + (int64_t)k - r;
                if (t < lo) t = lo;          /* .max(lo) */
                if (t > hi) t = hi;          /* .min(hi) */
                s[axis] = t;
                int64_t fi = flat_index(&j->src_reg, s, D) * C + c;
                double w = j->kernel[k];
                if (j->kind == PIX_F32) {
                    float x = ((const float *)j->src)[fi];
                    float p = x * (float)w;            /* separate rounding */
                    accf = accf + p;
                } else if (j->kind == PIX_U8) {
                    uint8_t x = ((const uint8_t *)j->src)[fi];
                    accu = (uint8_t)(accu + u8_scale(x, w)); /* wrapping add */
                } else {
                    double x = ((const double *)j->src)[fi];
                    accd = accd + x * w;
                }
            }
            int64_t oi = v * C + c;
            if (j->kind == PIX_F32) ((float *)j->out)[oi] = accf;
            else if (j->kind == PIX_U8) ((uint8_t *)j->out)[oi] = accu;
            else ((double *)j->out)[oi] = accd;
        }
        if (!j->indices) next_index(&j->req, idx, D);
    }
}

static size_t pix_bytes(pix_kind k, int comps) {
    return (size_t)comps * (k == PIX_F32 ? 4 : k == PIX_U8 ? 1 : 8);
}

typedef struct { conv_job job; } thread_arg;

static void *conv_thread(void *p) {
    conv_range(&((thread_arg *)p)->job);
    return NULL;
}

/* One convolve_axis call. nthreads<=1: serial.  nthreads>1: the reference's
 * structure -- serial build of the index vector (conv.rs:21-22), then the
 * output voxels split over threads (rayon par_iter, conv.rs:24-25). */
static int convolve_axis(const void *src, orc_region src_reg, int D, int comps, int axis,
                         const double *kernel, uint64_t K, orc_region req, void *out,
                         pix_kind kind, int nthreads) {
    int64_t n = region_len(&req, D);
    if (n == 0) return 0;
    conv_job base = {src, src_reg, D, comps, axis, kernel, K, req, out, kind, NULL, 0, n};
    if (nthreads <= 1) {
        conv_range(&base);
        return 0;
    }
    int64_t *indices = (int64_t *)malloc((size_t)n * D * sizeof(int64_t));
    if (!indices) return -1;
    {
        int64_t idx[ORC_MAXD];
        for (int d = 0; d < D; d++) idx[d] = req.index[d];
        for (int64_t v = 0; v < n; v++) {
            for (int d = 0; d < D; d++) indices[v * D + d] = idx[d];
            next_index(&req, idx, D);
        }
    }
    base.indices = indices;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    thread_arg *args = (thread_arg *)malloc(sizeof(thread_arg) * nthreads);
    for (int t = 0; t < nthreads; t++) {
        args[t].job = base;
        args[t].job.begin = n * t / nthreads;
        args[t].job.end = n * (t + 1) / nthreads;
        pthread_create(&th[t], NULL, conv_thread, &args[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th);
    free(args);
    free(indices);
    return 0;
}

/* Exported single-axis entry (used by tests of the per-axis semantics). */
int orc_convolve_axis(const void *src, const orc_region *src_reg, int D, int comps, int axis,
                      const double *kernel, uint64_t K, const orc_region *req, void *out,
                      int kind) {
    return convolve_axis(src, *src_reg, D, comps, axis, kernel, K, *req, out,
                         (pix_kind)kind, 1);
}

/* ---- Image leaf crop (source.rs:42-58) ---------------------------------- */

static void crop(const void *img, orc_region img_reg, orc_region want, int D, size_t pb,
                 void *out) {
    int64_t n = region_len(&want, D);
    if (n == 0) return;
    int64_t idx[ORC_MAXD];
    for (int d = 0; d < D; d++) idx[d] = want.index[d];
    for (int64_t v = 0; v < n; v++) {
        memcpy((char *)out + v * pb, (const char *)img + flat_index(&img_reg, idx, D) * pb, pb);
        next_index(&want, idx, D);
    }
}

/* ---- GaussianFilter::generate_region (gaussian.rs:59-91) ---------------- *
 * `img` is an Image leaf whose region is also largest_region (the bounds).
 * `out` receives `requested` (dense, requested.linear_len() pixels).
 * Returns 0, or -1 for allocation failure / absurd radius (the reference
 * would panic on capacity overflow). */
static int gaussian_region(const void *img, const orc_region *img_reg, const double *spacing,
                           int D, int comps, double sigma, const orc_region *requested,
                           void *out, pix_kind kind, int nthreads) {
    const orc_region bounds = *img_reg;
    uint64_t radii[ORC_MAXD] = {0, 0, 0};
    for (int d = 0; d < D; d++) {
        radii[d] = orc_kernel_radius(sigma, spacing[d]);
        if (radii[d] > (1u << 20)) return -1;
    }
    size_t pb = pix_bytes(kind, comps);
    orc_region in_reg = orc_clipped_to(orc_padded_per_axis(*requested, radii, D), bounds, D);
    void *cur = malloc((size_t)(region_len(&in_reg, D) * pb + 1));
    if (!cur) return -1;
    crop(img, *img_reg, in_reg, D, pb, cur);
    orc_region cur_reg = in_reg;
    for (int axis = 0; axis < D; axis++) {
        double sigma_px = sigma / spacing[axis];
        uint64_t K = 2 * radii[axis] + 1;
        double *kernel = (double *)malloc(K * sizeof(double));
        orc_build_kernel(sigma_px, radii[axis], kernel);
        orc_region out_reg;
        if (axis + 1 < D) {
            uint64_t rem[ORC_MAXD] = {0, 0, 0};
            for (int d = axis + 1; d < D; d++) rem[d] = radii[d];
            out_reg = orc_clipped_to(orc_padded_per_axis(*requested, rem, D), bounds, D);
        } else {
            out_reg = *requested;
        }
        void *nxt = (axis + 1 < D) ? malloc((size_t)(region_len(&out_reg, D) * pb + 1)) : out;
        if (!nxt) { free(kernel); free(cur); return -1; }
        convolve_axis(cur, cur_reg, D, comps, axis, kernel, K, out_reg, nxt, kind, nthreads);
        free(kernel);
        free(cur);
        cur = (axis + 1 < D) ? nxt : NULL;
        cur_reg = out_reg;
    }
    if (D == 0) free(cur);
    return 0;
}

int orc_gaussian_f32(const float *img, const orc_region *img_reg, const double *spacing, int D,
                     int comps, double sigma, const orc_region *requested, float *out) {
    return gaussian_region(img, img_reg, spacing, D, comps, sigma, requested, out, PIX_F32, 1);
}

int orc_gaussian_u8(const uint8_t *img, const orc_region *img_reg, const double *spacing,
                    int D, int comps, double sigma, const orc_region *requested,
                    uint8_t *out) {
    return gaussian_region(img, img_reg, spacing, D, comps, sigma, requested, out, PIX_U8, 1);
}

/* FP64 oracle: same kernel, same clamp boundary, f64 arithmetic end to end. */
int orc_gaussian_f64(const double *img, const orc_region *img_reg, const double *spacing,
                     int D, int comps, double sigma, const orc_region *requested,
                     double *out) {
    return gaussian_region(img, img_reg, spacing, D, comps, sigma, requested, out, PIX_F64, 1);
}

/* Timing port of the reference's rayon path (f32): serial index build then
 * `nthreads` workers per pass. Same arithmetic as orc_gaussian_f32. */
int orc_gaussian_f32_mt(const float *img, const orc_region *img_reg, const double *spacing,
                        int D, int comps, double sigma, const orc_region *requested,
                        float *out, int nthreads) {
    return gaussian_region(img, img_reg, spacing, D, comps, sigma, requested, out, PIX_F32,
                           nthreads < 1 ? 1 : nthreads);
}

/* ---- the convolve_axis family with explicit kernels -------------------- *
 * MeanFilter and BoxMeanFilterN (mean.rs:59-83, 116-136): one pass per axis
 * with that axis's box kernel, each weight 1/(2r+1) (mean.rs:15-18), and the
 * Gaussian's intermediate regions.  BinomialBlurFilter (binomial_blur.rs:
 * 57-89): `reps` rounds of one pass per axis with [1/4, 1/2, 1/4]; the input is
 * requested padded by reps per axis, pass (rep, axis) writes requested padded
 * by reps - rep - 1 on every axis and one more on the axes after `axis`
 * (clipped to the bounds), and the last pass writes requested.  Written for a
 * kernel of radius r_d on axis d, the pads are those counts times r_d; with
 * reps = 1 both schedules are the Gaussian's.  reps = 0 returns the crop of
 * requested (the reference runs no pass).  kernels[d]: 2 radii[d] + 1 f64
 * weights of axis d. */
static int separable_region(const void *img, const orc_region *img_reg, int D, int comps,
                            const uint64_t *radii, const double *const *kernels, uint64_t reps,
                            const orc_region *requested, void *out, pix_kind kind, int nthreads) {
    const orc_region bounds = *img_reg;
    size_t pb = pix_bytes(kind, comps);
    for (int d = 0; d < D; d++)
        if (radii[d] > (1u << 20)) return -1;
    uint64_t total[ORC_MAXD] = {0, 0, 0};
    for (int d = 0; d < D; d++) total[d] = reps * radii[d];
    orc_region in_reg = orc_clipped_to(orc_padded_per_axis(*requested, total, D), bounds, D);
    if (reps == 0) {
        crop(img, *img_reg, *requested, D, pb, out);
        return 0;
    }
    void *cur = malloc((size_t)(region_len(&in_reg, D) * pb + 1));
    if (!cur) return -1;
    crop(img, *img_reg, in_reg, D, pb, cur);
    orc_region cur_reg = in_reg;
    for (uint64_t rep = 0; rep < reps; rep++) {
        const uint64_t remaining = reps - rep - 1;
        for (int axis = 0; axis < D; axis++) {
            const int last = rep + 1 == reps && axis + 1 == D;
            orc_region out_reg;
            if (last) {
                out_reg = *requested;
            } else {
                uint64_t pad[ORC_MAXD] = {0, 0, 0};
                for (int d = 0; d < D; d++) pad[d] = (d > axis ? remaining + 1 : remaining) * radii[d];
                out_reg = orc_clipped_to(orc_padded_per_axis(*requested, pad, D), bounds, D);
            }
            void *nxt = last ? out : malloc((size_t)(region_len(&out_reg, D) * pb + 1));
            if (!nxt) { free(cur); return -1; }
            convolve_axis(cur, cur_reg, D, comps, axis, kernels[axis], 2 * radii[axis] + 1, out_reg, nxt,
                          kind, nthreads);
            free(cur);
            cur = last ? NULL : nxt;
            cur_reg = out_reg;
        }
    }
    return 0;
}

int orc_separable_f32(const float *img, const orc_region *img_reg, int D, int comps,
                      const uint64_t *radii, const double *const *kernels, uint64_t reps,
                      const orc_region *requested, float *out) {
    return separable_region(img, img_reg, D, comps, radii, kernels, reps, requested, out, PIX_F32, 1);
}

int orc_separable_u8(const uint8_t *img, const orc_region *img_reg, int D, int comps,
                     const uint64_t *radii, const double *const *kernels, uint64_t reps,
                     const orc_region *requested, uint8_t *out) {
    return separable_region(img, img_reg, D, comps, radii, kernels, reps, requested, out, PIX_U8, 1);
}

int orc_separable_f64(const double *img, const orc_region *img_reg, int D, int comps,
                      const uint64_t *radii, const double *const *kernels, uint64_t reps,
                      const orc_region *requested, double *out) {
    return separable_region(img, img_reg, D, comps, radii, kernels, reps, requested, out, PIX_F64, 1);
}

/* Timing port for the family (f32, `nthreads` workers per pass). */
int orc_separable_f32_mt(const float *img, const orc_region *img_reg, int D, int comps,
                         const uint64_t *radii, const double *const *kernels, uint64_t reps,
                         const orc_region *requested, float *out, int nthreads) {
    return separable_region(img, img_reg, D, comps, radii, kernels, reps, requested, out, PIX_F32,
                            nthreads < 1 ? 1 : nthreads);
}

/* ---- RecursiveGaussianFilter (recursive_gaussian.rs) --------------------- *
 * Young & van Vliet 3rd-order coefficients (recursive_gaussian.rs:33-49),
 * every product and sum rounded separately in the order written there. */
void orc_yvv_coeffs(double sigma, double *out4) {
    if (!(sigma > 0.5)) sigma = 0.5; /* sigma.max(0.5); f64::max takes 0.5 over NaN */
    double q = sigma >= 2.5 ? 0.98711 * sigma - 0.96330 : 3.97156 - 4.14554 * sqrt(1.0 - 0.26891 * sigma);
    double q2 = q * q;
    double q3 = q2 * q;
    double b0 = 1.57825 + 2.44413 * q + 1.4281 * q2 + 0.422205 * q3;
    double b1 = 2.44413 * q + 2.85619 * q2 + 1.26661 * q3;
    double b2 = -(1.4281 * q2 + 1.26661 * q3);
    double b3 = 0.422205 * q3;
    double big_b = 1.0 - (b1 + b2 + b3) / b0;
    out4[0] = big_b;
    out4[1] = b1 / b0;
    out4[2] = b2 / b0;
    out4[3] = b3 / b0;
}

/* filter_axis (recursive_gaussian.rs:93-130) on a dense f64 image of `size`
 * (axis 0 fastest): every line along `axis` gets the causal pass
 * (recursive_gaussian.rs:56-71), then the anticausal pass (73-88), in place;
 * lines of length <= 1 are left alone. */
static void iir_axis(double *data, const int64_t *size, int D, int axis, double sigma_px) {
    const int64_t n = size[axis];
    if (n <= 1) return;
    double c[4];
    orc_yvv_coeffs(sigma_px, c);
    const double B = c[0], a1 = c[1], a2 = c[2], a3 = c[3];
    int64_t stride[ORC_MAXD] = {1, 1, 1};
    for (int d = 1; d < D; d++) stride[d] = stride[d - 1] * size[d - 1];
    int64_t total = 1;
    for (int d = 0; d < D; d++) total *= size[d];
    const int64_t s = stride[axis];
    for (int64_t lin = 0; lin < total; lin++) {
        /* line starts: the voxels whose coordinate on `axis` is 0 */
        if ((lin / s) % n != 0) continue;
        double *p = data + lin;
        double ym1 = p[0], ym2 = p[0], ym3 = p[0];
        for (int64_t i = 0; i < n; i++) {
            double v = B * p[i * s] + a1 * ym1 + a2 * ym2 + a3 * ym3;
            ym3 = ym2; ym2 = ym1; ym1 = v;
            p[i * s] = v;
        }
        ym1 = ym2 = ym3 = p[(n - 1) * s];
        for (int64_t i = n - 1; i >= 0; i--) {
            double v = B * p[i * s] + a1 * ym1 + a2 * ym2 + a3 * ym3;
            ym3 = ym2; ym2 = ym1; ym1 = v;
            p[i * s] = v;
        }
    }
}

/* RecursiveGaussianFilter::generate_region (recursive_gaussian.rs:154-180) and
 * RecursiveGaussianAxisFilter (218-238, axis >= 0): `img` is the whole largest
 * region already converted to f64 (P::to_f64), filtered in place; sigma is in
 * physical units (sigma / spacing per axis).  The caller crops and converts
 * (P::from_f64). */
void orc_recursive_gaussian_f64(double *img, const int64_t *size, const double *spacing, int D,
                                double sigma, int axis) {
    for (int a = 0; a < D; a++)
        if (axis < 0 || axis == a) iir_axis(img, size, D, a, sigma / spacing[a]);
}

/* box_kernel (mean.rs:15-18) */
void orc_box_kernel(uint64_t radius, double *out) {
    const uint64_t len = 2 * radius + 1;
    for (uint64_t k = 0; k < len; k++) out[k] = 1.0 / (double)len;
}

/* ---- split_region (region_splitter.rs:17-48) ----------------------------- *
 * Writes up to num_pieces regions into `pieces`; returns the count. */
int64_t orc_split_region(const orc_region *region, int D, uint64_t num_pieces,
                         orc_region *pieces) {
    if (num_pieces < 1) num_pieces = 1;
    if (D == 0 || region_len(region, D) == 0) return 0;
    int slow = D - 1;
    uint64_t total = (uint64_t)region->size[slow];
    uint64_t actual = num_pieces < total ? num_pieces : total;
    if (actual < 1) actual = 1;
    uint64_t base = total / actual, rem = total % actual;
    int64_t start = region->index[slow];
    for (uint64_t i = 0; i < actual; i++) {
        uint64_t this_size = base + (i < rem ? 1 : 0);
        orc_region p = *region;
        p.index[slow] = start;
        p.size[slow] = (int64_t)this_size;
        pieces[i] = p;
        start += (int64_t)this_size;
    }
    return (int64_t)actual;
}

/* ---- stream_full (source.rs:81-98) for a Gaussian over an Image leaf ---- */
int orc_stream_full_f32(const float *img, const orc_region *img_reg, const double *spacing,
                        int D, int comps, double sigma, uint64_t num_pieces, float *out) {
    orc_region full = *img_reg;
    uint64_t np = num_pieces < 1 ? 1 : num_pieces;
    orc_region *pieces = (orc_region *)malloc(sizeof(orc_region) * np);
    int64_t cnt = orc_split_region(&full, D, np, pieces);
    size_t pb = pix_bytes(PIX_F32, comps);
    for (int64_t i = 0; i < cnt; i++) {
        int64_t n = region_len(&pieces[i], D);
        float *piece = (float *)malloc((size_t)n * pb + 1);
        int rc = orc_gaussian_f32(img, img_reg, spacing, D, comps, sigma, &pieces[i], piece);
        if (rc) { free(piece); free(pieces); return rc; }
        /* output.copy_from(&piece) -- image.rs:133-140 */
        int64_t idx[ORC_MAXD];
        for (int d = 0; d < D; d++) idx[d] = pieces[i].index[d];
        for (int64_t v = 0; v < n; v++) {
            memcpy((char *)out + flat_index(&full, idx, D) * pb, (char *)piece + v * pb, pb);
            next_index(&pieces[i], idx, D);
        }
        free(piece);
    }
    free(pieces);
    return 0;
}

/* ---- UnaryFilter casts around the Gaussian (tests/blur_png.rs:38-40) ---- */

/* |p: f32| p.round().clamp(0.0, 255.0) as u8 : Rust round is half away from
 * zero; NaN survives clamp and `as u8` maps it to 0. */
void orc_cast_f32_to_u8(const float *in, uint8_t *out, int64_t n) {
    for (int64_t i = 0; i < n; i++) {
        float v = roundf(in[i]);
        if (v != v) { out[i] = 0; continue; }
        if (v < 0.0f) v = 0.0f;
        if (v > 255.0f) v = 255.0f;
        out[i] = (uint8_t)v;
    }
}

/* ---- DemonsRegistrationFilter::compute (registration_methods.rs:39-100) ---- *
 * fixed: dense w x h at index freg (index[0..1], size[0..1]); moving: dense mw x mh
 * at mreg.  disp_x / disp_y: w * h f64 each, zeroed by the caller.  Each f64
 * operation is one C operation (no contraction).  Returns 0, or 1 where the
 * reference panics: a warped index whose flat offset (Image::flat_index,
 * image.rs:111-120, wrapping usize arithmetic) is outside the moving data. */
static int64_t sat_i64(double v) {  /* Rust's `f64 as i64` */
    if (v != v) return 0;
    if (v >= 9.2233720368547758e18) return INT64_MAX;
    if (v <= -9.2233720368547758e18) return INT64_MIN;
    return (int64_t)v;
}

int orc_demons_f64(const float *fixed, const orc_region *freg, const float *moving, const orc_region *mreg,
                   int iterations, double max_step, double *disp_x, double *disp_y) {
    const int64_t w = freg->size[0], h = freg->size[1], ox = freg->index[0], oy = freg->index[1];
    const uint64_t mw = (uint64_t)mreg->size[0], mlen = (uint64_t)(mreg->size[0] * mreg->size[1]);
    double *nx = (double *)malloc((size_t)(w * h) * sizeof(double) + 8);
    double *ny = (double *)malloc((size_t)(w * h) * sizeof(double) + 8);
    if (!nx || !ny) { free(nx); free(ny); return -1; }
    int err = 0;
#define FCLAMP(xx, yy) (((yy) < 0 ? 0 : ((yy) > h - 1 ? h - 1 : (yy))) * w + ((xx) < 0 ? 0 : ((xx) > w - 1 ? w - 1 : (xx))))
    for (int it = 0; it < iterations && !err; it++) {
        memcpy(nx, disp_x, (size_t)(w * h) * sizeof(double));  /* new = old.clone() (:55-56) */
        memcpy(ny, disp_y, (size_t)(w * h) * sizeof(double));
        for (int64_t y = 0; y < h; y++) {
            for (int64_t x = 0; x < w; x++) {
                const int64_t i = y * w + x;
                const double wx = (double)x + disp_x[i];
                const double wy = (double)y + disp_y[i];
                const uint64_t xi = (uint64_t)ox + (uint64_t)sat_i64(round(wx));
                const uint64_t yi = (uint64_t)oy + (uint64_t)sat_i64(round(wy));
                const uint64_t flat = (xi - (uint64_t)mreg->index[0]) + (yi - (uint64_t)mreg->index[1]) * mw;
                if (flat >= mlen) { err = 1; break; }
                const double m_val = (double)moving[flat];
                const double f_val = (double)fixed[i];
                const double gx = ((double)fixed[FCLAMP(x + 1, y)] - (double)fixed[FCLAMP(x - 1, y)]) * 0.5;
                const double gy = ((double)fixed[FCLAMP(x, y + 1)] - (double)fixed[FCLAMP(x, y - 1)]) * 0.5;
                const double diff = f_val - m_val;
                const double denom = gx * gx + gy * gy + diff * diff + 1e-6;
                const double step = diff / denom;
                const double dx = step * gx;
                const double dy = step * gy;
                const double norm = sqrt(dx * dx + dy * dy);
                const double scale = norm > max_step ? max_step / norm : 1.0;
                nx[i] = disp_x[i] + dx * scale;
                ny[i] = disp_y[i] + dy * scale;
            }
            if (err) break;
        }
        if (!err) {
            memcpy(disp_x, nx, (size_t)(w * h) * sizeof(double));
            memcpy(disp_y, ny, (size_t)(w * h) * sizeof(double));
        }
    }
#undef FCLAMP
    free(nx);
    free(ny);
    return err;
}

/* ---- N4BiasFieldCorrectionFilter::generate_region (bias_correction.rs:45-83) -- *
 * 2-D f32 image of region `reg` (its largest region); out: dense f32 of reg.
 * ln and exp are the C library's (the functions Rust's f64::ln / f64::exp
 * call on this host).  Returns the number of iterations run, or -1. */
int orc_n4_f32(const float *in, const orc_region *reg, const double *spacing, int iterations, double sigma,
               double threshold, float *out) {
    const int64_t n = reg->size[0] * reg->size[1];
    double *corr = (double *)malloc((size_t)n * sizeof(double) + 8);
    double *ld = (double *)malloc((size_t)n * sizeof(double) + 8);
    float *lf = (float *)malloc((size_t)n * sizeof(float) + 8);
    float *sm = (float *)malloc((size_t)n * sizeof(float) + 8);
    if (!corr || !ld || !lf || !sm) { free(corr); free(ld); free(lf); free(sm); return -1; }
    for (int64_t i = 0; i < n; i++) corr[i] = fmax((double)in[i], 1e-6);
    int run = 0;
    for (int it = 0; it < iterations; it++) {
        for (int64_t i = 0; i < n; i++) {
            ld[i] = log(corr[i]);
            lf[i] = (float)ld[i];
        }
        if (gaussian_region(lf, reg, spacing, 2, 1, sigma, reg, sm, PIX_F32, 1) != 0) { run = -1; break; }
        double sum = 0.0;
        for (int64_t i = 0; i < n; i++) {
            const double prev = corr[i];
            corr[i] = fmax(exp(ld[i] - (double)sm[i]), 1e-6);
            sum += fabs(corr[i] - prev);
        }
        run++;
        if (sum / (double)n < threshold) break;
    }
    if (run >= 0)
        for (int64_t i = 0; i < n; i++) out[i] = (float)corr[i];
    free(corr);
    free(ld);
    free(lf);
    free(sm);
    return run;
}
