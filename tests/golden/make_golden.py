"""Generate tests/golden/golden.npz -- small known-answer vectors for the
Gaussian path, from a literal pure-Python transcription of the reference.

The reference (a Rust crate) cannot be built here and ships no golden vectors,
so these vectors come from a second, independent restatement written line for
line after the reference code, using numpy float32 *scalars* so every product
and sum rounds to f32 separately, exactly as Rust evaluates `acc + x * (w as f32)`:

  kernel_radius     src/filters/gaussian.rs:24-27
  build_kernel      src/filters/gaussian.rs:29-40   (math.exp, f64)
  generate_region   src/filters/gaussian.rs:59-91
  convolve_axis     src/filters/conv.rs:11-41
  u8 scale          src/pixel.rs:430-435
  padded/clipped    src/image.rs:28-64
  split_region      src/region_splitter.rs:17-48
  stream_full       src/source.rs:81-98
and, for the rows beyond the Gaussian (case prefixes):
  sep_   MeanFilter / BoxMeanFilterN / BinomialBlurFilter   mean.rs, binomial_blur.rs
  rec_   RecursiveGaussianFilter (f64 before conversion)     recursive_gaussian.rs:33-239
  recd_  its derivative users (stencils on the smoothing)    filters/edges.rs:686-950
  recz_  ZeroCrossingBasedEdgeDetectionFilter               filters/edges.rs:1019-1052, 480-514
  ush_   UnsharpMaskFilter                                  filters/edges.rs:374-452
  cal_   SliceBySliceFilter, BSplineDownsampleFilter,
         DisplacementFieldToBSplineFilter                   filters/spatial.rs:1128-1166, 1284-1340, 1484-1525
  dem_   DemonsRegistrationFilter, DiffeomorphicDemons...   filters/registration_methods.rs:39-100, 126-148
  n4_    N4BiasFieldCorrectionFilter                        filters/bias_correction.rs:45-83

The oracle (oracle/gauss_oracle.c, oracle/oracle.py) is checked bit-exactly
against these vectors by tests/test_oracle*.py, and the GPU path by the
tests/test_gpu_*.py golden tests.
Run: python tests/golden/make_golden.py   (about a minute; pure Python loops)
"""
from __future__ import annotations

import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


# ---- Region (image.rs) ------------------------------------------------------
def padded_per_axis(index, size, radii):
    return ([i - r for i, r in zip(index, radii)], [s + 2 * r for s, r in zip(size, radii)])


def clipped_to(index, size, bidx, bsize):
    ni, ns = [], []
    for i, s, bi, bs in zip(index, size, bidx, bsize):
        st = max(i, bi)
        en = min(i + s, bi + bs)
        ni.append(st)
        ns.append(max(en - st, 0))
    return ni, ns


def iter_region(index, size):
    """Axis 0 fastest (image.rs:144-174)."""
    D = len(size)
    n = 1
    for s in size:
        n *= s
    if n == 0:
        return
    idx = list(index)
    while True:
        yield tuple(idx)
        carry = True
        for d in range(D):
            if carry:
                idx[d] += 1
                if idx[d] < index[d] + size[d]:
                    carry = False
                else:
                    idx[d] = index[d]
        if carry:
            break


def flat_index(index, size, idx):
    off, stride = 0, 1
    for d in range(len(size)):
        off += (idx[d] - index[d]) * stride
        stride *= size[d]
    return off


# ---- GaussianFilter (gaussian.rs) ------------------------------------------
def kernel_radius(sigma, spacing):
    c = math.ceil(3.0 * (sigma / spacing))
    return max(int(c), 0)


def build_kernel(sigma_px, radius):
    k = []
    for i in range(2 * radius + 1):
        x = float(i) - float(radius)
        t = x / sigma_px
        k.append(math.exp(-0.5 * (t * t)))
    s = 0.0
    for v in k:
        s += v
    return [v / s for v in k]


def scale_f32(x, w):
    return np.float32(x) * np.float32(w)  # x * (w as f32), rounded to f32


def scale_u8(x, w):
    v = float(x) * w
    a = abs(v)
    f = math.floor(a)
    r = (f + 1.0 if a - f >= 0.5 else f) * (1.0 if v >= 0 else -1.0)  # half away from zero
    return int(min(max(r, 0.0), 255.0))


def convolve_axis(src, axis, kernel, req_index, req_size, kind):
    """src = (index, size, data list of pixels); pixel = tuple of components."""
    s_index, s_size, s_data = src
    radius = len(kernel) // 2
    out = []
    for o in iter_region(req_index, req_size):
        comps = len(s_data[0])
        acc = [np.float32(0.0)] * comps if kind == "f32" else [0] * comps
        for k_i, w in enumerate(kernel):
            s = list(o)
            s[axis] = min(max(o[axis] + k_i - radius, s_index[axis]),
                          s_index[axis] + s_size[axis] - 1)
            px = s_data[flat_index(s_index, s_size, s)]
            for c in range(comps):
                if kind == "f32":
                    acc[c] = np.float32(acc[c] + scale_f32(px[c], w))
                else:
                    acc[c] = (acc[c] + scale_u8(px[c], w)) & 0xFF
        out.append(tuple(acc))
    return (list(req_index), list(req_size), out)


def generate_region(img, spacing, sigma, req_index, req_size, kind="f32"):
    b_index, b_size, data = img
    D = len(b_size)
    radii = [kernel_radius(sigma, spacing[d]) for d in range(D)]
    in_i, in_s = clipped_to(*padded_per_axis(req_index, req_size, radii), b_index, b_size)
    # Image leaf crop (source.rs:42-58)
    cur = (in_i, in_s, [data[flat_index(b_index, b_size, p)] for p in iter_region(in_i, in_s)])
    for axis in range(D):
        kernel = build_kernel(sigma / spacing[axis], radii[axis])
        if axis + 1 < D:
            rem = [radii[d] if d > axis else 0 for d in range(D)]
            oi, os_ = clipped_to(*padded_per_axis(req_index, req_size, rem), b_index, b_size)
        else:
            oi, os_ = list(req_index), list(req_size)
        cur = convolve_axis(cur, axis, kernel, oi, os_, kind)
    return cur


def box_kernel(radius):
    """mean.rs:15-18"""
    n = 2 * radius + 1
    return [1.0 / n] * n


BINOMIAL = [0.25, 0.5, 0.25]  # binomial_blur.rs:35


def separable_region(img, kernels, reps, req_index, req_size, kind="f32"):
    """MeanFilter / BoxMeanFilterN::generate_region (mean.rs:59-83, 116-136) when reps = 1,
    BinomialBlurFilter::generate_region (binomial_blur.rs:57-89) with kernels = [BINOMIAL] * D."""
    b_index, b_size, data = img
    D = len(b_size)
    radii = [len(k) // 2 for k in kernels]
    total = [reps * r for r in radii]
    in_i, in_s = clipped_to(*padded_per_axis(req_index, req_size, total), b_index, b_size)
    cur = (in_i, in_s, [data[flat_index(b_index, b_size, p)] for p in iter_region(in_i, in_s)])
    if reps == 0:
        return (list(req_index), list(req_size),
                [cur[2][flat_index(in_i, in_s, p)] for p in iter_region(req_index, req_size)])
    for rep in range(reps):
        remaining = reps - rep - 1
        for axis in range(D):
            if rep + 1 == reps and axis + 1 == D:
                oi, os_ = list(req_index), list(req_size)
            else:
                pad = [(remaining + 1 if d > axis else remaining) * radii[d] for d in range(D)]
                oi, os_ = clipped_to(*padded_per_axis(req_index, req_size, pad), b_index, b_size)
            cur = convolve_axis(cur, axis, kernels[axis], oi, os_, kind)
    return cur


def yvv_coeffs(sigma):
    """recursive_gaussian.rs:33-49"""
    sigma = 0.5 if not (sigma > 0.5) else sigma
    if sigma >= 2.5:
        q = 0.98711 * sigma - 0.96330
    else:
        q = 3.97156 - 4.14554 * math.sqrt(1.0 - 0.26891 * sigma)
    q2 = q * q
    q3 = q2 * q
    b0 = 1.57825 + 2.44413 * q + 1.4281 * q2 + 0.422205 * q3
    b1 = 2.44413 * q + 2.85619 * q2 + 1.26661 * q3
    b2 = -(1.4281 * q2 + 1.26661 * q3)
    b3 = 0.422205 * q3
    big_b = 1.0 - (b1 + b2 + b3) / b0
    return big_b, b1 / b0, b2 / b0, b3 / b0


def recursive_region(img, spacing, sigma, axis_only=None):
    """RecursiveGaussianFilter (recursive_gaussian.rs:154-180) / RecursiveGaussianAxisFilter
    (218-238) over the whole image: f64 pixels, per axis causal then anticausal line passes
    (56-88, 93-130).  Returns the f64 image (index, size, flat list)."""
    b_index, b_size, data = img
    D = len(b_size)
    vals = [float(p[0]) for p in data]
    for axis in range(D):
        if axis_only is not None and axis != axis_only:
            continue
        n = b_size[axis]
        if n <= 1:
            continue
        big_b, a1, a2, a3 = yvv_coeffs(sigma / spacing[axis])
        stripe = list(b_size)
        stripe[axis] = 1
        for start in iter_region(b_index, stripe):
            line = []
            for k in range(n):
                idx = list(start)
                idx[axis] += k
                line.append(flat_index(b_index, b_size, idx))
            ym1 = ym2 = ym3 = vals[line[0]]
            for i in range(n):
                v = big_b * vals[line[i]] + a1 * ym1 + a2 * ym2 + a3 * ym3
                ym3, ym2, ym1 = ym2, ym1, v
                vals[line[i]] = v
            ym1 = ym2 = ym3 = vals[line[n - 1]]
            for i in range(n - 1, -1, -1):
                v = big_b * vals[line[i]] + a1 * ym1 + a2 * ym2 + a3 * ym3
                ym3, ym2, ym1 = ym2, ym1, v
                vals[line[i]] = v
    return vals


def split_region(index, size, n):
    n = max(n, 1)
    D = len(size)
    total = size[D - 1]
    actual = max(min(n, total), 1)
    base, rem = divmod(total, actual)
    start = index[D - 1]
    out = []
    for i in range(actual):
        sz = base + (1 if i < rem else 0)
        ii, ss = list(index), list(size)
        ii[D - 1], ss[D - 1] = start, sz
        out.append((ii, ss))
        start += sz
    return out


# ---- numpy <-> reference image ----------------------------------------------
def to_ref(arr, comps=1):
    """numpy (…, z, y, x[, c]) -> (index, size, pixels in iteration order)."""
    spatial = arr.shape[:-1] if comps > 1 else arr.shape
    size = list(reversed(spatial))
    flat = arr.reshape(-1, comps) if comps > 1 else arr.reshape(-1, 1)
    return ([0] * len(size), size, [tuple(p) for p in flat.tolist()])


def from_ref(res, comps, dtype):
    idx, size, data = res
    a = np.array([list(p) for p in data], dtype=dtype)
    shape = tuple(reversed(size))
    return a.reshape(shape + ((comps,) if comps > 1 else ()))


def case(name, arr, sigma, spacing=None, requested=None, comps=1, kind="f32"):
    D = len(arr.shape) - (1 if comps > 1 else 0)
    spacing = spacing or [1.0] * D
    img = to_ref(arr, comps)
    ri, rs = requested if requested else (img[0], img[1])
    res = generate_region(img, spacing, sigma, list(ri), list(rs), kind)
    out = from_ref(res, comps, np.float32 if kind == "f32" else np.uint8)
    return {f"{name}__in": arr, f"{name}__out": out,
            f"{name}__meta": np.array([sigma] + list(spacing) + [comps] + list(ri) + list(rs),
                                      dtype=np.float64)}


# ---- Demons and N4 (the Gaussian callers that iterate) ------------------------
def rust_round(x):
    """f64::round: half away from zero (exact: |x| - floor(|x|) is exact)."""
    a = abs(x)
    r = math.floor(a)
    if a - r >= 0.5:
        r += 1.0
    return math.copysign(r, x)


def rust_as_i64(v):
    """`f64 as i64`: saturating, NaN -> 0."""
    if v != v:
        return 0
    return int(max(min(v, 9.2233720368547758e18), -9.2233720368547758e18))


def demons_compute(fixed, moving, iterations, max_step):
    """DemonsRegistrationFilter::compute (registration_methods.rs:39-100);
    images as (index, size, pixels) with 1-tuples of np.float32."""
    (fidx, fsize, fdata), (midx, msize, mdata) = fixed, moving
    w, h = fsize
    ox, oy = fidx
    M = 1 << 64

    def flat_clamp(x, y):
        xi = min(max(x - ox, 0), w - 1)
        yi = min(max(y - oy, 0), h - 1)
        return yi * w + xi

    def get_moving(xi, yi):  # Image::get_pixel with wrapping usize offsets (image.rs:111-125)
        off = (((xi - midx[0]) % M) + ((yi - midx[1]) % M) * msize[0]) % M
        if off >= len(mdata):
            raise IndexError("the reference panics: index out of bounds")
        return mdata[off][0]

    disp_x = [0.0] * (w * h)
    disp_y = [0.0] * (w * h)
    for _ in range(iterations):
        new_x = list(disp_x)
        new_y = list(disp_y)
        for y in range(h):
            for x in range(w):
                i = y * w + x
                wx = float(x) + disp_x[i]
                wy = float(y) + disp_y[i]
                xi = ox + rust_as_i64(rust_round(wx))
                yi = oy + rust_as_i64(rust_round(wy))
                m_val = float(get_moving(xi, yi))
                f_val = float(fdata[i][0])
                gx = (float(fdata[flat_clamp(ox + x + 1, oy + y)][0]) - float(fdata[flat_clamp(ox + x - 1, oy + y)][0])) * 0.5
                gy = (float(fdata[flat_clamp(ox + x, oy + y + 1)][0]) - float(fdata[flat_clamp(ox + x, oy + y - 1)][0])) * 0.5
                intensity_diff = f_val - m_val
                denom = gx * gx + gy * gy + intensity_diff * intensity_diff + 1e-6
                step = intensity_diff / denom
                dx = step * gx
                dy = step * gy
                norm = math.sqrt(dx * dx + dy * dy)
                scale = max_step / norm if norm > max_step else 1.0
                new_x[i] = disp_x[i] + dx * scale
                new_y[i] = disp_y[i] + dy * scale
        disp_x, disp_y = new_x, new_y
    return disp_x, disp_y


def n4_region(img, spacing, iterations, sigma, threshold):
    """N4BiasFieldCorrectionFilter::generate_region (bias_correction.rs:45-83)."""
    idx, size, data = img
    corrected = [max(float(p[0]), 1e-6) for p in data]
    run = 0
    for _ in range(iterations):
        log_data = [math.log(v) for v in corrected]
        log_img = (idx, size, [(np.float32(v),) for v in log_data])
        smoothed = generate_region(log_img, spacing, sigma, list(idx), list(size))[2]
        prev = corrected
        corrected = [max(math.exp(l - float(s[0])), 1e-6) for l, s in zip(log_data, smoothed)]
        run += 1
        diff = 0.0
        for a, b in zip(corrected, prev):
            diff += abs(a - b)
        diff /= float(len(corrected))
        if diff < threshold:
            break
    return [np.float32(v) for v in corrected], run


def main():
    rng = np.random.default_rng(20261203)
    cases = {}
    imp = np.zeros((21, 21), np.float32)
    imp[10, 10] = 1.0
    cases.update(case("impulse2d_s1p5", imp, 1.5))
    imp3 = np.zeros((11, 11, 11), np.float32)
    imp3[5, 5, 5] = 1.0
    cases.update(case("impulse3d_s1", imp3, 1.0))
    vec = np.zeros((11, 11, 3), np.float32)
    vec[5, 5] = [1.0, 2.0, 3.0]
    cases.update(case("vecpixel2d_s1", vec, 1.0, comps=3))
    r2 = rng.random((17, 23), dtype=np.float32)
    cases.update(case("rand2d_s1p5", r2, 1.5))
    cases.update(case("rand2d_sub_s1p5", r2, 1.5, requested=([4, 3], [12, 9])))
    r3 = (rng.standard_normal((9, 12, 14)) * 3).astype(np.float32)
    cases.update(case("rand3d_s1p2", r3, 1.2))
    cases.update(case("rand3d_aniso", r3, 1.5, spacing=[0.7, 0.9, 2.5]))
    cases.update(case("rand3d_sub_s2", r3, 2.0, requested=([2, 1, 3], [9, 10, 4])))
    # radius larger than the image (clamp on both ends)
    small = rng.random((5, 4), dtype=np.float32)
    cases.update(case("tiny2d_s3", small, 3.0))
    # 1-D
    cases.update(case("line1d_s2", rng.random((40,), dtype=np.float32), 2.0))
    # u8 NumericPixel arithmetic (wrapping u8 adds)
    u8 = rng.integers(0, 256, (13, 16), dtype=np.uint8)
    cases.update(case("u8pixel2d_s1p5", u8, 1.5, kind="u8"))
    u8w = np.full((8, 9), 255, np.uint8)
    cases.update(case("u8pixel2d_wrap_s1", u8w, 1.0, kind="u8"))
    # i16 -> f32 cast chain (UnaryFilter(p as f32) then Gaussian<f32>)
    i16 = rng.integers(-1000, 1500, (6, 10, 12)).astype(np.int16)
    c = case("i16cast3d_s1p5", i16.astype(np.float32), 1.5, spacing=[0.7, 0.7, 2.5])
    c["i16cast3d_s1p5__in"] = i16
    cases.update(c)
    # stream_full with 4 pieces on the impulse (tests/pipeline.rs:106-129)
    img = to_ref(np.pad(np.zeros((20, 20), np.float32), 0))
    data = [list(p) for p in img[2]]
    data[10 * 20 + 10] = [1.0]
    img = (img[0], img[1], [tuple(p) for p in data])
    full = np.zeros((20, 20), np.float32)
    for pi, ps in split_region([0, 0], [20, 20], 4):
        part = from_ref(generate_region(img, [1.0, 1.0], 1.5, pi, ps), 1, np.float32)
        full[pi[1]:pi[1] + ps[1], pi[0]:pi[0] + ps[0]] = part
    cases["stream4_impulse2d__out"] = full
    # the convolve_axis family: mean, per-axis box mean, binomial blur
    srng = np.random.default_rng(20261204)

    def sep_case(name, arr, family, param, requested=None, comps=1, kind="f32"):
        D = len(arr.shape) - (1 if comps > 1 else 0)
        if family == "mean":
            kernels, reps, radii = [box_kernel(param)] * D, 1, [param] * D
        elif family == "boxmean":
            kernels, reps, radii = [box_kernel(r) for r in param], 1, list(param)
        else:
            kernels, reps, radii = [BINOMIAL] * D, param, [1] * D
        img = to_ref(arr, comps)
        ri, rs = requested if requested else (img[0], img[1])
        res = separable_region(img, kernels, reps, list(ri), list(rs), kind)
        out = from_ref(res, comps, np.float32 if kind == "f32" else np.uint8)
        fam = {"mean": 0, "boxmean": 1, "binomial": 2}[family]
        rad3 = radii + [0] * (3 - D)
        return {f"sep_{name}__in": arr, f"sep_{name}__out": out,
                f"sep_{name}__meta": np.array([fam, reps, comps] + rad3 + list(ri) + list(rs),
                                              dtype=np.int64)}

    cases.update(sep_case("mean1d_const_r2", np.full((10,), 5.0, np.float32), "mean", 2))
    cases.update(sep_case("mean1d_ramp_r2", np.arange(20, dtype=np.float32), "mean", 2))
    cases.update(sep_case("boxmean2d_const", np.full((8, 8), 3.0, np.float32), "boxmean", (1, 2)))
    m2 = srng.random((13, 17), dtype=np.float32)
    cases.update(sep_case("mean2d_r3", m2, "mean", 3))
    cases.update(sep_case("mean2d_sub_r2", m2, "mean", 2, requested=([3, 2], [9, 8])))
    m3 = (srng.standard_normal((7, 9, 11)) * 2).astype(np.float32)
    cases.update(sep_case("mean3d_r2", m3, "mean", 2))
    cases.update(sep_case("boxmean3d_aniso", m3, "boxmean", (1, 3, 2)))
    cases.update(sep_case("mean2d_r6_tiny", srng.random((4, 5), dtype=np.float32), "mean", 6))
    cases.update(sep_case("mean_vec2d_r1", srng.random((6, 7, 3), dtype=np.float32), "mean", 1, comps=3))
    cases.update(sep_case("mean_u8_2d_r2", srng.integers(0, 256, (9, 10), dtype=np.uint8), "mean", 2,
                          kind="u8"))
    cases.update(sep_case("binomial1d_const_r4", np.full((20,), 3.0, np.float32), "binomial", 4))
    bimp = np.zeros((21,), np.float32)
    bimp[10] = 1.0
    cases.update(sep_case("binomial1d_impulse_r4", bimp, "binomial", 4))
    cases.update(sep_case("binomial2d_r3", m2, "binomial", 3))
    cases.update(sep_case("binomial2d_sub_r2", m2, "binomial", 2, requested=([2, 4], [11, 6])))
    cases.update(sep_case("binomial3d_r2", m3, "binomial", 2))
    cases.update(sep_case("binomial3d_r0", m3, "binomial", 0))
    cases.update(sep_case("binomial_u8_2d_r2", srng.integers(0, 256, (8, 9), dtype=np.uint8),
                          "binomial", 2, kind="u8"))
    # RecursiveGaussianFilter: f64 result before the output conversion, and the f32 output
    rrng = np.random.default_rng(20261205)

    def rec_case(name, arr, sigma, spacing=None, axis=None):
        D = arr.ndim
        spacing = spacing or [1.0] * D
        img = to_ref(arr)
        vals = recursive_region(img, spacing, sigma, axis)
        f64 = np.array(vals, dtype=np.float64).reshape(arr.shape)
        return {f"rec_{name}__in": arr, f"rec_{name}__f64": f64,
                f"rec_{name}__meta": np.array([sigma, -1 if axis is None else axis] + list(spacing), dtype=np.float64)}

    r1 = np.zeros((51,), np.float32)
    r1[25] = 1.0
    cases.update(rec_case("impulse1d_s2", r1, 2.0))
    cases.update(rec_case("const2d_s1p5", np.full((15, 15), 4.0, np.float32), 1.5))
    cases.update(rec_case("rand2d_s3", rrng.random((12, 17), dtype=np.float32), 3.0))
    cases.update(rec_case("rand3d_s1p2_aniso", (rrng.standard_normal((6, 8, 9)) * 2).astype(np.float32), 1.2,
                          spacing=[0.8, 1.0, 2.0]))
    cases.update(rec_case("rand3d_axis1_s0p3", rrng.random((5, 7, 6), dtype=np.float32), 0.3, axis=1))
    cases.update(rec_case("u8_2d_s2", rrng.integers(0, 256, (9, 11), dtype=np.uint8), 2.0))
    cases.update(rec_case("thin3d_s2", rrng.random((1, 6, 7), dtype=np.float32), 2.0))

    # derivative users of RecursiveGaussianFilter (edges.rs:686-950): stencils on the
    # smoothed image (pixel type of the input), clamped to the requested region
    def rec_deriv_case(name, arr, sigma, kind, spacing=None, axis=0, order=1, requested=None):
        D = arr.ndim
        spacing = spacing or [1.0] * D
        img = to_ref(arr)
        vals = recursive_region(img, spacing, sigma)
        ri, rs = requested if requested else (img[0], img[1])
        full_idx, full_size = img[0], img[1]
        def u8_from_f64(v):  # pixel.rs:36: round half away from zero, clamp, NaN -> 0
            if v != v:
                return 0.0
            a = abs(v)
            r = (math.floor(a) + (1.0 if a - math.floor(a) >= 0.5 else 0.0)) * (1.0 if v >= 0 else -1.0)
            return float(min(max(r, 0.0), 255.0))

        conv = u8_from_f64 if arr.dtype == np.uint8 else (lambda v: float(np.float32(v)))
        sm = {tuple(p): conv(vals[flat_index(full_idx, full_size, p)]) for p in iter_region(ri, rs)}

        def get(p, a, off):
            q = list(p)
            q[a] = min(max(p[a] + off, ri[a]), ri[a] + rs[a] - 1)
            return sm[tuple(q)]

        out = []
        for p in iter_region(ri, rs):
            p = tuple(p)
            if kind == 0:
                mag2 = 0.0
                for a in range(D):
                    dd = (get(p, a, 1) - get(p, a, -1)) / (2.0 * spacing[a])
                    mag2 += dd * dd
                out.append([math.sqrt(mag2)])
            elif kind == 1:
                lap = 0.0
                for a in range(D):
                    lap += (get(p, a, 1) - 2.0 * get(p, a, 0) + get(p, a, -1)) / (spacing[a] * spacing[a])
                out.append([lap])
            elif kind == 2:
                h = spacing[axis]
                v = ((get(p, axis, 1) - get(p, axis, -1)) / (2.0 * h) if order == 1 else
                     (get(p, axis, 1) - 2.0 * get(p, axis, 0) + get(p, axis, -1)) / (h * h) if order == 2 else 0.0)
                out.append([v])
            elif kind == 3:
                out.append([(get(p, a, 1) - get(p, a, -1)) / (2.0 * spacing[a]) for a in range(D)])
            else:
                hx, hy = spacing
                x0, y0 = p

                def g2(xi, yi):
                    return sm[(min(max(xi, ri[0]), ri[0] + rs[0] - 1), min(max(yi, ri[1]), ri[1] + rs[1] - 1))]
                h00 = (g2(x0 + 1, y0) - 2.0 * g2(x0, y0) + g2(x0 - 1, y0)) / (hx * hx)
                h11 = (g2(x0, y0 + 1) - 2.0 * g2(x0, y0) + g2(x0, y0 - 1)) / (hy * hy)
                h01 = (g2(x0 + 1, y0 + 1) - g2(x0 + 1, y0 - 1) - g2(x0 - 1, y0 + 1) + g2(x0 - 1, y0 - 1)) / (4.0 * hx * hy)
                out.append([h00, h11, h01])
        vec = kind >= 3
        shape = tuple(reversed(rs)) + ((len(out[0]),) if vec else ())
        if vec:
            res = np.array(out, dtype=np.float64).astype(np.float32).reshape(shape)
        elif arr.dtype == np.uint8:
            res = np.array([conv(o[0]) for o in out], dtype=np.float64).astype(np.uint8).reshape(shape)
        else:
            res = np.array([o[0] for o in out], dtype=np.float64).astype(np.float32).reshape(shape)
        return {f"recd_{name}__in": arr, f"recd_{name}__out": res,
                f"recd_{name}__meta": np.array([sigma, kind, axis, order] + list(spacing) + list(ri) + list(rs),
                                               dtype=np.float64)}

    d2 = rrng.random((11, 13), dtype=np.float32)
    d3 = (rrng.standard_normal((6, 7, 8)) * 3).astype(np.float32)
    cases.update(rec_deriv_case("gm2d", d2, 1.5, 0))
    cases.update(rec_deriv_case("gm3d_sub", d3, 1.2, 0, spacing=[0.8, 1.0, 1.5], requested=([1, 2, 1], [5, 4, 3])))
    cases.update(rec_deriv_case("lap2d", d2, 2.0, 1, spacing=[0.7, 1.3]))
    cases.update(rec_deriv_case("deriv3d_o1_a2", d3, 1.0, 2, axis=2, order=1))
    cases.update(rec_deriv_case("deriv2d_o2_a0_sub", d2, 1.7, 2, axis=0, order=2, requested=([3, 2], [6, 7])))
    cases.update(rec_deriv_case("deriv2d_o3", d2, 1.7, 2, axis=1, order=3))
    cases.update(rec_deriv_case("grad3d", d3, 1.4, 3, spacing=[1.0, 0.5, 2.0]))
    cases.update(rec_deriv_case("hess2d", d2, 1.1, 4, spacing=[0.9, 1.2]))
    cases.update(rec_deriv_case("hess2d_sub", d2, 1.1, 4, requested=([2, 3], [7, 6])))
    cases.update(rec_deriv_case("gm_u8_2d", rrng.integers(0, 256, (9, 10), dtype=np.uint8), 1.5, 0))

    # ZeroCrossingBasedEdgeDetectionFilter (edges.rs:1019-1052): zero crossings of the
    # Laplacian case above (same inputs), clamped to the requested region
    def zc_case(name, lap_name):
        lap = cases[f"recd_{lap_name}__out"]
        D = lap.ndim
        shape = lap.shape
        flat = lap.reshape(-1).tolist()
        size = list(reversed(shape))
        out = []
        for p in iter_region([0] * D, size):
            c = float(flat[flat_index([0] * D, size, p)])
            hit = False
            for a in range(D):
                for off in (-1, 1):
                    q = list(p)
                    q[a] = min(max(p[a] + off, 0), size[a] - 1)
                    if c * float(flat[flat_index([0] * D, size, q)]) < 0.0:
                        hit = True
            out.append(1.0 if hit else 0.0)
        res = np.array(out, dtype=lap.dtype).reshape(shape)
        return {f"recz_{name}__out": res}

    zd3 = (rrng.standard_normal((7, 8, 9)) * 3).astype(np.float32)
    cases.update(rec_deriv_case("lap3d_zc_sub", zd3, 1.3, 1, spacing=[1.0, 0.8, 1.2], requested=([1, 1, 2], [7, 6, 4])))
    cases.update(zc_case("lap2d", "lap2d"))
    cases.update(zc_case("lap3d_sub", "lap3d_zc_sub"))

    # UnsharpMaskFilter (edges.rs:406-452): the family blur with its own kernel on
    # every axis, then the f64 point-wise step on the requested region
    urng = np.random.default_rng(20261206)

    def unsharp_case(name, arr, sigma, amount, threshold, requested=None, comps=1):
        D = len(arr.shape) - (1 if comps > 1 else 0)
        kind = "u8" if arr.dtype == np.uint8 else "f32"
        r = int(math.ceil(3.0 * sigma))
        k = [math.exp(-((float(i) - float(r)) * (float(i) - float(r))) / (2.0 * sigma * sigma))
             for i in range(2 * r + 1)]
        s = 0.0
        for v in k:
            s += v
        k = [v / s for v in k]
        img = to_ref(arr, comps)
        ri, rs = requested if requested else (img[0], img[1])
        blur = separable_region(img, [k] * D, 1, list(ri), list(rs), kind)
        out = []
        for p, b in zip(iter_region(list(ri), list(rs)), blur[2]):
            orig = float(img[2][flat_index(img[0], img[1], p)][0])
            edge = orig - float(b[0])
            v = orig + amount * edge if abs(edge) > threshold else orig
            if kind == "u8":
                a = abs(v)
                q = (math.floor(a) + (1.0 if a - math.floor(a) >= 0.5 else 0.0)) * (1.0 if v >= 0 else -1.0)
                v = int(min(max(q, 0.0), 255.0))
            out.append(tuple([v] * comps))
        res = from_ref((list(ri), list(rs), out), comps, np.float32 if kind == "f32" else np.uint8)
        return {f"ush_{name}__in": arr, f"ush_{name}__out": res,
                f"ush_{name}__meta": np.array([sigma, amount, threshold, comps] + list(ri) + list(rs),
                                              dtype=np.float64)}

    u2 = urng.random((12, 15), dtype=np.float32)
    u3 = (urng.standard_normal((6, 7, 9)) * 2).astype(np.float32)
    cases.update(unsharp_case("f32_2d_s1", u2, 1.0, 0.5, 0.0))
    cases.update(unsharp_case("f32_2d_sub_s1p3", u2, 1.3, 1.5, 0.05, requested=([3, 2], [8, 7])))
    cases.update(unsharp_case("f32_3d_s0p8", u3, 0.8, 0.7, 0.5))
    cases.update(unsharp_case("f32_1d_s2", urng.random((30,), dtype=np.float32), 2.0, 0.5, 0.0))
    cases.update(unsharp_case("vec2d_s1", urng.random((7, 8, 3), dtype=np.float32), 1.0, 0.5, 0.0, comps=3))
    cases.update(unsharp_case("u8_2d_s1p5", urng.integers(0, 256, (10, 11), dtype=np.uint8), 1.5, 0.9, 3.0))
    # in-crate callers of GaussianFilter (spatial.rs): SliceBySliceFilter, BSplineDownsampleFilter
    crng = np.random.default_rng(20261207)

    def slice_case(name, arr, sigma, spacing, requested, kind="f32"):
        ri, rs = requested
        out = []
        for z in range(rs[2]):
            pix = [(arr[ri[2] + z, ri[1] + y, ri[0] + x],) for y in range(rs[1]) for x in range(rs[0])]
            img2 = ([ri[0], ri[1]], [rs[0], rs[1]], pix)
            res = generate_region(img2, spacing[:2], sigma, [ri[0], ri[1]], [rs[0], rs[1]], kind)
            out.append(from_ref(res, 1, np.float32 if kind == "f32" else np.uint8))
        return {f"cal_{name}__in": arr, f"cal_{name}__out": np.stack(out),
                f"cal_{name}__meta": np.array([0, sigma] + list(spacing) + list(ri) + list(rs), dtype=np.float64)}

    def bspline_case(name, arr, spacing, kind="f32"):
        img = to_ref(arr)
        res = generate_region(img, spacing, 1.0, img[0], img[1], kind)
        full = from_ref(res, 1, np.float32 if kind == "f32" else np.uint8)
        D = arr.ndim
        sub = np.ascontiguousarray(full[tuple([slice(None, None, 2)] * D)])
        return {f"cal_{name}__in": arr, f"cal_{name}__out": sub,
                f"cal_{name}__meta": np.array([1, 1.0] + list(spacing), dtype=np.float64)}

    c3 = (crng.standard_normal((5, 9, 11)) * 2).astype(np.float32)
    cases.update(slice_case("slices_s1p2", c3, 1.2, [1.0, 0.8, 2.0], ([1, 2, 1], [9, 6, 3])))
    cases.update(slice_case("slices_u8_s1", crng.integers(0, 256, (3, 7, 8), dtype=np.uint8), 1.0, [1.0, 1.0, 1.0],
                            ([0, 0, 0], [8, 7, 3]), kind="u8"))
    cases.update(bspline_case("bspline3d_odd", c3, [1.0, 1.0, 1.0]))
    cases.update(bspline_case("bspline2d_aniso", (crng.random((9, 12), dtype=np.float32)), [0.7, 1.5]))

    def dfb_case(name, field, sigma, requested):
        """DisplacementFieldToBSplineFilter (spatial.rs:1484-1525): the requested crop of a
        VecPixel<f32, 2> field, each component smoothed by GaussianFilter { sigma } over the crop
        as an image of its own (whose largest region, and so clamp bounds, is the crop)."""
        ri, rs = requested
        out = []
        for c in range(2):
            pix = [(field[ri[1] + y, ri[0] + x, c],) for y in range(rs[1]) for x in range(rs[0])]
            res = generate_region((list(ri), list(rs), pix), [1.0, 1.0], sigma, list(ri), list(rs))
            out.append(from_ref(res, 1, np.float32))
        return {f"cal_{name}__in": field, f"cal_{name}__out": np.stack(out, axis=-1),
                f"cal_{name}__meta": np.array([2, sigma] + list(ri) + list(rs), dtype=np.float64)}

    f2 = (crng.standard_normal((13, 17, 2)) * 1.5).astype(np.float32)
    cases.update(dfb_case("dfbspline_s2", f2, 2.0, ([0, 0], [17, 13])))
    cases.update(dfb_case("dfbspline_sub_s1p5", f2, 1.5, ([3, 2], [11, 8])))
    # kernels
    for s, sp in [(1.5, 1.0), (2.0, 1.0), (1.5, 0.7), (1.5, 2.5), (0.5, 1.0), (8.0, 1.0)]:
        cases[f"kernel_{s}_{sp}"] = np.array(build_kernel(s / sp, kernel_radius(s, sp)),
                                             dtype=np.float64)
    # Demons (forward field, f32 output) and its diffeomorphic smoothing
    drng = np.random.default_rng(20261205)
    # compact blobs well inside the frame: the field stays zero near the edges,
    # so no warped index leaves the moving image (where the reference panics)
    yy, xx = np.mgrid[0:14, 0:16].astype(np.float64)
    fixed = np.maximum(0.0, 1.0 - np.hypot(xx - 7.5, yy - 6.5) / 3.0).astype(np.float32)
    moving = np.maximum(0.0, 1.0 - np.hypot(xx - 8.0, yy - 7.0) / 3.0).astype(np.float32)
    moving += np.where(moving > 0, drng.standard_normal(moving.shape) * 0.01, 0.0).astype(np.float32)
    for name, iters, step, diffeo in [("blob_3", 3, 2.0, False), ("blob_6_step05", 6, 0.5, False),
                                      ("blob_3_diffeo", 3, 2.0, True)]:
        dxl, dyl = demons_compute(to_ref(fixed), to_ref(moving), iters, step)
        field = np.stack([np.array(dxl, np.float64).astype(np.float32).reshape(fixed.shape),
                          np.array(dyl, np.float64).astype(np.float32).reshape(fixed.shape)], axis=-1)
        if diffeo:
            sm = [from_ref(generate_region(to_ref(field[..., c]), [1.0, 1.0], 1.0, [0, 0], [16, 14]), 1, np.float32)
                  for c in range(2)]
            field = np.stack(sm, axis=-1)
        cases[f"dem_{name}__fixed"] = fixed
        cases[f"dem_{name}__moving"] = moving
        cases[f"dem_{name}__out"] = field
        cases[f"dem_{name}__meta"] = np.array([iters, step, 1.0 if diffeo else 0.0, 1.0], dtype=np.float64)
    # N4: a smooth multiplicative bias over a two-level image
    yy, xx = np.mgrid[0:6, 0:8].astype(np.float64)
    bias = 1.0 + 0.3 * (xx / 7.0) + 0.2 * (yy / 5.0)
    base = np.where((xx - 3.5) ** 2 + (yy - 2.5) ** 2 < 5.0, 100.0, 40.0)
    n4img = (base * bias + drng.standard_normal(base.shape)).astype(np.float32)
    for name, iters, sigma, spacing in [("default", 4, 30.0, [1.0, 1.0]), ("s2_aniso", 6, 2.0, [0.8, 1.2]),
                                        ("s1_one", 1, 1.0, [1.0, 1.0])]:
        out, run = n4_region(to_ref(n4img), spacing, iters, sigma, 1e-3)
        cases[f"n4_{name}__in"] = n4img
        cases[f"n4_{name}__out"] = np.array(out, np.float32).reshape(n4img.shape)
        cases[f"n4_{name}__meta"] = np.array([iters, sigma, 1e-3, run] + spacing, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **cases)
    print(f"wrote {len(cases)} arrays to golden.npz")


if __name__ == "__main__":
    main()
