"""CPU oracle for the separable Gaussian path -- TEST INFRASTRUCTURE ONLY.

Only tests/, the smoke check in __graft_entry__.py and bench.py's CPU-baseline
leg import this module; the product never does.  It wraps the C restatement
in gauss_oracle.c (reference semantics, see that file's header for the
file:line map) and adds numpy FP64 helpers for the adjoint checks.  The rows
beyond the Gaussian are restated here on top of the C core, each function
citing the reference lines it follows:
  separable_* / mean_f32 / binomial_f32   mean.rs, binomial_blur.rs (C core)
  recursive_gaussian_f64 / _f32           recursive_gaussian.rs:33-239 (C core)
  recursive_derivative / _difference_of_gaussians / _zero_crossing_edges
                                          filters/edges.rs:686-1052 (numpy f64)
  unsharp_kernel / unsharp_mask           filters/edges.rs:374-452 (math.exp, numpy f64)
  slice_by_slice / bspline_downsample     filters/spatial.rs:1128-1166, 1284-1340

Array convention used throughout the tests: a reference ``Image<P, D>`` with
axis 0 fastest is a C-ordered numpy array whose LAST spatial axis is the
reference's axis 0, i.e. shape (nz, ny, nx) for D=3 and (ny, nx) for D=2, with
a trailing component axis for ``VecPixel<f32, 3>``.  Regions are given in the
reference's axis order: ``index=(ix, iy, iz)``, ``size=(sx, sy, sz)``.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liborc.so")
_lib = None


class Region(ctypes.Structure):
    _fields_ = [("index", ctypes.c_int64 * 3), ("size", ctypes.c_int64 * 3)]


def build():
    """Compile the C restatement (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        src = os.path.join(_HERE, "gauss_oracle.c")
        if (not os.path.exists(_LIB_PATH)
                or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src)):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        R = ctypes.POINTER(Region)
        L.orc_kernel_radius.restype = ctypes.c_uint64
        L.orc_kernel_radius.argtypes = [ctypes.c_double, ctypes.c_double]
        L.orc_build_kernel.restype = None
        L.orc_build_kernel.argtypes = [ctypes.c_double, ctypes.c_uint64, P]
        for name in ("orc_gaussian_f32", "orc_gaussian_u8", "orc_gaussian_f64"):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [P, R, P, ctypes.c_int, ctypes.c_int, ctypes.c_double, R, P]
        L.orc_gaussian_f32_mt.restype = ctypes.c_int
        L.orc_gaussian_f32_mt.argtypes = [P, R, P, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_double, R, P, ctypes.c_int]
        L.orc_stream_full_f32.restype = ctypes.c_int
        L.orc_stream_full_f32.argtypes = [P, R, P, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_uint64, P]
        L.orc_split_region.restype = ctypes.c_int64
        L.orc_split_region.argtypes = [R, ctypes.c_int, ctypes.c_uint64, R]
        L.orc_convolve_axis.restype = ctypes.c_int
        L.orc_convolve_axis.argtypes = [P, R, ctypes.c_int, ctypes.c_int, ctypes.c_int, P,
                                        ctypes.c_uint64, R, P, ctypes.c_int]
        for name in ("orc_separable_f32", "orc_separable_u8", "orc_separable_f64"):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [P, R, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_uint64, R, P]
        L.orc_separable_f32_mt.restype = ctypes.c_int
        L.orc_separable_f32_mt.argtypes = [P, R, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_uint64,
                                           R, P, ctypes.c_int]
        L.orc_yvv_coeffs.restype = None
        L.orc_yvv_coeffs.argtypes = [ctypes.c_double, P]
        L.orc_recursive_gaussian_f64.restype = None
        L.orc_recursive_gaussian_f64.argtypes = [P, P, P, ctypes.c_int, ctypes.c_double, ctypes.c_int]
        L.orc_box_kernel.restype = None
        L.orc_box_kernel.argtypes = [ctypes.c_uint64, P]
        L.orc_cast_f32_to_u8.restype = None
        L.orc_cast_f32_to_u8.argtypes = [P, P, ctypes.c_int64]
        L.orc_demons_f64.restype = ctypes.c_int
        L.orc_demons_f64.argtypes = [P, R, P, R, ctypes.c_int, ctypes.c_double, P, P]
        L.orc_n4_f32.restype = ctypes.c_int
        L.orc_n4_f32.argtypes = [P, R, P, ctypes.c_int, ctypes.c_double, ctypes.c_double, P]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def make_region(index, size) -> Region:
    r = Region()
    for d in range(3):
        r.index[d] = int(index[d]) if d < len(index) else 0
        r.size[d] = int(size[d]) if d < len(size) else 1
    return r


def region_tuple(r: Region, D: int):
    return tuple(r.index[d] for d in range(D)), tuple(r.size[d] for d in range(D))


def kernel_radius(sigma: float, spacing: float) -> int:
    """gaussian.rs:24-27."""
    return int(lib().orc_kernel_radius(sigma, spacing))


def build_kernel(sigma_px: float, radius: int) -> np.ndarray:
    """gaussian.rs:29-40 (f64 weights)."""
    out = np.zeros(2 * radius + 1, dtype=np.float64)
    lib().orc_build_kernel(sigma_px, radius, _ptr(out))
    return out


def _dims(img: np.ndarray, comps: int):
    shape = img.shape[:-1] if comps > 1 else img.shape
    D = len(shape)
    return D, tuple(reversed(shape))  # reference axis order sizes


def _run(fn, img, dtype, sigma, spacing, index, requested, comps, extra=()):
    img = np.ascontiguousarray(img, dtype=dtype)
    D, sizes = _dims(img, comps)
    index = tuple(index) if index is not None else (0,) * D
    spacing = np.ascontiguousarray(spacing if spacing is not None else [1.0] * D,
                                   dtype=np.float64)
    img_reg = make_region(index, sizes)
    if requested is None:
        req = make_region(index, sizes)
    else:
        req = make_region(*requested)
    out_shape = tuple(reversed([req.size[d] for d in range(D)]))
    if comps > 1:
        out_shape = out_shape + (comps,)
    out = np.empty(out_shape, dtype=dtype)
    rc = fn(_ptr(img), ctypes.byref(img_reg), _ptr(spacing), D, comps, float(sigma),
            ctypes.byref(req), _ptr(out), *extra)
    if rc != 0:
        raise RuntimeError("oracle: generate_region failed (allocation or radius)")
    return out


def gaussian_f32(img, sigma, spacing=None, index=None, requested=None, comps=1):
    """GaussianFilter<Image<f32|VecPixel<f32,3>>>::generate_region, exact reference f32."""
    return _run(lib().orc_gaussian_f32, img, np.float32, sigma, spacing, index, requested,
                comps)


def gaussian_f32_mt(img, sigma, spacing=None, index=None, requested=None, comps=1,
                    nthreads=None):
    """Timing port (same arithmetic as gaussian_f32) with the reference's threading shape."""
    n = nthreads or os.cpu_count() or 1
    return _run(lib().orc_gaussian_f32_mt, img, np.float32, sigma, spacing, index,
                requested, comps, (n,))


def gaussian_u8(img, sigma, spacing=None, index=None, requested=None, comps=1):
    """GaussianFilter<Image<u8>>: per-tap f64 round+clamp, wrapping u8 adds (pixel.rs:430-435)."""
    return _run(lib().orc_gaussian_u8, img, np.uint8, sigma, spacing, index, requested,
                comps)


def gaussian_f64(img, sigma, spacing=None, index=None, requested=None, comps=1):
    """FP64 oracle: same kernel and clamp boundary, f64 arithmetic throughout."""
    return _run(lib().orc_gaussian_f64, img, np.float64, sigma, spacing, index, requested,
                comps)


def stream_full_f32(img, sigma, num_pieces, spacing=None, index=None, comps=1):
    """source.rs:81-98 over GaussianFilter<Image<f32>>."""
    img = np.ascontiguousarray(img, dtype=np.float32)
    D, sizes = _dims(img, comps)
    index = tuple(index) if index is not None else (0,) * D
    sp = np.ascontiguousarray(spacing if spacing is not None else [1.0] * D, dtype=np.float64)
    reg = make_region(index, sizes)
    out = np.empty_like(img)
    rc = lib().orc_stream_full_f32(_ptr(img), ctypes.byref(reg), _ptr(sp), D, comps,
                                   float(sigma), int(num_pieces), _ptr(out))
    if rc != 0:
        raise RuntimeError("oracle: stream_full failed")
    return out


BINOMIAL_KERNEL = np.array([0.25, 0.5, 0.25])  # binomial_blur.rs:35


def box_kernel(radius: int) -> np.ndarray:
    """box_kernel (mean.rs:15-18): 2r + 1 weights of 1 / (2r + 1)."""
    out = np.empty(2 * int(radius) + 1, dtype=np.float64)
    lib().orc_box_kernel(int(radius), _ptr(out))
    return out


def _run_separable(fn, img, dtype, kernels, reps, index, requested, comps, extra=()):
    img = np.ascontiguousarray(img, dtype=dtype)
    D, sizes = _dims(img, comps)
    index = tuple(index) if index is not None else (0,) * D
    ks = [np.ascontiguousarray(k, dtype=np.float64) for k in kernels]
    if len(ks) != D or any(len(k) % 2 != 1 for k in ks):
        raise ValueError("one odd-length kernel per axis")
    radii = (ctypes.c_uint64 * 3)(*([(len(k) - 1) // 2 for k in ks] + [0] * (3 - D)))
    kp = (ctypes.c_void_p * 3)(*([k.ctypes.data for k in ks] + [None] * (3 - D)))
    img_reg = make_region(index, sizes)
    req = make_region(index, sizes) if requested is None else make_region(*requested)
    out_shape = tuple(reversed([req.size[d] for d in range(D)]))
    if comps > 1:
        out_shape = out_shape + (comps,)
    out = np.empty(out_shape, dtype=dtype)
    rc = fn(_ptr(img), ctypes.byref(img_reg), D, comps, radii, kp, int(reps), ctypes.byref(req),
            _ptr(out), *extra)
    if rc != 0:
        raise RuntimeError("oracle: separable generate_region failed (allocation or radius)")
    return out


def separable_f32(img, kernels, reps=1, index=None, requested=None, comps=1):
    """The convolve_axis family (mean.rs, binomial_blur.rs) with one f64 kernel per axis
    and `reps` interleaved rounds, exact reference f32."""
    return _run_separable(lib().orc_separable_f32, img, np.float32, kernels, reps, index,
                          requested, comps)


def separable_u8(img, kernels, reps=1, index=None, requested=None, comps=1):
    """The family over Image<u8>: per-tap f64 round+clamp, wrapping u8 adds."""
    return _run_separable(lib().orc_separable_u8, img, np.uint8, kernels, reps, index,
                          requested, comps)


def separable_f64(img, kernels, reps=1, index=None, requested=None, comps=1):
    """FP64 oracle of the family: same schedule and clamp boundary, f64 arithmetic."""
    return _run_separable(lib().orc_separable_f64, img, np.float64, kernels, reps, index,
                          requested, comps)


def separable_f32_mt(img, kernels, reps=1, index=None, requested=None, comps=1, nthreads=None):
    """Timing port of the family (same arithmetic as separable_f32)."""
    n = nthreads or os.cpu_count() or 1
    return _run_separable(lib().orc_separable_f32_mt, img, np.float32, kernels, reps, index,
                          requested, comps, (n,))


def mean_f32(img, radius, **kw):
    """MeanFilter (mean.rs:27-84): the box kernel of `radius` on every axis."""
    D = _dims(np.asarray(img), kw.get("comps", 1))[0]
    return separable_f32(img, [box_kernel(radius)] * D, 1, **kw)


def box_mean_f32(img, radii, **kw):
    """BoxMeanFilterN (mean.rs:103-137): one box radius per axis (reference axis order)."""
    return separable_f32(img, [box_kernel(r) for r in radii], 1, **kw)


def binomial_f32(img, repetitions, **kw):
    """BinomialBlurFilter (binomial_blur.rs:17-89)."""
    D = _dims(np.asarray(img), kw.get("comps", 1))[0]
    return separable_f32(img, [BINOMIAL_KERNEL] * D, repetitions, **kw)


def slice_by_slice(img, sigma, spacing=None, index=None, requested=None, comps=1):
    """SliceBySliceFilter (spatial.rs:1304-1339) over a 3-D Image<f32> or Image<u8>: every
    z slice of the requested region, as a 2-D Image over the request's x-y window with the
    x and y spacing, through GaussianFilter (clamped to that window)."""
    x = np.asarray(img)
    D, sizes = _dims(x, comps)
    if D != 3:
        raise ValueError("SliceBySliceFilter is 3-D")
    idx = tuple(index) if index is not None else (0, 0, 0)
    ri, rs = requested if requested is not None else (idx, tuple(sizes))
    sl = tuple(slice(ri[d] - idx[d], ri[d] - idx[d] + rs[d]) for d in reversed(range(3)))
    crop = x[sl]
    sp2 = list(spacing[:2]) if spacing is not None else [1.0, 1.0]
    fn = gaussian_u8 if x.dtype == np.uint8 else gaussian_f32
    return np.ascontiguousarray(np.stack([fn(crop[k], sigma, sp2, comps=comps) for k in range(crop.shape[0])]))


def bspline_downsample(img, spacing=None, comps=1):
    """BSplineDownsampleFilter (spatial.rs:1155-1166): GaussianFilter sigma 1.0 over the whole
    image, then every other voxel from the first on every axis."""
    x = np.asarray(img)
    fn = gaussian_u8 if x.dtype == np.uint8 else gaussian_f32
    full = fn(x, 1.0, spacing, comps=comps)
    D = _dims(x, comps)[0]
    return np.ascontiguousarray(full[tuple([slice(None, None, 2)] * D)])


def displacement_field_to_bspline(field, sigma=2.0, spacing=None, index=None, requested=None):
    """DisplacementFieldToBSplineFilter (spatial.rs:1484-1525) over a 2-D
    VecPixel<f32, 2> field (numpy (y, x, 2)): the requested crop, each
    component smoothed by GaussianFilter { sigma } over the crop as an image of
    its own -- the crop is the Gaussian's largest region, so its taps clamp at
    the crop's edges, not the field's."""
    x = np.asarray(field, dtype=np.float32)
    if x.ndim != 3 or x.shape[2] != 2:
        raise ValueError("a 2-D VecPixel<f32, 2> field (y, x, 2)")
    idx = tuple(index) if index is not None else (0, 0)
    ri, rs = requested if requested is not None else (idx, (x.shape[1], x.shape[0]))
    crop = x[ri[1] - idx[1]:ri[1] - idx[1] + rs[1], ri[0] - idx[0]:ri[0] - idx[0] + rs[0]]
    out = [gaussian_f32(np.ascontiguousarray(crop[..., c]), sigma, spacing) for c in range(2)]
    return np.ascontiguousarray(np.stack(out, axis=-1))


def unsharp_kernel(sigma: float) -> np.ndarray:
    """UnsharpMaskFilter's blur kernel (edges.rs:408, 415-424): radius ceil(3 sigma),
    exp(-(d d) / (2 sigma sigma)) through the C library's exp, divided by the
    left-to-right f64 sum."""
    sigma = float(sigma)
    r = int(math.ceil(3.0 * sigma))
    w = [math.exp(-((float(i) - float(r)) * (float(i) - float(r))) / (2.0 * sigma * sigma)) for i in range(2 * r + 1)]
    s = 0.0
    for v in w:
        s += v
    return np.array([v / s for v in w], dtype=np.float64)


def unsharp_mask(img, sigma, amount=0.5, threshold=0.0, index=None, requested=None, comps=1):
    """UnsharpMaskFilter::generate_region (edges.rs:406-452) over Image<f32> or
    Image<u8>: the family blur with unsharp_kernel on every axis, then per voxel
    edge = orig - blur, |edge| > threshold ? orig + amount * edge : orig in f64,
    P::from_f64.  Vector pixels read component 0 and fill every component."""
    x = np.ascontiguousarray(img)
    D, sizes = _dims(x, comps)
    k = unsharp_kernel(sigma)
    sep = separable_u8 if x.dtype == np.uint8 else separable_f32
    blur = sep(x, [k] * D, 1, index=index, requested=requested, comps=comps)
    idx = tuple(index) if index is not None else (0,) * D
    ri, rs = requested if requested is not None else (idx, tuple(sizes))
    sl = tuple(slice(ri[d] - idx[d], ri[d] - idx[d] + rs[d]) for d in reversed(range(D)))
    orig = x[sl]
    if comps > 1:
        orig, blur = orig[..., 0], blur[..., 0]
    o = orig.astype(np.float64)
    edge = o - blur.astype(np.float64)
    v = np.where(np.abs(edge) > float(threshold), o + float(amount) * edge, o)
    out = from_f64_u8(v) if x.dtype == np.uint8 else v.astype(np.float32)
    if comps > 1:
        out = np.repeat(out[..., None], comps, axis=-1)
    return np.ascontiguousarray(out)


def yvv_coeffs(sigma: float) -> np.ndarray:
    """(B, a1, a2, a3) of recursive_gaussian.rs:33-49."""
    out = np.empty(4, dtype=np.float64)
    lib().orc_yvv_coeffs(float(sigma), _ptr(out))
    return out


def recursive_gaussian_f64(img, sigma, spacing=None, axis=-1):
    """RecursiveGaussianFilter (axis = -1) or RecursiveGaussianAxisFilter (axis >= 0,
    reference axis order) over the whole image, before the output conversion:
    the f64 image after every causal / anticausal line pass."""
    a = np.array(img, dtype=np.float64, order="C", copy=True)  # P::to_f64 (exact for f32, i16, u8)
    D = a.ndim
    size = np.ascontiguousarray(list(reversed(a.shape)), dtype=np.int64)
    sp = np.ascontiguousarray(spacing if spacing is not None else [1.0] * D, dtype=np.float64)
    lib().orc_recursive_gaussian_f64(_ptr(a), _ptr(size), _ptr(sp), D, float(sigma), int(axis))
    return a


def from_f64_u8(v: np.ndarray) -> np.ndarray:
    """u8::from_f64 (pixel.rs:36): round half away from zero, clamp to [0, 255], NaN -> 0."""
    v = np.asarray(v, dtype=np.float64)
    a = np.abs(v)
    f = np.floor(a)
    r = np.copysign(f + (a - f >= 0.5), v)  # a - f is exact
    r = np.clip(np.nan_to_num(r, nan=0.0), 0.0, 255.0)
    return r.astype(np.uint8)


def recursive_gaussian_f32(img, sigma, spacing=None, axis=-1, requested=None, index=None):
    """RecursiveGaussianFilter<Image<f32>>::generate_region: f64 filtering, crop, `as f32`."""
    full = recursive_gaussian_f64(img, sigma, spacing, axis)
    return _crop(full, requested, index).astype(np.float32)


REC_GRADIENT_MAGNITUDE, REC_LAPLACIAN, REC_DERIVATIVE, REC_GRADIENT, REC_HESSIAN, REC_DOG, REC_ZERO_CROSSING = range(7)


def recursive_difference_of_gaussians(img, sigma1, sigma2, spacing=None, requested=None, index=None):
    """DifferenceOfGaussiansFilter (edges.rs:955-1009): both smoothings of the requested
    region in the pixel type, then P::from_f64(s1 - s2)."""
    x = np.asarray(img)
    D = x.ndim
    sp = list(spacing) if spacing is not None else [1.0] * D
    s = []
    for sg in (sigma1, sigma2):
        full = _crop(recursive_gaussian_f64(x, sg, sp), requested, index)
        s.append(from_f64_u8(full).astype(np.float64) if x.dtype == np.uint8 else full.astype(np.float32).astype(np.float64))
    v = s[0] - s[1]
    return from_f64_u8(v) if x.dtype == np.uint8 else v.astype(np.float32)


def recursive_zero_crossing_edges(img, sigma, spacing=None, requested=None, index=None):
    """ZeroCrossingBasedEdgeDetectionFilter (edges.rs:1019-1052): the Laplacian of the
    smoothed requested region in the pixel type (LaplacianFilter, edges.rs:217-247, over
    an image whose region is the requested one), then ZeroCrossingFilter (edges.rs:480-514):
    1 where center * neighbour < 0 for a clamped neighbour along some axis, else 0."""
    x = np.asarray(img)
    D = x.ndim
    lap = recursive_derivative(x, sigma, REC_LAPLACIAN, spacing, requested=requested, index=index)
    c = lap.astype(np.float64)
    zc = np.zeros(c.shape, dtype=bool)
    for ax in range(D):
        n = c.shape[ax]
        for off in (-1, 1):
            nb = np.take(c, np.clip(np.arange(n) + off, 0, n - 1), axis=ax)
            with np.errstate(invalid="ignore"):
                zc |= (c * nb) < 0.0
    return zc.astype(np.uint8 if x.dtype == np.uint8 else np.float32)


def recursive_derivative(img, sigma, kind, spacing=None, axis=0, order=1, requested=None, index=None):
    """The derivative users of RecursiveGaussianFilter (edges.rs:686-950): the
    smoothed image is RecursiveGaussianFilter::generate_region(requested) in the
    input's pixel type (f32 or u8), then a central-difference stencil clamped to
    the requested region's bounds (the smoothed image is the stencil's whole
    source), in f64 with every operation rounded in the reference's order:
      GRADIENT_MAGNITUDE  sqrt(sum_a ((s[+1] - s[-1]) / (2 h_a))^2)      (edges.rs:162-189)
      LAPLACIAN           sum_a ((s[+1] - 2 s[0]) + s[-1]) / (h_a h_a)    (edges.rs:219-247)
      DERIVATIVE          order 1 or 2 of the above along `axis`, else 0  (edges.rs:48-78)
      GRADIENT            per axis (s[+1] - s[-1]) / (2 h_a) as f32      (edges.rs:848-877)
      HESSIAN (2-D)       [h00, h11, h01] as f32                          (edges.rs:920-950)
    Returns the output array (pixel type for the first three, f32 components last axis otherwise)."""
    x = np.asarray(img)
    D = x.ndim
    sp = list(spacing) if spacing is not None else [1.0] * D
    full = recursive_gaussian_f64(x, sigma, sp)
    sm = _crop(full, requested, index)
    sm = from_f64_u8(sm).astype(np.float64) if x.dtype == np.uint8 else sm.astype(np.float32).astype(np.float64)

    def shifted(a, ax_ref, off):  # a[clamp(i + off)] along reference axis ax_ref, clamped to the array
        ax = D - 1 - ax_ref
        n = a.shape[ax]
        idx = np.clip(np.arange(n) + off, 0, n - 1)
        return np.take(a, idx, axis=ax)

    def pixel_out(v):
        return from_f64_u8(v) if x.dtype == np.uint8 else v.astype(np.float32)

    if kind == REC_GRADIENT_MAGNITUDE:
        mag2 = np.zeros_like(sm)
        for a in range(D):
            d = (shifted(sm, a, 1) - shifted(sm, a, -1)) / (2.0 * sp[a])
            mag2 = mag2 + d * d
        return pixel_out(np.sqrt(mag2))
    if kind == REC_LAPLACIAN:
        lap = np.zeros_like(sm)
        for a in range(D):
            lap = lap + ((shifted(sm, a, 1) - 2.0 * sm) + shifted(sm, a, -1)) / (sp[a] * sp[a])
        return pixel_out(lap)
    if kind == REC_DERIVATIVE:
        if order == 1:
            v = (shifted(sm, axis, 1) - shifted(sm, axis, -1)) / (2.0 * sp[axis])
        elif order == 2:
            v = ((shifted(sm, axis, 1) - 2.0 * sm) + shifted(sm, axis, -1)) / (sp[axis] * sp[axis])
        else:
            v = np.zeros_like(sm)
        return pixel_out(v)
    if kind == REC_GRADIENT:
        comps = [((shifted(sm, a, 1) - shifted(sm, a, -1)) / (2.0 * sp[a])).astype(np.float32) for a in range(D)]
        return np.stack(comps, axis=-1)
    if kind == REC_HESSIAN:
        if D != 2:
            raise ValueError("the Hessian filter is 2-D")
        hx, hy = sp[0], sp[1]
        xp, xm = shifted(sm, 0, 1), shifted(sm, 0, -1)
        h00 = ((xp - 2.0 * sm) + xm) / (hx * hx)
        h11 = ((shifted(sm, 1, 1) - 2.0 * sm) + shifted(sm, 1, -1)) / (hy * hy)
        h01 = (((shifted(xp, 1, 1) - shifted(xp, 1, -1)) - shifted(xm, 1, 1)) + shifted(xm, 1, -1)) / (4.0 * hx * hy)
        return np.stack([h00.astype(np.float32), h11.astype(np.float32), h01.astype(np.float32)], axis=-1)
    raise ValueError(f"unknown kind {kind}")


def _crop(full, requested, index):
    if requested is None:
        return full
    D = full.ndim
    index = tuple(index) if index is not None else (0,) * D
    (ri, rs) = requested
    sl = tuple(slice(ri[d] - index[d], ri[d] - index[d] + rs[d]) for d in reversed(range(D)))
    return full[sl]


def split_region(index, size, num_pieces):
    """region_splitter.rs:17-48 -> list of (index, size) tuples."""
    D = len(size)
    reg = make_region(index, size)
    n = max(int(num_pieces), 1)
    arr = (Region * n)()
    cnt = lib().orc_split_region(ctypes.byref(reg), D, n, arr)
    return [region_tuple(arr[i], D) for i in range(cnt)]


def cast_f32_to_u8(a):
    """|p: f32| p.round().clamp(0.0, 255.0) as u8 (tests/blur_png.rs:40)."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    out = np.empty(a.shape, dtype=np.uint8)
    lib().orc_cast_f32_to_u8(_ptr(a), _ptr(out), a.size)
    return out


# ---------------------------------------------------------------------------
# FP64 numpy helpers for the adjoint (not in the reference: the reference has
# no VJP).  Per-axis clamped convolution as an explicit linear operator.
# ---------------------------------------------------------------------------

def _np_axis(D: int, axis: int) -> int:
    """numpy axis of reference axis `axis` for an array of D spatial dims."""
    return D - 1 - axis


def conv_axis_f64(x: np.ndarray, w: np.ndarray, axis: int, D: int) -> np.ndarray:
    """y[o] = sum_k w[k] x[clamp(o+k-r)] along reference axis `axis` (whole image)."""
    ax = _np_axis(D, axis)
    n = x.shape[ax]
    r = (len(w) - 1) // 2
    y = np.zeros(x.shape, dtype=np.float64)
    o = np.arange(n)
    for k in range(len(w)):
        idx = np.clip(o + k - r, 0, n - 1)
        y += w[k] * np.take(x, idx, axis=ax)
    return y


def conv_axis_adjoint_f64(g: np.ndarray, w: np.ndarray, axis: int, D: int) -> np.ndarray:
    """Transpose of conv_axis_f64: scatter-add through the same clamped index map."""
    ax = _np_axis(D, axis)
    n = g.shape[ax]
    r = (len(w) - 1) // 2
    xb = np.zeros(g.shape, dtype=np.float64)
    o = np.arange(n)
    gm = np.moveaxis(g, ax, 0)
    xm = np.moveaxis(xb, ax, 0)
    for k in range(len(w)):
        idx = np.clip(o + k - r, 0, n - 1)
        np.add.at(xm, idx, w[k] * gm)
    return xb


def kernel_and_derivative(sigma: float, spacing: float, radius: int | None = None):
    """f64 weights w_i and dw_i/dsigma (physical sigma) at a frozen radius."""
    sp = float(spacing)
    s = sigma / sp
    r = kernel_radius(sigma, sp) if radius is None else int(radius)
    x = np.arange(-r, r + 1, dtype=np.float64)
    g = np.exp(-0.5 * (x / s) ** 2)
    gp = g * x * x / s ** 3          # dg/dsigma_px
    S = g.sum()
    Sp = gp.sum()
    w = g / S
    dw = (gp * S - g * Sp) / (S * S) / sp
    return w, dw


def gaussian_whole_f64(x: np.ndarray, sigma: float, spacing=None, radii=None):
    """FP64 whole-image forward with optional frozen radii (scalar pixels)."""
    D = x.ndim
    spacing = spacing or [1.0] * D
    y = x.astype(np.float64)
    for a in range(D):
        r = None if radii is None else radii[a]
        w, _ = kernel_and_derivative(sigma, spacing[a], r)
        y = conv_axis_f64(y, w, a, D)
    return y


def gaussian_adjoint_f64(g: np.ndarray, sigma: float, spacing=None, radii=None):
    """x_bar = G_0^T ... G_{D-1}^T g (FP64)."""
    D = g.ndim
    spacing = spacing or [1.0] * D
    xb = g.astype(np.float64)
    for a in reversed(range(D)):
        r = None if radii is None else radii[a]
        w, _ = kernel_and_derivative(sigma, spacing[a], r)
        xb = conv_axis_adjoint_f64(xb, w, a, D)
    return xb


def gaussian_dsigma_f64(x: np.ndarray, sigma: float, spacing=None, radii=None):
    """dy/dsigma = sum_a (prod_{b!=a} G_b) dG_a x (FP64, frozen radii)."""
    D = x.ndim
    spacing = spacing or [1.0] * D
    total = np.zeros(x.shape, dtype=np.float64)
    for a in range(D):
        y = x.astype(np.float64)
        for b in range(D):
            r = None if radii is None else radii[b]
            w, dw = kernel_and_derivative(sigma, spacing[b], r)
            y = conv_axis_f64(y, dw if b == a else w, b, D)
        total += y
    return total


# ---- Gaussian callers that iterate around it (C core) ------------------------

def demons(fixed, moving, iterations, max_step_length=2.0, fixed_index=(0, 0), moving_index=(0, 0)):
    """DemonsRegistrationFilter::compute (registration_methods.rs:39-100): the
    f64 displacement (dx, dy) arrays, shape of `fixed`.  Raises where the
    reference panics (a warped index outside the moving image)."""
    f = np.ascontiguousarray(fixed, dtype=np.float32)
    m = np.ascontiguousarray(moving, dtype=np.float32)
    freg = make_region(fixed_index, (f.shape[1], f.shape[0]))
    mreg = make_region(moving_index, (m.shape[1], m.shape[0]))
    dx = np.zeros(f.shape, np.float64)
    dy = np.zeros(f.shape, np.float64)
    rc = lib().orc_demons_f64(_ptr(f), ctypes.byref(freg), _ptr(m), ctypes.byref(mreg), int(iterations),
                              float(max_step_length), _ptr(dx), _ptr(dy))
    if rc != 0:
        raise IndexError("demons: a warped index left the moving image (the reference panics)")
    return dx, dy


def demons_f32(fixed, moving, iterations, max_step_length=2.0, **kw):
    """The VecPixel<f32, 2> field the reference returns: shape (h, w, 2)."""
    dx, dy = demons(fixed, moving, iterations, max_step_length, **kw)
    return np.stack([dx.astype(np.float32), dy.astype(np.float32)], axis=-1)


def diffeomorphic_demons(fixed, moving, iterations, sigma_diff=1.0, spacing=None, **kw):
    """DiffeomorphicDemonsRegistrationFilter::compute (registration_methods.rs:126-148):
    the f32 demons field, each component smoothed by GaussianFilter { sigma_diff }."""
    field = demons_f32(fixed, moving, iterations, **kw)
    index = kw.get("fixed_index", (0, 0))
    sx = gaussian_f32(field[..., 0], sigma_diff, spacing=spacing, index=index)
    sy = gaussian_f32(field[..., 1], sigma_diff, spacing=spacing, index=index)
    return np.stack([sx, sy], axis=-1)


def n4(img, iterations=4, sigma=30.0, threshold=1e-3, spacing=None, index=(0, 0)):
    """N4BiasFieldCorrectionFilter::generate_region (bias_correction.rs:45-83):
    (the corrected f32 image, the number of iterations run)."""
    a = np.ascontiguousarray(img, dtype=np.float32)
    reg = make_region(index, (a.shape[1], a.shape[0]))
    sp = np.ascontiguousarray(spacing if spacing is not None else [1.0, 1.0], dtype=np.float64)
    out = np.empty_like(a)
    run = lib().orc_n4_f32(_ptr(a), ctypes.byref(reg), _ptr(sp), int(iterations), float(sigma), float(threshold),
                           _ptr(out))
    if run < 0:
        raise RuntimeError("oracle: n4 failed")
    return out, run
