"""Python mirror of itk-rs's Gaussian pipeline API over the itkg C ABI.

Mirrors (reference file:line):
  Region.padded_per_axis / clipped_to   src/image.rs:28-64
  Image (host buffer, axis 0 fastest)   src/image.rs:82-141
  ImageSource protocol                  src/source.rs:13-29 (+ Image leaf, 32-59)
  GaussianFilter(source, sigma)         src/filters/gaussian.rs:13-91
  UnaryFilter casts around the filter   src/filters/mod.rs:47-81,
                                        examples/blur_png.rs:35-37
  stream_full(source, num_pieces)       src/source.rs:81-98
  split_region(region, num_pieces)      src/region_splitter.rs:17-48

Numpy convention: a D-dimensional image is a C-ordered array whose LAST
spatial axis is the reference's axis 0 (shape (nz, ny, nx)), plus a trailing
component axis of length 3 for VecPixel<_, 3>.  Every filter call goes through
libitkg.so; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from ._abi import (ALGO_AUTO, ALGO_FUSED, ALGO_ONE_TRIP, ALGO_PER_AXIS, ALGO_TWO_PASS, ARITH_F32, ARITH_PIXEL_U8, BF16,
                   DEVICE, F16, F32, HOST, I16, ROUND_FMA, ROUND_REFERENCE, U8, ItkgError, check,
                   itkg_gaussian_params, itkg_image, itkg_recursive_derivative_params, itkg_recursive_params,
                   itkg_region, itkg_separable_params, itkg_unsharp_params, lib)

__all__ = [
    "Region", "Image", "DeviceImage", "GaussianFilter", "CastFilter", "stream_full",
    "split_region", "kernel_radius", "build_kernel", "ItkgError", "F32", "I16", "U8", "BF16",
    "F16", "ROUND_REFERENCE", "ROUND_FMA", "ALGO_AUTO", "ALGO_FUSED", "ALGO_PER_AXIS",
    "ALGO_TWO_PASS", "ALGO_ONE_TRIP", "ARITH_F32", "ARITH_PIXEL_U8", "gaussian", "Stream", "SeparableFilter",
    "MeanFilter", "BoxMeanFilterN", "BinomialBlurFilter", "box_kernel", "BINOMIAL_KERNEL",
    "RecursiveGaussianFilter", "RecursiveGaussianAxisFilter", "yvv_coeffs", "RecursiveGaussianDerivativeFilter",
    "GradientMagnitudeRecursiveGaussianFilter", "LaplacianRecursiveGaussianFilter",
    "DiscreteGaussianDerivativeFilter", "GradientRecursiveGaussianFilter", "HessianRecursiveGaussianFilter",
    "DifferenceOfGaussiansFilter", "UnsharpMaskFilter", "unsharp_kernel", "ZeroCrossingBasedEdgeDetectionFilter",
    "SliceBySliceFilter", "DisplacementFieldToBSplineFilter", "BSplineDownsampleFilter", "DemonsRegistrationFilter",
    "DiffeomorphicDemonsRegistrationFilter", "SyNRegistrationMethod", "N4BiasFieldCorrectionFilter",
    "MRIBiasFieldCorrectionFilter",
]

_NP_OF = {F32: np.float32, I16: np.int16, U8: np.uint8, F16: np.float16}


def dtype_code(np_dtype, bf16: bool = False) -> int:
    if bf16:
        return BF16
    d = np.dtype(np_dtype)
    for code, t in _NP_OF.items():
        if d == np.dtype(t):
            return code
    raise TypeError(f"unsupported pixel dtype {d}")


def _storage_np(code: int):
    """numpy dtype used to hold a storage type on the host (bf16 as uint16 bits)."""
    return np.uint16 if code == BF16 else _NP_OF[code]


# ---------------------------------------------------------------------------
# Region (image.rs:12-77)
# ---------------------------------------------------------------------------
@dataclass(frozen=True)
class Region:
    index: tuple
    size: tuple

    @property
    def dim(self) -> int:
        return len(self.size)

    def linear_len(self) -> int:
        n = 1
        for s in self.size:
            n *= int(s)
        return n

    def padded_per_axis(self, radii) -> "Region":
        return Region(tuple(i - r for i, r in zip(self.index, radii)),
                      tuple(s + 2 * r for s, r in zip(self.size, radii)))

    def clipped_to(self, bounds: "Region") -> "Region":
        idx, sz = [], []
        for i, s, bi, bs in zip(self.index, self.size, bounds.index, bounds.size):
            st, en = max(i, bi), min(i + s, bi + bs)
            idx.append(st)
            sz.append(max(en - st, 0))
        return Region(tuple(idx), tuple(sz))

    def contains(self, idx) -> bool:
        return all(i <= x < i + s for i, s, x in zip(self.index, self.size, idx))

    def to_c(self) -> itkg_region:
        r = itkg_region()
        for d in range(3):
            r.index[d] = int(self.index[d]) if d < self.dim else 0
            r.size[d] = int(self.size[d]) if d < self.dim else 1
        return r

    @staticmethod
    def from_c(r: itkg_region, dim: int) -> "Region":
        return Region(tuple(r.index[d] for d in range(dim)), tuple(r.size[d] for d in range(dim)))


def kernel_radius(sigma: float, spacing: float) -> int:
    """GaussianFilter::kernel_radius (gaussian.rs:24-27)."""
    return int(lib().itkg_kernel_radius(float(sigma), float(spacing)))


def build_kernel(sigma_px: float, radius: int) -> np.ndarray:
    """GaussianFilter::build_kernel (gaussian.rs:29-40)."""
    out = np.zeros(2 * radius + 1, dtype=np.float64)
    check(lib().itkg_build_kernel(float(sigma_px), int(radius), out.ctypes.data_as(ctypes.c_void_p)))
    return out


def split_region(region: Region, num_pieces: int):
    """split_region (region_splitter.rs:17-48)."""
    c = region.to_c()
    cnt = ctypes.c_uint64(0)
    check(lib().itkg_split_region(ctypes.byref(c), region.dim, int(num_pieces), None, 0,
                                  ctypes.byref(cnt)))
    arr = (itkg_region * max(cnt.value, 1))()
    check(lib().itkg_split_region(ctypes.byref(c), region.dim, int(num_pieces), arr, cnt.value,
                                  ctypes.byref(cnt)))
    return [Region.from_c(arr[i], region.dim) for i in range(cnt.value)]


class Stream:
    """Opaque cudaStream_t handle (an int); 0 is the legacy default stream."""

    def __init__(self, handle: int = 0):
        self.handle = int(handle)

    @property
    def ptr(self):
        return ctypes.c_void_p(self.handle) if self.handle else None

    def synchronize(self):
        check(lib().itkg_stream_synchronize(self.ptr))


_DEFAULT_STREAM = Stream(0)


# ---------------------------------------------------------------------------
# Images
# ---------------------------------------------------------------------------
class Image:
    """Host image: Image<P, D> (image.rs:82-141) backed by a numpy array."""

    def __init__(self, data: np.ndarray, index=None, spacing=None, origin=None, components=1,
                 bf16: bool = False):
        self.data = np.ascontiguousarray(data)
        self.components = components
        spatial = self.data.shape[:-1] if components > 1 else self.data.shape
        D = len(spatial)
        self.region = Region(tuple(index) if index is not None else (0,) * D,
                             tuple(reversed(spatial)))
        self.spacing = tuple(spacing) if spacing is not None else (1.0,) * D
        self.origin = tuple(origin) if origin is not None else (0.0,) * D
        self.dtype = dtype_code(self.data.dtype, bf16)

    @property
    def dim(self):
        return self.region.dim

    # Image acts as an ImageSource leaf (source.rs:32-59)
    def largest_region(self) -> Region:
        return self.region

    def to_c(self) -> itkg_image:
        im = itkg_image()
        im.dim = self.dim
        im.dtype = self.dtype
        im.components = self.components
        im.location = HOST
        im.region = self.region.to_c()
        isz = self.data.itemsize * self.components
        pitches = [isz]
        for d in range(1, self.dim):
            pitches.append(pitches[-1] * self.region.size[d - 1])
        for d in range(3):
            im.pitch[d] = pitches[d] if d < self.dim else pitches[-1] * int(self.region.size[-1])
            im.spacing[d] = self.spacing[d] if d < self.dim else 1.0
            im.origin[d] = self.origin[d] if d < self.dim else 0.0
        im.data = self.data.ctypes.data
        return im

    def get_pixel(self, idx):
        local = tuple(i - o for i, o in zip(idx, self.region.index))
        return self.data[tuple(reversed(local))]


class DeviceImage:
    """Device-resident image (pitched rows, 128-byte aligned) owned by libitkg."""

    def __init__(self, region: Region, dtype: int = F32, components: int = 1, spacing=None,
                 origin=None):
        D = region.dim
        self.c = itkg_image()
        sp = (ctypes.c_double * 3)(*([float(s) for s in (spacing or (1.0,) * D)] + [1.0] * (3 - D)))
        org = (ctypes.c_double * 3)(*([float(s) for s in (origin or (0.0,) * D)] + [0.0] * (3 - D)))
        r = region.to_c()
        check(lib().itkg_image_alloc_device(ctypes.byref(self.c), D, dtype, components,
                                            ctypes.byref(r), sp, org))
        self.region = region
        self.components = components
        self.dtype = dtype
        self.spacing = tuple(spacing or (1.0,) * D)
        self.origin = tuple(origin or (0.0,) * D)

    @property
    def dim(self):
        return self.region.dim

    def largest_region(self) -> Region:
        return self.region

    def to_c(self) -> itkg_image:
        return self.c

    def __del__(self):
        try:
            if self.c.data:
                lib().itkg_image_free(ctypes.byref(self.c))
        except Exception:
            pass

    @classmethod
    def from_host(cls, img: Image, stream: Stream = _DEFAULT_STREAM) -> "DeviceImage":
        dev = cls(img.region, img.dtype, img.components, img.spacing, img.origin)
        dev.upload(img.data, stream)
        return dev

    def _host_view(self, arr):
        arr = np.ascontiguousarray(arr)
        h = Image.__new__(Image)
        h.data = arr
        h.components = self.components
        h.region = self.region
        h.spacing = self.spacing
        h.origin = self.origin
        h.dtype = self.dtype
        return h

    def upload(self, arr: np.ndarray, stream: Stream = _DEFAULT_STREAM):
        """Copy a dense host array (same shape as the region) into the pitched buffer."""
        self._copy(self._host_view(arr), to_device=True, stream=stream)

    def download(self, stream: Stream = _DEFAULT_STREAM) -> np.ndarray:
        shape = tuple(reversed(self.region.size)) + ((self.components,) if self.components > 1 else ())
        out = np.empty(shape, dtype=_storage_np(self.dtype))
        self._copy(self._host_view(out), to_device=False, stream=stream)
        return out

    def _copy(self, host: Image, to_device: bool, stream: Stream):
        # Image::copy_from (image.rs:133-140) through the C ABI.
        hc = host.to_c()
        if to_device:
            check(lib().itkg_image_copy_from(ctypes.byref(self.c), ctypes.byref(hc), stream.ptr))
        else:
            check(lib().itkg_image_copy_from(ctypes.byref(hc), ctypes.byref(self.c), stream.ptr))
        stream.synchronize()


# ---------------------------------------------------------------------------
# Filters
# ---------------------------------------------------------------------------
class CastFilter:
    """UnaryFilter(|p| p as f32) in front of the Gaussian, or the output cast
    |p: f32| p.round().clamp(0,255) as u8 behind it (examples/blur_png.rs:35-37).
    The GPU fuses either cast into the Gaussian's load or store, so a CastFilter
    only records the storage type it converts to."""

    def __init__(self, source, to_dtype: int):
        self.source = source
        self.to_dtype = to_dtype

    def largest_region(self):
        return self.source.largest_region()

    @property
    def spacing(self):
        return self.source.spacing

    @property
    def origin(self):
        return self.source.origin

    def generate_region(self, requested: Region, stream: Stream = _DEFAULT_STREAM):
        src = self.source
        if isinstance(src, GaussianFilter):
            return src.generate_region(requested, stream=stream, out_dtype=self.to_dtype)
        raise TypeError("CastFilter output is consumed by GaussianFilter (fused load)")


class GaussianFilter:
    """GaussianFilter { source, sigma } (gaussian.rs:13-91) on the GPU."""

    def __init__(self, source, sigma: float, rounding: int = ROUND_REFERENCE,
                 algorithm: int = ALGO_AUTO, arithmetic: int | None = None):
        self.source = source
        self.sigma = float(sigma)
        self.rounding = rounding
        self.algorithm = algorithm
        self.arithmetic = arithmetic

    def _leaf(self):
        src = self.source
        if isinstance(src, CastFilter):
            src = src.source
        if not isinstance(src, (Image, DeviceImage)):
            raise TypeError("GaussianFilter source must be an Image, DeviceImage or CastFilter of one")
        return src

    def largest_region(self) -> Region:
        return self.source.largest_region()

    @property
    def spacing(self):
        return self._leaf().spacing

    @property
    def origin(self):
        return self._leaf().origin

    def input_region_for_output(self, out: Region) -> Region:
        radii = [kernel_radius(self.sigma, s) for s in self.spacing]
        return out.padded_per_axis(radii).clipped_to(self.largest_region())

    def params(self) -> itkg_gaussian_params:
        p = itkg_gaussian_params()
        p.sigma = self.sigma
        leaf = self._leaf()
        if self.arithmetic is not None:
            p.arithmetic = self.arithmetic
        else:
            # GaussianFilter directly over Image<u8> uses u8 pixel arithmetic;
            # through a cast node it is f32 arithmetic.
            p.arithmetic = ARITH_PIXEL_U8 if (leaf.dtype == U8 and not isinstance(self.source, CastFilter)) else ARITH_F32
        p.rounding = self.rounding
        p.algorithm = self.algorithm
        return p

    def generate_region(self, requested: Region, stream: Stream = _DEFAULT_STREAM,
                        out_dtype: int | None = None, out=None):
        """Returns a host Image for a host source, a DeviceImage for a device source."""
        leaf = self._leaf()
        prm = self.params()
        if out_dtype is None:
            out_dtype = U8 if prm.arithmetic == ARITH_PIXEL_U8 else F32
        largest = leaf.largest_region().to_c()
        req = requested.to_c()
        src = leaf.to_c()
        if isinstance(leaf, Image):
            shape = tuple(reversed(requested.size)) + ((leaf.components,) if leaf.components > 1 else ())
            host = out if out is not None else np.empty(shape, dtype=_storage_np(out_dtype))
            res = Image(host, index=requested.index, spacing=leaf.spacing, origin=leaf.origin,
                        components=leaf.components, bf16=(out_dtype == BF16))
            oc = res.to_c()
            self._call(src, largest, req, oc, stream)
            return res
        dev = out if out is not None else DeviceImage(requested, out_dtype, leaf.components,
                                                      leaf.spacing, leaf.origin)
        self._call(src, largest, req, dev.c, stream)
        return dev

    def _call(self, src, largest, req, out_c, stream):
        prm = self.params()
        check(lib().itkg_gaussian_generate_region(ctypes.byref(src), ctypes.byref(largest), ctypes.byref(req),
                                                  ctypes.byref(prm), ctypes.byref(out_c), stream.ptr))


BINOMIAL_KERNEL = np.array([0.25, 0.5, 0.25])  # binomial_blur.rs:35


def box_kernel(radius: int) -> np.ndarray:
    """box_kernel (mean.rs:15-18): 2r + 1 weights of 1 / (2r + 1)."""
    out = np.empty(2 * int(radius) + 1, dtype=np.float64)
    check(lib().itkg_box_kernel(int(radius), out.ctypes.data))
    return out


class SeparableFilter(GaussianFilter):
    """A filter of the convolve_axis family with explicit f64 kernels per axis
    (reference axis order) and `repetitions` rounds of one pass per axis: the
    engine of MeanFilter, BoxMeanFilterN and BinomialBlurFilter, and of the
    Gaussian stages of UnsharpMaskFilter / CannyEdgeDetectionFilter
    (edges.rs:406-430, 562-577), which build their own kernels."""

    def __init__(self, source, kernels, repetitions: int = 1, rounding: int = ROUND_REFERENCE,
                 algorithm: int = ALGO_AUTO, arithmetic: int | None = None):
        super().__init__(source, 0.0, rounding, algorithm, arithmetic)
        self.kernels = [np.ascontiguousarray(k, dtype=np.float64) for k in kernels]
        if any(k.ndim != 1 or len(k) % 2 != 1 for k in self.kernels):
            raise ValueError("each kernel is a 1-D array of odd length")
        self.repetitions = int(repetitions)

    @property
    def radii(self):
        return [(len(k) - 1) // 2 for k in self.kernels]

    def input_region_for_output(self, out: Region) -> Region:
        return out.padded_per_axis([r * self.repetitions for r in self.radii]).clipped_to(
            self.largest_region())

    def separable_params(self) -> itkg_separable_params:
        g = self.params()
        p = itkg_separable_params()
        if len(self.kernels) != len(self.largest_region().size):
            raise ValueError("one kernel per axis")
        for d, k in enumerate(self.kernels):
            p.radius[d] = (len(k) - 1) // 2
            p.weights[d] = k.ctypes.data
        p.repetitions = self.repetitions
        p.arithmetic, p.rounding, p.algorithm = g.arithmetic, g.rounding, g.algorithm
        return p

    def _call(self, src, largest, req, out_c, stream):
        prm = self.separable_params()
        check(lib().itkg_separable_generate_region(ctypes.byref(src), ctypes.byref(largest), ctypes.byref(req),
                                                   ctypes.byref(prm), ctypes.byref(out_c), stream.ptr))


class MeanFilter(SeparableFilter):
    """MeanFilter { source, radius } (mean.rs:27-84)."""

    def __init__(self, source, radius: int, **kw):
        D = len(source.largest_region().size)
        super().__init__(source, [box_kernel(radius)] * D, 1, **kw)
        self.radius = int(radius)


class BoxMeanFilterN(SeparableFilter):
    """BoxMeanFilterN { source, radii } (mean.rs:103-137), radii in reference axis order."""

    def __init__(self, source, radii, **kw):
        super().__init__(source, [box_kernel(r) for r in radii], 1, **kw)


class BinomialBlurFilter(SeparableFilter):
    """BinomialBlurFilter { source, repetitions } (binomial_blur.rs:17-89)."""

    def __init__(self, source, repetitions: int, **kw):
        D = len(source.largest_region().size)
        super().__init__(source, [BINOMIAL_KERNEL] * D, repetitions, **kw)

    @staticmethod
    def effective_sigma_pixels(repetitions: int) -> float:
        """binomial_blur.rs:28-30"""
        return (repetitions / 4.0) ** 0.5


class SliceBySliceFilter(GaussianFilter):
    """SliceBySliceFilter { source, sigma } (spatial.rs:1284-1340): a 2-D GaussianFilter on every
    z slice of the request, clamped to the request's x-y window; 3-D only."""

    def input_region_for_output(self, out: Region) -> Region:
        return out  # the reference asks its source for the request itself (spatial.rs:1305)

    def _call(self, src, largest, req, out_c, stream):
        prm = self.params()
        check(lib().itkg_slice_by_slice_generate_region(ctypes.byref(src), ctypes.byref(req), ctypes.byref(prm),
                                                        ctypes.byref(out_c), stream.ptr))


class DisplacementFieldToBSplineFilter(GaussianFilter):
    """DisplacementFieldToBSplineFilter { source, sigma } (spatial.rs:1484-1525), sigma 2.0 by
    default: each component of a 2-D VecPixel<f32, 2> field smoothed by GaussianFilter { sigma }.
    The reference smooths the source's generated request as an image of its own, so the request
    is also the Gaussian's largest region (its taps clamp at the request's edges)."""

    def __init__(self, source, sigma: float = 2.0, rounding: int = ROUND_REFERENCE, algorithm: int = ALGO_AUTO):
        super().__init__(source, sigma, rounding, algorithm)

    def input_region_for_output(self, out: Region) -> Region:
        return out  # the reference asks its source for the request itself (spatial.rs:1509)

    def _call(self, src, largest, req, out_c, stream):
        prm = self.params()
        check(lib().itkg_gaussian_generate_region(ctypes.byref(src), ctypes.byref(req), ctypes.byref(req),
                                                  ctypes.byref(prm), ctypes.byref(out_c), stream.ptr))


class BSplineDownsampleFilter(GaussianFilter):
    """BSplineDownsampleFilter { source } (spatial.rs:1128-1166): GaussianFilter sigma 1.0 over the
    whole largest region, then every other voxel.  largest_region() is the downsampled region;
    generate_region returns all of it whatever is requested, as the reference does."""

    def __init__(self, source, rounding: int = ROUND_REFERENCE, algorithm: int = ALGO_AUTO,
                 arithmetic: int | None = None):
        super().__init__(source, 1.0, rounding, algorithm, arithmetic)

    def largest_region(self) -> Region:
        r = self.source.largest_region()
        return Region(tuple(r.index), tuple((n + 1) // 2 for n in r.size))

    @property
    def spacing(self):
        return tuple(2.0 * v for v in self._leaf().spacing)

    def input_region_for_output(self, out: Region) -> Region:
        return self.source.largest_region()

    def generate_region(self, requested: Region = None, stream: Stream = _DEFAULT_STREAM, out_dtype: int | None = None):
        leaf = self._leaf()
        prm = self.params()
        if out_dtype is None:
            out_dtype = U8 if prm.arithmetic == ARITH_PIXEL_U8 else F32
        half = self.largest_region()
        largest = leaf.largest_region().to_c()
        src = leaf.to_c()
        if isinstance(leaf, Image):
            shape = tuple(reversed(half.size)) + ((leaf.components,) if leaf.components > 1 else ())
            res = Image(np.empty(shape, dtype=_storage_np(out_dtype)), index=half.index, spacing=self.spacing,
                        origin=leaf.origin, components=leaf.components)
            oc = res.to_c()
        else:
            res = DeviceImage(half, out_dtype, leaf.components, self.spacing, leaf.origin)
            oc = res.c
        check(lib().itkg_bspline_downsample_generate_region(ctypes.byref(src), ctypes.byref(largest),
                                                            ctypes.byref(prm), ctypes.byref(oc), stream.ptr))
        return res


def _image_leaf(src):
    if isinstance(src, (Image, DeviceImage)):
        return src
    raise TypeError("the source must be an Image or a DeviceImage")


class DemonsRegistrationFilter:
    """DemonsRegistrationFilter { fixed, moving, iterations, max_step_length }
    (registration_methods.rs:20-100): compute() returns the displacement field
    (in pixels) of the fixed image's region as a 2-component f32 image
    (VecPixel<f32, 2>): an Image for host sources, a DeviceImage for device ones."""

    _diffeomorphic = 0

    def __init__(self, fixed, moving, iterations: int, max_step_length: float = 2.0):
        self.fixed, self.moving = fixed, moving
        self.iterations = int(iterations)
        self.max_step_length = float(max_step_length)
        self.sigma_diff = 1.0

    def compute(self, stream: Stream = _DEFAULT_STREAM):
        f, m = _image_leaf(self.fixed), _image_leaf(self.moving)
        reg = f.region
        if isinstance(f, Image):
            res = Image(np.empty(tuple(reversed(reg.size)) + (2,), np.float32), index=reg.index, spacing=f.spacing,
                        origin=f.origin, components=2)
            oc = res.to_c()
        else:
            res = DeviceImage(reg, F32, 2, f.spacing, f.origin)
            oc = res.c
        fc, mc = f.to_c(), m.to_c()
        check(lib().itkg_demons_registration(ctypes.byref(fc), ctypes.byref(mc), self.iterations,
                                             self.max_step_length, self._diffeomorphic, float(self.sigma_diff),
                                             ctypes.byref(oc), stream.ptr))
        return res


class DiffeomorphicDemonsRegistrationFilter(DemonsRegistrationFilter):
    """DiffeomorphicDemonsRegistrationFilter { fixed, moving, iterations, sigma_diff }
    (registration_methods.rs:108-148): the demons field (max step 2.0), each
    component smoothed by GaussianFilter { sigma: sigma_diff }."""

    _diffeomorphic = 1

    def __init__(self, fixed, moving, iterations: int, sigma_diff: float = 1.0):
        super().__init__(fixed, moving, iterations)
        self.sigma_diff = float(sigma_diff)


class SyNRegistrationMethod(DiffeomorphicDemonsRegistrationFilter):
    """SyNRegistrationMethod { fixed, moving, iterations, sigma } (registration_methods.rs:193-218):
    the diffeomorphic demons with the sum of its iteration counts (its `sigma`
    is not read by the reference either; the smoothing uses sigma_diff 1.0)."""

    def __init__(self, fixed, moving, iterations=(20, 10, 5), sigma: float = 1.0):
        super().__init__(fixed, moving, sum(int(i) for i in iterations))
        self.sigma = float(sigma)


class N4BiasFieldCorrectionFilter:
    """N4BiasFieldCorrectionFilter { source, iterations, sigma, convergence_threshold }
    (bias_correction.rs:23-83): generate_region ignores the request and returns the
    corrected image of the whole largest region (f32).  iterations_run is set by
    each call."""

    def __init__(self, source, iterations: int = 4, sigma: float = 30.0, convergence_threshold: float = 1e-3):
        self.source = source
        self.iterations = int(iterations)
        self.sigma = float(sigma)
        self.convergence_threshold = float(convergence_threshold)
        self.iterations_run = None

    def largest_region(self) -> Region:
        return self.source.largest_region()

    @property
    def spacing(self):
        return _image_leaf(self.source).spacing

    @property
    def origin(self):
        return _image_leaf(self.source).origin

    def generate_region(self, requested: Region = None, stream: Stream = _DEFAULT_STREAM):
        leaf = _image_leaf(self.source)
        reg = leaf.largest_region()
        if isinstance(leaf, Image):
            res = Image(np.empty(tuple(reversed(reg.size)), np.float32), index=reg.index, spacing=leaf.spacing,
                        origin=leaf.origin)
            oc = res.to_c()
        else:
            res = DeviceImage(reg, F32, 1, leaf.spacing, leaf.origin)
            oc = res.c
        src, lg = leaf.to_c(), reg.to_c()
        run = ctypes.c_int32(0)
        check(lib().itkg_n4_bias_field_correction(ctypes.byref(src), ctypes.byref(lg), self.iterations, self.sigma,
                                                  self.convergence_threshold, ctypes.byref(oc), ctypes.byref(run),
                                                  stream.ptr))
        self.iterations_run = run.value
        return res


class MRIBiasFieldCorrectionFilter(N4BiasFieldCorrectionFilter):
    """MRIBiasFieldCorrectionFilter { source, polynomial_degree, iterations }
    (bias_correction.rs:92-121): N4 with sigma 20 and threshold 1e-3."""

    def __init__(self, source, polynomial_degree: int = 2, iterations: int = 3):
        super().__init__(source, iterations, 20.0, 1e-3)
        self.polynomial_degree = int(polynomial_degree)


def unsharp_kernel(sigma: float) -> np.ndarray:
    """UnsharpMaskFilter's blur kernel (edges.rs:408, 415-424): 2 ceil(3 sigma) + 1 weights."""
    r = ctypes.c_uint64()
    check(lib().itkg_unsharp_kernel(float(sigma), ctypes.byref(r), None, 0))
    out = np.empty(2 * r.value + 1, dtype=np.float64)
    check(lib().itkg_unsharp_kernel(float(sigma), ctypes.byref(r), out.ctypes.data, len(out)))
    return out


class UnsharpMaskFilter(GaussianFilter):
    """UnsharpMaskFilter { source, sigma, amount, threshold } (edges.rs:374-452):
    I + amount (I - blur(I)) where |I - blur(I)| > threshold, over Image<f32> or
    Image<u8> (and their 3-component vector pixels); sigma in pixels on every axis."""

    def __init__(self, source, sigma: float, amount: float = 0.5, threshold: float = 0.0,
                 rounding: int = ROUND_REFERENCE):
        if not isinstance(source, (Image, DeviceImage)):
            raise TypeError("UnsharpMaskFilter source must be an Image or a DeviceImage")
        super().__init__(source, sigma, rounding)
        self.amount = float(amount)
        self.threshold = float(threshold)

    def with_amount(self, a: float) -> "UnsharpMaskFilter":
        self.amount = float(a)
        return self

    def input_region_for_output(self, out: Region) -> Region:
        r = (len(unsharp_kernel(self.sigma)) - 1) // 2
        return out.padded_per_axis([r] * len(out.size)).clipped_to(self.largest_region())

    def unsharp_params(self) -> itkg_unsharp_params:
        p = itkg_unsharp_params()
        p.sigma, p.amount, p.threshold, p.rounding = self.sigma, self.amount, self.threshold, self.rounding
        return p

    def _call(self, src, largest, req, out_c, stream):
        prm = self.unsharp_params()
        check(lib().itkg_unsharp_mask_generate_region(ctypes.byref(src), ctypes.byref(largest), ctypes.byref(req),
                                                      ctypes.byref(prm), ctypes.byref(out_c), stream.ptr))


def yvv_coeffs(sigma: float) -> np.ndarray:
    """(B, a1, a2, a3) of recursive_gaussian.rs:33-49, sigma in pixels."""
    out = np.empty(4, dtype=np.float64)
    check(lib().itkg_yvv_coeffs(float(sigma), out.ctypes.data))
    return out


class RecursiveGaussianFilter:
    """RecursiveGaussianFilter { source, sigma } (recursive_gaussian.rs:133-181); with
    `axis` set, RecursiveGaussianAxisFilter { source, sigma, axis } (183-239).
    Filters the whole largest region; the source must be an Image or DeviceImage."""

    def __init__(self, source, sigma: float, axis: int | None = None, rounding: int = ROUND_REFERENCE):
        if not isinstance(source, (Image, DeviceImage)):
            raise TypeError("source must be an Image or a DeviceImage")
        self.source = source
        self.sigma = float(sigma)
        self.axis = -1 if axis is None else int(axis)
        self.rounding = rounding

    def largest_region(self) -> Region:
        return self.source.largest_region()

    def input_region_for_output(self, out: Region) -> Region:
        return self.largest_region()

    def params(self) -> itkg_recursive_params:
        p = itkg_recursive_params()
        p.sigma, p.axis, p.rounding = self.sigma, self.axis, self.rounding
        return p

    def generate_region(self, requested: Region, stream: Stream = _DEFAULT_STREAM, out_dtype: int | None = None):
        """Returns a host Image for a host source, a DeviceImage for a device source."""
        src = self.source
        if out_dtype is None:
            out_dtype = U8 if src.dtype == U8 else F32
        prm = self.params()
        largest = src.largest_region().to_c()
        req = requested.to_c()
        sc = src.to_c()
        if isinstance(src, Image):
            host = np.empty(tuple(reversed(requested.size)), dtype=_storage_np(out_dtype))
            res = Image(host, index=requested.index, spacing=src.spacing, origin=src.origin)
            oc = res.to_c()
            check(lib().itkg_recursive_gaussian_generate_region(ctypes.byref(sc), ctypes.byref(largest),
                                                                ctypes.byref(req), ctypes.byref(prm),
                                                                ctypes.byref(oc), stream.ptr))
            return res
        dev = DeviceImage(requested, out_dtype, 1, src.spacing, src.origin)
        check(lib().itkg_recursive_gaussian_generate_region(ctypes.byref(sc), ctypes.byref(largest),
                                                            ctypes.byref(req), ctypes.byref(prm),
                                                            ctypes.byref(dev.c), stream.ptr))
        return dev


class RecursiveGaussianAxisFilter(RecursiveGaussianFilter):
    """RecursiveGaussianAxisFilter { source, sigma, axis } (recursive_gaussian.rs:183-239)."""

    def __init__(self, source, sigma: float, axis: int, rounding: int = ROUND_REFERENCE):
        super().__init__(source, sigma, axis, rounding)


REC_GRADIENT_MAGNITUDE, REC_LAPLACIAN, REC_DERIVATIVE, REC_GRADIENT, REC_HESSIAN, REC_DOG, REC_ZERO_CROSSING = range(7)


class RecursiveGaussianDerivativeFilter(RecursiveGaussianFilter):
    """The derivative users of RecursiveGaussianFilter (edges.rs:686-950): the
    smoothed requested region, then a central-difference stencil of `kind`."""

    def __init__(self, source, sigma: float, kind: int, axis: int = 0, order: int = 1,
                 rounding: int = ROUND_REFERENCE, sigma2: float = 0.0):
        super().__init__(source, sigma, None, rounding)
        self.kind, self.deriv_axis, self.order, self.sigma2 = int(kind), int(axis), int(order), float(sigma2)

    def _out_layout(self):
        D = len(self.source.largest_region().size)
        if self.kind <= REC_DERIVATIVE or self.kind in (REC_DOG, REC_ZERO_CROSSING):
            return self.source.dtype, 1
        return F32, (D if self.kind == REC_GRADIENT else 3)

    def generate_region(self, requested: Region, stream: Stream = _DEFAULT_STREAM, out_dtype: int | None = None):
        src = self.source
        dtype, comps = self._out_layout()
        p = itkg_recursive_derivative_params()
        p.sigma, p.kind, p.axis, p.order, p.rounding = self.sigma, self.kind, self.deriv_axis, self.order, self.rounding
        p.sigma2 = self.sigma2
        largest = src.largest_region().to_c()
        req = requested.to_c()
        sc = src.to_c()
        if isinstance(src, Image):
            shape = tuple(reversed(requested.size)) + ((comps,) if comps > 1 else ())
            res = Image(np.empty(shape, dtype=_storage_np(dtype)), index=requested.index, spacing=src.spacing,
                        origin=src.origin, components=comps)
            oc = res.to_c()
            check(lib().itkg_recursive_gaussian_derivative_generate_region(
                ctypes.byref(sc), ctypes.byref(largest), ctypes.byref(req), ctypes.byref(p), ctypes.byref(oc),
                stream.ptr))
            return res
        dev = DeviceImage(requested, dtype, comps, src.spacing, src.origin)
        check(lib().itkg_recursive_gaussian_derivative_generate_region(
            ctypes.byref(sc), ctypes.byref(largest), ctypes.byref(req), ctypes.byref(p), ctypes.byref(dev.c),
            stream.ptr))
        return dev


class GradientMagnitudeRecursiveGaussianFilter(RecursiveGaussianDerivativeFilter):
    """GradientMagnitudeRecursiveGaussianFilter { source, sigma } (edges.rs:686-722)."""

    def __init__(self, source, sigma: float, **kw):
        super().__init__(source, sigma, REC_GRADIENT_MAGNITUDE, **kw)


class LaplacianRecursiveGaussianFilter(RecursiveGaussianDerivativeFilter):
    """LaplacianRecursiveGaussianFilter { source, sigma } (edges.rs:730-766)."""

    def __init__(self, source, sigma: float, **kw):
        super().__init__(source, sigma, REC_LAPLACIAN, **kw)


class DiscreteGaussianDerivativeFilter(RecursiveGaussianDerivativeFilter):
    """DiscreteGaussianDerivativeFilter { source, sigma, axis, order } (edges.rs:772-810)."""

    def __init__(self, source, sigma: float, axis: int, order: int = 1, **kw):
        super().__init__(source, sigma, REC_DERIVATIVE, axis=axis, order=order, **kw)


class GradientRecursiveGaussianFilter(RecursiveGaussianDerivativeFilter):
    """GradientRecursiveGaussianFilter { source, sigma } (edges.rs:819-878): VecPixel<f32, D>."""

    def __init__(self, source, sigma: float, **kw):
        super().__init__(source, sigma, REC_GRADIENT, **kw)


class DifferenceOfGaussiansFilter(RecursiveGaussianDerivativeFilter):
    """DifferenceOfGaussiansFilter { source, sigma1, sigma2 } (edges.rs:955-1009)."""

    def __init__(self, source, sigma1: float, sigma2: float, **kw):
        super().__init__(source, sigma1, REC_DOG, sigma2=sigma2, **kw)


class ZeroCrossingBasedEdgeDetectionFilter(RecursiveGaussianDerivativeFilter):
    """ZeroCrossingBasedEdgeDetectionFilter { source, sigma } (edges.rs:1019-1052): 1 at the
    zero crossings of the Laplacian of the smoothed image, else 0, in the pixel type."""

    def __init__(self, source, sigma: float, **kw):
        super().__init__(source, sigma, REC_ZERO_CROSSING, **kw)


class HessianRecursiveGaussianFilter(RecursiveGaussianDerivativeFilter):
    """HessianRecursiveGaussianFilter { source, sigma } (edges.rs:892-950): 2-D, VecPixel<f32, 3>."""

    def __init__(self, source, sigma: float, **kw):
        super().__init__(source, sigma, REC_HESSIAN, **kw)


def stream_full(source: GaussianFilter, num_pieces: int, stream: Stream = _DEFAULT_STREAM,
                out_dtype: int | None = None):
    """stream_full (source.rs:81-98): full output filled piece by piece."""
    leaf = source._leaf()
    prm = source.params()
    if out_dtype is None:
        out_dtype = U8 if prm.arithmetic == ARITH_PIXEL_U8 else F32
    full = leaf.largest_region()
    lc = full.to_c()
    src = leaf.to_c()
    if isinstance(leaf, Image):
        shape = tuple(reversed(full.size)) + ((leaf.components,) if leaf.components > 1 else ())
        res = Image(np.empty(shape, dtype=_storage_np(out_dtype)), index=full.index,
                    spacing=leaf.spacing, origin=leaf.origin, components=leaf.components,
                    bf16=(out_dtype == BF16))
        oc = res.to_c()
    else:
        res = DeviceImage(full, out_dtype, leaf.components, leaf.spacing, leaf.origin)
        oc = res.c
    check(lib().itkg_stream_full(ctypes.byref(src), ctypes.byref(lc), ctypes.byref(prm),
                                 int(num_pieces), ctypes.byref(oc), stream.ptr))
    return res


def gaussian(arr: np.ndarray, sigma: float, spacing=None, components: int = 1,
             rounding: int = ROUND_REFERENCE, algorithm: int = ALGO_AUTO,
             out_dtype: int | None = None, arithmetic: int | None = None, requested=None,
             index=None):
    """One-call convenience: host array in, host array out (through the C ABI)."""
    img = Image(arr, index=index, spacing=spacing, components=components)
    if arithmetic is None:
        arithmetic = ARITH_PIXEL_U8 if img.dtype == U8 else ARITH_F32
    src = img if (arithmetic == ARITH_PIXEL_U8 or img.dtype == F32) else CastFilter(img, F32)
    f = GaussianFilter(src, sigma, rounding=rounding, algorithm=algorithm, arithmetic=arithmetic)
    req = Region(*requested) if requested is not None else img.region
    return f.generate_region(req, out_dtype=out_dtype).data


VJP_ACCUMULATE_XBAR = 1
VJP_ACCUMULATE_SIGMA = 2
VJP_SIGMA_BAR_ON_DEVICE = 4


def vjp(x: DeviceImage, ybar: DeviceImage, sigma: float, xbar: DeviceImage | None = None,
        want_sigma: bool = True, flags: int = 0, sigma_bar_init: float = 0.0,
        stream: Stream = _DEFAULT_STREAM, algorithm: int = ALGO_AUTO):
    """GaussianFilter VJP over the whole image: returns (xbar, sigma_bar).

    xbar = G^T ybar (a DeviceImage, allocated if not given); sigma_bar =
    <ybar, dy/dsigma> as a Python float (None if not requested)."""
    p = itkg_gaussian_params()
    p.sigma = float(sigma)
    p.rounding = ROUND_FMA
    p.algorithm = algorithm
    if xbar is None:
        xbar = DeviceImage(x.region, F32, 1, x.spacing, x.origin)
    sb = ctypes.c_double(sigma_bar_init)
    check(lib().itkg_gaussian_vjp(ctypes.byref(x.c), ctypes.byref(ybar.c), ctypes.byref(p),
                                  ctypes.byref(xbar.c), ctypes.byref(sb) if want_sigma else None,
                                  int(flags), stream.ptr))
    return xbar, (sb.value if want_sigma else None)


def scale_stack_loss_vjp(x: DeviceImage, target: DeviceImage, sigmas, xbar: DeviceImage | None = None,
                         stream: Stream = _DEFAULT_STREAM):
    """L = sum_l |G_{sigma_l} x - target|^2 with dL/dx and dL/dsigma_l: (loss, xbar, [sigma_bar])."""
    n = len(sigmas)
    if xbar is None:
        xbar = DeviceImage(x.region, F32, 1, x.spacing, x.origin)
    sg = (ctypes.c_double * n)(*[float(s) for s in sigmas])
    sb = (ctypes.c_double * n)()
    loss = ctypes.c_double(0.0)
    check(lib().itkg_gaussian_scale_stack_loss_vjp(ctypes.byref(x.c), ctypes.byref(target.c), sg, n,
                                                   ctypes.byref(xbar.c), ctypes.byref(loss), sb, 0,
                                                   stream.ptr))
    return loss.value, xbar, list(sb)


class Batch:
    """itkg_batch: many forward / VJP requests planned once, replayed as a CUDA graph."""

    BATCH_NO_AUTOTUNE = 1

    def __init__(self):
        h = ctypes.c_void_p()
        check(lib().itkg_batch_create(ctypes.byref(h)))
        self.h = h
        self._keep = []  # keep device buffers referenced while the batch lives

    def add(self, src: DeviceImage, sigma: float, out: DeviceImage | None = None,
            requested: Region | None = None, rounding: int = ROUND_FMA,
            algorithm: int = ALGO_AUTO, largest: Region | None = None):
        req = requested or src.region
        if out is None:
            out = DeviceImage(req, F32, src.components, src.spacing, src.origin)
        p = itkg_gaussian_params()
        p.sigma = float(sigma)
        p.rounding = rounding
        p.algorithm = algorithm
        lg = (largest or src.region).to_c()
        rq = req.to_c()
        check(lib().itkg_batch_add(self.h, ctypes.byref(src.c), ctypes.byref(lg), ctypes.byref(rq),
                                   ctypes.byref(p), ctypes.byref(out.c)))
        self._keep += [src, out]
        return out

    def add_vjp(self, x: DeviceImage, ybar: DeviceImage, sigma: float,
                xbar: DeviceImage | None = None, sigma_bar_dev: int | None = None, flags: int = 0):
        if xbar is None:
            xbar = DeviceImage(x.region, F32, 1, x.spacing, x.origin)
        p = itkg_gaussian_params()
        p.sigma = float(sigma)
        p.rounding = ROUND_FMA
        check(lib().itkg_batch_add_vjp(self.h, ctypes.byref(x.c), ctypes.byref(ybar.c),
                                       ctypes.byref(p), ctypes.byref(xbar.c),
                                       ctypes.c_void_p(sigma_bar_dev) if sigma_bar_dev else None,
                                       int(flags)))
        self._keep += [x, ybar, xbar]
        return xbar

    def plan(self, autotune: bool = True, stream: Stream = _DEFAULT_STREAM):
        check(lib().itkg_batch_plan(self.h, 0 if autotune else self.BATCH_NO_AUTOTUNE, stream.ptr))

    def run(self, stream: Stream = _DEFAULT_STREAM):
        check(lib().itkg_batch_run(self.h, stream.ptr))

    def describe(self) -> str:
        return lib().itkg_batch_describe(self.h).decode()

    def __del__(self):
        try:
            lib().itkg_batch_destroy(self.h)
        except Exception:
            pass


def last_kernel() -> str:
    return lib().itkg_last_kernel().decode()


def device_count() -> int:
    n = ctypes.c_int32(0)
    check(lib().itkg_device_count(ctypes.byref(n)))
    return n.value
