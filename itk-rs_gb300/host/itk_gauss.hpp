// itk_gauss.hpp -- C++ host mirror of itk-rs's Gaussian pipeline API, calling
// the sm_103a kernels through the itkg C ABI (include/itkg.h).
//
// The reference is a Rust crate; with no Rust toolchain available this header
// is the compiled host side above the C ABI.  Names, argument meanings and
// ownership follow the reference:
//   Index / Size / Region           src/image.rs:1-77
//   Image<P, D>                     src/image.rs:79-174
//   VecPixel<T, N>                  src/pixel.rs:458-495
//   ImageSource (duck-typed)        src/source.rs:13-75
//   stream_full                     src/source.rs:81-98
//   split_region                    src/region_splitter.rs:17-48
//   GaussianFilter<S>               src/filters/gaussian.rs:13-91
//   UnaryFilter<S, F, P, Q>         src/filters/mod.rs:47-81
// Where the reference panics, these functions throw itk::Error.
#pragma once

#include <array>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "itkg.h"

namespace itk {

struct Error : std::runtime_error {
  itkg_status status;
  Error(itkg_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(itkg_status s) {
  if (s != ITKG_SUCCESS) throw Error(s, std::string("itkg: ") + itkg_last_error());
}

template <int D>
struct Index {
  std::array<int64_t, D> v{};
  int64_t operator[](int d) const { return v[d]; }
  bool operator==(const Index& o) const { return v == o.v; }
};

template <int D>
struct Region {
  std::array<int64_t, D> index{};
  std::array<uint64_t, D> size{};

  static Region make(std::array<int64_t, D> i, std::array<uint64_t, D> s) {
    Region r;
    r.index = i;
    r.size = s;
    return r;
  }
  uint64_t linear_len() const {
    uint64_t n = 1;
    for (int d = 0; d < D; ++d) n *= size[d];
    return n;
  }
  Region padded_per_axis(const std::array<uint64_t, D>& radii) const {
    Region r = *this;
    for (int d = 0; d < D; ++d) {
      r.index[d] -= (int64_t)radii[d];
      r.size[d] += 2 * radii[d];
    }
    return r;
  }
  Region padded(uint64_t radius) const {
    std::array<uint64_t, D> radii;
    radii.fill(radius);
    return padded_per_axis(radii);
  }
  Region clipped_to(const Region& b) const {
    Region r = *this;
    for (int d = 0; d < D; ++d) {
      const int64_t se = index[d] + (int64_t)size[d], be = b.index[d] + (int64_t)b.size[d];
      const int64_t s = index[d] > b.index[d] ? index[d] : b.index[d];
      const int64_t e = se < be ? se : be;
      r.index[d] = s;
      r.size[d] = e > s ? (uint64_t)(e - s) : 0;
    }
    return r;
  }
  bool contains(const Index<D>& i) const {
    for (int d = 0; d < D; ++d)
      if (i[d] < index[d] || i[d] >= index[d] + (int64_t)size[d]) return false;
    return true;
  }
  bool operator==(const Region& o) const { return index == o.index && size == o.size; }
  itkg_region to_c() const {
    itkg_region r;
    for (int d = 0; d < ITKG_MAX_DIM; ++d) {
      r.index[d] = d < D ? index[d] : 0;
      r.size[d] = d < D ? size[d] : 1;
    }
    return r;
  }
  static Region from_c(const itkg_region& c) {
    Region r;
    for (int d = 0; d < D; ++d) {
      r.index[d] = c.index[d];
      r.size[d] = c.size[d];
    }
    return r;
  }
};

template <typename T, int N>
struct VecPixel {
  std::array<T, N> c{};
};

// Pixel type -> (storage dtype, components, default arithmetic).
template <typename P>
struct PixelTraits;
template <>
struct PixelTraits<float> {
  static constexpr int dtype = ITKG_F32, comps = 1, arith = ITKG_ARITH_F32;
};
template <>
struct PixelTraits<uint8_t> {  // GaussianFilter<Image<u8>>: u8 NumericPixel arithmetic
  static constexpr int dtype = ITKG_U8, comps = 1, arith = ITKG_ARITH_PIXEL_U8;
};
template <>
struct PixelTraits<int16_t> {  // storage only (the reference has no NumericPixel for i16)
  static constexpr int dtype = ITKG_I16, comps = 1, arith = ITKG_ARITH_F32;
};
template <>
struct PixelTraits<VecPixel<float, 3>> {
  static constexpr int dtype = ITKG_F32, comps = 3, arith = ITKG_ARITH_F32;
};
template <>
struct PixelTraits<VecPixel<float, 2>> {  // 2-D displacement fields
  static constexpr int dtype = ITKG_F32, comps = 2, arith = ITKG_ARITH_F32;
};

template <typename P, int D>
struct Image {
  using Pixel = P;
  static constexpr int Dim = D;
  Region<D> region;
  std::array<double, D> spacing{};
  std::array<double, D> origin{};
  std::vector<P> data;

  static Image allocate(const Region<D>& r, std::array<double, D> sp, std::array<double, D> org,
                        P fill) {
    Image im;
    im.region = r;
    im.spacing = sp;
    im.origin = org;
    im.data.assign(r.linear_len(), fill);
    return im;
  }
  size_t flat_index(const Index<D>& i) const {
    size_t off = 0, stride = 1;
    for (int d = 0; d < D; ++d) {
      const int64_t local = i[d] - region.index[d];
      if (local < 0 || local >= (int64_t)region.size[d]) throw Error(ITKG_ERROR_INVALID_ARGUMENT, "index out of region");
      off += (size_t)local * stride;
      stride *= region.size[d];
    }
    return off;
  }
  P get_pixel(const Index<D>& i) const { return data[flat_index(i)]; }
  void set_pixel(const Index<D>& i, P v) { data[flat_index(i)] = v; }
  void copy_from(const Image& src) {
    itkg_image d = desc(), s = src.desc();
    check(itkg_image_copy_from(&d, &s, nullptr));
  }
  // ImageSource (source.rs:32-59)
  Region<D> largest_region() const { return region; }
  Image generate_region(const Region<D>& requested) const {
    Image out = allocate(requested.clipped_to(region), spacing, origin, P{});
    out.copy_from_region(*this);
    return out;
  }
  Region<D> input_region_for_output(const Region<D>& r) const { return r; }

  itkg_image desc(int dtype_override = -1) const {
    itkg_image im;
    std::memset(&im, 0, sizeof im);
    im.dim = D;
    im.dtype = dtype_override >= 0 ? dtype_override : PixelTraits<P>::dtype;
    im.components = PixelTraits<P>::comps;
    im.location = ITKG_HOST;
    im.region = region.to_c();
    int64_t p = (int64_t)sizeof(P);
    for (int d = 0; d < ITKG_MAX_DIM; ++d) {
      im.pitch[d] = p;
      if (d < D) p *= (int64_t)region.size[d];
      im.spacing[d] = d < D ? spacing[d] : 1.0;
      im.origin[d] = d < D ? origin[d] : 0.0;
    }
    im.data = const_cast<P*>(data.data());
    return im;
  }

 private:
  void copy_from_region(const Image& big) {
    if (region.linear_len() == 0) return;
    itkg_image d = desc();
    itkg_image s = big.desc();
    s.region = region.to_c();  // view of `big` restricted to our region
    int64_t off = 0;
    for (int dd = 0; dd < D; ++dd) off += (region.index[dd] - big.region.index[dd]) * s.pitch[dd];
    s.data = static_cast<char*>(s.data) + off;
    check(itkg_image_copy_from(&d, &s, nullptr));
  }
};

// Device-resident image (pitched, 128-byte rows) -- the device buffer the
// reference's Image gains on this path.  Move-only RAII owner.
template <typename P, int D>
struct DeviceImage {
  using Pixel = P;
  static constexpr int Dim = D;
  itkg_image c{};
  DeviceImage() = default;
  DeviceImage(const Region<D>& r, std::array<double, D> sp, std::array<double, D> org,
              int dtype = PixelTraits<P>::dtype) {
    itkg_region rc = r.to_c();
    double s3[3] = {1, 1, 1}, o3[3] = {0, 0, 0};
    for (int d = 0; d < D; ++d) {
      s3[d] = sp[d];
      o3[d] = org[d];
    }
    check(itkg_image_alloc_device(&c, D, dtype, PixelTraits<P>::comps, &rc, s3, o3));
  }
  DeviceImage(const DeviceImage&) = delete;
  DeviceImage& operator=(const DeviceImage&) = delete;
  DeviceImage(DeviceImage&& o) noexcept : c(o.c) { o.c.data = nullptr; }
  DeviceImage& operator=(DeviceImage&& o) noexcept {
    std::swap(c, o.c);
    return *this;
  }
  ~DeviceImage() {
    if (c.data) itkg_image_free(&c);
  }
  static DeviceImage upload(const Image<P, D>& h) {
    DeviceImage d(h.region, h.spacing, h.origin);
    itkg_image s = h.desc();
    check(itkg_image_copy_from(&d.c, &s, nullptr));
    return d;
  }
  Image<P, D> download() const {
    Image<P, D> h = Image<P, D>::allocate(region(), spacing(), origin(), P{});
    itkg_image d = h.desc();
    check(itkg_image_copy_from(&d, &c, nullptr));
    return h;
  }
  Region<D> region() const { return Region<D>::from_c(c.region); }
  Region<D> largest_region() const { return region(); }
  std::array<double, D> spacing() const {
    std::array<double, D> s;
    for (int d = 0; d < D; ++d) s[d] = c.spacing[d];
    return s;
  }
  std::array<double, D> origin() const {
    std::array<double, D> s;
    for (int d = 0; d < D; ++d) s[d] = c.origin[d];
    return s;
  }
};

// split_region (region_splitter.rs:17-48)
template <int D>
std::vector<Region<D>> split_region(const Region<D>& r, uint64_t num_pieces) {
  itkg_region c = r.to_c();
  uint64_t n = 0;
  check(itkg_split_region(&c, D, num_pieces, nullptr, 0, &n));
  std::vector<itkg_region> ps(n);
  check(itkg_split_region(&c, D, num_pieces, ps.data(), n, &n));
  std::vector<Region<D>> out;
  for (auto& p : ps) out.push_back(Region<D>::from_c(p));
  return out;
}

// UnaryFilter<S, F, P, Q> (filters/mod.rs:47-81): a host-side per-pixel map.
template <typename S, typename F, typename P, typename Q>
struct UnaryFilter {
  S source;
  F func;
  static constexpr int Dim = std::decay_t<S>::Dim;
  using Pixel = Q;
  Region<Dim> largest_region() const { return source.largest_region(); }
  Image<Q, Dim> generate_region(const Region<Dim>& requested) const {
    auto in = source.generate_region(requested);
    Image<Q, Dim> out;
    out.region = in.region;
    out.spacing = in.spacing;
    out.origin = in.origin;
    out.data.resize(in.data.size());
    for (size_t i = 0; i < in.data.size(); ++i) out.data[i] = func(in.data[i]);
    return out;
  }
};

// The reference's `UnaryFilter::new(img, |p| p as f32)` in front of the
// Gaussian.  Kept as its own node so GaussianFilter can fuse the exact cast
// into its load instead of materialising an f32 copy.
template <typename Img>
struct CastToF32 {
  const Img& source;
  static constexpr int Dim = Img::Dim;
  using Pixel = float;
  Region<Dim> largest_region() const { return source.largest_region(); }
};

template <typename T>
struct is_cast : std::false_type {};
template <typename Img>
struct is_cast<CastToF32<Img>> : std::true_type {};

// ImageSource::spacing (source.rs:16) as a free function: Image keeps the
// reference's public `spacing` field, so the trait method cannot share its name.
template <typename P, int D>
std::array<double, D> spacing_of(const Image<P, D>& s) { return s.spacing; }
template <typename P, int D>
std::array<double, D> spacing_of(const DeviceImage<P, D>& s) { return s.spacing(); }
template <typename Img>
auto spacing_of(const CastToF32<Img>& s) { return spacing_of(s.source); }
template <typename S, typename F, typename P, typename Q>
auto spacing_of(const UnaryFilter<S, F, P, Q>& s) { return spacing_of(s.source); }

// GaussianFilter<S> (gaussian.rs:13-91).  S may be Image<P,D>, DeviceImage<P,D>,
// CastToF32<Image<...>>, or any node with largest_region()/generate_region().
template <typename S>
struct GaussianFilter {
  S source;
  double sigma;
  int rounding = ITKG_ROUND_REFERENCE;
  int algorithm = ITKG_ALGO_AUTO;

  GaussianFilter(S s, double sg) : source(std::forward<S>(s)), sigma(sg) {}

  static constexpr int Dim = std::decay_t<S>::Dim;
  using Pixel = typename std::decay_t<S>::Pixel;

  Region<Dim> largest_region() const { return source.largest_region(); }

  Region<Dim> input_region_for_output(const Region<Dim>& out) const {
    itkg_region o = out.to_c(), l = largest_region().to_c(), in;
    auto sp = spacing();
    double s3[3] = {1, 1, 1};
    for (int d = 0; d < Dim; ++d) s3[d] = sp[d];
    check(itkg_gaussian_input_region_for_output(&o, &l, Dim, s3, sigma, &in));
    return Region<Dim>::from_c(in);
  }

  std::array<double, Dim> spacing() const { return spacing_of(source); }

  itkg_gaussian_params params(int arith) const {
    itkg_gaussian_params p;
    std::memset(&p, 0, sizeof p);
    p.sigma = sigma;
    p.arithmetic = arith;
    p.rounding = rounding;
    p.algorithm = algorithm;
    return p;
  }

  // Host result (Image) for host sources, as the reference returns.
  auto generate_region(const Region<Dim>& requested) const {
    using S0 = std::decay_t<S>;
    if constexpr (is_cast<S0>::value) {
      using Leaf = std::decay_t<decltype(source.source)>;
      const Leaf& leaf = source.source;
      Image<float, Dim> out = Image<float, Dim>::allocate(requested, leaf.spacing, leaf.origin, 0.0f);
      run(leaf.desc(), leaf.largest_region(), requested, ITKG_ARITH_F32, out.desc());
      return out;
    } else if constexpr (is_device<S0>::value) {
      DeviceImage<Pixel, Dim> out(requested, source.spacing(), source.origin());
      run(source.c, source.largest_region(), requested, PixelTraits<Pixel>::arith, out.c);
      return out;
    } else if constexpr (is_host_image<S0>::value) {
      auto out = Image<Pixel, Dim>::allocate(requested, source.spacing, source.origin, Pixel{});
      run(source.desc(), source.largest_region(), requested, PixelTraits<Pixel>::arith, out.desc());
      return out;
    } else {
      // Generic upstream node: pull the halo-padded region (gaussian.rs:71-72).
      auto in = source.generate_region(input_region_for_output(requested));
      auto out = Image<Pixel, Dim>::allocate(requested, in.spacing, in.origin, Pixel{});
      run(in.desc(), largest_region(), requested, PixelTraits<Pixel>::arith, out.desc());
      return out;
    }
  }

 private:
  template <typename T>
  struct is_device : std::false_type {};
  template <typename P, int D>
  struct is_device<DeviceImage<P, D>> : std::true_type {};
  template <typename T>
  struct is_host_image : std::false_type {};
  template <typename P, int D>
  struct is_host_image<Image<P, D>> : std::true_type {};

  void run(itkg_image in, const Region<Dim>& largest, const Region<Dim>& requested, int arith,
           itkg_image out) const {
    itkg_region l = largest.to_c(), r = requested.to_c();
    itkg_gaussian_params p = params(arith);
    check(itkg_gaussian_generate_region(&in, &l, &r, &p, &out, nullptr));
  }
};

template <typename S>
GaussianFilter<S> make_gaussian(S s, double sigma) {
  return GaussianFilter<S>(std::move(s), sigma);
}

template <typename S>
auto spacing_of(const GaussianFilter<S>& g) { return g.spacing(); }

// The convolve_axis family with explicit kernels (one f64 kernel per axis,
// `repetitions` rounds of one pass per axis): the engine of MeanFilter
// (mean.rs:27-84), BoxMeanFilterN (mean.rs:103-137) and BinomialBlurFilter
// (binomial_blur.rs:17-89); make_mean / make_box_mean / make_binomial build it.
template <typename S>
struct SeparableFilter {
  S source;
  std::vector<std::vector<double>> kernels;  // per axis, odd lengths
  uint64_t repetitions = 1;
  int rounding = ITKG_ROUND_REFERENCE;
  int algorithm = ITKG_ALGO_AUTO;

  static constexpr int Dim = std::decay_t<S>::Dim;
  using Pixel = typename std::decay_t<S>::Pixel;

  SeparableFilter(S s, std::vector<std::vector<double>> k, uint64_t reps)
      : source(std::forward<S>(s)), kernels(std::move(k)), repetitions(reps) {
    if ((int)kernels.size() != Dim) throw std::runtime_error("one kernel per axis");
    for (const auto& w : kernels)
      if (w.size() % 2 != 1) throw std::runtime_error("kernels have odd length");
  }

  Region<Dim> largest_region() const { return source.largest_region(); }
  std::array<double, Dim> spacing() const { return spacing_of(source); }

  Region<Dim> input_region_for_output(const Region<Dim>& out) const {
    itkg_region o = out.to_c(), l = largest_region().to_c(), in;
    uint64_t r[3] = {0, 0, 0};
    for (int d = 0; d < Dim; ++d) r[d] = (kernels[d].size() - 1) / 2;
    check(itkg_separable_input_region_for_output(&o, &l, Dim, r, repetitions, &in));
    return Region<Dim>::from_c(in);
  }

  itkg_separable_params params(int arith) const {
    itkg_separable_params p;
    std::memset(&p, 0, sizeof p);
    for (int d = 0; d < Dim; ++d) {
      p.radius[d] = (kernels[d].size() - 1) / 2;
      p.weights[d] = kernels[d].data();
    }
    p.repetitions = repetitions;
    p.arithmetic = arith;
    p.rounding = rounding;
    p.algorithm = algorithm;
    return p;
  }

  auto generate_region(const Region<Dim>& requested) const {
    using S0 = std::decay_t<S>;
    if constexpr (is_device_image<S0>::value) {
      DeviceImage<Pixel, Dim> out(requested, source.spacing(), source.origin());
      run(source.c, source.largest_region(), requested, PixelTraits<Pixel>::arith, out.c);
      return out;
    } else if constexpr (is_host_image_t<S0>::value) {
      auto out = Image<Pixel, Dim>::allocate(requested, source.spacing, source.origin, Pixel{});
      run(source.desc(), source.largest_region(), requested, PixelTraits<Pixel>::arith, out.desc());
      return out;
    } else {
      auto in = source.generate_region(input_region_for_output(requested));
      auto out = Image<Pixel, Dim>::allocate(requested, in.spacing, in.origin, Pixel{});
      run(in.desc(), largest_region(), requested, PixelTraits<Pixel>::arith, out.desc());
      return out;
    }
  }

 private:
  template <typename T>
  struct is_device_image : std::false_type {};
  template <typename P, int D>
  struct is_device_image<DeviceImage<P, D>> : std::true_type {};
  template <typename T>
  struct is_host_image_t : std::false_type {};
  template <typename P, int D>
  struct is_host_image_t<Image<P, D>> : std::true_type {};

  void run(itkg_image in, const Region<Dim>& largest, const Region<Dim>& requested, int arith,
           itkg_image out) const {
    itkg_region l = largest.to_c(), r = requested.to_c();
    itkg_separable_params p = params(arith);
    check(itkg_separable_generate_region(&in, &l, &r, &p, &out, nullptr));
  }
};

// box_kernel (mean.rs:15-18)
inline std::vector<double> box_kernel(uint64_t radius) {
  std::vector<double> w(2 * radius + 1);
  check(itkg_box_kernel(radius, w.data()));
  return w;
}

// MeanFilter::new(source, radius) (mean.rs:35-39)
template <typename S>
SeparableFilter<S> make_mean(S s, uint64_t radius) {
  constexpr int D = std::decay_t<S>::Dim;
  return SeparableFilter<S>(std::move(s), std::vector<std::vector<double>>(D, box_kernel(radius)), 1);
}

// BoxMeanFilterN::new(source, radii) (mean.rs:109-113)
template <typename S, size_t N>
SeparableFilter<S> make_box_mean(S s, const std::array<uint64_t, N>& radii) {
  std::vector<std::vector<double>> k;
  for (uint64_t r : radii) k.push_back(box_kernel(r));
  return SeparableFilter<S>(std::move(s), std::move(k), 1);
}

// BinomialBlurFilter::new(source, repetitions) (binomial_blur.rs:23-26)
template <typename S>
SeparableFilter<S> make_binomial(S s, uint64_t repetitions) {
  constexpr int D = std::decay_t<S>::Dim;
  return SeparableFilter<S>(std::move(s), std::vector<std::vector<double>>(D, {0.25, 0.5, 0.25}),
                            repetitions);
}

template <typename S>
auto spacing_of(const SeparableFilter<S>& f) { return f.spacing(); }

// UnsharpMaskFilter { source, sigma, amount, threshold } (edges.rs:374-452):
// I + amount (I - blur(I)) where |I - blur(I)| > threshold; the blur kernel
// has radius ceil(3 sigma) on every axis (itkg_unsharp_kernel).
template <typename S>
struct UnsharpMaskFilter {
  S source;
  double sigma;
  double amount = 0.5;     // UnsharpMaskFilter::new (edges.rs:387-389)
  double threshold = 0.0;
  int rounding = ITKG_ROUND_REFERENCE;

  static constexpr int Dim = std::decay_t<S>::Dim;
  using Pixel = typename std::decay_t<S>::Pixel;

  UnsharpMaskFilter(S s, double sg) : source(std::forward<S>(s)), sigma(sg) {}
  UnsharpMaskFilter& with_amount(double a) {  // edges.rs:390
    amount = a;
    return *this;
  }

  Region<Dim> largest_region() const { return source.largest_region(); }
  std::array<double, Dim> spacing() const { return spacing_of(source); }

  Region<Dim> input_region_for_output(const Region<Dim>& out) const {
    uint64_t r = 0;
    check(itkg_unsharp_kernel(sigma, &r, nullptr, 0));
    itkg_region o = out.to_c(), l = largest_region().to_c(), in;
    const uint64_t rr[3] = {r, r, r};
    check(itkg_separable_input_region_for_output(&o, &l, Dim, rr, 1, &in));
    return Region<Dim>::from_c(in);
  }

  auto generate_region(const Region<Dim>& requested) const {
    auto in = source.generate_region(input_region_for_output(requested));
    auto out = Image<Pixel, Dim>::allocate(requested, in.spacing, in.origin, Pixel{});
    itkg_unsharp_params p;
    std::memset(&p, 0, sizeof p);
    p.sigma = sigma;
    p.amount = amount;
    p.threshold = threshold;
    p.rounding = rounding;
    itkg_region l = largest_region().to_c(), r = requested.to_c();
    itkg_image ic = in.desc(), oc = out.desc();
    check(itkg_unsharp_mask_generate_region(&ic, &l, &r, &p, &oc, nullptr));
    return out;
  }
};

template <typename S>
auto spacing_of(const UnsharpMaskFilter<S>& f) { return f.spacing(); }

// SliceBySliceFilter { source, sigma } (spatial.rs:1284-1340), 3-D: every z
// slice of the request through a 2-D GaussianFilter over the request's x-y
// window.
template <typename S>
struct SliceBySliceFilter {
  S source;
  double sigma;
  int rounding = ITKG_ROUND_REFERENCE;

  static constexpr int Dim = std::decay_t<S>::Dim;
  using Pixel = typename std::decay_t<S>::Pixel;
  static_assert(Dim == 3, "SliceBySliceFilter is 3-D");

  SliceBySliceFilter(S s, double sg) : source(std::forward<S>(s)), sigma(sg) {}

  Region<Dim> largest_region() const { return source.largest_region(); }
  std::array<double, Dim> spacing() const { return spacing_of(source); }
  Region<Dim> input_region_for_output(const Region<Dim>& out) const { return out; }

  auto generate_region(const Region<Dim>& requested) const {
    auto in = source.generate_region(requested);  // spatial.rs:1305
    auto out = Image<Pixel, Dim>::allocate(requested, in.spacing, in.origin, Pixel{});
    itkg_gaussian_params p;
    std::memset(&p, 0, sizeof p);
    p.sigma = sigma;
    p.arithmetic = PixelTraits<Pixel>::arith;
    p.rounding = rounding;
    itkg_region r = requested.to_c();
    itkg_image ic = in.desc(), oc = out.desc();
    check(itkg_slice_by_slice_generate_region(&ic, &r, &p, &oc, nullptr));
    return out;
  }
};

template <typename S>
auto spacing_of(const SliceBySliceFilter<S>& f) { return f.spacing(); }

// DisplacementFieldToBSplineFilter { source, sigma } (spatial.rs:1484-1525),
// sigma 2.0 by default: each component of a 2-D VecPixel<f32, 2> field smoothed
// by GaussianFilter { sigma } over the generated request as an image of its own
// -- the request is the Gaussian's largest region, so its taps clamp there.
template <typename S>
struct DisplacementFieldToBSplineFilter {
  S source;
  double sigma = 2.0;
  int rounding = ITKG_ROUND_REFERENCE;

  static constexpr int Dim = std::decay_t<S>::Dim;
  using Pixel = typename std::decay_t<S>::Pixel;
  static_assert(Dim == 2 && std::is_same<Pixel, VecPixel<float, 2>>::value,
                "DisplacementFieldToBSplineFilter takes a 2-D VecPixel<f32, 2> field");

  explicit DisplacementFieldToBSplineFilter(S s, double sg = 2.0) : source(std::forward<S>(s)), sigma(sg) {}

  Region<Dim> largest_region() const { return source.largest_region(); }
  std::array<double, Dim> spacing() const { return spacing_of(source); }
  Region<Dim> input_region_for_output(const Region<Dim>& out) const { return out; }

  auto generate_region(const Region<Dim>& requested) const {
    auto in = source.generate_region(requested);  // spatial.rs:1509
    auto out = Image<Pixel, Dim>::allocate(requested, in.spacing, in.origin, Pixel{});
    itkg_gaussian_params p;
    std::memset(&p, 0, sizeof p);
    p.sigma = sigma;
    p.arithmetic = ITKG_ARITH_F32;
    p.rounding = rounding;
    const itkg_region r = requested.to_c();
    itkg_image ic = in.desc(), oc = out.desc();
    check(itkg_gaussian_generate_region(&ic, &r, &r, &p, &oc, nullptr));
    return out;
  }
};

template <typename S>
auto spacing_of(const DisplacementFieldToBSplineFilter<S>& f) { return f.spacing(); }

// stream_full (source.rs:81-98): allocate the full output once, fill it piece
// by piece along the slowest axis.
template <typename S>
auto stream_full(const S& source, uint64_t num_pieces) {
  constexpr int D = S::Dim;
  using P = typename S::Pixel;
  const Region<D> full = source.largest_region();
  auto sp = spacing_of(source);
  Image<P, D> output = Image<P, D>::allocate(full, sp, std::array<double, D>{}, P{});
  for (const Region<D>& piece : split_region(full, num_pieces)) {
    auto part = source.generate_region(piece);
    output.copy_from(part);
  }
  return output;
}

}  // namespace itk
