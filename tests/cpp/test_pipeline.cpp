// Host-mirror tests: the reference's pipeline tests (tests/pipeline.rs:19-153,
// src/filters/gaussian.rs:107-127, tests/blur_png.rs:17-73) written against the
// C++ mirror in itk-rs_gb300/host/itk_gauss.hpp, running on the GPU through
// libitkg.so.  Exit status 0 when every check passes; prints one line per test.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <string>

#include "itk_gauss.hpp"

using namespace itk;

static int g_fail = 0;
#define CHECK(cond, ...)                       \
  do {                                         \
    if (!(cond)) {                             \
      std::printf("  FAIL %s:%d: ", __FILE__, __LINE__); \
      std::printf(__VA_ARGS__);                \
      std::printf("\n");                       \
      ++g_fail;                                \
      return;                                  \
    }                                          \
  } while (0)

template <int D>
static Image<float, D> solid_image(std::array<uint64_t, D> size, float fill) {
  std::array<int64_t, D> z{};
  std::array<double, D> one, zero{};
  one.fill(1.0);
  return Image<float, D>::allocate(Region<D>::make(z, size), one, zero, fill);
}

// tests/pipeline.rs:19-31
static void test_image_source_identity_2d() {
  auto img = solid_image<2>({8, 8}, 0.0f);
  img.set_pixel({{3, 5}}, 42.0f);
  auto sub = Region<2>::make({2, 4}, {4, 3});
  auto cropped = img.generate_region(sub);
  CHECK(cropped.region == sub, "region");
  CHECK(cropped.get_pixel({{3, 5}}) == 42.0f, "pixel");
  CHECK(cropped.get_pixel({{2, 4}}) == 0.0f, "zero");
}

// tests/pipeline.rs:37-54 and gaussian.rs:107-127
static void test_gaussian_impulse_2d() {
  const uint64_t size = 21;
  const int64_t mid = size / 2;
  auto img = solid_image<2>({size, size}, 0.0f);
  img.set_pixel({{mid, mid}}, 1.0f);
  GaussianFilter<Image<float, 2>> filter(img, 1.5);
  auto out = filter.generate_region(filter.largest_region());
  float sum = 0.0f;
  for (float v : out.data) sum += v;
  CHECK(std::fabs(sum - 1.0f) < 0.01f, "energy not conserved: sum=%g", sum);
  const float peak = out.get_pixel({{mid, mid}});
  for (float v : out.data) CHECK(v <= peak + 1e-6f, "pixel %g > peak %g", v, peak);
}

// tests/pipeline.rs:60-72
static void test_gaussian_3d() {
  const uint64_t size = 11;
  const int64_t mid = size / 2;
  auto img = solid_image<3>({size, size, size}, 0.0f);
  img.set_pixel({{mid, mid, mid}}, 1.0f);
  GaussianFilter<Image<float, 3>> filter(img, 1.0);
  auto out = filter.generate_region(filter.largest_region());
  float sum = 0.0f;
  for (float v : out.data) sum += v;
  CHECK(std::fabs(sum - 1.0f) < 0.05f, "3D energy not conserved: sum=%g", sum);
}

// tests/pipeline.rs:78-100
static void test_vector_pixel_gaussian() {
  const uint64_t size = 11;
  const int64_t mid = size / 2;
  using V3 = VecPixel<float, 3>;
  auto img = Image<V3, 2>::allocate(Region<2>::make({0, 0}, {size, size}), {1.0, 1.0}, {0.0, 0.0}, V3{});
  img.set_pixel({{mid, mid}}, V3{{1.0f, 2.0f, 3.0f}});
  GaussianFilter<Image<V3, 2>> filter(img, 1.0);
  auto out = filter.generate_region(filter.largest_region());
  float s[3] = {0, 0, 0};
  for (const V3& p : out.data)
    for (int c = 0; c < 3; ++c) s[c] += p.c[c];
  CHECK(std::fabs(s[0] - 1.0f) < 0.05f, "ch0 sum=%g", s[0]);
  CHECK(std::fabs(s[1] - 2.0f) < 0.05f, "ch1 sum=%g", s[1]);
  CHECK(std::fabs(s[2] - 3.0f) < 0.05f, "ch2 sum=%g", s[2]);
}

// tests/pipeline.rs:106-129 (the GPU result is bitwise equal, stronger than 1e-6)
static void test_streaming_matches_full() {
  const uint64_t size = 20;
  const int64_t mid = size / 2;
  auto img = solid_image<2>({size, size}, 0.0f);
  img.set_pixel({{mid, mid}}, 1.0f);
  GaussianFilter<Image<float, 2>> filter(img, 1.5);
  auto full = filter.generate_region(filter.largest_region());
  auto streamed = stream_full(filter, 4);
  CHECK(full.data.size() == streamed.data.size(), "size");
  for (size_t i = 0; i < full.data.size(); ++i)
    CHECK(full.data[i] == streamed.data[i], "mismatch at %zu: %g vs %g", i, full.data[i], streamed.data[i]);
}

// tests/pipeline.rs:135-153
static void test_unary_filter_pipeline() {
  const uint64_t size = 21;
  const int64_t mid = size / 2;
  auto img = solid_image<2>({size, size}, 0.0f);
  img.set_pixel({{mid, mid}}, 1.0f);
  GaussianFilter<Image<float, 2>> gaussian(img, 1.5);
  auto thr = [](float p) { return p > 0.01f ? 1.0f : 0.0f; };
  UnaryFilter<GaussianFilter<Image<float, 2>>, decltype(thr), float, float> threshold{gaussian, thr};
  auto out = threshold.generate_region(threshold.largest_region());
  size_t lit = 0;
  for (float v : out.data) lit += v > 0.5f;
  CHECK(lit > 0, "no pixels above threshold");
  CHECK(lit < size * size, "all pixels above threshold");
}

// tests/blur_png.rs:17-73 without the PNG round trip: u8 -> f32 cast (fused
// into the load), Gaussian sigma 2, f32 -> u8 round+clamp on the host.
static void test_blur_u8_roundtrip() {
  const uint64_t size = 32;
  const int64_t mid = size / 2;
  auto img = Image<uint8_t, 2>::allocate(Region<2>::make({0, 0}, {size, size}), {1.0, 1.0}, {0.0, 0.0}, 0);
  img.set_pixel({{mid, mid}}, 255);
  CastToF32<Image<uint8_t, 2>> as_f32{img};
  GaussianFilter<CastToF32<Image<uint8_t, 2>>> blurred(as_f32, 2.0);
  auto f = blurred.generate_region(blurred.largest_region());
  std::vector<uint8_t> out(f.data.size());
  for (size_t i = 0; i < out.size(); ++i) {
    float r = std::round(f.data[i]);
    r = r < 0.0f ? 0.0f : (r > 255.0f ? 255.0f : r);
    out[i] = (uint8_t)r;
  }
  uint8_t peak = 0;
  uint32_t sum = 0;
  for (uint8_t v : out) {
    peak = v > peak ? v : peak;
    sum += v;
  }
  CHECK(peak < 255, "blur should reduce the peak");
  CHECK(out[mid * size + mid] == peak, "peak should remain at centre");
  CHECK(sum >= 255u * 85 / 100, "too much intensity lost: %u", sum);
}

// Device-resident source: generate_region returns a DeviceImage.
static void test_device_source_matches_host() {
  auto img = solid_image<3>({17, 13, 9}, 0.0f);
  for (size_t i = 0; i < img.data.size(); ++i) img.data[i] = (float)((i * 7919) % 113) / 113.0f;
  GaussianFilter<Image<float, 3>> host_f(img, 1.2);
  auto want = host_f.generate_region(host_f.largest_region());
  auto dev = DeviceImage<float, 3>::upload(img);
  GaussianFilter<DeviceImage<float, 3>&> dev_f(dev, 1.2);
  auto got = dev_f.generate_region(Region<3>::make({0, 0, 0}, {17, 13, 9})).download();
  for (size_t i = 0; i < want.data.size(); ++i)
    CHECK(want.data[i] == got.data[i], "device/host mismatch at %zu", i);
}

// mean.rs:254-292
static void test_mean_filters() {
  auto c = solid_image<1>({10}, 5.0f);
  auto m = make_mean(c, 2);
  auto out = m.generate_region(m.largest_region());
  for (float v : out.data) CHECK(std::fabs(v - 5.0f) < 1e-5f, "constant: %g", v);
  auto ramp = solid_image<1>({20}, 0.0f);
  for (int64_t i = 0; i < 20; ++i) ramp.set_pixel({{i}}, (float)i);
  auto mr = make_mean(ramp, 2);
  auto outr = mr.generate_region(mr.largest_region());
  for (int64_t i = 2; i < 18; ++i)
    CHECK(std::fabs(outr.get_pixel({{i}}) - (float)i) < 1e-4f, "ramp at %lld", (long long)i);
  auto c2 = solid_image<2>({8, 8}, 3.0f);
  auto bm = make_box_mean(c2, std::array<uint64_t, 2>{1, 2});
  auto out2 = bm.generate_region(bm.largest_region());
  for (float v : out2.data) CHECK(std::fabs(v - 3.0f) < 1e-5f, "box mean constant: %g", v);
}

// binomial_blur.rs:96-121
static void test_binomial_blur() {
  auto c = solid_image<1>({20}, 3.0f);
  auto b = make_binomial(c, 4);
  auto out = b.generate_region(b.largest_region());
  for (int64_t i = 4; i < 16; ++i) CHECK(std::fabs(out.get_pixel({{i}}) - 3.0f) < 1e-5f, "constant");
  auto imp = solid_image<1>({21}, 0.0f);
  imp.set_pixel({{10}}, 1.0f);
  auto bi = make_binomial(imp, 4);
  auto outi = bi.generate_region(bi.largest_region());
  const float peak = outi.get_pixel({{10}});
  float sum = 0.0f;
  for (float v : outi.data) sum += v;
  CHECK(peak > 0.0f && peak < 1.0f, "peak=%g", peak);
  CHECK(std::fabs(sum - 1.0f) < 0.05f, "sum=%g", sum);
}

// UnsharpMaskFilter (edges.rs:374-452): a constant stays constant (to the
// f32 blur's rounding); a step gets an undershoot and an overshoot.
static void test_unsharp_mask() {
  auto c = solid_image<2>({9, 7}, 4.0f);
  UnsharpMaskFilter<Image<float, 2>> u(c, 1.0);
  auto out = u.generate_region(u.largest_region());
  for (float v : out.data) CHECK(std::fabs(v - 4.0f) < 1e-5f, "constant: %g", v);
  auto step = solid_image<1>({20}, 0.0f);
  for (int64_t i = 10; i < 20; ++i) step.set_pixel({{i}}, 1.0f);
  UnsharpMaskFilter<Image<float, 1>> us(step, 1.0);
  us.with_amount(1.0);
  auto o = us.generate_region(us.largest_region());
  CHECK(o.get_pixel({{9}}) < 0.0f && o.get_pixel({{10}}) > 1.0f, "step: %g %g", o.get_pixel({{9}}),
        o.get_pixel({{10}}));
  auto sub = us.generate_region(Region<1>{{{5}}, {{10}}});
  for (int64_t i = 5; i < 15; ++i)
    CHECK(sub.get_pixel({{i}}) == o.get_pixel({{i}}), "sub-region at %lld", (long long)i);
}

// SliceBySliceFilter (spatial.rs:1284-1340): slices are smoothed on their own,
// so a volume constant on every slice comes back unchanged.
static void test_slice_by_slice() {
  auto v = solid_image<3>({6, 5, 4}, 0.0f);
  for (int64_t z = 0; z < 4; ++z)
    for (int64_t y = 0; y < 5; ++y)
      for (int64_t x = 0; x < 6; ++x) v.set_pixel({{x, y, z}}, (float)z);
  SliceBySliceFilter<Image<float, 3>> f(v, 1.5);
  auto out = f.generate_region(f.largest_region());
  for (int64_t z = 0; z < 4; ++z)
    CHECK(std::fabs(out.get_pixel({{2, 2, z}}) - (float)z) < 1e-5f, "slice %lld", (long long)z);
}

// DisplacementFieldToBSplineFilter (spatial.rs:1484-1525): a constant field
// comes back unchanged (the weights sum to one), and a sub-region request is
// smoothed as an image of its own -- it equals the filter over the crop.
static void test_displacement_field_to_bspline() {
  using V2 = VecPixel<float, 2>;
  std::array<int64_t, 2> z{};
  auto field = Image<V2, 2>::allocate(Region<2>::make(z, {20, 16}), {1.0, 1.0}, {0.0, 0.0}, V2{});
  for (int64_t y = 0; y < 16; ++y)
    for (int64_t x = 0; x < 20; ++x) field.set_pixel({{x, y}}, V2{{0.5f, -1.25f}});
  DisplacementFieldToBSplineFilter<Image<V2, 2>> f(field);
  auto out = f.generate_region(f.largest_region());
  for (int64_t y = 0; y < 16; ++y)
    for (int64_t x = 0; x < 20; ++x) {
      const V2 p = out.get_pixel({{x, y}});
      CHECK(std::fabs(p.c[0] - 0.5f) < 1e-5f && std::fabs(p.c[1] + 1.25f) < 1e-5f, "constant at %lld,%lld",
            (long long)x, (long long)y);
    }
  for (int64_t y = 0; y < 16; ++y)
    for (int64_t x = 0; x < 20; ++x) field.set_pixel({{x, y}}, V2{{(float)(x * x % 7), (float)(y * 3 % 5)}});
  const Region<2> sub = Region<2>::make({{4, 3}}, {{9, 7}});
  DisplacementFieldToBSplineFilter<Image<V2, 2>> fv(field);  // the filter keeps its own copy of the field
  auto a = fv.generate_region(sub);
  auto crop = field.generate_region(sub);
  DisplacementFieldToBSplineFilter<Image<V2, 2>> fc(crop);
  auto b = fc.generate_region(sub);
  for (int64_t y = 3; y < 10; ++y)
    for (int64_t x = 4; x < 13; ++x) {
      const V2 pa = a.get_pixel({{x, y}}), pb = b.get_pixel({{x, y}});
      CHECK(pa.c[0] == pb.c[0] && pa.c[1] == pb.c[1], "sub-region at %lld,%lld", (long long)x, (long long)y);
    }
}

int main() {
  int ndev = 0;
  itkg_device_count(&ndev);
  if (ndev < 1) {
    std::printf("SKIP: no CUDA device\n");
    return 77;
  }
  const std::pair<const char*, std::function<void()>> tests[] = {
      {"image_source_identity_2d", test_image_source_identity_2d},
      {"gaussian_impulse_2d", test_gaussian_impulse_2d},
      {"gaussian_3d", test_gaussian_3d},
      {"vector_pixel_gaussian", test_vector_pixel_gaussian},
      {"streaming_matches_full", test_streaming_matches_full},
      {"unary_filter_pipeline", test_unary_filter_pipeline},
      {"blur_u8_roundtrip", test_blur_u8_roundtrip},
      {"device_source_matches_host", test_device_source_matches_host},
      {"mean_filters", test_mean_filters},
      {"binomial_blur", test_binomial_blur},
      {"unsharp_mask", test_unsharp_mask},
      {"slice_by_slice", test_slice_by_slice},
      {"displacement_field_to_bspline", test_displacement_field_to_bspline},
  };
  for (auto& t : tests) {
    const int before = g_fail;
    try {
      t.second();
    } catch (const std::exception& e) {
      std::printf("  FAIL exception: %s\n", e.what());
      ++g_fail;
    }
    std::printf("%s %s\n", g_fail == before ? "ok  " : "FAIL", t.first);
  }
  return g_fail == 0 ? 0 : 1;
}
