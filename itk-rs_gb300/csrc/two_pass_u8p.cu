// The two-pass 3-D kernels in u8 pixel arithmetic (GaussianFilter<Image<u8>>,
// src/pixel.rs:430-435): the x-y kernels over clamped u8 tiles and the z
// kernels storing u8, radii 1 .. 12.
#include "two_pass.cuh"

namespace itkg {
namespace twopass {
namespace {
template <int R>
XYEntry make_xy_u8p() {
  using C = CfgXY<R, uint8_t>;
  const XYFn f = k_xy_pass<R, true, uint8_t, true>;
  return XYEntry{R, ITKG_U8, {f, f}, C::SMEM, C::NT, C::TX, C::TY, C::BW, C::IH};
}
const XYEntry kXYU8P[] = {make_xy_u8p<1>(), make_xy_u8p<2>(),  make_xy_u8p<3>(),  make_xy_u8p<4>(),
                          make_xy_u8p<5>(), make_xy_u8p<6>(),  make_xy_u8p<7>(),  make_xy_u8p<8>(),
                          make_xy_u8p<9>(), make_xy_u8p<10>(), make_xy_u8p<11>(), make_xy_u8p<12>()};
}  // namespace

#define ITKG_Z_U8P_ROW(ST)                                                                            \
  {                                                                                                   \
    k_z_pass<1, true, ST, false, true>, k_z_pass<2, true, ST, false, true>,                           \
        k_z_pass<3, true, ST, false, true>, k_z_pass<4, true, ST, false, true>,                       \
        k_z_pass<5, true, ST, false, true>, k_z_pass<6, true, ST, false, true>,                       \
        k_z_pass<7, true, ST, false, true>, k_z_pass<8, true, ST, false, true>,                       \
        k_z_pass<9, true, ST, false, true>, k_z_pass<10, true, ST, false, true>,                      \
        k_z_pass<11, true, ST, false, true>, k_z_pass<12, true, ST, false, true>                      \
  }

const XYEntry* xy_entries_u8p(int* n) {
  *n = (int)(sizeof(kXYU8P) / sizeof(kXYU8P[0]));
  return kXYU8P;
}
const ZFn* z_row_u8p_any() {
  static const ZFn row[kMaxR] = ITKG_Z_U8P_ROW(kStoreAny);
  return row;
}
const ZFn* z_row_u8p_u8q() {
  static const ZFn row[kMaxR] = ITKG_Z_U8P_ROW(kStoreU8Quad);
  return row;
}
}  // namespace twopass
}  // namespace itkg
