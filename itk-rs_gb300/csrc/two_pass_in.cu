// x-y pass tables of the two-kernel 3-D forward for i16 / u8 / bf16 / f16
// inputs (staged by TMA as loaded, converted exactly to f32 in the x pass).
#include "two_pass.cuh"

namespace itkg {
namespace twopass {
namespace {
const XYEntry kI16[] = ITKG_XY_TABLE(int16_t, ITKG_I16);
const XYEntry kU8[] = ITKG_XY_TABLE(uint8_t, ITKG_U8);
const XYEntry kBF16[] = ITKG_XY_TABLE(__nv_bfloat16, ITKG_BF16);
const XYEntry kF16[] = ITKG_XY_TABLE(__half, ITKG_F16);
template <size_t N>
const XYEntry* table(const XYEntry (&t)[N], int* n) {
  *n = (int)N;
  return t;
}
}  // namespace

const XYEntry* xy_entries_i16(int* n) { return table(kI16, n); }
const XYEntry* xy_entries_u8(int* n) { return table(kU8, n); }
const XYEntry* xy_entries_bf16(int* n) { return table(kBF16, n); }
const XYEntry* xy_entries_f16(int* n) { return table(kF16, n); }

}  // namespace twopass
}  // namespace itkg
