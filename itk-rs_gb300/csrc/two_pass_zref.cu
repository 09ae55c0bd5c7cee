// The z kernels of the two-pass 3-D forward in reference rounding, element-wise and f32-quad stores.
#include "two_pass.cuh"

namespace itkg {
namespace twopass {
const ZFn* z_row_ref_any() {
  static const ZFn row[kMaxR] = ITKG_Z_ROW(true, kStoreAny);
  return row;
}
const ZFn* z_row_ref_f32q() {
  static const ZFn row[kMaxR] = ITKG_Z_ROW(true, kStoreF32Quad);
  return row;
}
}  // namespace twopass
}  // namespace itkg
