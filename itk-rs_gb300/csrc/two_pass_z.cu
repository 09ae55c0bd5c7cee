// The z kernels of the two-pass 3-D forward in FMA rounding, element-wise and f32-quad stores.
#include "two_pass.cuh"

namespace itkg {
namespace twopass {
const ZFn* z_row_fma_any() {
  static const ZFn row[kMaxR] = ITKG_Z_ROW(false, kStoreAny);
  return row;
}
const ZFn* z_row_fma_f32q() {
  static const ZFn row[kMaxR] = ITKG_Z_ROW(false, kStoreF32Quad);
  return row;
}
}  // namespace twopass
}  // namespace itkg
