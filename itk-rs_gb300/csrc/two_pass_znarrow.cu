// The z kernels of the two-pass 3-D forward in FMA rounding that store bf16 / f16 quads.
#include "two_pass.cuh"

namespace itkg {
namespace twopass {
const ZFn* z_row_fma_bf16q() {
  static const ZFn row[kMaxR] = ITKG_Z_ROW(false, kStoreBF16Quad);
  return row;
}
const ZFn* z_row_fma_f16q() {
  static const ZFn row[kMaxR] = ITKG_Z_ROW(false, kStoreF16Quad);
  return row;
}
}  // namespace twopass
}  // namespace itkg
