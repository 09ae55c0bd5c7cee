// Fused 3-D Gaussian kernels for 16-bit inputs: i16 (the CT case, read as the
// reference's UnaryFilter(|p| p as f32) in front of the filter) and bf16/f16
// storage.  Templates in fused_kernel.cuh; dispatch in fused.cu.
#include "fused_kernel.cuh"

namespace itkg {
namespace fusedk {
namespace {
const Entry kTableI16[] = ITKG_FUSED_TABLE(int16_t);
const Entry kTableBF16[] = ITKG_FUSED_TABLE(__nv_bfloat16);
const Entry kTableF16[] = ITKG_FUSED_TABLE(__half);
}  // namespace
}  // namespace fusedk

const fusedk::Entry* fused_entries_i16(int* n) {
  *n = (int)(sizeof(fusedk::kTableI16) / sizeof(fusedk::kTableI16[0]));
  return fusedk::kTableI16;
}
const fusedk::Entry* fused_entries_bf16(int* n) {
  *n = (int)(sizeof(fusedk::kTableBF16) / sizeof(fusedk::kTableBF16[0]));
  return fusedk::kTableBF16;
}
const fusedk::Entry* fused_entries_f16(int* n) {
  *n = (int)(sizeof(fusedk::kTableF16) / sizeof(fusedk::kTableF16[0]));
  return fusedk::kTableF16;
}

}  // namespace itkg
