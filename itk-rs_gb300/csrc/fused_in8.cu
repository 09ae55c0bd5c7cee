// Fused 3-D Gaussian kernels for u8 inputs read through the reference's
// UnaryFilter(|p| p as f32) (f32 arithmetic; u8 pixel arithmetic stays on the
// per-axis path).  Templates in fused_kernel.cuh; dispatch in fused.cu.
#include "fused_kernel.cuh"

namespace itkg {
namespace fusedk {
namespace {
const Entry kTableU8[] = ITKG_FUSED_TABLE(uint8_t);
}  // namespace
}  // namespace fusedk

const fusedk::Entry* fused_entries_u8(int* n) {
  *n = (int)(sizeof(fusedk::kTableU8) / sizeof(fusedk::kTableU8[0]));
  return fusedk::kTableU8;
}

}  // namespace itkg
