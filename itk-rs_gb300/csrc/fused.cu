// Fused whole-filter kernels (placeholder until the fused kernels land).
#include "internal.hpp"

namespace itkg {

itkg_status launch_fused(const FusedGeom&, const float* const[kMaxDim], void*, bool) {
  return ITKG_ERROR_UNSUPPORTED;
}

}  // namespace itkg
