// The z kernels of the two-pass 3-D forward that store UnsharpMaskFilter's
// point-wise step (k_z_pass<R, REF, kStoreF32Quad, true>), in their own translation
// unit so they compile beside the plain ones.
#include "two_pass.cuh"

namespace itkg {
namespace twopass {
namespace {
struct ZUshEntry {
  int r;
  ZFn fn[2];  // [ref]
};
template <int R>
ZUshEntry make_z_ush() {
  return ZUshEntry{R, {k_z_pass<R, false, kStoreF32Quad, true>, k_z_pass<R, true, kStoreF32Quad, true>}};
}
const ZUshEntry kZUsh[] = {make_z_ush<1>(), make_z_ush<2>(),  make_z_ush<3>(),  make_z_ush<4>(),
                           make_z_ush<5>(), make_z_ush<6>(),  make_z_ush<7>(),  make_z_ush<8>(),
                           make_z_ush<9>(), make_z_ush<10>(), make_z_ush<11>(), make_z_ush<12>()};
}  // namespace

ZFn z_ush_fn(int r, bool ref) {
  for (const ZUshEntry& z : kZUsh)
    if (z.r == r) return z.fn[ref ? 1 : 0];
  return nullptr;
}
}  // namespace twopass
}  // namespace itkg
