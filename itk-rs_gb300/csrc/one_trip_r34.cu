// Kernel table of the one-trip 3-D forward for x-y radii 3 and 4 (every z
// radius 1..8, both roundings); one translation unit per radius pair so that
// the instantiations compile in parallel.
#include "one_trip.cuh"

namespace itkg {
namespace onetrip {
namespace {
template <int R, int RZ>
Fn pick(bool ref) {
  return ref ? k_one_trip<R, RZ, true> : k_one_trip<R, RZ, false>;
}
template <int R>
Fn pick_z(int rz, bool ref) {
  switch (rz) {
    case 1: return pick<R, 1>(ref);
    case 2: return pick<R, 2>(ref);
    case 3: return pick<R, 3>(ref);
    case 4: return pick<R, 4>(ref);
    case 5: return pick<R, 5>(ref);
    case 6: return pick<R, 6>(ref);
    case 7: return pick<R, 7>(ref);
    case 8: return pick<R, 8>(ref);
    default: return nullptr;
  }
}
}  // namespace

Fn one_trip_fn_r34(int r, int rz, bool ref) {
  return r == 3 ? pick_z<3>(rz, ref) : r == 4 ? pick_z<4>(rz, ref) : nullptr;
}

}  // namespace onetrip
}  // namespace itkg
