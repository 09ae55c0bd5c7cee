// The tiled dual-number passes of the VJP for radii 13 .. 24 (vjp_lines.cuh).
#include <cstring>

#include "vjp_lines.cuh"

namespace itkg {
namespace {
using namespace vjplines;
using LineFn = void (*)(const VjpAxisArgs, const LineTaps, const LineGeom);
struct Row {
  LineFn ax0, ax12;
};
template <int R>
constexpr Row row() { return {k_line_dual<R, true>, k_line_dual<R, false>}; }
const Row kDual[kMaxR - kMinR + 1] = {row<13>(), row<14>(), row<15>(), row<16>(), row<17>(), row<18>(),
                                      row<19>(), row<20>(), row<21>(), row<22>(), row<23>(), row<24>()};
}  // namespace

itkg_status launch_line_dual(const VjpAxisArgs& a, const float* w, const float* dw, void* stream) {
  if (a.radius < kMinR || a.radius > kMaxR) return ITKG_ERROR_UNSUPPORTED;
  LineGeom g;
  int64_t ntiles = 0;
  if (!line_geom(a, &g, &ntiles)) return ITKG_ERROR_UNSUPPORTED;
  LineTaps T;
  std::memset(&T, 0, sizeof T);
  for (int k = 0; k < 2 * a.radius + 1; ++k) T.w[k] = w[k], T.aux[k] = dw[k];
  line_taps_pairs(&T, a.radius);
  const Row& r = kDual[a.radius - kMinR];
  const LineFn fn = a.axis == 0 ? r.ax0 : r.ax12;
  const size_t smem = 2 * sizeof(float) *
                      (a.axis == 0 ? (size_t)kLines * ((kLen + 2 * a.radius) | 1) : (size_t)(kLen + 2 * a.radius) * kLines);
  fn<<<(unsigned)ntiles, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(a, T, g);
  note_launch("dual_lines_f32");
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(ITKG_ERROR_CUDA, "dual_lines launch: %s", cudaGetErrorString(e));
  return ITKG_SUCCESS;
}

}  // namespace itkg
