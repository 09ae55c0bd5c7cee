// Host side of the Gaussian VJP (no counterpart in the reference, which has
// no derivative): itkg_gaussian_vjp and itkg_gaussian_scale_stack_loss_vjp.
//
// Coefficients are computed on the host in f64 from the reference's kernel
// formula (gaussian.rs:29-40) at a radius frozen at r(sigma):
//   g_i = exp(-0.5 t_i^2), t_i = (i - r) / s, s = sigma / spacing,
//   w_i = g_i / S,  S = sum g,
//   dw_i/dsigma = (g_i' S - g_i S') / S^2 / spacing,  g_i' = g_i t_i^2 / s,
//   P_m = w_0 + ... + w_m  (adjoint edge folds).
// 3-D requests run as fused whole-filter launches where a kernel applies
// (fused.cu: one adjoint launch for dL/dx, three launches dotting D_a x with
// ybar for dL/dsigma); everything else runs per axis on f32 buffers from the
// stream-ordered scratch pool.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "geom.hpp"
#include "internal.hpp"

namespace itkg {
namespace {

struct AxisCoeffs {
  int r = 0;
  std::vector<float> w, dw, prefix;
};

void make_coeffs(double sigma, double spacing, int r, AxisCoeffs* c) {
  const double s = sigma / spacing;
  const int K = 2 * r + 1;
  std::vector<double> g(K), gp(K);
  double S = 0.0, Sp = 0.0;
  for (int i = 0; i < K; ++i) {
    const double t = ((double)i - (double)r) / s;
    g[i] = std::exp(-0.5 * (t * t));
    gp[i] = g[i] * t * t / s;
  }
  for (int i = 0; i < K; ++i) S += g[i];
  for (int i = 0; i < K; ++i) Sp += gp[i];
  c->r = r;
  c->w.resize(K);
  c->dw.resize(K);
  c->prefix.resize(K);
  double acc = 0.0;
  for (int i = 0; i < K; ++i) {
    const double w = g[i] / S;
    c->w[i] = (float)w;
    c->dw[i] = (float)((gp[i] * S - g[i] * Sp) / (S * S) / spacing);
    acc += w;
    c->prefix[i] = (float)acc;
  }
}

itkg_status check_f32_device(const itkg_image* im, const char* name, int D) {
  ITKG_TRY(validate_image(im, name));
  if (im->location != ITKG_DEVICE)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s: the VJP takes device buffers", name);
  if (im->dtype != ITKG_F32 || im->components != 1)
    return set_error(ITKG_ERROR_UNSUPPORTED, "%s: the VJP takes scalar f32 images", name);
  if (D && im->dim != D) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "%s: dim differs", name);
  return ITKG_SUCCESS;
}

bool same_size(const itkg_image& a, const itkg_image& b) {
  for (int d = 0; d < a.dim; ++d)
    if (a.region.size[d] != b.region.size[d] || a.region.index[d] != b.region.index[d]) return false;
  return true;
}

void view3(const itkg_image& im, int64_t* pitch, int64_t* size) {
  for (int d = 0; d < kMaxDim; ++d) {
    pitch[d] = d < im.dim ? im.pitch[d] : 0;
    size[d] = d < im.dim ? (int64_t)im.region.size[d] : 1;
  }
}

// Scratch images: dense f32 of the same size.
struct Scratch {
  std::vector<void*> ptrs;
  cudaStream_t s;
  explicit Scratch(cudaStream_t st) : s(st) {}
  ~Scratch() {
    for (void* p : ptrs) scratch_free(p, s);
  }
  itkg_status image(const itkg_image& like, itkg_image* out) {
    std::memset(out, 0, sizeof *out);
    out->dim = like.dim;
    out->dtype = ITKG_F32;
    out->components = 1;
    out->location = ITKG_DEVICE;
    out->region = like.region;
    dense_layout(out, 1);  // fully dense: the loss kernel indexes it linearly
    void* p = nullptr;
    ITKG_TRY(scratch_alloc(&p, image_bytes(*out), s));
    ptrs.push_back(p);
    out->data = p;
    return ITKG_SUCCESS;
  }
  itkg_status raw(size_t bytes, void** p) {
    ITKG_TRY(scratch_alloc(p, bytes, s));
    ptrs.push_back(*p);
    return ITKG_SUCCESS;
  }
};

VjpAxisArgs axis_args(const itkg_image& in, const itkg_image* din, const itkg_image& out,
                      const itkg_image* dout, int axis, int r, bool accumulate) {
  VjpAxisArgs a;
  std::memset(&a, 0, sizeof a);
  a.in = static_cast<const float*>(in.data);
  a.din = din ? static_cast<const float*>(din->data) : nullptr;
  a.out = static_cast<float*>(out.data);
  a.dout = dout ? static_cast<float*>(dout->data) : nullptr;
  int64_t sz[3];
  view3(in, a.in_pitch, sz);
  view3(out, a.out_pitch, a.size);
  a.axis = axis;
  a.radius = r;
  a.accumulate = accumulate ? 1 : 0;
  return a;
}

// xbar (+)= G^T ybar: passes along axes D-1 .. 0.
itkg_status adjoint_chain(const itkg_image& ybar, const AxisCoeffs* c, itkg_image* xbar,
                          bool accumulate, Scratch& sc) {
  const int D = ybar.dim;
  itkg_image t[2];
  if (D > 1) ITKG_TRY(sc.image(ybar, &t[0]));
  if (D > 2) ITKG_TRY(sc.image(ybar, &t[1]));
  const itkg_image* cur = &ybar;
  int k = 0;
  for (int a = D - 1; a >= 0; --a) {
    const bool last = a == 0;
    itkg_image* nxt = last ? xbar : &t[k++ & 1];
    ITKG_TRY(launch_adjoint_axis(axis_args(*cur, nullptr, *nxt, nullptr, a, c[a].r, last && accumulate),
                                 c[a].w.data(), c[a].prefix.data(), sc.s));
    cur = nxt;
  }
  return ITKG_SUCCESS;
}

// (y, dy/dsigma) of the forward: dual passes along axes 0 .. D-1.
itkg_status dual_chain(const itkg_image& x, const AxisCoeffs* c, itkg_image* y, itkg_image* dy,
                       Scratch& sc) {
  const int D = x.dim;
  itkg_image v[2], dv[2];
  for (int i = 0; i < 2 && i < D - 1; ++i) {
    ITKG_TRY(sc.image(x, &v[i]));
    ITKG_TRY(sc.image(x, &dv[i]));
  }
  const itkg_image* cv = &x;
  const itkg_image* cdv = nullptr;
  for (int a = 0; a < D; ++a) {
    const bool last = a == D - 1;
    itkg_image* nv = last ? y : &v[a & 1];
    itkg_image* ndv = last ? dy : &dv[a & 1];
    ITKG_TRY(launch_dual_axis(axis_args(*cv, cdv, *nv, ndv, a, c[a].r, false), c[a].w.data(),
                              c[a].dw.data(), sc.s));
    cv = nv;
    cdv = ndv;
  }
  return ITKG_SUCCESS;
}

itkg_status coeffs_for(const itkg_image& x, double sigma, AxisCoeffs* c) {
  if (!(sigma > 0.0) || !std::isfinite(sigma))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "the VJP needs a finite sigma > 0 (got %g)", sigma);
  for (int d = 0; d < x.dim; ++d) {
    const uint64_t r = kernel_radius(sigma, x.spacing[d]);
    if (2 * r + 1 > (uint64_t)kMaxVjpTaps)
      return set_error(ITKG_ERROR_UNSUPPORTED, "VJP radius %llu exceeds %d", (unsigned long long)r,
                       (kMaxVjpTaps - 1) / 2);
    make_coeffs(sigma, x.spacing[d], (int)r, &c[d]);
  }
  return ITKG_SUCCESS;
}

DotArgs dot_args(const itkg_image& p, const itkg_image& q) {
  DotArgs d;
  std::memset(&d, 0, sizeof d);
  d.p = static_cast<const float*>(p.data);
  d.q = static_cast<const float*>(q.data);
  view3(p, d.p_pitch, d.size);
  int64_t sz[3];
  view3(q, d.q_pitch, sz);
  return d;
}

// Fused geometry of a whole-image VJP launch: src over its own region, the
// request and the clamp bounds both the whole image.
FusedGeom whole_geom(const itkg_image& src, const itkg_image* dst, const AxisCoeffs* c) {
  FusedGeom g;
  std::memset(&g, 0, sizeof g);
  g.src = src.data;
  g.dst = dst ? dst->data : const_cast<void*>(src.data);
  const itkg_image& o = dst ? *dst : src;
  for (int d = 0; d < kMaxDim; ++d) {
    const bool in = d < src.dim;
    g.src_origin[d] = in ? src.region.index[d] : 0;
    g.src_size[d] = in ? (int64_t)src.region.size[d] : 1;
    g.src_pitch[d] = in ? src.pitch[d] : 0;
    g.dst_origin[d] = in ? o.region.index[d] : 0;
    g.dst_pitch[d] = in ? o.pitch[d] : 0;
    g.req_index[d] = g.src_origin[d];
    g.req_size[d] = g.src_size[d];
    g.lo[d] = g.src_origin[d];
    g.hi[d] = g.src_origin[d] + g.src_size[d] - 1;
    g.radius[d] = in ? c[d].r : 0;
  }
  g.dim = src.dim;
  g.comps = 1;
  g.in_dtype = ITKG_F32;
  g.out_dtype = ITKG_F32;
  g.rounding = ITKG_ROUND_FMA;
  return g;
}

}  // namespace
}  // namespace itkg

using namespace itkg;

extern "C" itkg_status itkg_gaussian_scale_stack_loss_vjp(
    const itkg_image* x, const itkg_image* target, const double* sigmas, int32_t nlevels,
    itkg_image* xbar, double* loss, double* sigma_bar, int32_t flags, void* stream) {
  ITKG_TRY(check_f32_device(x, "x", 0));
  ITKG_TRY(check_f32_device(target, "target", x->dim));
  if (!same_size(*x, *target)) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "x and target regions differ");
  if (xbar) {
    ITKG_TRY(check_f32_device(xbar, "xbar", x->dim));
    if (!same_size(*x, *xbar)) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "x and xbar regions differ");
  }
  if (!sigmas || nlevels < 1) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "need nlevels >= 1 sigmas");
  if (flags & ~ITKG_VJP_SIGMA_BAR_ON_DEVICE)
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "unknown flags 0x%x", flags);
  std::vector<AxisCoeffs> coeffs((size_t)nlevels * kMaxDim);
  for (int l = 0; l < nlevels; ++l) ITKG_TRY(coeffs_for(*x, sigmas[l], &coeffs[(size_t)l * kMaxDim]));
  const int64_t n = (int64_t)region_len(x->region, x->dim);
  if (n == 0) return ITKG_SUCCESS;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Scratch sc(s);
  itkg_image y, dy, yb;
  ITKG_TRY(sc.image(*x, &y));
  ITKG_TRY(sc.image(*x, &dy));
  ITKG_TRY(sc.image(*x, &yb));
  const int nb = dot_partial_blocks(n);
  void* part = nullptr;
  ITKG_TRY(sc.raw(sizeof(double) * (2 * nb + 1 + nlevels), &part));
  double* partials = static_cast<double*>(part);
  double* dloss = partials + 2 * nb;
  double* dsig = dloss + 1;
  const bool on_dev = flags & ITKG_VJP_SIGMA_BAR_ON_DEVICE;
  int fast_levels = 0;
  for (int l = 0; l < nlevels; ++l) {
    const AxisCoeffs* c = &coeffs[(size_t)l * kMaxDim];
    double* const sig_l = on_dev && sigma_bar ? sigma_bar + l : dsig + l;
    DotArgs t = dot_args(y, *target);  // q = target
    // Two-pass forward and VJP kernels where they apply (3-D, the dense scratch
    // rows 16-byte aligned): y_l, then ybar_l = 2 (y_l - t), then xbar and
    // dL/dsigma_l from the VJP kernels.
    VjpTwoPass v;
    v.x = x;
    v.ybar = &yb;
    v.xbar = xbar;
    v.sigma_out = sig_l;
    v.acc_x = l > 0;
    v.acc_sigma = false;
    for (int d = 0; d < x->dim; ++d) v.w[d] = c[d].w.data(), v.dw[d] = c[d].dw.data(), v.radius[d] = (int)c[d].r;
    if (x->dim == 3 && x->region.size[0] % 4 == 0 && launch_vjp_two_pass(v, s, true) == ITKG_SUCCESS) {
      itkg_gaussian_params p;
      std::memset(&p, 0, sizeof p);
      p.sigma = sigmas[l];
      p.arithmetic = ITKG_ARITH_F32;
      p.rounding = ITKG_ROUND_FMA;
      p.algorithm = ITKG_ALGO_AUTO;
      const itkg_region reg = x->region;
      ITKG_TRY(itkg_gaussian_generate_region(x, &reg, &reg, &p, &y, s));
      ITKG_TRY(launch_sqerr(static_cast<const float*>(y.data), nullptr, t, static_cast<float*>(yb.data),
                            partials, nb, dloss, nullptr, l > 0, s));
      ITKG_TRY(launch_vjp_two_pass(v, s, false));
      ++fast_levels;
      continue;
    }
    ITKG_TRY(dual_chain(*x, c, &y, &dy, sc));  // y_l and dy_l/dsigma_l, recomputed
    ITKG_TRY(launch_sqerr(static_cast<const float*>(y.data), static_cast<const float*>(dy.data), t,
                          static_cast<float*>(yb.data), partials, nb, dloss, sig_l, l > 0, s));
    if (xbar) ITKG_TRY(adjoint_chain(yb, c, xbar, l > 0, sc));
  }
  if (loss || (sigma_bar && !on_dev)) {
    std::vector<double> h(1 + nlevels);
    ITKG_CUDA(cudaMemcpyAsync(h.data(), dloss, sizeof(double) * (1 + nlevels), cudaMemcpyDeviceToHost, s));
    ITKG_CUDA(cudaStreamSynchronize(s));
    if (loss) *loss = h[0];
    if (sigma_bar && !on_dev)
      for (int l = 0; l < nlevels; ++l) sigma_bar[l] = h[1 + l];
  }
  set_last_kernel(fast_levels == nlevels ? "scale_stack_loss_vjp_two_pass_f32"
                  : fast_levels ? "scale_stack_loss_vjp_mixed_f32"
                                : "scale_stack_loss_vjp_per_axis_f32");
  return ITKG_SUCCESS;
}

extern "C" itkg_status itkg_gaussian_vjp(const itkg_image* x, const itkg_image* ybar,
                                         const itkg_gaussian_params* params, itkg_image* xbar,
                                         double* sigma_bar, int32_t flags, void* stream) {
  ITKG_TRY(check_f32_device(x, "x", 0));
  ITKG_TRY(check_f32_device(ybar, "ybar", x->dim));
  if (!params) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "params is NULL");
  if (!same_size(*x, *ybar)) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "x and ybar regions differ");
  if (xbar) {
    ITKG_TRY(check_f32_device(xbar, "xbar", x->dim));
    if (!same_size(*x, *xbar)) return set_error(ITKG_ERROR_INVALID_ARGUMENT, "x and xbar regions differ");
  }
  if (flags & ~(ITKG_VJP_ACCUMULATE_XBAR | ITKG_VJP_ACCUMULATE_SIGMA | ITKG_VJP_SIGMA_BAR_ON_DEVICE))
    return set_error(ITKG_ERROR_INVALID_ARGUMENT, "unknown flags 0x%x", flags);
  AxisCoeffs c[kMaxDim];
  ITKG_TRY(coeffs_for(*x, params->sigma, c));
  if (region_len(x->region, x->dim) == 0) return ITKG_SUCCESS;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Scratch sc(s);
  const int D = x->dim;
  const float* w[kMaxDim] = {nullptr, nullptr, nullptr};
  const float* P[kMaxDim] = {nullptr, nullptr, nullptr};
  for (int d = 0; d < D; ++d) w[d] = c[d].w.data(), P[d] = c[d].prefix.data();
  bool fused_x = false, fused_s = false;
  // ITKG_ALGO_PER_AXIS: the per-axis passes only (the plain form, for comparisons)
  const bool try_fused = D == 3 && params->algorithm != ITKG_ALGO_PER_AXIS;
  if (try_fused && params->algorithm != ITKG_ALGO_FUSED) {
    // z-adjoint and x-y kernels: xbar and sigma_bar in four launches
    VjpTwoPass v;
    v.x = x;
    v.ybar = ybar;
    v.xbar = xbar;
    v.acc_x = flags & ITKG_VJP_ACCUMULATE_XBAR;
    v.acc_sigma = (flags & ITKG_VJP_ACCUMULATE_SIGMA) && (flags & ITKG_VJP_SIGMA_BAR_ON_DEVICE);
    v.sigma_out = nullptr;
    for (int d = 0; d < D; ++d) v.w[d] = c[d].w.data(), v.dw[d] = c[d].dw.data(), v.radius[d] = (int)c[d].r;
    if (launch_vjp_two_pass(v, s, true) == ITKG_SUCCESS) {
      const bool on_dev = flags & ITKG_VJP_SIGMA_BAR_ON_DEVICE;
      double* dres = nullptr;
      if (sigma_bar) {
        if (on_dev) {
          v.sigma_out = sigma_bar;
        } else {
          void* res = nullptr;
          ITKG_TRY(sc.raw(sizeof(double), &res));
          dres = static_cast<double*>(res);
          v.sigma_out = dres;
        }
      }
      ITKG_TRY(launch_vjp_two_pass(v, s, false));
      if (sigma_bar && !on_dev) {
        double h = 0.0;
        ITKG_CUDA(cudaMemcpyAsync(&h, dres, sizeof h, cudaMemcpyDeviceToHost, s));
        ITKG_CUDA(cudaStreamSynchronize(s));
        *sigma_bar = (flags & ITKG_VJP_ACCUMULATE_SIGMA) ? *sigma_bar + h : h;
      }
      set_last_kernel("vjp_two_pass_f32");
      return ITKG_SUCCESS;
    }
  }
  if (xbar) {
    // fused adjoint (one pass) where a kernel applies, else D per-axis passes
    const FusedGeom g = whole_geom(*ybar, xbar, c);
    if (try_fused && launch_fused_vjp(2, g, w, P, nullptr, nullptr, nullptr, nullptr, nullptr, false, s,
                                      true) == ITKG_SUCCESS) {
      ITKG_TRY(launch_fused_vjp(2, g, w, P, nullptr, nullptr, nullptr, nullptr, nullptr,
                                flags & ITKG_VJP_ACCUMULATE_XBAR, s, false));
      fused_x = true;
    } else {
      ITKG_TRY(adjoint_chain(*ybar, c, xbar, flags & ITKG_VJP_ACCUMULATE_XBAR, sc));
    }
  }
  if (sigma_bar) {
    const bool on_dev = flags & ITKG_VJP_SIGMA_BAR_ON_DEVICE;
    const bool acc = flags & ITKG_VJP_ACCUMULATE_SIGMA;
    void* res = nullptr;
    ITKG_TRY(sc.raw(sizeof(double), &res));
    double* dres = static_cast<double*>(res);
    // dy/dsigma = sum_a D_a x, D_a the separable filter with dw/dsigma on axis a:
    // three fused launches that dot their output with ybar, or dual per-axis passes
    const FusedGeom g = whole_geom(*x, nullptr, c);
    int grid = 0;
    if (try_fused && launch_fused_vjp(1, g, w, nullptr, ybar->data, ybar->pitch, ybar->region.index, nullptr,
                                      &grid, false, s, true) == ITKG_SUCCESS) {
      void* part = nullptr;
      ITKG_TRY(sc.raw(sizeof(double) * 3 * grid, &part));
      double* partials = static_cast<double*>(part);
      for (int a = 0; a < 3; ++a) {
        const float* wa[kMaxDim] = {w[0], w[1], w[2]};
        wa[a] = c[a].dw.data();
        int g2 = 0;
        ITKG_TRY(launch_fused_vjp(1, g, wa, nullptr, ybar->data, ybar->pitch, ybar->region.index,
                                  partials + a * grid, &g2, false, s, false));
      }
      ITKG_TRY(launch_sum_partials(partials, 3 * grid, on_dev ? sigma_bar : dres, on_dev && acc, s));
      fused_s = true;
    } else {
      itkg_image y, dy;
      ITKG_TRY(sc.image(*x, &y));
      ITKG_TRY(sc.image(*x, &dy));
      ITKG_TRY(dual_chain(*x, c, &y, &dy, sc));
      const int nb = dot_partial_blocks((int64_t)region_len(x->region, x->dim));
      void* part = nullptr;
      ITKG_TRY(sc.raw(sizeof(double) * nb, &part));
      ITKG_TRY(launch_dot(dot_args(*ybar, dy), static_cast<double*>(part), nb,
                          on_dev ? sigma_bar : dres, on_dev && acc, s));
    }
    if (!on_dev) {
      double h = 0.0;
      ITKG_CUDA(cudaMemcpyAsync(&h, dres, sizeof h, cudaMemcpyDeviceToHost, s));
      ITKG_CUDA(cudaStreamSynchronize(s));
      *sigma_bar = acc ? *sigma_bar + h : h;
    }
  }
  set_last_kernel(fused_x || fused_s ? (fused_x && (fused_s || !sigma_bar) ? "vjp_fused_f32" : "vjp_mixed_f32")
                                     : "vjp_per_axis_f32");
  return ITKG_SUCCESS;
}
