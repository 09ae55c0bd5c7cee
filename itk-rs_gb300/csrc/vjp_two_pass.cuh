// Two-kernel-family VJP of the 3-D Gaussian (FMA rounding, f32, whole image).
// With G = Gz Gy Gx (clamped separable filter, fixed radii), ybar = dL/dy:
//   U  = Gz^T ybar,   U' = dGz^T ybar          (z adjoint kernel, k_z_adj)
//   xbar   = Gx^T Gy^T U                       (x-y kernel, adjoint mode)
//   sigma_bar = <U', Gy Gx x> + <U, (Gy dGx + dGy Gx) x>   (x-y kernel, dual-dot mode)
// because dy/dsigma = dGz Gy Gx x + Gz (Gy dGx + dGy Gx) x and Gz, Gy, Gx
// commute.  dG is the clamped filter with the weights' sigma derivatives (the
// radius frozen), so U' and the x-y dual pass reuse the same kernels.
//
// Boundaries.  Every kernel filters a zero-filled halo (TMA zero fill, or
// skipped slices on z).  The adjoint of the clamp folds the clamped taps onto
// the edge voxels: xbar[lo] += sum_{d<R} p[R-d] u[lo+d] (and mirrored at hi),
// p[j] = w[0] + ... + w[j-1]; the forward passes of the dual-dot mode add
// them back the other way: v[lo+d] += p[R-d] x[lo] for d < R.
#pragma once

#include "two_pass.cuh"

namespace itkg {
namespace vjp2 {

using twopass::kMaxK;
using twopass::kMaxR;
using twopass::kTileX;
using twopass::ld1;
using twopass::policy_evict_first;
using twopass::tma_load_3d_hint;
using fusedk::clampi;
using fusedk::load4;
using fusedk::mbar_expect_tx;
using fusedk::mbar_init;
using fusedk::mbar_wait;
using fusedk::smem_u32;

enum VjpMode { kAdjoint = 0, kDualDot = 1 };

struct XYVArgs {
  int32_t src_origin[3];
  int32_t lo[3], hi[3];  // the image (= the input buffer), inclusive
  int32_t ntx;           // tiles along x
  int32_t ns;            // slices
  int64_t units;         // tiles * slices
  unsigned int* fault;
  long long wait_limit;  // clock cycles a wait on a tile load may take
  // adjoint mode: xbar (f32), byte pitches; accumulate: xbar += result
  char* out;
  int64_t out_pitch[3];
  int32_t accumulate;
  int32_t pad_;
  // dual-dot mode: U (dotted with the derivative) and U' (with the value),
  // f32 with byte pitches; one f64 partial sum per CTA
  const char* u;
  const char* u2;
  int64_t u_pitch[3];
  double* partials;
  // weights: x as tap pairs (see two_pass.cuh) for w and dw, y as splat pairs
  f2_t we[kMaxR + 1], wo[kMaxR + 1], dwe[kMaxR + 1], dwo[kMaxR + 1];
  f2_t wy2[kMaxK], dwy2[kMaxK];
  // exclusive prefix sums of the x / y weights and derivative weights
  float px[kMaxR + 1], py[kMaxR + 1], pdx[kMaxR + 1], pdy[kMaxR + 1];
};

struct ZAArgs {
  const char* in;          // ybar (f32), byte pitches
  int64_t in_pitch[3];
  char* out;               // U (f32), byte pitches, same region
  int64_t out_pitch[3];
  int32_t nx, ny, nz;      // the image
  int32_t nqx;             // quads per row
  int64_t units;           // quad blocks * nz
  f2_t wz2[kMaxK];         // z weights (w or dw) as splat pairs
  float pz[kMaxR + 1];     // their exclusive prefix sums
  // k_z_adj2: the second output (U' = dGz^T ybar) and its weights
  char* out2;
  int32_t npx;             // column pairs per row
  int32_t pad2_;
  f2_t wz2d[kMaxK];
  float pzd[kMaxR + 1];
};

template <int R, int MODE>
struct CfgXYV {
  static constexpr int K = 2 * R + 1;
  static constexpr int NT = 256;
  static constexpr int TX = kTileX;
  static constexpr int MY = 4;
  static constexpr int TY = 16 * MY;  // 64
  static constexpr int MX = 8;
  static constexpr int SEGS = TX / MX;
  static constexpr int XA = (R + 3) / 4 * 4;
  static constexpr int BW = TX + 2 * XA + 4;  // +4: conflict-free 16-byte row loads
  static constexpr int IH = TY + 2 * R;
  static constexpr int NTASK = IH * SEGS;
  static constexpr int OFF = (XA - R) % 4;
  static constexpr int WB = XA - R - OFF;
  static constexpr int WIN = (MX + 2 * R + OFF + (OFF & 1) + 3) / 4 * 4;
  static constexpr int S = 2;
  static constexpr int BOX = IH * BW * 4;
  static constexpr int STAGE = (BOX + 127) / 128 * 128;
  static constexpr int TXP = TX + 4;
  static constexpr int XBUF = IH * TXP;
  static constexpr int NXB = MODE == kDualDot ? 2 : 1;  // x-filtered tiles per slice (value, derivative)
  static constexpr size_t SMEM = (size_t)S * STAGE + sizeof(float) * 2 * NXB * XBUF + 128;
  static_assert(WB + TX - MX + WIN <= BW, "x window stays inside the staged row");
  static_assert(NTASK <= 2 * NT, "at most two x-pass tasks per thread");
};

// x pass of one task (8 outputs of one staged row) in tap-pair form over the
// zero-filled halo: with (we, wo) or (dwe, dwo).
template <int R, int WIN, int OFF, int MX>
__device__ __forceinline__ void xconv(const f2_t (&E)[WIN / 2], const f2_t* we, const f2_t* wo, float (&o)[MX]) {
#pragma unroll
  for (int m = 0; m < MX; ++m) {
    const int q0 = m + OFF;
    f2_t ax = mul2(E[q0 / 2], (q0 & 1) ? wo[0] : we[0]);
#pragma unroll
    for (int i = 1; i <= R; ++i) ax = fma2(E[q0 / 2 + i], (q0 & 1) ? wo[i] : we[i], ax);
    float lo2, hi2;
    unpack2(ax, lo2, hi2);
    o[m] = lo2 + hi2;
  }
}

template <int R, int MODE>
__global__ void __launch_bounds__(256, 2)
    k_xy_vjp(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ XYVArgs a) {
  using C = CfgXYV<R, MODE>;
  constexpr int K = C::K, TX = C::TX, TY = C::TY, MY = C::MY, MX = C::MX, BW = C::BW, IH = C::IH, XA = C::XA,
                S = C::S, WIN = C::WIN, WB = C::WB, OFF = C::OFF, NT = C::NT, SEGS = C::SEGS, TXP = C::TXP,
                NTASK = C::NTASK, XBUF = C::XBUF, NXB = C::NXB;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar[S];
  __shared__ int s_fail;
  __shared__ double red[NT / 32];
  unsigned char* const stage0 = smem + ((128u - (smem_u32(smem) & 127u)) & 127u);
  float* const xbuf0 = reinterpret_cast<float*>(stage0 + S * C::STAGE);  // [2 buffers][NXB][XBUF]
  const uint32_t sbase = smem_u32(stage0);
  const uint32_t bbase = smem_u32(mbar);
  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int i = 0; i < S; ++i) mbar_init(bbase + 8 * i, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    s_fail = 0;
  }
  __syncthreads();
  uint32_t phase_bits = 0;
  // dual-dot mode: this thread's share, summed in f32 over 4 slices at a time
  // and folded into f64 then (an f64 add per voxel would hold this GPU's slow
  // FP64 pipe longer than the whole f32 arithmetic)
  double dot = 0.0;
  float fdot = 0.0f;
  int fdot_n = 0;

  const int64_t u_begin = a.units * blockIdx.x / gridDim.x;
  const int64_t u_end = a.units * (blockIdx.x + 1) / gridDim.x;
  const uint64_t pol_in = policy_evict_first();

  const int row_a = tid / SEGS, x0_a = (tid % SEGS) * MX;
  const int row_b = (tid + NT) / SEGS, x0_b = ((tid + NT) % SEGS) * MX;
  const bool has_a = tid < NTASK, has_b = tid + NT < NTASK;
  const int lane16 = tid & 15, grp = tid >> 4;
  const float* const ywin0 = xbuf0 + grp * MY * TXP + 2 * lane16;

  // x pass of one task; nl / cr: staged columns of the image's first / last column
  auto xtask = [&](const float* tile, float* xb, int row, int x0, int nl, int cr) {
    const float* const src = tile + row * BW;
    float v[WIN];
#pragma unroll
    for (int q = 0; q < WIN / 4; ++q) load4(src + x0 + WB + 4 * q, v + 4 * q);
    f2_t E[WIN / 2];
#pragma unroll
    for (int q = 0; q < WIN / 2; ++q) E[q] = pack2(v[2 * q], v[2 * q + 1]);
    float o[MX];
    xconv<R, WIN, OFF, MX>(E, a.we, a.wo, o);
    const int c0 = x0 + XA;  // staged column of output 0
    if constexpr (MODE == kAdjoint) {
      // fold the clamped taps onto the edge columns
      if (nl >= c0 && nl < c0 + MX) {
        float f = 0.0f;
        for (int d = 0; d < R; ++d) f = fmaf(a.px[R - d], ld1(src + nl + d), f);
#pragma unroll
        for (int m = 0; m < MX; ++m)
          if (c0 + m == nl) o[m] += f;
      }
      if (cr >= c0 && cr < c0 + MX) {
        float f = 0.0f;
        for (int d = 0; d < R; ++d) f = fmaf(a.px[R - d], ld1(src + cr - d), f);
#pragma unroll
        for (int m = 0; m < MX; ++m)
          if (c0 + m == cr) o[m] += f;
      }
    } else {
      float od[MX];
      xconv<R, WIN, OFF, MX>(E, a.dwe, a.dwo, od);
      // add the clamped taps back to the outputs d < R inside an edge
      if (c0 < nl + R || c0 + MX - 1 > cr - R) {
        const float xl = ld1(src + max(nl, 0)), xr = ld1(src + min(cr, BW - 1));
#pragma unroll
        for (int m = 0; m < MX; ++m) {
          const int dl = c0 + m - nl, dr = cr - c0 - m;
          if (dl >= 0 && dl < R) {
            o[m] = fmaf(a.px[R - dl], xl, o[m]);
            od[m] = fmaf(a.pdx[R - dl], xl, od[m]);
          }
          if (dr >= 0 && dr < R) {
            o[m] = fmaf(a.px[R - dr], xr, o[m]);
            od[m] = fmaf(a.pdx[R - dr], xr, od[m]);
          }
        }
      }
      float4* d4 = reinterpret_cast<float4*>(xb + XBUF + row * TXP + x0);
#pragma unroll
      for (int q = 0; q < MX / 4; ++q) d4[q] = make_float4(od[4 * q], od[4 * q + 1], od[4 * q + 2], od[4 * q + 3]);
    }
    float4* d4 = reinterpret_cast<float4*>(xb + row * TXP + x0);
#pragma unroll
    for (int q = 0; q < MX / 4; ++q) d4[q] = make_float4(o[4 * q], o[4 * q + 1], o[4 * q + 2], o[4 * q + 3]);
  };

  int st_issue = 0, st_use = 0;
  int64_t n_issued = 0, n_consumed = 0;
  uint32_t issue_bits = 0;
  for (int64_t u = u_begin; u < u_end;) {
    const int64_t tile = u / a.ns;
    const int s_a = a.lo[2] + (int)(u - tile * a.ns);
    const int64_t left_u = u_end - u;
    const int ns_seg = (int)(a.lo[2] + a.ns - s_a < left_u ? a.lo[2] + a.ns - s_a : left_u);
    u += ns_seg;
    const int64_t tyi = tile / a.ntx;
    const int tix = (int)(tile - tyi * a.ntx);
    const int tx0 = a.lo[0] + tix * TX, ty0 = a.lo[1] + (int)tyi * TY;
    const int gx0 = tx0 - XA, gy0 = ty0 - R;
    const int nl = a.lo[0] - gx0, cr = a.hi[0] - gx0;
    const int rlo = a.lo[1] - gy0, rhi = a.hi[1] - gy0;  // staged rows of the image's first / last row
    const int col = tx0 + 2 * lane16;                    // this thread's first output column
    const int r0 = grp * MY + R;                         // staged row of this thread's output 0

    auto issue = [&](int sl) {
      if (tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        const uint32_t bar = bbase + 8 * st_issue;
        mbar_expect_tx(bar, (uint32_t)C::BOX);
        tma_load_3d_hint(sbase + (uint32_t)(st_issue * C::STAGE), &tmap, gx0 - a.src_origin[0],
                         gy0 - a.src_origin[1], sl - a.src_origin[2], bar, pol_in);
      }
      issue_bits ^= 1u << st_issue;  // parity of the loads issued into this stage
      st_issue = st_issue + 1 == S ? 0 : st_issue + 1;
      ++n_issued;
    };
    auto xpass = [&](float* xb) {
      const float* const tile_s = reinterpret_cast<const float*>(stage0 + st_use * C::STAGE);
      if (!mbar_wait(bbase + 8 * st_use, (phase_bits >> st_use) & 1u, a.wait_limit)) s_fail = 1;
      phase_bits ^= 1u << st_use;
      st_use = st_use + 1 == S ? 0 : st_use + 1;
      ++n_consumed;
      if (has_a) xtask(tile_s, xb, row_a, x0_a, nl, cr);
      if (has_b) xtask(tile_s, xb, row_b, x0_b, nl, cr);
    };

    for (int q = 0; q < S && q < ns_seg; ++q) issue(s_a + q);
    xpass(xbuf0);
    for (int i = 0; i < ns_seg; ++i) {
      __syncthreads();
      if (s_fail) goto timeout;
      if (i + S < ns_seg) issue(s_a + i + S);
      if (i + 1 < ns_seg) xpass(xbuf0 + ((i + 1) & 1) * NXB * XBUF);
      const int sl = s_a + i;
      const float* const xcur = xbuf0 + (i & 1) * NXB * XBUF;
      const float* const yw = ywin0 + (i & 1) * NXB * XBUF;
      // dual-dot: this slice's U and U' at the thread's outputs, loaded before
      // the y pass so that their latency overlaps its arithmetic
      const bool c0ok = col <= a.hi[0], c1ok = col + 1 <= a.hi[0];
      float pu[MY][2], pu2[MY][2];
      if constexpr (MODE == kDualDot) {
#pragma unroll
        for (int m = 0; m < MY; ++m) {
          const int y = ty0 + grp * MY + m;
          pu[m][0] = pu[m][1] = pu2[m][0] = pu2[m][1] = 0.0f;
          if (y > a.hi[1] || !c0ok) continue;
          const int64_t off = (int64_t)(col - a.lo[0]) * a.u_pitch[0] + (int64_t)(y - a.lo[1]) * a.u_pitch[1] +
                              (int64_t)(sl - a.lo[2]) * a.u_pitch[2];
          const float* const ud = reinterpret_cast<const float*>(a.u + off);
          const float* const uv = reinterpret_cast<const float*>(a.u2 + off);
          pu[m][0] = __ldg(ud);
          pu2[m][0] = __ldg(uv);
          if (c1ok) {
            pu[m][1] = __ldg(ud + 1);
            pu2[m][1] = __ldg(uv + 1);
          }
        }
      }
      f2_t yv[MY], yd[MY];
      {
        f2_t win[MY + 2 * R];
#pragma unroll
        for (int q = 0; q < MY + 2 * R; ++q) win[q] = *reinterpret_cast<const f2_t*>(yw + q * TXP);
#pragma unroll
        for (int m = 0; m < MY; ++m) {
          f2_t ay = 0ull, ad = 0ull;
#pragma unroll
          for (int k = 0; k < K; ++k) {
            ay = fma2(win[m + k], a.wy2[k <= R ? k : 2 * R - k], ay);
            if constexpr (MODE == kDualDot) ad = fma2(win[m + k], a.dwy2[k <= R ? k : 2 * R - k], ad);
          }
          yv[m] = ay;
          yd[m] = ad;
        }
      }
      if constexpr (MODE == kDualDot) {  // + Gy on the x derivative
        f2_t win[MY + 2 * R];
#pragma unroll
        for (int q = 0; q < MY + 2 * R; ++q) win[q] = *reinterpret_cast<const f2_t*>(yw + XBUF + q * TXP);
#pragma unroll
        for (int m = 0; m < MY; ++m) {
          f2_t ad = yd[m];
#pragma unroll
          for (int k = 0; k < K; ++k) ad = fma2(win[m + k], a.wy2[k <= R ? k : 2 * R - k], ad);
          yd[m] = ad;
        }
      }
      // y edges
      if (rlo > 0 || rhi < IH - 1) {
        if constexpr (MODE == kAdjoint) {
          // fold the clamped taps onto the edge rows
#pragma unroll
          for (int m = 0; m < MY; ++m) {
            if (r0 + m == rlo) {
              f2_t f = 0ull;
              for (int d = 0; d < R; ++d) {
                const float c = a.py[R - d];
                f = fma2(*reinterpret_cast<const f2_t*>(xcur + (rlo + d) * TXP + 2 * lane16), pack2(c, c), f);
              }
              yv[m] = add2(yv[m], f);
            }
            if (r0 + m == rhi) {
              f2_t f = 0ull;
              for (int d = 0; d < R; ++d) {
                const float c = a.py[R - d];
                f = fma2(*reinterpret_cast<const f2_t*>(xcur + (rhi - d) * TXP + 2 * lane16), pack2(c, c), f);
              }
              yv[m] = add2(yv[m], f);
            }
          }
        } else {
          // add the clamped taps back to the rows d < R inside an edge
          const int el = max(rlo, 0), eh = min(rhi, IH - 1);
          const f2_t xl = *reinterpret_cast<const f2_t*>(xcur + el * TXP + 2 * lane16);
          const f2_t xh = *reinterpret_cast<const f2_t*>(xcur + eh * TXP + 2 * lane16);
          const f2_t dl = *reinterpret_cast<const f2_t*>(xcur + XBUF + el * TXP + 2 * lane16);
          const f2_t dh = *reinterpret_cast<const f2_t*>(xcur + XBUF + eh * TXP + 2 * lane16);
#pragma unroll
          for (int m = 0; m < MY; ++m) {
            const int d0 = r0 + m - rlo, d1 = rhi - r0 - m;
            if (d0 >= 0 && d0 < R) {
              const float c = a.py[R - d0], cd = a.pdy[R - d0];
              yv[m] = fma2(xl, pack2(c, c), yv[m]);
              yd[m] = fma2(dl, pack2(c, c), fma2(xl, pack2(cd, cd), yd[m]));
            }
            if (d1 >= 0 && d1 < R) {
              const float c = a.py[R - d1], cd = a.pdy[R - d1];
              yv[m] = fma2(xh, pack2(c, c), yv[m]);
              yd[m] = fma2(dh, pack2(c, c), fma2(xh, pack2(cd, cd), yd[m]));
            }
          }
        }
      }
      // outputs: rows ty0 + grp*MY + m, columns col, col + 1 (inside the image only)
#pragma unroll
      for (int m = 0; m < MY; ++m) {
        const int y = ty0 + grp * MY + m;
        if (y > a.hi[1] || !c0ok) continue;
        float v0, v1;
        unpack2(yv[m], v0, v1);
        if constexpr (MODE == kAdjoint) {
          char* const p = a.out + (int64_t)(col - a.lo[0]) * a.out_pitch[0] + (int64_t)(y - a.lo[1]) * a.out_pitch[1] +
                          (int64_t)(sl - a.lo[2]) * a.out_pitch[2];
          float* const q0 = reinterpret_cast<float*>(p);
          float* const q1 = reinterpret_cast<float*>(p + a.out_pitch[0]);
          if (a.accumulate) {
            v0 += *q0;
            if (c1ok) v1 += *q1;
          }
          *q0 = v0;
          if (c1ok) *q1 = v1;
        } else {
          float d0, d1;
          unpack2(yd[m], d0, d1);
          float s = fmaf(v0, pu2[m][0], d0 * pu[m][0]);
          if (c1ok) s = fmaf(v1, pu2[m][1], fmaf(d1, pu[m][1], s));
          fdot += s;
        }
      }
      if constexpr (MODE == kDualDot) {
        if (++fdot_n == 4) {
          dot += (double)fdot;
          fdot = 0.0f;
          fdot_n = 0;
        }
      }
    }
    __syncthreads();
  }
  if constexpr (MODE == kDualDot) {
    dot += (double)fdot;
    const int lane = tid & 31, warp = tid >> 5;
    for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
    if (lane == 0) red[warp] = dot;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < NT / 32; ++w) t += red[w];
      a.partials[blockIdx.x] = t;
    }
  }
  return;
timeout:
  if (tid == 0) {
    atomicExch(a.fault, 1u);
    // let every tile load this CTA issued land before it exits (default
    // bound): the latest load into each stage, the one given up on included
    (void)n_consumed;
    for (int q = 0; q < S && q < n_issued; ++q) mbar_wait(bbase + 8 * q, ((issue_bits >> q) & 1u) ^ 1u);
    if constexpr (MODE == kDualDot) a.partials[blockIdx.x] = 0.0;
  }
}

// z adjoint: out = Gz^T in over the whole image (zero outside it, the clamped
// taps folded onto the first and last slice).  One thread marches one quad of
// 4 columns of a row through z; a cp.async ring of KZ slices per thread.
template <int RZ>
__global__ void __launch_bounds__(256, RZ <= 8 ? 2 : 1) k_z_adj(const __grid_constant__ ZAArgs a) {
  constexpr int KZ = 2 * RZ + 1, S = KZ, NT = 256;
  extern __shared__ __align__(16) float4 zring[];  // [S][NT]
  const int tid = threadIdx.x;
  const int64_t u_begin = a.units * blockIdx.x / gridDim.x;
  const int64_t u_end = a.units * (blockIdx.x + 1) / gridDim.x;
  const uint32_t my_slot0 = smem_u32(zring + tid);
  const uint64_t pol = policy_evict_first();
  const int64_t nq = (int64_t)a.nqx * a.ny;

  for (int64_t u = u_begin; u < u_end;) {
    const int64_t blk = u / a.nz;
    const int zs = (int)(u - blk * a.nz);
    const int64_t zrem = zs + (u_end - u);
    const int ze = zrem < a.nz ? (int)zrem : a.nz;
    u += ze - zs;
    const int64_t q = blk * NT + tid;
    if (q >= nq) continue;
    const int cy = (int)(q / a.nqx), qx = (int)(q - (int64_t)cy * a.nqx);
    const int cx = 4 * qx;
    const int jb = zs - RZ, je = ze - 1 + RZ;
    const char* const src = a.in + (int64_t)cx * a.in_pitch[0] + (int64_t)cy * a.in_pitch[1];
    int jn = jb;
    auto prefetch = [&](int stage) {  // slice jn, clamped to the image (a valid address)
      twopass::cp_async16_hint(my_slot0 + (uint32_t)(stage * NT * 16),
                               src + (int64_t)clampi(jn, 0, a.nz - 1) * a.in_pitch[2], pol);
      fusedk::cp_async_commit();
      ++jn;
    };
#pragma unroll
    for (int i = 0; i < S; ++i) prefetch(i);
    f2_t acc[2][KZ];
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
      for (int k = 0; k < KZ; ++k) acc[m][k] = 0ull;
    f2_t flo[2] = {0ull, 0ull}, fhi[2] = {0ull, 0ull};
    const int ncols = min(4, a.nx - cx);
    char* dz = a.out + (int64_t)cx * a.out_pitch[0] + (int64_t)cy * a.out_pitch[1] + (int64_t)zs * a.out_pitch[2];
    for (int jbase = jb; jbase <= je; jbase += KZ) {
#pragma unroll
      for (int p = 0; p < KZ; ++p) {
        const int j = jbase + p;
        if (j > je) break;
        fusedk::cp_async_wait<S - 1>();
        const float4 f = zring[p * NT + tid];
        prefetch(p);
        const bool inside = j >= 0 && j < a.nz;  // outside: zero (no contribution)
        const f2_t v0 = inside ? pack2(f.x, f.y) : 0ull, v1 = inside ? pack2(f.z, f.w) : 0ull;
#pragma unroll
        for (int k = 0; k < KZ; ++k) {
          const int slot = (p - k + KZ) % KZ;
          const f2_t wk = a.wz2[k <= RZ ? k : 2 * RZ - k];
          acc[0][slot] = k == 0 ? mul2(v0, wk) : fma2(v0, wk, acc[0][slot]);
          acc[1][slot] = k == 0 ? mul2(v1, wk) : fma2(v1, wk, acc[1][slot]);
        }
        // folds: the clamped taps of slices 0 .. R-1 onto slice 0, of the last R onto the last
        if (inside && j < RZ) {
          const float c = a.pz[RZ - j];
          flo[0] = fma2(v0, pack2(c, c), flo[0]);
          flo[1] = fma2(v1, pack2(c, c), flo[1]);
        }
        if (inside && j > a.nz - 1 - RZ) {
          const float c = a.pz[RZ - (a.nz - 1 - j)];
          fhi[0] = fma2(v0, pack2(c, c), fhi[0]);
          fhi[1] = fma2(v1, pack2(c, c), fhi[1]);
        }
        const int D = (p + 1) % KZ;
        const int z = j - RZ;
        if (z >= zs) {
          f2_t d0 = acc[0][D], d1 = acc[1][D];
          if (z == 0) d0 = add2(d0, flo[0]), d1 = add2(d1, flo[1]);
          if (z == a.nz - 1) d0 = add2(d0, fhi[0]), d1 = add2(d1, fhi[1]);
          float o[4];
          unpack2(d0, o[0], o[1]);
          unpack2(d1, o[2], o[3]);
          if (ncols == 4) {
            *reinterpret_cast<float4*>(dz) = make_float4(o[0], o[1], o[2], o[3]);
          } else {
#pragma unroll
            for (int c = 0; c < 4; ++c)
              if (c < ncols) reinterpret_cast<float*>(dz)[c] = o[c];
          }
          dz += a.out_pitch[2];
        }
      }
    }
    fusedk::cp_async_wait<0>();
  }
}

// Both z adjoints at once: U = Gz^T ybar and U' = dGz^T ybar from one pass over
// ybar.  One thread marches one pair of columns (8-byte loads into its own
// cp.async ring) with two rings of 2 RZ + 1 packed accumulators, one per
// weight set; otherwise as k_z_adj.
__device__ __forceinline__ void cp_async8(uint32_t s, const void* g) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(g) : "memory");
}

template <int RZ>
__global__ void __launch_bounds__(256, RZ <= 6 ? 2 : 1) k_z_adj2(const __grid_constant__ ZAArgs a) {
  constexpr int KZ = 2 * RZ + 1, S = KZ, NT = 256;
  extern __shared__ __align__(16) float2 zring2[];  // [S][NT]
  const int tid = threadIdx.x;
  const int64_t u_begin = a.units * blockIdx.x / gridDim.x;
  const int64_t u_end = a.units * (blockIdx.x + 1) / gridDim.x;
  const uint32_t my_slot0 = smem_u32(zring2 + tid);
  const int64_t np = (int64_t)a.npx * a.ny;

  for (int64_t u = u_begin; u < u_end;) {
    const int64_t blk = u / a.nz;
    const int zs = (int)(u - blk * a.nz);
    const int64_t zrem = zs + (u_end - u);
    const int ze = zrem < a.nz ? (int)zrem : a.nz;
    u += ze - zs;
    const int64_t q = blk * NT + tid;
    if (q >= np) continue;
    const int cy = (int)(q / a.npx), px = (int)(q - (int64_t)cy * a.npx);
    const int cx = 2 * px;
    const int jb = zs - RZ, je = ze - 1 + RZ;
    const char* const src = a.in + (int64_t)cx * a.in_pitch[0] + (int64_t)cy * a.in_pitch[1];
    int jn = jb;
    auto prefetch = [&](int stage) {  // slice jn, clamped to the image (a valid address)
      cp_async8(my_slot0 + (uint32_t)(stage * NT * 8), src + (int64_t)clampi(jn, 0, a.nz - 1) * a.in_pitch[2]);
      fusedk::cp_async_commit();
      ++jn;
    };
#pragma unroll
    for (int i = 0; i < S; ++i) prefetch(i);
    f2_t acc[2][KZ];  // [weight set][slot]
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
      for (int k = 0; k < KZ; ++k) acc[m][k] = 0ull;
    f2_t flo[2] = {0ull, 0ull}, fhi[2] = {0ull, 0ull};
    const bool two = cx + 1 < a.nx;
    const int64_t ooff = (int64_t)cx * a.out_pitch[0] + (int64_t)cy * a.out_pitch[1] + (int64_t)zs * a.out_pitch[2];
    char* dz = a.out + ooff;
    char* dz2 = a.out2 + ooff;
    for (int jbase = jb; jbase <= je; jbase += KZ) {
#pragma unroll
      for (int p = 0; p < KZ; ++p) {
        const int j = jbase + p;
        if (j > je) break;
        fusedk::cp_async_wait<S - 1>();
        const float2 f = zring2[p * NT + tid];
        prefetch(p);
        const bool inside = j >= 0 && j < a.nz;  // outside: zero (no contribution)
        const f2_t v = inside ? pack2(f.x, f.y) : 0ull;
#pragma unroll
        for (int k = 0; k < KZ; ++k) {
          const int slot = (p - k + KZ) % KZ;
          const int kk = k <= RZ ? k : 2 * RZ - k;
          acc[0][slot] = k == 0 ? mul2(v, a.wz2[kk]) : fma2(v, a.wz2[kk], acc[0][slot]);
          acc[1][slot] = k == 0 ? mul2(v, a.wz2d[kk]) : fma2(v, a.wz2d[kk], acc[1][slot]);
        }
        // folds: the clamped taps of slices 0 .. R-1 onto slice 0, of the last R onto the last
        if (inside && j < RZ) {
          const float c = a.pz[RZ - j], cd = a.pzd[RZ - j];
          flo[0] = fma2(v, pack2(c, c), flo[0]);
          flo[1] = fma2(v, pack2(cd, cd), flo[1]);
        }
        if (inside && j > a.nz - 1 - RZ) {
          const float c = a.pz[RZ - (a.nz - 1 - j)], cd = a.pzd[RZ - (a.nz - 1 - j)];
          fhi[0] = fma2(v, pack2(c, c), fhi[0]);
          fhi[1] = fma2(v, pack2(cd, cd), fhi[1]);
        }
        const int D = (p + 1) % KZ;
        const int z = j - RZ;
        if (z >= zs) {
          f2_t d0 = acc[0][D], d1 = acc[1][D];
          if (z == 0) d0 = add2(d0, flo[0]), d1 = add2(d1, flo[1]);
          if (z == a.nz - 1) d0 = add2(d0, fhi[0]), d1 = add2(d1, fhi[1]);
          float o0, o1, e0, e1;
          unpack2(d0, o0, o1);
          unpack2(d1, e0, e1);
          if (two) {
            *reinterpret_cast<float2*>(dz) = make_float2(o0, o1);
            *reinterpret_cast<float2*>(dz2) = make_float2(e0, e1);
          } else {
            *reinterpret_cast<float*>(dz) = o0;
            *reinterpret_cast<float*>(dz2) = e0;
          }
          dz += a.out_pitch[2];
          dz2 += a.out_pitch[2];
        }
      }
    }
    fusedk::cp_async_wait<0>();
  }
}

}  // namespace vjp2
}  // namespace itkg
