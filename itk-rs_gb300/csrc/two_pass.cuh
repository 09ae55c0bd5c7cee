// Two-kernel 3-D Gaussian forward: GaussianFilter::generate_region
// (src/filters/gaussian.rs:74-88) as
//   xy pass: per slice, the x pass and then the y pass of a TX x TY tile,
//            written to an f32 intermediate T (the reference's intermediate
//            after its second pass, restricted to the requested x-y range);
//   z pass:  the third pass, streaming T along z.
// Neither kernel recomputes anything along z, and the z pass needs no shared
// tile and no block barrier.  Long z ranges are split into chunks whose
// intermediate fits a budget, so T stays a bounded scratch buffer.
//
// xy pass.  A CTA runs a contiguous range of (tile, slice) units.  The
// (TX + 2XA) x (TY + 2RY) input tile of each unit lands in shared memory by one
// TMA tile load (S units in flight, mbarrier completion, bounded waits).  The
// x pass reads clamped rows and, on tiles at an x edge of the image, replaces
// the halo columns outside the image by the edge column in registers
// (clamp-to-edge, conv.rs:31-33).  It writes a double-buffered f32 tile, so the
// x pass of unit i + 1 and the y pass of unit i share one barrier interval.
// The y pass gives each thread two adjacent columns (one packed f32x2 register
// per row) and MY consecutive rows, read from a register window.  Row strides
// of the staged and x-filtered tiles are padded so that these shared-memory
// accesses are free of bank conflicts.
//
// z pass.  A thread owns four consecutive columns of one row of T and marches
// a z-segment: slice j is copied by cp.async into the thread's own shared
// memory ring (S slices ahead; no other thread reads it, so no barrier), then
// pushed into a ring of KZ packed accumulators (output z = j + RZ - k gets
// w[k] * v); output j - RZ is complete and stored.  The loop is unrolled over
// the KZ phases so every ring slot is a compile-time register.
//
// Reference rounding: scalar acc = acc + x * w with separate roundings, in
// ascending tap order from zero, on f32 intermediates -- bit-identical to the
// reference pass by pass.  FMA rounding: packed fma.rn.f32x2.
#pragma once

#include <type_traits>

#include "fused_kernel.cuh"
#include "unsharp.cuh"

namespace itkg {
namespace twopass {

using fusedk::clampi;
using fusedk::load4;
using fusedk::mbar_expect_tx;
using fusedk::mbar_init;
using fusedk::mbar_wait;
using fusedk::smem_u32;
using fusedk::tma_load_3d;

constexpr int kMaxR = 12;
constexpr int kMaxK = 2 * kMaxR + 1;
// x-y tile: kTileX columns and 128 rows (64 for R > 8); T is stored
// tile-major: [slice][tile][tile rows][kTileX columns]
constexpr int kTileX = 32;
// z-pass store modes (k_z_pass's ST)
constexpr int kStoreAny = 0, kStoreF32Quad = 1, kStoreBF16Quad = 2, kStoreF16Quad = 3, kStoreU8Quad = 4;
constexpr int kMaxZSplit = 1024;  // z-pass CTAs with a per-CTA unit range
constexpr int kTileY = 128;  // the tallest tile

struct XYArgs {
  float* t;            // intermediate, [slice][tile][row][col] (tile-major)
  int64_t t_slice;     // floats between slices of T (tiles * tile floats)
  int32_t src_origin[3];
  int32_t lo[3], hi[3];  // gather bounds (image within the input buffer), inclusive
  int32_t x0, y0;        // first requested column / row (absolute)
  int32_t s0, ns;        // first slice of this launch (absolute z) and slice count
  int32_t t_s0;          // absolute z of T's slice 0
  int32_t ntx, nty;      // tiles along x and y
  int64_t units;         // ntx * nty * ns
  unsigned int* fault;
  long long wait_limit;  // clock cycles a wait on a tile load may take
  float wx[kMaxK], wy[kMaxK];
  f2_t wx2[kMaxK], wy2[kMaxK];
  // FMA rounding, x pass: weight pairs for an output whose first tap is at an
  // even (we) or odd (wo) window position, we[i] = (w[2i], w[2i+1]) and
  // wo[i] = (w[2i-1], w[2i]) with w[-1] = w[2R+1] = 0.
  f2_t we[kMaxR + 1], wo[kMaxR + 1];
  // FMA rounding: the weight of the clamped taps of each output column of the
  // first tile column (cxl) and of the last two (cxr, tile columns xr0 and
  // xr0 + 1), and of each output row of the first tile row (cyt) and of the
  // last two (cyb, tile rows yr0 and yr0 + 1): p[R - d] for an output d < R
  // inside an image edge (p[j] = w[0] + ... + w[j-1]; the same at both edges,
  // the kernel being symmetric), else 0.  Only these tiles reach an edge
  // (R < TX, TY).  edge: bit 0/1/2/3 = some coefficient of cxl/cxr/cyt/cyb is
  // nonzero.
  float cxl[kTileX], cxr[2 * kTileX], cyt[kTileY], cyb[2 * kTileY];
  int32_t xr0, yr0;
  int32_t edge;
  int32_t pad2_;
};

struct ZArgs {
  const float* t;
  int64_t t_slice;         // floats
  int32_t t_s0, t_s1;      // absolute z of T's first / last slice (the clamp bounds)
  int32_t nx, ny;          // requested columns / rows
  int32_t ntx;             // tiles along x
  int32_t tile_rows;       // rows of a T tile (64 or 128)
  int32_t z0, nz;          // output slices of this launch (absolute) and count
  int64_t units;           // quad blocks (256 quads each) * nz
  char* dst;               // output voxel (x0, y0, z0)
  int64_t dst_pitch[3];    // bytes
  int32_t out_dtype;
  int32_t vec_store;       // store mode of the launched variant (kStore*, see k_z_pass)
  const char* ush_src;     // UnsharpMaskFilter variant: input voxel (x0, y0, z0)
  int64_t ush_pitch[3];    // bytes
  UnsharpConsts ush;
  float wz[kMaxK];
  f2_t wz2[kMaxK];
  int32_t nsplit;          // > 0: CTA b processes units [split[b], split[b + 1]); 0: an even split
  int32_t split[kMaxZSplit + 1];
};

template <int R, typename Tin>
struct CfgXY {
  static constexpr int K = 2 * R + 1;
  static constexpr int ESZ = (int)sizeof(Tin);
  static constexpr int NT = 288;                // two x-pass tasks per thread (IH * SEGS <= 576)
  static constexpr int NTY = 256;               // threads of the y pass
  static constexpr int TX = kTileX;             // 16 lanes x 2 columns
  static constexpr int MY = R <= 8 ? 8 : 4;     // rows per thread in the y pass
  static constexpr int TY = (NTY / 16) * MY;    // 128 (64 for R > 8)
  static constexpr int MX = 8;                  // x outputs per x-pass task
  static constexpr int SEGS = TX / MX;
  static constexpr int AE = 16 / ESZ;
  static constexpr int XA = (R + AE - 1) / AE * AE;
  // Staged row: TX + 2XA columns; f32 rows get 4 more (loaded and unused) so
  // that consecutive rows start 16 banks + 4 apart (conflict-free 16-byte loads).
  static constexpr int PAD = 4;
  static constexpr int BW = TX + 2 * XA + (ESZ == 4 ? PAD : 0);
  static constexpr int IH = TY + 2 * R;
  static constexpr int NTASK = IH * SEGS;       // x-pass tasks per unit
  static constexpr int OFF = (XA - R) % 4;
  static constexpr int WB = XA - R - OFF;
  // window: the reference form reads MX + 2R elements from OFF; the tap-pair
  // form reads whole aligned pairs, one more when output MX - 1 starts even
  static constexpr int WIN = (MX + 2 * R + OFF + (OFF & 1) + 3) / 4 * 4;
  static constexpr int S = 2;                   // units in flight
  static constexpr int NXB = 2;                 // x-filtered tiles (2: one block barrier per slice)
  static constexpr int MINB = 2;                // CTAs per SM the register budget is set for
  static constexpr int BOX = IH * BW * ESZ;
  static constexpr int STAGE = (BOX + 127) / 128 * 128;
  static constexpr int TXP = TX + 4;            // x-filtered row stride (floats)
  static constexpr int XBUF = IH * TXP;         // floats per x-filtered tile
  static constexpr size_t SMEM = (size_t)S * STAGE + sizeof(float) * NXB * XBUF + 128;
  static_assert(WB + TX - MX + WIN <= BW, "x window stays inside the staged row");
  static_assert(TX % MX == 0, "x segments");
  static_assert(NTASK > NT && NTASK <= 2 * NT, "each thread runs one or two x-pass tasks");
  static_assert(TY <= kTileY, "tile height");
};

template <int RZ>
struct CfgZ {
  static constexpr int KZ = 2 * RZ + 1;
  static constexpr int NT = 256;
  static constexpr int QPT = 1;                 // quads (4 columns) per thread
  static constexpr int QB = NT * QPT;           // quads per block of work
  static constexpr int S = KZ;                  // slices in flight per thread: one per phase
  static constexpr size_t SMEM = (size_t)S * NT * 16 * QPT;
  static_assert((kTileX / 4 * 64) % QB == 0, "blocks of work tile the T tiles (64 or 128 rows)");
};

// ---------------------------------------------------------------------------
// L2 policies (createpolicy) for the cache hints of the loads and stores.
__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;\n" : "=l"(p));
  return p;
}
__device__ __forceinline__ void tma_load_3d_hint(uint32_t dst, const CUtensorMap* map, int x, int y, int z,
                                                 uint32_t bar, uint64_t pol) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1, {%2, %3, %4}], [%5], %6;\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar), "l"(pol)
      : "memory");
}
__device__ __forceinline__ void st_f2_hint(float* p, f2_t v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.b64 [%0], %1, %2;\n" ::"l"(p), "l"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ void cp_async16_hint(uint32_t s, const void* g, uint64_t pol) {
  asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;\n" ::"r"(s), "l"(g), "l"(pol)
               : "memory");
}

// One staged element -> f32 (exact).
__device__ __forceinline__ float ld1(const float* p) { return *p; }
__device__ __forceinline__ float ld1(const int16_t* p) { return (float)*p; }
__device__ __forceinline__ float ld1(const uint8_t* p) { return (float)*p; }
__device__ __forceinline__ float ld1(const __nv_bfloat16* p) { return __bfloat162float(*p); }
__device__ __forceinline__ float ld1(const __half* p) { return __half2float(*p); }

// ---------------------------------------------------------------------------
// u8 pixel arithmetic (GaussianFilter<Image<u8>>, NumericPixel for u8): each
// tap adds round(v as f64 * w).clamp(0, 255) as u8 to a u8 accumulator with a
// wrapping add, so a pass's output is the sum of its taps' values mod 256, in
// any order.  A tap's value is computed in f32: floor(fma(v, c, 0.5)) with a
// per-tap constant c that the host has checked against the f64 definition for
// all 256 values of v (an f32 near w; see u8_pixel_tap_consts).  Adding 2^23
// rounding down leaves floor(.) in the low mantissa bits of 2^23 + floor(.), a
// bit pattern whose low byte is the tap's value, so the taps' bit patterns are
// summed as integers and the sum's low byte is the pass's output.
__device__ __forceinline__ uint32_t u8p_tap(float v, float c) {
  return __float_as_uint(__fadd_rd(__fmaf_rn(v, c, 0.5f), 8388608.0f));
}
// the low byte of an accumulated sum, as an exact f32 (0 .. 255)
__device__ __forceinline__ float u8p_value(uint32_t acc) {
  return __fsub_rn(__uint_as_float(0x4B000000u | (acc & 255u)), 8388608.0f);
}

// ---------------------------------------------------------------------------
// xy pass
// U8P (with REF and u8 input): u8 pixel arithmetic; a.wx / a.wy hold the
// per-tap constants c, and T holds each y-pass output byte as an f32.
template <int R, bool REF, typename Tin, bool U8P = false>
__global__ void __launch_bounds__(288, CfgXY<R, Tin>::MINB)
    k_xy_pass(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ XYArgs a) {
  static_assert(!U8P || (REF && std::is_same<Tin, uint8_t>::value), "u8 pixel arithmetic: clamped u8 tiles");
  using C = CfgXY<R, Tin>;
  constexpr int K = C::K, TX = C::TX, TY = C::TY, MY = C::MY, MX = C::MX, BW = C::BW, IH = C::IH,
                XA = C::XA, S = C::S, WIN = C::WIN, WB = C::WB, OFF = C::OFF, NT = C::NT, SEGS = C::SEGS,
                TXP = C::TXP, NTASK = C::NTASK, NXB = C::NXB;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar[S];
  __shared__ int s_fail;
  unsigned char* const stage0 = smem + ((128u - (smem_u32(smem) & 127u)) & 127u);
  float* const xbuf0 = reinterpret_cast<float*>(stage0 + S * C::STAGE);
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

  // the dependent z pass may be scheduled now; it waits for this grid before reading T
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  // this grid is a programmatic dependent of the stream's previous kernel (which
  // may have written the input, or used the memory T now takes): wait for it
  // to complete before the first global memory access
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  const int64_t u_begin = a.units * blockIdx.x / gridDim.x;
  const int64_t u_end = a.units * (blockIdx.x + 1) / gridDim.x;
  const int n = (int)(u_end - u_begin);
  if (n <= 0) return;

  const uint64_t pol_in = policy_evict_first();
  const uint64_t pol_t = policy_evict_last();

  // this thread's x-pass tasks: (row, 8-column segment) tid and tid + NT (if < NTASK)
  const int row_a = tid / SEGS, x0_a = (tid % SEGS) * MX;
  const int row_b = (tid + NT) / SEGS, x0_b = ((tid + NT) % SEGS) * MX;
  const bool has_b = tid + NT < NTASK;
  // this thread's y-pass share: columns 2*lane16, +1; rows grp*MY .. +MY-1
  const int lane16 = tid & 15, grp = tid >> 4;
  const bool has_y = tid < C::NTY;
  const float* const ywin0 = xbuf0 + (has_y ? grp : 0) * MY * TXP + 2 * lane16;

  // One x-pass task: staged row `row`, columns x0 .. x0 + MX - 1 of the tile,
  // into xb.  nl / cr: staged columns of the image's first / last column;
  // rlo / rhi: staged rows of its first / last row.
  //   Reference rounding clamps: halo rows read the edge row, halo columns
  //   take the edge column's value (the reference's arithmetic exactly).
  //   FMA rounding filters the zero-filled halo (the input buffer lies inside
  //   the image) and adds the clamped taps back, p[R - d] * x[edge], to the
  //   outputs d < R columns inside an edge.
  auto xtask = [&](const Tin* tile, float* xb, int row, int x0, bool yedge, int rlo, int rhi, int xedge, int nl,
                   int cr) {
    float o[MX];
    if constexpr (REF) {
      const int srow = yedge ? min(max(row, rlo), rhi) : row;
      const Tin* const src = tile + srow * BW;
      float v[WIN];
#pragma unroll
      for (int q = 0; q < WIN / 4; ++q) load4(src + x0 + WB + 4 * q, v + 4 * q);
      if (xedge) {
        const float vl = ld1(src + max(nl, 0)), vr = ld1(src + min(cr, BW - 1));
        const int c0 = x0 + WB;
#pragma unroll
        for (int q = 0; q < WIN; ++q) {
          v[q] = c0 + q < nl ? vl : v[q];
          v[q] = c0 + q > cr ? vr : v[q];
        }
      }
#pragma unroll
      for (int m = 0; m < MX; ++m) {
        if constexpr (U8P) {
          uint32_t ia = 0;
#pragma unroll
          for (int k = 0; k < K; ++k) ia += u8p_tap(v[m + k + OFF], a.wx[k]);
          o[m] = u8p_value(ia);
        } else {
          float ax = 0.0f;
#pragma unroll
          for (int k = 0; k < K; ++k) ax = tap<true>(ax, v[m + k + OFF], a.wx[k]);
          o[m] = ax;
        }
      }
    } else {
      (void)yedge, (void)rlo, (void)rhi;
      const Tin* const src = tile + row * BW;
      float v[WIN];
#pragma unroll
      for (int q = 0; q < WIN / 4; ++q) load4(src + x0 + WB + 4 * q, v + 4 * q);
      // tap pairs over the aligned window pairs (no pair-forming moves): output m
      // sums E[j] * we[i] (first tap even) or * wo[i] (odd), then its two lanes
      f2_t E[WIN / 2];
#pragma unroll
      for (int q = 0; q < WIN / 2; ++q) E[q] = pack2(v[2 * q], v[2 * q + 1]);
#pragma unroll
      for (int m = 0; m < MX; ++m) {
        const int q0 = m + OFF;
        f2_t ax = mul2(E[q0 / 2], (q0 & 1) ? a.wo[0] : a.we[0]);
#pragma unroll
        for (int i = 1; i <= R; ++i) ax = fma2(E[q0 / 2 + i], (q0 & 1) ? a.wo[i] : a.we[i], ax);
        float lo2, hi2;
        unpack2(ax, lo2, hi2);
        o[m] = lo2 + hi2;
      }
      if (xedge) {  // here: bit 0 = first tile column, bit 1 = last, with corrections
        if (xedge & 1) {
          const float xl = ld1(src + nl);
#pragma unroll
          for (int m = 0; m < MX; ++m) o[m] = fmaf(a.cxl[x0 + m], xl, o[m]);
        }
        if (xedge & 2) {  // (xedge >> 2): which of the last two tile columns
          const float xr = ld1(src + min(cr, BW - 1));
          const float* const c = a.cxr + (xedge >> 2) * TX + x0;
#pragma unroll
          for (int m = 0; m < MX; ++m) o[m] = fmaf(c[m], xr, o[m]);
        }
      }
    }
    float4* d4 = reinterpret_cast<float4*>(xb + row * TXP + x0);
#pragma unroll
    for (int q = 0; q < MX / 4; ++q) d4[q] = make_float4(o[4 * q], o[4 * q + 1], o[4 * q + 2], o[4 * q + 3]);
  };
  int st_issue = 0, st_use = 0;       // stage ring positions (uniform)
  int64_t n_issued = 0, n_consumed = 0;  // tile loads issued / waited for (uniform)
  uint32_t issue_bits = 0;

  // The CTA's units are a run of slices of one tile, or the tail of one tile's
  // slices and the head of the next: one or two segments, each marching z.
  for (int64_t u = u_begin; u < u_end;) {
    const int64_t tile = u / a.ns;
    const int s_a = a.s0 + (int)(u - tile * a.ns);
    const int64_t left_u = u_end - u;
    const int ns_seg = (int)(a.s0 + a.ns - s_a < left_u ? a.s0 + a.ns - s_a : left_u);
    u += ns_seg;
    const int64_t tyi = tile / a.ntx;
    const int tix = (int)(tile - tyi * a.ntx);
    const int tx0 = a.x0 + tix * TX, ty0 = a.y0 + (int)tyi * TY;
    const int gx0 = tx0 - XA, gy0 = ty0 - R;
    // tile geometry, fixed over the segment
    const int nl = a.lo[0] - gx0;  // first in-image staged column (> 0 only at the left edge)
    const int cr = a.hi[0] - gx0;  // last in-image staged column (< BW - 1 only at the right edge)
    const int rlo = a.lo[1] - gy0, rhi = a.hi[1] - gy0;
    const bool yedge = rlo > 0 || rhi < IH - 1;
    int xedge;
    if constexpr (REF) {
      xedge = (nl > 0 || cr < BW - 1) ? 1 : 0;
    } else {  // first / last two tile columns with clamped taps to add back
      const int tcol = tix - a.xr0;
      xedge = (tix == 0 && (a.edge & 1) ? 1 : 0) | ((tcol >= 0) && (a.edge & 2) ? 2 | (tcol << 2) : 0);
    }
    const int trow = (int)tyi - a.yr0;
    const bool top = !REF && (a.edge & 4) && tyi == 0;
    const bool bot = !REF && (a.edge & 8) && trow >= 0 && rhi < IH;
    // T block of this tile; rows and columns beyond the request are stored too
    float* tp = a.t + (int64_t)(s_a - a.t_s0) * a.t_slice + tile * (TX * TY) + grp * MY * TX + 2 * lane16;

    auto issue = [&](int sl) {  // tile load of slice sl into the next stage
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
    auto xpass = [&](float* xb) {  // waits for the oldest load, x pass into xb
      const Tin* const tile_s = reinterpret_cast<const Tin*>(stage0 + st_use * C::STAGE);
      if (!mbar_wait(bbase + 8 * st_use, (phase_bits >> st_use) & 1u, a.wait_limit)) s_fail = 1;  // checked after the next barrier
      phase_bits ^= 1u << st_use;
      st_use = st_use + 1 == S ? 0 : st_use + 1;
      ++n_consumed;
      xtask(tile_s, xb, row_a, x0_a, yedge, rlo, rhi, xedge, nl, cr);
      if (has_b) xtask(tile_s, xb, row_b, x0_b, yedge, rlo, rhi, xedge, nl, cr);
    };

    // y pass of the x-filtered tile xb into T
    auto ypass = [&](const float* xb) {
      if (has_y) {
        const float* const yw = ywin0 + (xb - xbuf0);
        f2_t win[MY + 2 * R];
#pragma unroll
        for (int q = 0; q < MY + 2 * R; ++q) win[q] = *reinterpret_cast<const f2_t*>(yw + q * TXP);
        f2_t yv[MY];
#pragma unroll
        for (int m = 0; m < MY; ++m) {
          if constexpr (U8P) {
            uint32_t i0 = 0, i1 = 0;
#pragma unroll
            for (int k = 0; k < K; ++k) {
              float v0, v1;
              unpack2(win[m + k], v0, v1);
              i0 += u8p_tap(v0, a.wy[k]);
              i1 += u8p_tap(v1, a.wy[k]);
            }
            yv[m] = pack2(u8p_value(i0), u8p_value(i1));
          } else if constexpr (REF) {
            float y0 = 0.0f, y1 = 0.0f;
#pragma unroll
            for (int k = 0; k < K; ++k) {
              float v0, v1;
              unpack2(win[m + k], v0, v1);
              y0 = tap<true>(y0, v0, a.wy[k]);
              y1 = tap<true>(y1, v1, a.wy[k]);
            }
            yv[m] = pack2(y0, y1);
          } else {
            f2_t ay = 0ull;
#pragma unroll
            for (int k = 0; k < K; ++k) ay = fma2(win[m + k], a.wy2[k <= R ? k : 2 * R - k], ay);
            yv[m] = ay;
          }
        }
        if constexpr (!REF) {
          // first / last two tile rows: the clamped taps, c[row] * X[edge row]
          if (top) {
            const f2_t xe = *reinterpret_cast<const f2_t*>(xb + rlo * TXP + 2 * lane16);
#pragma unroll
            for (int m = 0; m < MY; ++m) {
              const float c = a.cyt[grp * MY + m];
              yv[m] = fma2(xe, pack2(c, c), yv[m]);
            }
          }
          if (bot) {
            const f2_t xe = *reinterpret_cast<const f2_t*>(xb + rhi * TXP + 2 * lane16);
#pragma unroll
            for (int m = 0; m < MY; ++m) {
              const float c = a.cyb[trow * TY + grp * MY + m];
              yv[m] = fma2(xe, pack2(c, c), yv[m]);
            }
          }
        }
#pragma unroll
        for (int m = 0; m < MY; ++m) st_f2_hint(tp + m * TX, yv[m], pol_t);
      }
    };

    for (int q = 0; q < S && q < ns_seg; ++q) issue(s_a + q);
    xpass(xbuf0);
    for (int i = 0; i < ns_seg; ++i) {
      const float* const xb = xbuf0 + (NXB == 2 ? (i & 1) * C::XBUF : 0);
      // x pass of slice i visible (and, with two x-filtered tiles, the y pass
      // of slice i - 1 done with the other one)
      __syncthreads();
      if (s_fail) goto timeout;
      if (i + S < ns_seg) issue(s_a + i + S);  // into the stage slice i's x pass has finished reading
      if constexpr (NXB == 2 && S >= 2) {
        if (i + 1 < ns_seg) xpass(xbuf0 + ((i + 1) & 1) * C::XBUF);
        ypass(xb);
      } else if constexpr (NXB == 2) {  // one stage: slice i + 1 lands during the y pass
        ypass(xb);
        if (i + 1 < ns_seg) xpass(xbuf0 + ((i + 1) & 1) * C::XBUF);
      } else {
        ypass(xb);
        __syncthreads();  // the y pass is done with the only x-filtered tile
        if (i + 1 < ns_seg) xpass(xbuf0);
      }
      tp += a.t_slice;
    }
    __syncthreads();  // the next segment reuses the x-filtered tiles
  }
  return;
timeout:
  if (tid == 0) {
    atomicExch(a.fault, 1u);
    // let every tile load this CTA issued land before it exits (default
    // bound): the latest load into each stage, the one given up on included
    (void)n_consumed;
    for (int q = 0; q < S && q < n_issued; ++q) mbar_wait(bbase + 8 * q, ((issue_bits >> q) & 1u) ^ 1u);
  }
}

// ---------------------------------------------------------------------------
// z pass
// ST: how a completed quad is stored.  kStoreAny: element by element, any
// output type and width.  kStoreF32Quad: one 16-byte store (f32 output whose
// rows allow it and whose width is a multiple of 4, every quad full).
// kStoreBF16Quad / kStoreF16Quad: the same for bf16 / f16 output, one 8-byte
// store of the four rounded values.  kStoreU8Quad (U8P only): one 4-byte store.
// U8P (with REF): u8 pixel arithmetic over T's bytes (see u8p_tap), a.wz
// holding the per-tap constants; the output is u8.
// USH (with kStoreF32Quad): store UnsharpMaskFilter's
// point-wise step of the input voxel and the blur instead of the blur --
// unsharp_cheap_f32 in FMA rounding, the exact f32 test (unsharp_quad_exact,
// one out-of-line copy) in reference rounding; the input quads travel in a
// second cp.async ring beside the T quads (the input quad of output z rides
// with T slice z + RZ).
template <int RZ, bool REF, int ST, bool USH = false, bool U8P = false>
__global__ void __launch_bounds__(256, RZ <= 8 ? 2 : 1) k_z_pass(const __grid_constant__ ZArgs a) {
  static_assert(!USH || ST == kStoreF32Quad, "the unsharp variant stores whole f32 quads");
  static_assert(!U8P || (REF && !USH && (ST == kStoreAny || ST == kStoreU8Quad)), "u8 pixel arithmetic stores u8");
  static_assert(ST != kStoreU8Quad || U8P, "the u8 quad store is the u8 pixel arithmetic's");
  using C = CfgZ<RZ>;
  constexpr int KZ = C::KZ, S = C::S, NT = C::NT;
  static_assert(C::QPT == 1, "one quad per thread");
  extern __shared__ __align__(16) float4 zring[];  // [S][NT], then (USH) the input ring [S][NT]
  const int tid = threadIdx.x;
  const int64_t u_begin = a.nsplit > 0 ? (int64_t)a.split[blockIdx.x] : a.units * blockIdx.x / gridDim.x;
  const int64_t u_end = a.nsplit > 0 ? (int64_t)a.split[blockIdx.x + 1] : a.units * (blockIdx.x + 1) / gridDim.x;
  const uint32_t my_slot0 = smem_u32(zring + tid);
  const uint32_t my_oslot0 = smem_u32(zring + S * NT + tid);
  const uint64_t pol_t = policy_evict_first();
  // the next call's x-y grid may be scheduled now; it waits for this grid
  // before its first global memory access
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  // T is written by the x-y grid this launch depends on (programmatic dependent
  // launch): wait for it to complete and its writes to be visible
  asm volatile("griddepcontrol.wait;\n" ::: "memory");

  for (int64_t u = u_begin; u < u_end;) {
    const int64_t blk = u / a.nz;
    const int zs = (int)(u - blk * a.nz);
    const int64_t zrem = zs + (u_end - u);
    const int ze = zrem < a.nz ? (int)zrem : a.nz;
    u += ze - zs;
    // this thread's quad: T tile `tl`, quad w (row w / 8, columns 4 (w % 8) .. + 3)
    const int64_t q = blk * C::QB + tid;
    const int tile_q = a.tile_rows * (kTileX / 4);  // quads per tile
    const int64_t tl = q / tile_q;
    const int w = (int)(q - tl * tile_q);
    const int64_t tly = tl / a.ntx;
    const int cx = (int)(tl - tly * a.ntx) * kTileX + 4 * (w & (kTileX / 4 - 1));  // first column
    const int cy = (int)tly * a.tile_rows + w / (kTileX / 4);                      // row
    if (cy >= a.ny || cx >= a.nx) continue;  // no barriers in this kernel: idle threads just skip
    const int z0 = a.z0 + zs, z1 = a.z0 + ze;  // outputs [z0, z1)
    const int jb = z0 - RZ;
    // prefetch cursor: slice jn (clamped to T) at pn
    const float* const tq = a.t + tl * (4 * tile_q) + 4 * w;
    int jn = jb;
    const float* pn = tq + (int64_t)(clampi(jn, a.t_s0, a.t_s1) - a.t_s0) * a.t_slice;
    const char* const oq = USH ? a.ush_src + (int64_t)cx * 4 + (int64_t)cy * a.ush_pitch[1] : nullptr;
    auto prefetch = [&](int stage) {
      cp_async16_hint(my_slot0 + (uint32_t)(stage * NT * 16), pn, pol_t);
      if constexpr (USH) {  // the input quad of output jn - RZ (clamped to this run's outputs)
        const int zo = clampi(jn - RZ, z0, z1 - 1);
        cp_async16_hint(my_oslot0 + (uint32_t)(stage * NT * 16), oq + (int64_t)(zo - a.z0) * a.ush_pitch[2], pol_t);
      }
      fusedk::cp_async_commit();
      ++jn;
      pn += (jn > a.t_s0 && jn <= a.t_s1) ? a.t_slice : 0;
    };
#pragma unroll
    for (int i = 0; i < S; ++i) prefetch(i);
    f2_t acc[2][KZ];
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
      for (int k = 0; k < KZ; ++k) acc[m][k] = 0ull;
    const int ncols = min(4, a.nx - cx);
    char* dz = a.dst + (int64_t)cx * a.dst_pitch[0] + (int64_t)cy * a.dst_pitch[1] +
               (int64_t)(z0 - a.z0) * a.dst_pitch[2];
    // One slice at phase p (a constant once the callers' loops are unrolled):
    // slice j = (period start) + p sits in stage p; push it, refill the stage
    // with slice j + S, pop output j - RZ and store it if `store`.
    auto step = [&](int p, bool store) {
      fusedk::cp_async_wait<S - 1>();
      const float4 f = zring[p * NT + tid];
      float4 og;
      if constexpr (USH) og = zring[S * NT + p * NT + tid];
      f2_t v[2] = {pack2(f.x, f.y), pack2(f.z, f.w)};
      prefetch(p);
#pragma unroll
      for (int k = 0; k < KZ; ++k) {
        const int slot = (p - k + KZ) % KZ;
#pragma unroll
        for (int m = 0; m < 2; ++m) {
          if constexpr (U8P) {
            float v0, v1;
            unpack2(v[m], v0, v1);
            const uint32_t a0 = (uint32_t)acc[m][slot] + u8p_tap(v0, a.wz[k]);
            const uint32_t a1 = (uint32_t)(acc[m][slot] >> 32) + u8p_tap(v1, a.wz[k]);
            acc[m][slot] = ((f2_t)a1 << 32) | a0;
          } else if constexpr (REF) {
            float a0, a1, v0, v1;
            unpack2(acc[m][slot], a0, a1);
            unpack2(v[m], v0, v1);
            acc[m][slot] = pack2(__fadd_rn(a0, __fmul_rn(v0, a.wz[k])), __fadd_rn(a1, __fmul_rn(v1, a.wz[k])));
          } else if (k == 0) {  // first contribution to output j + RZ: its slot was popped
            acc[m][slot] = mul2(v[m], a.wz2[0]);
          } else {
            acc[m][slot] = fma2(v[m], a.wz2[k <= RZ ? k : 2 * RZ - k], acc[m][slot]);
          }
        }
      }
      const int D = (p + 1) % KZ;
      const f2_t d0 = acc[0][D], d1 = acc[1][D];
      if constexpr (REF) {  // reference rounding adds the first product to zero
        acc[0][D] = 0ull;
        acc[1][D] = 0ull;
      }
      if (!store) return;
      float o[4];
      if constexpr (U8P) {
        if constexpr (ST == kStoreU8Quad) {
          __stcs(reinterpret_cast<unsigned int*>(dz), (uint32_t)(d0 & 255u) | (uint32_t)((d0 >> 24) & 0xFF00u) |
                                                          (uint32_t)((d1 & 255u) << 16) | (uint32_t)((d1 >> 8) & 0xFF000000u));
          dz += a.dst_pitch[2];
          return;
        }
        o[0] = u8p_value((uint32_t)d0);
        o[1] = u8p_value((uint32_t)(d0 >> 32));
        o[2] = u8p_value((uint32_t)d1);
        o[3] = u8p_value((uint32_t)(d1 >> 32));
      } else {
        unpack2(d0, o[0], o[1]);
        unpack2(d1, o[2], o[3]);
      }
      if constexpr (USH) {
        if constexpr (REF)
          __stcs(reinterpret_cast<float4*>(dz), unsharp_quad_exact(og, o[0], o[1], o[2], o[3], a.ush));
        else
          __stcs(reinterpret_cast<float4*>(dz),
                 make_float4(unsharp_cheap_f32(og.x, o[0], a.ush), unsharp_cheap_f32(og.y, o[1], a.ush),
                             unsharp_cheap_f32(og.z, o[2], a.ush), unsharp_cheap_f32(og.w, o[3], a.ush)));
      } else if constexpr (ST == kStoreF32Quad) {
        __stcs(reinterpret_cast<float4*>(dz), make_float4(o[0], o[1], o[2], o[3]));
      } else if constexpr (ST == kStoreBF16Quad || ST == kStoreF16Quad) {
        uint32_t h[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          if constexpr (ST == kStoreBF16Quad) h[c] = __bfloat16_as_ushort(from_f32<__nv_bfloat16>(o[c]));
          else h[c] = __half_as_ushort(from_f32<__half>(o[c]));
        }
        __stcs(reinterpret_cast<uint2*>(dz), make_uint2(h[0] | (h[1] << 16), h[2] | (h[3] << 16)));
      } else {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          if (c >= ncols) break;
          char* const dp = dz + c * a.dst_pitch[0];
          switch (a.out_dtype) {
            case ITKG_F32: *reinterpret_cast<float*>(dp) = o[c]; break;
            case ITKG_BF16: *reinterpret_cast<__nv_bfloat16*>(dp) = from_f32<__nv_bfloat16>(o[c]); break;
            case ITKG_F16: *reinterpret_cast<__half*>(dp) = from_f32<__half>(o[c]); break;
            default: *reinterpret_cast<uint8_t*>(dp) = from_f32<uint8_t>(o[c]); break;
          }
        }
      }
      dz += a.dst_pitch[2];
    };
    // first period: slices z0 - RZ .. z0 + RZ; only the last one completes an output (z0)
#pragma unroll
    for (int p = 0; p < KZ; ++p) step(p, p == KZ - 1);
    // then every slice completes one: whole periods, then the tail
    const int rest = z1 - z0 - 1;
    const int nfull = rest / KZ, tail = rest - nfull * KZ;
    for (int it = 0; it < nfull; ++it) {
#pragma unroll
      for (int p = 0; p < KZ; ++p) step(p, true);
    }
#pragma unroll
    for (int p = 0; p < KZ; ++p) {
      if (p >= tail) break;
      step(p, true);
    }
    fusedk::cp_async_wait<0>();
  }
}

// ---------------------------------------------------------------------------
// Kernel tables
using XYFn = void (*)(const CUtensorMap, const XYArgs);
using ZFn = void (*)(const ZArgs);

struct XYEntry {
  int r;
  int dtype;
  XYFn fn[2];  // [ref]
  size_t smem;
  int nt;              // threads per CTA
  int tx, ty, bw, ih;  // tile, TMA box
};

template <int R, typename Tin>
XYEntry make_xy(int dtype) {
  using C = CfgXY<R, Tin>;
  return XYEntry{R, dtype, {k_xy_pass<R, false, Tin>, k_xy_pass<R, true, Tin>}, C::SMEM, C::NT, C::TX, C::TY, C::BW,
                 C::IH};
}

// Tables: two_pass.cu (f32 x-y), two_pass_in.cu (i16, u8, bf16, f16 x-y), two_pass_z*.cu (z).
const XYEntry* xy_entries_f32(int* n);
const XYEntry* xy_entries_i16(int* n);
const XYEntry* xy_entries_u8(int* n);
const XYEntry* xy_entries_bf16(int* n);
const XYEntry* xy_entries_f16(int* n);
ZFn z_fn(int r, bool ref, int store, bool ush = false);
// The plain z kernels, split over translation units so they compile in
// parallel: [r - 1] of each row is k_z_pass<r, REF, ST>.
const ZFn* z_row_fma_any();     // two_pass_z.cu: REF false, kStoreAny
const ZFn* z_row_fma_f32q();    //                REF false, kStoreF32Quad
const ZFn* z_row_ref_any();     // two_pass_zref.cu: REF true, kStoreAny
const ZFn* z_row_ref_f32q();    //                   REF true, kStoreF32Quad
const ZFn* z_row_fma_bf16q();   // two_pass_znarrow.cu: REF false, kStoreBF16Quad
const ZFn* z_row_fma_f16q();    //                      REF false, kStoreF16Quad
const ZFn* z_row_ref_bf16q();   // two_pass_znarrow_ref.cu: REF true, kStoreBF16Quad
const ZFn* z_row_ref_f16q();    //                          REF true, kStoreF16Quad
// two_pass_u8p.cu: the u8 pixel-arithmetic kernels, [r - 1]
const XYEntry* xy_entries_u8p(int* n);
const ZFn* z_row_u8p_any();
const ZFn* z_row_u8p_u8q();
ZFn z_ush_fn(int r, bool ref);  // two_pass_ush.cu

#define ITKG_Z_ROW(REF, ST)                                                                             \
  {                                                                                                     \
    k_z_pass<1, REF, ST>, k_z_pass<2, REF, ST>, k_z_pass<3, REF, ST>, k_z_pass<4, REF, ST>,             \
        k_z_pass<5, REF, ST>, k_z_pass<6, REF, ST>, k_z_pass<7, REF, ST>, k_z_pass<8, REF, ST>,         \
        k_z_pass<9, REF, ST>, k_z_pass<10, REF, ST>, k_z_pass<11, REF, ST>, k_z_pass<12, REF, ST>       \
  }

#define ITKG_XY_TABLE(T, DT)                                                                      \
  {                                                                                              \
    make_xy<1, T>(DT), make_xy<2, T>(DT), make_xy<3, T>(DT), make_xy<4, T>(DT), make_xy<5, T>(DT), \
        make_xy<6, T>(DT), make_xy<7, T>(DT), make_xy<8, T>(DT), make_xy<9, T>(DT),               \
        make_xy<10, T>(DT), make_xy<11, T>(DT), make_xy<12, T>(DT)                                \
  }

}  // namespace twopass
}  // namespace itkg
