// One-trip 3-D Gaussian forward: GaussianFilter::generate_region
// (src/filters/gaussian.rs:74-88) with all three passes in one kernel, so that
// every input voxel is read from HBM once and every output voxel written once
// (the x-y halo of a tile comes from L2; nothing intermediate leaves the SM).
//
// A CTA (256 threads, two per SM) owns a TX x TY = 16 x 64 (x, y) tile and a
// z-segment of output slices [z0, z1); it marches the input slices
// z0 - RZ .. z1 - 1 + RZ (coordinates clamped to the image: the reference's
// clamp on z, conv.rs:31-33), SPI slices per barrier interval.  Three stages
// run in one interval, each on the slices the previous stage finished one
// interval earlier:
//   x stage (warps 0 .. 2, one staged row per thread): the (TX + 2XA + 4) x
//       (TY + 2R) input tile of a slice has landed in shared memory by one TMA
//       tile load (S loads in flight, mbarrier completion, bounded waits); the
//       thread filters its row's 16 outputs along x from a register window of
//       16-byte loads into the x-filtered tile X (double-buffered);
//   y stage (warps 4, 5): a thread owns two adjacent columns (one packed f32x2
//       register per row) and 8 output rows, read from a register window of X;
//       the y-filtered slice goes to Y (double-buffered);
//   z stage (every thread): a thread owns four consecutive columns of one row
//       and keeps a ring of 2RZ + 1 packed accumulators per column pair in
//       registers; a slice from Y is pushed into the ring (output z = j + RZ -
//       k gets w[k] * v), and the output it completes (z = j - RZ) is stored.
//       The ring slot is a compile-time function of the phase (j - jb) mod
//       (2RZ + 1), selected by a switch.
// Only the stages touch shared memory between them; Y rows are stored in
// row-pair-swizzled order and X rows at a 72-byte stride, which keeps the
// stages' shared accesses free of bank conflicts.
//
// Rounding.  Reference rounding: acc = 0; acc = acc + x * w with separate
// scalar roundings in ascending tap order on f32 intermediates, pass by pass
// x, y, z (conv.rs:26-36): bit-identical to the reference.  The halo of an
// edge tile is clamped exactly: halo columns take the edge column's value,
// halo rows read the edge row.  FMA rounding: packed fma.rn.f32x2; the x pass
// on output pairs (the input pairs at odd window positions are formed once
// per task), the zero-filled halo of the TMA load, and the clamped taps added
// back at the image's x and y edges (p[R - d] * x[edge] for the outputs d < R
// inside an edge, p the prefix sums of the weights).
#pragma once

#include "two_pass.cuh"

namespace itkg {
namespace onetrip {

using fusedk::clampi;
using fusedk::load4;
using fusedk::mbar_expect_tx;
using fusedk::mbar_init;
using fusedk::mbar_wait;
using fusedk::smem_u32;
using fusedk::tma_load_3d;

constexpr int kMaxR = 8;    // x and y radius
constexpr int kMaxRZ = 8;   // z radius
constexpr int kTX = 16;     // tile columns
constexpr int kTY = 64;     // tile rows
constexpr int kMaxSplit = 1024;

struct Args {
  char* dst;             // output voxel (x0, y0, z0)
  int64_t dst_pitch[3];  // bytes
  int32_t src_origin[3];
  int32_t lo[3], hi[3];  // gather bounds (image within the input buffer), inclusive
  int32_t x0, y0, z0;    // first requested voxel (absolute)
  int32_t nx, ny, nz;    // requested size
  int32_t ntx, nty;      // tiles along x and y
  int32_t out_dtype;
  int32_t vec;           // 1: f32 output with 16-byte aligned quads (every quad full)
  unsigned int* fault;
  long long wait_limit;
  int64_t units;         // ntx * nty * nz, tile-major
  int32_t nsplit;        // > 0: CTA b processes units [split[b], split[b + 1]); 0: an even split
  int32_t edge;          // FMA rounding: bit 0/1/2/3 = cxl/cxr/cyt/cyb hold a nonzero coefficient
  int32_t xr0, yr0;      // first of the last two tile columns / rows
  float wx[2 * kMaxR + 1], wy[2 * kMaxR + 1], wz[2 * kMaxRZ + 1];
  f2_t wx2[2 * kMaxR + 1], wy2[2 * kMaxR + 1], wz2[2 * kMaxRZ + 1];  // {w, w} pairs
  // FMA rounding: the weight of the clamped taps of each output column of the
  // first tile column (cxl) and of the last two (cxr), as pairs of adjacent
  // columns, and of each output row of the first tile row (cyt) and of the
  // last two (cyb), as {c, c} pairs.
  f2_t cxl[kTX / 2], cxr[kTX], cyt[kTY], cyb[2 * kTY];
  int32_t split[kMaxSplit + 1];
};

template <int R, int RZ>
struct Cfg {
  static constexpr int K = 2 * R + 1;
  static constexpr int KZ = 2 * RZ + 1;
  static constexpr int NT = 256;
  static constexpr int TX = kTX, TY = kTY;
  static constexpr int SPI = 2;                     // input slices per barrier interval
  static constexpr int XA = (R + 3) / 4 * 4;        // x halo, rounded up to 16 bytes
  static constexpr int BW = TX + 2 * XA + 4;        // staged row (floats); +4: rows 4 banks apart
  static constexpr int IH = TY + 2 * R;             // staged rows
  static constexpr int OFF = (XA - R) % 4;          // first tap of output 0 in the window
  static constexpr int WB = XA - R - OFF;           // window start (staged column), 0
  static constexpr int WIN = (TX + 2 * R + OFF + 3) / 4 * 4;  // window floats
  static constexpr int BOX = BW * IH * 4;           // bytes of one tile load
  static constexpr int STAGE = (BOX + 127) / 128 * 128;
  static constexpr int XP = 18;                     // X row stride (floats): 72 bytes
  static constexpr int XBUF = IH * XP;              // floats per X slice
  static constexpr int YBUF = TY * TX;              // floats per Y slice
  static constexpr int BUFS = 4 * 2 * SPI * (XBUF + YBUF);  // bytes of X and Y (double-buffered)
  // tile loads in flight: as many as fit beside X and Y in half of the SM's
  // shared memory (two CTAs per SM), a multiple of SPI, at most 8
  static constexpr int SFIT = (110 * 1024 - BUFS - 256) / STAGE / SPI * SPI;
  static constexpr int S = SFIT < 8 ? SFIT : 8;
  static constexpr int MY = 8;                      // y outputs per y task
  static constexpr int NYT = (TX / 2) * (TY / MY);  // y tasks: 64
  static constexpr int Y0 = 128;                    // first y-task thread
  static constexpr size_t SMEM = (size_t)S * STAGE + BUFS + 128;
  static_assert(WB == 0 && WIN <= BW, "x window inside the staged row");
  static_assert(IH <= Y0, "x tasks fit below the y tasks");
  static_assert(Y0 + NYT <= NT, "y tasks fit the block");
  static_assert(Y0 % 32 == 0 && NYT % 32 == 0 && (IH - 1) / 32 < Y0 / 32, "roles are whole warps");
  static_assert(TX * TY / 4 == NT, "one z quad per thread");
  static_assert(S >= 2 * SPI, "two intervals of tile loads in flight");
};

__device__ __forceinline__ void st_cs4(void* p, float a, float b, float c, float d) {
  asm volatile("st.global.cs.v4.f32 [%0], {%1, %2, %3, %4};\n" ::"l"(p), "f"(a), "f"(b), "f"(c), "f"(d)
               : "memory");
}

// z stage for phase P: push v (two packed column pairs) into the ring, return
// the completed slot (P + RZ + 1) mod KZ in `done` (and clear it in reference
// rounding, whose next output starts from zero).  The kernel is symmetric:
// tap k uses the weight of tap min(k, 2RZ - k).
template <int P, int KZ, bool REF>
__device__ __forceinline__ void z_push(f2_t (&acc)[2][KZ], const f2_t (&v)[2], const Args& a, f2_t (&done)[2]) {
  constexpr int RZ = (KZ - 1) / 2;
#pragma unroll
  for (int k = 0; k < KZ; ++k) {
    const int slot = (P + RZ - k + 2 * KZ) % KZ;  // output j + RZ - k
    const int kw = k <= RZ ? k : 2 * RZ - k;
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      if constexpr (REF) {  // scalar: separate roundings, as the reference
        float a0, a1, v0, v1;
        unpack2(acc[m][slot], a0, a1);
        unpack2(v[m], v0, v1);
        acc[m][slot] = pack2(__fadd_rn(a0, __fmul_rn(v0, a.wz[kw])), __fadd_rn(a1, __fmul_rn(v1, a.wz[kw])));
      } else if (k == 0) {  // first contribution to a fresh output
        acc[m][slot] = mul2(v[m], a.wz2[0]);
      } else {
        acc[m][slot] = fma2(v[m], a.wz2[kw], acc[m][slot]);
      }
    }
  }
  constexpr int D = (P + RZ + 1) % KZ;
#pragma unroll
  for (int m = 0; m < 2; ++m) {
    done[m] = acc[m][D];
    if constexpr (REF) acc[m][D] = 0ull;
  }
}

#define ITKG_OT_PUSH(N)                                       \
  case N:                                                     \
    if constexpr (N < KZ) z_push<N, KZ, REF>(acc, zv, a, done); \
    break;

template <int R, int RZ, bool REF>
__global__ void __launch_bounds__(256, 2) k_one_trip(const __grid_constant__ CUtensorMap tmap,
                                                     const __grid_constant__ Args a) {
  using C = Cfg<R, RZ>;
  constexpr int K = C::K, KZ = C::KZ, TX = C::TX, TY = C::TY, BW = C::BW, IH = C::IH, XA = C::XA,
                S = C::S, WIN = C::WIN, OFF = C::OFF, XP = C::XP, MY = C::MY, SPI = C::SPI;
  static_assert(KZ <= 17, "phase switch covers KZ <= 17");
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar[S];
  __shared__ int s_fail;
  unsigned char* const stage0 = smem + ((128u - (smem_u32(smem) & 127u)) & 127u);
  float* const xbuf = reinterpret_cast<float*>(stage0 + S * C::STAGE);  // [2 SPI][IH][XP]
  float* const ybuf = xbuf + 2 * SPI * C::XBUF;                        // [2 SPI][TY][TX], row-pair swizzled
  const uint32_t sbase = smem_u32(stage0);
  const uint32_t bbase = smem_u32(mbar);
  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int i = 0; i < S; ++i) mbar_init(bbase + 8 * i, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    s_fail = 0;
  }
  __syncthreads();
  // the stream's next kernel may be scheduled now; it waits for this grid
  // before its first global access
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  // this grid may read what the stream's previous kernel wrote
  asm volatile("griddepcontrol.wait;\n" ::: "memory");

  const int64_t u_begin = a.nsplit > 0 ? (int64_t)a.split[blockIdx.x] : a.units * blockIdx.x / gridDim.x;
  const int64_t u_end = a.nsplit > 0 ? (int64_t)a.split[blockIdx.x + 1] : a.units * (blockIdx.x + 1) / gridDim.x;

  // roles by warp (warp-uniform branches): warps 0 .. (IH - 1) / 32 run the x
  // task of staged row min(tid, IH - 1) (lanes past the last row repeat it and
  // store the same values), warps Y0 / 32 .. run the y tasks
  const int warp = __shfl_sync(0xffffffffu, tid >> 5, 0);
  const bool is_x = warp <= (IH - 1) / 32;
  const int xrow = tid < IH ? tid : IH - 1;
  const int yt = tid - C::Y0;
  const bool is_y = warp >= C::Y0 / 32 && warp < (C::Y0 + C::NYT) / 32;  // pair yp, rows 8 yg .. 8 yg + 7
  const int yp = yt & 7, yg = yt >> 3;
  const int zr = tid >> 2, zq = tid & 3;            // z: row zr, columns 4 zq .. 4 zq + 3
  // Y rows are stored row-pair swizzled: row r in slot r ^ ((r >> 3) & 1)
  const int zslot = zr ^ ((zr >> 3) & 1);

  uint32_t n_issued = 0, n_used = 0;  // tile loads issued / waited for (uniform over the CTA)

  for (int64_t u = u_begin; u < u_end;) {
    // ---- segment: one tile, output slices [z0, z1) ----
    const int64_t tile = u / a.nz;
    const int zs = (int)(u - tile * a.nz);
    const int64_t zrem = zs + (u_end - u);
    const int ze = zrem < a.nz ? (int)zrem : a.nz;
    u += ze - zs;
    const int tiy = (int)(tile / a.ntx), tix = (int)(tile - (int64_t)tiy * a.ntx);
    const int tx0 = a.x0 + tix * TX, ty0 = a.y0 + tiy * TY;
    const int gx0 = tx0 - XA, gy0 = ty0 - R;  // image coordinates of staged element (0, 0)
    const int z0 = a.z0 + zs;
    const int jb = z0 - RZ;                    // first input slice
    const int nout = ze - zs;                  // outputs of the segment
    // input slices z0 - RZ .. z1 - 1 + RZ, rounded up to whole intervals (the
    // extra slice, if any, feeds only an output past z1, which is not stored)
    const int n_int = (nout + 2 * RZ + SPI - 1) / SPI;
    const int n_in = n_int * SPI;
    // edges
    const int nl = a.lo[0] - gx0, cr = a.hi[0] - gx0;     // staged columns of the image's first / last column
    const int rlo = a.lo[1] - gy0, rhi = a.hi[1] - gy0;   // staged rows of its first / last row
    int xedge = 0;
    bool top = false, bot = false;
    int trow = 0;
    if constexpr (REF) {
      xedge = (nl > 0 || cr < BW - 1) ? 1 : 0;
    } else {
      const int tcol = tix - a.xr0;
      xedge = (tix == 0 && (a.edge & 1) ? 1 : 0) | ((tcol >= 0) && (a.edge & 2) ? 2 | (tcol << 2) : 0);
      trow = tiy - a.yr0;
      top = (a.edge & 4) && tiy == 0;
      bot = (a.edge & 8) && trow >= 0 && rhi < IH;
    }
    const bool yedge = rlo > 0 || rhi < IH - 1;

    auto issue = [&](int i) {  // tile load of input slice jb + i
      if (tid == 0) {
        const int st = (int)(n_issued % S);
        const uint32_t bar = bbase + 8 * st;
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        mbar_expect_tx(bar, (uint32_t)C::BOX);
        const int zc = clampi(jb + i, a.lo[2], a.hi[2]);
        tma_load_3d(sbase + (uint32_t)(st * C::STAGE), &tmap, gx0 - a.src_origin[0], gy0 - a.src_origin[1],
                    zc - a.src_origin[2], bar);
      }
      ++n_issued;
    };

    // x task: staged row xrow of a tile -> X row xrow (TX outputs)
    auto xtask = [&](const float* tile, float* xb) {
      const int srow = (REF && yedge) ? clampi(xrow, rlo, rhi) : xrow;
      const float* const src = tile + srow * BW;
      float v[WIN];
#pragma unroll
      for (int q = 0; q < WIN / 4; ++q) load4(src + 4 * q, v + 4 * q);
      f2_t* const d = reinterpret_cast<f2_t*>(xb + xrow * XP);
      if constexpr (REF) {
        if (xedge) {
          const float vl = src[max(nl, 0)], vr = src[min(cr, BW - 1)];
#pragma unroll
          for (int q = 0; q < WIN; ++q) {
            v[q] = q < nl ? vl : v[q];
            v[q] = q > cr ? vr : v[q];
          }
        }
#pragma unroll
        for (int j = 0; j < TX / 2; ++j) {
          float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
          for (int k = 0; k < K; ++k) {
            const float wk = a.wx[k <= R ? k : 2 * R - k];
            a0 = tap<true>(a0, v[2 * j + k + OFF], wk);
            a1 = tap<true>(a1, v[2 * j + 1 + k + OFF], wk);
          }
          d[j] = pack2(a0, a1);
        }
      } else {
        // output pairs (2j, 2j + 1): tap k multiplies the input pair at window
        // position 2j + OFF + k by {w_k, w_k}; pairs at even positions (E) are
        // register pairs as loaded, those at odd positions (O) are formed once
        // per task
        f2_t E[WIN / 2], O[WIN / 2 - 1];
#pragma unroll
        for (int q = 0; q < WIN / 2; ++q) E[q] = pack2(v[2 * q], v[2 * q + 1]);
#pragma unroll
        for (int q = 0; q < WIN / 2 - 1; ++q) O[q] = pack2(v[2 * q + 1], v[2 * q + 2]);
        auto pr = [&](int p) -> f2_t { return (p & 1) ? O[p / 2] : E[p / 2]; };
#pragma unroll
        for (int j = 0; j < TX / 2; ++j) {
          f2_t acc = mul2(pr(2 * j + OFF), a.wx2[0]);
#pragma unroll
          for (int k = 1; k < K; ++k) acc = fma2(pr(2 * j + OFF + k), a.wx2[k <= R ? k : 2 * R - k], acc);
          if (xedge & 1) {
            const float xl = src[nl];
            acc = fma2(pack2(xl, xl), a.cxl[j], acc);
          }
          if (xedge & 2) {
            const float xr = src[min(cr, BW - 1)];
            acc = fma2(pack2(xr, xr), a.cxr[(xedge >> 2) * (TX / 2) + j], acc);
          }
          d[j] = acc;
        }
      }
    };

    // y task: X -> Y rows 8 yg .. 8 yg + 7, columns 2 yp, 2 yp + 1
    auto ytask = [&](const float* xb, float* yb) {
      f2_t win[MY + 2 * R];
      const float* const col = xb + 2 * yp;
#pragma unroll
      for (int q = 0; q < MY + 2 * R; ++q) win[q] = *reinterpret_cast<const f2_t*>(col + (yg * MY + q) * XP);
      f2_t yv[MY];
#pragma unroll
      for (int m = 0; m < MY; ++m) {
        if constexpr (REF) {
          float y0 = 0.0f, y1 = 0.0f;
#pragma unroll
          for (int k = 0; k < K; ++k) {
            float v0, v1;
            unpack2(win[m + k], v0, v1);
            const float wk = a.wy[k <= R ? k : 2 * R - k];
            y0 = tap<true>(y0, v0, wk);
            y1 = tap<true>(y1, v1, wk);
          }
          yv[m] = pack2(y0, y1);
        } else {
          f2_t ay = mul2(win[m], a.wy2[0]);
#pragma unroll
          for (int k = 1; k < K; ++k) ay = fma2(win[m + k], a.wy2[k <= R ? k : 2 * R - k], ay);
          yv[m] = ay;
        }
      }
      if constexpr (!REF) {
        if (top) {
          const f2_t xe = *reinterpret_cast<const f2_t*>(col + rlo * XP);
#pragma unroll
          for (int m = 0; m < MY; ++m) yv[m] = fma2(xe, a.cyt[yg * MY + m], yv[m]);
        }
        if (bot) {
          const f2_t xe = *reinterpret_cast<const f2_t*>(col + rhi * XP);
#pragma unroll
          for (int m = 0; m < MY; ++m) yv[m] = fma2(xe, a.cyb[trow * TY + yg * MY + m], yv[m]);
        }
      }
      // row 8 yg + m lives in slot 8 yg + (m ^ (yg & 1))
      const int gb = yg & 1;
      f2_t* const ye = reinterpret_cast<f2_t*>(yb + (yg * MY + gb) * TX + 2 * yp);  // even m
      f2_t* const yo = reinterpret_cast<f2_t*>(yb + (yg * MY - gb) * TX + 2 * yp);  // odd m
#pragma unroll
      for (int m = 0; m < MY; ++m) {
        if (m & 1) yo[m * (TX / 2)] = yv[m];
        else ye[m * (TX / 2)] = yv[m];
      }
    };

    // this thread's output quad
    const int ox = tix * TX + 4 * zq, oy = tiy * TY + zr;  // relative to (x0, y0)
    const bool o_ok = ox < a.nx && oy < a.ny;
    const int ncols = min(4, a.nx - ox);
    char* dz = a.dst + (int64_t)ox * a.dst_pitch[0] + (int64_t)oy * a.dst_pitch[1] + (int64_t)zs * a.dst_pitch[2];
    auto store = [&](const f2_t (&done)[2]) {
      float o[4];
      unpack2(done[0], o[0], o[1]);
      unpack2(done[1], o[2], o[3]);
      if (a.vec) {
        st_cs4(dz, o[0], o[1], o[2], o[3]);
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

    f2_t acc[2][KZ];
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
      for (int k = 0; k < KZ; ++k) acc[m][k] = 0ull;

    for (int i = 0; i < S && i < n_in; ++i) issue(i);
    int phase = 0;  // (slice - jb) mod KZ of the next slice the z stage pushes
    int n_z = 0;    // slices pushed so far
    // interval t: x stage of slices SPI t .., y stage of the slices of
    // interval t - 1, z stage of those of interval t - 2
    for (int t = 0; t < n_int + 2; ++t) {
      if (t < n_int && is_x) {
#pragma unroll
        for (int h = 0; h < SPI; ++h) {
          const uint32_t n = n_used + h;
          const int st = (int)(n % S);
          if (!mbar_wait(bbase + 8 * st, (n / S) & 1u, a.wait_limit)) s_fail = 1;  // read after the barrier
          xtask(reinterpret_cast<const float*>(stage0 + st * C::STAGE), xbuf + ((t & 1) * SPI + h) * C::XBUF);
        }
      }
      if (t >= 1 && t <= n_int && is_y) {
#pragma unroll
        for (int h = 0; h < SPI; ++h)
          ytask(xbuf + (((t - 1) & 1) * SPI + h) * C::XBUF, ybuf + (((t - 1) & 1) * SPI + h) * C::YBUF);
      }
      if (t >= 2) {
#pragma unroll
        for (int h = 0; h < SPI; ++h) {
          const float4 f = *reinterpret_cast<const float4*>(ybuf + ((t & 1) * SPI + h) * C::YBUF + zslot * TX + 4 * zq);
          const f2_t zv[2] = {pack2(f.x, f.y), pack2(f.z, f.w)};
          f2_t done[2];
          switch (phase) {
            ITKG_OT_PUSH(0) ITKG_OT_PUSH(1) ITKG_OT_PUSH(2) ITKG_OT_PUSH(3) ITKG_OT_PUSH(4) ITKG_OT_PUSH(5)
            ITKG_OT_PUSH(6) ITKG_OT_PUSH(7) ITKG_OT_PUSH(8) ITKG_OT_PUSH(9) ITKG_OT_PUSH(10) ITKG_OT_PUSH(11)
            ITKG_OT_PUSH(12) ITKG_OT_PUSH(13) ITKG_OT_PUSH(14) ITKG_OT_PUSH(15) ITKG_OT_PUSH(16)
            default: break;
          }
          phase = phase + 1 == KZ ? 0 : phase + 1;
          // output z0 + n_z - 2RZ is complete
          if (n_z >= 2 * RZ && n_z - 2 * RZ < nout && o_ok) store(done);
          ++n_z;
        }
      }
      if (t < n_int) n_used += SPI;
      __syncthreads();  // X, Y and the stages of interval t are free for the next interval
      if (s_fail) goto timeout;
#pragma unroll
      for (int h = 0; h < SPI; ++h)
        if (SPI * t + h + S < n_in) issue(SPI * t + h + S);  // into the stages interval t has finished reading
    }
  }
  return;
timeout:
  if (tid == 0) {
    atomicExch(a.fault, 1u);
    // every load issued must land before the CTA exits (default bound): the
    // last S loads are the latest of each stage, the one given up on included
    // (a wait on an older, completed phase returns at once)
    for (uint32_t n = n_issued > S ? n_issued - S : 0; n < n_issued; ++n)
      mbar_wait(bbase + 8 * (n % S), (n / S) & 1u);
  }
}

#undef ITKG_OT_PUSH

using Fn = void (*)(const CUtensorMap, const Args);

}  // namespace onetrip
}  // namespace itkg
