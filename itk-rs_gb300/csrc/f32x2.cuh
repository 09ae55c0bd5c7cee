// Packed two-lane f32 arithmetic (PTX add/mul/fma .f32x2, sm_100+).
// Reference rounding does not use these: a packed mul.rn / add.rn pair was
// measured on the GPU to give results that differ from the scalar
// __fmul_rn / __fadd_rn sequence (in about 70% of the voxels of a 3-D filter),
// so every reference-rounding tap is scalar.
#pragma once

#include <cstdint>

namespace itkg {

typedef unsigned long long f2_t;  // {lo, hi} f32 pair in one 64-bit register

__device__ __forceinline__ f2_t pack2(float lo, float hi) {
  f2_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}

__device__ __forceinline__ void unpack2(f2_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}

__device__ __forceinline__ f2_t fma2(f2_t a, f2_t b, f2_t c) {
  f2_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

__device__ __forceinline__ f2_t mul2(f2_t a, f2_t b) {
  f2_t d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

__device__ __forceinline__ f2_t add2(f2_t a, f2_t b) {
  f2_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

// Host-side: the 64-bit pattern of the pair {w, w}.
inline unsigned long long splat2_host(float w) {
  unsigned int u;
  __builtin_memcpy(&u, &w, 4);
  return ((unsigned long long)u << 32) | u;
}

// Host-side: the 64-bit pattern of the pair {lo, hi} (lo in the low lane).
inline unsigned long long pack2_host(float lo, float hi) {
  unsigned int a, b;
  __builtin_memcpy(&a, &lo, 4);
  __builtin_memcpy(&b, &hi, 4);
  return ((unsigned long long)b << 32) | a;
}

}  // namespace itkg
