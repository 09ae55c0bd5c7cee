/*
 * Host check of the decision rule behind the GPU's UnsharpMaskFilter point-wise
 * step in reference rounding: unsharp_fast_f32 and unsharp_fast_u8 of
 * itk-rs_gb300/csrc/unsharp.cuh, restated here operation for operation (keep
 * the two in step), against the reference's f64 sequence (edges.rs:440-448,
 * P::from_f64).  Whenever the rule decides a voxel, its result must equal the
 * reference's bit for bit; undecided voxels (which the GPU sends to f64) are
 * only counted.
 *
 * f32: random pairs over the whole exponent range, near-equal pairs, exact
 * ties, thresholds equal to |o - b|, f32 and non-f32 amounts.  u8: every
 * (o, b) pair for a set of amounts and thresholds.
 * Build: gcc -O2 -ffp-contract=off -frounding-math unsharp_decision.c -lm
 */
#include <fenv.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  double amount, threshold;
  float ah, al, thr_up, thr_dn, u8_min_pass;
  int thr_neg, a_exact, fast;
} K;

static float fa(float a, float b) { volatile float r = a + b; return r; }
static float fs(float a, float b) { volatile float r = a - b; return r; }
static float fm(float a, float b) { volatile float r = a * b; return r; }
static float fadd_dir(float a, float b, int mode) {
  fesetround(mode);
  volatile float r = a + b;
  fesetround(FE_TONEAREST);
  return r;
}
static float fadd_ru(float a, float b) { return fadd_dir(a, b, FE_UPWARD); }
static float fadd_rd(float a, float b) { return fadd_dir(a, b, FE_DOWNWARD); }
static void two_sum(float a, float b, float* s, float* t) {
  *s = fa(a, b);
  float a1 = fs(*s, b), b1 = fs(*s, a1);
  *t = fa(fs(a, a1), fs(b, b1));
}
static uint32_t bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

/* unsharp_consts (unsharp.cu) */
static K consts(double amount, double threshold) {
  K k;
  memset(&k, 0, sizeof k);
  k.amount = amount;
  k.threshold = threshold;
  const double aa = fabs(amount);
  k.fast = aa <= 0x1p30 && (amount == 0.0 || aa >= 0x1p-30);
  k.ah = (float)amount;
  k.al = (float)(amount - (double)k.ah);
  k.a_exact = (double)k.ah == amount;
  k.thr_neg = threshold < 0.0;
  if (isnan(threshold)) k.u8_min_pass = INFINITY;
  else if (threshold < 0.0) k.u8_min_pass = 0.0f;
  else k.u8_min_pass = threshold >= 256.0 ? 256.0f : (float)(floor(threshold) + 1.0);
  if (isnan(threshold)) {
    k.thr_up = INFINITY;
    k.thr_dn = INFINITY;
  } else if (threshold <= 0.0) {
    k.thr_up = -1.0f;
    k.thr_dn = -1.0f;
  } else {
    const double up = threshold * (1.0 + 0x1p-20), dn = threshold * (1.0 - 0x1p-20);
    float fu = (float)up, fd = (float)dn;
    if ((double)fu < up) fu = nextafterf(fu, INFINITY);
    if ((double)fd > dn) fd = nextafterf(fd, 0.0f);
    if (threshold < 0x1p-100) {
      fu = fmaxf(fu, 0x1p-100f);
      fd = 0.0f;
    }
    k.thr_up = fu;
    k.thr_dn = fd;
  }
  return k;
}

/* unsharp_fast_f32 (unsharp.cuh) */
static int fast_f32(float o, float b, const K* k, float* out) {
  if (!(fmaxf(fabsf(o), fabsf(b)) < 0x1p90f)) return 0;
  float eh, el;
  two_sum(o, -b, &eh, &el);
  if (eh == 0.0f) {
    *out = k->thr_neg ? fa(o, fm(k->ah, eh)) : o;
    return 1;
  }
  const float ae = fabsf(eh);
  int pass;
  if (ae > k->thr_up) pass = 1;
  else if (ae < k->thr_dn) pass = 0;
  else return 0;
  if (!pass) {
    *out = o;
    return 1;
  }
  const float ph = fm(k->ah, eh);
  const float t = fmaf(k->ah, eh, -ph);
  const float pl = fa(t, fa(fm(k->ah, el), fm(k->al, eh)));
  float sh, s1;
  two_sum(o, ph, &sh, &s1);
  const float s2 = fa(s1, pl);
  const float scale = fadd_ru(fabsf(o), fabsf(ph));
  if (!(scale >= 0x1p-80f) || !(fabsf(ph) < 0x1p100f) || ae < 0x1p-60f) return 0;
  const float delta = fm(scale, 0x1p-40f);
  const float hi = fa(sh, fadd_ru(s2, delta)), lo = fa(sh, fadd_rd(s2, -delta));
  if (hi == lo) {
    *out = hi;
    return 1;
  }
  if (k->a_exact && (el == 0.0f || fabsf(el) >= fm(ae, 0x1p-29f))) {
    const float c = fm(k->ah, el), ce = fmaf(k->ah, el, -c);
    float p2, p2e, s2x, s2e;
    two_sum(t, c, &p2, &p2e);
    two_sum(s1, p2, &s2x, &s2e);
    if (ce == 0.0f && p2e == 0.0f && s2e == 0.0f && (p2 == 0.0f || fabsf(p2) >= fm(fabsf(ph), 0x1p-29f))) {
      *out = fa(sh, s2x);
      return 1;
    }
  }
  return 0;
}

static uint8_t u8f(float v) { return (uint8_t)fminf(fmaxf(roundf(v), 0.0f), 255.0f); }

/* unsharp_fast_u8 (unsharp.cuh) */
static int fast_u8(uint8_t ob, uint8_t bb, const K* k, uint8_t* out) {
  const float o = ob, e = fs(o, (float)bb);
  if (!(fabsf(e) >= k->u8_min_pass) || e == 0.0f) {
    *out = ob;
    return 1;
  }
  const float ph = fm(k->ah, e);
  const float t = fmaf(k->ah, e, -ph);
  const float pl = fa(t, fm(k->al, e));
  float sh, s1;
  two_sum(o, ph, &sh, &s1);
  const float s2 = fa(s1, pl);
  const float delta = fm(fadd_ru(o, fabsf(ph)), 0x1p-40f);
  const uint8_t qh = u8f(fadd_ru(sh, fadd_ru(s2, delta))), ql = u8f(fadd_rd(sh, fadd_rd(s2, -delta)));
  if (qh == ql) {
    *out = qh;
    return 1;
  }
  if (k->a_exact && t == 0.0f && s1 == 0.0f) {
    *out = u8f(sh);
    return 1;
  }
  return 0;
}

/* the reference: edges.rs:440-448 in f64, then P::from_f64 */
static double ref_v(double o, double b, double a, double thr) {
  volatile double e = o - b, p = a * e, v = o + p;
  return fabs(e) > thr ? v : o;
}
static uint8_t u8d(double v) {
  if (isnan(v)) return 0;
  const double r = fmin(fmax(round(v), 0.0), 255.0);
  return (uint8_t)r;
}

static uint64_t rs = 0x9E3779B97F4A7C15ull;
static uint64_t rnd(void) {
  rs ^= rs << 13;
  rs ^= rs >> 7;
  rs ^= rs << 17;
  return rs;
}
static double unif(void) { return (rnd() >> 11) * 0x1p-53; }
static float any_f32(int mode) {
  switch (mode) {
    case 0: return (float)unif();
    case 1: return (float)((unif() - 0.5) * 1000.0);
    case 2: {
      const uint32_t u = (uint32_t)rnd();
      float f;
      memcpy(&f, &u, 4);
      return f;
    }
    case 3: return (float)ldexp(unif() - 0.5, (int)(rnd() % 80) - 40);
    default: return (float)(rnd() % 256) + (float)(rnd() % 2) * 0.5f;
  }
}

int main(int argc, char** argv) {
  const long iters = argc > 1 ? atol(argv[1]) : 3000000;
  long n = 0, undecided = 0, bad = 0;
  for (long it = 0; it < iters; ++it) {
    const int mode = (int)(it % 5);
    const float o = any_f32(mode);
    float b;
    switch (rnd() % 4) {
      case 0: b = any_f32(mode); break;
      case 1: b = nextafterf(o, INFINITY); break;
      case 2: b = o * (float)(1.0 + (unif() - 0.5) * 1e-3); break;
      default: b = o;
    }
    double a;
    switch (rnd() % 5) {
      case 0: a = 0.5; break;
      case 1: a = unif() * 4.0 - 2.0; break;
      case 2: a = ldexp(unif(), (int)(rnd() % 60) - 30); break;
      case 3: a = (double)(float)(unif() * 4.0 - 2.0); break;
      default: a = -0.7;
    }
    const double e = (double)o - (double)b;
    double thr;
    switch (rnd() % 6) {
      case 0: thr = 0.0; break;
      case 1: thr = fabs(e); break;
      case 2: thr = fabs(e) * (1.0 + (unif() - 0.5) * 1e-5); break;
      case 3: thr = -1.0; break;
      case 4: thr = unif() * 0.1; break;
      default: thr = NAN;
    }
    const K k = consts(a, thr);
    const float want = (float)ref_v(o, b, a, thr);
    float got;
    ++n;
    if (!k.fast || !fast_f32(o, b, &k, &got)) {
      ++undecided;
      continue;
    }
    if (bits(got) != bits(want) && !(isnan(got) && isnan(want))) {
      if (bad < 5) printf("f32 mismatch o=%a b=%a amount=%a threshold=%a: %a vs %a\n", o, b, a, thr, got, want);
      ++bad;
    }
  }
  printf("f32: %ld cases, %ld undecided, %ld mismatches\n", n, undecided, bad);
  const double amounts[] = {0.5, 0.7, 1.5, 3.0, -0.5, 1.0 / 3.0, 0.1, 0x1p-20, 1000.0, 123.456, 2.0, 0.25, -1.75};
  const double thresholds[] = {0.0, 2.5, 3.0, -1.0, NAN, 300.0, 0.5, 254.9};
  long n8 = 0, u8u = 0, bad8 = 0;
  for (size_t ai = 0; ai < sizeof amounts / sizeof amounts[0]; ++ai)
    for (size_t ti = 0; ti < sizeof thresholds / sizeof thresholds[0]; ++ti) {
      const K k = consts(amounts[ai], thresholds[ti]);
      for (int o = 0; o < 256; ++o)
        for (int b = 0; b < 256; ++b) {
          const uint8_t want = u8d(ref_v(o, b, amounts[ai], thresholds[ti]));
          uint8_t got;
          ++n8;
          if (!k.fast || !fast_u8((uint8_t)o, (uint8_t)b, &k, &got)) {
            ++u8u;
            continue;
          }
          if (got != want) {
            if (bad8 < 5) printf("u8 mismatch o=%d b=%d amount=%g threshold=%g: %d vs %d\n", o, b, amounts[ai],
                                 thresholds[ti], got, want);
            ++bad8;
          }
        }
    }
  printf("u8: %ld cases, %ld undecided, %ld mismatches\n", n8, u8u, bad8);
  return bad + bad8 == 0 ? 0 : 1;
}
