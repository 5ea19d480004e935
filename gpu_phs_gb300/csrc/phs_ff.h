// phs_ff.h -- float-float ("FP32 pair") arithmetic for the FP32-pipe forward kernel.
//
// A value is hi + lo with two floats, |lo| <= ulp(hi)/2, about 48 significant bits.  The
// primitives are the error-free transformations of Knuth (TwoSum) and Dekker (Fast2Sum,
// and the product via FMA), composed as in Dekker, "A floating-point technique for
// extending the available precision", Numer. Math. 18 (1971).  Arithmetic goes through
// explicit round-to-nearest intrinsics so no compiler contraction or reassociation can
// break an error-free step.  The elementary functions reduce their argument with a table
// of exact multiples (kept in shared memory by the kernel) and evaluate short Taylor
// series; leading terms in float-float, the small tail in plain float.  Accuracy against
// long double on the host: 3e-14 relative for the arithmetic, 5e-14 absolute for sin and
// cos, 1.5e-13 relative for tan and exp, far inside what the forward map needs for momenta
// within 1e-6.
//
// The header also compiles as host C++ (for CPU validation of the functions).
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define FF_FN __host__ __device__ __forceinline__
#else
#define FF_FN inline
struct float2 { float x, y; };
struct float4 { float x, y, z, w; };
#endif

struct ff {
  float hi, lo;
};

#if defined(__CUDA_ARCH__)
FF_FN float f_add(float a, float b) { return __fadd_rn(a, b); }
FF_FN float f_sub(float a, float b) { return __fsub_rn(a, b); }
FF_FN float f_mul(float a, float b) { return __fmul_rn(a, b); }
FF_FN float f_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
FF_FN float f_sqrt(float a) { return __fsqrt_rn(a); }
FF_FN float f_div(float a, float b) { return __fdiv_rn(a, b); }
#else
FF_FN float f_add(float a, float b) { volatile float r = a + b; return r; }
FF_FN float f_sub(float a, float b) { volatile float r = a - b; return r; }
FF_FN float f_mul(float a, float b) { volatile float r = a * b; return r; }
FF_FN float f_fma(float a, float b, float c) { return fmaf(a, b, c); }
FF_FN float f_sqrt(float a) { return sqrtf(a); }
FF_FN float f_div(float a, float b) { volatile float r = a / b; return r; }
#endif

FF_FN ff ff_make(float hi, float lo) { ff r; r.hi = hi; r.lo = lo; return r; }
FF_FN ff ff_from_float(float a) { return ff_make(a, 0.0f); }

// Fast2Sum: |a| >= |b| (or a == 0).
FF_FN ff fast_two_sum(float a, float b) {
  float s = f_add(a, b);
  float e = f_sub(b, f_sub(s, a));
  return ff_make(s, e);
}

// TwoSum: any a, b.
FF_FN ff two_sum(float a, float b) {
  float s = f_add(a, b);
  float bb = f_sub(s, a);
  float e = f_add(f_sub(a, f_sub(s, bb)), f_sub(b, bb));
  return ff_make(s, e);
}

FF_FN ff two_prod(float a, float b) {
  float p = f_mul(a, b);
  float e = f_fma(a, b, -p);
  return ff_make(p, e);
}

FF_FN ff ff_neg(ff a) { return ff_make(-a.hi, -a.lo); }

FF_FN ff ff_add(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi);
  float e = f_add(s.lo, f_add(a.lo, b.lo));
  return fast_two_sum(s.hi, e);
}

FF_FN ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

FF_FN ff ff_add_f(ff a, float b) {
  ff s = two_sum(a.hi, b);
  float e = f_add(s.lo, a.lo);
  return fast_two_sum(s.hi, e);
}

FF_FN ff ff_mul(ff a, ff b) {
  ff p = two_prod(a.hi, b.hi);
  float e = f_fma(a.hi, b.lo, p.lo);
  e = f_fma(a.lo, b.hi, e);
  return fast_two_sum(p.hi, e);
}

FF_FN ff ff_mul_f(ff a, float b) {
  ff p = two_prod(a.hi, b);
  float e = f_fma(a.lo, b, p.lo);
  return fast_two_sum(p.hi, e);
}

// a*b + c
FF_FN ff ff_fma(ff a, ff b, ff c) { return ff_add(ff_mul(a, b), c); }

FF_FN ff ff_sqr(ff a) {
  ff p = two_prod(a.hi, a.hi);
  float e = f_fma(f_add(a.hi, a.hi), a.lo, p.lo);
  return fast_two_sum(p.hi, e);
}

FF_FN ff ff_div(ff a, ff b) {
  float q1 = f_div(a.hi, b.hi);
  ff r = ff_sub(a, ff_mul_f(b, q1));
  float q2 = f_div(r.hi, b.hi);
  ff q = fast_two_sum(q1, q2);
  r = ff_sub(a, ff_mul(b, q));
  float q3 = f_div(r.hi, b.hi);
  return ff_add_f(q, q3);
}

FF_FN ff ff_recip(ff b) { return ff_div(ff_from_float(1.0f), b); }

// sqrt(a), a >= 0; one Newton step on the float square root, residual in float-float.
FF_FN ff ff_sqrt(ff a) {
  if (!(a.hi > 0.0f)) return ff_make(a.hi == 0.0f ? 0.0f : f_sqrt(a.hi), 0.0f);
  float y = f_sqrt(a.hi);
  ff r = ff_sub(a, two_prod(y, y));
  float c = f_div(r.hi, f_add(y, y));
  return fast_two_sum(y, c);
}

#if defined(__CUDA_ARCH__)
FF_FN float f_rcp_approx(float a) { return __fdividef(1.0f, a); }   // hardware approximation
FF_FN float f_rsqrt_approx(float a) { return rsqrtf(a); }
#else
FF_FN float f_rcp_approx(float a) { return 1.0f / a; }
FF_FN float f_rsqrt_approx(float a) { return 1.0f / sqrtf(a); }
#endif

// 1/b: the hardware reciprocal estimate refined by one Newton step with the residual
// 1 - b y in float-float (~2^-44 relative).
FF_FN ff ff_recip_fast(ff b) {
  const float y = f_rcp_approx(b.hi);
  const ff p = two_prod(b.hi, y);
  const float e = f_sub(f_sub(f_sub(1.0f, p.hi), p.lo), f_mul(b.lo, y));
  return fast_two_sum(y, f_mul(y, e));
}

// a/b with the reciprocal estimate: q1 = a.hi y, then one correction from a - b q1.
FF_FN ff ff_div_fast(ff a, ff b) {
  const float y = f_rcp_approx(b.hi);
  const float q1 = f_mul(a.hi, y);
  const ff r = ff_sub(a, ff_mul_f(b, q1));
  return fast_two_sum(q1, f_mul(r.hi, y));
}

// sqrt(a), a >= 0, from the hardware rsqrt estimate and one Newton step in float-float.
FF_FN ff ff_sqrt_fast(ff a) {
  if (!(a.hi > 0.0f)) return ff_make(0.0f, 0.0f);
  const float y = f_rsqrt_approx(a.hi);
  const float s = f_mul(a.hi, y);
  const ff r = ff_sub(a, two_prod(s, s));
  return fast_two_sum(s, f_mul(f_mul(r.hi, y), 0.5f));
}

// a0 b0 + a1 b1 (+ a2 b2 + a3 b3): exact products of the high parts summed with TwoSum,
// every rounding error and cross term gathered in one float, one normalization at the end.
FF_FN ff ff_dot2(ff a0, ff b0, ff a1, ff b1) {
  const ff p0 = two_prod(a0.hi, b0.hi), p1 = two_prod(a1.hi, b1.hi);
  float e = f_fma(a0.hi, b0.lo, f_fma(a0.lo, b0.hi, p0.lo));
  e = f_add(e, f_fma(a1.hi, b1.lo, f_fma(a1.lo, b1.hi, p1.lo)));
  const ff s = two_sum(p0.hi, p1.hi);
  return fast_two_sum(s.hi, f_add(e, s.lo));
}

FF_FN ff ff_dot3(ff a0, ff b0, ff a1, ff b1, ff a2, ff b2) {
  const ff p0 = two_prod(a0.hi, b0.hi), p1 = two_prod(a1.hi, b1.hi);
  const ff p2 = two_prod(a2.hi, b2.hi);
  float e = f_fma(a0.hi, b0.lo, f_fma(a0.lo, b0.hi, p0.lo));
  e = f_add(e, f_fma(a1.hi, b1.lo, f_fma(a1.lo, b1.hi, p1.lo)));
  e = f_add(e, f_fma(a2.hi, b2.lo, f_fma(a2.lo, b2.hi, p2.lo)));
  ff s = two_sum(p0.hi, p1.hi);
  e = f_add(e, s.lo);
  s = two_sum(s.hi, p2.hi);
  return fast_two_sum(s.hi, f_add(e, s.lo));
}

FF_FN ff ff_dot4(ff a0, ff b0, ff a1, ff b1, ff a2, ff b2, ff a3, ff b3) {
  const ff p0 = two_prod(a0.hi, b0.hi), p1 = two_prod(a1.hi, b1.hi);
  const ff p2 = two_prod(a2.hi, b2.hi), p3 = two_prod(a3.hi, b3.hi);
  float e = f_fma(a0.hi, b0.lo, f_fma(a0.lo, b0.hi, p0.lo));
  e = f_add(e, f_fma(a1.hi, b1.lo, f_fma(a1.lo, b1.hi, p1.lo)));
  e = f_add(e, f_fma(a2.hi, b2.lo, f_fma(a2.lo, b2.hi, p2.lo)));
  e = f_add(e, f_fma(a3.hi, b3.lo, f_fma(a3.lo, b3.hi, p3.lo)));
  ff s = two_sum(p0.hi, p1.hi);
  e = f_add(e, s.lo);
  s = two_sum(s.hi, p2.hi);
  e = f_add(e, s.lo);
  s = two_sum(s.hi, p3.hi);
  return fast_two_sum(s.hi, f_add(e, s.lo));
}

FF_FN bool ff_gt(ff a, ff b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
FF_FN float ff_to_float(ff a) { return f_add(a.hi, a.lo); }

// Double <-> float-float.  from_double truncates to 48 bits (the pair holds 48).
FF_FN ff ff_from_double(double d) {
  float hi = (float)d;
  float lo = (float)(d - (double)hi);
  return ff_make(hi, lo);
}
FF_FN double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

#if defined(__CUDA_ARCH__)
FF_FN uint64_t ff_dbits(double d) { return (uint64_t)__double_as_longlong(d); }
FF_FN double ff_bitsd(uint64_t b) { return __longlong_as_double((long long)b); }
FF_FN uint32_t ff_fbits(float f) { return __float_as_uint(f); }
FF_FN float ff_bitsf(uint32_t b) { return __uint_as_float(b); }
FF_FN int ff_clz(uint32_t v) { return __clz((int)v); }
#else
FF_FN uint64_t ff_dbits(double d) { uint64_t b; memcpy(&b, &d, 8); return b; }
FF_FN double ff_bitsd(uint64_t b) { double d; memcpy(&d, &b, 8); return d; }
FF_FN uint32_t ff_fbits(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }
FF_FN float ff_bitsf(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
FF_FN int ff_clz(uint32_t v) { return v ? __builtin_clz(v) : 32; }
#endif

// The same conversions with integer operations only (no FP64 instructions): the mantissa
// bits of the double are cut into a 24-bit and a 29-bit field.  Truncates toward zero, so
// for 0 <= d < 1 the order against 0.5 is kept exactly (d < 0.5 iff hi < 0.5f).  Values
// below 2^-74 in magnitude (or non-finite) are not handled: their low part reads as 0.
FF_FN ff ff_from_double_int(double d) {
  const uint64_t b = ff_dbits(d);
  const uint32_t hw = (uint32_t)(b >> 32), lw = (uint32_t)b;
  const int e = (int)((hw >> 20) & 0x7ff) - 1023;   // unbiased exponent
  if (e < -126) return ff_make(0.0f, 0.0f);
  const uint32_t sign = hw & 0x80000000u;
  const uint32_t hi = sign | ((uint32_t)(e + 127) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29);
  const uint32_t r = lw & 0x1fffffffu;              // remaining 29 bits, weight 2^(e-52)
  float lo = 0.0f;
  if (r != 0) {
    const int p = 31 - ff_clz(r);                   // leading one of r
    const int fe = e - 52 + p + 127;                // biased exponent of the low part
    if (fe >= 1) {
      const uint32_t m = p >= 23 ? (r >> (p - 23)) : (r << (23 - p));
      lo = ff_bitsf(sign | ((uint32_t)fe << 23) | (m & 0x7fffffu));
    }
  }
  return ff_make(ff_bitsf(hi), lo);
}

// D * 2^e2 for an integer 0 < D < 2^63, truncated to 48 bits, with integer operations only.
FF_FN ff ff_from_mantissa(uint64_t D, int e2) {
  const uint32_t dh = (uint32_t)(D >> 32), dl = (uint32_t)D;
  const int p = dh ? 63 - ff_clz(dh) : 31 - ff_clz(dl);   // leading one of D
  const int fe = p + e2 + 127;
  if (fe < 1) return ff_make(0.0f, 0.0f);
  const uint32_t mh = p >= 23 ? (uint32_t)(D >> (p - 23)) : (uint32_t)(D << (23 - p));
  const float hi = ff_bitsf(((uint32_t)fe << 23) | (mh & 0x7fffffu));
  float lo = 0.0f;
  if (p > 23) {
    const uint64_t r = D & ((1ull << (p - 23)) - 1);       // bits below hi's last place
    if (r) {
      const uint32_t rh = (uint32_t)(r >> 32), rl = (uint32_t)r;
      const int q = rh ? 63 - ff_clz(rh) : 31 - ff_clz(rl);
      const int ge = q + e2 + 127;
      if (ge >= 1) {
        const uint32_t ml = q >= 23 ? (uint32_t)(r >> (q - 23)) : (uint32_t)(r << (23 - q));
        lo = ff_bitsf(((uint32_t)ge << 23) | (ml & 0x7fffffu));
      }
    }
  }
  return ff_make(hi, lo);
}

// 1 - x for 0 <= x <= 1, with integer operations only.  For x in [0.5, 1) the double
// difference is exact (x = M 2^-53, 1 - x = (2^53 - M) 2^-53) and so is this pair up to its
// 48 bits: the relative accuracy of 1 - x holds as x -> 1.
FF_FN ff ff_one_minus_double_int(double x) {
  const uint64_t b = ff_dbits(x);
  if (((b >> 52) & 0x7ff) == 1022) {
    const uint64_t M = (b & 0xfffffffffffffull) | (1ull << 52);
    const uint64_t D = (1ull << 53) - M;
    return ff_from_mantissa(D, -53);
  }
  const ff xf = ff_from_double_int(x);
  const ff s = two_sum(1.0f, -xf.hi);
  return fast_two_sum(s.hi, f_sub(s.lo, xf.lo));
}

// hi + lo as a double, exactly for a normalized pair (|lo| <= ulp(hi)/2) of normal floats;
// bits of lo below the double's last place are dropped.
FF_FN double ff_to_double_int(ff a) {
  const uint32_t hb = ff_fbits(a.hi), lb = ff_fbits(a.lo);
  const int eh = (int)((hb >> 23) & 0xff);
  if (eh == 0) return 0.0;
  const int64_t H = (int64_t)(((uint64_t)0x800000u | (hb & 0x7fffffu)) << 29);  // 2^(eh-179) units
  int64_t L = 0;
  const int el = (int)((lb >> 23) & 0xff);
  if (el != 0) {
    const uint64_t ml = (uint64_t)0x800000u | (lb & 0x7fffffu);
    const int sh = el - eh + 29;
    L = sh >= 0 ? (int64_t)(ml << sh) : (sh > -40 ? (int64_t)(ml >> -sh) : 0);
    if ((hb ^ lb) & 0x80000000u) L = -L;
  }
  int64_t S = H + L;
  int ex = eh - 127 + 1023;
  if (S < ((int64_t)1 << 52)) {
    S <<= 1;
    ex -= 1;
  }
  const uint64_t bits = ((uint64_t)(hb & 0x80000000u) << 32) | ((uint64_t)ex << 52) |
                        ((uint64_t)S & 0xfffffffffffffull);
  return ff_bitsd(bits);
}

// ------------------------------------------------------------------ elementary functions
// Cody-Waite splits (three floats summing to the constant to ~2^-72 relative).
#define FF_PI32_1 0.098174773156642914f
#define FF_PI32_2 -2.7319617679211206e-09f
#define FF_PI32_3 -1.0719528187536762e-16f
#define FF_LN2_32_1 0.021660849452018738f
#define FF_LN2_32_2 -5.9520444128935424e-11f
#define FF_LN2_32_3 -2.7447449183091686e-18f
#define FF_INV_PI32 10.185915946960449f     // 32/pi, for choosing the table index only
#define FF_INV_LN2_32 46.166240692138672f   // 32/ln 2, likewise
#define FF_PI_HI 3.1415927410125732f
#define FF_PI_LO -8.7422776573475858e-08f
#define FF_SIXTH_LO -4.9670538793122887e-09f  // 1/6 - (float)(1/6)

// sin and cos of f, |f| <= pi/64 (radians), float-float.
FF_FN void ff_sincos_small(ff f, ff &s, ff &c) {
  ff f2 = ff_sqr(f);
  float y = f2.hi;
  // sin f = f - f^3/6 + f^5 (1/120 - f^2/5040 + f^4/362880)
  ff f3 = ff_mul(f2, f);
  float ts = f_mul(f_mul(y, y), f_fma(y, f_fma(y, 1.0f / 362880.0f, -1.0f / 5040.0f), 1.0f / 120.0f));
  ff s1 = ff_sub(f, ff_mul_f(f3, 1.0f / 6.0f));
  // 1/6 is not exact in float: correct with the float-float constant's low part
  s1 = ff_add_f(s1, f_mul(-f3.hi, FF_SIXTH_LO));
  s = ff_add_f(s1, f_mul(f.hi, ts));
  // cos f = 1 - f^2/2 + f^4 (1/24 - f^2/720 + f^4/40320)
  float tc = f_mul(f_mul(y, y), f_fma(y, f_fma(y, 1.0f / 40320.0f, -1.0f / 720.0f), 1.0f / 24.0f));
  ff c1 = ff_add(ff_from_float(1.0f), ff_mul_f(f2, -0.5f));
  c = ff_add_f(c1, tc);
}

// Tables (built on the host, phs_ff_tables in phs_kernels_ff.cu):
//   trig[k] = {sin(k pi/32).hi, .lo, cos(k pi/32).hi, .lo}, k = 0..63
//   exp2[j] = {2^(j/32).hi, .lo}, j = 0..31
struct FFTables {
  float4 trig[64];
  float2 exp2[32];
};

FF_FN ff ff_pi() { return ff_make(FF_PI_HI, FF_PI_LO); }

// sin(2 pi x), cos(2 pi x) for x in [0, 1]: the reduction 64x - k is exact.
FF_FN void ff_sincos2pi(ff x, const FFTables &T, ff &s, ff &c) {
  ff y = ff_make(f_mul(x.hi, 64.0f), f_mul(x.lo, 64.0f));
  float kf = rintf(y.hi);
  ff g = ff_add_f(y, -kf);                       // exact: |g| <= 1/2
  ff f = ff_mul(g, ff_make(FF_PI32_1, FF_PI32_2)); // radians, |f| <= pi/64
  ff sf, cf;
  ff_sincos_small(f, sf, cf);
  int k = ((int)kf) & 63;
  float4 t = T.trig[k];
  ff sk = ff_make(t.x, t.y), ck = ff_make(t.z, t.w);
  s = ff_add(ff_mul(sk, cf), ff_mul(ck, sf));
  c = ff_sub(ff_mul(ck, cf), ff_mul(sk, sf));
}

// sin and cos of z (radians), |z| <= pi/2 + pi/64: Cody-Waite reduction by k pi/32.
FF_FN void ff_sincos(ff z, const FFTables &T, ff &s, ff &c) {
  float kf = rintf(f_mul(z.hi, FF_INV_PI32));
  ff f = ff_sub(z, two_prod(kf, FF_PI32_1));
  f = ff_add_f(f, f_mul(-kf, FF_PI32_2));
  f = ff_add_f(f, f_mul(-kf, FF_PI32_3));
  ff sf, cf;
  ff_sincos_small(f, sf, cf);
  int k = ((int)kf) & 63;
  float4 t = T.trig[k];
  ff sk = ff_make(t.x, t.y), ck = ff_make(t.z, t.w);
  s = ff_add(ff_mul(sk, cf), ff_mul(ck, sf));
  c = ff_sub(ff_mul(ck, cf), ff_mul(sk, sf));
}

// tan(z) for |z| < pi/2 (radians).
FF_FN ff ff_tan(ff z, const FFTables &T) {
  ff s, c;
  ff_sincos(z, T, s, c);
  return ff_div_fast(s, c);
}

// cot(u) = 1/tan(u) for 0 < |u| <= pi/2.
FF_FN ff ff_cot(ff u, const FFTables &T) {
  ff s, c;
  ff_sincos(u, T, s, c);
  return ff_div_fast(c, s);
}

// exp(y), |y| < 80.
FF_FN ff ff_exp(ff y, const FFTables &T) {
  float nf = rintf(f_mul(y.hi, FF_INV_LN2_32));
  ff r = ff_sub(y, two_prod(nf, FF_LN2_32_1));
  r = ff_add_f(r, f_mul(-nf, FF_LN2_32_2));
  r = ff_add_f(r, f_mul(-nf, FF_LN2_32_3));        // |r| <= ln2/64
  ff r2 = ff_sqr(r);
  float rh = r.hi;
  // exp r = 1 + r + r^2/2 + r^2 (r/6 + r^2/24 + r^3/120 + r^4/720)
  float tail = f_mul(r2.hi, f_mul(rh, f_fma(rh, f_fma(rh, f_fma(rh, 1.0f / 720.0f, 1.0f / 120.0f), 1.0f / 24.0f), 1.0f / 6.0f)));
  ff e = ff_add(ff_add_f(r, 1.0f), ff_mul_f(r2, 0.5f));
  e = ff_add_f(e, tail);
  int n = (int)nf;
  int j = n & 31, m = (n - j) / 32;
  float2 t = T.exp2[j];
  e = ff_mul(e, ff_make(t.x, t.y));
  float sc = ldexpf(1.0f, m);
  return ff_make(f_mul(e.hi, sc), f_mul(e.lo, sc));
}

// Fills the tables (host side).  Entries whose angle is a multiple of pi/2 are set to the
// exact 0 / +-1, so that tan near +-pi/2 keeps its relative accuracy.
inline void ff_fill_tables(FFTables &T) {
  for (int k = 0; k < 64; k++) {
    long double a = (long double)k * 3.14159265358979323846264338327950288L / 32.0L;
    long double sv = sinl(a), cv = cosl(a);
    if (k % 16 == 0) {
      sv = (k == 16) ? 1.0L : (k == 48 ? -1.0L : 0.0L);
      cv = (k == 0) ? 1.0L : (k == 32 ? -1.0L : 0.0L);
    }
    float sh = (float)sv, ch = (float)cv;
    T.trig[k].x = sh;
    T.trig[k].y = (float)(sv - (long double)sh);
    T.trig[k].z = ch;
    T.trig[k].w = (float)(cv - (long double)ch);
  }
  for (int j = 0; j < 32; j++) {
    long double v = exp2l((long double)j / 32.0L);
    float h = (float)v;
    T.exp2[j].x = h;
    T.exp2[j].y = (float)(v - (long double)h);
  }
}
