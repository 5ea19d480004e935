// phs_math.h -- elementary functions of the per-event-beam constants (host and device).
//
// The per-event forms evaluate, per Breit-Wigner branch and event, the upper bound
// a1 = atan((msq_max - m^2) / (m w)) of the mapping (phs_cpu.cpp:452-531 at the event's
// sqrt(s)).  Its argument is the branch's kinematic range in widths, at least ~10^3 for W
// and t at collider energies.  There atan(u) = pi/2 - atan(1/u), and for w = 1/u <= 2^-10
// the series atan(w) = w - w^3/3 + w^5/5 - ... needs three terms: the next, w^7/7, is below
// 2^-72, a millionth of an ulp of pi/2.  One division and three operations instead of the
// library's general atan; within an ulp of the exact value (pi/2 as a double plus its
// rounding error, added last).  Smaller arguments use the library's atan.
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define PHS_MATH_FN __host__ __device__ __forceinline__
#else
#define PHS_MATH_FN inline
#endif

#define PHS_PIO2_HI 1.5707963267948966       // pi/2 rounded to double
#define PHS_PIO2_LO 6.123233995736766e-17    // pi/2 - PHS_PIO2_HI

PHS_MATH_FN double phs_atan_large(double u) {
  const double w = 1.0 / u, w2 = w * w;
  const double s = w + w * w2 * (-1.0 / 3.0 + w2 * 0.2);
  return (PHS_PIO2_HI - s) + PHS_PIO2_LO;
}

// atan(u) of a Breit-Wigner bound: the series above for u >= 1024, else the library's.
PHS_MATH_FN double phs_atan_bw(double u) { return u >= 1024.0 ? phs_atan_large(u) : atan(u); }

// a / b for a constant b with rb = RN(1/b): the product a rb corrected once with its
// residual, q + (a - b q) rb, the residual exact through the FMA.  With rb correctly
// rounded this is a / b correctly rounded (Markstein's theorem on the corrected quotient;
// the host test checks it bit for bit against the division for the constants the volume
// program uses): three FP64 operations instead of a division's sequence.
PHS_MATH_FN double phs_div_by_const(double a, double b, double rb) {
  const double q = a * rb;
  return fma(fma(-q, b, a), rb, q);
}
