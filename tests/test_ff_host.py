"""Host-side checks of the arithmetic helpers in phs_ff.h and phs_math.h (the headers
compile as plain C++): the integer-only conversions between doubles and float pairs that
the FP32-pair kernels use to keep conversions off the FP64 pipe, against long-double
references; the series atan of large Breit-Wigner arguments; the corrected products that
stand for the volume program's divisions by constants."""
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "gpu_phs_gb300", "csrc")

DRIVER = r"""
#include <cstdio>
#include <cmath>
#include <random>
#include "phs_ff.h"
int main() {
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  long bad_to = 0, bad_from = 0, bad_om = 0, n = 0;
  double worst_to = 0;
  for (int i = 0; i < 2000000; i++) {
    // a normalized pair: hi any float, lo within half an ulp of hi
    const double mag = std::ldexp(1.0, (int)(u(rng) * 60));
    const float hi = (float)(u(rng) * mag);
    if (hi == 0.0f) continue;
    const int e = std::ilogb(hi);
    float lo = (float)(u(rng) * std::ldexp(1.0, e - 24) * (i % 7 == 0 ? 1e-6 : 1.0));
    ff a = fast_two_sum(hi, lo);                      // renormalized
    const long double exact = (long double)a.hi + (long double)a.lo;
    const double got = ff_to_double_int(a);
    // within one ulp of the double nearest to the exact sum (bits below it are dropped)
    const double near = (double)exact;
    const double ulp = std::nextafter(std::fabs(near), INFINITY) - std::fabs(near);
    const double err = std::fabs(got - near) / ulp;
    if (err > 1.0) bad_to++;
    if (err > worst_to) worst_to = err;
    // double -> pair (truncation to 48 bits) and back: within 2^-47 relative
    const double d = u(rng) * mag;
    if (d != 0.0) {
      const ff f = ff_from_double_int(d);
      const long double back = (long double)f.hi + (long double)f.lo;
      if (std::fabs((double)((back - d) / d)) > std::ldexp(1.0, -47)) bad_from++;
    }
    // 1 - x for x in [0, 1): relative accuracy 2^-46, also as x -> 1
    const double x = std::fabs(u(rng));
    const ff om = ff_one_minus_double_int(x);
    const long double want = 1.0L - (long double)x;
    if (want > 0 && std::fabs((double)(((long double)om.hi + om.lo - want) / want)) > std::ldexp(1.0, -46))
      bad_om++;
    n++;
  }
  std::printf("%ld %ld %ld %ld %.3f\n", n, bad_to, bad_from, bad_om, worst_to);
  return 0;
}
"""


def test_integer_conversions_of_float_pairs():
    try:
        subprocess.run(["g++", "--version"], check=True, capture_output=True)
    except (OSError, subprocess.CalledProcessError):
        pytest.skip("g++ not available")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "ff.cpp"), os.path.join(d, "ff")
        with open(src, "w") as fh:
            fh.write(DRIVER)
        subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-I", CSRC, src, "-o", exe],
                       check=True)
        n, bad_to, bad_from, bad_om, worst = subprocess.run(
            [exe], check=True, capture_output=True, text=True).stdout.split()
    assert int(n) > 1_900_000
    assert int(bad_to) == 0, f"ff_to_double_int off by more than an ulp ({worst} ulp)"
    assert int(bad_from) == 0 and int(bad_om) == 0


ATAN_DRIVER = r"""
#include <cmath>
#include <cstdio>
#include <random>
#include "phs_math.h"
int main() {
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> u(3.0, 13.0);
  double worst = 0;
  for (int i = 0; i < 2000000; i++) {
    const double x = std::pow(10.0, u(rng));          // 10^3 .. 10^13
    const long double exact = atanl((long double)x);
    const double got = phs_atan_bw(x);
    const double ulp = std::nextafter(1.5707963267948966, 0.0) - 1.5707963267948966;
    const double err = std::fabs((double)((long double)got - exact)) / std::fabs(ulp);
    if (err > worst) worst = err;
  }
  std::printf("%.4f\n", worst);
  return 0;
}
"""


def test_atan_of_large_breit_wigner_arguments():
    """phs_atan_bw: pi/2 - atan(1/u) by three series terms for u >= 1024, within one ulp
    of atan(u) over 10^3 .. 10^13 (long double reference)."""
    try:
        subprocess.run(["g++", "--version"], check=True, capture_output=True)
    except (OSError, subprocess.CalledProcessError):
        pytest.skip("g++ not available")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "at.cpp"), os.path.join(d, "at")
        with open(src, "w") as fh:
            fh.write(ATAN_DRIVER)
        subprocess.run(["g++", "-O2", "-std=c++17", "-I", CSRC, src, "-o", exe], check=True)
        worst = float(subprocess.run([exe], check=True, capture_output=True, text=True).stdout)
    assert worst <= 1.0, f"{worst} ulp"


DIV_DRIVER = r"""
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include "phs_math.h"
int main() {
  const double TWOPI2 = 39.47841760435743447534, TWOPI5 = 9792.62991312900650440772;
  const double cs[2] = {4 * TWOPI2, 4 * TWOPI5};   // the volume program's divisors
  std::mt19937_64 rng(11);
  long n = 0, bad = 0;
  for (double b : cs) {
    volatile double one = 1.0;
    const double rb = one / b;
    for (int i = 0; i < 20000000; i++) {
      // full random significand, exponent spread over 2^-300 .. 2^300, both signs
      const uint64_t bits = (rng() & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(1023 - 300 + rng() % 601) << 52);
      double a;
      std::memcpy(&a, &bits, 8);
      volatile double ref = a / b;
      n++;
      if (phs_div_by_const(a, b, rb) != ref) bad++;
    }
  }
  std::printf("%ld %ld\n", n, bad);
  return 0;
}
"""


def test_corrected_products_equal_the_divisions_by_constants():
    """phs_div_by_const(a, b, RN(1/b)) is a / b bit for bit for the volume program's
    constants 4 (2 pi)^2 and 4 (2 pi)^5, over 4e7 random a of every magnitude."""
    try:
        subprocess.run(["g++", "--version"], check=True, capture_output=True)
    except (OSError, subprocess.CalledProcessError):
        pytest.skip("g++ not available")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "dv.cpp"), os.path.join(d, "dv")
        with open(src, "w") as fh:
            fh.write(DIV_DRIVER)
        subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-I", CSRC, src, "-o", exe],
                       check=True)
        n, bad = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    assert int(n) == 40_000_000
    assert int(bad) == 0


FUNC_DRIVER = r"""
#include <cstdio>
#include <cmath>
#include <random>
#include "phs_ff.h"
static long double ld(ff a) { return (long double)a.hi + (long double)a.lo; }
static ff from_ld(long double v) { float hi = (float)v; float lo = (float)(v - hi); return ff_make(hi, lo); }
int main() {
  static FFTables T;
  ff_fill_tables(T);
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  const long double PI = 3.14159265358979323846264338327950288L;
  double w[10] = {0};
  for (int i = 0; i < 400000; i++) {
    ff x = from_ld((long double)u(rng)), s, c;            // sin, cos (2 pi x), x in [0, 1]
    ff_sincos2pi(x, T, s, c);
    const long double a = 2 * PI * ld(x);
    w[0] = std::fmax(w[0], (double)std::fmax(std::fabs(ld(s) - sinl(a)), std::fabs(ld(c) - cosl(a))));
    ff z = from_ld(((long double)u(rng) * 2 - 1) * (PI / 2 + PI / 64));   // sin, cos (z)
    ff_sincos(z, T, s, c);
    w[1] = std::fmax(w[1], (double)std::fmax(std::fabs(ld(s) - sinl(ld(z))), std::fabs(ld(c) - cosl(ld(z)))));
    ff zt = from_ld(((long double)u(rng) * 2 - 1) * (PI / 2 - 1e-3L));     // tan, relative
    const long double tt = tanl(ld(zt));
    if (tt != 0) w[2] = std::fmax(w[2], (double)std::fabs((ld(ff_tan(zt, T)) - tt) / tt));
    ff y = from_ld(((long double)u(rng) * 2 - 1) * 40);                    // exp, relative
    w[3] = std::fmax(w[3], (double)std::fabs((ld(ff_exp(y, T)) - expl(ld(y))) / expl(ld(y))));
    ff p = from_ld(std::ldexp((long double)u(rng) + 0.5L, (int)(u(rng) * 40) - 20));
    ff q = from_ld(std::ldexp((long double)u(rng) + 0.5L, (int)(u(rng) * 40) - 20));
    w[4] = std::fmax(w[4], (double)std::fabs((ld(ff_sqrt_fast(p)) - sqrtl(ld(p))) / sqrtl(ld(p))));
    w[5] = std::fmax(w[5], (double)std::fabs((ld(ff_div_fast(p, q)) - ld(p) / ld(q)) / (ld(p) / ld(q))));
    w[6] = std::fmax(w[6], (double)std::fabs((ld(ff_recip_fast(q)) - 1 / ld(q)) * ld(q)));
    w[7] = std::fmax(w[7], (double)std::fabs((ld(ff_mul(p, q)) - ld(p) * ld(q)) / (ld(p) * ld(q))));
    const long double sum = ld(p) + ld(q);
    w[8] = std::fmax(w[8], (double)std::fabs((ld(ff_add(p, q)) - sum) / sum));
    ff r1 = from_ld((long double)u(rng) - 0.5L), r2 = from_ld((long double)u(rng) - 0.5L);
    ff r3 = from_ld((long double)u(rng) - 0.5L), r4 = from_ld((long double)u(rng) - 0.5L);
    const long double d3 = ld(p) * ld(r1) + ld(q) * ld(r2) + ld(r3) * ld(r4);
    const long double mag = std::fabs(ld(p) * ld(r1)) + std::fabs(ld(q) * ld(r2)) + std::fabs(ld(r3) * ld(r4));
    w[9] = std::fmax(w[9], (double)(std::fabs(ld(ff_dot3(p, r1, q, r2, r3, r4)) - d3) / mag));
  }
  for (int k = 0; k < 10; k++) std::printf("%.6g ", w[k]);
  std::printf("\n");
  return 0;
}
"""


def test_float_pair_functions_against_long_double():
    """The float-float elementary functions and arithmetic of the FP32-pair kernels (table
    sin/cos, tan, exp, the reciprocal-estimate square root and division, product, sum,
    dot product) against long double, on the host (where the hardware estimates are exact
    divisions; the Newton steps bring the device's to the same accuracy).  Bars: absolute
    2e-13 for sin and cos, relative 5e-13 for tan (|z| < pi/2 - 1e-3) and exp (|y| < 40),
    relative 1e-13 for the arithmetic (the dot product relative to the sum of |terms|);
    measured 5e-14, 1.1e-13, 1.5e-13 and at most 3e-14."""
    try:
        subprocess.run(["g++", "--version"], check=True, capture_output=True)
    except (OSError, subprocess.CalledProcessError):
        pytest.skip("g++ not available")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "fn.cpp"), os.path.join(d, "fn")
        with open(src, "w") as fh:
            fh.write(FUNC_DRIVER)
        subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-I", CSRC, src, "-o", exe],
                       check=True)
        w = [float(v) for v in subprocess.run([exe], check=True, capture_output=True,
                                              text=True).stdout.split()]
    names = ["sincos2pi", "sincos", "tan", "exp", "sqrt", "div", "recip", "mul", "add", "dot3"]
    bars = [2e-13, 2e-13, 5e-13, 5e-13] + [1e-13] * 6
    for name, got, bar in zip(names, w, bars):
        assert got <= bar, f"{name}: {got:.3g} > {bar:g}"
