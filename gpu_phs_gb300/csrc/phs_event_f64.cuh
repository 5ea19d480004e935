// phs_event_f64.cuh -- one event of the forward map in FP64 (device code shared by the
// FP64 kernel and, as the exact fallback near kinematic limits, by the FP32-pair kernel).
//
// Arithmetic follows the reference CPU path (phs_cpu.cpp), whose expression order it keeps
// with explicit round-to-nearest intrinsics wherever a value feeds the kinematic ok test
// (msq mappings, the Kallen function and the mass sums), so ok flags match the reference
// bit for bit whenever the transcendental functions agree; factors and boosts use FMA.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "phs_device.h"
#include "phs_math.h"
#include "phs_program.h"

#define PHS_PI 3.14159265358979323846
#define PHS_TWOPI2 39.47841760435743447534
#define PHS_TWOPI5 9792.62991312900650440772
#define PHS_STATE 21  // doubles per saved frame: L[16], msq, m, p, m_max, E

namespace {


__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// msq from x (phs_cpu.cpp:12-61), same expression order, no contraction.  aux receives the
// mapping's transcendental term for the adjoint's derivatives: tan z (Breit-Wigner), the
// exponential term a0 exp(.) (collinear, infrared, radiation, t/u channel), exp(.)(1 + a1)
// (STEP_E); 0 otherwise.
__device__ __forceinline__ void map_msq(int t, double x, double s, double m, double w,
                                        double msq_min, double msq_max, double a0, double a1,
                                        double a2, double &msq, double &f, double &aux) {
  aux = 0.0;
  switch (t) {
    case PHS_MAP_NO:
      msq = dadd(dmul(dsub(1.0, x), msq_min), dmul(x, msq_max));
      f = (msq_max - msq_min) / s;
      break;
    case PHS_MAP_SCHANNEL: {
      double z = dadd(dmul(dsub(1.0, x), a0), dmul(x, a1));
      if (-PHS_PI / 2 < z && z < PHS_PI / 2) {
        double tz = tan(z);
        msq = dmul(m, dadd(m, dmul(w, tz)));
        f = a2 * (1.0 + tz * tz);
        aux = tz;
      } else {
        msq = 0.0;
        f = 0.0;
      }
      break;
    }
    case PHS_MAP_COLLINEAR:
    case PHS_MAP_INFRARED:
    case PHS_MAP_RADIATION: {
      double msq1 = dmul(a0, exp(dmul(x, a1)));
      msq = dadd(dsub(msq1, a0), msq_min);
      f = a2 * msq1;
      aux = msq1;
      break;
    }
    case PHS_MAP_TCHANNEL:
    case PHS_MAP_UCHANNEL: {
      // one exponential per lane: the side of x = 0.5 selects its argument and the sum
      const bool lower = x < 0.5;
      const double msq1 = dmul(a0, exp(dmul(lower ? x : dsub(1.0, x), a1)));
      msq = lower ? dadd(dsub(msq1, a0), msq_min) : dadd(-dsub(msq1, a0), msq_max);
      f = a2 * msq1;
      aux = msq1;
      break;
    }
    case PHS_MAP_STEP_H: {
      double am = dsub(a0, x);
      double z = dadd(dsub(a1 / am, a1 / a0), dmul(a2, x));
      msq = dadd(dmul(z, msq_max), dmul(dsub(1.0, z), msq_min));
      f = (a1 / (am * am) + a2) * (msq_max - msq_min) / s;
      break;
    }
    case PHS_MAP_STEP_E: {
      double tmp = dmul(exp(dmul(-x, a0) / a2), dadd(1.0, a1));
      double z = dmul(-a2, log(dsub(tmp, a1)));
      msq = dadd(dmul(z, msq_max), dmul(dsub(1.0, z), msq_min));
      f = a0 / (1.0 - a1 / tmp) * (msq_max - msq_min) / s;
      aux = tmp;
      break;
    }
    default:
      msq = 0.0;
      f = 0.0;
  }
}

__device__ __forceinline__ void map_msq(int t, double x, double s, double m, double w,
                                        double msq_min, double msq_max, double a0, double a1,
                                        double a2, double &msq, double &f) {
  double aux;
  map_msq(t, x, s, m, w, msq_min, msq_max, a0, a1, a2, msq, f, aux);
}

// cos(theta) from x (phs_cpu.cpp:112-146).  The collinear branch keeps the reference's
// rounding: sin(theta) = sqrt(1 - ct^2) is ill-conditioned as |ct| -> 1.
__device__ __forceinline__ void map_ct(int ct_class, double x, double b0, double b1, double &ct,
                                       double &st, double &f) {
  if (ct_class == PHS_CT_COLLINEAR) {
    const bool lower = x < 0.5;
    const double tmp = dmul(b0, exp(dmul(dmul(2.0, lower ? x : dsub(1.0, x)), b1)));
    ct = lower ? dsub(dsub(tmp, b0), 1.0) : dadd(-dsub(tmp, b0), 1.0);
    if (ct >= -1.0 && ct <= 1.0) {
      st = sqrt(dsub(1.0, dmul(ct, ct)));
      f = tmp * b1;
    } else {
      ct = 1.0;
      st = 0.0;
      f = 0.0;
    }
  } else {
    double tmp = 2.0 * (1.0 - x);
    ct = 1.0 - tmp;
    st = sqrt(tmp * (2.0 - tmp));
    f = 1.0;
  }
}

// Rotation taking the z axis onto the direction of (bx, by, bz) about the axis z x b
// (Rodrigues), row-major 3x3: the friend boost's rotation (phs.cu:753-781 restated; the
// reference's matrix equals this one whenever by = 0, which holds for friends on the root's
// daughters, the only ones Whizard's trees carry).  The symmetric part is written as
// cos + (1 - cos) k k^T with k k^T from the transverse components, as the reference does:
// the form cos + sin^2/(1 + cos) turns rounding of the normalisation into errors of order
// eps/(1 + cos) as the axis approaches -z.  An axis exactly along -z (where the reference
// divides 0 by 0) gives the rotation by pi about x.
__device__ __forceinline__ void rot_z_onto(double bx, double by, double bz, double R[9]) {
  const double n = sqrt(bx * bx + by * by + bz * bz);
  bx /= n;
  by /= n;
  bz /= n;
  const double t = bx * bx + by * by;
  double r00 = 1.0, r01 = 0.0, r11 = bz;
  if (t > 0.0) {
    const double w = (1.0 - bz) / t;
    r00 = bz + w * (by * by);
    r01 = -w * (bx * by);
    r11 = bz + w * (bx * bx);
  }
  R[0] = r00; R[1] = r01; R[2] = bx;
  R[3] = r01; R[4] = r11; R[5] = by;
  R[6] = -bx; R[7] = -by; R[8] = bz;
}

// The channel's phase-space volume at sqrt(s) (phs_cpu.cpp:194-213), bottom-up in post-order
// with the reference's operation order: for the per-event-beam paths.  The divisions by
// the two constants are the correctly rounded corrected products (phs_div_by_const): the
// same bits.
__device__ __forceinline__ double channel_volume(const PhsChannel &ch, double sqrts) {
  double vol[PHS_MAX_VISITS];
  constexpr double c_int = 4 * PHS_TWOPI2, c_root = 4 * PHS_TWOPI5;
  constexpr double r_int = 1.0 / c_int, r_root = 1.0 / c_root;
  for (int i = 0; i < ch.n_vol; i++) {
    int k1 = ch.vol_child[i][0], k2 = ch.vol_child[i][1];
    double v1 = k1 >= 0 ? vol[k1] : 1.0, v2 = k2 >= 0 ? vol[k2] : 1.0;
    vol[i] = ch.vol_is_root[i] ? phs_div_by_const(dmul(v1, v2), c_root, r_root)
                               : phs_div_by_const(dmul(dmul(dmul(v1, v2), sqrts), sqrts), c_int, r_int);
  }
  return vol[ch.n_vol - 1];
}

// Mapping constants at one sqrt(s) (phs_cpu.cpp:452-531), for the per-event-beam path.
// inv_s = 1/s of the event.  The reference divides a2 by s and the Breit-Wigner argument by
// m w; here they are products with 1/s (once per event) and the compiled 1/(m w), within an
// ulp of the quotients (a2 weights the factor; a1 = atan(u) at u >= 10^3 moves by ulp/u).
// msq_min = m_min^2 and m^2 do not depend on sqrt(s): the compiled values (the same bits).
__device__ void child_constants(const PhsChild &C, double sqrts, double m_tot, double inv_s,
                                double &a0, double &a1, double &a2, double &msq_min,
                                double &msq_max, double &m_max) {
  double m = C.m, w = C.w, m_min = C.m_min;
  m_max = dadd(dsub(sqrts, m_tot), m_min);
  msq_min = C.msq_min;
  msq_max = dmul(m_max, m_max);
  a0 = a1 = a2 = 0.0;
  switch (C.map_id) {
    case PHS_MAP_NO:
      a1 = msq_max - msq_min;
      a2 = a1 * inv_s;
      break;
    case PHS_MAP_SCHANNEL: {
      // a0 = atan((msq_min - m^2) / (m w)) does not depend on sqrt(s): the compiled
      // program's value (the host's atan of the same argument bits, as the reference's CPU
      // path computes it) serves every event
      const double mw = dmul(m, w);
      a0 = C.a0;
      a1 = phs_atan_bw(dsub(msq_max, C.msq0) * C.inv_mw);   // argument >= 10^3 here in practice
      a2 = dmul(dsub(a1, a0), mw) * inv_s;
      break;
    }
    case PHS_MAP_RADIATION:
    case PHS_MAP_COLLINEAR:
    case PHS_MAP_INFRARED: {
      double msq0 = C.map_id == PHS_MAP_RADIATION ? dmul(w, w) : dmul(m, m);
      a0 = msq0;
      a1 = log(dadd(dsub(msq_max, msq_min) / msq0, 1.0));
      a2 = a1 * inv_s;
      break;
    }
    case PHS_MAP_TCHANNEL:
    case PHS_MAP_UCHANNEL: {
      double msq0 = dmul(m, m);
      a0 = msq0;
      a1 = dmul(2.0, log(dadd(dsub(msq_max, msq_min) / dmul(2.0, msq0), 1.0)));
      a2 = a1 * inv_s;
      break;
    }
    case PHS_MAP_STEP_E: {
      double r = dmul(dmul(2.0, m), w) / dsub(msq_max, msq_min);
      a2 = r > 0.01 ? r : 0.01;
      a1 = exp(-(dsub(dmul(m, m), msq_min)) / dsub(msq_max, msq_min) / a2);
      a0 = dsub(1.0, dmul(a2, log(dadd(1.0, dmul(a1, exp(1.0 / a2))) / dadd(1.0, a1))));
      break;
    }
    case PHS_MAP_STEP_H: {
      a2 = dsub(dmul(m, m), msq_min) / dsub(msq_max, msq_min);
      double q = dmul(dmul(2.0, m), w) / dsub(msq_max, msq_min);
      double r = dmul(q, q) / a2;
      a1 = r > 0.000001 ? r : 0.000001;
      a0 = dadd(1.0, sqrt(dadd(1.0, dmul(4.0, a1) / dsub(1.0, a2)))) / 2.0;
      break;
    }
  }
}

#define PHS_TRIG_N 256   // entries of the sin/cos table: (sin, cos)(2 pi k / 256)

// sin and cos of 2 pi x: the nearest multiple k/256 of x, tab[k] = (sin, cos)(2 pi k / 256)
// from a table, and the Taylor series of sine and cosine of the remainder angle
// t = 2 pi (x - k/256), |t| <= pi/256 (terms through t^7 and t^6: the next ones are below
// 2e-20 of the result), joined by the angle-addition formulas.  Within 2 ulp of
// sincospi(2x).  x - k/256 is exact (Sterbenz); for 0 <= x < 2 (every x a phi mapping
// reads) k and the remainder come from the bits of x with integer operations, which keeps
// the reduction off the FP64 pipe (two FP64 operations: the remainder's conversion and its
// product with 2 pi), otherwise from rint.
__device__ __forceinline__ void sincos2pi_tab(double x, const double2 *tab, double &s, double &c) {
  const long long b = __double_as_longlong(x);
  const int bexp = (int)(b >> 52);   // biased exponent (b >= 0: the sign bit is clear)
  double t;
  int k;
  if (b >= 0 && bexp <= 1023) {
    // x = M 2^(e - 52) with the 53-bit significand M; 256 x = M 2^-sh, sh = 44 - e
    const bool small = bexp < 1023 - 9;   // x < 2^-9: k = 0, t = 2 pi x
    const int e = small ? -9 : bexp - 1023;
    const long long M = (b & ((1ll << 52) - 1)) | (1ll << 52);
    const int sh = 44 - e;                                   // 44 .. 53
    const int kk = (int)((M + (1ll << (sh - 1))) >> sh);     // round(256 x)
    const long long r = M - ((long long)kk << sh);           // x - k/256 = r 2^(e - 52)
    // 2 pi 2^(e - 52): 2 pi with its exponent lowered (a normal number, exact)
    const double c2 = __longlong_as_double(__double_as_longlong(6.283185307179586) +
                                           ((long long)(e - 52) << 52));
    k = small ? 0 : kk;
    t = (small ? x : (double)r) * (small ? 6.283185307179586 : c2);
  } else {
    const double kd = rint(x * (double)PHS_TRIG_N);
    k = (int)((long long)kd & (PHS_TRIG_N - 1));
    t = (x - kd * (1.0 / PHS_TRIG_N)) * 6.283185307179586;
  }
  const double t2 = t * t;
  const double sr = t + t * t2 * (-1.0 / 6 + t2 * (1.0 / 120 + t2 * (-1.0 / 5040)));
  const double cr = 1.0 + t2 * (-0.5 + t2 * (1.0 / 24 + t2 * (-1.0 / 720)));
  const double2 v = tab[k & (PHS_TRIG_N - 1)];
  s = v.x * cr + v.y * sr;
  c = v.y * cr - v.x * sr;
}

// Fills the PHS_TRIG_N-entry table of sincos2pi_tab (the block's threads in turn; the
// caller synchronises).  Multiples of pi/2 are exact.
__device__ __forceinline__ void fill_trig_table(double2 *tab) {
  for (int k = threadIdx.x; k < PHS_TRIG_N; k += blockDim.x) {
    double sv, cv;
    sincospi(k / (PHS_TRIG_N / 2.0), &sv, &cv);
    if (k % (PHS_TRIG_N / 4) == 0) {
      const int q = k / (PHS_TRIG_N / 4);
      sv = q == 1 ? 1.0 : (q == 3 ? -1.0 : 0.0);
      cv = q == 0 ? 1.0 : (q == 2 ? -1.0 : 0.0);
    }
    tab[k] = make_double2(sv, cv);
  }
}

// Frame stack slot k of depth `depth`: one column per thread of a BLOCK-thread block.
template <int BLOCK>
__device__ __forceinline__ void stack_store(double *smem, int depth, int k, double v) {
  smem[(depth * PHS_STATE + k) * BLOCK + threadIdx.x] = v;
}
template <int BLOCK>
__device__ __forceinline__ double stack_load(const double *smem, int depth, int k) {
  return smem[(depth * PHS_STATE + k) * BLOCK + threadIdx.x];
}

// One event: segment `seg`, local index `local` (< seg.ev_count).  smem is this block's
// frame stack, PHS_STATE * stack_depth doubles per thread of a BLOCK-thread block; trig the
// block's table of sincos2pi_tab.
// Checked build (phs_check.h): the event's channel, its whole x row, momentum row and event
// entries, and its program's visit count, before anything is read or written.
__device__ __forceinline__ bool event_in_bounds(const PhsLaunch &a, const PhsSegment &seg,
                                                int64_t local, int n_out, int n_visits) {
  const int64_t xrow = seg.x_base + local * seg.x_stride;
  const int64_t prow = seg.p_base + local * 4 * (int64_t)n_out;
  const int64_t ev = seg.ev_begin + local;
  return phs_in(local, seg.ev_count, PHS_CHK_EVENT) && phs_in(xrow, a.x_len, PHS_CHK_X) &&
         phs_in(xrow + seg.x_stride - 1, a.x_len, PHS_CHK_X) && phs_in(prow, a.p_len, PHS_CHK_P) &&
         phs_in(prow + 4 * (int64_t)n_out - 1, a.p_len, PHS_CHK_P) &&
         phs_in(ev, a.ev_len, PHS_CHK_EVENT) && phs_in(seg.factor_col, a.factor_stride, PHS_CHK_EVENT) &&
         phs_in(n_visits - 1, PHS_MAX_VISITS, PHS_CHK_VISITS);
}

// x[k] of an event row (checked build: k within the row; 0 otherwise).
__device__ __forceinline__ double xrow_at(const double *xe, int k, int stride) {
  return phs_in(k, stride, PHS_CHK_X) ? xe[k] : 0.0;
}

template <bool PER_EVENT, int BLOCK = PHS_FWD_BLOCK>
__device__ __forceinline__ void phs_event_f64(const PhsLaunch &a, const PhsSegment &seg,
                                              int64_t local, double *smem, const double2 *trig) {
  if (!phs_in(seg.channel, a.n_programs, PHS_CHK_CHANNEL)) return;
  const PhsChannel &ch = a.channels[seg.channel];
  if (!event_in_bounds(a, seg, local, ch.n_out, ch.n_visits)) return;
  const int64_t ev = seg.ev_begin + local;
  const double *xe = a.x + seg.x_base + local * seg.x_stride;
  double *out = a.p + seg.p_base + local * 4 * (int64_t)ch.n_out;

  double sqrts = ch.sqrts;
  double lab_bg = ch.lab_bg, lab_ga = ch.lab_gamma;
  bool lab = ch.lab != 0;
  if (PER_EVENT) {
    double E1 = a.E1[ev], E2 = a.E2[ev];
    double r = sqrt(dmul(E1, E2));
    sqrts = dmul(2.0, r);
    lab = E1 != E2;
    lab_bg = dsub(E1, E2) / dmul(2.0, r);
    lab_ga = sqrt(1.0 + lab_bg * lab_bg);
  }
  const double s = dmul(sqrts, sqrts);
  const double inv_s = PER_EVENT ? 1.0 / s : 0.0;   // per-event mapping constants

  // frame of the visited branch; the root's parent frame is the lab boost (or 1)
  double L[16];
#pragma unroll
  for (int i = 0; i < 16; i++) L[i] = 0.0;
  L[0] = lab ? lab_ga : 1.0;
  L[5] = 1.0;
  L[10] = 1.0;
  L[15] = L[0];
  L[3] = lab ? lab_bg : 0.0;
  L[12] = L[3];
  double msq_b = s, m_b = sqrts, p_b = 0.0, mmax_b = sqrts, E_b = sqrts;
  double factor = 1.0;
  bool ok = true;
  int sp = 0;

  const int n_visits = ch.n_visits;
  for (int v = 0; v < n_visits; v++) {
    const PhsVisit &V = ch.visit[v];
    double cmsq[2], cm[2], cmax[2];
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const PhsChild &C = V.child[j];
      if (!C.internal) {
        cmsq[j] = C.msq_leaf;
        cm[j] = C.m_leaf;
        cmax[j] = 0.0;
      } else {
        double a0 = C.a0, a1 = C.a1, a2 = C.a2, mn = C.msq_min, mx = C.msq_max;
        cmax[j] = C.m_max;
        if (PER_EVENT) child_constants(C, sqrts, ch.m_tot, inv_s, a0, a1, a2, mn, mx, cmax[j]);
        double f;
        map_msq(C.map_id, xrow_at(xe, C.x_msq, seg.x_stride), s, C.m, C.w, mn, mx, a0, a1, a2,
                cmsq[j], f);
        factor *= f;
        cm[j] = sqrt(cmsq[j]);
      }
    }
    // Kallen function and kinematic test at the visited branch (phs_cpu.cpp:218-233)
    double d = dsub(dsub(msq_b, cmsq[0]), cmsq[1]);
    double lda = dsub(dmul(d, d), dmul(dmul(4.0, cmsq[0]), cmsq[1]));
    ok = ok && (lda > 0.0) && (m_b > dadd(cm[0], cm[1])) && (m_b <= mmax_b);
    // one reciprocal of m serves p_decay = sqrt(lda)/(2m), sqrt(lda)/m^2, bg, gamma and the
    // daughters' energies E = (m^2 + m_j^2 - m_k^2)/(2m) (the two-body energy, equal to the
    // reference's sqrt(m_j^2 + p^2))
    const double sl = sqrt(lda);
    const double rm = m_b > 0.0 ? __drcp_rn(m_b) : 0.0;
    const double hm = 0.5 * rm;
    const double pc = sl * hm;
    factor *= (sl * rm) * rm;
    const double ce0 = (msq_b + cmsq[0] - cmsq[1]) * hm;
    const double ce1 = (msq_b + cmsq[1] - cmsq[0]) * hm;

    // rotation + boost of the visited branch (phs_cpu.cpp:299-330)
    const double bg = p_b * rm;
    const double ga = V.self_root ? 1.0 : E_b * rm;
    double sphi, cphi;
    sincos2pi_tab(xrow_at(xe, V.x_phi, seg.x_stride), trig, sphi, cphi);
    double b0 = V.b0, b1 = V.b1;
    if (PER_EVENT && V.ct_class == PHS_CT_COLLINEAR) {
      b0 = dmul(V.m, V.m) / s;
      b1 = log(dadd(b0, 1.0) / b0);
    }
    double ct, st, fct;
    map_ct(V.ct_class, xrow_at(xe, V.x_ct, seg.x_stride), b0, b1, ct, st, fct);
    if (V.ct_class == PHS_CT_COLLINEAR) factor *= fct;   // the uniform map's factor is 1
    const double e03 = bg * ct, e12 = -sphi, e13 = st * cphi;
    const double e22 = cphi, e23 = st * sphi, e33 = ga * ct;
    // the entries of L1 that only the frame's columns 1 and 2 read: formed in the branches
    // that write those (a leaf-only visit writes columns 0 and 3 only)
    const auto col12 = [&](double &e01, double &e11, double &e21, double &e31) {
      e01 = -bg * st;
      e11 = ct * cphi;
      e21 = ct * sphi;
      e31 = -ga * st;
    };

    // the frame is updated in place: row r of L L1 depends on row r of L only
    if (V.friend_sign != 0) {
      // friend boost (phs.cu:853-910): the decay angles are measured from the friend
      // beam's direction in the branch's rest frame, B_z(-bg) L^-1 (1, 0, 0, ff) (only
      // its direction matters, so the lab boost inside L needs no special case);
      // L1 = B_z(bg) diag(1, R_f R(theta, phi)).  Uniform per channel: no divergence.
      const double ff = V.friend_sign;
      const double u0 = L[0] - ff * L[12];
      double Rf[9];
      rot_z_onto(-(L[1] - ff * L[13]), -(L[2] - ff * L[14]),
                 -bg * u0 - ga * (L[3] - ff * L[15]), Rf);
      double e01, e11, e21, e31;
      col12(e01, e11, e21, e31);
      const double A[9] = {e11, e12, e13, e21, e22, e23, -st, 0.0, ct};
      double Q[9];
#pragma unroll
      for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++)
          Q[3 * r + c] = Rf[3 * r] * A[c] + Rf[3 * r + 1] * A[3 + c] + Rf[3 * r + 2] * A[6 + c];
      const double E1r[4] = {ga, bg * Q[6], bg * Q[7], bg * Q[8]};
      const double E2r[4] = {0.0, Q[0], Q[1], Q[2]};
      const double E3r[4] = {0.0, Q[3], Q[4], Q[5]};
      const double E4r[4] = {bg, ga * Q[6], ga * Q[7], ga * Q[8]};
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const double l0 = L[4 * r], l1 = L[4 * r + 1], l2 = L[4 * r + 2], l3 = L[4 * r + 3];
#pragma unroll
        for (int c = 0; c < 4; c++)
          L[4 * r + c] = l0 * E1r[c] + l1 * E2r[c] + l2 * E3r[c] + l3 * E4r[c];
      }
    } else if (V.self_root && !lab) {
      // parent frame is the identity: L0 * L1 = L1
      double e01, e11, e21, e31;
      col12(e01, e11, e21, e31);
      L[0] = ga;  L[1] = e01; L[2] = 0.0;  L[3] = e03;
      L[4] = 0.0; L[5] = e11; L[6] = e12;  L[7] = e13;
      L[8] = 0.0; L[9] = e21; L[10] = e22; L[11] = e23;
      L[12] = bg; L[13] = e31; L[14] = 0.0; L[15] = e33;
    } else if (PER_EVENT && V.self_root) {
      // (per-event beams, where nearly every event has a lab boost; the uniform-beam kernels
      // keep the general product, which leaves their registers to the common case)
      // the parent frame is the lab boost B_z(lab_bg): rows 1 and 2 are unit rows, and the
      // root's bg is 0 and its gamma 1
      double e01, e11, e21, e31;
      col12(e01, e11, e21, e31);
      const double g0 = L[0], b0 = L[3], b3 = L[12], g3 = L[15];
      L[0] = g0;     L[1] = b0 * e31;    L[2] = 0.0;  L[3] = b0 * e33;
      L[4] = 0.0;    L[5] = e11;         L[6] = e12;  L[7] = e13;
      L[8] = 0.0;    L[9] = e21;         L[10] = e22; L[11] = e23;
      L[12] = b3;    L[13] = g3 * e31;   L[14] = 0.0; L[15] = g3 * e33;
    } else if (V.parent_root && !lab) {
      // the parent frame is the root's rotation (its bg is 0 and its gamma 1): row 0 is
      // (1, 0, 0, 0) and L[4], L[8], L[12], L[14] are 0, so half the products drop out
      double e01 = 0.0, e11 = 0.0, e21 = 0.0, e31 = 0.0;
      if (!V.both_leaves) col12(e01, e11, e21, e31);
      L[0] = ga;  L[1] = e01; L[2] = 0.0;  L[3] = e03;
#pragma unroll
      for (int r = 1; r < 4; r++) {
        const double l1 = L[4 * r + 1], l2 = r < 3 ? L[4 * r + 2] : 0.0, l3 = L[4 * r + 3];
        L[4 * r + 0] = l3 * bg;
        L[4 * r + 3] = r < 3 ? l1 * e13 + l2 * e23 + l3 * e33 : l1 * e13 + l3 * e33;
        if (!V.both_leaves) {
          L[4 * r + 1] = r < 3 ? l1 * e11 + l2 * e21 + l3 * e31 : l1 * e11 + l3 * e31;
          L[4 * r + 2] = r < 3 ? l1 * e12 + l2 * e22 : l1 * e12;
        } else {
          L[4 * r + 1] = 0.0;
          L[4 * r + 2] = 0.0;
        }
      }
    } else if (PER_EVENT && V.parent_root) {
      // the root's frame with the lab boost: entries (0,2), (1,0), (2,0), (3,2) are 0
      double e01 = 0.0, e11 = 0.0, e21 = 0.0, e31 = 0.0;
      if (!V.both_leaves) col12(e01, e11, e21, e31);
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const double l0 = L[4 * r], l1 = L[4 * r + 1], l2 = L[4 * r + 2], l3 = L[4 * r + 3];
        const bool edge = r == 0 || r == 3;   // l2 = 0; otherwise l0 = 0
        L[4 * r + 0] = edge ? l0 * ga + l3 * bg : l3 * bg;
        L[4 * r + 3] = edge ? l0 * e03 + l1 * e13 + l3 * e33 : l1 * e13 + l2 * e23 + l3 * e33;
        if (!V.both_leaves) {
          L[4 * r + 1] = edge ? l0 * e01 + l1 * e11 + l3 * e31 : l1 * e11 + l2 * e21 + l3 * e31;
          L[4 * r + 2] = edge ? l1 * e12 : l1 * e12 + l2 * e22;
        } else {
          L[4 * r + 1] = 0.0;
          L[4 * r + 2] = 0.0;
        }
      }
    } else if (V.both_leaves) {
      // both daughters are leaves: their momenta read the frame's columns 0 and 3 only
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const double l0 = L[4 * r], l1 = L[4 * r + 1], l2 = L[4 * r + 2], l3 = L[4 * r + 3];
        L[4 * r + 0] = l0 * ga + l3 * bg;
        L[4 * r + 3] = l0 * e03 + l1 * e13 + l2 * e23 + l3 * e33;
        L[4 * r + 1] = 0.0;
        L[4 * r + 2] = 0.0;
      }
    } else {
      double e01, e11, e21, e31;
      col12(e01, e11, e21, e31);
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const double l0 = L[4 * r], l1 = L[4 * r + 1], l2 = L[4 * r + 2], l3 = L[4 * r + 3];
        L[4 * r + 0] = l0 * ga + l3 * bg;
        L[4 * r + 3] = l0 * e03 + l1 * e13 + l2 * e23 + l3 * e33;
        L[4 * r + 1] = l0 * e01 + l1 * e11 + l2 * e21 + l3 * e31;
        L[4 * r + 2] = l1 * e12 + l2 * e22;
      }
    }

    // leaf momenta: L_new * (E, 0, 0, +-p) (phs_cpu.cpp:286-291); the two leaves of a
    // leaf-only visit share the products L_new[r][3] p
    if (V.both_leaves) {
      double t3[4];
#pragma unroll
      for (int r = 0; r < 4; r++) t3[r] = L[4 * r + 3] * pc;
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const PhsChild &C = V.child[j];
        if (phs_in(C.out_index, ch.n_out, PHS_CHK_P)) {
          const double E = j == 0 ? ce0 : ce1;
          double q[4];
#pragma unroll
          for (int r = 0; r < 4; r++) q[r] = fma(L[4 * r], E, j == 0 ? t3[r] : -t3[r]);
          double2 *o = reinterpret_cast<double2 *>(out + 4 * C.out_index);
          o[0] = make_double2(q[0], q[1]);
          o[1] = make_double2(q[2], q[3]);
        }
      }
    } else {
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const PhsChild &C = V.child[j];
        if (!C.internal && phs_in(C.out_index, ch.n_out, PHS_CHK_P)) {
          double pj = j == 0 ? pc : -pc;
          const double E = j == 0 ? ce0 : ce1;
          double2 *o = reinterpret_cast<double2 *>(out + 4 * C.out_index);
          o[0] = make_double2(L[0] * E + L[3] * pj, L[4] * E + L[7] * pj);
          o[1] = make_double2(L[8] * E + L[11] * pj, L[12] * E + L[15] * pj);
        }
      }
    }

    // next frame: push one internal child, carry the other (or pop)
    // (selects instead of indexing keep the child values in registers)
    if (V.push >= 0 && phs_in(sp, a.stack_depth, PHS_CHK_STACK)) {
      const bool j0 = V.push == 0;
#pragma unroll
      for (int i = 0; i < 16; i++) stack_store<BLOCK>(smem, sp, i, L[i]);
      stack_store<BLOCK>(smem, sp, 16, j0 ? cmsq[0] : cmsq[1]);
      stack_store<BLOCK>(smem, sp, 17, j0 ? cm[0] : cm[1]);
      stack_store<BLOCK>(smem, sp, 18, j0 ? pc : -pc);
      stack_store<BLOCK>(smem, sp, 19, j0 ? cmax[0] : cmax[1]);
      stack_store<BLOCK>(smem, sp, 20, j0 ? ce0 : ce1);
      sp++;
    }
    if (V.carry >= 0) {
      const bool j0 = V.carry == 0;
      msq_b = j0 ? cmsq[0] : cmsq[1];
      m_b = j0 ? cm[0] : cm[1];
      p_b = j0 ? pc : -pc;
      mmax_b = j0 ? cmax[0] : cmax[1];
      E_b = j0 ? ce0 : ce1;
    } else if (sp > 0) {
      sp--;
#pragma unroll
      for (int i = 0; i < 16; i++) L[i] = stack_load<BLOCK>(smem, sp, i);
      msq_b = stack_load<BLOCK>(smem, sp, 16);
      m_b = stack_load<BLOCK>(smem, sp, 17);
      p_b = stack_load<BLOCK>(smem, sp, 18);
      mmax_b = stack_load<BLOCK>(smem, sp, 19);
      E_b = stack_load<BLOCK>(smem, sp, 20);
    }
  }

  a.volume[ev] = PER_EVENT ? channel_volume(ch, sqrts) : ch.volume;
  a.factor[ev * a.factor_stride + seg.factor_col] = ok ? factor : 0.0;
  a.ok[ev] = ok ? 1 : 0;
  if (!ok) {
    double2 *o = reinterpret_cast<double2 *>(out);
    for (int i = 0; i < 2 * ch.n_out; i++) o[i] = make_double2(0.0, 0.0);
  }
}


// Pass A of the compacting kernels: the kinematic test of one event alone -- the msq
// mappings of its internal branches and the Kallen / mass tests of phs_event_f64 in the
// same arithmetic, so the flag is the same bit -- without angles or boosts.  An event that
// fails gets its outputs here (momenta 0, factor 0, ok 0, the channel volume); one that
// passes gets them from phs_event_f64 in pass B.  Returns ok.  smem: the event's frame
// stack (only the msq, m and m_max slots are used).
template <bool PER_EVENT, int BLOCK = PHS_FWD_BLOCK>
__device__ __forceinline__ bool phs_ok_f64(const PhsLaunch &a, const PhsSegment &seg,
                                           int64_t local, double *smem) {
  if (!phs_in(seg.channel, a.n_programs, PHS_CHK_CHANNEL)) return false;
  const PhsChannel &ch = a.channels[seg.channel];
  if (!event_in_bounds(a, seg, local, ch.n_out, ch.n_visits)) return false;
  const int64_t ev = seg.ev_begin + local;
  const double *xe = a.x + seg.x_base + local * seg.x_stride;
  double sqrts = ch.sqrts;
  if (PER_EVENT) sqrts = dmul(2.0, sqrt(dmul(a.E1[ev], a.E2[ev])));
  const double s = dmul(sqrts, sqrts);
  const double inv_s = PER_EVENT ? 1.0 / s : 0.0;   // per-event mapping constants
  double msq_b = s, m_b = sqrts, mmax_b = sqrts;
  bool ok = true;
  int sp = 0;
  const int n_visits = ch.n_visits;
  for (int v = 0; v < n_visits; v++) {
    const PhsVisit &V = ch.visit[v];
    double cmsq[2], cm[2], cmax[2];
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const PhsChild &C = V.child[j];
      if (!C.internal) {
        cmsq[j] = C.msq_leaf;
        cm[j] = C.m_leaf;
        cmax[j] = 0.0;
      } else {
        double a0 = C.a0, a1 = C.a1, a2 = C.a2, mn = C.msq_min, mx = C.msq_max;
        cmax[j] = C.m_max;
        if (PER_EVENT) child_constants(C, sqrts, ch.m_tot, inv_s, a0, a1, a2, mn, mx, cmax[j]);
        double f;
        map_msq(C.map_id, xrow_at(xe, C.x_msq, seg.x_stride), s, C.m, C.w, mn, mx, a0, a1, a2,
                cmsq[j], f);
        cm[j] = sqrt(cmsq[j]);
      }
    }
    const double d = dsub(dsub(msq_b, cmsq[0]), cmsq[1]);
    const double lda = dsub(dmul(d, d), dmul(dmul(4.0, cmsq[0]), cmsq[1]));
    ok = ok && (lda > 0.0) && (m_b > dadd(cm[0], cm[1])) && (m_b <= mmax_b);
    if (V.push >= 0 && phs_in(sp, a.stack_depth, PHS_CHK_STACK)) {
      const bool j0 = V.push == 0;
      stack_store<BLOCK>(smem, sp, 16, j0 ? cmsq[0] : cmsq[1]);
      stack_store<BLOCK>(smem, sp, 17, j0 ? cm[0] : cm[1]);
      stack_store<BLOCK>(smem, sp, 19, j0 ? cmax[0] : cmax[1]);
      sp++;
    }
    if (V.carry >= 0) {
      const bool j0 = V.carry == 0;
      msq_b = j0 ? cmsq[0] : cmsq[1];
      m_b = j0 ? cm[0] : cm[1];
      mmax_b = j0 ? cmax[0] : cmax[1];
    } else if (sp > 0) {
      sp--;
      msq_b = stack_load<BLOCK>(smem, sp, 16);
      m_b = stack_load<BLOCK>(smem, sp, 17);
      mmax_b = stack_load<BLOCK>(smem, sp, 19);
    }
  }
  if (!ok) {
    double volume = ch.volume;
    if (PER_EVENT) {
      double vol[PHS_MAX_VISITS];
      const double c_int = 4 * PHS_TWOPI2, c_root = 4 * PHS_TWOPI5;
      for (int i = 0; i < ch.n_vol; i++) {
        int k1 = ch.vol_child[i][0], k2 = ch.vol_child[i][1];
        double v1 = k1 >= 0 ? vol[k1] : 1.0, v2 = k2 >= 0 ? vol[k2] : 1.0;
        vol[i] = ch.vol_is_root[i] ? dmul(v1, v2) / c_root
                                   : dmul(dmul(dmul(v1, v2), sqrts), sqrts) / c_int;
      }
      volume = vol[ch.n_vol - 1];
    }
    a.volume[ev] = volume;
    a.factor[ev * a.factor_stride + seg.factor_col] = 0.0;
    a.ok[ev] = 0;
    double2 *o = reinterpret_cast<double2 *>(a.p + seg.p_base + local * 4 * (int64_t)ch.n_out);
    for (int i = 0; i < 2 * ch.n_out; i++) o[i] = make_double2(0.0, 0.0);
  }
  return ok;
}

// The persistent loop of the compacting kernels.  Each warp runs pass A on its 32-event
// tiles (`pass_a(seg, local)` tests an event, writes it if it fails, and returns whether it
// passed) and appends the passing events to its queue in shared memory (q: 64 slots);
// pass B (`pass_b(seg_index, seg, local)`, the full event) drains the queue 32 events at a time with
// every lane busy.  The queue holds events of one segment only, so the visit program stays
// warp-uniform: a tile of another segment first drains it.  Pass A and pass B have one
// call site each, which keeps the (large) event code once in the kernel.
//
// Work is claimed in chunks of CHUNK consecutive tiles of one segment: CHUNK = 1 (single
// tiles), or PHS_CHUNK_TILES (PhsSegment::chunk_begin; a segment's last chunk may be
// shorter), whichever was measured faster for the kernel.  With a.work set, a warp claims
// its next chunk from that counter when it finishes one (events of different channels and
// kinematics cost very different amounts, and static shares leave SMs idle at the end);
// without, chunks are strided over the grid.
template <int CHUNK, class PassA, class PassB>
__device__ __forceinline__ void compacting_loop(const PhsLaunch &a, int64_t *q, PassA pass_a,
                                                PassB pass_b) {
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const PhsSegment *segs = a.n_segments <= PHS_INLINE_SEGS ? a.seg_inline : a.segments;
  int64_t claimed = 0;
  auto next_chunk = [&]() -> int64_t {
    if (a.work) {
      unsigned long long c = 0;
      if (lane == 0) c = atomicAdd(a.work, 1ull);
      return (int64_t)__shfl_sync(0xffffffffu, c, 0);
    }
    return warp0 + (claimed++) * n_warps;
  };
  int qn = 0, qseg = 0;  // warp-uniform: queue length and its segment
  int cseg = 0;          // segment of the current chunk
  int64_t tile = 0, tile_end = 0;
  bool done = false;
  static_assert(CHUNK == 1 || CHUNK == PHS_CHUNK_TILES, "chunks of 1 or PHS_CHUNK_TILES tiles");
  auto claim = [&]() {
    const int64_t c = next_chunk();
    done = c >= (CHUNK == 1 ? a.n_tiles : a.n_chunks);
    if (done) return;
    int lo = 0, hi = a.n_segments - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if ((CHUNK == 1 ? segs[mid].tile_begin : segs[mid].chunk_begin) <= c) lo = mid; else hi = mid - 1;
    }
    cseg = lo;
    if (CHUNK == 1) {
      tile = c;
      tile_end = c + 1;
      return;
    }
    const int64_t seg_tiles = (segs[lo].ev_count + 31) / 32;
    tile = segs[lo].tile_begin + (c - segs[lo].chunk_begin) * CHUNK;
    const int64_t end = tile + CHUNK, seg_end = segs[lo].tile_begin + seg_tiles;
    tile_end = end < seg_end ? end : seg_end;
  };
  claim();
  for (;;) {
    bool passed = false;
    int64_t local = 0;
    if (!done) {
      local = (tile - segs[cseg].tile_begin) * 32 + lane;
      if (local < segs[cseg].ev_count) passed = pass_a(segs[cseg], local);
    }
    const unsigned m = __ballot_sync(0xffffffffu, passed);
    // stage 0: drain the queue (end of the work, or a new segment); 1: append; 2: drain
    // full warps
    int stage = (done || (m != 0 && qn > 0 && qseg != cseg)) ? 0 : 1;
    for (;;) {
      int take;
      if (stage == 0) {
        if (qn == 0) { stage = 1; continue; }
        take = qn < 32 ? qn : 32;
      } else if (stage == 1) {
        if (m != 0) {
          const int slot = qn + __popc(m & ((1u << lane) - 1u));
          if (passed && phs_in(slot, 64, PHS_CHK_QUEUE)) q[slot] = local;
          qn += __popc(m);
          qseg = cseg;
        }
        stage = 2;
        continue;
      } else {
        if (qn < 32) break;
        take = 32;
      }
      __syncwarp();
      const int64_t l = lane < take && phs_in(qn - take + lane, 64, PHS_CHK_QUEUE) ? q[qn - take + lane] : -1;
      __syncwarp();
      qn -= take;
      if (l >= 0) pass_b(qseg, segs[qseg], l);
    }
    if (done) break;
    if (++tile == tile_end) claim();
  }
}

}  // namespace
