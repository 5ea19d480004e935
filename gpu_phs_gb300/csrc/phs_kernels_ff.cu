// phs_kernels_ff.cu -- forward phase-space kernel on the FP32 pipe (float-float pairs).
//
// Same walk as the FP64 kernel (visit programs, persistent grid, warp tiles of one
// channel), with every mapping, angle, boost and momentum in float-float arithmetic
// (phs_ff.h).  GB300 issues 64x more FP32 than FP64 operations per cycle, and a pair of
// floats carries ~48 bits, so momenta stay within ~1e-10 of the FP64 path.
//
// ok flags stay bit-exact with the reference: the kinematic test at every branch is
// decided in float-float only when the margins |m - m1 - m2| and |m_max - m| exceed
// 1e-5 of the mass (and msq is not within 1e-10 s of zero).  Otherwise -- and for channels
// with STEP mappings or friend boosts, which have no float-float form -- the event is
// queued for the exact FP64 path (phs_event_f64.cuh, launched behind this kernel by
// phs_launch_forward_exact), which also keeps p_decay near threshold in FP64.
// The Kallen function is evaluated in factored form, (m-m1-m2)(m+m1+m2)(m-m1+m2)(m+m1-m2),
// which keeps its relative accuracy close to threshold.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "phs_device.h"
#include "phs_event_f64.cuh"  // the compacting loop and rot_z_onto
#include "phs_ff.h"
#include "phs_program.h"

#define PHS_FF_STATE 40   // floats per saved frame: L[16], msq, m, p, m_max as pairs
#define PHS_FF_MARGIN 1e-5f     // kinematic margins decided in float-float
#define PHS_FF_MSQ_ZERO 1e-10f  // |msq| below this fraction of s takes the exact path
#define PHS_FF_TEST_MIN_BLOCKS 8  // resident blocks per SM of the stand-alone pre-test kernel

namespace {

__device__ __forceinline__ ff ld(const PhsFF &c) { return ff_make(c.hi, c.lo); }
__device__ __forceinline__ ff ffsel(bool c, ff a, ff b) { return c ? a : b; }

// A float-float frame value takes one 8-byte slot, (depth * 20 + k) * block + thread.
__device__ __forceinline__ void fstack_store(float *st, int depth, int k, ff v) {
  reinterpret_cast<float2 *>(st)[(depth * (PHS_FF_STATE / 2) + k) * PHS_FWD_BLOCK + threadIdx.x] =
      make_float2(v.hi, v.lo);
}
__device__ __forceinline__ ff fstack_load(const float *st, int depth, int k) {
  const float2 t =
      reinterpret_cast<const float2 *>(st)[(depth * (PHS_FF_STATE / 2) + k) * PHS_FWD_BLOCK + threadIdx.x];
  return ff_make(t.x, t.y);
}

__device__ __forceinline__ bool near_zero(ff v, float scale) {
  return fabsf(v.hi) <= PHS_FF_MARGIN * scale;
}
__device__ __forceinline__ bool msq_near_zero(ff v, float s) {
  return fabsf(v.hi) <= PHS_FF_MSQ_ZERO * s;
}

// The constants of an internal child that depend on sqrt(s): the mapping's a1 (Breit-Wigner:
// a1 - a0) and a2, pi/2 - a1, msq_max and the ok test's m_max.  From the channel program for
// uniform beams; per event from the FP64 constants for per-event beams (child_constants:
// what depends on sqrt(s) per event, as the reference's GPU path computes it).
struct ChildVar {
  ff a1, a2, u1, msq_max, m_max;
};
__device__ __forceinline__ ChildVar child_var(const PhsChildFF &C) {
  return {ld(C.a1), ld(C.a2), ld(C.u1), ld(C.msq_max), ld(C.m_max)};
}
__device__ __forceinline__ ChildVar child_var(const PhsChildFF &C, const PhsChild &C64,
                                              double sqrts, double m_tot, double inv_s) {
  double a0, a1, a2, mn, mx, mmax;
  child_constants(C64, sqrts, m_tot, inv_s, a0, a1, a2, mn, mx, mmax);
  // to pairs with integer operations: the FP64 pipe is the per-event path's scarce one
  ChildVar r;
  r.a2 = ff_from_double_int(a2);
  r.msq_max = ff_from_double_int(mx);
  r.m_max = ff_from_double_int(mmax);
  if (C.map_id == PHS_MAP_SCHANNEL) {
    r.a1 = ff_from_double_int(a1 - a0);
    // pi/2 - a1: exact for a1 >= pi/4 (the only case that uses it), then pi/2's low part
    r.u1 = ff_from_double_int((1.5707963267948966 - a1) + 6.123233995736766e-17);
  } else {
    r.a1 = ff_from_double_int(a1);
    r.u1 = ff_from_float(0.0f);
  }
  return r;
}

// Per-event constants in float-float (the FP32 pipe) for the uniform map and for
// Breit-Wigner maps whose range in widths u = (msq_max - m^2)/(m w) is at least 1024, where
// a1 = atan(u) = pi/2 - atan(1/u) and atan(w) = w - w^3/3 + w^5/5 for w = 1/u (the next term
// is below 2^-72 of pi/2, as in phs_math.h); pi/2 - a1 is that series itself.  Other maps
// and smaller u take the FP64 constants.  sqrts, inv_s: the event's sqrt(s) and 1/s.
__device__ __forceinline__ ChildVar child_var(const PhsChildFF &C, const PhsChild &C64, ff sqrts,
                                              ff inv_s, ff m_tot, double sqrts64, double m_tot64) {
  if (C.map_id == PHS_MAP_NO || C.map_id == PHS_MAP_SCHANNEL) {
    ChildVar r;
    r.m_max = ff_add(ff_sub(sqrts, m_tot), ld(C.m_min));
    r.msq_max = ff_sqr(r.m_max);
    if (C.map_id == PHS_MAP_NO) {
      r.a1 = ff_sub(r.msq_max, ld(C.msq_min));
      r.a2 = ff_mul(r.a1, inv_s);
      r.u1 = ff_from_float(0.0f);
      return r;
    }
    const ff u = ff_mul(ff_sub(r.msq_max, ld(C.m2)), ld(C.inv_mw));
    if (u.hi >= 1024.0f) {
      const ff w = ff_recip_fast(u), w2 = ff_sqr(w);
      r.u1 = ff_add(w, ff_mul(ff_mul(w, w2), ff_add_f(ff_mul_f(w2, 0.2f), -1.0f / 3.0f)));
      const ff a1 = ff_sub(ff_make(0.5f * FF_PI_HI, 0.5f * FF_PI_LO), r.u1);
      r.a1 = ff_sub(a1, ld(C.a0));                       // a1 - a0
      r.a2 = ff_mul(ff_mul(r.a1, ld(C.mw)), inv_s);
      return r;
    }
  }
  const double s64 = dmul(sqrts64, sqrts64);
  return child_var(C, C64, sqrts64, m_tot64, 1.0 / s64);
}

// msq from x in float-float; returns false when the event must take the exact path.
// x arrives as a float-float pair truncated from the double, so x < 0.5 is decided on its
// high part exactly as the reference decides it on the double.
__device__ __forceinline__ bool map_msq_ff(const PhsChildFF &C, const ChildVar &cv, double xd,
                                           const FFTables &T, ff &msq, ff &f) {
  const ff x = ff_from_double_int(xd);
  switch (C.map_id) {
    case PHS_MAP_NO:
      msq = ff_add(ld(C.msq_min), ff_mul(x, ff_sub(cv.msq_max, ld(C.msq_min))));
      f = cv.a2;
      return true;
    case PHS_MAP_SCHANNEL: {
      // z = (1-x) a0 + x a1; next to +-pi/2, tan z = -+cot(pi/2 -+ z) with pi/2 -+ z formed
      // from the host's pi/2 - a1 and pi/2 + a0, so its relative accuracy holds there.
      // Lanes of a warp fall on different sides: the argument and the quotient are
      // selected, and every lane runs one sincos and one division.
      ff z = ff_add(ld(C.a0), ff_mul(x, cv.a1));   // a1 holds a1 - a0
      if (!(fabsf(z.hi) < 1.5707962f)) return false;   // the reference's |z| < pi/2 test
      const bool hs = z.hi > 0.78539816f, ls = z.hi < -0.78539816f, cot = hs || ls;
      ff w = z;
      if (cot) w = ff_add(hs ? cv.u1 : ld(C.u0), ff_mul(hs ? ff_one_minus_double_int(xd) : x, cv.a1));
      ff sw, cw;
      ff_sincos(w, T, sw, cw);
      ff t = ff_div_fast(cot ? cw : sw, cot ? sw : cw);
      if (ls) t = ff_neg(t);
      msq = ff_add(ld(C.m2), ff_mul(ld(C.mw), t));
      f = ff_mul(cv.a2, ff_add_f(ff_sqr(t), 1.0f));
      return true;
    }
    case PHS_MAP_COLLINEAR:
    case PHS_MAP_INFRARED:
    case PHS_MAP_RADIATION:
    case PHS_MAP_TCHANNEL:
    case PHS_MAP_UCHANNEL: {
      // one exponential for all five: the t/u-channel maps take x >= 0.5 from the other
      // end, with the argument and the sum selected per lane
      const bool upper = (C.map_id == PHS_MAP_TCHANNEL || C.map_id == PHS_MAP_UCHANNEL) && !(x.hi < 0.5f);
      const ff msq1 = ff_mul(ld(C.a0), ff_exp(ff_mul(upper ? ff_one_minus_double_int(xd) : x, cv.a1), T));
      msq = upper ? ff_add(ff_sub(ld(C.a0), msq1), cv.msq_max)
                  : ff_add(ff_sub(msq1, ld(C.a0)), ld(C.msq_min));
      f = ff_mul(cv.a2, msq1);
      return true;
    }
  }
  return false;
}

// A pair as a double: two exact widenings and one add on the FP64 pipe (uniform beams,
// where the walk is bound by FP32 issue), or with integer operations (per-event beams, where
// the per-event constants keep the FP64 pipe busy).
template <bool INT>
__device__ __forceinline__ double widen(ff a) {
  return INT ? ff_to_double_int(a) : ff_to_double(a);
}

__device__ __forceinline__ ff ff_twice(ff a) { return ff_make(f_add(a.hi, a.hi), f_add(a.lo, a.lo)); }
__device__ __forceinline__ ff ff_half(ff a) { return ff_make(f_mul(a.hi, 0.5f), f_mul(a.lo, 0.5f)); }

// One event in float-float.  Returns false if it must be recomputed on the exact path
// (outputs written so far are then overwritten).  PER_EVENT: beam energies a.E1/a.E2 per
// event; the constants that depend on sqrt(s) come from FP64 per event (as the FP64 path
// computes them) and the walk stays in float-float.
template <bool PER_EVENT = false>
__device__ __forceinline__ bool phs_event_ff(const PhsLaunch &a, const PhsSegment &seg,
                                             int64_t local, const FFTables &T, float *fst) {
  if (!phs_in(seg.channel, a.n_programs, PHS_CHK_CHANNEL)) return true;
  const PhsChannelFF &ch = a.channels_ff[seg.channel];
  if (ch.exact_only) return false;
  if (!event_in_bounds(a, seg, local, ch.n_out, ch.n_visits)) return true;
  const int64_t ev = seg.ev_begin + local;
  const double *xe = a.x + seg.x_base + local * seg.x_stride;
  // the walk reads the row's x one visit at a time, each index from the program: fetch the
  // row's cache lines into L1 now, so only the first access waits for DRAM
  asm volatile("prefetch.global.L1 [%0];" ::"l"(xe));
  asm volatile("prefetch.global.L1 [%0];" ::"l"(xe + seg.x_stride - 1));
  double *out = a.p + seg.p_base + local * 4 * (int64_t)ch.n_out;
  const ff zero = ff_from_float(0.0f), one = ff_from_float(1.0f);

  // beams: the channel's, or this event's (phs_event_f64's expressions)
  ff sqrts_f = ld(ch.sqrts), s_f = ld(ch.s), lab_bg = ld(ch.lab_bg), lab_ga = ld(ch.lab_gamma);
  bool lab = ch.lab != 0;
  double sqrts64 = 0.0, s64 = 0.0;
  ff inv_s_f = zero;
  if (PER_EVENT) {
    // the beams in float-float; sqrt(s) in FP64 as well for the volume, the collinear
    // cos(theta) constants and the maps whose constants stay FP64
    const double E1 = a.E1[ev], E2 = a.E2[ev];
    sqrts64 = dmul(2.0, sqrt(dmul(E1, E2)));
    s64 = dmul(sqrts64, sqrts64);
    const ff e1 = ff_from_double_int(E1), e2 = ff_from_double_int(E2);
    const ff r = ff_sqrt_fast(ff_mul(e1, e2));
    sqrts_f = ff_twice(r);
    s_f = ff_sqr(sqrts_f);
    inv_s_f = ff_recip_fast(s_f);
    lab = E1 != E2;
    lab_bg = ff_div_fast(ff_sub(e1, e2), sqrts_f);
    lab_ga = ff_sqrt_fast(ff_add_f(ff_sqr(lab_bg), 1.0f));
  }
  const float s_scale = s_f.hi;

  // the frame of the visited branch, updated in place row by row
  ff L[16];
#pragma unroll
  for (int i = 0; i < 16; i++) L[i] = zero;
  L[0] = lab ? lab_ga : one;
  L[5] = one;
  L[10] = one;
  L[15] = L[0];
  L[3] = lab ? lab_bg : zero;
  L[12] = L[3];
  ff msq_b = s_f, m_b = sqrts_f, p_b = zero, mmax_b = sqrts_f;
  ff factor = one;
  bool ok = true;
  int sp = 0;

  const int n_visits = ch.n_visits;
  for (int v = 0; v < n_visits; v++) {
    const PhsVisitFF &V = ch.visit[v];
    ff cmsq[2], cm[2], cmax[2];
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const PhsChildFF &C = V.child[j];
      if (!C.internal) {
        cmsq[j] = ld(C.msq_leaf);
        cm[j] = ld(C.m_leaf);
        cmax[j] = zero;
      } else {
        ff f;
        const ChildVar cv = PER_EVENT
            ? child_var(C, a.channels[seg.channel].visit[v].child[j], sqrts_f, inv_s_f, ld(ch.m_tot),
                        sqrts64, a.channels[seg.channel].m_tot)
            : child_var(C);
        if (!map_msq_ff(C, cv, xrow_at(xe, C.x_msq, seg.x_stride), T, cmsq[j], f)) return false;
        factor = ff_mul(factor, f);
        if (msq_near_zero(cmsq[j], s_scale)) return false;
        if (cmsq[j].hi < 0.0f) {  // the reference takes sqrt of a negative: not ok
          ok = false;
          cmsq[j] = zero;
        }
        cm[j] = ff_sqrt_fast(cmsq[j]);
        cmax[j] = cv.m_max;
      }
    }
    // kinematic test at the visited branch, decided here only away from its limits
    const ff msum = ff_add(cm[0], cm[1]);
    const ff dlo = ff_sub(m_b, msum);
    if (near_zero(dlo, m_b.hi)) return false;
    ok = ok && dlo.hi > 0.0f;
    if (!V.self_root) {
      const ff dhi = ff_sub(mmax_b, m_b);
      if (near_zero(dhi, mmax_b.hi)) return false;
      ok = ok && dhi.hi > 0.0f;
    }
    // Kallen function, factored; one reciprocal of m serves p_decay, the factor and bg
    const ff mdiff = ff_sub(cm[0], cm[1]);
    ff lda = ff_mul(ff_mul(dlo, ff_add(m_b, msum)),
                    ff_mul(ff_sub(m_b, mdiff), ff_add(m_b, mdiff)));
    if (!(lda.hi > 0.0f)) lda = zero;
    const ff sl = ff_sqrt_fast(lda);
    const ff rm = m_b.hi > 0.0f ? ff_recip_fast(m_b) : zero;
    const ff slrm = ff_mul(sl, rm);
    const ff pc = ff_half(slrm);                       // sqrt(lambda) / (2 m)
    factor = ff_mul(factor, ff_mul(slrm, rm));         // sqrt(lambda) / m^2

    // rotation + boost of the visited branch
    const ff bg = ff_mul(p_b, rm);
    const ff ga = ff_sqrt_fast(ff_add_f(ff_sqr(bg), 1.0f));
    ff sphi, cphi;
    ff_sincos2pi(ff_from_double_int(xrow_at(xe, V.x_phi, seg.x_stride)), T, sphi, cphi);
    const double xctd = xrow_at(xe, V.x_ct, seg.x_stride);
    const ff xct = ff_from_double_int(xctd);
    ff ct, st, fct;
    if (V.ct_class == PHS_CT_COLLINEAR) {
      ff b0 = ld(V.b0), b1 = ld(V.b1);
      if (PER_EVENT) {
        const double m = a.channels[seg.channel].visit[v].m;
        const double b0d = dmul(m, m) / s64;
        b0 = ff_from_double_int(b0d);
        b1 = ff_from_double_int(log(dadd(b0d, 1.0) / b0d));
      }
      const bool lower = xct.hi < 0.5f;
      const ff tmp = ff_mul(b0, ff_exp(ff_mul(ff_twice(lower ? xct : ff_one_minus_double_int(xctd)), b1), T));
      ct = lower ? ff_add_f(ff_sub(tmp, b0), -1.0f) : ff_add_f(ff_sub(b0, tmp), 1.0f);
      if (ct.hi >= -1.0f && ct.hi <= 1.0f) {
        // 1 - ct^2 = (1 - ct)(1 + ct), each factor without cancellation
        st = ff_sqrt_fast(ff_mul(ff_sub(one, ct), ff_add_f(ct, 1.0f)));
        fct = ff_mul(tmp, b1);
      } else {
        ct = one;
        st = zero;
        fct = zero;
      }
    } else {
      // tmp = 2(1 - x), ct = 1 - tmp, st = sqrt(tmp (2 - tmp)) = 2 sqrt((1-x) x)
      const ff u = ff_one_minus_double_int(xctd);
      ct = ff_sub(xct, u);
      st = ff_twice(ff_sqrt_fast(ff_mul(u, xct)));
      fct = one;
    }
    if (V.ct_class == PHS_CT_COLLINEAR) factor = ff_mul(factor, fct);   // uniform: 1
    const ff e03 = ff_mul(bg, ct), e12 = ff_neg(sphi), e13 = ff_mul(st, cphi), e22 = cphi;
    const ff e23 = ff_mul(st, sphi), e33 = ff_mul(ga, ct);
    // the entries of L1 that only the frame's columns 1 and 2 read: formed in the branches
    // that write those (a leaf-only visit writes columns 0 and 3 only)
    const auto col12 = [&](ff &e01, ff &e11, ff &e21, ff &e31) {
      e01 = ff_neg(ff_mul(bg, st));
      e11 = ff_mul(ct, cphi);
      e21 = ff_mul(ct, sphi);
      e31 = ff_neg(ff_mul(ga, st));
    };

    if (V.self_root && !lab) {
      ff e01, e11, e21, e31;
      col12(e01, e11, e21, e31);
      L[0] = ga;   L[1] = e01;  L[2] = zero;  L[3] = e03;
      L[4] = zero; L[5] = e11;  L[6] = e12;   L[7] = e13;
      L[8] = zero; L[9] = e21;  L[10] = e22;  L[11] = e23;
      L[12] = bg;  L[13] = e31; L[14] = zero; L[15] = e33;
    } else if (PER_EVENT && V.self_root) {
      // (per-event beams, where nearly every event has a lab boost; the uniform-beam kernels
      // keep the general product, which leaves their registers to the common case)
      // the parent frame is the lab boost B_z(lab_bg): rows 1 and 2 are unit rows
      ff e01, e11, e21, e31;
      col12(e01, e11, e21, e31);
      const ff g0 = L[0], b0 = L[3];
      L[0] = ff_dot2(g0, ga, b0, bg);   L[1] = ff_dot2(g0, e01, b0, e31);
      L[2] = zero;                      L[3] = ff_dot2(g0, e03, b0, e33);
      L[4] = zero; L[5] = e11;  L[6] = e12;   L[7] = e13;
      L[8] = zero; L[9] = e21;  L[10] = e22;  L[11] = e23;
      L[12] = ff_dot2(b0, ga, g0, bg);  L[13] = ff_dot2(b0, e01, g0, e31);
      L[14] = zero;                     L[15] = ff_dot2(b0, e03, g0, e33);
    } else if (V.parent_root && !lab) {
      // the parent frame is the root's rotation (its bg is 0 and its gamma 1): row 0 is
      // (1, 0, 0, 0) and L[4], L[8], L[12], L[14] are 0, so half the products drop out
      ff e01 = zero, e11 = zero, e21 = zero, e31 = zero;
      if (!V.both_leaves) col12(e01, e11, e21, e31);
      L[0] = ga;   L[1] = e01;  L[2] = zero;  L[3] = e03;
#pragma unroll
      for (int r = 1; r < 4; r++) {
        const ff l1 = L[4 * r + 1], l2 = L[4 * r + 2], l3 = L[4 * r + 3];
        L[4 * r + 0] = ff_mul(l3, bg);
        L[4 * r + 3] = r < 3 ? ff_dot3(l1, e13, l2, e23, l3, e33) : ff_dot2(l1, e13, l3, e33);
        if (!V.both_leaves) {
          L[4 * r + 1] = r < 3 ? ff_dot3(l1, e11, l2, e21, l3, e31) : ff_dot2(l1, e11, l3, e31);
          L[4 * r + 2] = r < 3 ? ff_dot2(l1, e12, l2, e22) : ff_mul(l1, e12);
        }
      }
    } else if (PER_EVENT && V.parent_root) {
      // the root's frame with the lab boost: entries (0,2), (1,0), (2,0), (3,2) are 0
      ff e01 = zero, e11 = zero, e21 = zero, e31 = zero;
      if (!V.both_leaves) col12(e01, e11, e21, e31);
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const ff l0 = L[4 * r], l1 = L[4 * r + 1], l2 = L[4 * r + 2], l3 = L[4 * r + 3];
        const bool edge = r == 0 || r == 3;   // l2 = 0; otherwise l0 = 0
        L[4 * r + 0] = edge ? ff_dot2(l0, ga, l3, bg) : ff_mul(l3, bg);
        L[4 * r + 3] = edge ? ff_dot3(l0, e03, l1, e13, l3, e33) : ff_dot3(l1, e13, l2, e23, l3, e33);
        if (!V.both_leaves) {
          L[4 * r + 1] = edge ? ff_dot3(l0, e01, l1, e11, l3, e31) : ff_dot3(l1, e11, l2, e21, l3, e31);
          L[4 * r + 2] = edge ? ff_mul(l1, e12) : ff_dot2(l1, e12, l2, e22);
        }
      }
    } else if (V.both_leaves) {
      // both daughters are leaves: their momenta read the frame's columns 0 and 3 only
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const ff l0 = L[4 * r], l1 = L[4 * r + 1], l2 = L[4 * r + 2], l3 = L[4 * r + 3];
        L[4 * r + 0] = ff_dot2(l0, ga, l3, bg);
        L[4 * r + 3] = ff_dot4(l0, e03, l1, e13, l2, e23, l3, e33);
      }
    } else {
      // row r of L L1 depends on row r of L only: update in place
      ff e01, e11, e21, e31;
      col12(e01, e11, e21, e31);
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const ff l0 = L[4 * r], l1 = L[4 * r + 1], l2 = L[4 * r + 2], l3 = L[4 * r + 3];
        L[4 * r + 0] = ff_dot2(l0, ga, l3, bg);
        L[4 * r + 3] = ff_dot4(l0, e03, l1, e13, l2, e23, l3, e33);
        L[4 * r + 1] = ff_dot4(l0, e01, l1, e11, l2, e21, l3, e31);
        L[4 * r + 2] = ff_dot2(l1, e12, l2, e22);
      }
    }

    // leaf momenta L_new (E, 0, 0, +-p)
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const PhsChildFF &C = V.child[j];
      if (!C.internal && phs_in(C.out_index, ch.n_out, PHS_CHK_P)) {
        const ff pj = j == 0 ? pc : ff_neg(pc);
        const ff E = ff_sqrt_fast(ff_add(cmsq[j], ff_sqr(pj)));
        double2 *o = reinterpret_cast<double2 *>(out + 4 * C.out_index);
        // to double on the (otherwise idle) FP64 pipe: two exact widenings and one add
        o[0] = make_double2(widen<PER_EVENT>(ff_dot2(L[0], E, L[3], pj)),
                            widen<PER_EVENT>(ff_dot2(L[4], E, L[7], pj)));
        o[1] = make_double2(widen<PER_EVENT>(ff_dot2(L[8], E, L[11], pj)),
                            widen<PER_EVENT>(ff_dot2(L[12], E, L[15], pj)));
      }
    }

    if (V.push >= 0 && phs_in(sp, a.stack_depth, PHS_CHK_STACK)) {
      const bool j0 = V.push == 0;
#pragma unroll
      for (int i = 0; i < 16; i++) fstack_store(fst, sp, i, L[i]);
      fstack_store(fst, sp, 16, ffsel(j0, cmsq[0], cmsq[1]));
      fstack_store(fst, sp, 17, ffsel(j0, cm[0], cm[1]));
      fstack_store(fst, sp, 18, j0 ? pc : ff_neg(pc));
      fstack_store(fst, sp, 19, ffsel(j0, cmax[0], cmax[1]));
      sp++;
    }
    if (V.carry >= 0) {
      const bool j0 = V.carry == 0;
      msq_b = ffsel(j0, cmsq[0], cmsq[1]);
      m_b = ffsel(j0, cm[0], cm[1]);
      p_b = j0 ? pc : ff_neg(pc);
      mmax_b = ffsel(j0, cmax[0], cmax[1]);
    } else if (sp > 0) {
      sp--;
#pragma unroll
      for (int i = 0; i < 16; i++) L[i] = fstack_load(fst, sp, i);
      msq_b = fstack_load(fst, sp, 16);
      m_b = fstack_load(fst, sp, 17);
      p_b = fstack_load(fst, sp, 18);
      mmax_b = fstack_load(fst, sp, 19);
    }
  }

  a.volume[ev] = PER_EVENT ? channel_volume(a.channels[seg.channel], sqrts64) : ch.volume;
  a.factor[ev * a.factor_stride + seg.factor_col] = ok ? widen<PER_EVENT>(factor) : 0.0;
  a.ok[ev] = ok ? 1 : 0;
  if (!ok) {
    double2 *o = reinterpret_cast<double2 *>(out);
    for (int i = 0; i < 2 * ch.n_out; i++) o[i] = make_double2(0.0, 0.0);
  }
  return true;
}

// Pass A of the compacting variant, in plain FP32 with error bounds.  It only ever decides
// that an event FAILS.  Each internal msq is evaluated in FP32 together with a bound on its
// absolute error, 64 FP32 epsilons times the magnitudes of the terms it is made of (the
// Breit-Wigner tails through the same cot reformulation as the float-float path, whose
// tan error grows with 1 + tan^2; the exponential mappings through expm1f, whose error
// grows with the exponent): the reference's FP64 msq, and the exact one, lie inside
// [msq - e, msq + e].  Masses are then intervals, and a test fails here only if it fails
// for every value in them (with a further 1e-6 relative slack for the FP64 roundings of
// the reference's own sums and bounds), so such an event fails the reference's test too.
// Its outputs are written here.  Every other event goes to pass B, whose float-float /
// FP64 walk decides its flag exactly.  Returns false for a failed event.
#define PHS_F32_EPS_BOUND (64.0f * 5.9604645e-8f)
// c0..c5: the packed constants of PhsTestChild.
__device__ __forceinline__ float msq_f32(int map_id, float4 c, float c4, float c5, double xd,
                                         float &e) {
  const float x = (float)xd, k = PHS_F32_EPS_BOUND;
  switch (map_id) {
    case PHS_MAP_NO:
      e = k * (fabsf(c.x) + fabsf(c.y));
      return c.x + x * (c.y - c.x);
    case PHS_MAP_SCHANNEL: {
      // one tanf per lane, on z or on pi/2 -+ z (selected, not branched: lanes of a warp
      // take different sides)
      const float z = c.x + x * c.y;  // c.y holds a1 - a0
      const bool hi_side = z > 0.78539816f, lo_side = z < -0.78539816f;
      const float w = hi_side ? c.w + (float)(1.0 - xd) * c.y : (lo_side ? c.z + x * c.y : z);
      const float tw = tanf(w);
      const float t = hi_side ? 1.0f / tw : (lo_side ? -1.0f / tw : tw);
      e = k * (fabsf(c4) + fabsf(c5) * (1.0f + t * t));
      return c4 + c5 * t;
    }
    case PHS_MAP_COLLINEAR:
    case PHS_MAP_INFRARED:
    case PHS_MAP_RADIATION:
    case PHS_MAP_TCHANNEL:
    case PHS_MAP_UCHANNEL: {
      const bool upper = (map_id == PHS_MAP_TCHANNEL || map_id == PHS_MAP_UCHANNEL) && !(xd < 0.5);
      const float y = (upper ? (float)(1.0 - xd) : x) * c.y, em = expm1f(y);
      e = k * (fabsf(upper ? c.w : c.z) + fabsf(c.x) * (em + 1.0f) * (1.0f + fabsf(y)));
      return upper ? c.w - c.x * em : c.x * em + c.z;
    }
  }
  e = INFINITY;
  return 0.0f;
}

// Queues event `local` of segment si for the exact FP64 launch (each event at most once,
// so the slot stays below the segment's event count).
__device__ __forceinline__ void queue_exact(const PhsLaunch &a, int si, int64_t local) {
  if (!phs_in(si, a.n_segments, PHS_CHK_SEGMENT)) return;
  const PhsSegment *segs = a.n_segments <= PHS_INLINE_SEGS ? a.seg_inline : a.segments;
  const unsigned slot = atomicAdd(a.exact_count + si, 1u);
  if (phs_in(slot, segs[si].ev_count, PHS_CHK_QUEUE) &&
      phs_in(segs[si].tile_begin * 32 + slot, a.n_tiles * 32, PHS_CHK_QUEUE))
    a.exact_queue[segs[si].tile_begin * 32 + slot] = (int32_t)local;
}

// The reduction tables of the float-float functions, built per block in shared memory,
// exact at multiples of pi/2 (threads 0..95; the caller synchronises).
__device__ __forceinline__ void fill_ff_tables(FFTables &T) {
  if (threadIdx.x < 64) {
    const int k = threadIdx.x;
    double sv, cv;
    sincospi(k / 32.0, &sv, &cv);
    if (k % 16 == 0) {
      sv = k == 16 ? 1.0 : (k == 48 ? -1.0 : 0.0);
      cv = k == 0 ? 1.0 : (k == 32 ? -1.0 : 0.0);
    }
    const float sh = (float)sv, chh = (float)cv;
    T.trig[k] = make_float4(sh, (float)(sv - (double)sh), chh, (float)(cv - (double)chh));
  } else if (threadIdx.x < 96) {
    const int j = threadIdx.x - 64;
    const double v = exp2(j / 32.0);
    const float h = (float)v;
    T.exp2[j] = make_float2(h, (float)(v - (double)h));
  }
}

// An x value for the pre-test, which needs only the row's first few (msq) entries: the L2
// fetches 64 bytes around it rather than its default larger prefetch, so rows whose angle
// entries only the walk reads (for the events that survive) are not pulled in whole.
__device__ __forceinline__ double ld_x_narrow(const double *p) {
  double v;
  asm volatile("ld.global.L2::64B.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}

// Saved mass intervals of the pre-test: in shared memory inside the fused kernel (slots of
// the float-float frame stack, which that kernel owns anyway), in registers in the
// stand-alone test kernel (the depth is at most PHS_STACK_DEPTH).
struct SmemBounds {
  float *fst;
  __device__ __forceinline__ void push(int sp, float lo, float hi, float mx) {
    fstack_store(fst, sp, 17, ff_make(lo, hi));
    fstack_store(fst, sp, 19, ff_make(mx, 0.0f));
  }
  __device__ __forceinline__ void pop(int sp, float &lo, float &hi, float &mx) {
    const ff t = fstack_load(fst, sp, 17);
    lo = t.hi;
    hi = t.lo;
    mx = fstack_load(fst, sp, 19).hi;
  }
};
struct RegBounds {
  float lo_[PHS_STACK_DEPTH], hi_[PHS_STACK_DEPTH], mx_[PHS_STACK_DEPTH];
  __device__ __forceinline__ void push(int sp, float lo, float hi, float mx) {
#pragma unroll
    for (int i = 0; i < PHS_STACK_DEPTH; i++)
      if (i == sp) {
        lo_[i] = lo;
        hi_[i] = hi;
        mx_[i] = mx;
      }
  }
  __device__ __forceinline__ void pop(int sp, float &lo, float &hi, float &mx) {
#pragma unroll
    for (int i = 0; i < PHS_STACK_DEPTH; i++)
      if (i == sp) {
        lo = lo_[i];
        hi = hi_[i];
        mx = mx_[i];
      }
  }
};

// staged: the channel's packed visits (PhsChannelFF::test as 4 float4 per visit) staged in
// shared memory by the caller, or null: read from the channel program in global memory.
template <class Bounds>
__device__ __forceinline__ bool phs_ok_f32(const PhsLaunch &a, const PhsSegment &seg,
                                           int64_t local, Bounds &stack,
                                           const float4 *staged = nullptr) {
  if (!phs_in(seg.channel, a.n_programs, PHS_CHK_CHANNEL)) return true;
  const PhsChannelFF &ch = a.channels_ff[seg.channel];
  if (ch.exact_only) return true;
  if (!event_in_bounds(a, seg, local, ch.n_out, ch.n_visits)) return true;
  const double *xe = a.x + seg.x_base + local * seg.x_stride;
  const float up = 1.0f + 1e-6f, dn = 1.0f - 1e-6f;
  float mlo_b = ch.sqrts.hi * dn, mhi_b = ch.sqrts.hi * up, mmax_b = ch.sqrts.hi;
  bool fails = false;
  int sp = 0;
  const int n_visits = ch.n_visits;
  for (int v = 0; v < n_visits && !fails; v++) {
    // the visit in four independent 16-byte loads
    float4 A[2], B[2];
    if (staged) {
      const float4 *q = staged + 4 * v;
      A[0] = q[0]; B[0] = q[1]; A[1] = q[2]; B[1] = q[3];
    } else {
      const float4 *q = reinterpret_cast<const float4 *>(ch.test + v);
      A[0] = __ldg(q); B[0] = __ldg(q + 1); A[1] = __ldg(q + 2); B[1] = __ldg(q + 3);
    }
    const int code0 = __float_as_int(B[0].w);
    float lo[2], hi[2], cmax[2];
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const int code = __float_as_int(B[j].w);
      if (!(code & 1)) {
        lo[j] = B[j].z * dn;
        hi[j] = B[j].z * up;
        cmax[j] = 0.0f;
      } else {
        float e;
        const int xi = (code >> 8) & 255;
        const float msq = msq_f32((code >> 1) & 127, A[j], B[j].x, B[j].y,
                                  phs_in(xi, seg.x_stride, PHS_CHK_X) ? ld_x_narrow(xe + xi) : 0.0, e);
        fails = fails || msq + e < 0.0f;                // negative for certain: not ok
        lo[j] = sqrtf(fmaxf(msq - e, 0.0f)) * dn;       // NaN bounds decide nothing
        hi[j] = sqrtf(fmaxf(msq + e, 0.0f)) * up;
        cmax[j] = B[j].z;
      }
    }
    fails = fails || mhi_b < (lo[0] + lo[1]) * dn;     // below threshold for certain
    const int push = ((code0 >> 16) & 3) - 1, carry = ((code0 >> 18) & 3) - 1;
    if (!((code0 >> 20) & 1)) fails = fails || mlo_b > mmax_b * up;  // above the bound for certain
    if (push >= 0 && phs_in(sp, a.stack_depth, PHS_CHK_STACK)) {
      const bool j0 = push == 0;
      stack.push(sp, j0 ? lo[0] : lo[1], j0 ? hi[0] : hi[1], j0 ? cmax[0] : cmax[1]);
      sp++;
    }
    if (carry >= 0) {
      const bool j0 = carry == 0;
      mlo_b = j0 ? lo[0] : lo[1];
      mhi_b = j0 ? hi[0] : hi[1];
      mmax_b = j0 ? cmax[0] : cmax[1];
    } else if (sp > 0) {
      sp--;
      stack.pop(sp, mlo_b, mhi_b, mmax_b);
    }
  }
  return !fails;
}

// The outputs of an event that fails the kinematic test (as the walk writes them).
__device__ __forceinline__ void write_failed_event(const PhsLaunch &a, const PhsSegment &seg,
                                                   int64_t local) {
  if (!phs_in(seg.channel, a.n_programs, PHS_CHK_CHANNEL) ||
      !event_in_bounds(a, seg, local, seg.n_out, 1))
    return;
  const int64_t ev = seg.ev_begin + local;
  a.volume[ev] = a.channels_ff[seg.channel].volume;
  a.factor[ev * a.factor_stride + seg.factor_col] = 0.0;
  a.ok[ev] = 0;
  double2 *o = reinterpret_cast<double2 *>(a.p + seg.p_base + local * 4 * (int64_t)seg.n_out);
  for (int i = 0; i < 2 * seg.n_out; i++) o[i] = make_double2(0.0, 0.0);
}

// The same for the events of a warp tile (first event local0) whose lanes are set in
// `failed`, with the momentum rows written by the whole warp (the tile's rows are
// contiguous): 512 bytes per store instruction.  Volume, factor and ok are written for
// every event of the tile (`valid`), the survivors' with the failed values that the walk
// kernel behind this one overwrites: whole 32-byte sectors, where writes of the failing
// lanes alone would leave partial sectors for the DRAM to merge.
__device__ __forceinline__ void write_failed_tile(const PhsLaunch &a, const PhsSegment &seg,
                                                  int64_t local0, unsigned failed,
                                                  unsigned valid) {
  const int lane = threadIdx.x & 31;
  // checked build: the tile's first and last valid event and the channel
  if (!phs_in(seg.channel, a.n_programs, PHS_CHK_CHANNEL) ||
      !event_in_bounds(a, seg, local0, seg.n_out, 1) ||
      !event_in_bounds(a, seg, local0 + 31 - __clz(valid), seg.n_out, 1))
    return;
  if (valid >> lane & 1) {
    const int64_t ev = seg.ev_begin + local0 + lane;
    a.volume[ev] = a.channels_ff[seg.channel].volume;
    a.factor[ev * a.factor_stride + seg.factor_col] = 0.0;
    a.ok[ev] = 0;
  }
  const int row = 2 * seg.n_out;  // double2 per event
  const float inv_row = 1.0f / (float)row;
  double2 *o = reinterpret_cast<double2 *>(a.p + seg.p_base + local0 * 4 * (int64_t)seg.n_out);
  for (int i = lane; i < 32 * row; i += 32) {
    // event of entry i: the quotient is at least 0.5 / row from an integer, far above the
    // rounding of the product (i < 32 * 2 * PHS_MAX_OUT)
    const int e = __float2int_rz(((float)i + 0.5f) * inv_row);
    if (failed >> e & 1) o[i] = make_double2(0.0, 0.0);
  }
}

// MIN_BLOCKS: resident blocks per SM the register allocation targets; COMPACT: the
// two-pass form of phs_kernels.cu (pass A, here in FP32, settles the events that clearly
// fail; pass B computes the rest densely).  The autotuner in phs_api.cpp picks the faster instantiation per process.
template <int MIN_BLOCKS, bool COMPACT, bool PER_EVENT = false>
__global__ void __launch_bounds__(PHS_FWD_BLOCK, MIN_BLOCKS)
    phs_forward_ff_kernel(const __grid_constant__ PhsLaunch a) {
  static_assert(!(COMPACT && PER_EVENT), "the FP32 pre-test needs uniform beams");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FFTables &T = *reinterpret_cast<FFTables *>(smem_raw);
  // the float-float frame stack and the FP64 one share memory (fstack_store): a thread
  // uses one at a time, and no slot of one thread overlaps another thread's
  float *fst = reinterpret_cast<float *>(smem_raw + sizeof(FFTables));
  // events the float-float walk cannot decide go to the exact FP64 launch behind this one
  auto to_exact = [&](int si, int64_t loc) { queue_exact(a, si, loc); };

  fill_ff_tables(T);
  __syncthreads();

  const int lane = threadIdx.x & 31;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  if constexpr (COMPACT) {
    int64_t *q = reinterpret_cast<int64_t *>(smem_raw + sizeof(FFTables) +
                                             (size_t)a.stack_depth * (PHS_FF_STATE / 2) * PHS_FWD_BLOCK * sizeof(float2)) +
                 (threadIdx.x >> 5) * 64;
    compacting_loop<1>(
        a, q,
        [&](const PhsSegment &sg, int64_t loc) {
          SmemBounds st{fst};
          if (phs_ok_f32(a, sg, loc, st)) return true;
          write_failed_event(a, sg, loc);
          return false;
        },
        [&](int si, const PhsSegment &sg, int64_t loc) {
          if (!phs_event_ff(a, sg, loc, T, fst)) to_exact(si, loc);
        });
  } else {
    for (int64_t tile = warp0; tile < a.n_tiles; tile += n_warps) {
      const PhsSegment *segs = a.n_segments <= PHS_INLINE_SEGS ? a.seg_inline : a.segments;
      int lo = 0, hi = a.n_segments - 1;
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (segs[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
      }
      const PhsSegment seg = segs[lo];
      const int64_t local = (tile - seg.tile_begin) * 32 + lane;
      if (local >= seg.ev_count) continue;
      if (!phs_event_ff<PER_EVENT>(a, seg, local, T, fst)) to_exact(lo, local);
    }
  }
}

// Split form, kernel 1 of 3: the FP32 pre-test alone, at the occupancy its few registers
// allow (the fused kernel runs it at the float-float walk's).  A warp takes a chunk of
// PHS_CHUNK_TILES tiles of one segment; events that fail for certain get their outputs
// here, the others are gathered in shared memory and appended to their segment's queue
// (local event indices from tile_begin * 32 on, in any order) with one atomic per chunk.
__global__ void __launch_bounds__(PHS_FWD_BLOCK, PHS_FF_TEST_MIN_BLOCKS)
    phs_ff_test_kernel(const __grid_constant__ PhsLaunch a) {
  __shared__ int32_t gathered[PHS_FWD_BLOCK / 32][PHS_CHUNK_TILES * 32];
  // each warp's chunk is of one channel: its packed visits, staged once per channel change
  __shared__ float4 visits[PHS_FWD_BLOCK / 32][4 * PHS_MAX_VISITS];
  const int lane = threadIdx.x & 31;
  int32_t *buf = gathered[threadIdx.x >> 5];
  float4 *prog = visits[threadIdx.x >> 5];
  int staged_channel = -1;  // warp-uniform
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const PhsSegment *segs = a.n_segments <= PHS_INLINE_SEGS ? a.seg_inline : a.segments;
  for (int64_t chunk = warp0; chunk < a.n_chunks; chunk += n_warps) {
    int lo = 0, hi = a.n_segments - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (segs[mid].chunk_begin <= chunk) lo = mid; else hi = mid - 1;
    }
    const PhsSegment &seg = segs[lo];
    const int64_t t0 = (chunk - seg.chunk_begin) * PHS_CHUNK_TILES;
    const int64_t seg_tiles = (seg.ev_count + 31) / 32;
    const int n_t = (int)(seg_tiles - t0 < PHS_CHUNK_TILES ? seg_tiles - t0 : PHS_CHUNK_TILES);
    if (seg.channel != staged_channel && phs_in(seg.channel, a.n_programs, PHS_CHK_CHANNEL)) {
      const PhsChannelFF &ch = a.channels_ff[seg.channel];
      const int nv = ch.n_visits < PHS_MAX_VISITS ? ch.n_visits : PHS_MAX_VISITS;
      const float4 *src = reinterpret_cast<const float4 *>(ch.test);
      __syncwarp();
      for (int i = lane; i < 4 * nv; i += 32) prog[i] = __ldg(src + i);
      __syncwarp();
      staged_channel = seg.channel;
    }
    int n_pass = 0;
    for (int t = 0; t < n_t; t++) {
      const int64_t local0 = (t0 + t) * 32, local = local0 + lane;
      const bool valid = local < seg.ev_count;
      RegBounds st;
      const bool pass = valid && phs_ok_f32(a, seg, local, st, prog);
      const unsigned m = __ballot_sync(0xffffffffu, pass);
      const unsigned failed = __ballot_sync(0xffffffffu, valid && !pass);
      const unsigned in_seg = __ballot_sync(0xffffffffu, valid);
      const int slot = n_pass + __popc(m & ((1u << lane) - 1u));
      if (pass && phs_in(slot, PHS_CHUNK_TILES * 32, PHS_CHK_QUEUE)) buf[slot] = (int32_t)local;
      n_pass += __popc(m);
      if (failed) write_failed_tile(a, seg, local0, failed, in_seg);
    }
    __syncwarp();
    if (n_pass > 0) {
      unsigned base = 0;
      if (lane == 0) base = atomicAdd(a.pass_count + lo, (unsigned)n_pass);
      base = __shfl_sync(0xffffffffu, base, 0);
      // base + n_pass <= ev_count: at most ev_count events of the segment pass
      int32_t *dst = a.pass_queue + seg.tile_begin * 32 + base;
      if (phs_in(base + n_pass - 1, seg.ev_count, PHS_CHK_QUEUE) &&
          phs_in(seg.tile_begin * 32 + base + n_pass - 1, a.n_tiles * 32, PHS_CHK_QUEUE) &&
          phs_in(n_pass - 1, PHS_CHUNK_TILES * 32, PHS_CHK_QUEUE))
        for (int i = lane; i < n_pass; i += 32) dst[i] = buf[i];
    }
    __syncwarp();
  }
}

// Kernel 2 of 3 (one block): tile[s] = sum over the segments before s of
// ceil(count / 32), the dense numbering of the next kernel's warp claims; tile[n] is their
// total.  Also serves the exact path's queues.
__global__ void __launch_bounds__(1024)
    phs_count_scan_kernel(const unsigned int *count, int64_t *tile, int n) {
  __shared__ int64_t warp_sum[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int64_t carry = 0;
  for (int base = 0; base < n; base += blockDim.x) {
    const int s = base + threadIdx.x;
    const int64_t v = s < n ? ((int64_t)count[s] + 31) / 32 : 0;
    int64_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) warp_sum[wid] = inc;
    __syncthreads();
    int64_t before = 0, total = 0;
    for (int w = 0; w < nw; w++) {
      if (w < wid) before += warp_sum[w];
      total += warp_sum[w];
    }
    if (s < n) tile[s] = carry + before + inc - v;
    carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) tile[n] = carry;
}

// Kernel 3 of 3: the float-float walk over the queued events, 32 of one segment per warp
// claim (a.work counts the claims, zeroed before the launch), so every warp runs one
// channel's program with all lanes busy except at a segment's last claim.
template <int MIN_BLOCKS>
__global__ void __launch_bounds__(PHS_FWD_BLOCK, MIN_BLOCKS)
    phs_ff_walk_kernel(const __grid_constant__ PhsLaunch a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FFTables &T = *reinterpret_cast<FFTables *>(smem_raw);
  float *fst = reinterpret_cast<float *>(smem_raw + sizeof(FFTables));
  fill_ff_tables(T);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const PhsSegment *segs = a.n_segments <= PHS_INLINE_SEGS ? a.seg_inline : a.segments;
  const int64_t n_claims = a.pass_tile[a.n_segments];
  for (;;) {
    unsigned long long c = 0;
    if (lane == 0) c = atomicAdd(a.work, 1ull);
    const int64_t t = (int64_t)__shfl_sync(0xffffffffu, c, 0);
    if (t >= n_claims) break;
    // the last segment whose first claim is <= t (empty segments share the next one's)
    int lo = 0, hi = a.n_segments - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (a.pass_tile[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const PhsSegment &seg = segs[lo];
    const int64_t idx = (t - a.pass_tile[lo]) * 32 + lane;
    if (idx >= (int64_t)a.pass_count[lo]) continue;
    if (!phs_in(idx, seg.ev_count, PHS_CHK_QUEUE) ||
        !phs_in(seg.tile_begin * 32 + idx, a.n_tiles * 32, PHS_CHK_QUEUE))
      continue;
    const int64_t local = a.pass_queue[seg.tile_begin * 32 + idx];
    if (!phs_event_ff(a, seg, local, T, fst)) {
      queue_exact(a, lo, local);
    }
  }
}

}  // namespace

size_t phs_forward_ff_smem_bytes(int stack_depth) {
  return sizeof(FFTables) + (size_t)stack_depth * (PHS_FF_STATE / 2) * PHS_FWD_BLOCK * sizeof(float2) +
         (size_t)(PHS_FWD_BLOCK / 32) * 64 * sizeof(int64_t);
}

cudaError_t phs_launch_pretest(const PhsLaunch &a, cudaStream_t stream) {
  if (a.n_tiles <= 0) return cudaSuccess;
  int dev = 0, sms = 1, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, phs_ff_test_kernel, PHS_FWD_BLOCK, 0);
  const int64_t want = (a.n_chunks + PHS_FWD_BLOCK / 32 - 1) / (PHS_FWD_BLOCK / 32);
  const int64_t cap = (int64_t)(sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
  phs_ff_test_kernel<<<(int)(want < cap ? want : cap), PHS_FWD_BLOCK, 0, stream>>>(a);
  phs_count_scan_kernel<<<1, 1024, 0, stream>>>(a.pass_count, a.pass_tile, a.n_segments);
  return cudaGetLastError();
}

cudaError_t phs_launch_count_scan(const unsigned int *count, int64_t *tile, int n,
                                  cudaStream_t stream) {
  phs_count_scan_kernel<<<1, 1024, 0, stream>>>(count, tile, n);
  return cudaGetLastError();
}

// variant bit 0: register budget for 4 (1) or 3 (0) resident blocks; bit 1: compacting
// (fused pre-test); variants 4 and 5: the split form (pre-test kernel, scan, walk kernel).
static size_t ff_walk_smem_bytes(int stack_depth) {
  return sizeof(FFTables) + (size_t)stack_depth * (PHS_FF_STATE / 2) * PHS_FWD_BLOCK * sizeof(float2);
}

static const void *ff_kernel(int variant) {
  switch (variant) {
    case 1: return (const void *)phs_forward_ff_kernel<4, false>;
    case 2: return (const void *)phs_forward_ff_kernel<3, true>;
    case 3: return (const void *)phs_forward_ff_kernel<4, true>;
    case 4: return (const void *)phs_ff_walk_kernel<3>;
    case 5: return (const void *)phs_ff_walk_kernel<4>;
    default: return (const void *)phs_forward_ff_kernel<3, false>;
  }
}

int phs_forward_ff_blocks_per_sm(int stack_depth, int variant) {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &n, ff_kernel(variant), PHS_FWD_BLOCK,
      variant >= 4 ? ff_walk_smem_bytes(stack_depth) : phs_forward_ff_smem_bytes(stack_depth));
  return n > 0 ? n : 1;
}

cudaError_t phs_launch_forward_ff(const PhsLaunch &a, int n_blocks, int variant, cudaStream_t stream) {
  if (a.n_tiles <= 0) return cudaSuccess;
  if (a.E1 || a.E2) {
    // per-event beams: the one-pass walk (the pre-test needs uniform constants); bit 0 of
    // the variant picks the register budget
    if (!a.E1 || !a.E2) return cudaErrorInvalidValue;
    const size_t smem = phs_forward_ff_smem_bytes(a.stack_depth);
    if (variant & 1)
      phs_forward_ff_kernel<4, false, true><<<n_blocks, PHS_FWD_BLOCK, smem, stream>>>(a);
    else
      phs_forward_ff_kernel<3, false, true><<<n_blocks, PHS_FWD_BLOCK, smem, stream>>>(a);
    return cudaGetLastError();
  }
  if (variant >= 4) {
    cudaError_t e = phs_launch_pretest(a, stream);
    if (e != cudaSuccess) return e;
    const size_t smem = ff_walk_smem_bytes(a.stack_depth);
    if (variant == 5)
      phs_ff_walk_kernel<4><<<n_blocks, PHS_FWD_BLOCK, smem, stream>>>(a);
    else
      phs_ff_walk_kernel<3><<<n_blocks, PHS_FWD_BLOCK, smem, stream>>>(a);
    return cudaGetLastError();
  }
  const size_t smem = phs_forward_ff_smem_bytes(a.stack_depth);
  switch (variant) {
    case 1: phs_forward_ff_kernel<4, false><<<n_blocks, PHS_FWD_BLOCK, smem, stream>>>(a); break;
    case 2: phs_forward_ff_kernel<3, true><<<n_blocks, PHS_FWD_BLOCK, smem, stream>>>(a); break;
    case 3: phs_forward_ff_kernel<4, true><<<n_blocks, PHS_FWD_BLOCK, smem, stream>>>(a); break;
    default: phs_forward_ff_kernel<3, false><<<n_blocks, PHS_FWD_BLOCK, smem, stream>>>(a);
  }
  return cudaGetLastError();
}

PHS_CHECK_COLLECTOR(phs_check_collect_ff)
