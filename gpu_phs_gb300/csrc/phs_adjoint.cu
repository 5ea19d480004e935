// phs_adjoint.cu -- reverse-mode derivatives of the forward map (FP64).
//
// For cotangents pbar (of the momenta) and jbar (of the log-Jacobian log(factor)), one
// thread per event computes
//     xbar[k]      = sum pbar . dp/dx_k + jbar dlogJ/dx_k                 (every x)
//     thbar[b][0/1] = the same for d/dm and d/dGamma of Breit-Wigner branch b
// (b = the branch's msq x index).  Two passes per event:
//   1. the forward walk of phs_event_f64.cuh recomputed, keeping only the state each visit
//      starts from (msq, m, p, E of the visited branch) and the frame current before each
//      pop -- no per-branch matrices;
//   2. the visits in reverse.  The frame of a visit's parent is recovered from the visit's
//      own frame with the inverse rotation+boost, L_pre = L_post eta L1^T eta, so the boost
//      chain is recomputed backwards.  Adjoints of frames and states travel up the tree
//      with a stack that mirrors the forward one.
// Friend (beam-axis) visits rotate the decay frame onto an axis computed from the parent
// frame; the forward pass keeps that axis per visit, and the reverse walk rebuilds the
// rotation and differentiates it (a forward-mode evaluation with three tangents).
// Uniform beams only.  Events with ok = 0 get zero derivatives.
//
// STORED instantiations are the stored-matrix form for comparison: the forward pass writes
// every visit's parent frame (16 doubles per visit and event) to a device buffer, as the
// reference keeps its per-event boost chain in device memory (Ld, 16 N_BOOSTS doubles per
// event, phs.cu:1421-1422), and the reverse walk reads the parent frames back instead of
// recovering them with the inverse boost.  Same derivatives up to rounding; it costs the
// buffer (n_events x max_visits x 128 bytes) and its HBM traffic.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "phs_device.h"
#include "phs_event_f64.cuh"
#include "phs_program.h"

#define PHS_ADJ_BLOCK 64
#define PHS_ADJ_STATE 6    // per visit: msq, m, p, E of the visited branch, sqrt(lambda), 1/m
#define PHS_ADJ_ANG 7      // per visit: cos phi, sin phi, ct, st, dct/dx, dst/dx, dlog fct/dx
#define PHS_ADJ_DER 6      // per visited branch: dmsq/dx, dlog f/dx, dmsq/dm, dmsq/dw, dlogf/dm, dlogf/dw
#define PHS_ADJ_FRAME 20   // adjoint stack entry: Lbar[16], msqbar, mbar, pbar, Ebar

namespace {

struct AdjLayout {
  int state0, ang0, der0, pop0, stack0;  // offsets (in slots) of the per-thread regions
  int trig0;                             // the block's sin/cos table (8 slots)
  int fr0;                               // friend visits: the rotation axis, 3 per visit
  int nv, npops, depth;                  // visits, pop frames and stack depth the regions hold
};

// A value with its derivatives along three directions (forward-mode differentiation).
struct D3 {
  double v, d[3];
};
__device__ __forceinline__ D3 d3(double v, int k) {
  D3 r = {v, {0.0, 0.0, 0.0}};
  if (k >= 0) r.d[k] = 1.0;
  return r;
}
__device__ __forceinline__ D3 operator+(D3 a, D3 b) {
  return {a.v + b.v, {a.d[0] + b.d[0], a.d[1] + b.d[1], a.d[2] + b.d[2]}};
}
__device__ __forceinline__ D3 operator-(D3 a, D3 b) {
  return {a.v - b.v, {a.d[0] - b.d[0], a.d[1] - b.d[1], a.d[2] - b.d[2]}};
}
__device__ __forceinline__ D3 operator-(D3 a) { return {-a.v, {-a.d[0], -a.d[1], -a.d[2]}}; }
__device__ __forceinline__ D3 operator*(D3 a, D3 b) {
  return {a.v * b.v, {a.d[0] * b.v + a.v * b.d[0], a.d[1] * b.v + a.v * b.d[1],
                      a.d[2] * b.v + a.v * b.d[2]}};
}
__device__ __forceinline__ D3 operator/(D3 a, D3 b) {
  const double q = a.v / b.v, r = 1.0 / b.v;
  return {q, {(a.d[0] - q * b.d[0]) * r, (a.d[1] - q * b.d[1]) * r, (a.d[2] - q * b.d[2]) * r}};
}
__device__ __forceinline__ D3 d3_sqrt(D3 a) {
  const double s = sqrt(a.v), h = 0.5 / s;
  return {s, {a.d[0] * h, a.d[1] * h, a.d[2] * h}};
}

// dR[i]/d(bx, by, bz) of rot_z_onto (same formula and branch): J[3 i + k].
__device__ __forceinline__ void rot_z_onto_jacobian(double bx0, double by0, double bz0,
                                                    double J[27]) {
  D3 bx = d3(bx0, 0), by = d3(by0, 1), bz = d3(bz0, 2);
  const D3 n = d3_sqrt(bx * bx + by * by + bz * bz);
  bx = bx / n;
  by = by / n;
  bz = bz / n;
  const D3 t = bx * bx + by * by;
  D3 r00 = d3(1.0, -1), r01 = d3(0.0, -1), r11 = bz;
  if (t.v > 0.0) {
    const D3 w = (d3(1.0, -1) - bz) / t;
    r00 = bz + w * (by * by);
    r01 = -(w * (bx * by));
    r11 = bz + w * (bx * bx);
  }
  const D3 R[9] = {r00, r01, bx, r01, r11, by, -bx, -by, bz};
#pragma unroll
  for (int i = 0; i < 9; i++)
#pragma unroll
    for (int k = 0; k < 3; k++) J[3 * i + k] = R[i].d[k];
}

// Q = R_f A(theta, phi), the friend visit's spatial rotation (phs_event_f64.cuh).
__device__ __forceinline__ void friend_rotation(const double Rf[9], double ct, double st,
                                                double cphi, double sphi, double Q[9]) {
  const double A[9] = {ct * cphi, -sphi, st * cphi, ct * sphi, cphi, st * sphi, -st, 0.0, ct};
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int c = 0; c < 3; c++)
      Q[3 * r + c] = Rf[3 * r] * A[c] + Rf[3 * r + 1] * A[3 + c] + Rf[3 * r + 2] * A[6 + c];
}

__device__ __forceinline__ double &slot(double *sm, int i) {
  return sm[i * PHS_ADJ_BLOCK + threadIdx.x];
}

// msq mapping derivatives at x: dmsq/dx, dlog f/dx, and for Breit-Wigner branches the
// derivatives in the mass and the width (through the atan bounds a0, a1 as well).  aux is
// the forward map's transcendental term (map_msq): tan z, a0 exp(.), or exp(.)(1 + a1).
__device__ void map_derivs(const PhsChild &C, const PhsAdjChild &A, double x, double aux,
                           double &dmsq_dx, double &dlf_dx, double &dmsq_dm, double &dmsq_dw,
                           double &dlf_dm, double &dlf_dw) {
  dmsq_dm = dmsq_dw = dlf_dm = dlf_dw = 0.0;
  switch (C.map_id) {
    case PHS_MAP_NO:
      dmsq_dx = C.msq_max - C.msq_min;
      dlf_dx = 0.0;
      break;
    case PHS_MAP_SCHANNEL: {
      const double da = C.a1 - C.a0;
      const double t = aux, u = 1.0 + t * t, mw = C.m * C.w;
      dmsq_dx = mw * u * da;
      dlf_dx = 2.0 * t * da;
      const double dz_dm = (1.0 - x) * A.da0_dm + x * A.da1_dm;
      const double dz_dw = (1.0 - x) * A.da0_dw + x * A.da1_dw;
      dmsq_dm = 2.0 * C.m + C.w * t + mw * u * dz_dm;
      dmsq_dw = C.m * t + mw * u * dz_dw;
      dlf_dm = A.dlf_dm0 + 2.0 * t * dz_dm;
      dlf_dw = A.dlf_dw0 + 2.0 * t * dz_dw;
      break;
    }
    case PHS_MAP_COLLINEAR:
    case PHS_MAP_INFRARED:
    case PHS_MAP_RADIATION:
      dmsq_dx = C.a1 * aux;
      dlf_dx = C.a1;
      break;
    case PHS_MAP_TCHANNEL:
    case PHS_MAP_UCHANNEL:
      dmsq_dx = C.a1 * aux;
      dlf_dx = x < 0.5 ? C.a1 : -C.a1;
      break;
    case PHS_MAP_STEP_H: {
      const double q = C.a0 - x, g = C.a1 / (q * q) + C.a2;
      dmsq_dx = (C.msq_max - C.msq_min) * g;
      dlf_dx = 2.0 * C.a1 / (q * q * q) / g;
      break;
    }
    case PHS_MAP_STEP_E: {
      const double tmp = aux;
      dmsq_dx = C.a0 * tmp / (tmp - C.a1) * (C.msq_max - C.msq_min);
      dlf_dx = C.a0 * C.a1 / (C.a2 * (tmp - C.a1));
      break;
    }
    default:
      dmsq_dx = dlf_dx = 0.0;
  }
}

// cos(theta) mapping with derivatives in x.
__device__ __forceinline__ void ct_derivs(int ct_class, double x, double b0, double b1, double ct,
                                          double st, double &dct, double &dst, double &dlf) {
  if (ct_class == PHS_CT_COLLINEAR) {
    const double tmp = x < 0.5 ? b0 * exp(2.0 * x * b1) : b0 * exp(2.0 * (1.0 - x) * b1);
    if (st > 0.0) {
      dct = 2.0 * b1 * tmp;
      dst = -ct / st * dct;
      dlf = x < 0.5 ? 2.0 * b1 : -2.0 * b1;
    } else {
      dct = dst = dlf = 0.0;  // outside the mapped range: constant
    }
  } else {
    dct = 2.0;
    dst = st > 0.0 ? -2.0 * ct / st : 0.0;
    dlf = 0.0;
  }
}

// FRIENDS: the process has friend visits (a separate instantiation keeps their code out of
// the register allocation of the others).  STORED: the stored-matrix form (above); store
// holds frame slot (v * 16 + i) of event ev at store[(v * 16 + i) * store_events + ev].
template <bool FRIENDS, bool STORED>
__global__ void __launch_bounds__(PHS_ADJ_BLOCK)
    phs_adjoint_kernel(const __grid_constant__ PhsLaunch a, const PhsAdjChannel *__restrict__ adj,
                       const double *__restrict__ pbar, const double *__restrict__ jbar,
                       double *__restrict__ xbar, double *__restrict__ thbar, int th_stride,
                       AdjLayout lay, double *__restrict__ store, int64_t store_events) {
  extern __shared__ double sm[];
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double2 *trig = reinterpret_cast<double2 *>(sm + (size_t)lay.trig0 * PHS_ADJ_BLOCK);
  fill_trig_table(trig);
  __syncthreads();

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
    if (!phs_in(seg.channel, a.n_programs, PHS_CHK_CHANNEL)) continue;
    const PhsChannel &ch = a.channels[seg.channel];
    const PhsAdjChannel &ad = adj[seg.channel];
    // checked build: the rows of x, xbar (x's layout), pbar (p's) and thbar, and a program
    // that fits the shared-memory regions sized for it
    if (!event_in_bounds(a, seg, local, ch.n_out, ch.n_visits) ||
        !phs_in(ch.n_visits - 1, lay.nv, PHS_CHK_VISITS) ||
        !phs_in(ad.n_pops, lay.npops + 1, PHS_CHK_VISITS))
      continue;
    const int64_t ev = seg.ev_begin + local;
    const double *xe = a.x + seg.x_base + local * seg.x_stride;
    double *xb = xbar + seg.x_base + local * seg.x_stride;
    double *tb = thbar + ev * th_stride;
    const double *pb = pbar + seg.p_base + local * 4 * (int64_t)ch.n_out;
    const double jb = jbar ? jbar[ev] : 0.0;
    for (int k = 0; k < seg.x_stride; k++) xb[k] = 0.0;
    for (int k = 0; k < th_stride; k++) tb[k] = 0.0;

    const double sqrts = ch.sqrts, s = dmul(sqrts, sqrts);
    const bool lab = ch.lab != 0;
    const int n_visits = ch.n_visits;

    // ---------------------------------------------------------------- 1. forward walk
    double L[16];
#pragma unroll
    for (int i = 0; i < 16; i++) L[i] = 0.0;
    L[0] = lab ? ch.lab_gamma : 1.0;
    L[5] = 1.0;
    L[10] = 1.0;
    L[15] = L[0];
    L[3] = lab ? ch.lab_bg : 0.0;
    L[12] = L[3];
    double msq_b = s, m_b = sqrts, p_b = 0.0, mmax_b = sqrts, E_b = sqrts;
    bool ok = true;
    int sp = 0, np = 0;
    for (int v = 0; v < n_visits; v++) {
      const PhsVisit &V = ch.visit[v];
      if (STORED && phs_in(ev, store_events, PHS_CHK_STORE)) {
#pragma unroll
        for (int i = 0; i < 16; i++) store[(int64_t)(v * 16 + i) * store_events + ev] = L[i];
      }
      slot(sm, lay.state0 + PHS_ADJ_STATE * v + 0) = msq_b;
      slot(sm, lay.state0 + PHS_ADJ_STATE * v + 1) = m_b;
      slot(sm, lay.state0 + PHS_ADJ_STATE * v + 2) = p_b;
      slot(sm, lay.state0 + PHS_ADJ_STATE * v + 3) = E_b;
      double cmsq[2], cm[2], cmax[2];
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const PhsChild &C = V.child[j];
        if (!C.internal) {
          cmsq[j] = C.msq_leaf;
          cm[j] = C.m_leaf;
          cmax[j] = 0.0;
        } else {
          double f, aux;
          const double xm = xrow_at(xe, C.x_msq, seg.x_stride);
          map_msq(C.map_id, xm, s, C.m, C.w, C.msq_min, C.msq_max, C.a0, C.a1, C.a2, cmsq[j], f,
                  aux);
          cm[j] = sqrt(cmsq[j]);
          cmax[j] = C.m_max;
          double dd[6];
          map_derivs(C, ad.visit[v].child[j], xm, aux, dd[0], dd[1], dd[2], dd[3], dd[4], dd[5]);
          const int cv = ad.visit[v].child_visit[j];
          if (phs_in(cv, n_visits, PHS_CHK_VISITS)) {
#pragma unroll
            for (int k = 0; k < 6; k++) slot(sm, lay.der0 + PHS_ADJ_DER * cv + k) = dd[k];
          }
        }
      }
      const double d = dsub(dsub(msq_b, cmsq[0]), cmsq[1]);
      const double lda = dsub(dmul(d, d), dmul(dmul(4.0, cmsq[0]), cmsq[1]));
      ok = ok && (lda > 0.0) && (m_b > dadd(cm[0], cm[1])) && (m_b <= mmax_b);
      const double sl = sqrt(lda);
      const double rm = m_b > 0.0 ? __drcp_rn(m_b) : 0.0;
      slot(sm, lay.state0 + PHS_ADJ_STATE * v + 4) = sl;
      slot(sm, lay.state0 + PHS_ADJ_STATE * v + 5) = rm;
      const double hm = 0.5 * rm;
      const double pc = sl * hm;
      const double ce0 = (msq_b + cmsq[0] - cmsq[1]) * hm;
      const double ce1 = (msq_b + cmsq[1] - cmsq[0]) * hm;
      const double bg = p_b * rm;
      const double ga = V.self_root ? 1.0 : E_b * rm;
      double sphi, cphi, ct, st, fct;
      const double x_phi = xrow_at(xe, V.x_phi, seg.x_stride);
      const double x_ct = xrow_at(xe, V.x_ct, seg.x_stride);
      sincos2pi_tab(x_phi, trig, sphi, cphi);
      map_ct(V.ct_class, x_ct, V.b0, V.b1, ct, st, fct);
      {
        double dct, dst, dlf;
        ct_derivs(V.ct_class, x_ct, V.b0, V.b1, ct, st, dct, dst, dlf);
        const int b = lay.ang0 + PHS_ADJ_ANG * v;
        slot(sm, b + 0) = cphi;
        slot(sm, b + 1) = sphi;
        slot(sm, b + 2) = ct;
        slot(sm, b + 3) = st;
        slot(sm, b + 4) = dct;
        slot(sm, b + 5) = dst;
        slot(sm, b + 6) = dlf;
      }
      if (FRIENDS && V.friend_sign != 0) {
        // L1 = B_z(bg) diag(1, R_f A(theta, phi)), R_f onto the friend beam's direction in
        // the branch's rest frame; the axis is kept for the reverse walk
        const double ff = V.friend_sign;
        const double u0 = L[0] - ff * L[12];
        const double ax = -(L[1] - ff * L[13]), ay = -(L[2] - ff * L[14]);
        const double az = -bg * u0 - ga * (L[3] - ff * L[15]);
        const int fb = lay.fr0 + 3 * v;
        slot(sm, fb + 0) = ax;
        slot(sm, fb + 1) = ay;
        slot(sm, fb + 2) = az;
        double Rf[9], Q[9];
        rot_z_onto(ax, ay, az, Rf);
        friend_rotation(Rf, ct, st, cphi, sphi, Q);
#pragma unroll
        for (int r = 0; r < 4; r++) {
          const double l0 = L[4 * r], l1 = L[4 * r + 1], l2 = L[4 * r + 2], l3 = L[4 * r + 3];
          L[4 * r + 0] = l0 * ga + l3 * bg;
#pragma unroll
          for (int c = 0; c < 3; c++)
            L[4 * r + 1 + c] = (l0 * bg + l3 * ga) * Q[6 + c] + l1 * Q[c] + l2 * Q[3 + c];
        }
      } else if (V.both_leaves) {
        // both daughters are leaves: the frame stays the parent's.  The reverse walk forms
        // the two columns the leaves read from it and needs no inverse boost to recover it.
      } else {
        const double e01 = -bg * st, e03 = bg * ct, e11 = ct * cphi, e12 = -sphi, e13 = st * cphi;
        const double e21 = ct * sphi, e22 = cphi, e23 = st * sphi, e31 = -ga * st, e33 = ga * ct;
        if (V.self_root && !lab) {
          // the parent frame is the identity
          L[0] = ga;  L[1] = e01; L[2] = 0.0;  L[3] = e03;
          L[4] = 0.0; L[5] = e11; L[6] = e12;  L[7] = e13;
          L[8] = 0.0; L[9] = e21; L[10] = e22; L[11] = e23;
          L[12] = bg; L[13] = e31; L[14] = 0.0; L[15] = e33;
        } else if (V.parent_root && !lab) {
          // the parent frame is the root's rotation (its bg is 0 and its gamma 1): row 0 is
          // (1, 0, 0, 0) and L[4], L[8], L[12], L[14] are 0
          L[0] = ga;  L[1] = e01; L[2] = 0.0;  L[3] = e03;
#pragma unroll
          for (int r = 1; r < 4; r++) {
            const double l1 = L[4 * r + 1], l2 = r < 3 ? L[4 * r + 2] : 0.0, l3 = L[4 * r + 3];
            L[4 * r + 0] = l3 * bg;
            L[4 * r + 1] = r < 3 ? l1 * e11 + l2 * e21 + l3 * e31 : l1 * e11 + l3 * e31;
            L[4 * r + 2] = r < 3 ? l1 * e12 + l2 * e22 : l1 * e12;
            L[4 * r + 3] = r < 3 ? l1 * e13 + l2 * e23 + l3 * e33 : l1 * e13 + l3 * e33;
          }
        } else {
#pragma unroll
          for (int r = 0; r < 4; r++) {
            const double l0 = L[4 * r], l1 = L[4 * r + 1], l2 = L[4 * r + 2], l3 = L[4 * r + 3];
            L[4 * r + 0] = l0 * ga + l3 * bg;
            L[4 * r + 1] = l0 * e01 + l1 * e11 + l2 * e21 + l3 * e31;
            L[4 * r + 2] = l1 * e12 + l2 * e22;
            L[4 * r + 3] = l0 * e03 + l1 * e13 + l2 * e23 + l3 * e33;
          }
        }
      }
      if (V.push >= 0 && phs_in(sp, lay.depth, PHS_CHK_STACK)) {
        const bool j0 = V.push == 0;
        const int base = lay.stack0 + PHS_STATE * sp;
#pragma unroll
        for (int i = 0; i < 16; i++) slot(sm, base + i) = L[i];
        slot(sm, base + 16) = j0 ? cmsq[0] : cmsq[1];
        slot(sm, base + 17) = j0 ? cm[0] : cm[1];
        slot(sm, base + 18) = j0 ? pc : -pc;
        slot(sm, base + 19) = j0 ? cmax[0] : cmax[1];
        slot(sm, base + 20) = j0 ? ce0 : ce1;
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
        // the frame the reverse walk resumes with after this pop
        if (phs_in(np, lay.npops, PHS_CHK_STACK)) {
#pragma unroll
          for (int i = 0; i < 16; i++) slot(sm, lay.pop0 + 16 * np + i) = L[i];
        }
        np++;
        sp--;
        const int base = lay.stack0 + PHS_STATE * sp;
#pragma unroll
        for (int i = 0; i < 16; i++) L[i] = slot(sm, base + i);
        msq_b = slot(sm, base + 16);
        m_b = slot(sm, base + 17);
        p_b = slot(sm, base + 18);
        mmax_b = slot(sm, base + 19);
        E_b = slot(sm, base + 20);
      }
    }
    if (!ok) continue;  // zero derivatives

    // ---------------------------------------------------------------- 2. reverse walk
    // L holds the frame after the last visit; Lb the adjoint of the current visit's frame
    double Lb[16];
#pragma unroll
    for (int i = 0; i < 16; i++) Lb[i] = 0.0;
    double sb_msq = 0.0, sb_m = 0.0, sb_p = 0.0, sb_E = 0.0;  // carried child's state adjoint
    int asp = 0;
    for (int v = n_visits - 1; v >= 0; v--) {
      const PhsVisit &V = ch.visit[v];
      const PhsAdjVisit &A = ad.visit[v];
      const double msq_v = slot(sm, lay.state0 + PHS_ADJ_STATE * v + 0);
      const double m_v = slot(sm, lay.state0 + PHS_ADJ_STATE * v + 1);
      const double p_v = slot(sm, lay.state0 + PHS_ADJ_STATE * v + 2);
      const double E_v = slot(sm, lay.state0 + PHS_ADJ_STATE * v + 3);
      double cmsq[2], cm[2];
      double c_msqb[2] = {0.0, 0.0}, c_mb[2] = {0.0, 0.0}, c_pb[2] = {0.0, 0.0}, c_Eb[2] = {0.0, 0.0};
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const PhsChild &C = V.child[j];
        if (!C.internal) {
          cmsq[j] = C.msq_leaf;
          cm[j] = C.m_leaf;
        } else if (phs_in(A.child_visit[j], n_visits, PHS_CHK_VISITS)) {
          cmsq[j] = slot(sm, lay.state0 + PHS_ADJ_STATE * A.child_visit[j] + 0);
          cm[j] = slot(sm, lay.state0 + PHS_ADJ_STATE * A.child_visit[j] + 1);
        } else {
          cmsq[j] = cm[j] = 1.0;
        }
      }
      if (V.carry >= 0) {
        const int j = V.carry;
        c_msqb[j] = sb_msq; c_mb[j] = sb_m; c_pb[j] = sb_p; c_Eb[j] = sb_E;
      }
      if (V.push >= 0 && phs_in(asp - 1, lay.depth, PHS_CHK_STACK)) {
        asp--;
        const int base = lay.stack0 + PHS_ADJ_FRAME * asp;
#pragma unroll
        for (int i = 0; i < 16; i++) Lb[i] += slot(sm, base + i);
        const int j = V.push;
        c_msqb[j] = slot(sm, base + 16);
        c_mb[j] = slot(sm, base + 17);
        c_pb[j] = slot(sm, base + 18);
        c_Eb[j] = slot(sm, base + 19);
      }
      // local quantities of the visit (the square root and the reciprocal as the forward
      // pass left them)
      const double d = msq_v - cmsq[0] - cmsq[1];
      const double sl = slot(sm, lay.state0 + PHS_ADJ_STATE * v + 4);
      const double rm = slot(sm, lay.state0 + PHS_ADJ_STATE * v + 5), hm = 0.5 * rm;
      const double pc = sl * hm;
      const double A0 = msq_v + cmsq[0] - cmsq[1], A1 = msq_v + cmsq[1] - cmsq[0];
      const double ce0 = A0 * hm, ce1 = A1 * hm;
      const double bg = p_v * rm;
      const double ga = V.self_root ? 1.0 : E_v * rm;
      const int ab = lay.ang0 + PHS_ADJ_ANG * v;
      const double cphi = slot(sm, ab + 0), sphi = slot(sm, ab + 1);
      const double ct = slot(sm, ab + 2), st = slot(sm, ab + 3);
      double L1[16] = {ga,  -bg * st, 0.0,   bg * ct,
                       0.0, ct * cphi, -sphi, st * cphi,
                       0.0, ct * sphi, cphi,  st * sphi,
                       bg,  -ga * st, 0.0,   ga * ct};
      // the frame's columns 0 and 3, which the leaves read: at a leaf-only visit (not a
      // friend's) L is still the parent frame, and they are formed here
      const bool kept = V.both_leaves && !(FRIENDS && V.friend_sign != 0);
      double Lc0[4], Lc3[4];
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const double l0 = L[4 * r], l1 = L[4 * r + 1], l2 = L[4 * r + 2], l3 = L[4 * r + 3];
        Lc0[r] = kept ? l0 * ga + l3 * bg : l0;
        Lc3[r] = kept ? l0 * L1[3] + l1 * L1[7] + l2 * L1[11] + l3 * L1[15] : l3;
      }
      // leaf children: P_j = L (ce_j, 0, 0, +-pc)
      double pcb = 0.0, ceb[2] = {0.0, 0.0};
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const PhsChild &C = V.child[j];
        if (!C.internal && phs_in(C.out_index, ch.n_out, PHS_CHK_ADJ)) {
          const double sj = j == 0 ? 1.0 : -1.0;
          const double ce = j == 0 ? ce0 : ce1;
          const double *P = pb + 4 * C.out_index;
          double v0 = 0.0, v3 = 0.0;
#pragma unroll
          for (int r = 0; r < 4; r++) {
            Lb[4 * r + 0] += P[r] * ce;
            Lb[4 * r + 3] += P[r] * sj * pc;
            v0 += Lc0[r] * P[r];
            v3 += Lc3[r] * P[r];
          }
          ceb[j] += v0;
          pcb += sj * v3;
        } else if (C.internal) {
          ceb[j] += c_Eb[j];
          pcb += (j == 0 ? 1.0 : -1.0) * c_pb[j];
        }
      }
      const double eta[4] = {1.0, -1.0, -1.0, -1.0};
      double Lp[16], Lpb[16];
      double gab, bgb, ctb, stb, cpb, spb;
      if (FRIENDS && V.friend_sign != 0) {
        // friend visit: L1 = F = B_z(bg) diag(1, Q), Q = R_f(axis) A(theta, phi), axis from
        // the parent frame (kept by the forward pass).  L_pre = L eta F^T eta,
        // Lpre_bar = Lb F^T, Fbar = L_pre^T Lb, then through Q to the angles, R_f and the
        // axis, and from the axis back to the parent frame, bg and gamma.
        const double ff = V.friend_sign;
        const int fb = lay.fr0 + 3 * v;
        const double ax = slot(sm, fb + 0), ay = slot(sm, fb + 1), az = slot(sm, fb + 2);
        double Rf[9], Q[9];
        rot_z_onto(ax, ay, az, Rf);
        friend_rotation(Rf, ct, st, cphi, sphi, Q);
        const double F[16] = {ga,  bg * Q[6], bg * Q[7], bg * Q[8],
                              0.0, Q[0],      Q[1],      Q[2],
                              0.0, Q[3],      Q[4],      Q[5],
                              bg,  ga * Q[6], ga * Q[7], ga * Q[8]};
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
          for (int c = 0; c < 4; c++) {
            double acc = 0.0, accb = 0.0;
#pragma unroll
            for (int k = 0; k < 4; k++) {
              if ((c == 1 || c == 2) && k == 0) continue;  // F's zeros
              if (!STORED) acc += L[4 * r + k] * (eta[k] * eta[c]) * F[4 * c + k];
              accb += Lb[4 * r + k] * F[4 * c + k];
            }
            Lp[4 * r + c] = STORED && phs_in(ev, store_events, PHS_CHK_STORE)
                                ? store[(int64_t)(v * 16 + 4 * r + c) * store_events + ev] : acc;
            Lpb[4 * r + c] = accb;
          }
        double Fb[16];
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
          for (int c = 0; c < 4; c++) {
            double acc = 0.0;
#pragma unroll
            for (int k = 0; k < 4; k++) acc += Lp[4 * k + r] * Lb[4 * k + c];
            Fb[4 * r + c] = acc;
          }
        gab = Fb[0] + Fb[13] * Q[6] + Fb[14] * Q[7] + Fb[15] * Q[8];
        bgb = Fb[12] + Fb[1] * Q[6] + Fb[2] * Q[7] + Fb[3] * Q[8];
        double Qb[9];
#pragma unroll
        for (int c = 0; c < 3; c++) {
          Qb[c] = Fb[5 + c];
          Qb[3 + c] = Fb[9 + c];
          Qb[6 + c] = bg * Fb[1 + c] + ga * Fb[13 + c];
        }
        // Q = R_f A: Abar = R_f^T Qbar, R_f bar = Qbar A^T
        const double A[9] = {ct * cphi, -sphi, st * cphi, ct * sphi, cphi, st * sphi, -st, 0.0, ct};
        double Ab[9], Rb[9];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = 0; j < 3; j++) {
            Ab[3 * i + j] = Rf[i] * Qb[j] + Rf[3 + i] * Qb[3 + j] + Rf[6 + i] * Qb[6 + j];
            Rb[3 * i + j] = Qb[3 * i] * A[3 * j] + Qb[3 * i + 1] * A[3 * j + 1] + Qb[3 * i + 2] * A[3 * j + 2];
          }
        ctb = Ab[0] * cphi + Ab[3] * sphi + Ab[8];
        stb = Ab[2] * cphi + Ab[5] * sphi - Ab[6];
        cpb = Ab[0] * ct + Ab[2] * st + Ab[4];
        spb = -Ab[1] + Ab[3] * ct + Ab[5] * st;
        // R_f(axis): axis bar = J^T R_f bar
        double J[27];
        rot_z_onto_jacobian(ax, ay, az, J);
        double axb[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int i = 0; i < 9; i++)
#pragma unroll
          for (int k = 0; k < 3; k++) axb[k] += Rb[i] * J[3 * i + k];
        // axis = (-(Lp01 - ff Lp31), -(Lp02 - ff Lp32), -bg u0 - gamma (Lp03 - ff Lp33)),
        // u0 = Lp00 - ff Lp30
        const double u0 = Lp[0] - ff * Lp[12];
        Lpb[1] -= axb[0];
        Lpb[13] += ff * axb[0];
        Lpb[2] -= axb[1];
        Lpb[14] += ff * axb[1];
        Lpb[0] -= bg * axb[2];
        Lpb[12] += ff * bg * axb[2];
        Lpb[3] -= ga * axb[2];
        Lpb[15] += ff * ga * axb[2];
        bgb -= u0 * axb[2];
        gab -= (Lp[3] - ff * Lp[15]) * axb[2];
      } else {
        // parent frame L_pre = L eta L1^T eta; adjoints L1bar = L_pre^T Lb, Lpre_bar = Lb L1^T.
        // L1 has zeros at (0,2), (1,0), (2,0), (3,2), and only its other 12 entries carry
        // adjoints; the loops skip the zero terms (the compiler folds the constant ones).
        double L1b[16];
        if (kept) {
          // leaf-only visit: L is the parent frame itself.  The leaves read the frame's
          // columns 0 and 3 only and no daughter visit adds to its adjoint, so Lb's columns
          // 1 and 2 are 0: Lpre_bar = Lb L1^T over k = 0, 3 and L1bar = L^T Lb in columns 0, 3.
#pragma unroll
          for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
              double accb = 0.0;
#pragma unroll
              for (int k = 0; k < 4; k += 3) {
                if ((c == 1 || c == 2) && k == 0) continue;   // L1's zeros
                accb += Lb[4 * r + k] * L1[4 * c + k];
              }
              Lp[4 * r + c] = L[4 * r + c];
              Lpb[4 * r + c] = accb;
            }
#pragma unroll
          for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
              if ((r == 0 && c == 2) || (r == 1 && c == 0) || (r == 2 && c == 0) || (r == 3 && c == 2) ||
                  c == 1 || c == 2) {
                L1b[4 * r + c] = 0.0;
                continue;
              }
              double acc = 0.0;
#pragma unroll
              for (int k = 0; k < 4; k++) acc += L[4 * k + r] * Lb[4 * k + c];
              L1b[4 * r + c] = acc;
            }
        } else if (V.self_root && !lab) {
          // the root's parent frame is the identity: L1bar = Lb, and no parent adjoint
#pragma unroll
          for (int i = 0; i < 16; i++) L1b[i] = Lb[i];
        } else if (V.parent_root && !lab) {
          // the parent frame is the root's rotation (the root's bg is 0, its gamma 1): row 0
          // is (1, 0, 0, 0) and entries (1,0), (2,0), (3,0), (3,2) are 0.  Those are set, not
          // recovered; the root's reverse step reads only the adjoints of L1's 12 entries
          // that are not structurally 0, so the parent adjoint skips (0,2), (1,0), (2,0), (3,2).
#pragma unroll
          for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
              const int i = 4 * r + c;
              const bool fixed = r == 0 || c == 0 || i == 14;
              const bool unread = i == 2 || i == 4 || i == 8 || i == 14;
              double acc = 0.0, accb = 0.0;
#pragma unroll
              for (int k = 0; k < 4; k++) {
                if ((c == 0 && k == 2) || (c == 1 && k == 0) || (c == 2 && k == 0) || (c == 3 && k == 2))
                  continue;
                if (!STORED && !fixed) acc += L[4 * r + k] * (eta[k] * eta[c]) * L1[4 * c + k];
                if (!unread) accb += Lb[4 * r + k] * L1[4 * c + k];
              }
              Lp[i] = fixed ? (i == 0 ? 1.0 : 0.0)
                            : (STORED && phs_in(ev, store_events, PHS_CHK_STORE)
                                   ? store[(int64_t)(v * 16 + i) * store_events + ev] : acc);
              Lpb[i] = accb;
            }
          // L1bar = Lp^T Lb over Lp's entries that are not 0 (column 0 of Lp is (1, 0, 0, 0))
#pragma unroll
          for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
              if ((r == 0 && c == 2) || (r == 1 && c == 0) || (r == 2 && c == 0) || (r == 3 && c == 2)) {
                L1b[4 * r + c] = 0.0;
                continue;
              }
              if (r == 0) {
                L1b[c] = Lb[c];
                continue;
              }
              double acc = 0.0;
#pragma unroll
              for (int k = 1; k < 4; k++) {
                if (k == 3 && r == 2) continue;   // Lp (3,2) = 0
                acc += Lp[4 * k + r] * Lb[4 * k + c];
              }
              L1b[4 * r + c] = acc;
            }
        } else {
#pragma unroll
          for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
              double acc = 0.0, accb = 0.0;
#pragma unroll
              for (int k = 0; k < 4; k++) {
                if ((c == 0 && k == 2) || (c == 1 && k == 0) || (c == 2 && k == 0) || (c == 3 && k == 2))
                  continue;
                if (!STORED) acc += L[4 * r + k] * (eta[k] * eta[c]) * L1[4 * c + k];
                accb += Lb[4 * r + k] * L1[4 * c + k];
              }
              Lp[4 * r + c] = STORED && phs_in(ev, store_events, PHS_CHK_STORE)
                                  ? store[(int64_t)(v * 16 + 4 * r + c) * store_events + ev] : acc;
              Lpb[4 * r + c] = accb;
            }
#pragma unroll
          for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
              if ((r == 0 && c == 2) || (r == 1 && c == 0) || (r == 2 && c == 0) || (r == 3 && c == 2)) {
                L1b[4 * r + c] = 0.0;
                continue;
              }
              double acc = 0.0;
#pragma unroll
              for (int k = 0; k < 4; k++) acc += Lp[4 * k + r] * Lb[4 * k + c];
              L1b[4 * r + c] = acc;
            }
        }
        gab = L1b[0] - L1b[13] * st + L1b[15] * ct;
        bgb = -L1b[1] * st + L1b[3] * ct + L1b[12];
        ctb = L1b[3] * bg + L1b[5] * cphi + L1b[9] * sphi + L1b[15] * ga;
        stb = -L1b[1] * bg + L1b[7] * cphi + L1b[11] * sphi - L1b[13] * ga;
        cpb = L1b[5] * ct + L1b[7] * st + L1b[10];
        spb = -L1b[6] + L1b[9] * ct + L1b[11] * st;
      }
      if (phs_in(V.x_phi, seg.x_stride, PHS_CHK_ADJ)) xb[V.x_phi] = 2.0 * PHS_PI * (-sphi * cpb + cphi * spb);
      if (phs_in(V.x_ct, seg.x_stride, PHS_CHK_ADJ))
        xb[V.x_ct] = ctb * slot(sm, ab + 4) + stb * slot(sm, ab + 5) + jb * slot(sm, ab + 6);
      // bg = p rm, gamma = E rm
      double vb_p = 0.0, vb_E = 0.0, rmb = 0.0;
      if (!V.self_root) {
        vb_p = bgb * rm;
        vb_E = gab * rm;
        rmb = bgb * p_v + gab * E_v;
      }
      // p_decay, daughter energies, log-Jacobian term log(sl) - 2 log(m)
      const double slb = pcb * hm + jb / sl;
      const double hmb = pcb * sl + ceb[0] * A0 + ceb[1] * A1;
      double vb_msq = (ceb[0] + ceb[1]) * hm;
      double cmsqb[2] = {(ceb[0] - ceb[1]) * hm, (ceb[1] - ceb[0]) * hm};
      rmb += 0.5 * hmb + 2.0 * jb * m_v;
      const double vb_m = -rmb * rm * rm;
      const double ldab = slb / (2.0 * sl);
      const double db = 2.0 * d * ldab;
      vb_msq += db;
      cmsqb[0] += -4.0 * cmsq[1] * ldab - db;
      cmsqb[1] += -4.0 * cmsq[0] * ldab - db;
      // internal children: their msq is complete now; map it to x and the mapping parameters
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const PhsChild &C = V.child[j];
        if (!C.internal || !phs_in(A.child_visit[j], n_visits, PHS_CHK_VISITS) ||
            !phs_in(C.x_msq, seg.x_stride, PHS_CHK_ADJ))
          continue;
        const double msqb = cmsqb[j] + c_msqb[j] + c_mb[j] / (2.0 * cm[j]);
        const int db = lay.der0 + PHS_ADJ_DER * A.child_visit[j];
        xb[C.x_msq] = msqb * slot(sm, db + 0) + jb * slot(sm, db + 1);
        if (C.map_id == PHS_MAP_SCHANNEL && 2 * C.x_msq + 1 < th_stride) {
          tb[2 * C.x_msq] = msqb * slot(sm, db + 2) + jb * slot(sm, db + 4);
          tb[2 * C.x_msq + 1] = msqb * slot(sm, db + 3) + jb * slot(sm, db + 5);
        }
      }
      // on to the previous visit
      if (v > 0) {
        if (A.entered_by_pop && phs_in(asp, lay.depth, PHS_CHK_STACK) &&
            phs_in(A.pop_slot, lay.npops, PHS_CHK_STACK)) {
          const int base = lay.stack0 + PHS_ADJ_FRAME * asp;
#pragma unroll
          for (int i = 0; i < 16; i++) slot(sm, base + i) = Lpb[i];
          slot(sm, base + 16) = vb_msq;
          slot(sm, base + 17) = vb_m;
          slot(sm, base + 18) = vb_p;
          slot(sm, base + 19) = vb_E;
          asp++;
#pragma unroll
          for (int i = 0; i < 16; i++) {
            L[i] = slot(sm, lay.pop0 + 16 * A.pop_slot + i);
            Lb[i] = 0.0;
          }
          sb_msq = sb_m = sb_p = sb_E = 0.0;
        } else {
#pragma unroll
          for (int i = 0; i < 16; i++) {
            L[i] = Lp[i];
            Lb[i] = Lpb[i];
          }
          sb_msq = vb_msq; sb_m = vb_m; sb_p = vb_p; sb_E = vb_E;
        }
      }
    }
  }
}

}  // namespace

void phs_adjoint_sizes(int max_visits, int max_pops, int stack_depth, bool friends, int *state0,
                       int *ang0, int *der0, int *pop0, int *stack0, int *trig0, int *fr0,
                       size_t *smem) {
  *state0 = 0;
  *ang0 = PHS_ADJ_STATE * max_visits;
  *der0 = *ang0 + PHS_ADJ_ANG * max_visits;
  *pop0 = *der0 + PHS_ADJ_DER * max_visits;
  *stack0 = *pop0 + 16 * max_pops;
  *trig0 = *stack0 + PHS_STATE * (stack_depth > 0 ? stack_depth : 0);
  static_assert(PHS_TRIG_N * sizeof(double2) % (PHS_ADJ_BLOCK * sizeof(double)) == 0,
                "the sin/cos table fills whole slots");
  *fr0 = *trig0 + (int)(PHS_TRIG_N * sizeof(double2) / (PHS_ADJ_BLOCK * sizeof(double)));
  const int slots = *fr0 + (friends ? 3 * max_visits : 0);
  *smem = (size_t)slots * PHS_ADJ_BLOCK * sizeof(double);
}

template <bool FRIENDS, bool STORED>
static const void *adjoint_kernel() {
  return (const void *)phs_adjoint_kernel<FRIENDS, STORED>;
}

static const void *adjoint_kernel(bool friends, bool stored) {
  if (stored) return friends ? adjoint_kernel<true, true>() : adjoint_kernel<false, true>();
  return friends ? adjoint_kernel<true, false>() : adjoint_kernel<false, false>();
}

cudaError_t phs_launch_adjoint(const PhsLaunch &a, const PhsAdjChannel *adj, const double *pbar,
                               const double *jbar, double *xbar, double *thbar, int th_stride,
                               int max_visits, int max_pops, bool friends, int n_blocks,
                               cudaStream_t stream, double *store, int64_t store_events) {
  if (a.n_tiles <= 0) return cudaSuccess;
  AdjLayout lay;
  size_t smem;
  phs_adjoint_sizes(max_visits, max_pops, a.stack_depth, friends, &lay.state0, &lay.ang0,
                    &lay.der0, &lay.pop0, &lay.stack0, &lay.trig0, &lay.fr0, &smem);
  lay.nv = max_visits;
  lay.npops = max_pops;
  lay.depth = a.stack_depth;
  const bool stored = store != nullptr;
  const void *k = adjoint_kernel(friends, stored);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
#define PHS_ADJ_LAUNCH(F, S)                                                                   \
  phs_adjoint_kernel<F, S><<<n_blocks, PHS_ADJ_BLOCK, smem, stream>>>(a, adj, pbar, jbar, xbar, \
                                                                     thbar, th_stride, lay,     \
                                                                     store, store_events)
  if (stored) {
    if (friends) PHS_ADJ_LAUNCH(true, true); else PHS_ADJ_LAUNCH(false, true);
  } else {
    if (friends) PHS_ADJ_LAUNCH(true, false); else PHS_ADJ_LAUNCH(false, false);
  }
#undef PHS_ADJ_LAUNCH
  return cudaGetLastError();
}

int phs_adjoint_blocks_per_sm(int max_visits, int max_pops, int stack_depth, bool friends,
                              bool stored) {
  int s0, a0, d0, p0, k0, t0, f0;
  size_t smem;
  phs_adjoint_sizes(max_visits, max_pops, stack_depth, friends, &s0, &a0, &d0, &p0, &k0, &t0, &f0,
                    &smem);
  const void *k = adjoint_kernel(friends, stored);
  if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, PHS_ADJ_BLOCK, smem);
  return n > 0 ? n : 1;
}

PHS_CHECK_COLLECTOR(phs_check_collect_adjoint)
