// phs_inverse.cu -- the inverse map: momenta of generated events -> x and factor of every
// channel (the reference's do_inverse_mapping pass of gen_phs_from_x_gpu, phs.cu:1499-1554,
// with _combine_particles 1262-1283, _apply_msq_inv 626-675, the boost inversion 924-1244
// and the inverse mappings of mappings_gpu.hpp:15-219).
//
// The reference runs this as a host loop over channels, each iteration a chain of
// event-parallel kernels (combine, msq, one launch per boost level, with and without
// friends) that round-trip msq, p_decay, phi/ct/st and a 4x4 matrix per boost through HBM.
// Here one persistent kernel does all of it: a block takes PHS_INV_BLOCK consecutive events
// at a time, queues the ok ones, stages their CM-frame momenta in shared memory once, and
// every thread then walks the visit
// program (phs_program.h) of each channel in turn for its event, with the running frame in
// registers and the channel's branch momenta in its shared-memory column.  Per (event,
// channel) the only HBM traffic is the x row and the factor written.
//
// At a visit of branch b, with Gp and (theta, phi) the frame and angles of b's parent:
//   G   = [R_f^-1] B_z(-bg_b) R_y(-theta) R_z(-phi) Gp   b's rest frame, z along its flight
//                                                         (or friend) axis
//   msq of both daughters from their summed momenta; inverse msq maps of internal ones
//   Kallen function at b -> daughters' decay momentum; factor *= sqrt(lambda)/msq_b
//   q   = G p(daughter 1) -> phi = atan2(q_y, q_x), cos(theta) = q_z/|q| -> x, inverse ct map
//   (G, theta, phi) handed to the internal daughters (carry / stack)
// The friend rotation R_f is the exact rotation onto the friend beam's direction; the
// reference's differs from it only away from the root's daughters (phs.cu:1183-1244).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "phs_device.h"
#include "phs_event_f64.cuh"
#include "phs_program.h"

#define PHS_INV_STATE 23  // doubles per saved frame: G[16], ct, st, cos phi, sin phi, msq, p_decay, m
// per visit, from the geometry walk to the mapping pass: msq of both daughters, cos(theta)
// and x_phi of daughter 1, sqrt(lambda) / msq of the visited branch
#define PHS_INV_GEO 5
// per visit, the last mapping results (x, f) of daughter 0, daughter 1 and cos(theta), which
// the next channel of the shape reuses where its mapping is the same (left out when the
// block's shared memory would not hold it: the largest trees)
#define PHS_INV_CACHE 6

namespace {

// mappings_gpu.hpp:15-172 (mapping_x_from_msq_*), constants as in phs_cpu.cpp:452-531.
__device__ __forceinline__ void map_msq_inverse(int t, double msq, double s, double m, double w,
                                                double msq_min, double msq_max, double a0,
                                                double a1, double a2, double &x, double &f) {
  switch (t) {
    case PHS_MAP_NO:
      x = (msq - msq_min) / (msq_max - msq_min);
      f = (msq_max - msq_min) / s;
      break;
    case PHS_MAP_SCHANNEL: {
      const double z = (msq - m * m) / (m * w);
      x = (atan(z) - a0) / (a1 - a0);
      f = a2 * (1.0 + z * z);
      break;
    }
    case PHS_MAP_COLLINEAR:
    case PHS_MAP_INFRARED:
    case PHS_MAP_RADIATION: {
      const double z = msq - msq_min + a0;
      x = log(z / a0) / a1;
      f = a2 * z;
      break;
    }
    case PHS_MAP_TCHANNEL:
    case PHS_MAP_UCHANNEL: {
      // one logarithm per lane: the side of the midpoint selects its argument
      const bool lower = msq < (msq_max + msq_min) / 2;
      const double z = lower ? msq - msq_min + a0 : msq_max - msq + a0;
      const double lx = log(z / a0) / a1;
      x = lower ? lx : 1.0 - lx;
      f = a2 * z;
      break;
    }
    case PHS_MAP_STEP_E: {
      const double z1 = (msq - msq_min) / (msq_max - msq_min);
      const double z2 = 1.0 + a1 * exp(z1 / a2);
      x = (z1 - a2 * log(z2 / (1.0 + a1))) / a0;
      f = a0 * z2 * (msq_max - msq_min) / s;
      break;
    }
    case PHS_MAP_STEP_H: {
      const double z1 = (msq - msq_min) / (msq_max - msq_min);
      const double z3 = a0 - z1 / a2;
      x = ((a0 + z1 / a2 + z1) - sqrt(z3 * z3 + 2.0 * z1 * (a0 + z1 / a2) + z1 * z1)) / 2.0;
      f = (a1 / (a0 - x) / (a0 - x) + a2) * (msq_max - msq_min) / s;
      break;
    }
    default:
      x = 0.0;
      f = 0.0;
  }
}

// mappings_gpu.hpp:184-219 (mapping_x_from_ct_*).
__device__ __forceinline__ void map_ct_inverse(int ct_class, double ct, double b0, double b1,
                                               double &x, double &f) {
  if (ct_class == PHS_CT_COLLINEAR) {
    // one logarithm per lane, as for the msq maps
    const bool lower = ct < 0.0;
    const double ct1 = lower ? ct + b0 + 1.0 : -ct + b0 + 1.0;
    const double lx = log(ct1 / b0) / (2.0 * b1);
    x = lower ? lx : 1.0 - lx;
    f = ct1 * b1;
  } else {
    x = (ct + 1.0) / 2.0;
    f = 1.0;
  }
}

__device__ __forceinline__ void inv_store(double *stk, int depth, int k, double v) {
  stk[(depth * PHS_INV_STATE + k) * PHS_INV_BLOCK + threadIdx.x] = v;
}
__device__ __forceinline__ double inv_load(const double *stk, int depth, int k) {
  return stk[(depth * PHS_INV_STATE + k) * PHS_INV_BLOCK + threadIdx.x];
}

// Momentum slots of one thread's event: slot j < n_out is outgoing particle j, slot
// n_out + i the i-th internal branch in post-order.  Internal sums sit in shared memory at
// pm[(4 (j - n_out) + mu) PHS_INV_BLOCK].  The outgoing momenta are either staged in shared
// memory below them (pm[(4 j + mu) PHS_INV_BLOCK], the CM momenta after the inverse lab
// boost) or, where there is no lab boost (CM = lab, the same bits), read from the event's
// row of p through the L1 (lab != null): that leaves 4 n_out doubles per thread of shared
// memory free for more resident blocks.
struct InvMomenta {
  double *pm;          // internal sums (and, lab == null, the staged outgoing momenta first)
  const double *lab;   // the event's p row, or null
  int n_out;
  // checked build: slot j of the 2 n_out - 1 (the root's sum is never formed or read)
  __device__ __forceinline__ double get(int j, int mu) const {
    if (!phs_in(j, 2 * n_out - 2, PHS_CHK_SLOT)) return 0.0;
    if (lab) return j < n_out ? __ldg(lab + 4 * j + mu) : pm[(4 * (j - n_out) + mu) * PHS_INV_BLOCK];
    return pm[(4 * j + mu) * PHS_INV_BLOCK];
  }
  __device__ __forceinline__ void set_internal(int j, int mu, double v) const {
    if (!phs_in(j - n_out, n_out - 2, PHS_CHK_SLOT)) return;
    pm[(4 * (lab ? j - n_out : j) + mu) * PHS_INV_BLOCK] = v;
  }
};

// The geometry of one (event, channel shape): the walk of the visit program without the
// mappings, leaving per visit in geo (slot (v PHS_INV_GEO + k) PHS_INV_BLOCK) what the
// mappings of every channel of that shape need (inverse_maps).
// The arithmetic keeps the reference's operation order (this file is compiled without
// contraction): x(p) is ill-conditioned near the poles of each decay (cos(theta) -> +-1,
// where 1 - cos^2 cancels) and for soft daughters of fast branches, and there any other
// rounding order moves the result by far more than the input's own rounding does.  The
// exceptions are divisions by constants of an output that is not ill-conditioned in them,
// done as products with the constant's reciprocal (one rounding more): x_phi = phi / 2 pi
// and the Breit-Wigner inverse's divisions by m w and a1 - a0.
__device__ void inverse_geometry(const PhsChannel &ch, const InvMomenta &pm, double sqrts,
                                 double *stk, double *geo, int stack_depth) {
  const double s = sqrts * sqrts;
  // internal momenta as sums of their daughters in post-order (_combine_particles,
  // phs.cu:1262-1283); the root's (the last) is never a daughter
  for (int i = 0; i + 1 < ch.n_vol; i++) {
    const int a = ch.comb[i][0], b = ch.comb[i][1], o = ch.n_out + i;
#pragma unroll
    for (int mu = 0; mu < 4; mu++) pm.set_internal(o, mu, pm.get(a, mu) + pm.get(b, mu));
  }
  // carried state of the visited branch: its parent's frame Gp and angles, its msq, decay
  // momentum and mass
  double Gp[16];
  double ct0 = 1.0, st0 = 0.0, cp0 = 1.0, sp0 = 0.0;
  double msq_b = s, pd_b = 0.0, m_b = sqrts;
  int sp = 0;
  const int n_visits = ch.n_visits;
  for (int v = 0; v < n_visits; v++) {
    const PhsVisit &V = ch.visit[v];
    // the branch's frame G: CM momenta -> its rest frame, z along its flight (or friend)
    // axis.  The root's is the identity; else L_r3_r2_b3(-bg, gamma, ct0, -st0, cp0, -sp0)
    // times the parent's (phs.cu:1114-1125)
    double G[16];
    if (V.self_root) {
#pragma unroll
      for (int i = 0; i < 16; i++) G[i] = (i % 5 == 0) ? 1.0 : 0.0;
    } else {
      const double bg = m_b > 0.0 ? pd_b / m_b : 0.0;
      const double ga = sqrt(1.0 + bg * bg);
      const double t01 = -bg * st0 * cp0, t02 = -bg * st0 * sp0, t03 = -bg * ct0;
      const double t11 = ct0 * cp0, t12 = ct0 * sp0;
      const double t31 = ga * st0 * cp0, t32 = ga * st0 * sp0, t33 = ga * ct0;
      if (V.parent_root) {
        // the parent's frame is the root's, the identity: G is the step's own matrix (the
        // product below with Gp = 1 gives the same bits)
        G[0] = ga;    G[1] = t01;   G[2] = t02;  G[3] = t03;
        G[4] = 0.0;   G[5] = t11;   G[6] = t12;  G[7] = -st0;
        G[8] = 0.0;   G[9] = -sp0;  G[10] = cp0; G[11] = 0.0;
        G[12] = -bg;  G[13] = t31;  G[14] = t32; G[15] = t33;
      } else {
#pragma unroll
        for (int c = 0; c < 4; c++) {
          const double g0 = Gp[c], g1 = Gp[4 + c], g2 = Gp[8 + c], g3 = Gp[12 + c];
          // row 0 only feeds the frames of internal daughters
          if (!V.both_leaves) G[c] = ga * g0 + t01 * g1 + t02 * g2 + t03 * g3;
          G[4 + c] = t11 * g1 + t12 * g2 + (-st0) * g3;
          G[8 + c] = (-sp0) * g1 + cp0 * g2;
          G[12 + c] = (-bg) * g0 + t31 * g1 + t32 * g2 + t33 * g3;
        }
        if (V.both_leaves) G[0] = G[1] = G[2] = G[3] = 0.0;
      }
      if (V.friend_sign != 0) {
        // rotate the friend beam's direction G (1, 0, 0, ff) onto z (phs.cu:1183-1206);
        // uniform per channel
        const double ff = V.friend_sign;
        double Rf[9];
        rot_z_onto(G[4] + ff * G[7], G[8] + ff * G[11], G[12] + ff * G[15], Rf);
        double Gn[12];
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
          for (int c = 0; c < 4; c++)
            Gn[4 * r + c] = Rf[r] * G[4 + c] + Rf[3 + r] * G[8 + c] + Rf[6 + r] * G[12 + c];
#pragma unroll
        for (int i = 0; i < 12; i++) G[4 + i] = Gn[i];
      }
    }

    // daughters' momenta and invariant masses
    double q0[4], q1[4];
#pragma unroll
    for (int mu = 0; mu < 4; mu++) {
      q0[mu] = pm.get(V.slot[0], mu);
      q1[mu] = pm.get(V.slot[1], mu);
    }
    double cmsq[2];
    cmsq[0] = q0[0] * q0[0] - q0[1] * q0[1] - q0[2] * q0[2] - q0[3] * q0[3];
    cmsq[1] = q1[0] * q1[0] - q1[1] * q1[1] - q1[2] * q1[2] - q1[3] * q1[3];

    geo[(PHS_INV_GEO * v + 0) * PHS_INV_BLOCK] = cmsq[0];
    geo[(PHS_INV_GEO * v + 1) * PHS_INV_BLOCK] = cmsq[1];

    // Kallen function at the visited branch
    const double d = msq_b - cmsq[0] - cmsq[1];
    const double sl = sqrt(d * d - 4.0 * cmsq[0] * cmsq[1]);
    const double pd = sl / (2.0 * m_b);
    geo[(PHS_INV_GEO * v + 4) * PHS_INV_BLOCK] = sl / msq_b;

    // angles of daughter 1 in the branch's frame (azimuthal_angle, polar_angle_ct,
    // phs.cu:913-922)
    // (the root's frame is the identity: the same bits without the products)
    const double qx = V.self_root ? q0[1] : G[4] * q0[0] + G[5] * q0[1] + G[6] * q0[2] + G[7] * q0[3];
    const double qy = V.self_root ? q0[2] : G[8] * q0[0] + G[9] * q0[1] + G[10] * q0[2] + G[11] * q0[3];
    const double qz = V.self_root ? q0[3] : G[12] * q0[0] + G[13] * q0[1] + G[14] * q0[2] + G[15] * q0[3];
    double phi = atan2(qy, qx);
    if (phi < 0.0) phi += 2.0 * PHS_PI;
    geo[(PHS_INV_GEO * v + 3) * PHS_INV_BLOCK] = phi * (1.0 / (2.0 * PHS_PI));   // x_phi
    const double ct = qz / sqrt(qx * qx + qy * qy + qz * qz);
    geo[(PHS_INV_GEO * v + 2) * PHS_INV_BLOCK] = ct;
    if (V.both_leaves) {
      if (sp > 0) {
        sp--;
#pragma unroll
        for (int i = 0; i < 16; i++) Gp[i] = inv_load(stk, sp, i);
        ct0 = inv_load(stk, sp, 16);
        st0 = inv_load(stk, sp, 17);
        cp0 = inv_load(stk, sp, 18);
        sp0 = inv_load(stk, sp, 19);
        msq_b = inv_load(stk, sp, 20);
        pd_b = inv_load(stk, sp, 21);
        m_b = inv_load(stk, sp, 22);
      }
      continue;
    }
    const double st = sqrt(1.0 - ct * ct);
    double sph, cph;
    sincos(phi, &sph, &cph);
    if (V.push >= 0 && phs_in(sp, stack_depth, PHS_CHK_STACK)) {
      const bool j0 = V.push == 0;
#pragma unroll
      for (int i = 0; i < 16; i++) inv_store(stk, sp, i, G[i]);
      inv_store(stk, sp, 16, ct);
      inv_store(stk, sp, 17, st);
      inv_store(stk, sp, 18, cph);
      inv_store(stk, sp, 19, sph);
      const double mq = j0 ? cmsq[0] : cmsq[1];
      inv_store(stk, sp, 20, mq);
      inv_store(stk, sp, 21, j0 ? pd : -pd);
      inv_store(stk, sp, 22, sqrt(mq));
      sp++;
    }
    if (V.carry >= 0) {
      const bool j0 = V.carry == 0;
#pragma unroll
      for (int i = 0; i < 16; i++) Gp[i] = G[i];
      ct0 = ct;
      st0 = st;
      cp0 = cph;
      sp0 = sph;
      msq_b = j0 ? cmsq[0] : cmsq[1];
      pd_b = j0 ? pd : -pd;
      m_b = sqrt(msq_b);
    }
  }
}

// The mappings of one (event, channel) after inverse_geometry of its shape: writes the
// channel's x entries of xr and returns its factor, in the reference's order of factors.
// Bit 3 v + k of reuse (k = 0, 1: the daughters' msq maps, 2: the cos(theta) map): the
// previous channel of the shape had the same mapping there, so its (x, f) is taken from
// cache (null: no cache, reuse 0).  xr null: the mappings run (the next channel may reuse
// them) but write nothing.
template <bool PER_EVENT>
__device__ double inverse_maps(const PhsChannel &ch, double sqrts, const double *geo,
                               double *cache, double *xr, uint64_t reuse, int n_x) {
  const double s = sqrts * sqrts;
  double factor = 1.0;
  const int n_visits = ch.n_visits;
  for (int v = 0; v < n_visits; v++) {
    const PhsVisit &V = ch.visit[v];
    // inverse msq maps of the internal daughters
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const PhsChild &C = V.child[j];
      if (C.internal) {
        double *slot = cache ? cache + (PHS_INV_CACHE * v + 2 * j) * PHS_INV_BLOCK : nullptr;
        double x, f;
        if (reuse >> (3 * v + j) & 1) {
          x = slot[0];
          f = slot[PHS_INV_BLOCK];
        } else {
          double a0 = C.a0, a1 = C.a1, a2 = C.a2, mn = C.msq_min, mx = C.msq_max, mmax;
          if (PER_EVENT) child_constants(C, sqrts, ch.m_tot, 1.0 / s, a0, a1, a2, mn, mx, mmax);
          const double msq = geo[(PHS_INV_GEO * v + j) * PHS_INV_BLOCK];
          if (C.map_id == PHS_MAP_SCHANNEL) {
            // mapping_x_from_msq_schannel with its divisors m w and a1 - a0 (constants of the
            // channel) as compiled reciprocals
            const double z = (msq - C.msq0) * C.inv_mw;
            x = PER_EVENT ? (atan(z) - a0) / (a1 - a0) : (atan(z) - a0) * C.inv_da;
            f = a2 * (1.0 + z * z);
          } else {
            map_msq_inverse(C.map_id, msq, s, C.m, C.w, mn, mx, a0, a1, a2, x, f);
          }
          if (slot) {
            slot[0] = x;
            slot[PHS_INV_BLOCK] = f;
          }
        }
        if (xr && phs_in(C.x_msq, n_x, PHS_CHK_INV)) xr[C.x_msq] = x;
        factor *= f;
      }
    }
    factor *= geo[(PHS_INV_GEO * v + 4) * PHS_INV_BLOCK];  // sqrt(lambda) / msq
    if (xr && phs_in(V.x_phi, n_x, PHS_CHK_INV)) xr[V.x_phi] = geo[(PHS_INV_GEO * v + 3) * PHS_INV_BLOCK];
    double *slot = cache ? cache + (PHS_INV_CACHE * v + 4) * PHS_INV_BLOCK : nullptr;
    double x, f;
    if (reuse >> (3 * v + 2) & 1) {
      x = slot[0];
      f = slot[PHS_INV_BLOCK];
    } else {
      double b0 = V.b0, b1 = V.b1;
      if (PER_EVENT && V.ct_class == PHS_CT_COLLINEAR) {
        b0 = V.m * V.m / s;
        b1 = log((b0 + 1.0) / b0);
      }
      map_ct_inverse(V.ct_class, geo[(PHS_INV_GEO * v + 2) * PHS_INV_BLOCK], b0, b1, x, f);
      if (slot) {
        slot[0] = x;
        slot[PHS_INV_BLOCK] = f;
      }
    }
    if (xr && phs_in(V.x_ct, n_x, PHS_CHK_INV)) xr[V.x_ct] = x;
    factor *= f;
  }
  return factor;
}

// LAB_ROWS: no lab boost (uniform beams with E1 = E2): the outgoing momenta are read from p
// instead of staged in shared memory (InvMomenta).
template <bool PER_EVENT, bool LAB_ROWS>
__global__ void __launch_bounds__(PHS_INV_BLOCK)
    phs_inverse_kernel(const __grid_constant__ PhsInvLaunch a) {
  static_assert(!(PER_EVENT && LAB_ROWS), "per-event beams stage their CM momenta");
  extern __shared__ double sm[];
  double *pm = sm;  // [4 (n_out - 1), or 4 (2 n_out - 1) with staging][block]
  double *stk = sm + (size_t)4 * (LAB_ROWS ? a.n_out - 1 : 2 * a.n_out - 1) * PHS_INV_BLOCK;  // frame stack
  double *geo = stk + (size_t)PHS_INV_STATE * a.stack_depth * PHS_INV_BLOCK;  // per-visit geometry
  double *cache = a.group_reuse ? geo + (size_t)PHS_INV_GEO * a.max_visits * PHS_INV_BLOCK
                                : nullptr;  // per-visit mapping results
  const int tid = threadIdx.x;
  const int64_t n_tiles = (a.n_events + PHS_INV_BLOCK - 1) / PHS_INV_BLOCK;
  const PhsChannel &ch0 = a.channels[0];

  // the ok events of this block's tiles, queued: a walk takes PHS_INV_BLOCK of them at a
  // time, so every thread has an event (the rest, fewer, wait for the next tile)
  __shared__ int64_t q_ev[2 * PHS_INV_BLOCK];
  __shared__ int q_own[2 * PHS_INV_BLOCK];
  __shared__ int warp_ok[PHS_INV_BLOCK / 32];
  const int lane = tid & 31, wid = tid >> 5;
  int queued = 0;  // block-uniform

  for (int64_t tile = blockIdx.x;; tile += gridDim.x) {
    const bool more = tile < n_tiles;
    // 1. per event: the outputs that need no arithmetic (the generating channel's own x and
    // factor, x padding beyond a channel's n_x_used, zeros for ok = false events)
    const int64_t ev = tile * PHS_INV_BLOCK + tid;
    const bool valid = more && ev < a.n_events;
    int own = 0;
    bool ok = false;
    if (valid) {
      // the generating channel: the last c with ch_begin[c] <= ev
      int lo = 0, hi = a.n_channels - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a.ch_begin[mid] <= ev) lo = mid; else hi = mid - 1;
      }
      own = lo;
      ok = a.ok ? a.ok[ev] != 0 : true;
      const double *xo = a.x_own ? a.x_own + ev * a.n_x : nullptr;
      // (checked build: a row beyond x_out's events writes nothing; no early exit, the
      // block's barriers below must be reached by every thread)
      const bool rows_in = phs_in(ev, a.x_ch_stride, PHS_CHK_INV);
      for (int c = 0; c < (a.write_fixed && rows_in ? a.n_channels : 0); c++) {
        double *xr = a.x_out + ((int64_t)c * a.x_ch_stride + ev) * a.n_x;
        double *fo = a.all_factors + ev * a.n_channels + c;
        if (c == own && xo) {
          // the generating channel keeps its own x and factor (_move_x/_move_factors)
          for (int k = 0; k < a.n_x; k++) xr[k] = xo[k];
          *fo = a.factor_own ? a.factor_own[ev] : 0.0;
          continue;
        }
        const int n_used = a.channels[c].n_x_used;
        for (int k = n_used; k < a.n_x; k++) xr[k] = xo ? xo[k] : 0.0;
        if (!ok) {
          for (int k = 0; k < n_used; k++) xr[k] = 0.0;
          *fo = 0.0;
        }
      }
    }
    // 2. queue the ok events: the inversions run in full warps (an FP64 instruction costs
    // the pipe the same whatever the number of active lanes)
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    if (lane == 0) warp_ok[wid] = __popc(m);
    __syncthreads();
    int before = 0, n_ok = 0;
    for (int w = 0; w < PHS_INV_BLOCK / 32; w++) {
      if (w < wid) before += warp_ok[w];
      n_ok += warp_ok[w];
    }
    if (ok) {
      const int d = queued + before + __popc(m & ((1u << lane) - 1u));
      if (phs_in(d, 2 * PHS_INV_BLOCK, PHS_CHK_SLOT)) {
        q_ev[d] = ev;
        q_own[d] = own;
      }
    }
    queued += n_ok;
    __syncthreads();  // the queue is complete; warp_ok is read
    if (queued < PHS_INV_BLOCK && (more || queued == 0)) {
      if (!more) break;
      continue;
    }
    const int n_walk = min(queued, PHS_INV_BLOCK);
    // 3. every other channel of the tid-th queued event
    if (tid < n_walk && phs_in(q_ev[tid], a.n_events, PHS_CHK_SLOT) &&
        phs_in(q_ev[tid], a.x_ch_stride, PHS_CHK_INV)) {
      const int64_t e = q_ev[tid];
      const int own_e = q_own[tid];
      double sqrts = ch0.sqrts, lab_bg = ch0.lab ? ch0.lab_bg : 0.0;
      double lab_ga = ch0.lab ? ch0.lab_gamma : 1.0;
      if (PER_EVENT) {
        const double E1 = a.E1[e], E2 = a.E2[e], r = sqrt(E1 * E2);
        sqrts = 2.0 * r;
        lab_bg = (E1 - E2) / (2.0 * r);
        lab_ga = sqrt(1.0 + lab_bg * lab_bg);
      }
      // this event's momenta, lab -> CM (the inverse of phs.cu:1286-1301)
      const double *prow = a.p + e * 4 * (int64_t)a.n_out;
      if (!LAB_ROWS) {
        const double2 *pe = reinterpret_cast<const double2 *>(prow);
        for (int k = 0; k < a.n_out; k++) {
          const double2 e_x = pe[2 * k], y_z = pe[2 * k + 1];
          pm[(4 * k + 0) * PHS_INV_BLOCK + tid] = dsub(dmul(lab_ga, e_x.x), dmul(lab_bg, y_z.y));
          pm[(4 * k + 1) * PHS_INV_BLOCK + tid] = e_x.y;
          pm[(4 * k + 2) * PHS_INV_BLOCK + tid] = y_z.x;
          pm[(4 * k + 3) * PHS_INV_BLOCK + tid] = dadd(dmul(-lab_bg, e_x.x), dmul(lab_ga, y_z.y));
        }
      }
      const InvMomenta mom{pm + tid, LAB_ROWS ? prow : nullptr, a.n_out};
      // the geometry once per tree shape, then the mappings of each channel of that shape
      // (of this launch's slice of the group order)
      const bool has_own = a.x_own != nullptr;
      for (int g = 0; g < a.n_groups; g++) {
        const int gb = a.group_begin[g], ge = a.group_begin[g + 1];
        const int lo = max(gb, a.order_lo), hi = min(ge, a.order_hi);
        if (lo >= hi || (has_own && hi - lo == 1 && a.group_order[lo] == own_e)) continue;
        // checked build: the group's entries, its shape's program and the regions sized for it
        if (!phs_in(gb, a.n_channels, PHS_CHK_SLOT) || !phs_in(hi - 1, a.n_channels, PHS_CHK_SLOT) ||
            !phs_in(a.group_order[gb], a.n_channels, PHS_CHK_CHANNEL) ||
            !phs_in(a.channels[a.group_order[gb]].n_visits - 1, a.max_visits, PHS_CHK_VISITS) ||
            !phs_in(a.channels[a.group_order[gb]].n_out - 1, a.n_out, PHS_CHK_SLOT))
          continue;
        inverse_geometry(a.channels[a.group_order[gb]], mom, sqrts, stk, geo + tid, a.stack_depth);
        for (int i = lo; i < hi; i++) {
          const int c = a.group_order[i];
          if (!phs_in(c, a.n_channels, PHS_CHK_CHANNEL) ||
              !phs_in(a.channels[c].n_visits - 1, a.max_visits, PHS_CHK_VISITS))
            continue;
          // the generating channel keeps its own row, but its mappings still run when a
          // later channel of the shape reuses them
          const bool own_row = c == own_e && has_own;
          if (own_row && (!cache || i + 1 == hi || a.group_reuse[i + 1] == 0)) continue;
          double *xr = own_row ? nullptr : a.x_out + ((int64_t)c * a.x_ch_stride + e) * a.n_x;
          // the first channel of a shape (or of the slice) computes every mapping
          const uint64_t reuse = i == lo || !cache ? 0ull : a.group_reuse[i];
          const double fac = inverse_maps<PER_EVENT>(a.channels[c], sqrts, geo + tid,
                                                     cache ? cache + tid : nullptr, xr, reuse, a.n_x);
          if (!own_row) a.all_factors[e * a.n_channels + c] = fac;
        }
      }
    }
    __syncthreads();  // every walked entry is read
    // the events beyond the walked ones move to the front (fewer than PHS_INV_BLOCK)
    const int rest = queued - n_walk;
    int64_t e_rest = 0;
    int o_rest = 0;
    if (tid < rest && phs_in(PHS_INV_BLOCK + tid, 2 * PHS_INV_BLOCK, PHS_CHK_SLOT)) {
      e_rest = q_ev[PHS_INV_BLOCK + tid];
      o_rest = q_own[PHS_INV_BLOCK + tid];
    }
    __syncthreads();
    if (tid < rest) {
      q_ev[tid] = e_rest;
      q_own[tid] = o_rest;
    }
    queued = rest;
    __syncthreads();
    if (!more && queued == 0) break;
  }
}

}  // namespace

size_t phs_inverse_smem_bytes(int n_out, int stack_depth, int max_visits, bool cache, bool lab_rows) {
  return ((size_t)4 * (lab_rows ? n_out - 1 : 2 * n_out - 1) + (size_t)PHS_INV_STATE * stack_depth +
          (size_t)(PHS_INV_GEO + (cache ? PHS_INV_CACHE : 0)) * max_visits) *
         PHS_INV_BLOCK * sizeof(double);
}

bool phs_inverse_fits_cache(int n_out, int stack_depth, int max_visits) {
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return phs_inverse_smem_bytes(n_out, stack_depth, max_visits, true, false) <= (size_t)optin;
}

static const void *inverse_kernel(bool per_event, bool lab_rows) {
  if (per_event) return (const void *)phs_inverse_kernel<true, false>;
  return lab_rows ? (const void *)phs_inverse_kernel<false, true>
                  : (const void *)phs_inverse_kernel<false, false>;
}

int phs_inverse_blocks_per_sm(int n_out, int stack_depth, int max_visits, bool per_event,
                              bool cache, bool lab_rows) {
  int n = 0;
  lab_rows = lab_rows && !per_event;
  const size_t smem = phs_inverse_smem_bytes(n_out, stack_depth, max_visits, cache, lab_rows);
  const void *k = inverse_kernel(per_event, lab_rows);
  if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, PHS_INV_BLOCK, smem);
  return n > 0 ? n : 1;
}

cudaError_t phs_launch_inverse(const PhsInvLaunch &a, int n_blocks, cudaStream_t stream) {
  if (a.n_events <= 0) return cudaSuccess;
  const bool per_event = a.E1 && a.E2;
  const bool lab_rows = !per_event && !a.lab;
  const size_t smem = phs_inverse_smem_bytes(a.n_out, a.stack_depth, a.max_visits,
                                             a.group_reuse != nullptr, lab_rows);
  const void *k = inverse_kernel(per_event, lab_rows);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  if (per_event)
    phs_inverse_kernel<true, false><<<n_blocks, PHS_INV_BLOCK, smem, stream>>>(a);
  else if (lab_rows)
    phs_inverse_kernel<false, true><<<n_blocks, PHS_INV_BLOCK, smem, stream>>>(a);
  else
    phs_inverse_kernel<false, false><<<n_blocks, PHS_INV_BLOCK, smem, stream>>>(a);
  return cudaGetLastError();
}

PHS_CHECK_COLLECTOR(phs_check_collect_inverse)
