/*
 * phs_oracle.c -- CPU restatement of gpu_phs's forward phase-space generator.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle for the CUDA path: only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 * Nothing in the gpu_phs_gb300 package links, imports or calls it.
 *
 * It restates the reference's CPU path for one event (x -> momenta, factor,
 * volume, ok) with the same floating-point expression order, so that on
 * identical x it reproduces the reference bit for bit when both are compiled
 * with -O2 -ffp-contract=off (no FMA contraction on any host):
 *
 *   mapping_msq_from_x      phs_cpu.cpp:12-61
 *   mapping_ct_from_x       phs_cpu.cpp:112-146
 *   set_msq  (post-order)   phs_cpu.cpp:174-234
 *   set_angles (pre-order)  phs_cpu.cpp:283-345
 *   mapping constants       phs_cpu.cpp:452-531
 *   leaf masses             phs_cpu.cpp:541-547
 *   per-event driver        phs_cpu.cpp:582-600
 *   mass sums               phs.cu:61-78
 *   lab-frame boost         phs.cu:1286-1301 (the CPU path has none; used only
 *                           when the two beam energies differ)
 *   friend (beam-axis) boost  phs.cu:853-910 (GPU only; restated exactly, below)
 *   inverse mapping         phs.cu:626-675 (_apply_msq_inv), 924-1244 (boost
 *                           inversion), 1262-1283 (_combine_particles), inverse
 *                           maps mappings_gpu.hpp:15-219 (GPU only)
 *
 * Friend boosts and the inverse have no CPU implementation in the reference; they are
 * pinned against Whizard's own golden events (samples/bwbw.ref momenta and
 * all_factors).  Where the reference's GPU formulas are not the exact Lorentz
 * algebra, this file uses the exact algebra, which is what the golden events follow:
 *   - friend axis: the reference's z component carries -bg*L0[3][0]*pf where the
 *     inverse boost gives +bg*L0[3][0]*pf (phs.cu:890); equal when L0 has no boost;
 *   - rotation onto the axis: L_rot_to_2nd (phs.cu:753-781) flips the sign of the
 *     (y,z) and (z,y) elements of the Rodrigues rotation; equal when the axis has no
 *     y component;
 *   - inverse with a friend: the branch's frame is stored as L0*L_friend
 *     (phs.cu:1237-1244) where the chain needs L_friend*L0; equal when the branch
 *     has no internal daughter.
 * Whizard trees carry friends only on the root's daughters, where all three agree.
 *
 * Differences from the reference, all on events the reference leaves undefined:
 *   - ok=false events get momenta 0 and factor 0 (the reference CPU returns
 *     early and leaves partial values), and the full channel volume.
 *   - mapping ids outside the implemented set are rejected at set-up (the
 *     reference's switch falls through and leaves msq/factor unset).
 *
 * Trees use Whizard binary codes: outgoing particle j has code 2^j, a branch's
 * code is the OR of its leaves, the root is 2^n_out - 1.  Daughter tables are
 * indexed by code-1 and hold daughter codes (0 = none), as the reference's
 * .ref files and its C-ABI (whizard_gpu_phs.cpp:79-87) do.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OR_PI 3.14159265358979323846
#define OR_TWOPI 6.28318530717958647693
#define OR_TWOPI2 39.47841760435743447534
#define OR_TWOPI5 9792.62991312900650440772

enum {
  OR_MAP_NO = 0, OR_MAP_SCHANNEL = 1, OR_MAP_TCHANNEL = 2, OR_MAP_UCHANNEL = 3,
  OR_MAP_RADIATION = 4, OR_MAP_COLLINEAR = 5, OR_MAP_INFRARED = 6,
  OR_MAP_STEP_E = 11, OR_MAP_STEP_H = 12
};

typedef struct {
  int n_in, n_out, n_channels;
  int n_codes;            /* 2^n_out - 1: codes 1..n_codes */
  int stride;             /* n_codes + 1, per-channel stride of code tables */
  int *k1, *k2, *has_ch;  /* [c*stride + code] daughter codes (0 = none) */
  int *map_id;
  double *m, *w, *mass_sum;
  double *a, *b;          /* [(c*stride + code)*3 + i] */
  double *flv_masses;     /* n_in + n_out */
  int *friend_sign;       /* [c*stride + code]: 0, or the beam direction +-1 of a friend */
  double sqrts;           /* sqrts the constants were computed for */
  int nudge;              /* per-event constants moved by this many ulps (see below) */
} oracle_t;

static int map_id_known(int t) {
  return t == OR_MAP_NO || t == OR_MAP_SCHANNEL || t == OR_MAP_TCHANNEL || t == OR_MAP_UCHANNEL ||
         t == OR_MAP_RADIATION || t == OR_MAP_COLLINEAR || t == OR_MAP_INFRARED ||
         t == OR_MAP_STEP_E || t == OR_MAP_STEP_H;
}

/* phs.cu:61-78: m_min of a branch is the sum of its leaf masses. */
static double mass_sum_rec(const oracle_t *o, int c, int code) {
  int i = c * o->stride + code;
  if (o->has_ch[i]) {
    double s1 = mass_sum_rec(o, c, o->k1[i]);
    double s2 = mass_sum_rec(o, c, o->k2[i]);
    o->mass_sum[i] = s1 + s2;
  } else {
    int ld2 = 0, bb = code;
    while (bb > 1) { bb /= 2; ld2++; }
    o->mass_sum[i] = o->flv_masses[o->n_in + ld2];
  }
  return o->mass_sum[i];
}

/* x moved by k ulps (k > 0 up, k < 0 down). */
static double ulps_moved(double x, int k) {
  for (; k > 0; k--) x = nextafter(x, INFINITY);
  for (; k < 0; k++) x = nextafter(x, -INFINITY);
  return x;
}

/* phs_cpu.cpp:452-531, for one channel and one sqrts, into a/b.  nudge != 0 (a test's
 * sensitivity probe, never the reference's arithmetic) moves every constant that a
 * transcendental function returns -- the Breit-Wigner bound a1 = atan(.), the logarithms
 * of the exponential maps and of the cos(theta) map, each exp and log of the STEP_E
 * constants -- by nudge ulps where it is formed, so that the constants computed from it
 * (a2 = (a1 - a0) m w / s, STEP_E's a0 = 1 - a2 log(...)) follow (STEP_H's constants are
 * correctly rounded operations, the same bits everywhere): a device evaluating them per
 * event with its own library (or its own series) is within a few ulps of these, and far
 * in a Breit-Wigner tail one ulp of a1 moves the mapped mass by m w (1 + u^2) ulp(a1). */
static void constants_for(const oracle_t *o, int c, double sqrts, double *a_out, double *b_out,
                          int nudge) {
  double m_tot = o->mass_sum[c * o->stride + o->n_codes];
  for (int code = 1; code <= o->n_codes; code++) {
    int i = c * o->stride + code;
    int t = o->map_id[i];
    double *a = a_out + 3 * code, *b = b_out + 3 * code;
    double m = o->m[i], w = o->w[i];
    double m_min = o->mass_sum[i];
    double m_max = sqrts - m_tot + m_min;
    double msq_min = m_min * m_min, msq_max = m_max * m_max;
    double s = sqrts * sqrts;
    double msq0;
    a[0] = a[1] = a[2] = 0;
    switch (t) {
      case OR_MAP_NO:
        a[0] = 0;
        a[1] = msq_max - msq_min;
        a[2] = a[1] / s;
        break;
      case OR_MAP_SCHANNEL:
        msq0 = m * m;
        a[0] = atan((msq_min - msq0) / (m * w));
        a[1] = ulps_moved(atan((msq_max - msq0) / (m * w)), nudge);
        a[2] = (a[1] - a[0]) * (m * w) / s;
        break;
      case OR_MAP_RADIATION:
      case OR_MAP_COLLINEAR:
      case OR_MAP_INFRARED:
        msq0 = (t == OR_MAP_RADIATION) ? w * w : m * m;
        a[0] = msq0;
        a[1] = ulps_moved(log((msq_max - msq_min) / msq0 + 1), nudge);
        a[2] = a[1] / s;
        break;
      case OR_MAP_TCHANNEL:
      case OR_MAP_UCHANNEL:
        msq0 = m * m;
        a[0] = msq0;
        a[1] = ulps_moved(2 * log((msq_max - msq_min) / (2 * msq0) + 1), nudge);
        a[2] = a[1] / s;
        break;
      case OR_MAP_STEP_E: {
        double r = 2 * m * w / (msq_max - msq_min);
        a[2] = r > 0.01 ? r : 0.01;
        a[1] = ulps_moved(exp(-(m * m - msq_min) / (msq_max - msq_min) / a[2]), nudge);
        a[0] = 1 - a[2] * ulps_moved(log((1 + a[1] * ulps_moved(exp(1 / a[2]), nudge)) / (1 + a[1])),
                                     nudge);
        break;
      }
      case OR_MAP_STEP_H: {
        a[2] = (m * m - msq_min) / (msq_max - msq_min);
        double r = pow(2 * m * w / (msq_max - msq_min), 2) / a[2];
        a[1] = r > 0.000001 ? r : 0.000001;
        a[0] = (1 + sqrt(1 + 4 * a[1] / (1 - a[2]))) / 2;
        break;
      }
    }
    switch (t) {
      case OR_MAP_TCHANNEL:
      case OR_MAP_UCHANNEL:
      case OR_MAP_COLLINEAR:
        b[0] = m * m / s;
        b[1] = ulps_moved(log((b[0] + 1) / b[0]), nudge);
        b[2] = 0;
        break;
      default:
        b[0] = b[1] = b[2] = 0;
    }
  }
}

/* phs_cpu.cpp:12-61 */
static void msq_from_x(int t, double x, double s, double m, double w, double msq_min, double msq_max,
                       const double *a, double *msq, double *factor, int nudge) {
  double msq1, tmp, z;
  switch (t) {
    case OR_MAP_NO:
      *msq = (1 - x) * msq_min + x * msq_max;
      *factor = (msq_max - msq_min) / s;
      break;
    case OR_MAP_SCHANNEL:
      z = (1 - x) * a[0] + x * a[1];
      if (-OR_PI / 2 < z && z < OR_PI / 2) {
        tmp = ulps_moved(tan(z), nudge);
        *msq = m * (m + w * tmp);
        *factor = a[2] * (1 + tmp * tmp);
      } else {
        *msq = 0;
        *factor = 0;
      }
      break;
    case OR_MAP_COLLINEAR:
    case OR_MAP_INFRARED:
    case OR_MAP_RADIATION:
      msq1 = a[0] * ulps_moved(exp(x * a[1]), nudge);
      *msq = msq1 - a[0] + msq_min;
      *factor = a[2] * msq1;
      break;
    case OR_MAP_TCHANNEL:
    case OR_MAP_UCHANNEL:
      if (x < 0.5) {
        msq1 = a[0] * ulps_moved(exp(x * a[1]), nudge);
        *msq = msq1 - a[0] + msq_min;
      } else {
        msq1 = a[0] * ulps_moved(exp((1 - x) * a[1]), nudge);
        *msq = -(msq1 - a[0]) + msq_max;
      }
      *factor = a[2] * msq1;
      break;
    case OR_MAP_STEP_H:
      z = a[1] / (a[0] - x) - a[1] / a[0] + a[2] * x;
      *msq = z * msq_max + (1 - z) * msq_min;
      *factor = (a[1] / ((a[0] - x) * (a[0] - x)) + a[2]) * (msq_max - msq_min) / s;
      break;
    case OR_MAP_STEP_E:
      tmp = ulps_moved(exp(-x * a[0] / a[2]), nudge) * (1 + a[1]);
      z = -a[2] * ulps_moved(log(tmp - a[1]), nudge);
      *msq = z * msq_max + (1 - z) * msq_min;
      *factor = a[0] / (1 - a[1] / tmp) * (msq_max - msq_min) / s;
      break;
  }
}

/* phs_cpu.cpp:112-146 */
static void ct_from_x(int t, double x, const double *b, double *ct, double *st, double *factor,
                      int nudge) {
  double tmp;
  switch (t) {
    case OR_MAP_COLLINEAR:
    case OR_MAP_TCHANNEL:
    case OR_MAP_UCHANNEL:
      if (x < 0.5) {
        tmp = b[0] * ulps_moved(exp(2 * x * b[1]), nudge);
        *ct = tmp - b[0] - 1;
      } else {
        tmp = b[0] * ulps_moved(exp(2 * (1 - x) * b[1]), nudge);
        *ct = -(tmp - b[0]) + 1;
      }
      if (*ct >= -1 && *ct <= 1) {
        *st = sqrt(1 - *ct * *ct);
        *factor = tmp * b[1];
      } else {
        *ct = 1;
        *st = 0;
        *factor = 0;
      }
      break;
    default: /* NO, SCHANNEL, INFRARED, RADIATION, STEP_E, STEP_H */
      tmp = 2 * (1 - x);
      *ct = 1 - tmp;
      *st = sqrt(tmp * (2 - tmp));
      *factor = 1;
  }
}

typedef struct {
  const oracle_t *o;
  int c;
  const double *a, *b; /* this channel's constants, indexed 3*code */
  const double *x;
  size_t id_x;
  double sqrts, m_tot;
  double *p2, *p_decay; /* [code] */
  double (*p)[4];       /* [code][4] */
  int ok;
  double kappa;         /* condition of the Kallen functions (see oracle_generate_cond) */
} ev_t;

/* Rotation taking the z axis onto the direction of (bx, by, bz) about the axis z x b
 * (Rodrigues), as a 3x3 matrix, with the symmetric part cos + (1 - cos) k k^T formed from
 * the transverse components as L_rot_to_2nd (phs.cu:753-781) does (stable as the axis
 * nears -z).  An axis exactly along -z gives the rotation by pi about x. */
static void rot_z_onto(double bx, double by, double bz, double R[3][3]) {
  double n = sqrt(bx * bx + by * by + bz * bz);
  bx /= n; by /= n; bz /= n;
  double t = bx * bx + by * by, r00 = 1, r01 = 0, r11 = bz;
  if (t > 0) {
    double w = (1 - bz) / t;
    r00 = bz + w * (by * by);
    r01 = -w * (bx * by);
    r11 = bz + w * (bx * bx);
  }
  R[0][0] = r00; R[0][1] = r01; R[0][2] = bx;
  R[1][0] = r01; R[1][1] = r11; R[1][2] = by;
  R[2][0] = -bx; R[2][1] = -by; R[2][2] = bz;
}

/* phs_cpu.cpp:174-234 */
static void set_msq(ev_t *e, int code, double *factor, double *volume) {
  const oracle_t *o = e->o;
  int i = e->c * o->stride + code;
  int k1 = o->k1[i], k2 = o->k2[i];
  double f1, f2, v1, v2;
  if (o->has_ch[e->c * o->stride + k1]) {
    set_msq(e, k1, &f1, &v1);
    if (!e->ok) return;
  } else {
    f1 = 1; v1 = 1;
  }
  if (o->has_ch[e->c * o->stride + k2]) {
    set_msq(e, k2, &f2, &v2);
    if (!e->ok) return;
  } else {
    f2 = 1; v2 = 1;
  }
  double sqrts = e->sqrts, m_max;
  if (code == o->n_codes) {
    e->p2[code] = sqrts * sqrts;
    m_max = sqrts;
    *factor = f1 * f2;
    *volume = v1 * v2 / (4 * OR_TWOPI5);
  } else {
    double m_min = o->mass_sum[i];
    m_max = sqrts - e->m_tot + m_min;
    msq_from_x(o->map_id[i], e->x[e->id_x], sqrts * sqrts, o->m[i], o->w[i], m_min * m_min,
               m_max * m_max, e->a + 3 * code, &e->p2[code], factor, o->nudge);
    e->id_x++;
    *factor *= f1 * f2;
    *volume = v1 * v2 * sqrts * sqrts / (4 * OR_TWOPI2);
  }
  double msq = e->p2[code], msq1 = e->p2[k1], msq2 = e->p2[k2];
  double m1 = sqrt(msq1), m2 = sqrt(msq2), m = sqrt(msq);
  double lda = (msq - msq1 - msq2) * (msq - msq1 - msq2) - 4 * msq1 * msq2;
  if (lda > 0 && m > m1 + m2 && m <= m_max) {
    {
      /* relative change of lda per relative change of msq, msq1, msq2 (summed): how much
       * the branch amplifies one-ulp differences of the mapped masses (it diverges at
       * threshold, where lda -> 0); kept apart from every value the restatement returns */
      const double d = msq - msq1 - msq2;
      const double k = (fabs(2 * d) * msq + fabs(2 * d + 4 * msq2) * msq1 +
                        fabs(2 * d + 4 * msq1) * msq2) / lda;
      if (k > e->kappa) e->kappa = k;
    }
    e->p_decay[k1] = sqrt(lda) / (2 * m);
    e->p_decay[k2] = -e->p_decay[k1];
    *factor *= sqrt(lda) / msq;
  } else {
    e->ok = 0;
  }
}

/* phs_cpu.cpp:283-345 */
static void set_angles(ev_t *e, int code, double *factor, double L0[4][4]) {
  const oracle_t *o = e->o;
  int i = e->c * o->stride + code;
  double p = e->p_decay[code];
  double m = sqrt(e->p2[code]);
  double E = sqrt(e->p2[code] + p * p);
  for (int r = 0; r < 4; r++) e->p[code][r] = L0[r][0] * E + L0[r][3] * p;
  if (!o->has_ch[i]) return;
  double bg = m > 0 ? p / m : 0;
  double gamma = sqrt(1 + bg * bg);
  double phi = e->x[e->id_x] * OR_TWOPI;
  e->id_x++;
  double cp = cos(phi), sp = sin(phi);
  double xx = e->x[e->id_x];
  e->id_x++;
  double ct, st, f;
  ct_from_x(o->map_id[i], xx, e->b + 3 * code, &ct, &st, &f, o->nudge);
  *factor *= f;
  double L1[4][4] = {
      {gamma, -bg * st, 0, bg * ct},
      {0, ct * cp, -sp, st * cp},
      {0, ct * sp, cp, st * sp},
      {bg, -gamma * st, 0, gamma * ct}};
  int ff = o->friend_sign ? o->friend_sign[i] : 0;
  if (ff) {
    /* phs.cu:853-910: the decay angles are measured from the friend beam's direction in
     * the branch's rest frame, B_z(-bg) L0^-1 (1, 0, 0, ff) (only its direction matters) */
    double u0 = L0[0][0] - ff * L0[3][0];
    double ax = -(L0[0][1] - ff * L0[3][1]);
    double ay = -(L0[0][2] - ff * L0[3][2]);
    double az = -bg * u0 - gamma * (L0[0][3] - ff * L0[3][3]);
    double Rf[3][3], Q[3][3];
    double A[3][3] = {{ct * cp, -sp, st * cp}, {ct * sp, cp, st * sp}, {-st, 0, ct}};
    rot_z_onto(ax, ay, az, Rf);
    for (int r = 0; r < 3; r++)
      for (int s = 0; s < 3; s++) Q[r][s] = Rf[r][0] * A[0][s] + Rf[r][1] * A[1][s] + Rf[r][2] * A[2][s];
    /* L1 = B_z(bg) diag(1, Q) */
    L1[0][0] = gamma; L1[1][0] = 0; L1[2][0] = 0; L1[3][0] = bg;
    for (int s = 0; s < 3; s++) {
      L1[0][s + 1] = bg * Q[2][s];
      L1[1][s + 1] = Q[0][s];
      L1[2][s + 1] = Q[1][s];
      L1[3][s + 1] = gamma * Q[2][s];
    }
  }
  double Ln[4][4];
  memset(Ln, 0, sizeof Ln);
  for (int r = 0; r < 4; r++)
    for (int s = 0; s < 4; s++)
      for (int k = 0; k < 4; k++) Ln[r][s] += L0[r][k] * L1[k][s];
  set_angles(e, o->k1[i], factor, Ln);
  set_angles(e, o->k2[i], factor, Ln);
}

static double volume_rec(const oracle_t *o, int c, int code, double sqrts) {
  int i = c * o->stride + code;
  if (!o->has_ch[i]) return 1;
  double v1 = volume_rec(o, c, o->k1[i], sqrts);
  double v2 = volume_rec(o, c, o->k2[i], sqrts);
  if (code == o->n_codes) return v1 * v2 / (4 * OR_TWOPI5);
  return v1 * v2 * sqrts * sqrts / (4 * OR_TWOPI2);
}

/* ---------------------------------------------------------------------------------- API */

void oracle_destroy(oracle_t *o) {
  if (!o) return;
  free(o->k1); free(o->k2); free(o->has_ch); free(o->map_id);
  free(o->m); free(o->w); free(o->mass_sum); free(o->a); free(o->b); free(o->flv_masses);
  free(o->friend_sign);
  free(o);
}

/* d1/d2/has_children: [n_channels][2^(n_in+n_out)-1] by code-1, daughter codes (0 = none).
 * map_ids/map_masses/map_widths: [n_channels][2^n_out-1] by code-1.
 * Returns NULL on a malformed tree or an unknown mapping id. */
oracle_t *oracle_create(int n_in, int n_out, int n_channels, const int *d1, const int *d2,
                        const int *has_children, const int *map_ids, const double *map_masses,
                        const double *map_widths, const double *flv_masses) {
  if (n_in < 1 || n_in > 2 || n_out < 2 || n_out > 16 || n_channels < 1) return NULL;
  oracle_t *o = (oracle_t *)calloc(1, sizeof(oracle_t));
  o->n_in = n_in; o->n_out = n_out; o->n_channels = n_channels;
  o->n_codes = (1 << n_out) - 1;
  o->stride = o->n_codes + 1;
  int n_prt = (1 << (n_in + n_out)) - 1;
  size_t nt = (size_t)n_channels * o->stride;
  o->k1 = calloc(nt, sizeof(int)); o->k2 = calloc(nt, sizeof(int));
  o->has_ch = calloc(nt, sizeof(int)); o->map_id = calloc(nt, sizeof(int));
  o->m = calloc(nt, sizeof(double)); o->w = calloc(nt, sizeof(double));
  o->mass_sum = calloc(nt, sizeof(double));
  o->a = calloc(nt * 3, sizeof(double)); o->b = calloc(nt * 3, sizeof(double));
  o->flv_masses = calloc(n_in + n_out, sizeof(double));
  memcpy(o->flv_masses, flv_masses, (n_in + n_out) * sizeof(double));
  for (int c = 0; c < n_channels; c++) {
    for (int code = 1; code <= o->n_codes; code++) {
      int i = c * o->stride + code;
      int src = c * n_prt + code - 1, srm = c * o->n_codes + code - 1;
      o->has_ch[i] = has_children[src] != 0;
      o->k1[i] = d1[src]; o->k2[i] = d2[src];
      o->map_id[i] = map_ids[srm];
      o->m[i] = map_masses[srm]; o->w[i] = map_widths[srm];
      if (o->has_ch[i]) {
        int a = o->k1[i], b = o->k2[i];
        if (a < 1 || b < 1 || a > o->n_codes || b > o->n_codes || (a & b) || (a | b) != code) {
          oracle_destroy(o);
          return NULL;
        }
        if (!map_id_known(o->map_id[i])) { oracle_destroy(o); return NULL; }
      } else if (code & (code - 1)) { /* a composite code without children */
        /* only reachable codes matter; checked by the walk below */
      }
    }
    /* every code reachable from the root must be a leaf (power of two) or have children */
    int stack[64], sp = 0;
    stack[sp++] = o->n_codes;
    while (sp) {
      int code = stack[--sp];
      int i = c * o->stride + code;
      if (o->has_ch[i]) { stack[sp++] = o->k1[i]; stack[sp++] = o->k2[i]; }
      else if (code & (code - 1)) { oracle_destroy(o); return NULL; }
    }
    if (!o->has_ch[c * o->stride + o->n_codes]) { oracle_destroy(o); return NULL; }
    mass_sum_rec(o, c, o->n_codes);
  }
  return o;
}

void oracle_set_sqrts(oracle_t *o, double sqrts) {
  o->sqrts = sqrts;
  for (int c = 0; c < o->n_channels; c++)
    constants_for(o, c, sqrts, o->a + (size_t)c * o->stride * 3, o->b + (size_t)c * o->stride * 3, 0);
}

/* A test's sensitivity probe, never the reference's arithmetic: every value a
 * transcendental function returns on the mapping path -- the forward and inverse maps' own
 * tan, atan, exp and log and, with per-event beams, the constants formed per event
 * (constants_for) -- moved by `ulps` ulps from here on; 0 restores the reference's
 * arithmetic.  The uniform-beam constants (formed once, as the device takes them from the
 * host) are never moved. */
void oracle_set_nudge(oracle_t *o, int ulps) { o->nudge = ulps; }

/* Constants for channel c at sqrts, [3*(2^n_out)] each, for inspection by tests. */
void oracle_get_constants(const oracle_t *o, int c, double *a, double *b) {
  memcpy(a, o->a + (size_t)c * o->stride * 3, (size_t)o->stride * 3 * sizeof(double));
  memcpy(b, o->b + (size_t)c * o->stride * 3, (size_t)o->stride * 3 * sizeof(double));
}

double oracle_mass_sum(const oracle_t *o, int c, int code) { return o->mass_sum[c * o->stride + code]; }

typedef struct {
  const oracle_t *o;
  long lo, hi;
  int n_x;
  const double *x;
  const int *channels;
  const double *E1, *E2; /* NULL: uniform beams at o->sqrts, constants precomputed */
  double *p, *factors, *volumes;
  unsigned char *oks;
  double *kappa; /* optional per-event output */
} job_t;

static void *run_job(void *arg) {
  job_t *j = (job_t *)arg;
  const oracle_t *o = j->o;
  int nc = o->n_codes;
  double *p2 = malloc((nc + 1) * sizeof(double));
  double *pd = malloc((nc + 1) * sizeof(double));
  double(*pp)[4] = malloc((nc + 1) * sizeof(double[4]));
  double *a_ev = malloc((size_t)o->stride * 3 * sizeof(double));
  double *b_ev = malloc((size_t)o->stride * 3 * sizeof(double));
  for (long ev = j->lo; ev < j->hi; ev++) {
    int c = j->channels ? j->channels[ev] : 0;
    ev_t e;
    e.o = o; e.c = c; e.x = j->x + (size_t)j->n_x * ev; e.id_x = 0;
    double bg_lab = 0, ga_lab = 1;
    int lab = 0;
    if (j->E1) {
      double E1 = j->E1[ev], E2 = j->E2[ev];
      e.sqrts = 2 * sqrt(E1 * E2);
      constants_for(o, c, e.sqrts, a_ev, b_ev, o->nudge);
      e.a = a_ev; e.b = b_ev;
      if (E1 != E2) { /* phs.cu:1286-1301 */
        lab = 1;
        bg_lab = (E1 - E2) / (2 * sqrt(E1 * E2));
        ga_lab = sqrt(1 + bg_lab * bg_lab);
      }
    } else {
      e.sqrts = o->sqrts;
      e.a = o->a + (size_t)c * o->stride * 3;
      e.b = o->b + (size_t)c * o->stride * 3;
    }
    e.m_tot = o->mass_sum[c * o->stride + nc];
    e.p2 = p2; e.p_decay = pd; e.p = pp; e.ok = 1; e.kappa = 0;
    /* phs_cpu.cpp:586-593 */
    memset(pd, 0, (nc + 1) * sizeof(double));
    memset(pp, 0, (nc + 1) * sizeof(double[4]));
    memset(p2, 0, (nc + 1) * sizeof(double));
    for (int k = 0; k < o->n_out; k++) {
      double mk = o->flv_masses[o->n_in + k];
      p2[1 << k] = mk * mk;
    }
    double factor = 0, volume = 0;
    set_msq(&e, nc, &factor, &volume);
    double *pout = j->p + (size_t)4 * o->n_out * ev;
    if (e.ok) {
      double L0[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
      set_angles(&e, nc, &factor, L0);
      for (int k = 0; k < o->n_out; k++) {
        double *q = pp[1 << k];
        if (lab) {
          double q0 = ga_lab * q[0] + bg_lab * q[3];
          double q3 = bg_lab * q[0] + ga_lab * q[3];
          q[0] = q0; q[3] = q3;
        }
        for (int r = 0; r < 4; r++) pout[4 * k + r] = q[r];
      }
      j->factors[ev] = factor;
      j->volumes[ev] = volume;
      j->oks[ev] = 1;
    } else {
      memset(pout, 0, (size_t)4 * o->n_out * sizeof(double));
      j->factors[ev] = 0;
      j->volumes[ev] = volume_rec(o, c, nc, e.sqrts);
      j->oks[ev] = 0;
    }
    if (j->kappa) j->kappa[ev] = e.kappa;
  }
  free(p2); free(pd); free(pp); free(a_ev); free(b_ev);
  return NULL;
}

static int run_threads(job_t *base, long n_events, int n_threads) {
  if (n_threads < 1) n_threads = 1;
  if (n_threads > 512) n_threads = 512;
  if (n_events < n_threads) n_threads = n_events > 0 ? (int)n_events : 1;
  pthread_t th[512];
  job_t jobs[512];
  for (int t = 0; t < n_threads; t++) {
    jobs[t] = *base;
    jobs[t].lo = n_events * t / n_threads;
    jobs[t].hi = n_events * (t + 1) / n_threads;
  }
  for (int t = 1; t < n_threads; t++) pthread_create(&th[t], NULL, run_job, &jobs[t]);
  run_job(&jobs[0]);
  for (int t = 1; t < n_threads; t++) pthread_join(th[t], NULL);
  return 0;
}

/* Uniform beams: constants and msq bounds at the sqrts given to oracle_set_sqrts (the
 * reference CPU path's semantics, phs_cpu.cpp:550-600).  channels may be NULL (all 0). */
int oracle_generate(const oracle_t *o, long n_events, int n_x, const double *x, const int *channels,
                    double *p, double *factors, double *volumes, unsigned char *oks, int n_threads) {
  job_t j = {o, 0, 0, n_x, x, channels, NULL, NULL, p, factors, volumes, oks, NULL};
  return run_threads(&j, n_events, n_threads);
}

/* As oracle_generate, and per event kappa[ev] = the largest, over the branches whose
 * kinematic test passed, of sum_q |d lda / d q| q / lda (q = msq of the branch and of its
 * two daughters, lda the Kallen function): the relative change of sqrt(lda), and so of the
 * factor, is kappa / 2 times a relative change of the masses.  A one-ulp difference of a
 * transcendental function (tan, exp, log) between two libraries moves a mapped mass by
 * about one ulp, so two correct FP64 implementations can disagree on the factor by a few
 * ulps times kappa.  0 for events that fail the test before any branch passes. */
int oracle_generate_cond(const oracle_t *o, long n_events, int n_x, const double *x,
                         const int *channels, double *p, double *factors, double *volumes,
                         unsigned char *oks, double *kappa, int n_threads) {
  job_t j = {o, 0, 0, n_x, x, channels, NULL, NULL, p, factors, volumes, oks, kappa};
  return run_threads(&j, n_events, n_threads);
}

/* Per-event beams: sqrts = 2 sqrt(E1 E2) per event, constants recomputed per event with
 * the formulas of phs_cpu.cpp:452-531, and the longitudinal lab boost of phs.cu:1286-1301
 * when E1 != E2. */
int oracle_generate_beams(const oracle_t *o, long n_events, int n_x, const double *x,
                          const int *channels, const double *E1, const double *E2, double *p,
                          double *factors, double *volumes, unsigned char *oks, int n_threads) {
  job_t j = {o, 0, 0, n_x, x, channels, E1, E2, p, factors, volumes, oks, NULL};
  return run_threads(&j, n_events, n_threads);
}

/* friends: [n_channels][2^(n_in+n_out)-1] by code-1, the Whizard code of the incoming
 * particle a branch is paired with (0 = none), as c_whizard_fill_tree_structure takes it
 * (whizard_gpu_phs.cpp:79-87).  As extract_boost_origins (phs.cu:268-292) reads it, code
 * 2^n_out selects the beam along -z and 2^(n_out+1) the beam along +z; other values and
 * leaves are ignored.  A friend on the root is rejected (-1): the reference divides by
 * zero there (phs.cu:753-765 with both axes along z). */
int oracle_set_friends(oracle_t *o, const int *friends) {
  int n_prt = (1 << (o->n_in + o->n_out)) - 1;
  size_t nt = (size_t)o->n_channels * o->stride;
  if (!o->friend_sign) o->friend_sign = calloc(nt, sizeof(int));
  for (int c = 0; c < o->n_channels; c++)
    for (int code = 1; code <= o->n_codes; code++) {
      int i = c * o->stride + code, f = friends[c * n_prt + code - 1];
      int sgn = f == (1 << o->n_out) ? -1 : f == (1 << (o->n_out + 1)) ? 1 : 0;
      if (!o->has_ch[i]) sgn = 0;
      if (sgn && code == o->n_codes) return -1;
      o->friend_sign[i] = sgn;
    }
  return 0;
}

/* ---------------------------------------------------------------------------------- */
/* Inverse mapping: momenta -> (x, factor) of a channel.                                */

/* mappings_gpu.hpp:15-172 (mapping_x_from_msq_*), with the constants of
 * init_mapping_constants_cpu. */
static void msq_to_x(int t, double msq, double s, double m, double w, double msq_min,
                     double msq_max, const double *a, double *x, double *factor, int nudge) {
  double z, z1, z2, z3;
  switch (t) {
    case OR_MAP_NO:
      *x = (msq - msq_min) / (msq_max - msq_min);
      *factor = (msq_max - msq_min) / s;
      break;
    case OR_MAP_SCHANNEL:
      z = (msq - m * m) / (m * w);
      *x = (ulps_moved(atan(z), nudge) - a[0]) / (a[1] - a[0]);
      *factor = a[2] * (1 + z * z);
      break;
    case OR_MAP_COLLINEAR:
    case OR_MAP_INFRARED:
    case OR_MAP_RADIATION:
      z = msq - msq_min + a[0];
      *x = ulps_moved(log(z / a[0]), nudge) / a[1];
      *factor = a[2] * z;
      break;
    case OR_MAP_TCHANNEL:
    case OR_MAP_UCHANNEL:
      if (msq < (msq_max + msq_min) / 2) {
        z = msq - msq_min + a[0];
        *x = ulps_moved(log(z / a[0]), nudge) / a[1];
      } else {
        z = msq_max - msq + a[0];
        *x = 1 - ulps_moved(log(z / a[0]), nudge) / a[1];
      }
      *factor = a[2] * z;
      break;
    case OR_MAP_STEP_E:
      z1 = (msq - msq_min) / (msq_max - msq_min);
      z2 = 1 + a[1] * ulps_moved(exp(z1 / a[2]), nudge);
      *x = (z1 - a[2] * ulps_moved(log(z2 / (1 + a[1])), nudge)) / a[0];
      *factor = a[0] * z2 * (msq_max - msq_min) / s;
      break;
    case OR_MAP_STEP_H:
      z1 = (msq - msq_min) / (msq_max - msq_min);
      z3 = a[0] - z1 / a[2];
      *x = ((a[0] + z1 / a[2] + z1) - sqrt(z3 * z3 + 2 * z1 * (a[0] + z1 / a[2]) + z1 * z1)) / 2;
      *factor = (a[1] / (a[0] - *x) / (a[0] - *x) + a[2]) * (msq_max - msq_min) / s;
      break;
    default:
      *x = 0;
      *factor = 0;
  }
}

/* mappings_gpu.hpp:184-219 (mapping_x_from_ct_*) */
static void ct_to_x(int t, double ct, const double *b, double *x, double *factor, int nudge) {
  double ct1;
  switch (t) {
    case OR_MAP_COLLINEAR:
    case OR_MAP_TCHANNEL:
    case OR_MAP_UCHANNEL:
      if (ct < 0) {
        ct1 = ct + b[0] + 1;
        *x = ulps_moved(log(ct1 / b[0]), nudge) / (2 * b[1]);
      } else {
        ct1 = -ct + b[0] + 1;
        *x = 1 - ulps_moved(log(ct1 / b[0]), nudge) / (2 * b[1]);
      }
      *factor = ct1 * b[1];
      break;
    default:
      *x = (ct + 1) / 2;
      *factor = 1;
  }
}

typedef struct {
  const oracle_t *o;
  int c;
  const double *a, *b;
  double sqrts;
  double *x;            /* output row */
  int id_x;
  double *msq, *pd;     /* [code] */
  double (*p)[4];       /* [code][4], CM frame */
  double factor;
} inv_t;

static void matvec4(const double M[4][4], const double v[4], double out[4]) {
  for (int r = 0; r < 4; r++) {
    out[r] = 0;
    for (int k = 0; k < 4; k++) out[r] += M[r][k] * v[k];
  }
}

/* _combine_particles (phs.cu:1262-1283): internal momenta as sums of their daughters in
 * post-order, and msq of every branch from its momentum. */
static void inv_combine(inv_t *e, int code) {
  const oracle_t *o = e->o;
  int i = e->c * o->stride + code;
  if (o->has_ch[i]) {
    int k1 = o->k1[i], k2 = o->k2[i];
    inv_combine(e, k1);
    inv_combine(e, k2);
    for (int r = 0; r < 4; r++) e->p[code][r] = e->p[k1][r] + e->p[k2][r];
  }
  double *q = e->p[code];
  e->msq[code] = q[0] * q[0] - q[1] * q[1] - q[2] * q[2] - q[3] * q[3];
}

/* _apply_msq_inv (phs.cu:626-675): post-order; returns the subtree's factor. */
static double inv_msq(inv_t *e, int code) {
  const oracle_t *o = e->o;
  int i = e->c * o->stride + code;
  int k1 = o->k1[i], k2 = o->k2[i];
  double f1 = o->has_ch[e->c * o->stride + k1] ? inv_msq(e, k1) : 1;
  double f2 = o->has_ch[e->c * o->stride + k2] ? inv_msq(e, k2) : 1;
  double f;
  if (code == o->n_codes) {
    e->msq[code] = e->sqrts * e->sqrts;
    f = f1 * f2;
  } else {
    double m_tot = o->mass_sum[e->c * o->stride + o->n_codes];
    double m_min = o->mass_sum[i], m_max = e->sqrts - m_tot + m_min;
    msq_to_x(o->map_id[i], e->msq[code], e->sqrts * e->sqrts, o->m[i], o->w[i], m_min * m_min,
             m_max * m_max, e->a + 3 * code, &e->x[e->id_x], &f, o->nudge);
    e->id_x++;
    f *= f1 * f2;
  }
  double msq0 = e->msq[code], msq1 = e->msq[k1], msq2 = e->msq[k2];
  double m0 = sqrt(msq0);
  double lda = (msq0 - msq1 - msq2) * (msq0 - msq1 - msq2) - 4 * msq1 * msq2;
  e->pd[k1] = sqrt(lda) / (2 * m0);
  e->pd[k2] = -sqrt(lda) / (2 * m0);
  return f * (sqrt(lda) / msq0);
}

/* The boost inversion (phs.cu:924-1244), pre-order.  G takes CM momenta into the
 * branch's rest frame with z along the branch's flight direction (or its friend axis). */
static void inv_angles(inv_t *e, int code, double G[4][4]) {
  const oracle_t *o = e->o;
  int i = e->c * o->stride + code;
  int k1 = o->k1[i], k2 = o->k2[i];
  double q[4];
  matvec4((const double(*)[4])G, e->p[k1], q);
  /* azimuthal_angle, polar_angle_ct (phs.cu:913-922) */
  double phi = atan2(q[2], q[1]);
  if (phi < 0) phi += OR_TWOPI;
  e->x[e->id_x++] = phi / OR_TWOPI;
  double dn = sqrt(q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  double ct = q[3] / dn, st = sqrt(1 - ct * ct), f;
  ct_to_x(o->map_id[i], ct, e->b + 3 * code, &e->x[e->id_x++], &f, o->nudge);
  e->factor *= f;
  double cp = cos(phi), sp = sin(phi);
  int kids[2] = {k1, k2};
  for (int j = 0; j < 2; j++) {
    int kc = kids[j], ki = e->c * o->stride + kc;
    if (!o->has_ch[ki]) continue;
    double m = sqrt(e->msq[kc]);
    double bg = m > 0 ? e->pd[kc] / m : 0;
    double gamma = sqrt(1 + bg * bg);
    /* L_r3_r2_b3(-bg, gamma, ct, -st, cp, -sp) = B_z(-bg) R_y(-theta) R_z(-phi) */
    double T[4][4] = {
        {gamma, -bg * st * cp, -bg * st * sp, -bg * ct},
        {0, ct * cp, ct * sp, -st},
        {0, -sp, cp, 0},
        {-bg, gamma * st * cp, gamma * st * sp, gamma * ct}};
    double H[4][4];
    for (int r = 0; r < 4; r++)
      for (int s = 0; s < 4; s++) {
        H[r][s] = 0;
        for (int k = 0; k < 4; k++) H[r][s] += T[r][k] * G[k][s];
      }
    int ff = o->friend_sign ? o->friend_sign[ki] : 0;
    if (ff) {
      /* rotate the friend beam's direction H (1, 0, 0, ff) onto z (phs.cu:1183-1206) */
      double Rf[3][3], Hn[4][4];
      rot_z_onto(H[1][0] + ff * H[1][3], H[2][0] + ff * H[2][3], H[3][0] + ff * H[3][3], Rf);
      for (int s = 0; s < 4; s++) {
        Hn[0][s] = H[0][s];
        for (int r = 0; r < 3; r++)
          Hn[r + 1][s] = Rf[0][r] * H[1][s] + Rf[1][r] * H[2][s] + Rf[2][r] * H[3][s];
      }
      memcpy(H, Hn, sizeof H);
    }
    inv_angles(e, kc, H);
  }
}

typedef struct {
  const oracle_t *o;
  long lo, hi;
  int n_x;
  const double *p;
  const int *channels;
  const unsigned char *oks;
  const double *E1, *E2;
  const double *x_own, *factor_own;
  double *all_factors, *x_out;
  long n_events;
} inv_job_t;

static void *run_inv_job(void *arg) {
  inv_job_t *j = (inv_job_t *)arg;
  const oracle_t *o = j->o;
  int nc = o->n_codes, n_ch = o->n_channels;
  double *msq = malloc((nc + 1) * sizeof(double)), *pd = malloc((nc + 1) * sizeof(double));
  double(*pp)[4] = malloc((nc + 1) * sizeof(double[4]));
  double *a_ev = malloc((size_t)o->stride * 3 * sizeof(double));
  double *b_ev = malloc((size_t)o->stride * 3 * sizeof(double));
  for (long ev = j->lo; ev < j->hi; ev++) {
    int own = j->channels ? j->channels[ev] : 0;
    int ok = j->oks ? j->oks[ev] != 0 : 1;
    double sqrts = o->sqrts, bg_lab = 0, ga_lab = 1;
    if (j->E1) {
      double E1 = j->E1[ev], E2 = j->E2[ev];
      sqrts = 2 * sqrt(E1 * E2);
      bg_lab = (E1 - E2) / (2 * sqrt(E1 * E2));
      ga_lab = sqrt(1 + bg_lab * bg_lab);
    }
    for (int c = 0; c < n_ch; c++) {
      double *xr = j->x_out + ((size_t)c * j->n_events + ev) * j->n_x;
      double *fo = j->all_factors + (size_t)ev * n_ch + c;
      if (c == own && j->x_own) {
        memcpy(xr, j->x_own + (size_t)ev * j->n_x, j->n_x * sizeof(double));
        *fo = j->factor_own ? j->factor_own[ev] : 0;
        continue;
      }
      if (j->x_own) memcpy(xr, j->x_own + (size_t)ev * j->n_x, j->n_x * sizeof(double));
      else memset(xr, 0, j->n_x * sizeof(double));
      if (!ok) {
        memset(xr, 0, (size_t)(3 * o->n_out - 4) * sizeof(double));
        *fo = 0;
        continue;
      }
      inv_t e;
      e.o = o; e.c = c; e.sqrts = sqrts; e.x = xr; e.id_x = 0;
      e.msq = msq; e.pd = pd; e.p = pp; e.factor = 1;
      if (j->E1) {
        constants_for(o, c, sqrts, a_ev, b_ev, o->nudge);
        e.a = a_ev; e.b = b_ev;
      } else {
        e.a = o->a + (size_t)c * o->stride * 3;
        e.b = o->b + (size_t)c * o->stride * 3;
      }
      memset(pd, 0, (nc + 1) * sizeof(double));
      for (int k = 0; k < o->n_out; k++) {
        const double *q = j->p + ((size_t)ev * o->n_out + k) * 4;
        double *t = pp[1 << k];
        t[0] = ga_lab * q[0] - bg_lab * q[3];  /* lab -> CM (phs.cu:1286-1301 inverted) */
        t[1] = q[1];
        t[2] = q[2];
        t[3] = -bg_lab * q[0] + ga_lab * q[3];
      }
      inv_combine(&e, nc);
      double fmsq = inv_msq(&e, nc);
      double G[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
      inv_angles(&e, nc, G);
      *fo = fmsq * e.factor;
    }
  }
  free(msq); free(pd); free(pp); free(a_ev); free(b_ev);
  return NULL;
}

/* All-channel factors and x of generated events (gen_phs_from_x_gpu with
 * do_inverse_mapping, phs.cu:1499-1554).  p: [n][n_out][4] lab momenta; channels: the
 * generating channel per event (NULL: 0); oks (NULL: all 1); E1/E2 per event (NULL:
 * uniform beams at the oracle's sqrts).  Outputs all_factors [n][n_channels] and
 * x_out [n_channels][n][n_x].  For the generating channel the row is x_own and the
 * factor factor_own (copies, as the reference's _move_x/_move_factors) when x_own is
 * given, else the inverse itself.  Events with ok = 0 get factor 0 and x 0 for the
 * other channels. */
int oracle_inverse(const oracle_t *o, long n_events, int n_x, const double *p,
                   const int *channels, const unsigned char *oks, const double *E1,
                   const double *E2, const double *x_own, const double *factor_own,
                   double *all_factors, double *x_out, int n_threads) {
  if (n_threads < 1) n_threads = 1;
  if (n_threads > 512) n_threads = 512;
  if (n_events < n_threads) n_threads = n_events > 0 ? (int)n_events : 1;
  pthread_t th[512];
  inv_job_t jobs[512];
  for (int t = 0; t < n_threads; t++) {
    inv_job_t jb = {o, n_events * t / n_threads, n_events * (t + 1) / n_threads, n_x, p,
                    channels, oks, E1, E2, x_own, factor_own, all_factors, x_out, n_events};
    jobs[t] = jb;
  }
  for (int t = 1; t < n_threads; t++) pthread_create(&th[t], NULL, run_inv_job, &jobs[t]);
  run_inv_job(&jobs[0]);
  for (int t = 1; t < n_threads; t++) pthread_join(th[t], NULL);
  return 0;
}

/* ------------------------------------------------------------------------ Philox x
 * The benchmark's x stream on the host, multi-threaded: Philox4x32-10 (Salmon et al.,
 * SC'11) with the layout of gpu_phs_gb300/philox.py (element e of the flat array takes
 * block e >> 1, counter (block lo, block hi, 0, 0), key (seed lo, seed hi); the output
 * words give two doubles ((r0 << 32 | r1) >> 11) 2^-53 and ((r2 << 32 | r3) >> 11) 2^-53,
 * element e the (e & 1)-th).  For full-size comparisons, where numpy is too slow. */
typedef struct {
  uint64_t seed;
  long e0, n; /* flat elements [e0, e0 + n) of the stream, written to out[0 .. n) */
  double *out;
} philox_job_t;

static void philox_block(uint64_t block, uint64_t seed, double u[2]) {
  uint32_t c0 = (uint32_t)block, c1 = (uint32_t)(block >> 32), c2 = 0, c3 = 0;
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (int r = 0; r < 10; r++) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n1 = (uint32_t)p1;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1, n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  u[0] = (double)((((uint64_t)c0 << 32) | c1) >> 11) * 0x1.0p-53;
  u[1] = (double)((((uint64_t)c2 << 32) | c3) >> 11) * 0x1.0p-53;
}

static void *run_philox(void *arg) {
  const philox_job_t *j = (const philox_job_t *)arg;
  for (long i = 0; i < j->n; i++) {
    const long e = j->e0 + i;
    double u[2];
    philox_block((uint64_t)(e >> 1), j->seed, u);
    j->out[i] = u[e & 1];
  }
  return NULL;
}

int oracle_uniform_x(uint64_t seed, long first_event, long n_events, int n_x, double *x,
                     int n_threads) {
  if (n_events < 0 || n_x < 1 || first_event < 0) return -1;
  const long n = n_events * n_x, e0 = first_event * n_x;
  if (n_threads < 1) n_threads = 1;
  if (n_threads > 512) n_threads = 512;
  if (n < 4096L * n_threads) n_threads = 1;
  philox_job_t jobs[512];
  pthread_t th[512];
  for (int t = 0; t < n_threads; t++) {
    const long lo = n * t / n_threads, hi = n * (t + 1) / n_threads;
    philox_job_t jb = {seed, e0 + lo, hi - lo, x + lo};
    jobs[t] = jb;
  }
  for (int t = 1; t < n_threads; t++) pthread_create(&th[t], NULL, run_philox, &jobs[t]);
  run_philox(&jobs[0]);
  for (int t = 1; t < n_threads; t++) pthread_join(th[t], NULL);
  return 0;
}
