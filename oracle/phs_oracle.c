/*
 * phs_oracle.c -- CPU restatement of gpu_phs's forward phase-space generator.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA path: only
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
  double sqrts;           /* sqrts the constants were computed for */
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

/* phs_cpu.cpp:452-531, for one channel and one sqrts, into a/b. */
static void constants_for(const oracle_t *o, int c, double sqrts, double *a_out, double *b_out) {
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
        a[1] = atan((msq_max - msq0) / (m * w));
        a[2] = (a[1] - a[0]) * (m * w) / s;
        break;
      case OR_MAP_RADIATION:
      case OR_MAP_COLLINEAR:
      case OR_MAP_INFRARED:
        msq0 = (t == OR_MAP_RADIATION) ? w * w : m * m;
        a[0] = msq0;
        a[1] = log((msq_max - msq_min) / msq0 + 1);
        a[2] = a[1] / s;
        break;
      case OR_MAP_TCHANNEL:
      case OR_MAP_UCHANNEL:
        msq0 = m * m;
        a[0] = msq0;
        a[1] = 2 * log((msq_max - msq_min) / (2 * msq0) + 1);
        a[2] = a[1] / s;
        break;
      case OR_MAP_STEP_E: {
        double r = 2 * m * w / (msq_max - msq_min);
        a[2] = r > 0.01 ? r : 0.01;
        a[1] = exp(-(m * m - msq_min) / (msq_max - msq_min) / a[2]);
        a[0] = 1 - a[2] * log((1 + a[1] * exp(1 / a[2])) / (1 + a[1]));
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
        b[1] = log((b[0] + 1) / b[0]);
        b[2] = 0;
        break;
      default:
        b[0] = b[1] = b[2] = 0;
    }
  }
}

/* phs_cpu.cpp:12-61 */
static void msq_from_x(int t, double x, double s, double m, double w, double msq_min, double msq_max,
                       const double *a, double *msq, double *factor) {
  double msq1, tmp, z;
  switch (t) {
    case OR_MAP_NO:
      *msq = (1 - x) * msq_min + x * msq_max;
      *factor = (msq_max - msq_min) / s;
      break;
    case OR_MAP_SCHANNEL:
      z = (1 - x) * a[0] + x * a[1];
      if (-OR_PI / 2 < z && z < OR_PI / 2) {
        tmp = tan(z);
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
      msq1 = a[0] * exp(x * a[1]);
      *msq = msq1 - a[0] + msq_min;
      *factor = a[2] * msq1;
      break;
    case OR_MAP_TCHANNEL:
    case OR_MAP_UCHANNEL:
      if (x < 0.5) {
        msq1 = a[0] * exp(x * a[1]);
        *msq = msq1 - a[0] + msq_min;
      } else {
        msq1 = a[0] * exp((1 - x) * a[1]);
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
      tmp = exp(-x * a[0] / a[2]) * (1 + a[1]);
      z = -a[2] * log(tmp - a[1]);
      *msq = z * msq_max + (1 - z) * msq_min;
      *factor = a[0] / (1 - a[1] / tmp) * (msq_max - msq_min) / s;
      break;
  }
}

/* phs_cpu.cpp:112-146 */
static void ct_from_x(int t, double x, const double *b, double *ct, double *st, double *factor) {
  double tmp;
  switch (t) {
    case OR_MAP_COLLINEAR:
    case OR_MAP_TCHANNEL:
    case OR_MAP_UCHANNEL:
      if (x < 0.5) {
        tmp = b[0] * exp(2 * x * b[1]);
        *ct = tmp - b[0] - 1;
      } else {
        tmp = b[0] * exp(2 * (1 - x) * b[1]);
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
} ev_t;

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
               m_max * m_max, e->a + 3 * code, &e->p2[code], factor);
    e->id_x++;
    *factor *= f1 * f2;
    *volume = v1 * v2 * sqrts * sqrts / (4 * OR_TWOPI2);
  }
  double msq = e->p2[code], msq1 = e->p2[k1], msq2 = e->p2[k2];
  double m1 = sqrt(msq1), m2 = sqrt(msq2), m = sqrt(msq);
  double lda = (msq - msq1 - msq2) * (msq - msq1 - msq2) - 4 * msq1 * msq2;
  if (lda > 0 && m > m1 + m2 && m <= m_max) {
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
  ct_from_x(o->map_id[i], xx, e->b + 3 * code, &ct, &st, &f);
  *factor *= f;
  double L1[4][4] = {
      {gamma, -bg * st, 0, bg * ct},
      {0, ct * cp, -sp, st * cp},
      {0, ct * sp, cp, st * sp},
      {bg, -gamma * st, 0, gamma * ct}};
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
    constants_for(o, c, sqrts, o->a + (size_t)c * o->stride * 3, o->b + (size_t)c * o->stride * 3);
}

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
      constants_for(o, c, e.sqrts, a_ev, b_ev);
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
    e.p2 = p2; e.p_decay = pd; e.p = pp; e.ok = 1;
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
  job_t j = {o, 0, 0, n_x, x, channels, NULL, NULL, p, factors, volumes, oks};
  return run_threads(&j, n_events, n_threads);
}

/* Per-event beams: sqrts = 2 sqrt(E1 E2) per event, constants recomputed per event with
 * the formulas of phs_cpu.cpp:452-531, and the longitudinal lab boost of phs.cu:1286-1301
 * when E1 != E2. */
int oracle_generate_beams(const oracle_t *o, long n_events, int n_x, const double *x,
                          const int *channels, const double *E1, const double *E2, double *p,
                          double *factors, double *volumes, unsigned char *oks, int n_threads) {
  job_t j = {o, 0, 0, n_x, x, channels, E1, E2, p, factors, volumes, oks};
  return run_threads(&j, n_events, n_threads);
}
