// phs_compile.cpp -- tree compiler: Whizard channel tables -> visit program.
//
// Replaces the reference's host-side flattening of the recursion (init_phs_gpu,
// phs.cu:327-509, with extract_msq_branch_idx 248, extract_boost_origins 268 and
// extract_boost_targets 294) and its device-side per-event constant evaluation
// (mappings_gpu.hpp:23-99): constants are computed once here with the formulas of
// init_mapping_constants_cpu (phs_cpu.cpp:452-531), mass sums as set_mass_sum
// (phs.cu:61-78), and the channel volume with the recursion of set_msq_cpu
// (phs_cpu.cpp:194-213).  This file is compiled with -ffp-contract=off so the constants
// equal the reference CPU path's bit for bit on every host.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <functional>

#include "../../include/gpu_phs.h"
#include "phs_host.h"

namespace phs {

static const double kTwoPi2 = 39.47841760435743447534;
static const double kTwoPi5 = 9792.62991312900650440772;

static bool map_id_known(int t) {
  switch (t) {
    case PHS_MAP_NO: case PHS_MAP_SCHANNEL: case PHS_MAP_TCHANNEL: case PHS_MAP_UCHANNEL:
    case PHS_MAP_RADIATION: case PHS_MAP_COLLINEAR: case PHS_MAP_INFRARED:
    case PHS_MAP_STEP_E: case PHS_MAP_STEP_H:
      return true;
  }
  return false;
}

static int ct_class_of(int t) {
  return (t == PHS_MAP_COLLINEAR || t == PHS_MAP_TCHANNEL || t == PHS_MAP_UCHANNEL)
             ? PHS_CT_COLLINEAR : PHS_CT_UNIFORM;
}

// phs_cpu.cpp:452-531 for one branch.
static void branch_constants(int t, double m, double w, double m_min, double m_max, double s,
                             double a[3], double b[3]) {
  double msq_min = m_min * m_min, msq_max = m_max * m_max, msq0;
  a[0] = a[1] = a[2] = 0;
  switch (t) {
    case PHS_MAP_NO:
      a[0] = 0;
      a[1] = msq_max - msq_min;
      a[2] = a[1] / s;
      break;
    case PHS_MAP_SCHANNEL:
      msq0 = m * m;
      a[0] = atan((msq_min - msq0) / (m * w));
      a[1] = atan((msq_max - msq0) / (m * w));
      a[2] = (a[1] - a[0]) * (m * w) / s;
      break;
    case PHS_MAP_RADIATION:
    case PHS_MAP_COLLINEAR:
    case PHS_MAP_INFRARED:
      msq0 = (t == PHS_MAP_RADIATION) ? w * w : m * m;
      a[0] = msq0;
      a[1] = log((msq_max - msq_min) / msq0 + 1);
      a[2] = a[1] / s;
      break;
    case PHS_MAP_TCHANNEL:
    case PHS_MAP_UCHANNEL:
      msq0 = m * m;
      a[0] = msq0;
      a[1] = 2 * log((msq_max - msq_min) / (2 * msq0) + 1);
      a[2] = a[1] / s;
      break;
    case PHS_MAP_STEP_E: {
      double r = 2 * m * w / (msq_max - msq_min);
      a[2] = r > 0.01 ? r : 0.01;
      a[1] = exp(-(m * m - msq_min) / (msq_max - msq_min) / a[2]);
      a[0] = 1 - a[2] * log((1 + a[1] * exp(1 / a[2])) / (1 + a[1]));
      break;
    }
    case PHS_MAP_STEP_H: {
      a[2] = (m * m - msq_min) / (msq_max - msq_min);
      double r = pow(2 * m * w / (msq_max - msq_min), 2) / a[2];
      a[1] = r > 0.000001 ? r : 0.000001;
      a[0] = (1 + sqrt(1 + 4 * a[1] / (1 - a[2]))) / 2;
      break;
    }
  }
  if (ct_class_of(t) == PHS_CT_COLLINEAR) {
    b[0] = m * m / s;
    b[1] = log((b[0] + 1) / b[0]);
    b[2] = 0;
  } else {
    b[0] = b[1] = b[2] = 0;
  }
}

int validate_process(const Process &p, std::string &err) {
  if (p.n_in < 1 || p.n_in > 2) { err = "n_in must be 1 or 2"; return PHS_ERR_INVALID_ARG; }
  if (p.n_out < 2 || p.n_out > PHS_MAX_OUT) {
    err = "n_out must be in [2, " + std::to_string(PHS_MAX_OUT) + "]";
    return PHS_ERR_UNSUPPORTED;
  }
  if (p.n_channels < 1) { err = "n_channels must be >= 1"; return PHS_ERR_INVALID_ARG; }
  if (p.n_x < 3 * p.n_out - 4) {
    err = "n_x = " + std::to_string(p.n_x) + " is below the " + std::to_string(3 * p.n_out - 4) +
          " random numbers a tree with n_out = " + std::to_string(p.n_out) + " consumes";
    return PHS_ERR_INVALID_ARG;
  }
  return PHS_OK;
}

int compile_channel(const Process &p, int c, double sqrts, PhsChannel &out, ChannelInfo &info,
                    std::string &err) {
  const int R = (1 << p.n_out) - 1;
  auto ix = [&](int code) { return (size_t)c * p.n_prt + code - 1; };
  auto mx = [&](int code) { return (size_t)c * p.n_prt_out + code - 1; };
  auto internal = [&](int code) { return p.has_children[ix(code)] != 0; };
  auto kid = [&](int code, int j) { return j == 0 ? p.d1[ix(code)] : p.d2[ix(code)]; };
  const std::string where = "channel " + std::to_string(c) + ": ";

  // structure: every reachable branch splits into two disjoint codes that OR to it
  if (!internal(R)) { err = where + "the root has no daughters"; return PHS_ERR_TREE; }
  std::vector<int> todo{R}, internals;
  while (!todo.empty()) {
    int code = todo.back();
    todo.pop_back();
    if (!internal(code)) {
      if (code & (code - 1)) {
        err = where + "branch " + std::to_string(code) + " is composite but has no daughters";
        return PHS_ERR_TREE;
      }
      continue;
    }
    int a = kid(code, 0), b = kid(code, 1);
    if (a < 1 || b < 1 || a > R || b > R || (a & b) || (a | b) != code) {
      err = where + "daughters " + std::to_string(a) + ", " + std::to_string(b) +
            " do not split branch " + std::to_string(code);
      return PHS_ERR_TREE;
    }
    int t = p.map_id[mx(code)];
    if (!map_id_known(t)) {
      err = where + "mapping id " + std::to_string(t) + " of branch " + std::to_string(code) +
            " is not implemented";
      return PHS_ERR_MAPPING;
    }
    internals.push_back(code);
    todo.push_back(a);
    todo.push_back(b);
  }
  if ((int)internals.size() != p.n_out - 1) { err = where + "malformed tree"; return PHS_ERR_TREE; }

  // mass sums (phs.cu:61-78)
  std::vector<double> ms(R + 1, 0.0);
  std::function<double(int)> msum = [&](int code) -> double {
    if (internal(code)) return ms[code] = msum(kid(code, 0)) + msum(kid(code, 1));
    int ld2 = 0, bb = code;
    while (bb > 1) { bb /= 2; ld2++; }
    return ms[code] = p.flv_m[p.n_in + ld2];
  };
  msum(R);
  const double m_tot = ms[R], s = sqrts * sqrts;

  // x indices: msq x's in post-order over non-root internals, then (phi, ct) in pre-order
  std::vector<int> x_msq(R + 1, -1), x_ang(R + 1, -1);
  int nm = 0, na = 0;
  std::function<void(int)> post = [&](int code) {
    if (!internal(code)) return;
    post(kid(code, 0));
    post(kid(code, 1));
    if (code != R) x_msq[code] = nm++;
  };
  post(R);
  std::function<void(int)> pre = [&](int code) {
    if (!internal(code)) return;
    x_ang[code] = (p.n_out - 2) + 2 * na++;
    pre(kid(code, 0));
    pre(kid(code, 1));
  };
  pre(R);

  memset(&out, 0, sizeof(out));
  out.n_out = p.n_out;
  out.n_x_used = 3 * p.n_out - 4;
  out.m_tot = m_tot;

  auto fill_child = [&](int code, PhsChild &ch) {
    memset(&ch, 0, sizeof(ch));
    if (!internal(code)) {
      int ld2 = 0, bb = code;
      while (bb > 1) { bb /= 2; ld2++; }
      double fm = p.flv_m[p.n_in + ld2];
      ch.internal = 0;
      ch.out_index = ld2;
      ch.msq_leaf = fm * fm;
      ch.m_leaf = sqrt(ch.msq_leaf);
      return;
    }
    double a[3], b[3];
    double m_min = ms[code];
    double m_max = sqrts - m_tot + m_min;
    int t = p.map_id[mx(code)];
    branch_constants(t, p.map_m[mx(code)], p.map_w[mx(code)], m_min, m_max, s, a, b);
    ch.internal = 1;
    ch.out_index = -1;
    ch.map_id = t;
    ch.x_msq = x_msq[code];
    ch.m = p.map_m[mx(code)];
    ch.w = p.map_w[mx(code)];
    ch.a0 = a[0]; ch.a1 = a[1]; ch.a2 = a[2];
    ch.msq_min = m_min * m_min;
    ch.msq_max = m_max * m_max;
    ch.m_max = m_max;
    ch.m_min = m_min;
    if (t == PHS_MAP_SCHANNEL) {
      ch.msq0 = ch.m * ch.m;
      ch.inv_mw = 1.0 / (ch.m * ch.w);
      ch.inv_da = 1.0 / (ch.a1 - ch.a0);
    }
  };

  // visit order: carry the child with fewer leaves, push the other
  std::vector<int> stack;
  int cur = R, depth = 0, v = 0;
  for (;;) {
    PhsVisit &V = out.visit[v++];
    fill_child(kid(cur, 0), V.child[0]);
    fill_child(kid(cur, 1), V.child[1]);
    int t = p.map_id[mx(cur)];
    double a[3], b[3];
    double m_min = ms[cur];
    double m_max = cur == R ? sqrts : sqrts - m_tot + m_min;
    branch_constants(t, p.map_m[mx(cur)], p.map_w[mx(cur)], m_min, m_max, s, a, b);
    V.x_phi = x_ang[cur];
    V.x_ct = x_ang[cur] + 1;
    V.ct_class = ct_class_of(t);
    V.map_id = t;
    V.b0 = b[0];
    V.b1 = b[1];
    V.m = p.map_m[mx(cur)];
    V.self_m_min = m_min;
    V.self_m_max = m_max;
    V.self_root = cur == R;
    V.parent_root = cur != R && (kid(R, 0) == cur || kid(R, 1) == cur);
    // friends (extract_boost_origins, phs.cu:268-292): code 2^n_out pairs the branch with
    // the beam along -z, 2^(n_out+1) with the beam along +z; anything else is no friend
    const int fr = p.friends[ix(cur)];
    V.friend_sign = fr == (1 << p.n_out) ? -1 : fr == (1 << (p.n_out + 1)) ? 1 : 0;
    if (V.friend_sign && cur == R) {
      err = where + "the root branch cannot have a friend (its decay axis is the beam axis)";
      return PHS_ERR_TREE;
    }
    const bool i0 = internal(kid(cur, 0)), i1 = internal(kid(cur, 1));
    V.both_leaves = !i0 && !i1;
    V.push = V.carry = -1;
    if (i0 && i1) {
      int n0 = __builtin_popcount(kid(cur, 0)), n1 = __builtin_popcount(kid(cur, 1));
      V.carry = n0 <= n1 ? 0 : 1;
      V.push = 1 - V.carry;
      stack.push_back(kid(cur, V.push));
      depth = std::max(depth, (int)stack.size());
      cur = kid(cur, V.carry);
    } else if (i0 || i1) {
      V.carry = i0 ? 0 : 1;
      cur = kid(cur, V.carry);
    } else {
      if (stack.empty()) break;
      cur = stack.back();
      stack.pop_back();
    }
  }
  out.n_visits = v;
  if (depth > PHS_STACK_DEPTH) { err = where + "tree too deep for the visit stack"; return PHS_ERR_UNSUPPORTED; }
  info.stack_depth = depth;
  info.n_internal = v;

  // volume: constant at sqrts (phs_cpu.cpp:194-213), and its post-order program
  std::function<double(int)> vol = [&](int code) -> double {
    if (!internal(code)) return 1;
    double v1 = vol(kid(code, 0)), v2 = vol(kid(code, 1));
    if (code == R) return v1 * v2 / (4 * kTwoPi5);
    return v1 * v2 * sqrts * sqrts / (4 * kTwoPi2);
  };
  out.volume = vol(R);
  std::vector<int> entry(R + 1, -1);
  int ne = 0;
  std::function<void(int)> vpost = [&](int code) {
    if (!internal(code)) return;
    vpost(kid(code, 0));
    vpost(kid(code, 1));
    int e = ne++;
    entry[code] = e;
    out.vol_child[e][0] = (int8_t)entry[kid(code, 0)];
    out.vol_child[e][1] = (int8_t)entry[kid(code, 1)];
    out.vol_is_root[e] = code == R;
  };
  vpost(R);
  out.n_vol = ne;
  // momentum slots for the inverse map: leaves by output index, internals after them
  auto slot_of = [&](int code) -> int {
    if (internal(code)) return p.n_out + entry[code];
    int ld2 = 0, bb = code;
    while (bb > 1) { bb /= 2; ld2++; }
    return ld2;
  };
  for (int code = 1; code <= R; code++) {
    if (!internal(code) || entry[code] < 0) continue;
    out.comb[entry[code]][0] = (int8_t)slot_of(kid(code, 0));
    out.comb[entry[code]][1] = (int8_t)slot_of(kid(code, 1));
  }
  {
    // visits in program order: the code of each visited branch
    std::vector<int> st2;
    int cur2 = R;
    for (int v2 = 0; v2 < out.n_visits; v2++) {
      PhsVisit &V = out.visit[v2];
      V.slot[0] = (int8_t)slot_of(kid(cur2, 0));
      V.slot[1] = (int8_t)slot_of(kid(cur2, 1));
      if (V.push >= 0) st2.push_back(kid(cur2, V.push));
      if (V.carry >= 0) {
        cur2 = kid(cur2, V.carry);
      } else if (!st2.empty()) {
        cur2 = st2.back();
        st2.pop_back();
      }
    }
  }
  return PHS_OK;
}

static PhsFF split(double d) {
  PhsFF r;
  r.hi = (float)d;
  r.lo = (float)(d - (double)r.hi);
  return r;
}

static PhsFF split_ld(long double d) {
  PhsFF r;
  r.hi = (float)d;
  r.lo = (float)(d - (long double)r.hi);
  return r;
}

void channel_to_ff(const PhsChannel &in, PhsChannelFF &out) {
  memset(&out, 0, sizeof(out));
  out.n_out = in.n_out;
  out.n_visits = in.n_visits;
  out.lab = in.lab;
  out.sqrts = split(in.sqrts);
  out.s = split(in.sqrts * in.sqrts);
  out.lab_bg = split(in.lab_bg);
  out.lab_gamma = split(in.lab_gamma);
  out.m_tot = split(in.m_tot);
  out.volume = in.volume;
  for (int v = 0; v < in.n_visits; v++) {
    const PhsVisit &V = in.visit[v];
    PhsVisitFF &F = out.visit[v];
    for (int j = 0; j < 2; j++) {
      const PhsChild &C = V.child[j];
      PhsChildFF &G = F.child[j];
      G.internal = C.internal;
      G.out_index = C.out_index;
      G.map_id = C.map_id;
      G.x_msq = C.x_msq;
      G.msq_leaf = split(C.msq_leaf);
      G.m_leaf = split(C.m_leaf);
      G.m2 = split(C.m * C.m);
      G.mw = split(C.m * C.w);
      G.a0 = split(C.a0);
      G.a1 = split(C.map_id == PHS_MAP_SCHANNEL ? C.a1 - C.a0 : C.a1);
      G.a2 = split(C.map_id == PHS_MAP_NO ? (C.msq_max - C.msq_min) / (in.sqrts * in.sqrts) : C.a2);
      G.msq_min = split(C.msq_min);
      G.msq_max = split(C.msq_max);
      G.m_max = split(C.m_max);
      G.m_min = split(C.m_min);
      if (C.map_id == PHS_MAP_SCHANNEL) G.inv_mw = split_ld(1.0L / ((long double)C.m * (long double)C.w));
      if (C.map_id == PHS_MAP_SCHANNEL) {
        const long double half_pi = 1.57079632679489661923132169163975144L;
        G.u0 = split_ld(half_pi + (long double)C.a0);
        G.u1 = split_ld(half_pi - (long double)C.a1);
      }
      if (C.internal && (C.map_id == PHS_MAP_STEP_E || C.map_id == PHS_MAP_STEP_H)) out.exact_only = 1;
    }
    if (V.friend_sign) out.exact_only = 1;
    F.x_phi = V.x_phi;
    F.x_ct = V.x_ct;
    F.ct_class = V.ct_class;
    F.carry = V.carry;
    F.push = V.push;
    F.self_root = V.self_root;
    F.both_leaves = V.both_leaves;
    F.parent_root = V.parent_root;
    F.b0 = split(V.b0);
    F.b1 = split(V.b1);
    F.self_m_max = split(V.self_m_max);
    PhsTestVisit &P = out.test[v];
    for (int j = 0; j < 2; j++) {
      const PhsChildFF &G = F.child[j];
      PhsTestChild &Q = P.child[j];
      switch (G.map_id) {
        case PHS_MAP_NO:
          Q.c[0] = G.msq_min.hi;
          Q.c[1] = G.msq_max.hi;
          break;
        case PHS_MAP_SCHANNEL:
          Q.c[0] = G.a0.hi;
          Q.c[1] = G.a1.hi;
          Q.c[2] = G.u0.hi;
          Q.c[3] = G.u1.hi;
          Q.c[4] = G.m2.hi;
          Q.c[5] = G.mw.hi;
          break;
        default:
          Q.c[0] = G.a0.hi;
          Q.c[1] = G.a1.hi;
          Q.c[2] = G.msq_min.hi;
          Q.c[3] = G.msq_max.hi;
      }
      Q.m = G.internal ? G.m_max.hi : G.m_leaf.hi;
      Q.code = (G.internal ? 1 : 0) | (G.map_id & 127) << 1 | (G.x_msq & 255) << 8;
    }
    P.child[0].code |= (V.push + 1) << 16 | (V.carry + 1) << 18 | (V.self_root ? 1 : 0) << 20;
  }
}

// Which visit holds each internal child, and where a pop enters a visit: the adjoint walks
// the visits backwards and, at a visit entered by a pop, resumes with the frame that the
// forward walk saved just before the pop.
void channel_adjoint(const PhsChannel &in, PhsAdjChannel &out) {
  memset(&out, 0, sizeof(out));
  std::vector<std::pair<int, int>> pushed;  // (visit, child) awaiting their visit
  int pops = 0;
  for (int v = 0; v < in.n_visits; v++) {
    const PhsVisit &V = in.visit[v];
    PhsAdjVisit &A = out.visit[v];
    A.child_visit[0] = A.child_visit[1] = -1;
    for (int j = 0; j < 2; j++) {
      const PhsChild &C = V.child[j];
      if (C.internal && C.map_id == PHS_MAP_SCHANNEL) {
        const double m2 = C.m * C.m, mw = C.m * C.w;
        const double u0 = (C.msq_min - m2) / mw, u1 = (C.msq_max - m2) / mw;
        A.child[j].da0_dm = -(C.msq_min + m2) / (m2 * C.w) / (1 + u0 * u0);
        A.child[j].da1_dm = -(C.msq_max + m2) / (m2 * C.w) / (1 + u1 * u1);
        A.child[j].da0_dw = -u0 / (C.w * (1 + u0 * u0));
        A.child[j].da1_dw = -u1 / (C.w * (1 + u1 * u1));
        const double da = C.a1 - C.a0;
        A.child[j].dlf_dm0 = (A.child[j].da1_dm - A.child[j].da0_dm) / da + 1.0 / C.m;
        A.child[j].dlf_dw0 = (A.child[j].da1_dw - A.child[j].da0_dw) / da + 1.0 / C.w;
      }
    }
    if (V.carry >= 0) A.child_visit[V.carry] = v + 1;
    if (V.push >= 0) pushed.push_back({v, V.push});
    if (V.carry < 0 && v + 1 < in.n_visits) {
      const auto vj = pushed.back();
      pushed.pop_back();
      out.visit[vj.first].child_visit[vj.second] = v + 1;
      out.visit[v + 1].entered_by_pop = 1;
      out.visit[v + 1].pop_slot = pops++;
    }
  }
  out.n_pops = pops;
}

}  // namespace phs
