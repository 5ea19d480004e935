// phs_program.h -- the compiled form of one channel tree, shared by host and device.
//
// The host tree compiler (phs_compile.cpp) turns a Whizard channel (daughter codes,
// mapping ids, masses, widths) into a flat "visit program" that the fused kernel walks
// once per event, top-down, with no recursion and no per-branch arrays:
//
//   * one visit per internal branch (n_out - 1 visits, the root first);
//   * a visit of branch b receives b's frame matrix L0 (its parent's boost), b's msq,
//     mass and decay momentum, maps its internal children's msq from x, evaluates the
//     Kallen function and the kinematic ok test at b, builds b's rotation+boost L1,
//     forms L0*L1, and writes the momenta of its leaf children;
//   * the next visit continues with an internal child ("carry"), and a second internal
//     child is pushed on a per-thread stack of depth <= PHS_STACK_DEPTH (the smaller
//     subtree is carried first, so the depth is <= 2 for n_out <= 15).
//
// The inverse map (phs_inverse.cu) walks the same program: at each visit it recovers the
// visited branch's angles and its children's msq x from the event's momenta.
//
// x indices are static: the reference consumes x in a fixed order (msq x's of the
// non-root internal branches in post-order, then phi and cos(theta) per internal branch
// in pre-order; phs_cpu.cpp:174-234, 283-345), so the visit order is free.
#pragma once
#include <stdint.h>

#define PHS_MAX_OUT 12
#define PHS_MAX_VISITS (PHS_MAX_OUT - 1)
#define PHS_STACK_DEPTH 2

// Mapping ids (phs.h:8-17).
enum {
  PHS_MAP_NO = 0, PHS_MAP_SCHANNEL = 1, PHS_MAP_TCHANNEL = 2, PHS_MAP_UCHANNEL = 3,
  PHS_MAP_RADIATION = 4, PHS_MAP_COLLINEAR = 5, PHS_MAP_INFRARED = 6,
  PHS_MAP_STEP_E = 11, PHS_MAP_STEP_H = 12
};

// cos(theta) mapping classes (phs_cpu.cpp:112-146).
enum { PHS_CT_UNIFORM = 0, PHS_CT_COLLINEAR = 1 };

// One daughter of a visited branch.
struct PhsChild {
  int32_t internal;   // 0: outgoing particle (leaf); 1: internal branch
  int32_t out_index;  // leaf: output particle index j (Whizard code 2^j)
  int32_t map_id;     // internal: msq mapping id
  int32_t x_msq;      // internal: index of its msq x within the event's x row
  double msq_leaf;    // leaf: m^2 (flv mass squared, phs_cpu.cpp:541-547)
  double m_leaf;      // leaf: sqrt(m^2), correctly rounded
  double m, w;        // internal: mapping mass and width
  double a0, a1, a2;  // internal: msq mapping constants at the handle's sqrt(s)
  double msq_min, msq_max;  // internal: m_min^2, m_max^2 at the handle's sqrt(s)
  double m_max;       // internal: sqrt(s) - m_tot + m_min (the ok test's upper bound)
  double m_min;       // internal: sum of leaf masses below it (phs.cu:61-78)
  double msq0;        // internal Breit-Wigner: m^2
  double inv_mw;      //   1 / (m w)
  double inv_da;      //   1 / (a1 - a0) at the handle's sqrt(s) (the inverse map's divisors)
};

struct PhsVisit {
  PhsChild child[2];  // child[0] = daughters1 (+p_decay), child[1] = daughters2 (-p_decay)
  int32_t x_phi;      // index of the phi x
  int32_t x_ct;       // index of the cos(theta) x
  int32_t ct_class;   // PHS_CT_UNIFORM or PHS_CT_COLLINEAR
  int32_t map_id;     // the visited branch's own mapping id (selects the ct mapping)
  int32_t carry;      // child continued by the next visit (0/1), -1: next visit pops
  int32_t push;       // child pushed on the stack after this visit (0/1), -1: none
  double b0, b1;      // collinear cos(theta) constants at the handle's sqrt(s)
  double m;           // the visited branch's mapping mass (per-event b0 = m^2/s)
  double self_m_min;  // the visited branch's m_min (per-event m_max)
  double self_m_max;  // the visited branch's ok-test bound at the handle's sqrt(s)
  int32_t self_root;  // 1 for the root visit
  int32_t both_leaves;  // 1 when neither child is internal (only L columns 0,3 needed)
  int32_t friend_sign;  // 0, or the beam (+1: along +z, -1: along -z) that the visited
                        // branch's decay angles are measured from (phs.cu:853-910)
  int8_t slot[2];       // inverse map: momentum slot of each child (see PhsChannel::comb)
  int8_t parent_root;   // 1 when the visited branch is a daughter of the root: without a lab
                        // boost its parent frame is the root's rotation, rows
                        // (1,0,0,0), (0,*,*,*), (0,*,*,*), (0,*,0,*)
  int8_t pad1;
};

struct PhsChannel {
  int32_t n_out;
  int32_t n_visits;
  int32_t n_x_used;   // 3 n_out - 4
  int32_t n_vol;      // entries of the volume program
  double m_tot;       // sum of all outgoing masses
  double volume;      // channel volume at the handle's sqrt(s) (phs_cpu.cpp:194-213)
  double sqrts;       // uniform beams: sqrt(s) = 2 sqrt(E1 E2) the constants were made for
  double lab_bg;      // uniform beams: longitudinal lab boost (E1-E2)/(2 sqrt(E1 E2))
  double lab_gamma;   //   and its gamma (phs.cu:1286-1301)
  int32_t lab;        //   1 when E1 != E2
  int32_t pad0;
  PhsVisit visit[PHS_MAX_VISITS];
  // Volume program for per-event sqrt(s): post-order internal branches; for entry i,
  // vol_child[i][j] >= 0 is the entry index of an internal child, -1 a leaf (volume 1).
  int8_t vol_child[PHS_MAX_VISITS][2];
  int8_t vol_is_root[PHS_MAX_VISITS];
  // Momentum sums of the inverse map (_combine_particles, phs.cu:1262-1283): slots
  // 0..n_out-1 hold the outgoing momenta, slot n_out + i the i-th internal branch in
  // post-order (the volume program's order), = slot comb[i][0] + slot comb[i][1].
  int8_t comb[PHS_MAX_VISITS][2];
  int8_t pad[1];
};

// A contiguous run of events of one channel within a launch.
struct PhsSegment {
  int32_t channel;      // index into the launch's channel table
  int32_t n_out;
  int64_t ev_begin;     // global index of the first event (factor/volume/ok index)
  int64_t ev_count;
  int64_t x_base;       // element offset of the first event's x row
  int64_t p_base;       // element offset of the first event's momenta
  int64_t tile_begin;   // first warp tile of this segment (prefix sum)
  int32_t x_stride;     // x row length (>= n_x_used)
  int32_t factor_col;   // column added to the factor index (whizard: own channel)
  int64_t chunk_begin;  // first work chunk of this segment for the compacting FP64 kernel:
                        // chunks of PHS_CHUNK_TILES tiles never cross a segment boundary
};

#define PHS_CHUNK_TILES 8

// ------------------------------------------------------------------------------------
// Float-float form of a channel program, for the FP32-pipe kernel: every constant is a
// pair of floats hi + lo (about 48 bits).  Built on the host from PhsChannel.
struct PhsFF {
  float hi, lo;
};

struct PhsChildFF {
  int32_t internal, out_index, map_id, x_msq;
  PhsFF msq_leaf, m_leaf;
  PhsFF m2, mw;       // Breit-Wigner: m^2 and m*w
  PhsFF a0, a1, a2;   // mapping constants; Breit-Wigner keeps a1 - a0 in a1
  PhsFF msq_min, msq_max, m_max;
  PhsFF u0, u1;       // Breit-Wigner: pi/2 + a0 and pi/2 - a1 (z near -+pi/2 as cot)
  PhsFF m_min;        // internal: the sum of the leaf masses below it (per-event m_max)
  PhsFF inv_mw;       // Breit-Wigner: 1 / (m w) (per-event a1)
};

struct PhsVisitFF {
  PhsChildFF child[2];
  int32_t x_phi, x_ct, ct_class, carry, push, self_root, both_leaves;
  int32_t parent_root;  // as PhsVisit::parent_root
  PhsFF b0, b1, self_m_max;
};

// The FP32 pre-test's view of a visit (high parts only), four 16-byte loads.  Per child
// c[0..5] by mapping: none {msq_min, msq_max}; Breit-Wigner {a0, a1 - a0, pi/2 + a0,
// pi/2 - a1, m^2, m w}; exponential {a0, a1, msq_min, msq_max}; m = m_max (internal) or
// the leaf mass; code = internal | map_id << 1 | x_msq << 8, and child 0's code also holds
// push + 1 (bits 16-17), carry + 1 (bits 18-19) and self_root (bit 20).
struct PhsTestChild {
  float c[6];
  float m;
  int32_t code;
};
struct alignas(16) PhsTestVisit {
  PhsTestChild child[2];
};
struct PhsChannelFF {
  int32_t n_out, n_visits;
  int32_t exact_only;  // 1: STEP_E/STEP_H mappings or a friend boost: FP64 path
  int32_t lab;
  PhsFF sqrts, s, lab_bg, lab_gamma;
  PhsFF m_tot;        // the sum of all outgoing masses (per-event m_max)
  double volume;
  PhsVisitFF visit[PHS_MAX_VISITS];
  PhsTestVisit test[PHS_MAX_VISITS];
};

// ------------------------------------------------------------------------------------
// Reverse-walk tables of a channel, for the adjoint kernel (phs_adjoint.cu).
struct PhsAdjChild {
  double da0_dm, da0_dw, da1_dm, da1_dw;  // Breit-Wigner: derivatives of the atan bounds
  double dlf_dm0, dlf_dw0;  // the x-independent parts of dlog f/dm and dlog f/dw:
                            // (da1 - da0)/(a1 - a0) + 1/m (and 1/w)
};

struct PhsAdjVisit {
  int32_t child_visit[2];  // visit index where an internal child is the visited branch, -1: leaf
  int32_t entered_by_pop;  // 1: this visit follows a pop (its predecessor ends a subtree)
  int32_t pop_slot;        // frame slot holding the predecessor's frame (entered_by_pop)
  PhsAdjChild child[2];
};

struct PhsAdjChannel {
  int32_t n_pops;
  int32_t pad;
  PhsAdjVisit visit[PHS_MAX_VISITS];
};
