// phs_host.h -- host-side process model and tree compiler (internal to libgpuphs).
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "phs_program.h"

namespace phs {

// One Whizard process: n_channels trees over n_in + n_out external particles, with the
// tables the reference's C-ABI takes (whizard_gpu_phs.cpp:12-87).
struct Process {
  int n_in = 0, n_out = 0, n_channels = 0, n_x = 0;
  int n_prt = 0, n_prt_out = 0;
  std::vector<int> d1, d2, has_children, friends;  // [c * n_prt + code - 1]
  std::vector<int> map_id;                          // [c * n_prt_out + code - 1]
  std::vector<double> map_m, map_w;                 // [c * n_prt_out + code - 1]
  std::vector<double> flv_m, flv_w;                 // [n_in + n_out]
};

// Per-channel facts the compiler derives (exposed for inspection and tests).
struct ChannelInfo {
  int stack_depth = 0;  // pushes needed by the visit order
  int n_internal = 0;
};

// Validates channel c of p and compiles it at sqrt(s) = sqrts into out.  Returns 0 or a
// negative status with a message in err.
int compile_channel(const Process &p, int c, double sqrts, PhsChannel &out, ChannelInfo &info,
                    std::string &err);

// Float-float copy of a compiled channel (same visit order and x indices).
void channel_to_ff(const PhsChannel &in, PhsChannelFF &out);

// Reverse-walk tables of a compiled channel for the adjoint kernel.
void channel_adjoint(const PhsChannel &in, PhsAdjChannel &out);

// Validates the sizes and tables of a whole process (no sqrt(s) needed).
int validate_process(const Process &p, std::string &err);

}  // namespace phs
