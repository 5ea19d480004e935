// phs_device.h -- launch interface of the device kernels (host side of phs_kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "phs_check.h"
#include "phs_program.h"

#define PHS_INLINE_SEGS 64

// One forward launch over a list of segments (runs of events of one channel).
struct PhsLaunch {
  const PhsChannel *channels;  // device, per channel
  const PhsChannelFF *channels_ff;  // device, float-float copies (FP32-pair kernel only)
  const PhsSegment *segments;  // device table, used when n_segments > PHS_INLINE_SEGS
  PhsSegment seg_inline[PHS_INLINE_SEGS];  // sorted by tile_begin
  int32_t n_segments;
  int32_t stack_depth;         // max push depth over the launched channels
  int64_t n_tiles;             // total 32-event warp tiles
  int64_t n_chunks;            // total work chunks (PhsSegment::chunk_begin)
  const double *x;
  double *p;
  double *factor;
  double *volume;
  uint8_t *ok;
  int64_t factor_stride;       // factor index = event * factor_stride + segment.factor_col
  const double *E1;            // per-event beams (both non-null) or null
  const double *E2;
  unsigned long long *work;    // compacting kernels: chunk counter, zeroed before the
                               // launch (warps claim chunks dynamically); null: static
  // FP32-pair launches: the events queued for the exact FP64 path, per segment as the
  // pre-test survivors are (count zeroed before the launch; local indices from
  // tile_begin * 32 on; the dense claim numbering [n_segments + 1]; the exact launch's
  // claim counter, zeroed before the launch)
  unsigned int *exact_count;
  int32_t *exact_queue;
  int64_t *exact_tile;
  unsigned long long *exact_work;
  // FP32-pair split form: per segment, the events that passed the pre-test (count, zeroed
  // before the launch), the walk's dense claim numbering ([n_segments + 1]) and their local
  // indices (segment s from tile_begin * 32 on; n_tiles * 32 entries).
  unsigned int *pass_count;
  int64_t *pass_tile;
  int32_t *pass_queue;
  // extents for the checked build's bounds checks (phs_check.h): elements of x and p,
  // entries of volume and ok (factor: ev_len * factor_stride), channel programs
  int64_t x_len, p_len, ev_len;
  int32_t n_programs;
};

// Block size and resident blocks per SM of the forward kernel.
#define PHS_FWD_BLOCK 128

// Variants, each a form at one block shape (threads per block x resident blocks per SM):
// 0: one pass, 128 x 4; 1, 2: compacting (pass A tests every event and writes the
// failures, pass B computes the passing events densely), 128 x 4 and 128 x 3; 3, 4: one
// pass, 256 x 2 and 64 x 8; 5-8: split (the FP32 pre-test of phs_launch_pretest, then the
// FP64 walk over its survivors; uniform beams only, needs the a.pass_* buffers and a.work
// zeroed), 128 x 4, 128 x 3, 256 x 2, 64 x 8.  PHS_F64_VARIANTS of them; the first
// PHS_F64_VARIANTS_PER_EVENT serve per-event beams.
#define PHS_F64_VARIANTS 9
#define PHS_F64_VARIANTS_PER_EVENT 5
cudaError_t phs_launch_forward_f64(const PhsLaunch &a, int n_blocks, int variant,
                                   cudaStream_t stream);
int phs_forward_blocks_per_sm(int stack_depth, bool per_event, int variant);
int phs_forward_block_size(int variant);
size_t phs_forward_smem_bytes(int stack_depth, int block = PHS_FWD_BLOCK);

// Philox4x32-10 uniform doubles for events [first_event, first_event + n_events) of the
// stream `seed`, row length n_x (the layout is documented in gpu_phs_gb300/philox.py).
cudaError_t phs_launch_philox(double *x, int64_t n_events, int32_t n_x, uint64_t seed,
                              int64_t first_event, cudaStream_t stream);

// FMA-throughput probe (8 independent chains per thread, `iters` rounds): 16 * iters flops
// per thread.  Used to measure the FP64 and FP32 peaks the roofline is quoted against.
cudaError_t phs_launch_fma_rate(void *out, int fp64, int blocks, int threads, int iters,
                                cudaStream_t stream);

// Whizard's sparse momentum layout (phs.cu:1364-1373): out[event][n_prt][4], slot code - 1
// for every Whizard code up to n_prt = 2^(n_in + n_out) - 1.  Outgoing particles (codes
// 2^k) hold their lab momenta; every code that is an internal branch of some channel
// (bit code of `internal`) holds the sum of its particles' momenta in the centre-of-mass
// frame, as the reference's buffer ends up after its inverse-map loop (phs.cu:1262-1283;
// its lab boost touches the outgoing codes only, phs.cu:1286-1301); every other slot is 0.
#define PHS_SPARSE_MAX_OUT 12
struct PhsSparseLaunch {
  const double *p;         // [event][n_out][4] lab momenta
  const double *E1, *E2;   // per-event beams, or null: e1, e2 for every event
  double e1, e2;
  double *out;
  int64_t n_events;
  int32_t n_out, n_prt;
  uint32_t internal[(1 << PHS_SPARSE_MAX_OUT) / 32];
};
cudaError_t phs_launch_whizard_sparse(const PhsSparseLaunch &a, cudaStream_t stream);

// Forward launch whose channel programs and segment table are copied into a file-scope
// device array of phs_kernels.cu (no device allocation; see there).  At most
// PHS_NOALLOC_MAX_CHANNELS channels and as many segments; returns cudaErrorInvalidValue
// beyond that.  The first call on a device resolves the array's device address.
#define PHS_NOALLOC_MAX_CHANNELS 256
cudaError_t phs_launch_forward_f64_noalloc(PhsLaunch a, const PhsChannel *channels,
                                           int n_channels, const PhsSegment *segments,
                                           int n_segments, int n_blocks, cudaStream_t stream);
size_t phs_noalloc_scratch_bytes();

// Forward launch on the FP32 pipe (float-float arithmetic), FP64 only for events within
// 1e-5 of a kinematic limit, which it queues for phs_launch_forward_exact (phs_kernels_ff.cu).
// Needs a.channels, a.channels_ff and the a.exact_* buffers (count and work zeroed);
// uniform beams only.
// variant bit 0: registers for 4 (1) or 3 (0) resident blocks per SM; bit 1: the
// compacting two-pass form; variants 4 and 5 (bit 0 as before): the split form, the FP32
// pre-test as a kernel of its own, then the float-float walk over the events it passed
// (needs a.pass_count zeroed, a.pass_tile, a.pass_queue).  PHS_FF_VARIANTS in all.
#define PHS_FF_VARIANTS 6
cudaError_t phs_launch_forward_ff(const PhsLaunch &a, int n_blocks, int variant, cudaStream_t stream);
int phs_forward_ff_blocks_per_sm(int stack_depth, int variant);
size_t phs_forward_ff_smem_bytes(int stack_depth);
// The FP32 pre-test of the split forms (phs_kernels_ff.cu): writes the outputs of the
// events whose kinematic test fails for certain, and queues the others per segment in
// a.pass_queue / a.pass_count (zeroed before) with the dense claim numbering a.pass_tile.
// Uniform beams only (it reads the float-float programs' constants).
cudaError_t phs_launch_pretest(const PhsLaunch &a, cudaStream_t stream);
// Dense claim numbering of per-segment queues: tile[s] = sum over the segments before s of
// ceil(count / 32), tile[n] their total (one block).
cudaError_t phs_launch_count_scan(const unsigned int *count, int64_t *tile, int n,
                                  cudaStream_t stream);
// The exact FP64 path over the events an FP32-pair launch queued (a.exact_queue): the scan
// of their counts, then the FP64 walk, 32 events of one segment per warp claim.
cudaError_t phs_launch_forward_exact(const PhsLaunch &a, int n_blocks, cudaStream_t stream);

// Reverse-mode derivatives (phs_adjoint.cu): xbar [event][x stride] and thbar
// [event][th_stride] (d/dm, d/dGamma per Breit-Wigner branch, at 2 * its msq x index).
// store == null: the recompute form (no scratch); else the stored-matrix form, with
// store[max_visits * 16 * store_events] doubles (store_events >= the launch's events).
cudaError_t phs_launch_adjoint(const PhsLaunch &a, const PhsAdjChannel *adj, const double *pbar,
                               const double *jbar, double *xbar, double *thbar, int th_stride,
                               int max_visits, int max_pops, bool friends, int n_blocks,
                               cudaStream_t stream, double *store = nullptr,
                               int64_t store_events = 0);
int phs_adjoint_blocks_per_sm(int max_visits, int max_pops, int stack_depth, bool friends,
                              bool stored = false);
void phs_adjoint_sizes(int max_visits, int max_pops, int stack_depth, bool friends, int *state0,
                       int *ang0, int *der0, int *pop0, int *stack0, int *trig0, int *fr0,
                       size_t *smem);
#define PHS_ADJ_BLOCK_HOST 64

// Inverse map (phs_inverse.cu): for every event and every channel, the x row and factor
// that channel assigns to the event's momenta.  Threads per block (and events per tile and
// per walk): with ~84 doubles of shared memory per thread, 64-thread blocks keep 5 blocks
// (10 warps) resident per SM where 128-thread blocks keep 2 (8 warps).
#define PHS_INV_BLOCK 64
struct PhsInvLaunch {
  const PhsChannel *channels;  // device, per channel (uniform-beam constants)
  const int64_t *ch_begin;     // device, [n_channels]: first event of each generating channel
  const double *p;             // [n][n_out][4] lab momenta
  const uint8_t *ok;           // [n] or null (all valid)
  const double *E1, *E2;       // per-event beams, or null (the programs' beams)
  const double *x_own;         // [n][n_x]: the generating channel's x (copied), or null
  const double *factor_own;    // [n]: the generating channel's factor, or null
  double *all_factors;         // [n][n_channels]
  double *x_out;               // [n_channels][x_ch_stride][n_x], events 0 .. n - 1 of each
  // channels of equal tree shape (the geometry of the inverse map is the same for them):
  // group g is group_order[group_begin[g] .. group_begin[g + 1]), each channel once
  const int32_t *group_order;
  const int32_t *group_begin;
  const uint64_t *group_reuse;  // [n_channels] by group_order position: mappings equal to the
                                // previous channel's (bit 3 visit + 0/1 daughter msq, + 2 ct);
                                // null: no reuse (and no shared memory for it)
  int32_t n_groups;
  // this launch inverts the channels at group_order positions [order_lo, order_hi) (all:
  // 0, n_channels); write_fixed: it also writes every channel's outputs that need no
  // arithmetic (own rows, x padding, ok = false events), which one launch of a split set does
  int32_t order_lo, order_hi, write_fixed;
  int64_t n_events;
  int64_t x_ch_stride;         // rows per channel in x_out (n_events, or more for a launch
                               // over a range of the events of a longer array)
  int32_t n_channels, n_out, n_x, stack_depth, max_visits;
  int32_t lab;                 // uniform beams: 1 when E1 != E2 (the programs' lab boost)
};
cudaError_t phs_launch_inverse(const PhsInvLaunch &a, int n_blocks, cudaStream_t stream);
// cache: the per-visit mapping results that channels of a shape reuse (a.group_reuse set);
// phs_inverse_fits_cache tells whether the block's shared memory holds them.  lab_rows:
// uniform beams without a lab boost, where the kernel reads the outgoing momenta from p
// instead of staging them in shared memory (4 n_out doubles less per thread).
int phs_inverse_blocks_per_sm(int n_out, int stack_depth, int max_visits, bool per_event,
                              bool cache, bool lab_rows);
size_t phs_inverse_smem_bytes(int n_out, int stack_depth, int max_visits, bool cache,
                              bool lab_rows);
bool phs_inverse_fits_cache(int n_out, int stack_depth, int max_visits);

// Per-channel x grid of the warm-up (phs_grid.cu): weights [n_channels][n_x][PHS_GRID_BINS].
#define PHS_GRID_BINS 10
// x holds the Philox uniforms on entry and the grid-distributed x on return.
cudaError_t phs_launch_grid_sample(double *x, int64_t n_events, int n_x, const int64_t *ch_begin,
                                   int n_channels, const double *weights, int sm_count,
                                   cudaStream_t stream);
cudaError_t phs_launch_grid_update(const double *x, const uint8_t *ok, int64_t n_events, int n_x,
                                   const int64_t *ch_begin, int n_channels,
                                   unsigned long long *bins, unsigned long long *n_ok,
                                   double *weights, int sm_count, cudaStream_t stream);
