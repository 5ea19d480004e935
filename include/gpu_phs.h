/*
 * gpu_phs.h -- C ABI of libgpuphs, the GB300 (sm_103a) phase-space generator.
 *
 * Two layers, both plain C (pointers and sizes, no C++ or framework types):
 *
 *  1. The Whizard binding: the same 14 symbols, signatures and by-reference argument
 *     conventions as the reference's C-ABI (whizard_gpu_phs.cpp:12-249), so the reference's
 *     Fortran module gpu_phs_whizard_interface.f90 links against this library unchanged.
 *     These keep the reference's void returns; failures are logged to stderr and kept for
 *     phs_last_error().
 *
 *  2. A handle API (phs_*) with status codes, device-pointer and host-pointer entry points,
 *     per-event beams, and multi-process batches.  The Whizard binding is built on it.
 *
 * Data layouts (identical to the reference, phs.cu:1564-1602):
 *   x        [n_events][n_x]            doubles in [0,1), event-major
 *   p        [n_events][n_out][4]       (E, px, py, pz) of the outgoing particles, particle j
 *                                       is the leaf with Whizard code 2^j
 *   factors  [n_events]                 phase-space Jacobian of the event's channel
 *   volumes  [n_events]
 *   oks      [n_events]                 1 byte each (C bool)
 * Events are grouped by channel: channel_counts[c] consecutive events belong to channel c.
 * For ok = 0 events, p and factor are 0 and volume is the channel volume.
 *
 * Tree tables (as whizard_gpu_phs.cpp:57-87 and the .ref files, file_input.cpp:183-250):
 *   daughters1/daughters2/has_children/friends  [n_channels][2^(n_in+n_out)-1], indexed by
 *       Whizard code - 1, holding daughter codes (0 = none)
 *   map_ids/map_masses/map_widths               [n_channels][2^n_out-1], by code - 1
 *   flv_masses/flv_widths                       [n_in + n_out], incoming first
 */
#ifndef GPU_PHS_H
#define GPU_PHS_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------- status codes */
#define PHS_OK 0
#define PHS_ERR_INVALID_ARG (-1) /* null pointer, bad size, counts not summing to n_events */
#define PHS_ERR_TREE (-2)        /* daughters do not form a binary tree over the outgoing codes */
#define PHS_ERR_MAPPING (-3)     /* mapping id without an implementation (e.g. 99 ONSHELL) */
#define PHS_ERR_CUDA (-4)        /* a CUDA runtime call failed (message has the CUDA error) */
#define PHS_ERR_STATE (-5)       /* call out of order (e.g. generate before beams are set) */
#define PHS_ERR_ALLOC (-6)       /* device or host allocation failed */
#define PHS_ERR_UNSUPPORTED (-7) /* n_out above PHS_MAX_OUT_API or feature not built */

#define PHS_MAX_OUT_API 12

/* Arithmetic of the forward kernel (phs_process_set_precision / phs_batch_set_precision). */
#define PHS_PRECISION_F64 0   /* IEEE FP64 throughout (default) */
#define PHS_PRECISION_F32X2 1 /* float-float pairs on the FP32 pipe (~48 bits); events within
                                 1e-5 of a kinematic limit are recomputed in FP64, so ok flags
                                 stay bit-exact */

typedef struct phs_process *phs_process_t;
typedef struct phs_batch *phs_batch_t;

/* Message of the last failure on the calling thread ("" if none). */
const char *phs_last_error(void);
const char *phs_version(void);

/* Device memory of the library's own buffers (channel programs, segment tables, work
 * queues, the host path's chunk buffers, the stored-matrix adjoint's frames): by default
 * cudaMalloc and cudaFree.  A caller that owns the device heap through an allocator of its
 * own (a pool, an arena, a framework's caching allocator) routes them through it: alloc
 * sets *ptr to at least `bytes` of device memory of the current device, 256-byte aligned,
 * and returns 0, or returns non-zero (the library call then fails with PHS_ERR_ALLOC and
 * the size in its message); free takes back a pointer alloc gave.  Before handing a buffer
 * back the library synchronizes the device, as cudaFree does.  Both NULL restore the
 * default; a buffer is always freed by the allocator that made it.  Process-wide; the
 * library calls the functions from the thread of the API call that needs the buffer.
 * Returns PHS_ERR_INVALID_ARG if only one of the two is given.  No counterpart in the
 * reference, which allocates and frees its device memory inside every generate call
 * (phs.cu:1338-1426, 1604-1635). */
/* The bounds-checked build.  libgpuphs_checked.so is this library compiled with
 * -DPHS_CHECKED: every index its kernels compute from run-time data (programs, segment
 * tables, queues, event rows, stack depths) is compared with the extent of the array it
 * addresses before the access; an index out of range is not used (a read gives 0, a write
 * is dropped), and its site is recorded.  phs_check_status waits for the device, returns
 * the sites recorded since its last call as a bit mask (bit numbers: PhsCheckSite in the
 * library's phs_check.h: 0 channel, 1 x, 2 momenta, 3 event arrays, 4 frame stack, 5 visit
 * count, 6 queue slot, 7 segment, 8 adjoint arrays, 9 stored frames, 10 inverse outputs,
 * 11 inverse slots and queues, 12 grid) and the first offending index, and clears them.
 * In libgpuphs.so the checks are not compiled in: phs_is_checked_build() returns 0 and
 * phs_check_status PHS_ERR_UNSUPPORTED.  No counterpart in the reference. */
int phs_is_checked_build(void);
int phs_check_status(uint64_t *sites, int64_t *first_index);

typedef int (*phs_device_alloc_fn)(void **ptr, size_t bytes, void *user);
typedef void (*phs_device_free_fn)(void *ptr, void *user);
int phs_set_device_allocator(phs_device_alloc_fn alloc, phs_device_free_fn free, void *user);

/* ------------------------------------------------------------------ handle API: process */

/* Validates and stores a process.  Replaces the reference's global set-up sequence
 * c_whizard_set_particle_structure / set_flavors / init_mappings / fill_mapping /
 * init_tree_structures / fill_tree_structure / init_gpu_phs (whizard_gpu_phs.cpp:12-108,
 * init_phs_gpu phs.cu:327-509).  friends and flv_widths may be NULL.  The device is the
 * current CUDA device at creation; all later calls on the handle must use it. */
int phs_process_create(phs_process_t *out, int n_in, int n_out, int n_channels, int n_x,
                       const int *daughters1, const int *daughters2, const int *has_children,
                       const int *friends, const int *map_ids, const double *map_masses,
                       const double *map_widths, const double *flv_masses,
                       const double *flv_widths);
int phs_process_destroy(phs_process_t proc);

/* Uniform beam energies for all events: sqrt(s) = 2 sqrt(E1 E2) (phs.cu:1313-1317).  Compiles
 * the channel programs with the mapping constants at this sqrt(s) (init_mapping_constants_cpu,
 * phs_cpu.cpp:452-531) and uploads them.  E1 != E2 adds the longitudinal lab boost
 * (phs.cu:1286-1301). */
int phs_process_set_beams(phs_process_t proc, double E1, double E2);

/* Arithmetic of the uniform-beam generate calls (phs_generate_device/_host and batches built
 * afterwards keep their own setting): PHS_PRECISION_F64 or PHS_PRECISION_F32X2.  With
 * per-event beams (phs_generate_beams_device) F32X2 evaluates the constants that depend on
 * sqrt(s) per event in FP64 and walks in float-float, or runs the FP64 compacting kernel
 * where the autotuner finds that faster (few events passing).  No counterpart in the
 * reference (FP64 only). */
int phs_process_set_precision(phs_process_t proc, int precision);

/* The autotuned kernel variants of the handle's uniform-beam launches, or -1 before the
 * first launch of at least 2^18 events (outside stream capture) has timed them.  FP32 pair
 * (ff_variant): 0-3: bit 0 register budget for 4 (1) or 3 (0) resident blocks per SM, bit 1
 * the compacting two-pass form; 4 and 5: the split form (an FP32 pre-test kernel, then the
 * float-float walk over the events it passed) with 3 or 4 blocks.  FP64 (f64_variant), each
 * at one block shape (threads per block x resident blocks per SM): 0 one pass 128 x 4; 1, 2
 * compacting 128 x 4, 128 x 3; 3, 4 one pass 256 x 2, 64 x 8; 5-8 split (the FP32 pre-test,
 * then the FP64 walk) 128 x 4, 128 x 3, 256 x 2, 64 x 8 (per-event beams run 5-8 as 1-4).  The
 * compacting and split forms test every event first and compute only the passing ones,
 * densely; they win where many events fail the kinematic test.  Variants compute identical
 * bits.  Either pointer may be NULL. */
int phs_process_tuning(phs_process_t proc, int *ff_variant, int *f64_variant);

/* Pins the kernel variants (values as phs_process_tuning reports; -1 re-enables tuning), for
 * reproducible timings or to skip the tuning launches. */
int phs_process_set_variants(phs_process_t proc, int ff_variant, int f64_variant);

/* Sizes: any pointer may be NULL. */
int phs_process_info(phs_process_t proc, int *n_in, int *n_out, int *n_channels, int *n_x,
                     int *max_stack_depth);

/* Forward generation on device pointers, stream-ordered on `stream` (a cudaStream_t, NULL =
 * legacy default stream).  Up to 64 channels with events travel in the kernel parameters;
 * beyond that a per-handle device table is (re)uploaded when the counts change.  Replaces
 * gen_phs_from_x_gpu (phs.cu:1333-1636) without its host copies and repack. */
int phs_generate_device(phs_process_t proc, int64_t n_events, const int64_t *channel_counts,
                        const double *x, double *p, double *factors, double *volumes,
                        uint8_t *oks, void *stream);

/* As phs_generate_device with per-event beam energies E1[n_events], E2[n_events] (device):
 * mapping constants are evaluated per event and the lab boost applied where E1 != E2, as the
 * reference GPU path does per event (mappings_gpu.hpp:23-99, phs.cu:1286-1301). */
int phs_generate_beams_device(phs_process_t proc, int64_t n_events, const int64_t *channel_counts,
                              const double *E1, const double *E2, const double *x, double *p,
                              double *factors, double *volumes, uint8_t *oks, void *stream);

/* Forward generation for callers that cannot allocate device memory (a host that owns the
 * device heap through its own allocator, a sandbox or plug-in host that denies cudaMalloc,
 * or a loop that must not pay for the device-wide synchronisation cudaMalloc/cudaFree
 * imply).  Uniform beams E1, E2 given here (no phs_process_set_beams needed).  It always
 * runs the plain FP64 one-pass kernel (128 threads x 4 blocks per SM): the precision and
 * the kernel variants set on the handle do not apply; its outputs equal phs_generate_device's
 * FP64 outputs bit for bit.  It allocates nothing: the channel programs, compiled on the
 * host at every call, and the event segments go into one static device array of the
 * library, so the process may have at most 256 channels (PHS_ERR_UNSUPPORTED beyond).  Those
 * uploads come from pageable host memory, so the call may block the host until they are
 * staged and may synchronise with `stream`.  The first call on a device resolves that
 * array's address; make it before any stream capture.  A call on a stream that is being
 * captured is refused (PHS_ERR_UNSUPPORTED) before anything is enqueued, since the uploads
 * read host memory that is released when the call returns.  All calls share the array,
 * so calls that overlap on the GPU race.  No counterpart in the reference. */
int phs_generate_device_noalloc(phs_process_t proc, double E1, double E2, int64_t n_events,
                                const int64_t *channel_counts, const double *x, double *p,
                                double *factors, double *volumes, uint8_t *oks, void *stream);

/* Reverse-mode derivatives (FP64, uniform beams) of the forward map on device pointers.
 * Given cotangents pbar [n_events][n_out][4] of the momenta and jbar [n_events] of the
 * log-Jacobian log(factor) (jbar may be NULL), writes
 *   xbar  [n_events][n_x]            sum pbar . dp/dx + jbar dlog(factor)/dx
 *   thbar [n_events][n_out - 2][2]   the same for d/dm and d/dGamma of the Breit-Wigner
 *                                    branch whose msq x index is the middle index (0 else).
 * ok = 0 events get zeros.  The boost chain is recomputed backwards from the last frame;
 * no per-branch matrices are stored (friend visits keep their 3-vector rotation axis).  All
 * trees the forward map takes, friend boosts included.  No counterpart in the reference
 * (forward only). */
int phs_adjoint_device(phs_process_t proc, int64_t n_events, const int64_t *channel_counts,
                       const double *x, const double *pbar, const double *jbar, double *xbar,
                       double *thbar, void *stream);

/* How phs_adjoint_device gets each visit's parent frame in its reverse walk.
 * PHS_ADJOINT_RECOMPUTE (default): recovered from the child's frame with the inverse
 * rotation+boost; no device memory beyond the outputs.  PHS_ADJOINT_STORED: the
 * stored-matrix form the reference's device path uses for its boost chain (Ld, 16 doubles
 * per boost and event, phs.cu:1421-1422): the forward pass writes the frames to a device
 * buffer the handle keeps (n_events x max visits x 128 bytes, grown as needed, released
 * when the mode goes back to RECOMPUTE), the reverse walk reads them back.  Same derivatives
 * up to rounding; kept for the memory and time comparison. */
#define PHS_ADJOINT_RECOMPUTE 0
#define PHS_ADJOINT_STORED 1
int phs_process_set_adjoint_storage(phs_process_t proc, int storage);

/* Inverse map on device pointers: for events grouped by generating channel
 * (channel_counts), with lab momenta p [n_events][n_out][4] (16-byte aligned), writes for
 * EVERY channel c the x row and factor that channel assigns to the same momenta:
 *   all_factors [n_events][n_channels]        (factors[n_channels * i + c], phs.cu:1580-1583)
 *   x_out       [n_channels][n_events][n_x]   (x_out[n_x * n_events * c + n_x * i + k], :1585)
 * Replaces the do_inverse_mapping pass of gen_phs_from_x_gpu (phs.cu:1499-1554 with
 * _apply_msq_inv 626-675, the boost inversion 924-1244 and mappings_gpu.hpp:15-219).
 * E1/E2 (device, both or neither): per-event beams; NULL uses the handle's beams.  oks may
 * be NULL (all events valid); events with ok = 0 get factor 0 and x 0 in the other channels.
 * x_own [n_events][n_x] and factor_own [n_events] (may be NULL): the generating channel's
 * row is copied from them, as the reference does (_move_x, _move_factors phs.cu:203-232);
 * with x_own NULL it is inverted like the others.  x entries past 3 n_out - 4 are copied
 * from x_own (0 without).  FP64. */
int phs_inverse_device(phs_process_t proc, int64_t n_events, const int64_t *channel_counts,
                       const double *E1, const double *E2, const double *p, const uint8_t *oks,
                       const double *x_own, const double *factor_own, double *all_factors,
                       double *x_out, void *stream);

/* Host pointers in and out (pinned memory is fastest); copies run chunk-pipelined with the
 * kernel.  Synchronous. */
int phs_generate_host(phs_process_t proc, int64_t n_events, const int64_t *channel_counts,
                      const double *x, double *p, double *factors, double *volumes,
                      uint8_t *oks);

/* -------------------------------------------------------------------- handle API: batches */

/* Many processes (uneven n_out and n_x) generated in one persistent launch.  Batch channel k
 * enumerates the channels of procs[0], then procs[1], ...  Every process must have beams. */
int phs_batch_create(phs_batch_t *out, int n_procs, const phs_process_t *procs);
int phs_batch_destroy(phs_batch_t batch);
int phs_batch_info(phs_batch_t batch, int *n_channels, int64_t *x_stride_sum, int *max_n_out);

/* Events grouped by batch channel, counts[n_channels]; channel k's events read x rows of that
 * process's n_x and write p rows of 4 n_out, blocks concatenated in channel order. */
int phs_batch_generate_device(phs_batch_t batch, const int64_t *counts, const double *x,
                              double *p, double *factors, double *volumes, uint8_t *oks,
                              void *stream);

/* Kernel variants of the batch's launches, tuned and pinned as for a process. */
int phs_batch_tuning(phs_batch_t batch, int *ff_variant, int *f64_variant);
int phs_batch_set_variants(phs_batch_t batch, int ff_variant, int f64_variant);

/* Arithmetic of the batch's launches (PHS_PRECISION_F64 or PHS_PRECISION_F32X2). */
int phs_batch_set_precision(phs_batch_t batch, int precision);

/* Offsets of channel k's first x element and first p element for the given counts
 * (x_offsets/p_offsets [n_channels + 1], host). */
int phs_batch_offsets(phs_batch_t batch, const int64_t *counts, int64_t *x_offsets,
                      int64_t *p_offsets);

/* ----------------------------------------------------------------------- CUDA graphs */

typedef struct phs_graph *phs_graph_t;

/* One generate call with fixed pointers and counts as a CUDA graph.  Creation runs the call
 * once (uploads, FP32-pair autotuning), then captures it on a private stream; launching
 * replays the single persistent kernel with no host work.  The reference launches
 * 3 + 2(n_out - 1) kernels with a device synchronization after each (phs.cu:1427-1560). */
int phs_batch_graph_create(phs_graph_t *out, phs_batch_t batch, const int64_t *counts,
                           const double *x, double *p, double *factors, double *volumes,
                           uint8_t *oks);
int phs_process_graph_create(phs_graph_t *out, phs_process_t proc, int64_t n_events,
                             const int64_t *channel_counts, const double *x, double *p,
                             double *factors, double *volumes, uint8_t *oks);
int phs_graph_launch(phs_graph_t graph, void *stream);
int phs_graph_destroy(phs_graph_t graph);

/* ---------------------------------------------------------------------- random numbers */

/* Philox4x32-10 uniform doubles in [0,1) for events [first_event, first_event + n_events) of
 * stream `seed`, rows of n_x, into device memory x (layout in gpu_phs_gb300/philox.py).
 * Replaces the host sampler rng_generate (rng.cpp:69-108) for benchmark inputs. */
int phs_philox_fill(double *x, int64_t n_events, int n_x, uint64_t seed, int64_t first_event,
                    void *stream);

/* ---------------------------------------------------------------------- measurement */

/* Measured FMA throughput of the current device in GFLOP/s (an FMA counts 2), FP64 when
 * fp64 != 0 else FP32: the pipe peaks the forward kernel's roofline is quoted against.  No
 * counterpart in the reference, which records only host wall-clock (monitoring.h:32-40). */
int phs_measure_fma_peak(int fp64, double *gflops);

/* ------------------------------------------------- Whizard binding (whizard_gpu_phs.cpp) */

/* whizard_gpu_phs.cpp:12 */
void c_whizard_set_particle_structure(int *n_channels, int *n_trees, int *n_groves, int *n_x,
                                      int *n_in, int *n_out);
/* whizard_gpu_phs.cpp:35 -- masses/widths [n_in + n_out] */
void c_whizard_set_flavors(double *masses, double *widths);
/* whizard_gpu_phs.cpp:42 */
void c_whizard_init_mappings(void);
/* whizard_gpu_phs.cpp:57 -- channel is 1-based; arrays [2^n_out - 1] */
void c_whizard_fill_mapping(int *channel, int *map_ids, double *masses, double *widths);
/* whizard_gpu_phs.cpp:66 */
void c_whizard_init_tree_structures(void);
/* whizard_gpu_phs.cpp:79 -- channel is 1-based; arrays [2^(n_in+n_out) - 1] */
void c_whizard_fill_tree_structure(int *channel, int *daughters1, int *daughters2,
                                   int *has_children, int *friends);
/* whizard_gpu_phs.cpp:89 -- channel_limits[n_channels]: cumulative event counts */
void c_whizard_init_channel_ids(int *batch_size, int *n_channels, int *channel_limits);
/* whizard_gpu_phs.cpp:100 -- accepted for compatibility; launch shapes come from the
 * occupancy calculator instead */
void c_whizard_set_threads(int *msq_threads, int *cb_threads, int *ab_threads);
/* whizard_gpu_phs.cpp:106 -- validates and stores the trees */
void c_whizard_init_gpu_phs(void);
/* whizard_gpu_phs.cpp:110 */
void c_whizard_finalize_gpu_phs(void);
/* whizard_gpu_phs.cpp:114 -- host arrays; factors [n_events][n_channels], x_out
 * [n_channels][n_events][n_x] (phs.cu:1580-1585).  Synchronous.  The forward map runs in
 * chunks of events with the copies in and back beside the kernels, the inverse map in
 * launches over slices of the channels beside the copies of the finished ones; the
 * results equal one unchunked pass bit for bit.  Device buffers grow to the largest call
 * and stay until c_whizard_reset_generator or c_whizard_finalize_gpu_phs. */
void c_whizard_gen_phs_from_x_gpu(double *E1_in, double *E2_in, bool *requires_boost_to_lab,
                                  int *n_events, int *n_channels, int *n_x, double *x,
                                  double *factors, double *volumes, bool *oks, double *p,
                                  double *x_out);
/* whizard_gpu_phs.cpp:124 -- a no-op in the reference (its argument is passed by value) */
void c_whizard_get_momentum_device_pointer(double *p);
/* whizard_gpu_phs.cpp:128 */
void c_whizard_reset_generator(void);
/* whizard_gpu_phs.cpp:132 */
void c_whizard_show_module(void);

/* Device buffer holding the momenta of the last c_whizard_gen_phs_from_x_gpu call,
 * [n_events][n_out][4], valid until the next generate/reset/finalize; NULL if none.
 * Replaces get_momentum_device_pointer (phs.cu:1638-1640, transfer_to_whizard.h:1). */
double *phs_whizard_momentum_device_pointer(void);

/* ---------------------------------------------------------------- x grids (warm-up) */

/* The per-channel x grid of the reference's warm-up (rng.cpp, main.cpp:145-157): per channel
 * and x dimension, 10 equal-width bins on [0, 1) with weights, starting uniform
 * (init_rng, rng.cpp:19-30).  Replaces the host sampler with device kernels. */
typedef struct phs_grid *phs_grid_t;
int phs_grid_create(phs_grid_t *out, int n_channels, int n_x);
int phs_grid_destroy(phs_grid_t grid);

/* x [n_events][n_x] (device) for events grouped by channel (channel_counts), drawn from each
 * channel's piecewise-constant density (rng_generate, rng.cpp:69-90): the Philox stream of
 * phs_philox_fill (seed, first_event) mapped through the inverse distribution function.
 * The reference draws from std::default_random_engine instead; the distribution is the
 * same. */
int phs_grid_sample_device(phs_grid_t grid, int64_t n_events, const int64_t *channel_counts,
                           uint64_t seed, int64_t first_event, double *x, void *stream);

/* Sets each weight to the fraction of the channel's ok events (oks, 1 byte each) whose x
 * falls into the bin (update_weights, rng.cpp:34-67).  A channel without ok events keeps its
 * weights (the reference divides by zero there). */
int phs_grid_update_device(phs_grid_t grid, int64_t n_events, const int64_t *channel_counts,
                           const double *x, const uint8_t *oks, void *stream);

/* Copies the weights, [n_channels][n_x][10] doubles, to host memory. */
int phs_grid_weights(phs_grid_t grid, double *weights);

#ifdef __cplusplus
}
#endif
#endif
