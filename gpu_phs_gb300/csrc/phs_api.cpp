// phs_api.cpp -- the C ABI of libgpuphs (include/gpu_phs.h): handle API, batches, the
// chunk-pipelined host path, and the Whizard binding (whizard_gpu_phs.cpp:12-249).
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <mutex>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/gpu_phs.h"
#include "../../include/gpu_phs_transfer.h"
#include "phs_device.h"
#include "phs_host.h"

// NVTX range around an entry point's body (tracing under nsys or ncu --nvtx; the NVTX
// calls are no-ops unless a tool is attached).
namespace {
struct TraceRange {
  explicit TraceRange(const char *name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
};
}  // namespace
#define PHS_TRACE(name) TraceRange phs_trace_range_(name)

// ---------------------------------------------------------------------------- errors
static thread_local std::string g_err;

static int fail(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

// Entry points run their bodies through these: no exception may leave a C function, so a
// host failure (std::bad_alloc, std::system_error) becomes PHS_ERR_ALLOC with its message;
// the void Whizard calls also print it, as they print every error.
template <class Body>
static int guarded(Body &&body) {
  try {
    return body();
  } catch (const std::exception &ex) {
    return fail(PHS_ERR_ALLOC, "host: %s", ex.what());
  } catch (...) {
    return fail(PHS_ERR_ALLOC, "host: unknown exception");
  }
}
template <class Body>
static void guarded_void(Body &&body) {
  if (guarded([&]() -> int { body(); return PHS_OK; }) != PHS_OK)
    fprintf(stderr, "gpu_phs: %s\n", g_err.c_str());
}

#define CUDA_TRY(call)                                                                    \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(PHS_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));          \
  } while (0)

extern "C" const char *phs_last_error(void) { return g_err.c_str(); }

extern "C" const char *phs_version(void) { return "gpu_phs_gb300 0.1 (sm_103a, fp64 fused)"; }

// ------------------------------------------------------------------- device buffers
namespace {

// The device allocator of the library's buffers (phs_set_device_allocator): null
// functions mean cudaMalloc/cudaFree.
struct DeviceAllocator {
  phs_device_alloc_fn alloc = nullptr;
  phs_device_free_fn free = nullptr;
  void *user = nullptr;
};
std::mutex g_alloc_mu;
DeviceAllocator g_alloc;

DeviceAllocator current_allocator() {
  std::lock_guard<std::mutex> lock(g_alloc_mu);
  return g_alloc;
}

struct DevBuf {
  void *ptr = nullptr;
  size_t cap = 0;
  DeviceAllocator by;  // the allocator that made ptr (its free hands it back)
  int reserve(size_t bytes) {
    if (bytes <= cap) return PHS_OK;
    release();
    const DeviceAllocator a = current_allocator();
    if (a.alloc) {
      void *p = nullptr;
      const int rc = a.alloc(&p, bytes, a.user);
      if (rc != 0 || !p)
        return fail(PHS_ERR_ALLOC, "the device allocator failed for %zu bytes (returned %d)",
                    bytes, rc);
      ptr = p;
    } else {
      cudaError_t e = cudaMalloc(&ptr, bytes);
      if (e != cudaSuccess) {
        ptr = nullptr;
        return fail(PHS_ERR_ALLOC, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
      }
    }
    by = a;
    cap = bytes;
    return PHS_OK;
  }
  void release() {
    if (ptr) {
      if (by.alloc) {
        // as cudaFree would: no kernel that uses the buffer is still running when the
        // caller's allocator gets it back
        cudaDeviceSynchronize();
        if (by.free) by.free(ptr, by.user);
      } else {
        cudaFree(ptr);
      }
    }
    ptr = nullptr;
    cap = 0;
    by = DeviceAllocator();
  }
  template <class T> T *as() const { return static_cast<T *>(ptr); }
};

// Segment list of one launch, built from per-channel event counts.
struct Segments {
  std::vector<PhsSegment> host;
  DevBuf dev;
  std::vector<PhsSegment> uploaded;  // content of dev
  DevBuf work;                       // chunk counter of the compacting kernels
  DevBuf exact_n, exact_q, exact_t;  // FP32-pair launches: the exact-path queues
  DevBuf pass_n, pass_t, pass_q;     // FP32-pair split form: pre-test survivors per segment
  int64_t n_tiles = 0;
  int64_t n_chunks = 0;
  int64_t n_events = 0;
  void release() {
    dev.release();
    work.release();
    exact_n.release();
    exact_q.release();
    exact_t.release();
    pass_n.release();
    pass_t.release();
    pass_q.release();
    uploaded.clear();
  }
};

struct ChanLayout {  // per launched channel: shape of its x and p rows
  int n_out;
  int x_stride;
};

int build_segments(Segments &S, const int64_t *counts, int n_channels,
                   const std::vector<ChanLayout> &lay, int64_t ev0, int64_t x0, int64_t p0,
                   bool whizard_cols) {
  S.host.clear();
  int64_t ev = ev0, x = x0, p = p0, tile = 0, chunk = 0;
  for (int c = 0; c < n_channels; c++) {
    const int64_t n = counts[c];
    if (n < 0) return fail(PHS_ERR_INVALID_ARG, "channel %d has a negative event count", c);
    if (n == 0) continue;
    PhsSegment g;
    memset(&g, 0, sizeof g);
    g.channel = c;
    g.n_out = lay[c].n_out;
    g.ev_begin = ev;
    g.ev_count = n;
    g.x_base = x;
    g.p_base = p;
    g.tile_begin = tile;
    g.x_stride = lay[c].x_stride;
    g.factor_col = whizard_cols ? c : 0;
    g.chunk_begin = chunk;
    S.host.push_back(g);
    const int64_t tiles = (n + 31) / 32;
    tile += tiles;
    chunk += (tiles + PHS_CHUNK_TILES - 1) / PHS_CHUNK_TILES;
    ev += n;
    x += n * lay[c].x_stride;
    p += n * 4 * lay[c].n_out;
  }
  S.n_tiles = tile;
  S.n_chunks = chunk;
  S.n_events = ev - ev0;
  return PHS_OK;
}

// Fills the launch's segment fields; uploads the table when it does not fit the params.
int attach_segments(Segments &S, PhsLaunch &a, cudaStream_t stream) {
  a.n_segments = (int32_t)S.host.size();
  a.n_tiles = S.n_tiles;
  a.n_chunks = S.n_chunks;
  // the arrays' extents as the segments address them (the checked build's bounds)
  a.x_len = a.p_len = a.ev_len = 0;
  for (const PhsSegment &g : S.host) {
    a.x_len = std::max(a.x_len, g.x_base + g.ev_count * g.x_stride);
    a.p_len = std::max(a.p_len, g.p_base + g.ev_count * 4 * (int64_t)g.n_out);
    a.ev_len = std::max(a.ev_len, g.ev_begin + g.ev_count);
  }
  a.segments = nullptr;
  if (int rc = S.work.reserve(2 * sizeof(unsigned long long))) return rc;
  a.work = S.work.as<unsigned long long>();
  if (S.host.size() <= PHS_INLINE_SEGS) {
    std::copy(S.host.begin(), S.host.end(), a.seg_inline);
    return PHS_OK;
  }
  const size_t bytes = S.host.size() * sizeof(PhsSegment);
  bool same = S.uploaded.size() == S.host.size() &&
              memcmp(S.uploaded.data(), S.host.data(), bytes) == 0;
  if (!same) {
    int rc = S.dev.reserve(bytes);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(S.dev.ptr, S.host.data(), bytes, cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    S.uploaded = S.host;
  }
  a.segments = S.dev.as<PhsSegment>();
  return PHS_OK;
}

int sm_count(int device) {
  static int cached[64] = {0};
  if (device >= 0 && device < 64 && cached[device]) return cached[device];
  int n = 0;
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device);
  if (n <= 0) n = 1;
  if (device >= 0 && device < 64) cached[device] = n;
  return n;
}

int grid_for(int64_t n_tiles, int device, int stack_depth, bool per_event, int variant) {
  const int warps_per_block = phs_forward_block_size(variant) / 32;
  int64_t want = (n_tiles + warps_per_block - 1) / warps_per_block;
  int64_t cap =
      (int64_t)sm_count(device) * phs_forward_blocks_per_sm(stack_depth, per_event, variant);
  return (int)std::max<int64_t>(1, std::min(want, cap));
}

int grid_for_ff(int64_t n_tiles, int device, int stack_depth, int variant) {
  const int warps_per_block = PHS_FWD_BLOCK / 32;
  int64_t want = (n_tiles + warps_per_block - 1) / warps_per_block;
  int64_t cap = (int64_t)sm_count(device) * phs_forward_ff_blocks_per_sm(stack_depth, variant);
  return (int)std::max<int64_t>(1, std::min(want, cap));
}

// Launch with autotuning.  A kernel comes in n_variants forms that compute identical bits
// (register budgets, one- or two-pass); which is fastest depends on the trees and on how
// many events pass the kinematic test.  The first launch of at least kTuneEvents events,
// outside stream capture, runs every variant twice on the real data, times them with
// CUDA events on the launch stream and keeps the fastest in `variant`; later launches use
// it.  launch(v) enqueues variant v.
const int64_t kTuneEvents = 1 << 18;

const int kMaxVariants = 16;
static_assert(PHS_F64_VARIANTS <= kMaxVariants && PHS_FF_VARIANTS <= kMaxVariants,
              "launch_tuned keeps one timing per variant");

template <class Launch>
int launch_tuned(int &variant, int n_variants, int64_t n_events, cudaStream_t st, Launch launch) {
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(st, &cap);
  if (n_variants > kMaxVariants) return fail(PHS_ERR_INVALID_ARG, "too many kernel variants");
  if (variant < 0 && n_events >= kTuneEvents && cap == cudaStreamCaptureStatusNone) {
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    float best[kMaxVariants];
    for (int v = 0; v < n_variants; v++) best[v] = 1e30f;
    for (int rep = 0; rep < 2; rep++) {
      for (int v = 0; v < n_variants; v++) {
        CUDA_TRY(cudaEventRecord(e0, st));
        CUDA_TRY(launch(v));
        CUDA_TRY(cudaEventRecord(e1, st));
        CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        best[v] = std::min(best[v], ms);
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int bv = 0;
    for (int v = 1; v < n_variants; v++)
      if (best[v] < best[bv]) bv = v;
    variant = bv;
    return PHS_OK;  // the timed launches already wrote the outputs
  }
  CUDA_TRY(launch(variant < 0 ? 0 : variant));
  return PHS_OK;
}

// FP32-pair launch: the float-float kernel, then the exact FP64 path over the events it
// queued (a handful of blocks: they are about 0.1 % of the events, or all events of a
// channel without a float-float form).
// Scratch of the split forms: pre-test survivors per segment, their claim numbering and
// their indices (n_tiles * 32 entries).
int attach_pass_buffers(Segments &S, PhsLaunch &a) {
  const size_t n_seg = (size_t)std::max(a.n_segments, 1);
  if (int rc = S.pass_n.reserve(n_seg * sizeof(unsigned int))) return rc;
  if (int rc = S.pass_t.reserve((n_seg + 1) * sizeof(int64_t))) return rc;
  if (int rc = S.pass_q.reserve((size_t)std::max<int64_t>(a.n_tiles, 1) * 32 * sizeof(int32_t)))
    return rc;
  a.pass_count = S.pass_n.as<unsigned int>();
  a.pass_tile = S.pass_t.as<int64_t>();
  a.pass_queue = S.pass_q.as<int32_t>();
  return PHS_OK;
}

int launch_ff_tuned(int &variant, Segments &S, PhsLaunch a, int device, int depth,
                    int64_t n_events, cudaStream_t st) {
  const size_t n_seg = (size_t)std::max(a.n_segments, 1);
  if (int rc = S.exact_n.reserve(n_seg * sizeof(unsigned int))) return rc;
  if (int rc = S.exact_t.reserve((n_seg + 1) * sizeof(int64_t))) return rc;
  if (int rc = S.exact_q.reserve((size_t)std::max<int64_t>(a.n_tiles, 1) * 32 * sizeof(int32_t)))
    return rc;
  if (int rc = attach_pass_buffers(S, a)) return rc;
  a.exact_work = a.work + 1;  // attach_segments reserved two counters
  a.exact_count = S.exact_n.as<unsigned int>();
  a.exact_queue = S.exact_q.as<int32_t>();
  a.exact_tile = S.exact_t.as<int64_t>();
  const int exact_grid = sm_count(device) * 4;
  // per-event beams: the float-float one pass at either register budget (variants 0, 1;
  // the pre-test needs uniform constants), or the FP64 compacting kernel (2, 3: FP64
  // variants 1, 2), whose FP64 results meet this precision's bar too and which wins where
  // few events pass
  const bool per_event = a.E1 != nullptr;
  return launch_tuned(variant, per_event ? 4 : PHS_FF_VARIANTS, n_events, st, [&](int v) {
    if (per_event && v >= 2) {
      const int f64v = v >= 4 ? 1 + (v & 1) : v - 1;
      cudaError_t e = cudaMemsetAsync(a.work, 0, 2 * sizeof(unsigned long long), st);
      if (e == cudaSuccess)
        e = phs_launch_forward_f64(a, grid_for(a.n_tiles, device, depth, true, f64v), f64v, st);
      return e;
    }
    if (per_event) v &= 1;
    cudaError_t e = cudaMemsetAsync(a.exact_count, 0, (size_t)a.n_segments * sizeof(unsigned int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.work, 0, 2 * sizeof(unsigned long long), st);
    if (e == cudaSuccess && v >= 4)
      e = cudaMemsetAsync(a.pass_count, 0, (size_t)a.n_segments * sizeof(unsigned int), st);
    if (e == cudaSuccess) e = phs_launch_forward_ff(a, grid_for_ff(a.n_tiles, device, depth, v), v, st);
    if (e == cudaSuccess) e = phs_launch_forward_exact(a, exact_grid, st);
    return e;
  });
}

int launch_f64_tuned(int &variant, Segments &S, PhsLaunch a, int device, int depth,
                     int64_t n_events, cudaStream_t st) {
  const bool per_event = a.E1 != nullptr;
  if (!per_event)
    if (int rc = attach_pass_buffers(S, a)) return rc;
  const int n_variants = per_event ? PHS_F64_VARIANTS_PER_EVENT : PHS_F64_VARIANTS;
  return launch_tuned(variant, n_variants, n_events, st, [&](int v) {
    // per-event beams have no pre-test: a pinned split form runs as the compacting or
    // one-pass form of the same block shape
    if (per_event && v >= PHS_F64_VARIANTS_PER_EVENT) v -= 4;
    cudaError_t e = cudaSuccess;
    if (a.work) e = cudaMemsetAsync(a.work, 0, sizeof(unsigned long long), st);
    if (e == cudaSuccess && v >= PHS_F64_VARIANTS_PER_EVENT)
      e = cudaMemsetAsync(a.pass_count, 0, (size_t)a.n_segments * sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
    return phs_launch_forward_f64(a, grid_for(a.n_tiles, device, depth, per_event, v), v, st);
  });
}

// Restores the caller's current device on scope exit.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

}  // namespace

extern "C" int phs_set_device_allocator(phs_device_alloc_fn alloc, phs_device_free_fn free_fn,
                                        void *user) {
  if ((alloc == nullptr) != (free_fn == nullptr))
    return fail(PHS_ERR_INVALID_ARG, "give both allocator functions or neither");
  std::lock_guard<std::mutex> lock(g_alloc_mu);
  g_alloc.alloc = alloc;
  g_alloc.free = free_fn;
  g_alloc.user = user;
  return PHS_OK;
}

extern "C" int phs_is_checked_build(void) {
#ifdef PHS_CHECKED
  return 1;
#else
  return 0;
#endif
}

extern "C" int phs_check_status(uint64_t *sites, int64_t *first_index) {
  return guarded([&]() -> int {
    if (!sites) return fail(PHS_ERR_INVALID_ARG, "null sites pointer");
    *sites = 0;
    if (first_index) *first_index = 0;
    if (!phs_is_checked_build())
      return fail(PHS_ERR_UNSUPPORTED, "bounds checks are compiled into libgpuphs_checked.so only");
    cudaError_t (*collect[])(unsigned long long *, long long *) = {
        phs_check_collect_kernels, phs_check_collect_ff, phs_check_collect_adjoint,
        phs_check_collect_inverse, phs_check_collect_grid};
    CUDA_TRY(cudaDeviceSynchronize());
    bool have_first = false;
    for (auto fn : collect) {
      unsigned long long w = 0;
      long long f = 0;
      CUDA_TRY(fn(&w, &f));
      if (w && !have_first && first_index) {
        *first_index = f;
        have_first = true;
      }
      *sites |= w;
    }
    return PHS_OK;
  });
}

// -------------------------------------------------------------------------- process
struct phs_process {
  phs::Process p;
  int device = 0;
  bool beams = false;
  double E1 = 0, E2 = 0;
  int precision = PHS_PRECISION_F64;
  int ff_variant_ev[2] = {-1, -1};  // autotuned FP32-pair variant: uniform, per-event beams
  int f64_variant[2] = {-1, -1};  // autotuned FP64 variant: uniform, per-event beams
  std::vector<PhsChannel> prog;
  std::vector<PhsChannelFF> prog_ff;
  std::vector<PhsAdjChannel> prog_adj;
  std::vector<ChanLayout> lay;
  int stack_depth = 0, max_visits = 0, max_pops = 0;
  bool has_friends = false;
  DevBuf d_prog, d_prog_ff, d_prog_adj;
  int adjoint_storage = PHS_ADJOINT_RECOMPUTE;
  DevBuf d_adj_store;                 // stored-matrix adjoint: the parent frames per visit
  DevBuf d_ch_begin;                  // inverse map: first event per generating channel
  DevBuf d_inv_groups;                // inverse map: channels by tree shape, group starts,
                                      // mapping reuse masks
  int n_inv_groups = 0;
  std::vector<int32_t> inv_order;     // the channels in the group order (host copy)
  std::vector<int32_t> inv_group_begin;  // each group's first position in it, then n_channels
  size_t inv_reuse_offset = 0;        // byte offset of the reuse masks in d_inv_groups
  std::vector<int64_t> ch_begin_up;   // content of d_ch_begin
  Segments segs;
  // host-path pipeline
  static const int kStreams = 3;
  cudaStream_t streams[kStreams] = {nullptr, nullptr};
  DevBuf bx[kStreams], bp[kStreams], bf[kStreams], bv[kStreams], bo[kStreams];
  Segments pseg[kStreams];
  int64_t chunk = 0;
};

static int check_proc(phs_process_t h) {
  if (!h) return fail(PHS_ERR_INVALID_ARG, "null process handle");
  return PHS_OK;
}

extern "C" int phs_process_create(phs_process_t *out, int n_in, int n_out, int n_channels, int n_x,
                                  const int *d1, const int *d2, const int *hc, const int *friends,
                                  const int *map_ids, const double *map_m, const double *map_w,
                                  const double *flv_m, const double *flv_w) {
  return guarded([&]() -> int {
    if (!out) return fail(PHS_ERR_INVALID_ARG, "null output handle pointer");
    *out = nullptr;
    if (!d1 || !d2 || !hc || !map_ids || !map_m || !map_w || !flv_m)
      return fail(PHS_ERR_INVALID_ARG, "null table pointer");
    phs::Process P;
    P.n_in = n_in;
    P.n_out = n_out;
    P.n_channels = n_channels;
    P.n_x = n_x;
    std::string err;
    int rc = phs::validate_process(P, err);
    if (rc) return fail(rc, "%s", err.c_str());
    P.n_prt = (1 << (n_in + n_out)) - 1;
    P.n_prt_out = (1 << n_out) - 1;
    const size_t nt = (size_t)n_channels * P.n_prt, nm = (size_t)n_channels * P.n_prt_out;
    P.d1.assign(d1, d1 + nt);
    P.d2.assign(d2, d2 + nt);
    P.has_children.assign(hc, hc + nt);
    P.friends = friends ? std::vector<int>(friends, friends + nt) : std::vector<int>(nt, 0);
    P.map_id.assign(map_ids, map_ids + nm);
    P.map_m.assign(map_m, map_m + nm);
    P.map_w.assign(map_w, map_w + nm);
    P.flv_m.assign(flv_m, flv_m + n_in + n_out);
    P.flv_w = flv_w ? std::vector<double>(flv_w, flv_w + n_in + n_out)
                    : std::vector<double>(n_in + n_out, 0.0);
    // structural validation at a nominal sqrt(s) (constants are recompiled by set_beams)
    for (int c = 0; c < n_channels; c++) {
      PhsChannel tmp;
      phs::ChannelInfo info;
      double m_tot = 0;
      for (int k = 0; k < n_out; k++) m_tot += P.flv_m[n_in + k];
      rc = phs::compile_channel(P, c, 2 * m_tot + 1000.0, tmp, info, err);
      if (rc) return fail(rc, "%s", err.c_str());
    }
    phs_process *h = new phs_process;
    h->p = std::move(P);
    cudaGetDevice(&h->device);
    *out = h;
    return PHS_OK;
  });
}

extern "C" int phs_process_destroy(phs_process_t h) {
  return guarded([&]() -> int {
    if (!h) return PHS_OK;
    DeviceGuard g(h->device);
    for (int s = 0; s < phs_process::kStreams; s++) {
      if (h->streams[s]) cudaStreamDestroy(h->streams[s]);
      h->bx[s].release(); h->bp[s].release(); h->bf[s].release(); h->bv[s].release();
      h->bo[s].release(); h->pseg[s].release();
    }
    h->d_prog.release();
    h->d_prog_ff.release();
    h->d_prog_adj.release();
    h->d_adj_store.release();
    h->d_ch_begin.release();
    h->d_inv_groups.release();
    h->segs.release();
    delete h;
    return PHS_OK;
  });
}

extern "C" int phs_process_set_beams(phs_process_t h, double E1, double E2) {
  PHS_TRACE("phs_process_set_beams");
  return guarded([&]() -> int {
    if (int rc = check_proc(h)) return rc;
    if (!(E1 > 0) || !(E2 > 0) || !isfinite(E1) || !isfinite(E2))
      return fail(PHS_ERR_INVALID_ARG, "beam energies must be positive and finite");
    if (h->beams && h->E1 == E1 && h->E2 == E2) return PHS_OK;
    DeviceGuard g(h->device);
    const phs::Process &P = h->p;
    const double sqrts = 2 * sqrt(E1 * E2);
    double m_tot = 0;
    for (int k = 0; k < P.n_out; k++) m_tot += P.flv_m[P.n_in + k];
    if (!(sqrts > m_tot))
      return fail(PHS_ERR_INVALID_ARG, "sqrt(s) = %g is below the final-state mass sum %g", sqrts,
                  m_tot);
    std::vector<PhsChannel> prog(P.n_channels);
    int depth = 0;
    std::string err;
    const double bg = (E1 - E2) / (2 * sqrt(E1 * E2));
    for (int c = 0; c < P.n_channels; c++) {
      phs::ChannelInfo info;
      int rc = phs::compile_channel(P, c, sqrts, prog[c], info, err);
      if (rc) return fail(rc, "%s", err.c_str());
      prog[c].sqrts = sqrts;
      prog[c].lab = E1 != E2;
      prog[c].lab_bg = bg;
      prog[c].lab_gamma = sqrt(1 + bg * bg);
      depth = std::max(depth, info.stack_depth);
    }
    std::vector<PhsChannelFF> prog_ff(prog.size());
    std::vector<PhsAdjChannel> prog_adj(prog.size());
    int max_visits = 0, max_pops = 0;
    for (size_t c = 0; c < prog.size(); c++) {
      phs::channel_to_ff(prog[c], prog_ff[c]);
      phs::channel_adjoint(prog[c], prog_adj[c]);
      max_visits = std::max(max_visits, (int)prog[c].n_visits);
      max_pops = std::max(max_pops, (int)prog_adj[c].n_pops);
    }
    int rc = h->d_prog.reserve(prog.size() * sizeof(PhsChannel));
    if (rc) return rc;
    if ((rc = h->d_prog_ff.reserve(prog_ff.size() * sizeof(PhsChannelFF)))) return rc;
    if ((rc = h->d_prog_adj.reserve(prog_adj.size() * sizeof(PhsAdjChannel)))) return rc;
    CUDA_TRY(cudaMemcpy(h->d_prog_adj.ptr, prog_adj.data(), prog_adj.size() * sizeof(PhsAdjChannel),
                        cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(h->d_prog.ptr, prog.data(), prog.size() * sizeof(PhsChannel),
                        cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(h->d_prog_ff.ptr, prog_ff.data(), prog_ff.size() * sizeof(PhsChannelFF),
                        cudaMemcpyHostToDevice));
    // channels of equal tree shape share the inverse map's geometry: order them by shape
    {
      std::vector<std::vector<int32_t>> keys;
      std::vector<std::vector<int32_t>> members;
      for (int c = 0; c < (int)prog.size(); c++) {
        const PhsChannel &ch = prog[c];
        std::vector<int32_t> key = {ch.n_out, ch.n_visits, ch.n_vol};
        for (int i = 0; i < ch.n_vol; i++) {
          key.push_back(ch.comb[i][0]);
          key.push_back(ch.comb[i][1]);
        }
        for (int v = 0; v < ch.n_visits; v++) {
          const PhsVisit &V = ch.visit[v];
          key.insert(key.end(), {V.slot[0], V.slot[1], V.friend_sign, V.carry, V.push,
                                 V.both_leaves, V.self_root, V.x_phi, V.x_ct});
          for (int j = 0; j < 2; j++)
            key.insert(key.end(), {V.child[j].internal, V.child[j].x_msq, V.child[j].out_index});
        }
        size_t g = 0;
        while (g < keys.size() && keys[g] != key) g++;
        if (g == keys.size()) {
          keys.push_back(key);
          members.emplace_back();
        }
        members[g].push_back(c);
      }
      // within a shape, channels in order of their mappings, so that equal ones follow each
      // other: a channel reuses the previous channel's mapping results wherever the two have
      // the same mapping (position 3 v + 0/1: a daughter's msq map, 3 v + 2: the cos(theta) map)
      auto mapping = [&](int c, int v, int k) {
        std::vector<double> sig;
        const PhsVisit &V = prog[c].visit[v];
        if (k < 2) {
          const PhsChild &C = V.child[k];
          if (!C.internal) return sig;
          sig = {(double)C.map_id, C.m, C.w, C.m_min, C.a0, C.a1, C.a2, C.msq_min, C.msq_max};
        } else {
          sig = {(double)V.ct_class, V.b0, V.b1, V.m};
        }
        return sig;
      };
      // signatures compare by their bits (a strict weak order even with -0.0 or NaN)
      auto bits = [](const std::vector<double> &x) {
        std::vector<uint64_t> b(x.size());
        if (!x.empty()) memcpy(b.data(), x.data(), x.size() * sizeof(double));
        return b;
      };
      auto same = [&](const std::vector<double> &x, const std::vector<double> &y) {
        return bits(x) == bits(y);
      };
      std::vector<int32_t> order;
      std::vector<uint64_t> reuse;
      for (auto &m : members) {
        const int nv = prog[m[0]].n_visits;
        std::stable_sort(m.begin(), m.end(), [&](int c1, int c2) {
          for (int v = 0; v < nv; v++)
            for (int k = 0; k < 3; k++) {
              const auto x = bits(mapping(c1, v, k)), y = bits(mapping(c2, v, k));
              if (x != y) return x < y;
            }
          return false;
        });
        for (size_t i = 0; i < m.size(); i++) {
          uint64_t mask = 0;
          if (i > 0)
            for (int v = 0; v < nv && 3 * v + 2 < 64; v++)
              for (int k = 0; k < 3; k++) {
                const auto x = mapping(m[i], v, k);
                if (!x.empty() && same(x, mapping(m[i - 1], v, k))) mask |= 1ull << (3 * v + k);
              }
          order.push_back(m[i]);
          reuse.push_back(mask);
        }
      }
      // [order n_channels][begin n_groups + 1], then the reuse masks (8-byte aligned)
      std::vector<int32_t> table = order;
      int32_t at = 0;
      table.push_back(at);
      for (const auto &m : members) table.push_back(at += (int32_t)m.size());
      if (table.size() % 2) table.push_back(0);
      const size_t head = table.size() * sizeof(int32_t);
      if ((rc = h->d_inv_groups.reserve(head + reuse.size() * sizeof(uint64_t)))) return rc;
      CUDA_TRY(cudaMemcpy(h->d_inv_groups.ptr, table.data(), head, cudaMemcpyHostToDevice));
      CUDA_TRY(cudaMemcpy(static_cast<char *>(h->d_inv_groups.ptr) + head, reuse.data(),
                          reuse.size() * sizeof(uint64_t), cudaMemcpyHostToDevice));
      h->n_inv_groups = (int)members.size();
      h->inv_reuse_offset = head;
      h->inv_order = order;
      h->inv_group_begin.assign(table.begin() + order.size(), table.begin() + order.size() + members.size() + 1);
    }
    h->prog = std::move(prog);
    h->prog_ff = std::move(prog_ff);
    h->prog_adj = std::move(prog_adj);
    h->max_visits = max_visits;
    h->max_pops = max_pops;
    h->lay.assign(P.n_channels, ChanLayout{P.n_out, P.n_x});
    h->has_friends = false;
    for (const auto &ch : h->prog)
      for (int v = 0; v < ch.n_visits; v++) h->has_friends |= ch.visit[v].friend_sign != 0;
    h->stack_depth = depth;
    h->E1 = E1;
    h->E2 = E2;
    h->beams = true;
    return PHS_OK;
  });
}

extern "C" int phs_process_set_precision(phs_process_t h, int precision) {
  return guarded([&]() -> int {
    if (int rc = check_proc(h)) return rc;
    if (precision != PHS_PRECISION_F64 && precision != PHS_PRECISION_F32X2)
      return fail(PHS_ERR_INVALID_ARG, "unknown precision mode %d", precision);
    h->precision = precision;
    return PHS_OK;
  });
}

extern "C" int phs_process_tuning(phs_process_t h, int *ff_variant, int *f64_variant) {
  return guarded([&]() -> int {
    if (int rc = check_proc(h)) return rc;
    if (ff_variant) *ff_variant = h->ff_variant_ev[0];
    if (f64_variant) *f64_variant = h->f64_variant[0];
    return PHS_OK;
  });
}

static int check_variants(int ff_variant, int f64_variant) {
  if (ff_variant < -1 || ff_variant >= PHS_FF_VARIANTS)
    return fail(PHS_ERR_INVALID_ARG, "FP32-pair variant %d is not in [-1, %d)", ff_variant,
                PHS_FF_VARIANTS);
  if (f64_variant < -1 || f64_variant >= PHS_F64_VARIANTS)
    return fail(PHS_ERR_INVALID_ARG, "FP64 variant %d is not in [-1, %d)", f64_variant,
                PHS_F64_VARIANTS);
  return PHS_OK;
}

extern "C" int phs_process_set_variants(phs_process_t h, int ff_variant, int f64_variant) {
  return guarded([&]() -> int {
    if (int rc = check_proc(h)) return rc;
    if (int rc = check_variants(ff_variant, f64_variant)) return rc;
    h->ff_variant_ev[0] = h->ff_variant_ev[1] = ff_variant;
    h->f64_variant[0] = h->f64_variant[1] = f64_variant;
    return PHS_OK;
  });
}

extern "C" int phs_process_info(phs_process_t h, int *n_in, int *n_out, int *n_channels, int *n_x,
                                int *depth) {
  return guarded([&]() -> int {
    if (int rc = check_proc(h)) return rc;
    if (n_in) *n_in = h->p.n_in;
    if (n_out) *n_out = h->p.n_out;
    if (n_channels) *n_channels = h->p.n_channels;
    if (n_x) *n_x = h->p.n_x;
    if (depth) {
      int d = 0;
      for (int c = 0; c < h->p.n_channels; c++) {
        PhsChannel tmp;
        phs::ChannelInfo info;
        std::string err;
        if (phs::compile_channel(h->p, c, 1e4, tmp, info, err) == 0) d = std::max(d, info.stack_depth);
      }
      *depth = d;
    }
    return PHS_OK;
  });
}

static int check_counts(const int64_t *counts, int n_channels, int64_t n_events) {
  if (n_events < 0) return fail(PHS_ERR_INVALID_ARG, "n_events < 0");
  if (!counts) {
    if (n_channels != 1)
      return fail(PHS_ERR_INVALID_ARG, "channel_counts is required for %d channels", n_channels);
    return PHS_OK;
  }
  int64_t sum = 0;
  for (int c = 0; c < n_channels; c++) {
    if (counts[c] < 0) return fail(PHS_ERR_INVALID_ARG, "channel %d has a negative count", c);
    sum += counts[c];
  }
  if (sum != n_events)
    return fail(PHS_ERR_INVALID_ARG, "channel counts sum to %lld, not n_events = %lld",
                (long long)sum, (long long)n_events);
  return PHS_OK;
}

static int launch_process(phs_process_t h, Segments &S, int64_t n_events, const int64_t *counts,
                          int64_t ev0, const double *x, double *p, double *f, double *v,
                          uint8_t *ok, const double *E1, const double *E2, int64_t fstride,
                          bool whizard_cols, cudaStream_t stream) {
  int64_t one = n_events;
  const int64_t *cnt = counts ? counts : &one;
  int rc = build_segments(S, cnt, h->p.n_channels, h->lay, ev0, 0, 0, whizard_cols);
  if (rc) return rc;
  PhsLaunch a;
  memset(&a, 0, sizeof a);
  a.channels = h->d_prog.as<PhsChannel>();
  a.channels_ff = h->d_prog_ff.as<PhsChannelFF>();
  a.stack_depth = h->stack_depth;
  a.x = x;
  a.p = p;
  a.factor = f;
  a.volume = v;
  a.ok = ok;
  a.factor_stride = fstride;
  a.E1 = E1;
  a.E2 = E2;
  a.n_programs = h->p.n_channels;
  // segment events are numbered from ev0 within this launch's output arrays
  for (auto &g : S.host) g.ev_begin -= ev0;
  if ((rc = attach_segments(S, a, stream))) return rc;
  if (a.n_tiles == 0) return PHS_OK;
  if (h->precision == PHS_PRECISION_F32X2)
    return launch_ff_tuned(h->ff_variant_ev[E1 != nullptr], S, a, h->device, h->stack_depth,
                           n_events, stream);
  return launch_f64_tuned(h->f64_variant[E1 != nullptr], S, a, h->device, h->stack_depth, n_events,
                          stream);
}

static int check_ptrs(int64_t n, const void *x, const void *p, const void *f, const void *v,
                      const void *o) {
  if (n > 0 && (!x || !p || !f || !v || !o)) return fail(PHS_ERR_INVALID_ARG, "null data pointer");
  if (((uintptr_t)p & 15) != 0) return fail(PHS_ERR_INVALID_ARG, "p must be 16-byte aligned");
  return PHS_OK;
}

extern "C" int phs_generate_device(phs_process_t h, int64_t n_events, const int64_t *counts,
                                   const double *x, double *p, double *f, double *v, uint8_t *ok,
                                   void *stream) {
  PHS_TRACE("phs_generate_device");
  return guarded([&]() -> int {
    if (int rc = check_proc(h)) return rc;
    if (!h->beams) return fail(PHS_ERR_STATE, "phs_process_set_beams has not been called");
    if (int rc = check_counts(counts, h->p.n_channels, n_events)) return rc;
    if (int rc = check_ptrs(n_events, x, p, f, v, ok)) return rc;
    DeviceGuard g(h->device);
    return launch_process(h, h->segs, n_events, counts, 0, x, p, f, v, ok, nullptr, nullptr, 1,
                          false, (cudaStream_t)stream);
  });
}

extern "C" int phs_generate_beams_device(phs_process_t h, int64_t n_events, const int64_t *counts,
                                         const double *E1, const double *E2, const double *x,
                                         double *p, double *f, double *v, uint8_t *ok,
                                         void *stream) {
  PHS_TRACE("phs_generate_beams_device");
  return guarded([&]() -> int {
    if (int rc = check_proc(h)) return rc;
    if (int rc = check_counts(counts, h->p.n_channels, n_events)) return rc;
    if (int rc = check_ptrs(n_events, x, p, f, v, ok)) return rc;
    if (n_events > 0 && (!E1 || !E2)) return fail(PHS_ERR_INVALID_ARG, "null beam energy pointer");
    DeviceGuard g(h->device);
    if (!h->beams) {
      // programs need compiling once; per-event constants replace the uniform ones
      double m_tot = 0;
      for (int k = 0; k < h->p.n_out; k++) m_tot += h->p.flv_m[h->p.n_in + k];
      int rc = phs_process_set_beams(h, m_tot + 500.0, m_tot + 500.0);
      if (rc) return rc;
    }
    return launch_process(h, h->segs, n_events, counts, 0, x, p, f, v, ok, E1, E2, 1, false,
                          (cudaStream_t)stream);
  });
}

// Reverse-mode derivatives for cotangents pbar (momenta) and jbar (log-Jacobian).
extern "C" int phs_adjoint_device(phs_process_t h, int64_t n_events, const int64_t *counts,
                                  const double *x, const double *pbar, const double *jbar,
                                  double *xbar, double *thbar, void *stream) {
  PHS_TRACE("phs_adjoint_device");
  return guarded([&]() -> int {
    if (int rc = check_proc(h)) return rc;
    if (!h->beams) return fail(PHS_ERR_STATE, "phs_process_set_beams has not been called");
    if (int rc = check_counts(counts, h->p.n_channels, n_events)) return rc;
    if (n_events > 0 && (!x || !pbar || !xbar || !thbar))
      return fail(PHS_ERR_INVALID_ARG, "null data pointer");
    DeviceGuard g(h->device);
    int64_t one = n_events;
    int rc = build_segments(h->segs, counts ? counts : &one, h->p.n_channels, h->lay, 0, 0, 0, false);
    if (rc) return rc;
    PhsLaunch a;
    memset(&a, 0, sizeof a);
    a.channels = h->d_prog.as<PhsChannel>();
    a.stack_depth = h->stack_depth;
    a.x = x;
    a.factor_stride = 1;
    a.n_programs = h->p.n_channels;
    if ((rc = attach_segments(h->segs, a, (cudaStream_t)stream))) return rc;
    if (a.n_tiles == 0) return PHS_OK;
    const bool stored = h->adjoint_storage == PHS_ADJOINT_STORED;
    double *store = nullptr;
    if (stored) {
      // the stored-matrix form: every visit's parent frame of every event
      if ((rc = h->d_adj_store.reserve((size_t)n_events * h->max_visits * 16 * sizeof(double))))
        return rc;
      store = h->d_adj_store.as<double>();
    }
    const int per_sm = phs_adjoint_blocks_per_sm(h->max_visits, h->max_pops, h->stack_depth,
                                                 h->has_friends, stored);
    const int64_t want = (a.n_tiles + PHS_ADJ_BLOCK_HOST / 32 - 1) / (PHS_ADJ_BLOCK_HOST / 32);
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sm_count(h->device) * per_sm));
    CUDA_TRY(phs_launch_adjoint(a, h->d_prog_adj.as<PhsAdjChannel>(), pbar, jbar, xbar, thbar,
                                2 * std::max(1, h->p.n_out - 2), h->max_visits, h->max_pops,
                                h->has_friends, grid, (cudaStream_t)stream, store, n_events));
    return PHS_OK;
  });
}

extern "C" int phs_process_set_adjoint_storage(phs_process_t h, int storage) {
  return guarded([&]() -> int {
    if (int rc = check_proc(h)) return rc;
    if (storage != PHS_ADJOINT_RECOMPUTE && storage != PHS_ADJOINT_STORED)
      return fail(PHS_ERR_INVALID_ARG, "unknown adjoint storage mode %d", storage);
    h->adjoint_storage = storage;
    if (storage == PHS_ADJOINT_RECOMPUTE) {
      DeviceGuard g(h->device);
      h->d_adj_store.release();
    }
    return PHS_OK;
  });
}

// Inverse map: all-channel factors and x of generated events.
static int inverse_launch(phs_process_t h, int64_t n_events, const int64_t *d_ch_begin,
                          const double *E1, const double *E2, const double *p, const uint8_t *ok,
                          const double *x_own, const double *factor_own, double *all_factors,
                          double *x_out, cudaStream_t st, int order_lo = 0, int order_hi = -1,
                          bool write_fixed = true, int64_t x_ch_stride = 0);

extern "C" int phs_inverse_device(phs_process_t h, int64_t n_events, const int64_t *counts,
                                  const double *E1, const double *E2, const double *p,
                                  const uint8_t *ok, const double *x_own,
                                  const double *factor_own, double *all_factors, double *x_out,
                                  void *stream) {
  PHS_TRACE("phs_inverse_device");
  return guarded([&]() -> int {
    if (int rc = check_proc(h)) return rc;
    if (int rc = check_counts(counts, h->p.n_channels, n_events)) return rc;
    if (n_events > 0 && (!p || !all_factors || !x_out))
      return fail(PHS_ERR_INVALID_ARG, "null data pointer");
    if ((E1 == nullptr) != (E2 == nullptr))
      return fail(PHS_ERR_INVALID_ARG, "give both beam energy arrays or neither");
    if (((uintptr_t)p & 15) != 0) return fail(PHS_ERR_INVALID_ARG, "p must be 16-byte aligned");
    DeviceGuard g(h->device);
    if (!h->beams) {
      if (!E1) return fail(PHS_ERR_STATE, "phs_process_set_beams has not been called");
      double m_tot = 0;
      for (int k = 0; k < h->p.n_out; k++) m_tot += h->p.flv_m[h->p.n_in + k];
      int rc = phs_process_set_beams(h, m_tot + 500.0, m_tot + 500.0);
      if (rc) return rc;
    }
    if (n_events == 0) return PHS_OK;
    const int nch = h->p.n_channels;
    std::vector<int64_t> begin(nch, 0);
    for (int c = 1; c < nch; c++) begin[c] = begin[c - 1] + (counts ? counts[c - 1] : n_events);
    cudaStream_t st = (cudaStream_t)stream;
    if (begin != h->ch_begin_up) {
      int rc = h->d_ch_begin.reserve(nch * sizeof(int64_t));
      if (rc) return rc;
      CUDA_TRY(cudaMemcpyAsync(h->d_ch_begin.ptr, begin.data(), nch * sizeof(int64_t),
                               cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaStreamSynchronize(st));
      h->ch_begin_up = begin;
    }
    return inverse_launch(h, n_events, h->d_ch_begin.as<int64_t>(), E1, E2, p, ok, x_own,
                          factor_own, all_factors, x_out, st);
  });
}

// The inverse-map launch of n_events (channel starts d_ch_begin[n_channels] on the device)
// for the channels at group-order positions [order_lo, order_hi) (order_hi < 0: to the end);
// x_out holds x_ch_stride rows per channel (0: n_events).
static int inverse_launch(phs_process_t h, int64_t n_events, const int64_t *d_ch_begin,
                          const double *E1, const double *E2, const double *p, const uint8_t *ok,
                          const double *x_own, const double *factor_own, double *all_factors,
                          double *x_out, cudaStream_t st, int order_lo, int order_hi,
                          bool write_fixed, int64_t x_ch_stride) {
  const int nch = h->p.n_channels;
  PhsInvLaunch a;
  memset(&a, 0, sizeof a);
  a.channels = h->d_prog.as<PhsChannel>();
  a.ch_begin = d_ch_begin;
  a.p = p;
  a.ok = ok;
  a.E1 = E1;
  a.E2 = E2;
  a.x_own = x_own;
  a.factor_own = factor_own;
  a.all_factors = all_factors;
  a.x_out = x_out;
  a.n_events = n_events;
  a.x_ch_stride = x_ch_stride > 0 ? x_ch_stride : n_events;
  a.n_channels = nch;
  a.n_out = h->p.n_out;
  a.n_x = h->p.n_x;
  a.stack_depth = h->stack_depth;
  a.max_visits = h->max_visits;
  a.group_order = h->d_inv_groups.as<int32_t>();
  a.group_begin = a.group_order + nch;
  const bool cache = phs_inverse_fits_cache(a.n_out, a.stack_depth, a.max_visits);
  a.group_reuse = cache ? reinterpret_cast<const uint64_t *>(
                              static_cast<const char *>(h->d_inv_groups.ptr) + h->inv_reuse_offset)
                        : nullptr;
  a.n_groups = h->n_inv_groups;
  a.order_lo = order_lo;
  a.order_hi = order_hi < 0 ? nch : order_hi;
  a.write_fixed = write_fixed ? 1 : 0;
  a.lab = h->prog.empty() ? 0 : h->prog[0].lab;
  const int64_t tiles = (n_events + PHS_INV_BLOCK - 1) / PHS_INV_BLOCK;
  const int64_t cap = (int64_t)sm_count(h->device) *
                      phs_inverse_blocks_per_sm(a.n_out, a.stack_depth, a.max_visits,
                                                E1 != nullptr, cache, !a.lab);
  CUDA_TRY(phs_launch_inverse(a, (int)std::max<int64_t>(1, std::min(tiles, cap)), st));
  return PHS_OK;
}

// Host path: 512 Ki-event chunks rotate over three streams (measured best on GB300: copies in
// both directions overlap the neighbours' kernels); each stream's buffers are reused only
// after its previous chunk's copies back have been ordered before the next copy in.  The
// first copy in and the last copies back overlap no kernel, so the chunks ramp up from an
// eighth of the size at the start and down to an eighth at the end.
static std::vector<int64_t> host_chunks(int64_t n, int64_t chunk) {
  const int64_t ramp[3] = {chunk / 8, chunk / 4, chunk / 2};
  const int64_t ends = 2 * (ramp[0] + ramp[1] + ramp[2]);
  std::vector<int64_t> out;
  if (ramp[0] < 1 || n < ends + chunk) {
    for (int64_t e0 = 0; e0 < n; e0 += chunk) out.push_back(std::min(chunk, n - e0));
    return out;
  }
  out.assign(ramp, ramp + 3);
  const int64_t mid = n - ends, k = (mid + chunk - 1) / chunk;
  for (int64_t i = 0; i < k; i++) out.push_back(mid / k + (i < mid % k ? 1 : 0));
  out.insert(out.end(), {ramp[2], ramp[1], ramp[0]});
  return out;
}

extern "C" int phs_generate_host(phs_process_t h, int64_t n_events, const int64_t *counts,
                                 const double *x, double *p, double *f, double *v, uint8_t *ok) {
  PHS_TRACE("phs_generate_host");
  return guarded([&]() -> int {
    if (int rc = check_proc(h)) return rc;
    if (!h->beams) return fail(PHS_ERR_STATE, "phs_process_set_beams has not been called");
    if (int rc = check_counts(counts, h->p.n_channels, n_events)) return rc;
    if (n_events > 0 && (!x || !p || !f || !v || !ok)) return fail(PHS_ERR_INVALID_ARG, "null data pointer");
    if (n_events == 0) return PHS_OK;
    DeviceGuard g(h->device);
    const int n_out = h->p.n_out, n_x = h->p.n_x, nch = h->p.n_channels;
    const int64_t chunk = std::min<int64_t>(n_events, 1 << 19);
    for (int s = 0; s < phs_process::kStreams; s++) {
      if (!h->streams[s]) CUDA_TRY(cudaStreamCreateWithFlags(&h->streams[s], cudaStreamNonBlocking));
      int rc;
      if ((rc = h->bx[s].reserve(chunk * n_x * sizeof(double)))) return rc;
      if ((rc = h->bp[s].reserve(chunk * 4 * n_out * sizeof(double)))) return rc;
      if ((rc = h->bf[s].reserve(chunk * sizeof(double)))) return rc;
      if ((rc = h->bv[s].reserve(chunk * sizeof(double)))) return rc;
      if ((rc = h->bo[s].reserve(chunk))) return rc;
    }
    std::vector<int64_t> cnt(nch, 0), prefix(nch + 1, 0);
    if (counts) std::copy(counts, counts + nch, cnt.begin()); else cnt[0] = n_events;
    for (int c = 0; c < nch; c++) prefix[c + 1] = prefix[c] + cnt[c];
    int k = 0;
    int64_t e0 = 0;
    for (const int64_t n : host_chunks(n_events, chunk)) {
      const int s = k++ % phs_process::kStreams;
      cudaStream_t st = h->streams[s];
      // this chunk's per-channel counts
      std::vector<int64_t> cc(nch, 0);
      for (int c = 0; c < nch; c++) {
        int64_t lo = std::max(prefix[c], e0), hi = std::min(prefix[c + 1], e0 + n);
        cc[c] = hi > lo ? hi - lo : 0;
      }
      CUDA_TRY(cudaMemcpyAsync(h->bx[s].ptr, x + e0 * n_x, n * n_x * sizeof(double),
                               cudaMemcpyHostToDevice, st));
      int rc = launch_process(h, h->pseg[s], n, cc.data(), 0, h->bx[s].as<double>(),
                              h->bp[s].as<double>(), h->bf[s].as<double>(), h->bv[s].as<double>(),
                              h->bo[s].as<uint8_t>(), nullptr, nullptr, 1, false, st);
      if (rc) return rc;
      CUDA_TRY(cudaMemcpyAsync(p + e0 * 4 * n_out, h->bp[s].ptr, n * 4 * n_out * sizeof(double),
                               cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaMemcpyAsync(f + e0, h->bf[s].ptr, n * sizeof(double), cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaMemcpyAsync(ok + e0, h->bo[s].ptr, n, cudaMemcpyDeviceToHost, st));
      e0 += n;
    }
    // The volume of an event is its channel's (uniform beams: the kernels write the compiled
    // PhsChannel::volume), so the host writes it while the copies run instead of copying
    // 8 bytes per event back across the host link, which the copies nearly fill.
    for (int c = 0; c < nch; c++) std::fill(v + prefix[c], v + prefix[c + 1], h->prog[c].volume);
    for (int s = 0; s < phs_process::kStreams; s++) CUDA_TRY(cudaStreamSynchronize(h->streams[s]));
    return PHS_OK;
  });
}

// ---------------------------------------------------------------------------- batches
struct phs_batch {
  int device = 0;
  int precision = PHS_PRECISION_F64;
  int ff_variant = -1;
  int f64_variant = -1;
  std::vector<PhsChannel> prog;
  std::vector<PhsChannelFF> prog_ff;
  std::vector<ChanLayout> lay;
  int stack_depth = 0;
  DevBuf d_prog, d_prog_ff;
  Segments segs;
};

extern "C" int phs_batch_create(phs_batch_t *out, int n_procs, const phs_process_t *procs) {
  return guarded([&]() -> int {
    if (!out) return fail(PHS_ERR_INVALID_ARG, "null output handle pointer");
    *out = nullptr;
    if (n_procs < 1 || !procs) return fail(PHS_ERR_INVALID_ARG, "no processes");
    phs_batch *b = new phs_batch;
    cudaGetDevice(&b->device);
    for (int i = 0; i < n_procs; i++) {
      phs_process_t h = procs[i];
      if (!h || !h->beams) {
        delete b;
        return fail(PHS_ERR_STATE, "process %d is null or has no beams set", i);
      }
      b->prog.insert(b->prog.end(), h->prog.begin(), h->prog.end());
      b->prog_ff.insert(b->prog_ff.end(), h->prog_ff.begin(), h->prog_ff.end());
      b->lay.insert(b->lay.end(), h->lay.begin(), h->lay.end());
      b->stack_depth = std::max(b->stack_depth, h->stack_depth);
    }
    DeviceGuard g(b->device);
    int rc = b->d_prog.reserve(b->prog.size() * sizeof(PhsChannel));
    if (rc) { delete b; return rc; }
    rc = b->d_prog_ff.reserve(b->prog_ff.size() * sizeof(PhsChannelFF));
    if (rc) { b->d_prog.release(); delete b; return rc; }
    cudaError_t e = cudaMemcpy(b->d_prog.ptr, b->prog.data(), b->prog.size() * sizeof(PhsChannel),
                               cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(b->d_prog_ff.ptr, b->prog_ff.data(), b->prog_ff.size() * sizeof(PhsChannelFF),
                     cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      b->d_prog.release();
      b->d_prog_ff.release();
      delete b;
      return fail(PHS_ERR_CUDA, "cudaMemcpy of batch programs failed: %s", cudaGetErrorString(e));
    }
    *out = b;
    return PHS_OK;
  });
}

extern "C" int phs_batch_destroy(phs_batch_t b) {
  return guarded([&]() -> int {
    if (!b) return PHS_OK;
    DeviceGuard g(b->device);
    b->d_prog.release();
    b->d_prog_ff.release();
    b->segs.release();
    delete b;
    return PHS_OK;
  });
}

extern "C" int phs_batch_info(phs_batch_t b, int *n_channels, int64_t *x_stride_sum, int *max_n_out) {
  return guarded([&]() -> int {
    if (!b) return fail(PHS_ERR_INVALID_ARG, "null batch handle");
    if (n_channels) *n_channels = (int)b->prog.size();
    int64_t xs = 0;
    int mo = 0;
    for (auto &l : b->lay) { xs += l.x_stride; mo = std::max(mo, l.n_out); }
    if (x_stride_sum) *x_stride_sum = xs;
    if (max_n_out) *max_n_out = mo;
    return PHS_OK;
  });
}

extern "C" int phs_batch_offsets(phs_batch_t b, const int64_t *counts, int64_t *xo, int64_t *po) {
  return guarded([&]() -> int {
    if (!b || !counts || !xo || !po) return fail(PHS_ERR_INVALID_ARG, "null argument");
    const int n = (int)b->prog.size();
    xo[0] = po[0] = 0;
    for (int c = 0; c < n; c++) {
      xo[c + 1] = xo[c] + counts[c] * b->lay[c].x_stride;
      po[c + 1] = po[c] + counts[c] * 4 * b->lay[c].n_out;
    }
    return PHS_OK;
  });
}

extern "C" int phs_batch_generate_device(phs_batch_t b, const int64_t *counts, const double *x,
                                         double *p, double *f, double *v, uint8_t *ok,
                                         void *stream) {
  PHS_TRACE("phs_batch_generate_device");
  return guarded([&]() -> int {
    if (!b) return fail(PHS_ERR_INVALID_ARG, "null batch handle");
    if (!counts) return fail(PHS_ERR_INVALID_ARG, "null counts");
    const int n = (int)b->prog.size();
    int64_t n_events = 0;
    for (int c = 0; c < n; c++) n_events += counts[c] > 0 ? counts[c] : 0;
    if (int rc = check_counts(counts, n, n_events)) return rc;
    if (int rc = check_ptrs(n_events, x, p, f, v, ok)) return rc;
    DeviceGuard g(b->device);
    int rc = build_segments(b->segs, counts, n, b->lay, 0, 0, 0, false);
    if (rc) return rc;
    PhsLaunch a;
    memset(&a, 0, sizeof a);
    a.channels = b->d_prog.as<PhsChannel>();
    a.channels_ff = b->d_prog_ff.as<PhsChannelFF>();
    a.stack_depth = b->stack_depth;
    a.x = x;
    a.p = p;
    a.factor = f;
    a.volume = v;
    a.ok = ok;
    a.factor_stride = 1;
    a.n_programs = n;
    if ((rc = attach_segments(b->segs, a, (cudaStream_t)stream))) return rc;
    if (a.n_tiles == 0) return PHS_OK;
    if (b->precision == PHS_PRECISION_F32X2)
      return launch_ff_tuned(b->ff_variant, b->segs, a, b->device, b->stack_depth, n_events,
                             (cudaStream_t)stream);
    return launch_f64_tuned(b->f64_variant, b->segs, a, b->device, b->stack_depth, n_events,
                            (cudaStream_t)stream);
  });
}

extern "C" int phs_batch_set_variants(phs_batch_t b, int ff_variant, int f64_variant) {
  return guarded([&]() -> int {
    if (!b) return fail(PHS_ERR_INVALID_ARG, "null batch handle");
    if (int rc = check_variants(ff_variant, f64_variant)) return rc;
    b->ff_variant = ff_variant;
    b->f64_variant = f64_variant;
    return PHS_OK;
  });
}

extern "C" int phs_batch_tuning(phs_batch_t b, int *ff_variant, int *f64_variant) {
  return guarded([&]() -> int {
    if (!b) return fail(PHS_ERR_INVALID_ARG, "null batch handle");
    if (ff_variant) *ff_variant = b->ff_variant;
    if (f64_variant) *f64_variant = b->f64_variant;
    return PHS_OK;
  });
}

extern "C" int phs_batch_set_precision(phs_batch_t b, int precision) {
  return guarded([&]() -> int {
    if (!b) return fail(PHS_ERR_INVALID_ARG, "null batch handle");
    if (precision != PHS_PRECISION_F64 && precision != PHS_PRECISION_F32X2)
      return fail(PHS_ERR_INVALID_ARG, "unknown precision mode %d", precision);
    b->precision = precision;
    return PHS_OK;
  });
}

// ------------------------------------------------------- generation without allocation
// For callers that cannot allocate device memory: the channel programs are compiled here
// on the host at the given beams, and the programs and the segment table go into the
// library's file-scope device scratch array (phs_kernels.cu) instead of buffers from
// cudaMalloc.  Nothing on this path calls cudaMalloc, cudaFree or an allocating library
// routine.  At most PHS_NOALLOC_MAX_CHANNELS channels.  The first call on a device
// resolves the scratch array's address (make it before any stream capture).  Calls that
// overlap on the GPU share the scratch array and race.  It always runs the plain FP64
// one-pass kernel (variant 0), whatever precision or variants the handle has set.  Its
// uploads read the host vectors of this call, which are gone when it returns, so a call on
// a stream that is being captured is refused before anything is enqueued.
extern "C" int phs_generate_device_noalloc(phs_process_t h, double E1, double E2,
                                           int64_t n_events, const int64_t *counts,
                                           const double *x, double *p, double *f, double *v,
                                           uint8_t *ok, void *stream) {
  PHS_TRACE("phs_generate_device_noalloc");
  return guarded([&]() -> int {
    if (int rc = check_proc(h)) return rc;
    if (int rc = check_counts(counts, h->p.n_channels, n_events)) return rc;
    if (int rc = check_ptrs(n_events, x, p, f, v, ok)) return rc;
    if (!(E1 > 0) || !(E2 > 0) || !isfinite(E1) || !isfinite(E2))
      return fail(PHS_ERR_INVALID_ARG, "beam energies must be positive and finite");
    const phs::Process &P = h->p;
    if (P.n_channels > PHS_NOALLOC_MAX_CHANNELS)
      return fail(PHS_ERR_UNSUPPORTED, "phs_generate_device_noalloc takes at most %d channels "
                  "(its static device scratch holds %zu bytes); this process has %d",
                  PHS_NOALLOC_MAX_CHANNELS, phs_noalloc_scratch_bytes(), P.n_channels);
    const double sqrts = 2 * sqrt(E1 * E2);
    double m_tot = 0;
    for (int k = 0; k < P.n_out; k++) m_tot += P.flv_m[P.n_in + k];
    if (!(sqrts > m_tot))
      return fail(PHS_ERR_INVALID_ARG, "sqrt(s) = %g is below the final-state mass sum %g", sqrts,
                  m_tot);
    DeviceGuard g(h->device);
    {
      cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
      cudaError_t e = cudaStreamIsCapturing((cudaStream_t)stream, &cap);
      if (e != cudaSuccess)
        return fail(PHS_ERR_CUDA, "phs_generate_device_noalloc: cudaStreamIsCapturing: %s",
                    cudaGetErrorString(e));
      if (cap != cudaStreamCaptureStatusNone)
        return fail(PHS_ERR_UNSUPPORTED, "phs_generate_device_noalloc refuses a stream that is "
                    "being captured: its uploads read host memory that is released when the "
                    "call returns");
    }
    std::vector<PhsChannel> prog(P.n_channels);
    int depth = 0;
    std::string err;
    const double bg = (E1 - E2) / (2 * sqrt(E1 * E2));
    for (int c = 0; c < P.n_channels; c++) {
      phs::ChannelInfo info;
      int rc = phs::compile_channel(P, c, sqrts, prog[c], info, err);
      if (rc) return fail(rc, "%s", err.c_str());
      prog[c].sqrts = sqrts;
      prog[c].lab = E1 != E2;
      prog[c].lab_bg = bg;
      prog[c].lab_gamma = sqrt(1 + bg * bg);
      depth = std::max(depth, info.stack_depth);
    }
    std::vector<ChanLayout> lay(P.n_channels, ChanLayout{P.n_out, P.n_x});
    int64_t one = n_events;
    Segments S;
    int rc = build_segments(S, counts ? counts : &one, P.n_channels, lay, 0, 0, 0, false);
    if (rc) return rc;
    PhsLaunch a;
    memset(&a, 0, sizeof a);
    a.stack_depth = depth;
    a.n_tiles = S.n_tiles;
    a.x = x;
    a.p = p;
    a.factor = f;
    a.volume = v;
    a.ok = ok;
    a.factor_stride = 1;
    a.n_programs = P.n_channels;
    a.x_len = n_events * P.n_x;
    a.p_len = n_events * 4 * (int64_t)P.n_out;
    a.ev_len = n_events;
    if (S.host.size() <= PHS_INLINE_SEGS) std::copy(S.host.begin(), S.host.end(), a.seg_inline);
    const int grid = a.n_tiles > 0 ? grid_for(a.n_tiles, h->device, depth, false, 0) : 1;
    cudaError_t e = phs_launch_forward_f64_noalloc(a, prog.data(), P.n_channels, S.host.data(),
                                                   (int)S.host.size(), grid, (cudaStream_t)stream);
    if (e != cudaSuccess)
      return fail(PHS_ERR_CUDA, "phs_generate_device_noalloc: %s", cudaGetErrorString(e));
    return PHS_OK;
  });
}

// ----------------------------------------------------------------------- CUDA graphs
// A graph holds one generate call with fixed pointers and counts.  Creation runs the call
// once on a private stream (segment table upload, FP32-pair autotuning: everything that
// may synchronize), then captures it; launching replays the kernel with no host work.
struct phs_graph {
  int device = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

template <class Call>
static int capture_graph(phs_graph_t *out, int device, Call call) {
  if (!out) return fail(PHS_ERR_INVALID_ARG, "null output handle pointer");
  *out = nullptr;
  DeviceGuard g(device);
  cudaStream_t st;
  CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  int rc = call(st);
  if (rc == PHS_OK) {
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = fail(PHS_ERR_CUDA, "warm-up run: %s", cudaGetErrorString(e));
  }
  phs_graph *G = nullptr;
  if (rc == PHS_OK) {
    G = new phs_graph;
    G->device = device;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      rc = call(st);
      cudaError_t e2 = cudaStreamEndCapture(st, &G->graph);
      if (rc == PHS_OK && e2 != cudaSuccess)
        rc = fail(PHS_ERR_CUDA, "stream capture: %s", cudaGetErrorString(e2));
    } else {
      rc = fail(PHS_ERR_CUDA, "cudaStreamBeginCapture: %s", cudaGetErrorString(e));
    }
    if (rc == PHS_OK) {
      e = cudaGraphInstantiate(&G->exec, G->graph, 0);
      if (e != cudaSuccess) rc = fail(PHS_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
    }
    if (rc != PHS_OK) {
      if (G->exec) cudaGraphExecDestroy(G->exec);
      if (G->graph) cudaGraphDestroy(G->graph);
      delete G;
      G = nullptr;
    }
  }
  cudaStreamDestroy(st);
  *out = G;
  return rc;
}

extern "C" int phs_batch_graph_create(phs_graph_t *out, phs_batch_t b, const int64_t *counts,
                                      const double *x, double *p, double *f, double *v,
                                      uint8_t *ok) {
  PHS_TRACE("phs_batch_graph_create");
  return guarded([&]() -> int {
    if (!b) return fail(PHS_ERR_INVALID_ARG, "null batch handle");
    return capture_graph(out, b->device, [&](cudaStream_t st) {
      return phs_batch_generate_device(b, counts, x, p, f, v, ok, st);
    });
  });
}

extern "C" int phs_process_graph_create(phs_graph_t *out, phs_process_t h, int64_t n_events,
                                        const int64_t *counts, const double *x, double *p,
                                        double *f, double *v, uint8_t *ok) {
  PHS_TRACE("phs_process_graph_create");
  return guarded([&]() -> int {
    if (int rc = check_proc(h)) return rc;
    return capture_graph(out, h->device, [&](cudaStream_t st) {
      return phs_generate_device(h, n_events, counts, x, p, f, v, ok, st);
    });
  });
}

extern "C" int phs_graph_launch(phs_graph_t G, void *stream) {
  PHS_TRACE("phs_graph_launch");
  return guarded([&]() -> int {
    if (!G) return fail(PHS_ERR_INVALID_ARG, "null graph handle");
    DeviceGuard g(G->device);
    CUDA_TRY(cudaGraphLaunch(G->exec, (cudaStream_t)stream));
    return PHS_OK;
  });
}

extern "C" int phs_graph_destroy(phs_graph_t G) {
  return guarded([&]() -> int {
    if (!G) return PHS_OK;
    DeviceGuard g(G->device);
    if (G->exec) cudaGraphExecDestroy(G->exec);
    if (G->graph) cudaGraphDestroy(G->graph);
    delete G;
    return PHS_OK;
  });
}

// ---------------------------------------------------------------------- random numbers
extern "C" int phs_philox_fill(double *x, int64_t n_events, int n_x, uint64_t seed,
                               int64_t first_event, void *stream) {
  PHS_TRACE("phs_philox_fill");
  return guarded([&]() -> int {
    if (n_events < 0 || n_x < 1 || first_event < 0) return fail(PHS_ERR_INVALID_ARG, "bad sizes");
    if (n_events > 0 && !x) return fail(PHS_ERR_INVALID_ARG, "null x");
    CUDA_TRY(phs_launch_philox(x, n_events, n_x, seed, first_event, (cudaStream_t)stream));
    return PHS_OK;
  });
}

// --------------------------------------------------------------- peak measurement
extern "C" int phs_measure_fma_peak(int fp64, double *gflops) {
  return guarded([&]() -> int {
    if (!gflops) return fail(PHS_ERR_INVALID_ARG, "null output");
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    const int blocks = sm_count(dev) * 8, threads = 256, iters = fp64 ? 4096 : 65536;
    DevBuf out;
    if (int rc = out.reserve((size_t)blocks * threads * 8)) return rc;
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
      CUDA_TRY(cudaEventRecord(e0, nullptr));
      CUDA_TRY(phs_launch_fma_rate(out.ptr, fp64, blocks, threads, iters, nullptr));
      CUDA_TRY(cudaEventRecord(e1, nullptr));
      CUDA_TRY(cudaEventSynchronize(e1));
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) best = std::min(best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    out.release();
    *gflops = 16.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e9;
    return PHS_OK;
  });
}

// -------------------------------------------------------------------- Whizard binding
// Process-global state, as in the reference (global_phs.cpp, whizard_gpu_phs.cpp:10): one
// process per library instance, driven by Whizard's single host thread.
namespace {
// The inverse map of a Whizard call runs in up to this many launches over slices of the
// channels, whose copies back overlap the next slice's kernel.
constexpr int kWhizardSlices = 8;
// The last slice runs in up to this many chunks of events: the factors of a chunk's events
// are final when it ends, and their copy overlaps the next chunk.
constexpr int kWhizardLastChunks = 4;
constexpr int kWhizardLaunches = kWhizardSlices - 1 + kWhizardLastChunks;
// The forward map of a Whizard call runs in up to this many chunks of events, each of at
// least kWhizardChunkMin events (a launch that fills the GPU).
constexpr int kWhizardChunks = 8;
constexpr int64_t kWhizardChunkMin = 1 << 18;
struct Whizard {
  std::mutex mu;
  int n_channels = 0, n_trees = 0, n_groves = 0, n_x = 0, n_in = 0, n_out = 0;
  int n_prt = 0, n_prt_out = 0;
  bool structure = false, flavors = false, mappings = false, trees = false;
  std::vector<double> flv_m, flv_w;
  std::vector<int> map_id, d1, d2, hc, fr;
  std::vector<double> map_m, map_w;
  std::vector<int64_t> counts;  // from init_channel_ids
  int64_t batch_size = 0;
  phs_process_t proc = nullptr;
  DevBuf dx, dp, df, dv, dok;
  DevBuf dfa, dxo;  // all-channel factors and x of the inverse map (more than one channel)
  DevBuf dsparse, din;  // device handoff in the reference's layouts, built on request
  DevBuf dchb;          // per inverse launch, each channel's first event relative to its own
  cudaStream_t streams[4] = {};                 // compute, copies back, compute, copies in
  cudaEvent_t done[kWhizardLaunches + 1] = {};  // the forward map, each inverse launch done
  cudaEvent_t x_in[kWhizardChunks] = {}, fwd[kWhizardChunks] = {};  // per forward chunk
  bool sparse_ok = false, in_ok = false, last_uniform = true;
  double last_e1 = 0, last_e2 = 0;
  std::vector<uint32_t> internal;  // bit code: an internal branch of some channel
  int64_t last_events = 0;
  int msq_threads = 0, cb_threads = 0, ab_threads = 0;
};
Whizard W;

// Whether every event has the first event's beams (the process's compiled constants serve
// them all); large arrays are scanned by several host threads.
bool beams_uniform(const double *E1, const double *E2, int64_t n) {
  auto scan = [&](int64_t lo, int64_t hi) {
    for (int64_t i = lo; i < hi; i++)
      if (E1[i] != E1[0] || E2[i] != E2[0]) return false;
    return true;
  };
  const int64_t per = 1 << 20;
  const int n_threads = (int)std::min<int64_t>(16, (n + per - 1) / per);
  if (n_threads <= 1) return scan(0, n);
  std::vector<char> ok(n_threads, 1);
  std::vector<std::thread> th;
  int started = 1;
  try {
    for (; started < n_threads; started++)
      th.emplace_back([&, started] {
        ok[started] = scan(n * started / n_threads, n * (started + 1) / n_threads);
      });
  } catch (const std::system_error &) {
    // no more threads: this one scans the parts not handed out
  }
  ok[0] = scan(0, n / n_threads);
  for (int t = started; t < n_threads; t++) ok[t] = scan(n * t / n_threads, n * (t + 1) / n_threads);
  for (auto &t : th) t.join();
  return std::all_of(ok.begin(), ok.end(), [](char v) { return v != 0; });
}

// Cuts of the group order of n_channels channels into at most n_slices slices of about
// equal size: at the end of a tree-shape group (group_begin) where one lies within half a
// slice of the even cut, else at the even cut.  Returns the n_slices' + 1 boundaries.
std::vector<int> channel_slices(int n_channels, int n_slices, const std::vector<int32_t> &group_begin) {
  std::vector<int> slice = {0};
  for (int k = 1; k < n_slices; k++) {
    const double want = (double)n_channels * k / n_slices, half = 0.5 * n_channels / n_slices;
    int cut = -1;
    for (int32_t b : group_begin)
      if (b > slice.back() && b < n_channels && (cut < 0 || fabs(b - want) < fabs(cut - want))) cut = b;
    if (cut < 0 || fabs(cut - want) > half) cut = (int)llround(want);
    if (cut > slice.back() && cut < n_channels) slice.push_back(cut);
  }
  slice.push_back(n_channels);
  return slice;
}

void whizard_log(int rc) {
  if (rc) fprintf(stderr, "gpu_phs: %s\n", g_err.c_str());
}

void whizard_release_device() {
  W.dx.release(); W.dp.release(); W.df.release(); W.dv.release(); W.dok.release();
  W.dfa.release(); W.dxo.release();
  W.dsparse.release(); W.din.release(); W.dchb.release();
  W.sparse_ok = W.in_ok = false;
  W.last_events = 0;
}
}  // namespace

extern "C" void c_whizard_set_particle_structure(int *n_channels, int *n_trees, int *n_groves,
                                                 int *n_x, int *n_in, int *n_out) {
  guarded_void([&]() {
    std::lock_guard<std::mutex> lk(W.mu);
    if (!n_channels || !n_trees || !n_groves || !n_x || !n_in || !n_out) {
      whizard_log(fail(PHS_ERR_INVALID_ARG, "c_whizard_set_particle_structure: null argument"));
      return;
    }
    if (*n_out < 2 || *n_out > PHS_MAX_OUT || *n_in < 1 || *n_in > 2 || *n_channels < 1) {
      whizard_log(fail(PHS_ERR_UNSUPPORTED, "c_whizard_set_particle_structure: n_in=%d n_out=%d "
                       "n_channels=%d not supported", *n_in, *n_out, *n_channels));
      return;
    }
    W.n_channels = *n_channels;
    W.n_trees = *n_trees;
    W.n_groves = *n_groves;
    W.n_x = *n_x;
    W.n_in = *n_in;
    W.n_out = *n_out;
    W.n_prt = (1 << (W.n_in + W.n_out)) - 1;
    W.n_prt_out = (1 << W.n_out) - 1;
    W.flv_m.assign(W.n_in + W.n_out, 0.0);
    W.flv_w.assign(W.n_in + W.n_out, 0.0);
    W.structure = true;
    W.flavors = W.mappings = W.trees = false;
  });
}

extern "C" void c_whizard_set_flavors(double *masses, double *widths) {
  guarded_void([&]() {
    std::lock_guard<std::mutex> lk(W.mu);
    if (!W.structure || !masses || !widths) {
      whizard_log(fail(PHS_ERR_STATE, "c_whizard_set_flavors: no particle structure or null input"));
      return;
    }
    std::copy(masses, masses + W.n_in + W.n_out, W.flv_m.begin());
    std::copy(widths, widths + W.n_in + W.n_out, W.flv_w.begin());
    W.flavors = true;
  });
}

extern "C" void c_whizard_init_mappings(void) {
  guarded_void([&]() {
    std::lock_guard<std::mutex> lk(W.mu);
    if (!W.structure) { whizard_log(fail(PHS_ERR_STATE, "c_whizard_init_mappings: no particle structure")); return; }
    const size_t n = (size_t)W.n_channels * W.n_prt_out;
    W.map_id.assign(n, 0);
    W.map_m.assign(n, 0.0);
    W.map_w.assign(n, 0.0);
    W.mappings = true;
  });
}

extern "C" void c_whizard_fill_mapping(int *channel, int *map_ids, double *masses, double *widths) {
  guarded_void([&]() {
    std::lock_guard<std::mutex> lk(W.mu);
    if (!W.mappings || !channel || !map_ids || !masses || !widths || *channel < 1 ||
        *channel > W.n_channels) {
      whizard_log(fail(PHS_ERR_INVALID_ARG, "c_whizard_fill_mapping: bad channel or state"));
      return;
    }
    const size_t o = (size_t)(*channel - 1) * W.n_prt_out;
    std::copy(map_ids, map_ids + W.n_prt_out, W.map_id.begin() + o);
    std::copy(masses, masses + W.n_prt_out, W.map_m.begin() + o);
    std::copy(widths, widths + W.n_prt_out, W.map_w.begin() + o);
  });
}

extern "C" void c_whizard_init_tree_structures(void) {
  guarded_void([&]() {
    std::lock_guard<std::mutex> lk(W.mu);
    if (!W.structure) { whizard_log(fail(PHS_ERR_STATE, "c_whizard_init_tree_structures: no particle structure")); return; }
    const size_t n = (size_t)W.n_channels * W.n_prt;
    W.d1.assign(n, 0);
    W.d2.assign(n, 0);
    W.hc.assign(n, 0);
    W.fr.assign(n, 0);
    W.trees = true;
  });
}

extern "C" void c_whizard_fill_tree_structure(int *channel, int *d1, int *d2, int *hc, int *friends) {
  guarded_void([&]() {
    std::lock_guard<std::mutex> lk(W.mu);
    if (!W.trees || !channel || !d1 || !d2 || !hc || !friends || *channel < 1 ||
        *channel > W.n_channels) {
      whizard_log(fail(PHS_ERR_INVALID_ARG, "c_whizard_fill_tree_structure: bad channel or state"));
      return;
    }
    const size_t o = (size_t)(*channel - 1) * W.n_prt;
    std::copy(d1, d1 + W.n_prt, W.d1.begin() + o);
    std::copy(d2, d2 + W.n_prt, W.d2.begin() + o);
    std::copy(hc, hc + W.n_prt, W.hc.begin() + o);
    std::copy(friends, friends + W.n_prt, W.fr.begin() + o);
  });
}

// channel_limits[c] is the cumulative number of events up to and including channel c; events
// are grouped by channel (whizard_gpu_phs.cpp:89-98).  Empty channels anywhere are allowed.
extern "C" void c_whizard_init_channel_ids(int *batch_size, int *n_channels, int *channel_limits) {
  guarded_void([&]() {
    std::lock_guard<std::mutex> lk(W.mu);
    if (!batch_size || !n_channels || !channel_limits || *n_channels < 1 || *batch_size < 0) {
      whizard_log(fail(PHS_ERR_INVALID_ARG, "c_whizard_init_channel_ids: bad arguments"));
      return;
    }
    W.counts.assign(*n_channels, 0);
    int64_t prev = 0;
    for (int c = 0; c < *n_channels; c++) {
      int64_t lim = std::min<int64_t>(channel_limits[c], *batch_size);
      W.counts[c] = std::max<int64_t>(0, lim - prev);
      prev = std::max(prev, lim);
    }
    W.batch_size = *batch_size;
  });
}

extern "C" void c_whizard_set_threads(int *msq_threads, int *cb_threads, int *ab_threads) {
  guarded_void([&]() {
    std::lock_guard<std::mutex> lk(W.mu);
    W.msq_threads = msq_threads ? *msq_threads : 0;
    W.cb_threads = cb_threads ? *cb_threads : 0;
    W.ab_threads = ab_threads ? *ab_threads : 0;
  });
}

extern "C" void c_whizard_init_gpu_phs(void) {
  guarded_void([&]() {
    std::lock_guard<std::mutex> lk(W.mu);
    if (!W.structure || !W.flavors || !W.mappings || !W.trees) {
      whizard_log(fail(PHS_ERR_STATE, "c_whizard_init_gpu_phs: structure, flavors, mappings and "
                       "trees must be set first"));
      return;
    }
    if (W.proc) { phs_process_destroy(W.proc); W.proc = nullptr; }
    // codes of internal branches over all channels, for the sparse momentum handoff
    W.internal.assign((1 << PHS_SPARSE_MAX_OUT) / 32, 0u);
    for (int c = 0; c < W.n_channels && W.n_out <= PHS_SPARSE_MAX_OUT; c++)
      for (int code = 1; code < (1 << W.n_out); code++)
        if (W.hc[(size_t)c * W.n_prt + code - 1]) W.internal[code >> 5] |= 1u << (code & 31);
    whizard_log(phs_process_create(&W.proc, W.n_in, W.n_out, W.n_channels, W.n_x, W.d1.data(),
                                   W.d2.data(), W.hc.data(), W.fr.data(), W.map_id.data(),
                                   W.map_m.data(), W.map_w.data(), W.flv_m.data(), W.flv_w.data()));
  });
}

extern "C" void c_whizard_finalize_gpu_phs(void) {
  guarded_void([&]() {
    std::lock_guard<std::mutex> lk(W.mu);
    if (W.proc) phs_process_destroy(W.proc);
    W.proc = nullptr;
    whizard_release_device();
    for (cudaStream_t &st : W.streams) {
      if (st) cudaStreamDestroy(st);
      st = nullptr;
    }
    for (cudaEvent_t *evs : {W.done, W.x_in, W.fwd}) {
      const int m = evs == W.done ? kWhizardLaunches + 1 : kWhizardChunks;
      for (int i = 0; i < m; i++) {
        if (evs[i]) cudaEventDestroy(evs[i]);
        evs[i] = nullptr;
      }
    }
    W.map_id.clear(); W.map_m.clear(); W.map_w.clear();
    W.d1.clear(); W.d2.clear(); W.hc.clear(); W.fr.clear();
    W.flv_m.clear(); W.flv_w.clear();
    W.counts.clear();
    W.structure = W.flavors = W.mappings = W.trees = false;
  });
}

extern "C" void c_whizard_gen_phs_from_x_gpu(double *E1_in, double *E2_in,
                                             bool *requires_boost_to_lab, int *n_events_p,
                                             int *n_channels_p, int *n_x_p, double *x,
                                             double *factors, double *volumes, bool *oks,
                                             double *p, double *x_out) {
  PHS_TRACE("c_whizard_gen_phs_from_x_gpu");
  (void)requires_boost_to_lab;  // stored but unused by the reference (phs.cu:1559)
  std::lock_guard<std::mutex> lk(W.mu);
  g_err.clear();  // the call returns nothing: phs_last_error() reports this call alone
  int rc = PHS_OK;
  try {  // nothing may leave a C entry point by an exception
    do {
      if (!W.proc) { rc = fail(PHS_ERR_STATE, "c_whizard_gen_phs_from_x_gpu: init_gpu_phs not done"); break; }
      if (!n_events_p || !n_channels_p || !n_x_p || !E1_in || !E2_in) {
        rc = fail(PHS_ERR_INVALID_ARG, "c_whizard_gen_phs_from_x_gpu: null argument");
        break;
      }
      const int64_t n = *n_events_p;
      const int nch = *n_channels_p, n_x = *n_x_p, n_out = W.n_out;
      if (nch != W.n_channels || n_x != W.n_x) {
        rc = fail(PHS_ERR_INVALID_ARG, "n_channels/n_x differ from the particle structure");
        break;
      }
      if (n < 0) { rc = fail(PHS_ERR_INVALID_ARG, "n_events = %lld < 0", (long long)n); break; }
      if (n == 0) break;
      if (!x || !factors || !volumes || !oks || !p) { rc = fail(PHS_ERR_INVALID_ARG, "null data pointer"); break; }
      std::vector<int64_t> counts = W.counts;
      int64_t sum = 0;
      for (auto c : counts) sum += c;
      if (counts.size() != (size_t)nch || sum != n) {
        rc = fail(PHS_ERR_INVALID_ARG, "channel ids from c_whizard_init_channel_ids cover %lld "
                  "events, not %lld", (long long)sum, (long long)n);
        break;
      }
      const bool uniform = beams_uniform(E1_in, E2_in, n);
      DeviceGuard g(W.proc->device);
      if ((rc = W.dx.reserve(n * n_x * sizeof(double)))) break;
      if ((rc = W.dp.reserve(n * 4 * n_out * sizeof(double)))) break;
      if ((rc = W.df.reserve(n * sizeof(double) * (uniform ? 1 : 3)))) break;
      if ((rc = W.dv.reserve(n * sizeof(double)))) break;
      if ((rc = W.dok.reserve(n))) break;
      if (nch > 1 && (rc = W.dfa.reserve((size_t)n * nch * sizeof(double)))) break;
      if (nch > 1 && (rc = W.dxo.reserve((size_t)nch * n * n_x * sizeof(double)))) break;
      if (uniform && (rc = phs_process_set_beams(W.proc, E1_in[0], E2_in[0]))) break;
      cudaError_t e = cudaSuccess;
      for (int i = 0; i < 4 && e == cudaSuccess; i++)
        if (!W.streams[i]) e = cudaStreamCreateWithFlags(&W.streams[i], cudaStreamNonBlocking);
      for (int i = 0; i <= kWhizardLaunches && e == cudaSuccess; i++)
        if (!W.done[i]) e = cudaEventCreateWithFlags(&W.done[i], cudaEventDisableTiming);
      for (int i = 0; i < kWhizardChunks && e == cudaSuccess; i++) {
        if (!W.x_in[i]) e = cudaEventCreateWithFlags(&W.x_in[i], cudaEventDisableTiming);
        if (e == cudaSuccess && !W.fwd[i]) e = cudaEventCreateWithFlags(&W.fwd[i], cudaEventDisableTiming);
      }
      if (e != cudaSuccess) { rc = fail(PHS_ERR_CUDA, "set-up: %s", cudaGetErrorString(e)); break; }
      cudaStream_t cs[2] = {W.streams[0], W.streams[2]}, ms = W.streams[1], hs = W.streams[3];
      double *dx = W.dx.as<double>(), *dp = W.dp.as<double>(), *df = W.df.as<double>();
      double *dv = W.dv.as<double>(), *dxo = W.dxo.as<double>();
      uint8_t *dok = W.dok.as<uint8_t>();
      const double *dE1 = uniform ? nullptr : df + n, *dE2 = uniform ? nullptr : df + 2 * n;
      // The forward map in chunks of events: the copies in of the next chunks (on their own
      // stream) and the copies back of chunk k - 1 (momenta, volumes, ok flags; with one
      // channel also its x and factors, which are the input's and the forward map's) run
      // beside the kernels of chunk k.
      const int64_t fchunk = std::max<int64_t>(kWhizardChunkMin, (n + kWhizardChunks - 1) / kWhizardChunks);
      const int n_fchunks = (int)((n + fchunk - 1) / fchunk);
      std::vector<int64_t> beg(nch, 0), fcnt((size_t)n_fchunks * nch, 0);
      for (int c = 1; c < nch; c++) beg[c] = beg[c - 1] + counts[c - 1];
      for (int c = 0; c < nch; c++)
        for (int k = 0; k < n_fchunks; k++) {
          const int64_t e0 = k * fchunk, e1 = std::min(n, e0 + fchunk);
          fcnt[(size_t)k * nch + c] =
              std::max<int64_t>(0, std::min(e1, beg[c] + counts[c]) - std::max(e0, beg[c]));
        }
      auto copy_in = [&](int k) -> cudaError_t {
        const int64_t e0 = k * fchunk, nk = std::min(n, e0 + fchunk) - e0;
        cudaError_t ee = cudaMemcpyAsync(dx + e0 * n_x, x + e0 * n_x, nk * n_x * sizeof(double),
                                         cudaMemcpyHostToDevice, hs);
        if (ee == cudaSuccess && !uniform)
          ee = cudaMemcpyAsync(df + n + e0, E1_in + e0, nk * sizeof(double), cudaMemcpyHostToDevice, hs);
        if (ee == cudaSuccess && !uniform)
          ee = cudaMemcpyAsync(df + 2 * n + e0, E2_in + e0, nk * sizeof(double), cudaMemcpyHostToDevice, hs);
        return ee == cudaSuccess ? cudaEventRecord(W.x_in[k], hs) : ee;
      };
      auto forward = [&](int k) -> int {
        const int64_t e0 = k * fchunk, nk = std::min(n, e0 + fchunk) - e0;
        const int64_t *ck = fcnt.data() + (size_t)k * nch;
        cudaError_t ee = cudaStreamWaitEvent(cs[0], W.x_in[k], 0);
        if (ee != cudaSuccess) return fail(PHS_ERR_CUDA, "%s", cudaGetErrorString(ee));
        int r = uniform
            ? phs_generate_device(W.proc, nk, ck, dx + e0 * n_x, dp + e0 * 4 * n_out, df + e0,
                                  dv + e0, dok + e0, cs[0])
            : phs_generate_beams_device(W.proc, nk, ck, dE1 + e0, dE2 + e0, dx + e0 * n_x,
                                        dp + e0 * 4 * n_out, df + e0, dv + e0, dok + e0, cs[0]);
        if (r) return r;
        ee = cudaEventRecord(W.fwd[k], cs[0]);
        return ee == cudaSuccess ? PHS_OK : fail(PHS_ERR_CUDA, "%s", cudaGetErrorString(ee));
      };
      auto copy_back = [&](int k) -> cudaError_t {
        const int64_t e0 = k * fchunk, nk = std::min(n, e0 + fchunk) - e0;
        cudaError_t ee = cudaStreamWaitEvent(ms, W.fwd[k], 0);
        if (ee == cudaSuccess)
          ee = cudaMemcpyAsync(p + e0 * 4 * n_out, dp + e0 * 4 * n_out, nk * 4 * n_out * sizeof(double),
                               cudaMemcpyDeviceToHost, ms);
        if (ee == cudaSuccess)
          ee = cudaMemcpyAsync(volumes + e0, dv + e0, nk * sizeof(double), cudaMemcpyDeviceToHost, ms);
        if (ee == cudaSuccess) ee = cudaMemcpyAsync(oks + e0, dok + e0, nk, cudaMemcpyDeviceToHost, ms);
        // one channel: the generating channel keeps its own x and factor (phs.cu:1580-1585)
        if (ee == cudaSuccess && nch == 1 && x_out)
          ee = cudaMemcpyAsync(x_out + e0 * n_x, dx + e0 * n_x, nk * n_x * sizeof(double),
                               cudaMemcpyDeviceToHost, ms);
        if (ee == cudaSuccess && nch == 1)
          ee = cudaMemcpyAsync(factors + e0, df + e0, nk * sizeof(double), cudaMemcpyDeviceToHost, ms);
        return ee;
      };
      // With more than one chunk the copies in run on a helper thread (a copy from pageable
      // memory holds its thread until done), so that they overlap the copies back, which this
      // thread issues; chunk k's kernels are queued once its copy in is.
      std::mutex in_mu;
      std::condition_variable in_cv;
      int in_queued = 0;
      cudaError_t in_err = cudaSuccess;
      std::atomic<bool> in_stop{false};
      std::thread loader;
      bool threaded = false;
      if (n_fchunks > 1) {
        const int dev = W.proc->device;
        try {
          loader = std::thread([&, dev] {
            cudaError_t ee = cudaSetDevice(dev);
            for (int k = 0; k < n_fchunks && ee == cudaSuccess && !in_stop.load(); k++) {
              ee = copy_in(k);
              std::lock_guard<std::mutex> lk(in_mu);
              if (ee == cudaSuccess) in_queued = k + 1;
              in_cv.notify_all();
            }
            std::lock_guard<std::mutex> lk(in_mu);
            in_err = ee;
            if (ee == cudaSuccess && in_queued < n_fchunks) in_err = cudaErrorNotReady;  // stopped
            in_cv.notify_all();
          });
          threaded = true;
        } catch (const std::system_error &) {
          // no helper thread: this thread copies each chunk in before its kernels
        }
      }
      auto wait_in = [&](int k) -> cudaError_t {
        if (!threaded) return copy_in(k);
        std::unique_lock<std::mutex> lk(in_mu);
        in_cv.wait(lk, [&] { return in_queued > k || in_err != cudaSuccess; });
        return in_queued > k ? cudaSuccess : in_err;
      };
      try {  // the helper thread is joined below whatever happens here
        for (int k = 0; k < n_fchunks && rc == PHS_OK; k++) {
          if ((e = wait_in(k)) != cudaSuccess) { rc = fail(PHS_ERR_CUDA, "copy in: %s", cudaGetErrorString(e)); break; }
          if ((rc = forward(k))) break;
          if (k > 0 && (e = copy_back(k - 1)) != cudaSuccess)
            rc = fail(PHS_ERR_CUDA, "copy back: %s", cudaGetErrorString(e));
        }
      } catch (const std::exception &ex) {
        rc = fail(PHS_ERR_ALLOC, "host: %s", ex.what());
      }
      if (rc) in_stop = true;
      if (loader.joinable()) loader.join();
      if (rc) {
        cudaStreamSynchronize(hs);
        cudaStreamSynchronize(cs[0]);
        cudaStreamSynchronize(ms);
        break;
      }
      // More than one channel: the inverse map (factors [n][n_channels], x [n_channels][n][n_x])
      // in launches over slices of the channels in the order of the tree-shape groups (cut
      // where a group ends, if one ends near the even cut: the geometry of a shape is computed
      // once per event and launch), each over every event so that it fills the GPU, the last
      // slice in chunks of events; the launches alternate over two compute streams, so that
      // one's tail overlaps the next one's start.  They are queued before the last forward
      // chunk's copies back; the copies of each launch's x rows (contiguous per channel on both
      // sides) then run beside the later kernels, and after each chunk of the last slice the
      // factors of its events, which every earlier launch has finished.
      struct Unit { int lo, hi; int64_t e0, e1; };
      std::vector<Unit> units;
      if (nch > 1) {
        if ((int)W.proc->inv_group_begin.size() < 2 || (int)W.proc->inv_order.size() != nch) {
          rc = fail(PHS_ERR_STATE, "inverse map: channel groups not built");
          cudaStreamSynchronize(cs[0]);
          cudaStreamSynchronize(ms);
          break;
        }
        const std::vector<int> slice = channel_slices(
            nch, (int64_t)n * nch < (1 << 20) ? 1 : std::min(nch, kWhizardSlices),
            W.proc->inv_group_begin);
        const int n_slices = (int)slice.size() - 1;
        for (int k = 0; k + 1 < n_slices; k++) units.push_back({slice[k], slice[k + 1], 0, n});
        const int n_last =
            n_slices > 1 ? (int)std::min<int64_t>(kWhizardLastChunks, std::max<int64_t>(1, n >> 15)) : 1;
        for (int j = 0; j < n_last; j++)
          units.push_back({slice[n_slices - 1], nch, n * j / n_last, n * (j + 1) / n_last});
        // channel starts relative to each launch's first event
        std::vector<int64_t> begs((size_t)units.size() * nch);
        for (size_t u = 0; u < units.size(); u++)
          for (int c = 0; c < nch; c++) begs[u * nch + c] = beg[c] - units[u].e0;
        if ((rc = W.dchb.reserve(begs.size() * sizeof(int64_t)))) { cudaStreamSynchronize(cs[0]); break; }
        e = cudaMemcpyAsync(W.dchb.ptr, begs.data(), begs.size() * sizeof(int64_t), cudaMemcpyHostToDevice, cs[0]);
        if (e == cudaSuccess) e = cudaEventRecord(W.done[0], cs[0]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(cs[1], W.done[0], 0);
        if (e != cudaSuccess) rc = fail(PHS_ERR_CUDA, "%s", cudaGetErrorString(e));
        // do_inverse_mapping is forced on (whizard_gpu_phs.cpp:118): every channel's factor
        // and x; the generating channel keeps its own x and factor (phs.cu:1580-1585), written
        // with the other no-arithmetic outputs by the first launch (over every event)
        for (size_t u = 0; u < units.size() && rc == PHS_OK; u++) {
          const Unit &U = units[u];
          const int64_t e0 = U.e0;
          rc = inverse_launch(W.proc, U.e1 - e0, W.dchb.as<int64_t>() + u * nch,
                              uniform ? nullptr : dE1 + e0, uniform ? nullptr : dE2 + e0,
                              dp + e0 * 4 * n_out, dok + e0, dx + e0 * n_x, df + e0,
                              W.dfa.as<double>() + e0 * nch, dxo + e0 * n_x, cs[u & 1], U.lo, U.hi,
                              u == 0, n);
          if (rc == PHS_OK && (e = cudaEventRecord(W.done[u + 1], cs[u & 1])) != cudaSuccess)
            rc = fail(PHS_ERR_CUDA, "%s", cudaGetErrorString(e));
        }
      }
      if (rc == PHS_OK && (e = copy_back(n_fchunks - 1)) != cudaSuccess)
        rc = fail(PHS_ERR_CUDA, "copy back: %s", cudaGetErrorString(e));
      const int32_t *order = W.proc->inv_order.data();
      // the copy stream waits for the launches in order: launch u's rows are copied after
      // every launch up to u (the first one's fixed outputs included) is done
      for (size_t u = 0; u < units.size() && rc == PHS_OK && e == cudaSuccess; u++) {
        const Unit &U = units[u];
        e = cudaStreamWaitEvent(ms, W.done[u + 1], 0);
        // device rows sit where the caller's do: a run of channels whose ids step evenly
        // goes as one strided copy (one copy per row costs far more than its bytes)
        const size_t width = (size_t)(U.e1 - U.e0) * n_x * sizeof(double);
        for (int i = U.lo; i < U.hi && e == cudaSuccess && x_out;) {
          const int step = i + 1 < U.hi ? order[i + 1] - order[i] : 0;
          int j = i + 1;
          if (step > 0)
            while (j < U.hi && order[j] - order[j - 1] == step) j++;
          const size_t pitch = step > 0 ? (size_t)step * n * n_x * sizeof(double) : width;
          const size_t off = ((size_t)order[i] * n + U.e0) * n_x;
          e = cudaMemcpy2DAsync(x_out + off, pitch, dxo + off, pitch, width, j - i,
                                cudaMemcpyDeviceToHost, ms);
          i = j;
        }
        if (e == cudaSuccess && U.hi == nch)
          e = cudaMemcpyAsync(factors + U.e0 * nch, W.dfa.as<double>() + U.e0 * nch,
                              (size_t)(U.e1 - U.e0) * nch * sizeof(double), cudaMemcpyDeviceToHost, ms);
        if (e != cudaSuccess) rc = fail(PHS_ERR_CUDA, "copy back: %s", cudaGetErrorString(e));
      }
      if (rc == PHS_OK && (e = cudaStreamSynchronize(ms)) != cudaSuccess)
        rc = fail(PHS_ERR_CUDA, "copy back: %s", cudaGetErrorString(e));
      if (rc) {
        for (cudaStream_t st : W.streams) cudaStreamSynchronize(st);
        break;
      }
      W.last_events = n;
      W.sparse_ok = W.in_ok = false;  // the handoff buffers are rebuilt on request
      W.last_uniform = uniform;
      W.last_e1 = E1_in[0];
      W.last_e2 = E2_in[0];
    } while (0);
  } catch (const std::exception &ex) {
    rc = fail(PHS_ERR_ALLOC, "c_whizard_gen_phs_from_x_gpu: %s", ex.what());
    for (cudaStream_t st : W.streams)
      if (st) cudaStreamSynchronize(st);
  }
  whizard_log(rc);
}

extern "C" void c_whizard_get_momentum_device_pointer(double *p) { (void)p; }

extern "C" double *phs_whizard_momentum_device_pointer(void) {
  std::lock_guard<std::mutex> lk(W.mu);
  return W.last_events ? W.dp.as<double>() : nullptr;
}

// The device handoff of the reference's transfer_to_whizard.h (C++ linkage, as there):
// the last c_whizard_gen_phs_from_x_gpu call's momenta in the sparse Whizard layout, its
// beam energies [E1...; E2...] and its ok flags, in device memory the library owns until
// the next call, c_whizard_reset_generator or c_whizard_finalize_gpu_phs.  Null before the
// first call or on error (phs_last_error).
double *get_momentum_device_pointer() {
  std::lock_guard<std::mutex> lk(W.mu);
  if (!W.last_events || !W.proc) return nullptr;
  if (W.sparse_ok) return W.dsparse.as<double>();
  if (W.n_out > PHS_SPARSE_MAX_OUT) {
    whizard_log(fail(PHS_ERR_UNSUPPORTED, "sparse momentum layout: n_out > %d", PHS_SPARSE_MAX_OUT));
    return nullptr;
  }
  DeviceGuard g(W.proc->device);
  const int64_t n = W.last_events;
  int rc = W.dsparse.reserve((size_t)n * W.n_prt * 4 * sizeof(double));
  if (rc) { whizard_log(rc); return nullptr; }
  PhsSparseLaunch a;
  memset(&a, 0, sizeof a);
  a.p = W.dp.as<double>();
  a.E1 = W.last_uniform ? nullptr : W.df.as<double>() + n;
  a.E2 = W.last_uniform ? nullptr : W.df.as<double>() + 2 * n;
  a.e1 = W.last_e1;
  a.e2 = W.last_e2;
  a.out = W.dsparse.as<double>();
  a.n_events = n;
  a.n_out = W.n_out;
  a.n_prt = W.n_prt;
  std::copy(W.internal.begin(), W.internal.end(), a.internal);
  cudaError_t e = phs_launch_whizard_sparse(a, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    whizard_log(fail(PHS_ERR_CUDA, "sparse momentum layout: %s", cudaGetErrorString(e)));
    return nullptr;
  }
  W.sparse_ok = true;
  return W.dsparse.as<double>();
}

double *get_in_momentum_device_pointer() {
  std::lock_guard<std::mutex> lk(W.mu);
  if (!W.last_events || !W.proc) return nullptr;
  const int64_t n = W.last_events;
  if (!W.last_uniform) return W.df.as<double>() + n;  // [E1; E2] as the per-event launch read them
  if (W.in_ok) return W.din.as<double>();
  DeviceGuard g(W.proc->device);
  int rc = W.din.reserve((size_t)2 * n * sizeof(double));
  if (rc) { whizard_log(rc); return nullptr; }
  std::vector<double> h((size_t)2 * n, W.last_e1);
  std::fill(h.begin() + n, h.end(), W.last_e2);
  cudaError_t e = cudaMemcpy(W.din.ptr, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    whizard_log(fail(PHS_ERR_CUDA, "beam energies: %s", cudaGetErrorString(e)));
    return nullptr;
  }
  W.in_ok = true;
  return W.din.as<double>();
}

bool *get_ok_device_pointer() {
  std::lock_guard<std::mutex> lk(W.mu);
  return W.last_events ? reinterpret_cast<bool *>(W.dok.ptr) : nullptr;
}

extern "C" void c_whizard_reset_generator(void) {
  guarded_void([&]() {
    std::lock_guard<std::mutex> lk(W.mu);
    // phs.cu:1303-1308: drops the flavors and the retained device buffers
    std::fill(W.flv_m.begin(), W.flv_m.end(), 0.0);
    std::fill(W.flv_w.begin(), W.flv_w.end(), 0.0);
    W.flavors = false;
    whizard_release_device();
  });
}

extern "C" void c_whizard_show_module(void) {
  guarded_void([&]() {
    std::lock_guard<std::mutex> lk(W.mu);
    printf("n_channels: %d\n", W.n_channels);
    printf("n_ext_in: %d\n", W.n_in);
    printf("n_ext_out: %d\n", W.n_out);
    printf("n_ext_tot: %d\n", W.n_in + W.n_out);
    printf("n_prt: %d\n", W.n_prt);
    printf("n_prt_out: %d\n", W.n_prt_out);
    printf("n_x: %d\n", W.n_x);
    printf("root_branch: %d\n", W.n_prt_out - 1);
    printf("n_branches: %d\n", 2 * W.n_out - 1);
    printf("\nMappings: \n");
    if (!W.mappings) {
      printf(" MAPPINGS NOT SET UP!\n");
      return;
    }
    for (int c = 0; c < W.n_channels; c++) {
      printf(" c: %d\n ids: ", c);
      for (int i = 0; i < W.n_prt_out; i++) printf("%d ", W.map_id[(size_t)c * W.n_prt_out + i]);
      printf("\n masses: ");
      for (int i = 0; i < W.n_prt_out; i++) printf("%lf ", W.map_m[(size_t)c * W.n_prt_out + i]);
      printf("\n widths: ");
      for (int i = 0; i < W.n_prt_out; i++) printf("%lf ", W.map_w[(size_t)c * W.n_prt_out + i]);
      printf("\n");
    }
    if (W.trees) {
      printf("Children: \n");
      for (int c = 0; c < W.n_channels; c++) {
        for (auto *t : {&W.d1, &W.d2, &W.hc}) {
          for (int i = 0; i < W.n_prt; i++) printf("%d ", (*t)[(size_t)c * W.n_prt + i]);
          printf("\n");
        }
      }
      printf("Friends: \n");
      for (int c = 0; c < W.n_channels; c++) {
        printf("channel %d: ", c);
        for (int i = 0; i < W.n_prt; i++) printf("%d ", W.fr[(size_t)c * W.n_prt + i]);
        printf("\n");
      }
    }
    if (W.proc && W.proc->beams) {
      printf("Visit programs (sqrt(s) = %g): \n", W.proc->prog[0].sqrts);
      for (int c = 0; c < W.n_channels; c++) {
        const PhsChannel &ch = W.proc->prog[c];
        printf("  channel %d: %d visits, volume %.17g\n", c, ch.n_visits, ch.volume);
        for (int v = 0; v < ch.n_visits; v++) {
          const PhsVisit &V = ch.visit[v];
          printf("    visit %d: x_phi %d x_ct %d ct_class %d carry %d push %d children", v, V.x_phi,
                 V.x_ct, V.ct_class, V.carry, V.push);
          for (int j = 0; j < 2; j++) {
            const PhsChild &C = V.child[j];
            if (C.internal) printf(" [map %d x %d]", C.map_id, C.x_msq);
            else printf(" [leaf %d]", C.out_index);
          }
          printf("\n");
        }
      }
    }
    printf("END OF MODULE\n");
  });
}

// -------------------------------------------------------------------------- x grids
struct phs_grid {
  int device = 0;
  int n_channels = 0, n_x = 0;
  DevBuf weights, bins, n_ok, ch_begin;
  std::vector<int64_t> ch_begin_up;
};

extern "C" int phs_grid_create(phs_grid_t *out, int n_channels, int n_x) {
  return guarded([&]() -> int {
    if (!out) return fail(PHS_ERR_INVALID_ARG, "null output handle pointer");
    *out = nullptr;
    if (n_channels < 1 || n_x < 1) return fail(PHS_ERR_INVALID_ARG, "n_channels and n_x must be >= 1");
    phs_grid *g = new phs_grid;
    cudaGetDevice(&g->device);
    g->n_channels = n_channels;
    g->n_x = n_x;
    const size_t nb = (size_t)n_channels * n_x * PHS_GRID_BINS;
    int rc = g->weights.reserve(nb * sizeof(double));
    if (!rc) rc = g->bins.reserve(nb * sizeof(unsigned long long));
    if (!rc) rc = g->n_ok.reserve(n_channels * sizeof(unsigned long long));
    if (rc) { delete g; return rc; }
    std::vector<double> w(nb, 1.0 / PHS_GRID_BINS);   // rng.cpp:19-29: uniform start
    cudaError_t e = cudaMemcpy(g->weights.ptr, w.data(), nb * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      delete g;
      return fail(PHS_ERR_CUDA, "grid upload: %s", cudaGetErrorString(e));
    }
    *out = g;
    return PHS_OK;
  });
}

extern "C" int phs_grid_destroy(phs_grid_t g) {
  return guarded([&]() -> int {
    if (!g) return PHS_OK;
    DeviceGuard dg(g->device);
    g->weights.release();
    g->bins.release();
    g->n_ok.release();
    g->ch_begin.release();
    delete g;
    return PHS_OK;
  });
}

static int grid_channels(phs_grid_t g, int64_t n_events, const int64_t *counts, cudaStream_t st) {
  if (int rc = check_counts(counts, g->n_channels, n_events)) return rc;
  std::vector<int64_t> begin(g->n_channels, 0);
  for (int c = 1; c < g->n_channels; c++) begin[c] = begin[c - 1] + (counts ? counts[c - 1] : n_events);
  if (begin != g->ch_begin_up) {
    if (int rc = g->ch_begin.reserve(g->n_channels * sizeof(int64_t))) return rc;
    CUDA_TRY(cudaMemcpyAsync(g->ch_begin.ptr, begin.data(), g->n_channels * sizeof(int64_t),
                             cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    g->ch_begin_up = begin;
  }
  return PHS_OK;
}

extern "C" int phs_grid_sample_device(phs_grid_t g, int64_t n_events, const int64_t *counts,
                                      uint64_t seed, int64_t first_event, double *x,
                                      void *stream) {
  PHS_TRACE("phs_grid_sample_device");
  return guarded([&]() -> int {
    if (!g) return fail(PHS_ERR_INVALID_ARG, "null grid handle");
    if (n_events > 0 && !x) return fail(PHS_ERR_INVALID_ARG, "null x");
    DeviceGuard dg(g->device);
    cudaStream_t st = (cudaStream_t)stream;
    if (int rc = grid_channels(g, n_events, counts, st)) return rc;
    if (n_events == 0) return PHS_OK;
    CUDA_TRY(phs_launch_philox(x, n_events, g->n_x, seed, first_event, st));
    CUDA_TRY(phs_launch_grid_sample(x, n_events, g->n_x, g->ch_begin.as<int64_t>(), g->n_channels,
                                    g->weights.as<double>(), sm_count(g->device), st));
    return PHS_OK;
  });
}

extern "C" int phs_grid_update_device(phs_grid_t g, int64_t n_events, const int64_t *counts,
                                      const double *x, const uint8_t *oks, void *stream) {
  PHS_TRACE("phs_grid_update_device");
  return guarded([&]() -> int {
    if (!g) return fail(PHS_ERR_INVALID_ARG, "null grid handle");
    if (n_events > 0 && (!x || !oks)) return fail(PHS_ERR_INVALID_ARG, "null data pointer");
    DeviceGuard dg(g->device);
    cudaStream_t st = (cudaStream_t)stream;
    if (int rc = grid_channels(g, n_events, counts, st)) return rc;
    CUDA_TRY(phs_launch_grid_update(x, oks, n_events, g->n_x, g->ch_begin.as<int64_t>(),
                                    g->n_channels, g->bins.as<unsigned long long>(),
                                    g->n_ok.as<unsigned long long>(), g->weights.as<double>(),
                                    sm_count(g->device), st));
    return PHS_OK;
  });
}

extern "C" int phs_grid_weights(phs_grid_t g, double *weights) {
  return guarded([&]() -> int {
    if (!g || !weights) return fail(PHS_ERR_INVALID_ARG, "null argument");
    DeviceGuard dg(g->device);
    CUDA_TRY(cudaMemcpy(weights, g->weights.ptr,
                        (size_t)g->n_channels * g->n_x * PHS_GRID_BINS * sizeof(double),
                        cudaMemcpyDeviceToHost));
    return PHS_OK;
  });
}
