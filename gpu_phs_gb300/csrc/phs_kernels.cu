// phs_kernels.cu -- fused forward phase-space kernel (FP64) and the Philox x generator.
//
// One persistent kernel per batch.  Each warp takes 32-event tiles of one channel (tiles
// never straddle channels, so every branch of the visit program is warp-uniform); each
// thread walks its event's visit program top-down (phs_program.h) with the running 4x4
// boost in registers and at most two saved frames on a per-thread shared-memory stack.
//
// The per-event arithmetic is in phs_event_f64.cuh.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <mutex>

#include "phs_device.h"
#include "phs_event_f64.cuh"
#include "phs_program.h"

namespace {

// The sin/cos table sits after the frame stack and the queues (phs_forward_smem_bytes).
template <int BLOCK = PHS_FWD_BLOCK>
__device__ __forceinline__ double2 *phs_trig_table(double *smem, int stack_depth) {
  return reinterpret_cast<double2 *>(smem + (size_t)stack_depth * PHS_STATE * BLOCK +
                                     (size_t)(BLOCK / 32) * 64);
}

// COMPACT: events whose kinematic test fails need no angles or boosts.  Where many fail
// (low ok fractions: multi-channel batches, hard cuts), pass A tests each event, writes
// the failures, and queues the rest per warp; pass B runs them densely.  Where nearly all
// pass, the plain loop avoids the second msq evaluation; the launcher times both.
// BLOCK threads per block (the block shape the autotuner tries), MIN_BLOCKS resident.
template <bool PER_EVENT, bool COMPACT, int MIN_BLOCKS, int BLOCK = PHS_FWD_BLOCK>
__global__ void __launch_bounds__(BLOCK, MIN_BLOCKS)
    phs_forward_f64_kernel(const __grid_constant__ PhsLaunch a) {
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double2 *trig = phs_trig_table<BLOCK>(smem, a.stack_depth);
  fill_trig_table(trig);
  __syncthreads();
  if constexpr (COMPACT) {
    int64_t *q = reinterpret_cast<int64_t *>(smem + (size_t)a.stack_depth * PHS_STATE * BLOCK) +
                 (threadIdx.x >> 5) * 64;
    compacting_loop<PHS_CHUNK_TILES>(
        a, q,
        [&](const PhsSegment &sg, int64_t loc) { return phs_ok_f64<PER_EVENT, BLOCK>(a, sg, loc, smem); },
        [&](int, const PhsSegment &sg, int64_t loc) {
          phs_event_f64<PER_EVENT, BLOCK>(a, sg, loc, smem, trig);
        });
  } else {
    for (int64_t tile = warp0; tile < a.n_tiles; tile += n_warps) {
      // the segment holding this tile (warp-uniform binary search on tile_begin)
      const PhsSegment *segs = a.n_segments <= PHS_INLINE_SEGS ? a.seg_inline : a.segments;
      int lo = 0, hi = a.n_segments - 1;
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (segs[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
      }
      const PhsSegment seg = segs[lo];
      const int64_t local = (tile - seg.tile_begin) * 32 + lane;
      if (local >= seg.ev_count) continue;
      phs_event_f64<PER_EVENT, BLOCK>(a, seg, local, smem, trig);
    }
  }
}

// The exact FP64 path for the events the FP32-pair kernel queued, per segment
// (a.exact_queue from tile_begin * 32 on, a.exact_count entries, claims numbered by
// a.exact_tile).  Those are events within 1e-5 of a kinematic limit, and all events of
// channels whose mappings or boosts have no float-float form; keeping their FP64 code out
// of the FP32-pair kernel keeps that kernel's body small.  Warps claim 32 events of one
// segment (a.exact_work counts the claims), so each runs one channel's program; the counts
// are read on the device, so the launch can sit in a CUDA graph behind the FP32-pair one.
template <bool PER_EVENT>
__global__ void __launch_bounds__(PHS_FWD_BLOCK, 4)
    phs_forward_exact_kernel(const __grid_constant__ PhsLaunch a) {
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31;
  double2 *trig = phs_trig_table(smem, a.stack_depth);
  fill_trig_table(trig);
  __syncthreads();
  const PhsSegment *segs = a.n_segments <= PHS_INLINE_SEGS ? a.seg_inline : a.segments;
  const int64_t n_claims = a.exact_tile[a.n_segments];
  for (;;) {
    unsigned long long c = 0;
    if (lane == 0) c = atomicAdd(a.exact_work, 1ull);
    const int64_t t = (int64_t)__shfl_sync(0xffffffffu, c, 0);
    if (t >= n_claims) break;
    int lo = 0, hi = a.n_segments - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (a.exact_tile[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const PhsSegment seg = segs[lo];
    const int64_t idx = (t - a.exact_tile[lo]) * 32 + lane;
    if (idx >= (int64_t)a.exact_count[lo]) continue;
    // the queue slot lies in the segment's run of a.n_tiles * 32 entries, the event in the segment
    if (!phs_in(idx, seg.ev_count, PHS_CHK_QUEUE) ||
        !phs_in(seg.tile_begin * 32 + idx, a.n_tiles * 32, PHS_CHK_QUEUE))
      continue;
    phs_event_f64<PER_EVENT>(a, seg, a.exact_queue[seg.tile_begin * 32 + idx], smem, trig);
  }
}

// Split form of the FP64 kernel: after the FP32 pre-test (phs_launch_pretest, which writes
// the outputs of the events that fail for certain and queues the others per segment), the
// FP64 walk over the queued events, 32 of one segment per warp claim (a.work counts the
// claims, zeroed before the launch).  The pre-test only settles failures that the FP64
// test makes too, so the outputs are the one-pass kernel's bits.  Uniform beams only.
template <int MIN_BLOCKS, int BLOCK = PHS_FWD_BLOCK>
__global__ void __launch_bounds__(BLOCK, MIN_BLOCKS)
    phs_f64_walk_kernel(const __grid_constant__ PhsLaunch a) {
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31;
  double2 *trig = phs_trig_table<BLOCK>(smem, a.stack_depth);
  fill_trig_table(trig);
  __syncthreads();
  const PhsSegment *segs = a.n_segments <= PHS_INLINE_SEGS ? a.seg_inline : a.segments;
  const int64_t n_claims = a.pass_tile[a.n_segments];
  for (;;) {
    unsigned long long c = 0;
    if (lane == 0) c = atomicAdd(a.work, 1ull);
    const int64_t t = (int64_t)__shfl_sync(0xffffffffu, c, 0);
    if (t >= n_claims) break;
    // the last segment whose first claim is <= t (empty segments share the next one's)
    int lo = 0, hi = a.n_segments - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (a.pass_tile[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const PhsSegment seg = segs[lo];
    const int64_t idx = (t - a.pass_tile[lo]) * 32 + lane;
    if (idx >= (int64_t)a.pass_count[lo]) continue;
    if (!phs_in(idx, seg.ev_count, PHS_CHK_QUEUE) ||
        !phs_in(seg.tile_begin * 32 + idx, a.n_tiles * 32, PHS_CHK_QUEUE))
      continue;
    phs_event_f64<false, BLOCK>(a, seg, a.pass_queue[seg.tile_begin * 32 + idx], smem, trig);
  }
}

// Whizard's sparse momentum buffer from the dense one (layout in phs_device.h): one thread
// per 32-byte slot, consecutive threads on consecutive slots.
__global__ void phs_whizard_sparse_kernel(const __grid_constant__ PhsSparseLaunch a) {
  const int64_t total = a.n_events * a.n_prt;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ev = i / a.n_prt;
    const int code = (int)(i - ev * a.n_prt) + 1;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    const double *pe = a.p + ev * 4 * a.n_out;
    if (code < (1 << a.n_out)) {
      if ((code & (code - 1)) == 0) {
        const int k = __ffs(code) - 1;
#pragma unroll
        for (int mu = 0; mu < 4; mu++) v[mu] = pe[4 * k + mu];
      } else if (a.internal[code >> 5] >> (code & 31) & 1u) {
        // back to the centre-of-mass frame: the inverse of the lab boost
        // p0 = gamma p0* + bg p3*, p3 = bg p0* + gamma p3* (phs.cu:1286-1301)
        const double e1 = a.E1 ? a.E1[ev] : a.e1, e2 = a.E2 ? a.E2[ev] : a.e2;
        const double bg = (e1 - e2) / (2.0 * sqrt(e1 * e2)), ga = sqrt(1.0 + bg * bg);
        for (int k = 0; k < a.n_out; k++) {
          if (!(code >> k & 1)) continue;
          const double *q = pe + 4 * k;
          v[0] += ga * q[0] - bg * q[3];
          v[1] += q[1];
          v[2] += q[2];
          v[3] += ga * q[3] - bg * q[0];
        }
      }
    }
    double2 *o = reinterpret_cast<double2 *>(a.out + 4 * i);
    o[0] = make_double2(v[0], v[1]);
    o[1] = make_double2(v[2], v[3]);
  }
}

// Philox4x32-10 (Salmon et al., SC'11); layout documented in gpu_phs_gb300/philox.py.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}

__global__ void phs_philox_kernel(double *x, int64_t e0, int64_t n, uint64_t seed) {
  const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
  const int64_t b_first = e0 >> 1, b_last = (e0 + n - 1) >> 1;
  for (int64_t b = b_first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b <= b_last;
       b += (int64_t)gridDim.x * blockDim.x) {
    uint4 r = philox4x32_10(make_uint4((uint32_t)b, (uint32_t)((uint64_t)b >> 32), 0u, 0u), key);
    const double u0 = (double)((((uint64_t)r.x << 32) | r.y) >> 11) * 0x1.0p-53;
    const double u1 = (double)((((uint64_t)r.z << 32) | r.w) >> 11) * 0x1.0p-53;
    const int64_t e = 2 * b;
    if (e >= e0 && e < e0 + n) x[e - e0] = u0;
    if (e + 1 >= e0 && e + 1 < e0 + n) x[e + 1 - e0] = u1;
  }
}

// Arithmetic-throughput probe: each thread runs `iters` rounds of 8 independent FMA
// chains (FP64 or FP32), enough independent work to keep the pipe busy; the result is
// stored so the chains are live.
template <typename T>
__global__ void phs_fma_rate_kernel(T *out, int iters, T a, T b) {
  T v[8];
#pragma unroll
  for (int i = 0; i < 8; i++) v[i] = (T)(threadIdx.x + i);
  for (int k = 0; k < iters; k++) {
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = fma(v[i], a, b);
  }
  T s = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) s += v[i];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

cudaError_t phs_launch_fma_rate(void *out, int fp64, int blocks, int threads, int iters,
                                cudaStream_t stream) {
  if (fp64)
    phs_fma_rate_kernel<double><<<blocks, threads, 0, stream>>>((double *)out, iters, 0.999999, 1e-7);
  else
    phs_fma_rate_kernel<float><<<blocks, threads, 0, stream>>>((float *)out, iters, 0.999999f, 1e-7f);
  return cudaGetLastError();
}

size_t phs_forward_smem_bytes(int stack_depth, int block) {
  // frame stack, the compacting variant's per-warp queues (64 events per warp), the
  // sin/cos table
  return (size_t)stack_depth * PHS_STATE * block * sizeof(double) +
         (size_t)(block / 32) * 64 * sizeof(int64_t) + PHS_TRIG_N * sizeof(double2);
}

// Variants (each at one block shape, BLOCK threads, and a register budget): 0: one pass,
// 128 threads x 4 blocks per SM; 1, 2: compacting, 128 x 4 and 128 x 3 (no spills);
// 3, 4: one pass, 256 x 2 and 64 x 8; 5-8: split (the FP32 pre-test, then the walk over its
// survivors; uniform beams only), 128 x 4, 128 x 3, 256 x 2, 64 x 8.  The 128-register
// budget is the same for 64 x 8, 128 x 4 and 256 x 2.
static int f64_block(int variant) {
  switch (variant) {
    case 3: case 7: return 256;
    case 4: case 8: return 64;
    default: return PHS_FWD_BLOCK;
  }
}

template <bool PER_EVENT>
static const void *f64_kernel(int variant) {
  switch (variant) {
    case 1: return (const void *)phs_forward_f64_kernel<PER_EVENT, true, 4>;
    case 2: return (const void *)phs_forward_f64_kernel<PER_EVENT, true, 3>;
    case 3: return (const void *)phs_forward_f64_kernel<PER_EVENT, false, 2, 256>;
    case 4: return (const void *)phs_forward_f64_kernel<PER_EVENT, false, 8, 64>;
    case 5: return (const void *)phs_f64_walk_kernel<4>;
    case 6: return (const void *)phs_f64_walk_kernel<3>;
    case 7: return (const void *)phs_f64_walk_kernel<2, 256>;
    case 8: return (const void *)phs_f64_walk_kernel<8, 64>;
    default: return (const void *)phs_forward_f64_kernel<PER_EVENT, false, 4>;
  }
}

int phs_forward_block_size(int variant) { return f64_block(variant); }

// Shared memory above the 48 KB default (256-thread blocks with two saved frames) needs
// the kernel's opt-in.
static cudaError_t allow_smem(const void *kernel, size_t smem) {
  if (smem <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

int phs_forward_blocks_per_sm(int stack_depth, bool per_event, int variant) {
  int n = 0;
  const int block = f64_block(variant);
  const size_t smem = phs_forward_smem_bytes(stack_depth, block);
  const void *k = per_event ? f64_kernel<true>(variant) : f64_kernel<false>(variant);
  if (allow_smem(k, smem) != cudaSuccess) return 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, block, smem);
  return n > 0 ? n : 1;
}

template <bool PER_EVENT>
static cudaError_t launch_f64(const PhsLaunch &a, int n_blocks, int variant, cudaStream_t stream) {
  const int block = f64_block(variant);
  const size_t smem = phs_forward_smem_bytes(a.stack_depth, block);
  const cudaError_t e = allow_smem(f64_kernel<PER_EVENT>(variant), smem);
  if (e != cudaSuccess) return e;
  switch (variant) {
    case 1:
      phs_forward_f64_kernel<PER_EVENT, true, 4><<<n_blocks, block, smem, stream>>>(a);
      break;
    case 2:
      phs_forward_f64_kernel<PER_EVENT, true, 3><<<n_blocks, block, smem, stream>>>(a);
      break;
    case 3:
      phs_forward_f64_kernel<PER_EVENT, false, 2, 256><<<n_blocks, block, smem, stream>>>(a);
      break;
    case 4:
      phs_forward_f64_kernel<PER_EVENT, false, 8, 64><<<n_blocks, block, smem, stream>>>(a);
      break;
    default:
      phs_forward_f64_kernel<PER_EVENT, false, 4><<<n_blocks, block, smem, stream>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t phs_launch_forward_f64(const PhsLaunch &a, int n_blocks, int variant,
                                   cudaStream_t stream) {
  if (a.n_tiles <= 0) return cudaSuccess;
  if (variant >= 5) {
    if (a.E1 || a.E2) return cudaErrorInvalidValue;  // the pre-test needs uniform beams
    cudaError_t e = phs_launch_pretest(a, stream);
    if (e != cudaSuccess) return e;
    const int block = f64_block(variant);
    const size_t smem = phs_forward_smem_bytes(a.stack_depth, block);
    e = allow_smem(f64_kernel<false>(variant), smem);
    if (e != cudaSuccess) return e;
    switch (variant) {
      case 5: phs_f64_walk_kernel<4><<<n_blocks, block, smem, stream>>>(a); break;
      case 6: phs_f64_walk_kernel<3><<<n_blocks, block, smem, stream>>>(a); break;
      case 7: phs_f64_walk_kernel<2, 256><<<n_blocks, block, smem, stream>>>(a); break;
      default: phs_f64_walk_kernel<8, 64><<<n_blocks, block, smem, stream>>>(a);
    }
    return cudaGetLastError();
  }
  return a.E1 && a.E2 ? launch_f64<true>(a, n_blocks, variant, stream)
                      : launch_f64<false>(a, n_blocks, variant, stream);
}

cudaError_t phs_launch_forward_exact(const PhsLaunch &a, int n_blocks, cudaStream_t stream) {
  if (a.n_tiles <= 0) return cudaSuccess;
  cudaError_t e = phs_launch_count_scan(a.exact_count, a.exact_tile, a.n_segments, stream);
  if (e != cudaSuccess) return e;
  const size_t smem = phs_forward_smem_bytes(a.stack_depth, PHS_FWD_BLOCK);
  e = allow_smem(a.E1 && a.E2 ? (const void *)phs_forward_exact_kernel<true>
                              : (const void *)phs_forward_exact_kernel<false>, smem);
  if (e != cudaSuccess) return e;
  if (a.E1 && a.E2)
    phs_forward_exact_kernel<true><<<n_blocks, PHS_FWD_BLOCK, smem, stream>>>(a);
  else
    phs_forward_exact_kernel<false><<<n_blocks, PHS_FWD_BLOCK, smem, stream>>>(a);
  return cudaGetLastError();
}

// SMs of the current device (grid caps of the grid-stride kernels below).
static int current_sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

cudaError_t phs_launch_whizard_sparse(const PhsSparseLaunch &a, cudaStream_t stream) {
  const int64_t total = a.n_events * a.n_prt;
  if (total <= 0) return cudaSuccess;
  const int64_t blocks = (total + 255) / 256, cap = (int64_t)current_sm_count() * 32;
  phs_whizard_sparse_kernel<<<(int)(blocks < cap ? blocks : cap), 256, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t phs_launch_philox(double *x, int64_t n_events, int32_t n_x, uint64_t seed,
                              int64_t first_event, cudaStream_t stream) {
  const int64_t n = n_events * n_x;
  if (n <= 0) return cudaSuccess;
  const int64_t blocks_needed = ((n >> 1) + 2 + 255) / 256, cap = (int64_t)current_sm_count() * 16;
  const int grid = (int)(blocks_needed < cap ? blocks_needed : cap);
  phs_philox_kernel<<<grid, 256, 0, stream>>>(x, first_event * n_x, n, seed);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------------------
// Forward generation without device allocation.
//
// For callers that must not allocate device memory: code running inside a host that
// owns the device heap through its own allocator, sandboxes or plugins denied cudaMalloc,
// and drivers that would otherwise synchronise the device inside their hot loop.  The
// channel programs and the segment table, which the regular entry points keep in buffers
// the library allocates, live here in one file-scope device array instead.  Every GPU
// that loads the library holds this array (sizeof(PhsNoAllocScratch), about 1 MB) until
// the process exits.  All calls share it and it keeps the last call's contents; each call
// overwrites everything it reads, so nothing needs clearing, but calls that overlap on
// the GPU (different streams or host threads) race on it.
struct PhsNoAllocScratch {
  PhsChannel channels[PHS_NOALLOC_MAX_CHANNELS];
  PhsSegment segments[PHS_NOALLOC_MAX_CHANNELS];
};

static __device__ __align__(256) unsigned char phs_noalloc_scratch[sizeof(PhsNoAllocScratch)];

// Device address of the scratch array per device (filled at set-up; in host code the
// array's name only stands in for the symbol and is never a device address).  The mutex
// orders first calls from several host threads.
static void *g_noalloc_addr[256];
static std::mutex g_noalloc_mu;

size_t phs_noalloc_scratch_bytes() { return sizeof(PhsNoAllocScratch); }

cudaError_t phs_launch_forward_f64_noalloc(PhsLaunch a, const PhsChannel *channels,
                                           int n_channels, const PhsSegment *segments,
                                           int n_segments, int n_blocks, cudaStream_t stream) {
  if (n_channels > PHS_NOALLOC_MAX_CHANNELS || n_segments > PHS_NOALLOC_MAX_CHANNELS)
    return cudaErrorInvalidValue;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 256) return cudaErrorInvalidDevice;
  void *addr = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
      // set-up, once per device, with that device current
      void *ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, phs_noalloc_scratch);
      if (e != cudaSuccess) return e;
      g_noalloc_addr[dev] = ptr;
    }
    addr = g_noalloc_addr[dev];
  }
  PhsNoAllocScratch *s = static_cast<PhsNoAllocScratch *>(addr);
  // pageable host sources: each copy has read its source when the call returns
  e = cudaMemcpyAsync(s->channels, channels, (size_t)n_channels * sizeof(PhsChannel),
                      cudaMemcpyHostToDevice, stream);
  if (e != cudaSuccess) return e;
  if (n_segments > 0) {
    e = cudaMemcpyAsync(s->segments, segments, (size_t)n_segments * sizeof(PhsSegment),
                        cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return e;
  }
  a.channels = s->channels;
  a.segments = s->segments;
  a.n_segments = n_segments;
  if (a.n_tiles <= 0) return cudaSuccess;
  const size_t smem = phs_forward_smem_bytes(a.stack_depth, PHS_FWD_BLOCK);
  e = allow_smem(f64_kernel<false>(0), smem);
  if (e != cudaSuccess) return e;
  phs_forward_f64_kernel<false, false, 4><<<n_blocks, PHS_FWD_BLOCK, smem, stream>>>(a);
  return cudaGetLastError();
}

PHS_CHECK_COLLECTOR(phs_check_collect_kernels)
