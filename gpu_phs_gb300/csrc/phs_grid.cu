// phs_grid.cu -- the per-channel x grid of the reference's warm-up (rng.cpp), on the device.
//
// Per channel and x dimension, PHS_GRID_BINS equal-width bins on [0, 1) with weights (the
// bin probabilities, rng.cpp:5-30).  Sampling draws x from that piecewise-constant density
// (rng.cpp:69-90 uses std::piecewise_constant_distribution): here the Philox uniform u of
// the element is mapped through the inverse distribution function, bin b with
// C[b] <= u < C[b+1] (C the running sum of the weights) and x = (b + (u - C[b]) / w[b]) /
// PHS_GRID_BINS.  Updating sets each weight to the fraction of the channel's ok events
// whose x fell into the bin (rng.cpp:34-67).
#include <cuda_runtime.h>
#include <stdint.h>

#include "phs_device.h"

namespace {

// The generating channel of event ev: the last c with ch_begin[c] <= ev.
__device__ __forceinline__ int channel_of(const int64_t *ch_begin, int n_channels, int64_t ev) {
  int lo = 0, hi = n_channels - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (ch_begin[mid] <= ev) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void phs_grid_sample_kernel(double *x, int64_t n_events, int n_x,
                                       const int64_t *ch_begin, int n_channels,
                                       const double *weights) {
  const int64_t n = n_events * n_x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ev = i / n_x;
    const int d = (int)(i - ev * n_x);
    const int ch = channel_of(ch_begin, n_channels, ev);
    if (!phs_in(ch, n_channels, PHS_CHK_GRID)) continue;
    const double *w = weights + ((int64_t)ch * n_x + d) * PHS_GRID_BINS;
    const double u = x[i];
    double c = 0.0;
    int b = 0;
    // the last bin with positive weight whose start lies at or below u
    for (int k = 0; k < PHS_GRID_BINS; k++) {
      if (w[k] > 0.0 && c <= u) b = k;
      c += w[k];
    }
    double cb = 0.0;
    for (int k = 0; k < b; k++) cb += w[k];
    double t = (u - cb) / w[b];
    t = t < 0.0 ? 0.0 : (t >= 1.0 ? 0x1.fffffffffffffp-1 : t);  // rounding at the bin edges
    x[i] = (b + t) / PHS_GRID_BINS;
  }
}

// Histogram of ok events per (channel, dimension, bin): one warp per 32 consecutive events;
// lanes with the same bin combine into one atomic.
__global__ void phs_grid_count_kernel(const double *x, const uint8_t *ok, int64_t n_events,
                                      int n_x, const int64_t *ch_begin, int n_channels,
                                      unsigned long long *bins, unsigned long long *n_ok) {
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = warp0; t * 32 < n_events; t += n_warps) {
    const int64_t ev = t * 32 + lane;
    const bool live = ev < n_events && ok[ev] != 0;
    const int c = ev < n_events ? channel_of(ch_begin, n_channels, ev) : -1;
    // key = channel * BINS + bin: lanes of one tile can span a channel boundary
    {
      const unsigned m = __match_any_sync(0xffffffffu, live ? c : -1);
      if (live && lane == __ffs(m) - 1) atomicAdd(&n_ok[c], (unsigned long long)__popc(m));
    }
    for (int d = 0; d < n_x; d++) {
      int key = -1;
      if (live) {
        int b = (int)(x[ev * n_x + d] * PHS_GRID_BINS);
        b = b < 0 ? 0 : (b >= PHS_GRID_BINS ? PHS_GRID_BINS - 1 : b);
        key = c * PHS_GRID_BINS + b;
      }
      const unsigned m = __match_any_sync(0xffffffffu, key);
      if (key >= 0 && lane == __ffs(m) - 1 && phs_in(key, (int64_t)n_channels * PHS_GRID_BINS, PHS_CHK_GRID)) {
        const int cc = key / PHS_GRID_BINS, b = key % PHS_GRID_BINS;
        atomicAdd(&bins[((int64_t)cc * n_x + d) * PHS_GRID_BINS + b], (unsigned long long)__popc(m));
      }
    }
  }
}

// weights = count / (ok events of the channel); a channel without ok events keeps its
// weights (the reference divides by zero there, rng.cpp:60-66).
__global__ void phs_grid_normalise_kernel(const unsigned long long *bins,
                                          const unsigned long long *n_ok, int n_channels,
                                          int n_x, double *weights) {
  const int64_t n = (int64_t)n_channels * n_x * PHS_GRID_BINS;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i / ((int64_t)n_x * PHS_GRID_BINS));
    if (n_ok[c] > 0) weights[i] = (double)bins[i] / (double)n_ok[c];
  }
}

}  // namespace

cudaError_t phs_launch_grid_sample(double *x, int64_t n_events, int n_x, const int64_t *ch_begin,
                                   int n_channels, const double *weights, int sm_count,
                                   cudaStream_t stream) {
  if (n_events <= 0) return cudaSuccess;
  const int64_t blocks = (n_events * n_x + 255) / 256;
  const int grid = (int)(blocks < (int64_t)sm_count * 8 ? blocks : (int64_t)sm_count * 8);
  phs_grid_sample_kernel<<<grid, 256, 0, stream>>>(x, n_events, n_x, ch_begin, n_channels, weights);
  return cudaGetLastError();
}

cudaError_t phs_launch_grid_update(const double *x, const uint8_t *ok, int64_t n_events, int n_x,
                                   const int64_t *ch_begin, int n_channels,
                                   unsigned long long *bins, unsigned long long *n_ok,
                                   double *weights, int sm_count, cudaStream_t stream) {
  const size_t nb = (size_t)n_channels * n_x * PHS_GRID_BINS;
  cudaError_t e = cudaMemsetAsync(bins, 0, nb * sizeof(unsigned long long), stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(n_ok, 0, n_channels * sizeof(unsigned long long), stream);
  if (e != cudaSuccess) return e;
  if (n_events > 0) {
    const int64_t warps = (n_events + 31) / 32;
    const int64_t blocks = (warps + 7) / 8;
    const int grid = (int)(blocks < (int64_t)sm_count * 8 ? blocks : (int64_t)sm_count * 8);
    phs_grid_count_kernel<<<grid, 256, 0, stream>>>(x, ok, n_events, n_x, ch_begin, n_channels,
                                                    bins, n_ok);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  const int g2 = (int)((nb + 255) / 256);
  phs_grid_normalise_kernel<<<g2, 256, 0, stream>>>(bins, n_ok, n_channels, n_x, weights);
  return cudaGetLastError();
}

PHS_CHECK_COLLECTOR(phs_check_collect_grid)
