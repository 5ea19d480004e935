// phs_check.h -- bounds checks of the checked build (PHS_CHECKED).
//
// The library is built twice: libgpuphs.so and, compiled with -DPHS_CHECKED,
// libgpuphs_checked.so.  In the checked build every index that device code computes from
// run-time data (channel programs, segment tables, queues, event, row and stack offsets)
// is compared with the extent of the array it addresses before the access.  An index out
// of range sets the bit of its site in the translation unit's check word, records the
// first such index, and the access is skipped (a read gives 0).  phs_check_status() (the C
// API) collects and clears the words of every translation unit.  In the other build the
// checks compile to nothing.  This stands in for compute-sanitizer, which is not
// available on the GPU pool: small cases run through the checked build and must leave
// every word at zero with the same outputs as the unchecked build.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

// Check sites (bit numbers of the check word).
enum PhsCheckSite {
  PHS_CHK_CHANNEL = 0,  // channel index into a program table
  PHS_CHK_X = 1,        // x element of an event row
  PHS_CHK_P = 2,        // momentum element of an event row
  PHS_CHK_EVENT = 3,    // factor / volume / ok entry
  PHS_CHK_STACK = 4,    // frame-stack depth
  PHS_CHK_VISITS = 5,   // visit count of a channel program
  PHS_CHK_QUEUE = 6,    // survivor / exact-path queue slot
  PHS_CHK_SEGMENT = 7,  // segment index of a claim
  PHS_CHK_ADJ = 8,      // adjoint cotangent or output entry
  PHS_CHK_STORE = 9,    // stored-matrix adjoint frame buffer
  PHS_CHK_INV = 10,     // inverse-map outputs (x_out, all_factors)
  PHS_CHK_SLOT = 11,    // inverse-map momentum slot, group order or tile queue
  PHS_CHK_GRID = 12,    // warm-up grid bin or channel
};

#ifdef __CUDACC__
#ifdef PHS_CHECKED
namespace {
// One word per translation unit (device variables are not shared between the separately
// compiled units): bit per failed site, and the first failing index.
__device__ unsigned long long phs_check_word;
__device__ unsigned long long phs_check_first;

// i in [0, n)?  Records and returns false otherwise.
__device__ __forceinline__ bool phs_in(int64_t i, int64_t n, int site) {
  if (i >= 0 && i < n) return true;
  if (atomicOr(&phs_check_word, 1ull << site) == 0ull)
    atomicExch(&phs_check_first, (unsigned long long)i);
  return false;
}
}  // namespace
// Host side of a translation unit: reads its word and first index, then clears them.
#define PHS_CHECK_COLLECTOR(fn)                                                           \
  cudaError_t fn(unsigned long long *word, long long *first) {                           \
    unsigned long long w = 0, f = 0, z = 0;                                               \
    cudaError_t e = cudaMemcpyFromSymbol(&w, phs_check_word, sizeof w);                   \
    if (e == cudaSuccess) e = cudaMemcpyFromSymbol(&f, phs_check_first, sizeof f);        \
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(phs_check_word, &z, sizeof z);           \
    *word = w;                                                                            \
    *first = (long long)f;                                                                \
    return e;                                                                             \
  }
#else
__device__ __forceinline__ bool phs_in(int64_t, int64_t, int) { return true; }
#define PHS_CHECK_COLLECTOR(fn)                                                           \
  cudaError_t fn(unsigned long long *word, long long *first) {                           \
    *word = 0;                                                                            \
    *first = 0;                                                                           \
    return cudaSuccess;                                                                   \
  }
#endif
#endif  // __CUDACC__

// The collectors of the translation units (phs_kernels.cu, phs_kernels_ff.cu,
// phs_adjoint.cu, phs_inverse.cu, phs_grid.cu).
cudaError_t phs_check_collect_kernels(unsigned long long *word, long long *first);
cudaError_t phs_check_collect_ff(unsigned long long *word, long long *first);
cudaError_t phs_check_collect_adjoint(unsigned long long *word, long long *first);
cudaError_t phs_check_collect_inverse(unsigned long long *word, long long *first);
cudaError_t phs_check_collect_grid(unsigned long long *word, long long *first);
