// phs_kernels.cu -- fused forward phase-space kernel (FP64) and the Philox x generator.
//
// One persistent kernel per batch.  Each warp takes 32-event tiles of one channel (tiles
// never straddle channels, so every branch of the visit program is warp-uniform); each
// thread walks its event's visit program top-down (phs_program.h) with the running 4x4
// boost in registers and at most two saved frames on a per-thread shared-memory stack.
//
// Arithmetic follows the reference CPU path (phs_cpu.cpp), whose expression order it keeps
// with explicit round-to-nearest intrinsics wherever a value feeds the kinematic ok test
// (msq mappings, the Kallen function and the mass sums), so ok flags match the reference
// bit for bit whenever the transcendental functions agree; factors and boosts use FMA.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "phs_device.h"
#include "phs_program.h"

#define PHS_PI 3.14159265358979323846
#define PHS_TWOPI2 39.47841760435743447534
#define PHS_TWOPI5 9792.62991312900650440772
#define PHS_STATE 20  // doubles per saved frame: L[16], msq, m, p, m_max

namespace {

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// msq from x (phs_cpu.cpp:12-61), same expression order, no contraction.
__device__ __forceinline__ void map_msq(int t, double x, double s, double m, double w,
                                        double msq_min, double msq_max, double a0, double a1,
                                        double a2, double &msq, double &f) {
  switch (t) {
    case PHS_MAP_NO:
      msq = dadd(dmul(dsub(1.0, x), msq_min), dmul(x, msq_max));
      f = (msq_max - msq_min) / s;
      break;
    case PHS_MAP_SCHANNEL: {
      double z = dadd(dmul(dsub(1.0, x), a0), dmul(x, a1));
      if (-PHS_PI / 2 < z && z < PHS_PI / 2) {
        double tz = tan(z);
        msq = dmul(m, dadd(m, dmul(w, tz)));
        f = a2 * (1.0 + tz * tz);
      } else {
        msq = 0.0;
        f = 0.0;
      }
      break;
    }
    case PHS_MAP_COLLINEAR:
    case PHS_MAP_INFRARED:
    case PHS_MAP_RADIATION: {
      double msq1 = dmul(a0, exp(dmul(x, a1)));
      msq = dadd(dsub(msq1, a0), msq_min);
      f = a2 * msq1;
      break;
    }
    case PHS_MAP_TCHANNEL:
    case PHS_MAP_UCHANNEL: {
      double msq1;
      if (x < 0.5) {
        msq1 = dmul(a0, exp(dmul(x, a1)));
        msq = dadd(dsub(msq1, a0), msq_min);
      } else {
        msq1 = dmul(a0, exp(dmul(dsub(1.0, x), a1)));
        msq = dadd(-dsub(msq1, a0), msq_max);
      }
      f = a2 * msq1;
      break;
    }
    case PHS_MAP_STEP_H: {
      double am = dsub(a0, x);
      double z = dadd(dsub(a1 / am, a1 / a0), dmul(a2, x));
      msq = dadd(dmul(z, msq_max), dmul(dsub(1.0, z), msq_min));
      f = (a1 / (am * am) + a2) * (msq_max - msq_min) / s;
      break;
    }
    case PHS_MAP_STEP_E: {
      double tmp = dmul(exp(dmul(-x, a0) / a2), dadd(1.0, a1));
      double z = dmul(-a2, log(dsub(tmp, a1)));
      msq = dadd(dmul(z, msq_max), dmul(dsub(1.0, z), msq_min));
      f = a0 / (1.0 - a1 / tmp) * (msq_max - msq_min) / s;
      break;
    }
    default:
      msq = 0.0;
      f = 0.0;
  }
}

// cos(theta) from x (phs_cpu.cpp:112-146).  The collinear branch keeps the reference's
// rounding: sin(theta) = sqrt(1 - ct^2) is ill-conditioned as |ct| -> 1.
__device__ __forceinline__ void map_ct(int ct_class, double x, double b0, double b1, double &ct,
                                       double &st, double &f) {
  if (ct_class == PHS_CT_COLLINEAR) {
    double tmp;
    if (x < 0.5) {
      tmp = dmul(b0, exp(dmul(dmul(2.0, x), b1)));
      ct = dsub(dsub(tmp, b0), 1.0);
    } else {
      tmp = dmul(b0, exp(dmul(dmul(2.0, dsub(1.0, x)), b1)));
      ct = dadd(-dsub(tmp, b0), 1.0);
    }
    if (ct >= -1.0 && ct <= 1.0) {
      st = sqrt(dsub(1.0, dmul(ct, ct)));
      f = tmp * b1;
    } else {
      ct = 1.0;
      st = 0.0;
      f = 0.0;
    }
  } else {
    double tmp = 2.0 * (1.0 - x);
    ct = 1.0 - tmp;
    st = sqrt(tmp * (2.0 - tmp));
    f = 1.0;
  }
}

// Mapping constants at one sqrt(s) (phs_cpu.cpp:452-531), for the per-event-beam path.
__device__ void child_constants(const PhsChild &C, double sqrts, double m_tot, double &a0,
                                double &a1, double &a2, double &msq_min, double &msq_max,
                                double &m_max) {
  double m = C.m, w = C.w, m_min = C.m_min;
  m_max = dadd(dsub(sqrts, m_tot), m_min);
  msq_min = dmul(m_min, m_min);
  msq_max = dmul(m_max, m_max);
  double s = dmul(sqrts, sqrts);
  a0 = a1 = a2 = 0.0;
  switch (C.map_id) {
    case PHS_MAP_NO:
      a1 = msq_max - msq_min;
      a2 = a1 / s;
      break;
    case PHS_MAP_SCHANNEL: {
      double msq0 = dmul(m, m), mw = dmul(m, w);
      a0 = atan(dsub(msq_min, msq0) / mw);
      a1 = atan(dsub(msq_max, msq0) / mw);
      a2 = dmul(dsub(a1, a0), mw) / s;
      break;
    }
    case PHS_MAP_RADIATION:
    case PHS_MAP_COLLINEAR:
    case PHS_MAP_INFRARED: {
      double msq0 = C.map_id == PHS_MAP_RADIATION ? dmul(w, w) : dmul(m, m);
      a0 = msq0;
      a1 = log(dadd(dsub(msq_max, msq_min) / msq0, 1.0));
      a2 = a1 / s;
      break;
    }
    case PHS_MAP_TCHANNEL:
    case PHS_MAP_UCHANNEL: {
      double msq0 = dmul(m, m);
      a0 = msq0;
      a1 = dmul(2.0, log(dadd(dsub(msq_max, msq_min) / dmul(2.0, msq0), 1.0)));
      a2 = a1 / s;
      break;
    }
    case PHS_MAP_STEP_E: {
      double r = dmul(dmul(2.0, m), w) / dsub(msq_max, msq_min);
      a2 = r > 0.01 ? r : 0.01;
      a1 = exp(-(dsub(dmul(m, m), msq_min)) / dsub(msq_max, msq_min) / a2);
      a0 = dsub(1.0, dmul(a2, log(dadd(1.0, dmul(a1, exp(1.0 / a2))) / dadd(1.0, a1))));
      break;
    }
    case PHS_MAP_STEP_H: {
      a2 = dsub(dmul(m, m), msq_min) / dsub(msq_max, msq_min);
      double q = dmul(dmul(2.0, m), w) / dsub(msq_max, msq_min);
      double r = dmul(q, q) / a2;
      a1 = r > 0.000001 ? r : 0.000001;
      a0 = dadd(1.0, sqrt(dadd(1.0, dmul(4.0, a1) / dsub(1.0, a2)))) / 2.0;
      break;
    }
  }
}

__device__ __forceinline__ void stack_store(double *smem, int depth, int k, double v) {
  smem[(depth * PHS_STATE + k) * PHS_FWD_BLOCK + threadIdx.x] = v;
}
__device__ __forceinline__ double stack_load(const double *smem, int depth, int k) {
  return smem[(depth * PHS_STATE + k) * PHS_FWD_BLOCK + threadIdx.x];
}

template <bool PER_EVENT>
__global__ void __launch_bounds__(PHS_FWD_BLOCK)
    phs_forward_f64_kernel(const __grid_constant__ PhsLaunch a) {
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;

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
    const PhsChannel &ch = a.channels[seg.channel];
    const int64_t ev = seg.ev_begin + local;
    const double *xe = a.x + seg.x_base + local * seg.x_stride;
    double *out = a.p + seg.p_base + local * 4 * (int64_t)ch.n_out;

    double sqrts = ch.sqrts;
    double lab_bg = ch.lab_bg, lab_ga = ch.lab_gamma;
    bool lab = ch.lab != 0;
    if (PER_EVENT) {
      double E1 = a.E1[ev], E2 = a.E2[ev];
      double r = sqrt(dmul(E1, E2));
      sqrts = dmul(2.0, r);
      lab = E1 != E2;
      lab_bg = dsub(E1, E2) / dmul(2.0, r);
      lab_ga = sqrt(1.0 + lab_bg * lab_bg);
    }
    const double s = dmul(sqrts, sqrts);

    // frame of the visited branch; the root's parent frame is the lab boost (or 1)
    double L[16];
#pragma unroll
    for (int i = 0; i < 16; i++) L[i] = 0.0;
    L[0] = lab ? lab_ga : 1.0;
    L[5] = 1.0;
    L[10] = 1.0;
    L[15] = L[0];
    L[3] = lab ? lab_bg : 0.0;
    L[12] = L[3];
    double msq_b = s, m_b = sqrts, p_b = 0.0, mmax_b = sqrts;
    double factor = 1.0;
    bool ok = true;
    int sp = 0;

    const int n_visits = ch.n_visits;
    for (int v = 0; v < n_visits; v++) {
      const PhsVisit &V = ch.visit[v];
      double cmsq[2], cm[2], cmax[2];
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const PhsChild &C = V.child[j];
        if (!C.internal) {
          cmsq[j] = C.msq_leaf;
          cm[j] = C.m_leaf;
          cmax[j] = 0.0;
        } else {
          double a0 = C.a0, a1 = C.a1, a2 = C.a2, mn = C.msq_min, mx = C.msq_max;
          cmax[j] = C.m_max;
          if (PER_EVENT) child_constants(C, sqrts, ch.m_tot, a0, a1, a2, mn, mx, cmax[j]);
          double f;
          map_msq(C.map_id, xe[C.x_msq], s, C.m, C.w, mn, mx, a0, a1, a2, cmsq[j], f);
          factor *= f;
          cm[j] = sqrt(cmsq[j]);
        }
      }
      // Kallen function and kinematic test at the visited branch (phs_cpu.cpp:218-233)
      double d = dsub(dsub(msq_b, cmsq[0]), cmsq[1]);
      double lda = dsub(dmul(d, d), dmul(dmul(4.0, cmsq[0]), cmsq[1]));
      ok = ok && (lda > 0.0) && (m_b > dadd(cm[0], cm[1])) && (m_b <= mmax_b);
      double sl = sqrt(lda);
      double pc = sl / (2.0 * m_b);
      factor *= sl / msq_b;

      // rotation + boost of the visited branch (phs_cpu.cpp:299-330)
      double bg = m_b > 0.0 ? p_b / m_b : 0.0;
      double ga = sqrt(1.0 + bg * bg);
      double sphi, cphi;
      sincospi(2.0 * xe[V.x_phi], &sphi, &cphi);
      double b0 = V.b0, b1 = V.b1;
      if (PER_EVENT && V.ct_class == PHS_CT_COLLINEAR) {
        b0 = dmul(V.m, V.m) / s;
        b1 = log(dadd(b0, 1.0) / b0);
      }
      double ct, st, fct;
      map_ct(V.ct_class, xe[V.x_ct], b0, b1, ct, st, fct);
      factor *= fct;
      const double e01 = -bg * st, e03 = bg * ct, e11 = ct * cphi, e12 = -sphi, e13 = st * cphi;
      const double e21 = ct * sphi, e22 = cphi, e23 = st * sphi, e31 = -ga * st, e33 = ga * ct;

      double Ln[16];
      if (V.self_root && !lab) {
        // parent frame is the identity: L0 * L1 = L1
        Ln[0] = ga;  Ln[1] = e01; Ln[2] = 0.0;  Ln[3] = e03;
        Ln[4] = 0.0; Ln[5] = e11; Ln[6] = e12;  Ln[7] = e13;
        Ln[8] = 0.0; Ln[9] = e21; Ln[10] = e22; Ln[11] = e23;
        Ln[12] = bg; Ln[13] = e31; Ln[14] = 0.0; Ln[15] = e33;
      } else {
#pragma unroll
        for (int r = 0; r < 4; r++) {
          const double l0 = L[4 * r], l1 = L[4 * r + 1], l2 = L[4 * r + 2], l3 = L[4 * r + 3];
          Ln[4 * r + 0] = l0 * ga + l3 * bg;
          Ln[4 * r + 3] = l0 * e03 + l1 * e13 + l2 * e23 + l3 * e33;
          if (!V.both_leaves) {
            Ln[4 * r + 1] = l0 * e01 + l1 * e11 + l2 * e21 + l3 * e31;
            Ln[4 * r + 2] = l1 * e12 + l2 * e22;
          } else {
            Ln[4 * r + 1] = 0.0;
            Ln[4 * r + 2] = 0.0;
          }
        }
      }

      // leaf momenta: L_new * (E, 0, 0, +-p) (phs_cpu.cpp:286-291)
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const PhsChild &C = V.child[j];
        if (!C.internal) {
          double pj = j == 0 ? pc : -pc;
          double E = sqrt(cmsq[j] + pj * pj);
          double2 *o = reinterpret_cast<double2 *>(out + 4 * C.out_index);
          o[0] = make_double2(Ln[0] * E + Ln[3] * pj, Ln[4] * E + Ln[7] * pj);
          o[1] = make_double2(Ln[8] * E + Ln[11] * pj, Ln[12] * E + Ln[15] * pj);
        }
      }

      // next frame: push one internal child, carry the other (or pop)
      // (selects instead of indexing keep the child values in registers)
      if (V.push >= 0) {
        const bool j0 = V.push == 0;
#pragma unroll
        for (int i = 0; i < 16; i++) stack_store(smem, sp, i, Ln[i]);
        stack_store(smem, sp, 16, j0 ? cmsq[0] : cmsq[1]);
        stack_store(smem, sp, 17, j0 ? cm[0] : cm[1]);
        stack_store(smem, sp, 18, j0 ? pc : -pc);
        stack_store(smem, sp, 19, j0 ? cmax[0] : cmax[1]);
        sp++;
      }
      if (V.carry >= 0) {
        const bool j0 = V.carry == 0;
#pragma unroll
        for (int i = 0; i < 16; i++) L[i] = Ln[i];
        msq_b = j0 ? cmsq[0] : cmsq[1];
        m_b = j0 ? cm[0] : cm[1];
        p_b = j0 ? pc : -pc;
        mmax_b = j0 ? cmax[0] : cmax[1];
      } else if (sp > 0) {
        sp--;
#pragma unroll
        for (int i = 0; i < 16; i++) L[i] = stack_load(smem, sp, i);
        msq_b = stack_load(smem, sp, 16);
        m_b = stack_load(smem, sp, 17);
        p_b = stack_load(smem, sp, 18);
        mmax_b = stack_load(smem, sp, 19);
      }
    }

    double volume = ch.volume;
    if (PER_EVENT) {
      // phs_cpu.cpp:194-213, bottom-up in post-order with the reference's operation order
      double vol[PHS_MAX_VISITS];
      const double c_int = 4 * PHS_TWOPI2, c_root = 4 * PHS_TWOPI5;
      for (int i = 0; i < ch.n_vol; i++) {
        int k1 = ch.vol_child[i][0], k2 = ch.vol_child[i][1];
        double v1 = k1 >= 0 ? vol[k1] : 1.0, v2 = k2 >= 0 ? vol[k2] : 1.0;
        vol[i] = ch.vol_is_root[i] ? dmul(v1, v2) / c_root
                                   : dmul(dmul(dmul(v1, v2), sqrts), sqrts) / c_int;
      }
      volume = vol[ch.n_vol - 1];
    }
    a.volume[ev] = volume;
    a.factor[ev * a.factor_stride + seg.factor_col] = ok ? factor : 0.0;
    a.ok[ev] = ok ? 1 : 0;
    if (!ok) {
      double2 *o = reinterpret_cast<double2 *>(out);
      for (int i = 0; i < 2 * ch.n_out; i++) o[i] = make_double2(0.0, 0.0);
    }
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

size_t phs_forward_smem_bytes(int stack_depth) {
  return (size_t)stack_depth * PHS_STATE * PHS_FWD_BLOCK * sizeof(double);
}

int phs_forward_blocks_per_sm(int stack_depth, bool per_event) {
  int n = 0;
  size_t smem = phs_forward_smem_bytes(stack_depth);
  if (per_event)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, phs_forward_f64_kernel<true>, PHS_FWD_BLOCK, smem);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, phs_forward_f64_kernel<false>, PHS_FWD_BLOCK, smem);
  return n > 0 ? n : 1;
}

cudaError_t phs_launch_forward_f64(const PhsLaunch &a, int n_blocks, cudaStream_t stream) {
  if (a.n_tiles <= 0) return cudaSuccess;
  size_t smem = phs_forward_smem_bytes(a.stack_depth);
  if (a.E1 && a.E2)
    phs_forward_f64_kernel<true><<<n_blocks, PHS_FWD_BLOCK, smem, stream>>>(a);
  else
    phs_forward_f64_kernel<false><<<n_blocks, PHS_FWD_BLOCK, smem, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t phs_launch_philox(double *x, int64_t n_events, int32_t n_x, uint64_t seed,
                              int64_t first_event, cudaStream_t stream) {
  const int64_t n = n_events * n_x;
  if (n <= 0) return cudaSuccess;
  const int64_t blocks_needed = ((n >> 1) + 2 + 255) / 256;
  const int grid = (int)(blocks_needed < 152 * 16 ? blocks_needed : 152 * 16);
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
// that loads the library holds this array (sizeof(PhsNoAllocScratch), about 0.8 MB) until
// the process exits.  All calls share it and it keeps the last call's contents; each call
// overwrites everything it reads, so nothing needs clearing, but calls that overlap on
// the GPU (different streams or host threads) race on it.
struct PhsNoAllocScratch {
  PhsChannel channels[PHS_NOALLOC_MAX_CHANNELS];
  PhsSegment segments[PHS_NOALLOC_MAX_CHANNELS];
};

static __device__ __align__(256) unsigned char phs_noalloc_scratch[sizeof(PhsNoAllocScratch)];

// Device address of the scratch array per device (filled at set-up; in host code the
// array's name only stands in for the symbol and is never a device address).
static void *g_noalloc_addr[256];

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
  if (!g_noalloc_addr[dev]) {
    // set-up, once per device, with that device current
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, phs_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_addr[dev] = ptr;
  }
  PhsNoAllocScratch *s = static_cast<PhsNoAllocScratch *>(g_noalloc_addr[dev]);
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
  const size_t smem = phs_forward_smem_bytes(a.stack_depth);
  phs_forward_f64_kernel<false><<<n_blocks, PHS_FWD_BLOCK, smem, stream>>>(a);
  return cudaGetLastError();
}
