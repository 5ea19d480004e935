// ref_harness.cpp -- drives the reference's own, unmodified CPU path.
//
// TEST INFRASTRUCTURE ONLY.  Linked (by oracle/Makefile, target _ref) with the
// reference sources phs_cpu.cpp and global_phs.cpp, compiled where they lie,
// into oracle/_ref/libphsref.so.  It exists to pin the restatement in
// phs_oracle.c against the reference bit for bit, and to time the reference
// CPU path as a baseline.  The product never loads it.
//
// It supplies what phs_cpu.cpp expects from the rest of the reference program:
//   - the tree globals daughters1/daughters2/has_children (phs.h:39-42), holding
//     0-based slots (code-1) as init_phs_gpu leaves them (phs.cu:392-397);
//   - input_control (file_input.h:14-27; file_input.cpp needs rapidjson, which
//     the reference does not vendor, so it is not linked);
//   - the size globals set as main.cpp:271-285 sets them;
//   - mass sums, restated from set_mass_sum (phs.cu:61-78, a CUDA file);
// and runs the per-event loop of phs_cpu.cpp:582-600 (init_msq_cpu, set_msq_cpu,
// set_angles_cpu) over all host threads.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "file_input.h"
#include "global_phs.h"
#include "phs.h"

int **daughters1 = nullptr;
int **daughters2 = nullptr;
int **has_children = nullptr;
int **friends = nullptr;
int **i_scatter = nullptr;
int **i_gather = nullptr;
int *cmd_msq = nullptr;
int *cmd_boost_o = nullptr;
int *cmd_boost_t = nullptr;
input_control_t input_control;

// Defined in phs_cpu.cpp (signatures at phs_cpu.cpp:174, 283, 541); phs.h does not declare them.
void set_msq_cpu(int channel, int branch_idx, double m_tot, double *x, size_t *id_x, double sqrts,
                 phs_prt_t *prt, double *factor, double *volume, bool *ok, double *p_decay);
void set_angles_cpu(int i_event, int channel, int branch_idx, double *x, size_t *idx_x, double s,
                    double *factor, double *p_decay, phs_prt_t *prt, double L0[4][4]);
void init_msq_cpu(phs_prt_t *prt);

static int g_channels = 0;

static void harness_mass_sum(int c, int slot) {
  double *ms = mappings_host[c].mass_sum;
  if (has_children[c][slot]) {
    int k1 = daughters1[c][slot], k2 = daughters2[c][slot];
    harness_mass_sum(c, k1);
    harness_mass_sum(c, k2);
    ms[slot] = ms[k1] + ms[k2];
  } else {
    int ld2 = 0, bb = slot + 1;
    while (bb > 1) { bb /= 2; ld2++; }
    ms[slot] = flv_masses[ld2 + N_EXT_IN];
  }
}

extern "C" void ref_teardown() {
  for (int c = 0; c < g_channels; c++) {
    free(daughters1[c]); free(daughters2[c]); free(has_children[c]); free(friends[c]);
    free(mappings_host[c].map_id); free(mappings_host[c].masses); free(mappings_host[c].widths);
    free(mappings_host[c].a); free(mappings_host[c].b); free(mappings_host[c].mass_sum);
  }
  free(daughters1); free(daughters2); free(has_children); free(friends); free(mappings_host);
  free(flv_masses); free(flv_widths);
  daughters1 = daughters2 = has_children = friends = nullptr;
  mappings_host = nullptr; flv_masses = flv_widths = nullptr;
  g_channels = 0;
}

// Tables as the reference's C-ABI takes them (whizard_gpu_phs.cpp:57-87): daughters and
// has_children over N_PRT codes (1-based daughter codes, 0 = none), mappings over N_PRT_OUT.
extern "C" int ref_setup(int n_in, int n_out, int n_channels, const int *d1, const int *d2,
                         const int *hc, const int *map_ids, const double *map_masses,
                         const double *map_widths, const double *flv_m, const double *flv_w,
                         double sqrts) {
  if (g_channels) ref_teardown();
  N_CHANNELS = n_channels;
  N_EXT_IN = n_in;
  N_EXT_OUT = n_out;
  N_EXT_TOT = n_in + n_out;
  N_PRT = (1 << N_EXT_TOT) - 1;
  N_PRT_OUT = (1 << N_EXT_OUT) - 1;
  PRT_STRIDE = 4 * N_PRT;
  ROOT_BRANCH = N_PRT_OUT - 1;
  N_BRANCHES = 2 * N_EXT_OUT - 1;
  N_BRANCHES_INTERNAL = N_BRANCHES - N_EXT_OUT;
  N_MSQ = N_EXT_OUT - 2;
  N_LAMBDA_IN = N_EXT_OUT - 1;
  N_BOOSTS = N_LAMBDA_IN + 1;
  N_LAMBDA_OUT = N_BRANCHES;
  g_channels = n_channels;
  flv_masses = (double *)malloc(N_EXT_TOT * sizeof(double));
  flv_widths = (double *)malloc(N_EXT_TOT * sizeof(double));
  memcpy(flv_masses, flv_m, N_EXT_TOT * sizeof(double));
  memcpy(flv_widths, flv_w, N_EXT_TOT * sizeof(double));
  daughters1 = (int **)malloc(n_channels * sizeof(int *));
  daughters2 = (int **)malloc(n_channels * sizeof(int *));
  has_children = (int **)malloc(n_channels * sizeof(int *));
  friends = (int **)malloc(n_channels * sizeof(int *));
  mappings_host = (mapping_t *)calloc(n_channels, sizeof(mapping_t));
  for (int c = 0; c < n_channels; c++) {
    daughters1[c] = (int *)malloc(N_PRT * sizeof(int));
    daughters2[c] = (int *)malloc(N_PRT * sizeof(int));
    has_children[c] = (int *)malloc(N_PRT * sizeof(int));
    friends[c] = (int *)calloc(N_PRT, sizeof(int));
    for (int i = 0; i < N_PRT; i++) {
      daughters1[c][i] = d1[c * N_PRT + i] - 1;
      daughters2[c][i] = d2[c * N_PRT + i] - 1;
      has_children[c][i] = hc[c * N_PRT + i];
    }
    mapping_t &mh = mappings_host[c];
    mh.map_id = (int *)malloc(N_PRT_OUT * sizeof(int));
    mh.masses = (double *)malloc(N_PRT_OUT * sizeof(double));
    mh.widths = (double *)malloc(N_PRT_OUT * sizeof(double));
    mh.a = (map_constant_t *)malloc(N_PRT_OUT * sizeof(map_constant_t));
    mh.b = (map_constant_t *)malloc(N_PRT_OUT * sizeof(map_constant_t));
    mh.mass_sum = (double *)calloc(N_PRT_OUT, sizeof(double));
    for (int i = 0; i < N_PRT_OUT; i++) {
      mh.map_id[i] = map_ids[c * N_PRT_OUT + i];
      mh.masses[i] = map_masses[c * N_PRT_OUT + i];
      mh.widths[i] = map_widths[c * N_PRT_OUT + i];
    }
    harness_mass_sum(c, ROOT_BRANCH);
  }
  input_control.check_cpu = false;
  input_control.do_inverse_mapping = false;
  init_mapping_constants_cpu(n_channels, sqrts);
  return 0;
}

// One event as phs_cpu.cpp:583-600 runs it.  Outputs for ok=false events are left as
// the reference leaves them: momenta 0 (they are never written), factor/volume partial.
static void ref_range(long lo, long hi, int n_x, const double *x, const int *channels,
                      double sqrts, double *p, double *factors, double *volumes,
                      unsigned char *oks) {
  std::vector<phs_prt_t> prt(N_PRT);
  std::vector<double> p_decay(N_PRT);
  double L0[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
  for (long i = lo; i < hi; i++) {
    bool ok = true;
    int ch = channels ? channels[i] : 0;
    std::fill(p_decay.begin(), p_decay.end(), 0.0);
    memset(prt.data(), 0, N_PRT * sizeof(phs_prt_t));
    init_msq_cpu(prt.data());
    size_t id_x = 0;
    double factor = 0, volume = 0;
    double m_tot = mappings_host[ch].mass_sum[ROOT_BRANCH];
    set_msq_cpu(ch, ROOT_BRANCH, m_tot, const_cast<double *>(x) + (size_t)n_x * i, &id_x, sqrts,
                prt.data(), &factor, &volume, &ok, p_decay.data());
    if (ok)
      set_angles_cpu((int)i, ch, ROOT_BRANCH, const_cast<double *>(x) + (size_t)n_x * i, &id_x,
                     sqrts * sqrts, &factor, p_decay.data(), prt.data(), L0);
    for (int j = 0; j < N_EXT_OUT; j++)
      for (int r = 0; r < 4; r++) p[(size_t)4 * N_EXT_OUT * i + 4 * j + r] = prt[(1 << j) - 1].p[r];
    factors[i] = factor;
    volumes[i] = volume;
    oks[i] = ok ? 1 : 0;
  }
}

extern "C" int ref_generate(long n_events, int n_x, const double *x, const int *channels,
                            double sqrts, double *p, double *factors, double *volumes,
                            unsigned char *oks, int n_threads) {
  if (!g_channels) return -1;
  if (n_threads < 1) n_threads = 1;
  if (n_events < n_threads) n_threads = n_events > 0 ? (int)n_events : 1;
  std::vector<std::thread> th;
  for (int t = 1; t < n_threads; t++)
    th.emplace_back(ref_range, n_events * t / n_threads, n_events * (t + 1) / n_threads, n_x, x,
                    channels, sqrts, p, factors, volumes, oks);
  ref_range(0, n_events / n_threads, n_x, x, channels, sqrts, p, factors, volumes, oks);
  for (auto &t : th) t.join();
  return 0;
}
