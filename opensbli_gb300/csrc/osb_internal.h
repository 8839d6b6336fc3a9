// osb_internal.h -- host-side types shared by the translation units of libosb_gb300.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/osb_gb300.h"
#include "osb_kernels.cuh"

namespace osb {

int fail(int code, const char* fmt, ...);

#define OSB_CK(call)                                                                             \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return ::osb::fail(OSB_ECUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

struct Block {
  osb_block_desc d;
  BlockK k;
  float* mf_buf = nullptr;   // FP32 copies of the metrics (FP32-residual path, curvilinear)
  void* ys_buf = nullptr;    // stretched y grid: D11, SD111 rows (FP64) and their FP32 copies
  float* qf_base = nullptr;  // FP32 state buffer allocated with the block (FP32-residual path)
  float* qf_alt = nullptr;   // second FP32 state buffer of the persistent stage's ping-pong
  void* filt_ws = nullptr;   // filtered blocks: kappa + 15 filter-flux arrays (residual precision)
  int* xrows = nullptr;      // x-sweep rows (linear index of x = 0) grouped by 32-byte-sector phase
};

// Kernel families for per-kernel timing (osb_timing_report).
enum { FAM_FLUX_X = 0, FAM_FLUX_Y, FAM_FLUX_Z, FAM_CENTRAL, FAM_RK, FAM_BC, FAM_REDUCE, FAM_PERSISTENT, FAM_FILTER, FAM_N };

struct BatchBlock;

// Device tables of the persistent stage (osb_batch.cu).
struct BatchState {
  BatchBlock* tab[2] = {nullptr, nullptr};  // per FP32-buffer parity
  int4* work = nullptr;                     // tiles: (block, x0, y0, -)
  int* counter = nullptr;                   // dynamic tile claiming
  int nwork = 0;
  bool ready = false;
};

struct TimedEvent {
  cudaEvent_t a, b;
  int fam;
};

}  // namespace osb

struct osb_ctx {
  int device = 0;
  int prec = OSB_PREC_FP64;
  cudaStream_t stream = nullptr;
  std::vector<osb::Block> blocks;
  int rk_kind = OSB_RK_LOW_STORAGE;
  int nst = 3;
  double A[8] = {0.0, -5.0 / 9.0, -153.0 / 128.0};
  double B[8] = {1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0};
  bool graphs = true;
  cudaGraphExec_t gexec = nullptr;
  cudaGraphExec_t gexec_p[2] = {nullptr, nullptr};  // persistent stage: one graph per FP32 parity
  osb_schedule sched = {OSB_SCHED_AUTO, 16, 2, 1, 0, 1};
  osb::BatchState batch;
  int qf_parity = 0;
  void* resident = nullptr;  // device table of the resident 1D path (osb_resident.cu)
  int resident_n = 0;
  double g_dt = 0.0;
  long long g_kernels = 0;
  double* red = nullptr;              // device reduction partials (+ final slot)
  double* red_host = nullptr;         // pinned
  unsigned long long* bad = nullptr;  // [0] non-finite values, [1] staging waits that ran out
  int red_slots = 0;
  long long launches = 0;
  int variant = -1;
  int central_bulk = 0;  // FP32 central kernel: raw planes by register loads (0) or bulk copies (1)
  int sm_count = 152;
  bool timing = false;                    // per-kernel CUDA-event timing (graphs bypassed)
  std::vector<osb::TimedEvent> events;    // pending timed launches
  std::vector<cudaEvent_t> event_pool;
  double fam_ms[osb::FAM_N] = {0};
  long long fam_count[osb::FAM_N] = {0};
  // osb_step_requests: copy streams, two device staging slots per direction and their events
  cudaStream_t cs_in = nullptr, cs_out = nullptr;
  void* stage_in[2] = {nullptr, nullptr};
  void* stage_out[2] = {nullptr, nullptr};
  size_t stage_bytes = 0;
  cudaEvent_t ev_in[2] = {nullptr, nullptr}, ev_used[2] = {nullptr, nullptr};
  cudaEvent_t ev_res[2] = {nullptr, nullptr}, ev_out[2] = {nullptr, nullptr};
};

namespace osb {

// Brackets one kernel launch with events when timing is enabled.
void timing_begin(osb_ctx* c, int fam);
void timing_end(osb_ctx* c);

// Characteristic flux sweeps of one block (x writes R, y/z accumulate; with rf the last sweep
// applies the RK update, FP32 path, 2D/3D); one instantiation per precision and dimension lives
// in osb_flux.cu.
int flux_f64_1d(osb_ctx* c, Block& bl, const SchemeParams& sp, const RkFuse* rf);
int flux_f64_2d(osb_ctx* c, Block& bl, const SchemeParams& sp, const RkFuse* rf);
int flux_f64_3d(osb_ctx* c, Block& bl, const SchemeParams& sp, const RkFuse* rf);
int flux_f32_1d(osb_ctx* c, Block& bl, const SchemeParams& sp, const RkFuse* rf);
int flux_f32_2d(osb_ctx* c, Block& bl, const SchemeParams& sp, const RkFuse* rf);
int flux_f32_3d(osb_ctx* c, Block& bl, const SchemeParams& sp, const RkFuse* rf);
// The same for curvilinear blocks (metric arrays present).
int flux_curv_f64_2d(osb_ctx* c, Block& bl, const SchemeParams& sp, const RkFuse* rf);
int flux_curv_f64_3d(osb_ctx* c, Block& bl, const SchemeParams& sp, const RkFuse* rf);
int flux_curv_f32_2d(osb_ctx* c, Block& bl, const SchemeParams& sp, const RkFuse* rf);
int flux_curv_f32_3d(osb_ctx* c, Block& bl, const SchemeParams& sp, const RkFuse* rf);
// Persistent fused stage for batches of 2D periodic blocks (osb_batch.cu).
bool batch_eligible(const osb_ctx* c, std::string* why);
int batch_build(osb_ctx* c);
void batch_free(osb_ctx* c);
void batch_set_parity(osb_ctx* c, int parity);
int batch_stage(osb_ctx* c, int s, double dt);
size_t batch_smem(int ty);
// Central convective and/or viscous terms of one 3D block (osb_central.cu).
// Resident CTAs per SM of a kernel at a launch shape (occupancy calculator; 1 if it fails).
template <typename K>
inline int resident_ctas(K kern, int threads, size_t smem) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, threads, smem) != cudaSuccess) {
    cudaGetLastError();
    nb = 1;
  }
  return nb > 0 ? nb : 1;
}

// Number of chunks a line of n work units (interfaces, planes) is cut into when each chunk
// count k gives ctas_per_chunk * k CTAs over `slots` resident CTA slots: minimises
// waves * (chunk length + overhead), where overhead is the start-up cost of a chunk in work
// units, so the last wave is nearly full without paying for many short chunks.  Chunks are at
// least min_len long unless the line is shorter.
inline int wave_chunks(int n, long ctas_per_chunk, long slots, double overhead, int min_len) {
  int best = 1;
  double best_cost = 1e300;
  for (int k = 1; k <= n; ++k) {
    const int len = (n + k - 1) / k;
    if (k > 1 && len < min_len) break;
    if ((n + len - 1) / len != k) continue;  // the same split as a smaller k
    const long waves = (ctas_per_chunk * k + slots - 1) / slots;
    const double cost = (double)waves * (len + overhead);
    if (cost < best_cost * (1.0 - 1e-9)) {
      best_cost = cost;
      best = k;
    }
  }
  return best;
}

// Grid size of a grid-stride launch over n items: enough CTAs to cover them, at most 8 per SM.
int grid_for(osb_ctx* c, long n, int threads);

// Whole osb_step calls of small 1D blocks in one launch, one CTA per block (osb_resident.cu).
bool resident_eligible(const osb_ctx* c);
int resident_step(osb_ctx* c, double dt, int nsteps);
int resident_f64(osb_ctx* c, double dt, int nsteps);
int resident_f32(osb_ctx* c, double dt, int nsteps);

// Non-linear WENO filter step of a filtered block (osb_filter.cu), after a full RK step.
int filter_f64(osb_ctx* c, Block& bl, double dt);
int filter_f32(osb_ctx* c, Block& bl, double dt);
// TVD filter: u at index -2 of each direction from the state the last RK stage reads (launched
// before that stage)
int tvd_stale_f64(osb_ctx* c, Block& bl);
int tvd_stale_f32(osb_ctx* c, Block& bl);

int central_f64(osb_ctx* c, Block& bl, bool conv, int first, const RkFuse* rf);
int central_f32(osb_ctx* c, Block& bl, bool conv, int first, const RkFuse* rf);

}  // namespace osb
