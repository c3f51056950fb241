// Host-side context, workspace and batch engine shared by the C ABI files.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/entropical_gb300.h"

namespace ent { struct ILogEntry; }

// Grow-only device workspace. Blocks are kept across calls; a call that
// needed more than one block coalesces them into one when it ends.
struct Arena {
  struct Block {
    void* ptr;
    size_t size;
  };
  std::vector<Block> blocks;
  size_t used_in_last = 0;
  size_t total_used = 0;
  size_t peak = 0;  // largest total_used since the last reset
  void* alloc(size_t bytes);
  void reset();
  void coalesce();  // one block of this call's peak use (contents discarded)
  void release();
  size_t spare() const;  // bytes the next allocations get without cudaMalloc
  // Rewinding to a mark gives back what was allocated after it; blocks added
  // since are freed but the last, which is kept empty. Only while nothing
  // in flight uses that memory (the stream idle).
  struct Mark {
    size_t n_blocks, used_in_last, total_used;
  };
  Mark mark() const { return {blocks.size(), used_in_last, total_used}; }
  void rewind(const Mark& m);
};

struct Ctx {
  int device = 0;
  int n_sms = 1;
  cudaStream_t stream = nullptr;
  uint32_t* d_err = nullptr;
  double2* d_logtab = nullptr;  // LOG64_TABLE_ENTRIES entries of log_fp64
  ent::ILogEntry* d_ilogtab = nullptr;  // table of the strip-moment epilogue's log
  cudaEvent_t ev_call0 = nullptr, ev_call1 = nullptr;
  cudaEvent_t ev_k0 = nullptr, ev_k1 = nullptr;
  cudaEvent_t ev_d[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
  bool ran_d[3] = {false, false, false};
  // strip moments: edge (symmetric) kernel and target kernel
  cudaEvent_t ev_m[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  bool ran_m = false;
  bool ran_k = false;  // ev_k0 / ev_k1 bracket this call's pair kernels
  uint64_t h_nsrc_d[3] = {0, 0, 0};
  Arena arena;
  std::string last_error;
  ent_call_stats stats{};
  bool pending_pairs = false;
  uint32_t strip_subdiv = 2;  // cells per bandwidth along dimension 1 (d = 2)
  uint32_t strip_subdiv3 = 1;  // cells per bandwidth along dimensions 1, 2 (d = 3)
  // autotune cache: (d << 8 | size bucket) -> {pair body, targets per warp,
  // cells per bandwidth}
  struct TuneChoice {
    int variant, tile_r;
    uint32_t cells;
  };
  std::map<uint32_t, TuneChoice> tune_cache;
  int tile_r[3] = {16, 16, 8};  // targets per warp of the pair kernel, by d
  // pair body per dimension: 0 min-based, 1 saturating FMA, 2 saturating at
  // 5 CTAs/SM, 3 as 2 with larger chunks (fastest measured: 2, 2, 1)
  // PAIR_RANGE for d = 1, PAIR_MOMENT for d = 2, PAIR_SYM for d = 3 (engine.h)
  int pair_variant[3] = {6, 7, 4};
  // While the 2-D body is the default, the engine picks per instance: the
  // strip moments for supports of at least MOMENT_MIN_SUPPORT neighbours per
  // target when such instances hold MOMENT_MIN_POINTS points together, else
  // PAIR_SYM (its work items fill the GPU where one thread per target cannot,
  // and it is faster on small supports). An explicit choice (set_tuning, the
  // autotuner) clears it: then every 2-D instance takes the moments.
  bool moment_auto = true;
  uint32_t moment_cells = 3;  // strips per bandwidth of PAIR_MOMENT (2..12)
  bool use_graphs = true;       // capture the batch kernel sequence in a CUDA graph
  // Instances of one engine run (at most 65535); an estimator job with more,
  // or more than the device's free memory holds, runs as several batches.
  uint32_t max_batch_instances = 65535;
  // The batch's executable graph, kept across calls: a later batch is
  // captured again and, when its kernel sequence has the same shape, the
  // executable is updated in place (cudaGraphExecUpdate: new pointers, sizes
  // and grids) instead of being instantiated anew.
  cudaGraphExec_t graph_exec = nullptr;
  uint32_t graph_updates = 0, graph_instantiations = 0;
  // Pinned host staging for file loads: two buffers of stage_bytes, filled
  // by the host threads in turn while the other one is being copied; kept
  // across calls (allocated on first use, freed with the context).
  uint8_t* h_stage[2] = {nullptr, nullptr};
  cudaEvent_t ev_stage[2] = {nullptr, nullptr};
  size_t stage_bytes = 0;
  int ensure_staging(size_t bytes);

  // grid of a persistent kernel: resident CTAs per SM x SMs, capped by work
  unsigned persistent_grid(uint32_t n_work, const void* kern, int threads, size_t smem);
  int fail(int status, const std::string& msg);
  int cuda_fail(cudaError_t e, const char* where);
  int begin_call();
  int end_call();
  void collect_kernel_stats();
};

// A device column view of n float32 values.
struct ViewSpec {
  const float* x;
  uint32_t n;
};

// One density instance over d views.
struct InstSpec {
  uint32_t d = 1;
  uint32_t n = 0;
  uint32_t view[3] = {0, 0, 0};
  float h[3] = {1.f, 1.f, 1.f};
  double norm = 1.0;
  double* out = nullptr;  // device, by original index (nullable)
  uint32_t S = 2;
  // d = 3: cells per bandwidth along dimensions 1 and 2 (0: the context's)
  uint32_t S3[2] = {0, 0};
  // target share: only the targets at sorted positions [n part / n_parts,
  // n (part + 1) / n_parts) are computed (the reference's split of one
  // density's target rows over GPUs); a share runs the ordered pair kernel,
  // which sums each target fully within its own tile
  uint32_t part = 0, n_parts = 1;
};

namespace ent { struct ViewStats; }
#include "engine.h"

// Column statistics and value order of a set of views (one host sync).
struct SortedViews {
  std::vector<ent::ViewStats> stats;
  std::vector<uint64_t> off;  // element offset of each view in perm
  uint32_t* perm = nullptr;   // device: per view, sorted local indices
  uint32_t* keys = nullptr;   // device: per view, the sorted orderable keys
  uint32_t max_n = 0;
};
int sort_views(Ctx& c, const std::vector<ViewSpec>& views, SortedViews* out);

// AMISE convolution / bandwidth search over device columns stored back to
// back in `raw`. mode 0: convolution at the given bandwidths; 1: full
// interval search; 2: search warm-started from the given bandwidths.
int hestimate_engine(Ctx& c, const float* raw, const std::vector<uint64_t>& raw_off,
                     const std::vector<uint32_t>& lens, int mode, const float* h_fixed_or_init,
                     int skip, float* h_out, float* conv_out, ent_hest_stats* stats,
                     const float* d_log_ratio);

// Learned warm start (mlp.cu): features of device instances and the MLP
// forward pass on device data.
int mlp_features_device(Ctx& c, const std::vector<const float*>& base,
                        const std::vector<uint32_t>& n, const std::vector<uint32_t>& d,
                        float* d_feat);
int mlp_forward_device(Ctx& c, ent_mlp* net, float* d_feat, size_t B, float* d_out);

struct EngineOut {
  double* d_logsum_sorted = nullptr;  // per instance, in slot order
  std::vector<uint32_t> slot_order;   // slot rank -> instance index
};

struct Engine {
  uint32_t group_base[4] = {0, 0, 0, 0};
  uint32_t group_slots[4] = {0, 0, 0, 0};
  int run(Ctx& c, const std::vector<ViewSpec>& views,
          const std::vector<InstSpec>& insts, uint32_t mode, EngineOut* out);
};

// Runs `insts` as one engine batch when the job fits one (at most
// c.max_batch_instances instances and 65535 views, its estimated workspace
// within the device's free memory), else as consecutive batches of as many
// instances as fit, each with the views it uses. After each run,
// done(first, count, out) gets the run's instances [first, first + count)
// and its EngineOut (slot_order indexes the run's instances). Between runs
// of a split job the stream is synchronised and the run's workspace given
// back; the single run returns with its work in flight, as Engine::run does.
typedef int (*BatchDone)(void* arg, size_t first, size_t count, const EngineOut& out);

// Device memory one batch or pass may take: the device's free memory and the
// workspace already held, less an eighth (at least 2 GB) for the allocator's
// rounding, graphs and other work on the device.
size_t device_budget(Ctx& c);
int run_engine_batches(Ctx& c, const std::vector<ViewSpec>& views,
                       const std::vector<InstSpec>& insts, uint32_t mode, BatchDone done,
                       void* arg);

int validate_selection(Ctx& c, size_t n_rows, size_t n_cols,
                       const uint32_t* i_cols, const float* h,
                       const uint32_t* tau, uint32_t d, size_t* n_sel);
