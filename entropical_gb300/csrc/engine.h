// Internal interfaces between the CUDA translation units of the entropical
// GB300 library. Not part of the public C ABI (include/entropical_gb300.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace ent {

// ------------------------------------------------------------ radix sort
struct SegTableDev {
  const uint64_t* seg_off;   // element offset of segment s
  const uint32_t* seg_len;   // element count of segment s
  const uint32_t* seg_blk0;  // first radix block of segment s (n_seg + 1)
  const uint32_t* blk_seg;   // segment of every radix block
  uint32_t* hist;            // 256 counters per radix block
};

uint32_t radix_blocks_for(uint32_t len);
// Sorts every segment of (keys, vals) on bits [begin_bit, end_bit). The
// pointers are swapped so that on return keys/vals hold the result.
cudaError_t seg_radix_sort(cudaStream_t st, const SegTableDev& t,
                           uint32_t n_seg, uint32_t total_blocks,
                           uint32_t*& keys, uint32_t*& vals, uint32_t*& ktmp,
                           uint32_t*& vtmp, int begin_bit, int end_bit);

// -------------------------------------------------------- density engine
// candidate runs per tile: 2S+1 strips for d = 2 (S <= 4 cells per
// bandwidth), (2S+1)^2 for d = 3 (S <= 2)
constexpr int MAX_RUNS = 25;

// One column view: a contiguous float32 range on the device (a selected,
// possibly lagged coordinate column).
struct ViewDev {
  const float* x;
  uint32_t n;
  uint32_t pad;
};

struct ViewStats {
  float mn, mx;
  uint32_t nonfinite;
  uint32_t pad;
};

// One density instance: d coordinate views of n points, bandwidths h.
struct InstDev {
  const float* x[3];        // coordinates by original (instance-local) index
  uint32_t n, d, S, n_strips;
  uint32_t ncell1, ncell2;  // cells along dims 1 and 2 (1 when absent)
  uint32_t tile_base, tile_cap;
  float lo1, lo2;           // cell-grid origins
  float inv_w1, inv_w2;     // inverse cell widths (cell width = h/S, widened so
                            // that the FP32 cell index of k_strip_keys can
                            // never put two points within h more than S apart)
  float sc[3];  // exact power-of-two scale 2^k_j with g_j = h_j 2^k_j in [0.5, 1)
  float g2[3];  // g_j^2: the support radius squared in scaled units
  const uint32_t* perm0;    // dimension-0 sorted order (view sort)
  uint32_t* perm;           // final strip-major order
  const uint32_t* skeys;    // sorted strip keys (d >= 2)
  void* pts;                // sorted points x_j * sc_j (float/float2/float4)
  uint32_t* strip_start;    // n_strips + 1
  uint32_t* tile_off;       // n_strips + 1
  double scale;             // 0.75^d / (norm * prod h_j * prod g_j^2)
  double* out;              // per-point density by original index (nullable)
  uint32_t tt;              // targets per tile
  uint32_t sym;             // 1: symmetric evaluation (each unordered pair once)
  uint32_t S2;              // d = 3: cells per bandwidth along dimension 2
  uint32_t parts;           // work items per tile (source runs split; 0 = 1);
                            // tile_cap counts work-item slots
  double* acc;              // symmetric mode: unscaled sums by sorted position
  uint32_t fused;           // 1: the strip-moment kernel owns this instance:
                            // its tiles carry only the edge run (the strip S
                            // above), the symmetric pair kernel sums those
                            // pairs into acc and its finish skips it
  uint32_t pad2;
  uint32_t t_lo, t_hi;      // targets computed: sorted positions [t_lo, t_hi)
};

struct TileDesc {
  uint32_t inst;
  uint32_t t_begin;  // first target (position in the sorted order)
  uint32_t t_count;  // 0 marks an unused slot
  uint32_t n_runs;
  uint32_t part;     // which share of the tile's sources (symmetric kernel)
  uint32_t pad;
  uint32_t lo[MAX_RUNS];   // candidate-source runs (sorted positions)
  uint32_t len[MAX_RUNS];
};

// Epilogue modes of the density kernel.
enum : uint32_t {
  DM_WRITE_F64 = 1u,  // out[perm[k]] = density (double)
  DM_LOGSUM = 2u,     // tile_logsum[g] = sum of log(density) over the tile
  DM_COUNT = 4u,      // count in-support pairs instead of summing the kernel
  DM_SUMV = 8u,       // tile_logsum[g] = sum of the per-point values (no log)
};

// Kernel launch helpers (density.cu).
cudaError_t launch_colstats(cudaStream_t st, const ViewDev* views,
                            uint32_t n_views, ViewStats* stats);
cudaError_t launch_view_keys(cudaStream_t st, const ViewDev* views,
                             const uint64_t* view_off, uint32_t n_views,
                             uint32_t max_n, uint32_t* keys, uint32_t* vals);
cudaError_t launch_strip_keys(cudaStream_t st, const InstDev* insts,
                              const uint32_t* inst_ids, const uint64_t* seg_off,
                              uint32_t n_seg, uint32_t max_n, uint32_t* keys,
                              uint32_t* vals);
// strip_start of every instance (max_strips: the largest n_strips)
cudaError_t launch_strip_bounds(cudaStream_t st, const InstDev* insts,
                                uint32_t n_inst, uint32_t max_strips);
cudaError_t launch_tile_offsets(cudaStream_t st, const InstDev* insts,
                                uint32_t n_inst);
cudaError_t launch_gather_pts(cudaStream_t st, const InstDev* insts,
                              uint32_t n_inst, uint32_t max_n);
cudaError_t launch_plan(cudaStream_t st, const InstDev* insts, uint32_t n_inst,
                        const uint32_t* inst_tile_base, TileDesc* tiles,
                        uint32_t n_slots, uint64_t* n_src_total);
// v: pair body, 0 = min-based, 1 = saturating FMA (needs g^2 < 1), 2-3 as 1
// with other occupancy / chunk sizes, 4-5 symmetric (PAIR_SYM; r ignored),
// 6 range sums (PAIR_RANGE, d = 1), 7 strip moments (PAIR_MOMENT, d = 2);
// those two are not launched through here
cudaError_t launch_density(cudaStream_t st, int d, int r, int v, const TileDesc* tiles,
                           uint32_t n_slots, const InstDev* insts,
                           uint32_t* work_counter, uint32_t* err,
                           double* tile_logsum, uint32_t mode, int n_sms,
                           int* launched_ctas);
// the original (min-based) pair body
cudaError_t launch_density(cudaStream_t st, int d, int r, const TileDesc* tiles,
                           uint32_t n_slots, const InstDev* insts,
                           uint32_t* work_counter, uint32_t* err,
                           double* tile_logsum, uint32_t mode, int n_sms,
                           int* launched_ctas);
// targets per warp R available for dimension d; tile = 4 warps x R targets
int density_r_supported(int d, int r);
int density_variant_supported(int d, int r, int v);
int density_tile_targets(int d, int r);
// Pair bodies PAIR_SYM and PAIR_SYM + 1 (density_sym.cu) evaluate every
// unordered pair once and add it to both points: the plan keeps only sources
// at or after the tile's first target (InstDev::sym), the kernel accumulates
// into InstDev::acc (zeroed first), and launch_sym_finish turns the sums
// into the epilogue of `mode`. Their tile shape is their own (sym_tile_r).
constexpr int PAIR_SYM = 4;
__host__ __device__ constexpr bool pair_is_sym(int v) {
  return v == PAIR_SYM || v == PAIR_SYM + 1;
}
// Pair body PAIR_RANGE (d = 1 only, range1d.cu): the support of a target in
// the value-sorted points is one index range, so its sum comes from exact
// fixed-point prefix sums after two binary searches. It writes InstDev::acc
// and is finished by launch_sym_finish like the symmetric bodies.
constexpr int PAIR_RANGE = 6;
// Pair body PAIR_MOMENT (d = 2 only, moments2d.cu): per target and strip,
// the x-support is one index range; strips within S - 1 of the target's own
// are summed from exact fixed-point moment prefix sums, the two edge strips
// at distance S pair by pair by the symmetric kernel (edge-only tiles), which
// runs first and leaves its sums in InstDev::acc.
constexpr int PAIR_MOMENT = 7;
constexpr uint64_t MOMENT_MIN_POINTS = 1000000;  // default rule: see Ctx::moment_auto
// Default rule per instance: the moments take a 2-D instance with at least
// this many in-support neighbours per target (sampled estimate, within 15 %
// of the true mean on the bench data). Measured with the edge strips on the
// symmetric kernel and the fixed-point epilogue (thresholds 0 / 2,000 /
// 4,000 / 6,000): TE 32 x 200k x 3 lags 1018 / 1021 / 1024 / 1058 ms, the
// uneven batch's 2-D part 7.64 / 6.86 / 7.07 / 7.30 ms, MI unchanged.
constexpr float MOMENT_MIN_SUPPORT = 2000.f;
__host__ __device__ constexpr bool pair_uses_acc(int v) {
  return pair_is_sym(v) || v == PAIR_RANGE || v == PAIR_MOMENT;
}
int sym_tile_r(int d, int v);
int sym_tile_targets(int d, int v);
struct Range1D {
  const float* y;       // value-sorted scaled points (InstDev::pts)
  double* acc;          // unscaled sums by sorted position (InstDev::acc)
  void* P;              // (n + 1) x {sum Y, sum Y^2}, 128-bit each
  uint32_t n;
  float g2;
  uint32_t chunk_base;  // first prefix chunk of the instance
  uint32_t blk_base;    // first target block of the instance
};
uint32_t range1d_chunks(uint32_t n);
uint32_t range1d_blocks(uint32_t n);
size_t range1d_prefix_bytes(uint32_t n);
// rs: 1-D instances in ascending blk_base; chunk_tot: 32 B per chunk
cudaError_t launch_range1d(cudaStream_t st, const Range1D* rs, uint32_t n_inst, uint32_t max_n,
                           const uint32_t* blk_base, uint32_t n_blocks, void* chunk_tot);
struct Mom2D {
  const float2* pts;            // strip-major scaled points (InstDev::pts)
  const uint32_t* skeys;        // strip of every sorted position
  const uint32_t* strip_start;  // n_strips + 1
  float2* ybound;               // per strip: smallest and largest scaled y
  void* P;                      // (n + 1) x 8 moment prefix sums, 128-bit each
  const uint32_t* perm;         // original index of every sorted position
  double* out;                  // per-point density by original index (nullable)
  const double* acc;            // edge-strip sums by sorted position (InstDev::acc)
  double scale;                 // InstDev::scale
  double logc;                  // log(scale) - 92 log 2 (the epilogue's offset)
  uint32_t n, n_strips, S;      // strips within S - 1 of a target's own are
                                // summed here, those at S by the pair kernel
  float g2[2];
  uint32_t chunk_base;          // first prefix chunk of the instance
  uint32_t blk_base;            // first target block of the instance
  uint32_t slot_base;           // first tile_logsum slot (one per target block)
};
// Table entry of the strip-moment epilogue's log (moments2d.cu): inv ~ 1/c,
// c = 1 + (k + 1/2)/256, and log(1/inv) in 2^-56 fixed point.
struct ILogEntry {
  float inv;
  float pad;
  long long l56;
};
constexpr int ILOG_TABLE_ENTRIES = 256;
cudaError_t launch_ilog_test(cudaStream_t st, const unsigned long long* t, size_t n,
                             const ILogEntry* tab, long long* out);
uint32_t moments2d_chunks(uint32_t n);
uint32_t moments2d_blocks(uint32_t n);
size_t moments2d_prefix_bytes(uint32_t n);
// The strip extents and moment prefix sums (four kernels), then the target
// kernel with its epilogue. ms: 2-D instances in ascending blk_base;
// chunk_tot: 128 B per chunk; mode: the DM_* epilogue (no DM_COUNT).
cudaError_t launch_moments2d_prefix(cudaStream_t st, const Mom2D* ms, uint32_t n_inst,
                                    uint32_t max_n, uint32_t max_strips, void* chunk_tot);
cudaError_t launch_moments2d_targets(cudaStream_t st, const Mom2D* ms, uint32_t n_inst,
                                     const uint32_t* blk_base, uint32_t n_blocks,
                                     const ILogEntry* ilog, double* tile_logsum, uint32_t mode);
// Mean in-support neighbours per target of 2-D instances, sampled: per
// instance 32 targets at quantiles of dimension 0, each with its window
// count in dimension 0 times the y-support fraction of up to 32 window points.
struct SupportEst {
  const uint32_t* keys0;  // dimension-0 sorted orderable keys of the instance
  const uint32_t* perm0;  // their original indices
  const float* y1;        // dimension-1 coordinates by original index
  uint32_t n;
  float h0, h1;
};
cudaError_t launch_support_est(cudaStream_t st, const SupportEst* in, uint32_t n_inst,
                               float* est);
uint32_t moments2d_block_targets();  // targets per block (= per tile slot)
cudaError_t launch_density_sym(cudaStream_t st, int d, int v, const TileDesc* tiles,
                               uint32_t n_slots, const InstDev* insts,
                               uint32_t* work_counter, uint32_t* err, int n_sms,
                               int* launched_ctas);
cudaError_t launch_sym_finish(cudaStream_t st, const TileDesc* tiles,
                              uint32_t n_slots, const InstDev* insts,
                              const double2* logtab, double* tile_logsum, uint32_t mode);
// a bounded mbarrier wait that runs out: sets EF_TIMEOUT in *err
cudaError_t launch_wait_test(cudaStream_t st, uint32_t* err);
// out[i] = log_fp64(x[i]) (device arrays; self-test of the epilogue log)
cudaError_t launch_log64_test(cudaStream_t st, const double* x, size_t n,
                              const double2* logtab, double* out);
cudaError_t launch_inst_logsum(cudaStream_t st, const InstDev* insts,
                               uint32_t n_inst, const double* tile_logsum,
                               double* inst_logsum);

}  // namespace ent
