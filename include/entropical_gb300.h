/*
 * entropical_gb300.h -- C ABI of the GB300 (sm_103a) density hot path of
 * lettis/entropical.
 *
 * Plain C: pointers, sizes and status codes only, so that the reference's
 * C++ host code (through entropical_gb300/shim/densities_gb300.hpp), ctypes,
 * or any FFI can bind it. Coordinates follow the reference's layout: a
 * column-major float32 buffer of n_rows x n_cols (column j at
 * coords[j*n_rows + i], tools.hxx:153-235).
 *
 * Every call is synchronous with respect to the host, as the reference's
 * combined_densities() is (densities_cuda.cu:46-105). A context is bound to
 * one CUDA device, owns one stream and a grow-only device workspace, and must
 * not be used by two host threads at once. Errors are returned as status
 * codes; the reference instead printed a message and called exit(), which
 * the C++ shim reproduces.
 */
#ifndef ENTROPICAL_GB300_H
#define ENTROPICAL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ent_ctx ent_ctx;

enum ent_status {
  ENT_OK = 0,
  ENT_ERR_DIM = 1,         /* d not in {1,2,3} (densities_common.hxx:15-19) */
  ENT_ERR_H_COUNT = 2,     /* bandwidth count != d (densities_common.hxx:20-25) */
  ENT_ERR_TAU_COUNT = 3,   /* lag count != d (densities_common.hxx:26-31) */
  ENT_ERR_ARG = 4,         /* null pointer, column index out of range,
                              lag >= n_rows, bandwidth not finite and > 0 */
  ENT_ERR_NONFINITE = 5,   /* NaN or Inf among the selected coordinates */
  ENT_ERR_CUDA = 6,        /* CUDA runtime error (tools.cuh:32-42) */
  ENT_ERR_NO_DEVICE = 7,   /* no CUDA device (density_1d.cuh:306-309) */
  ENT_ERR_TIMEOUT = 8,     /* a bounded device-side wait expired */
  ENT_ERR_TOO_LARGE = 9,   /* more rows than 32-bit point indices allow */
  ENT_ERR_STATE = 10,      /* call not valid in the current state */
  ENT_ERR_IO = 11          /* coordinate file unreadable or malformed */
};

/* flags for ent_densities* */
#define ENT_COMPAT_NORM 1u /* divide by the original n_rows, as the reference
                              CUDA build does even when lags shorten the
                              sample (densities_cuda.cu:98-103); default is
                              the selected sample size n_rows - max(tau) */

/* Statistics of the last call on a context. */
typedef struct {
  uint64_t candidate_pairs; /* (target, candidate source) pairs evaluated */
  uint64_t tiles;           /* target tiles processed */
  uint32_t kernel_launches; /* kernels this library launched for the call */
  uint32_t instances;       /* density instances computed */
  float pair_kernel_ms;     /* device time of the pair kernel(s) */
  float total_ms;           /* device time of the whole call */
  uint64_t candidate_pairs_by_dim[3]; /* same, split by density dimension */
  float pair_kernel_ms_by_dim[3];     /* device time of each persistent launch */
  float moment_target_ms; /* 2-D strip moments: device time of the target kernel
                             (k_m2_density), 0 when the call had none */
  float moment_edge_ms;   /* ... and of the symmetric pair kernel that sums
                             their edge strips (with any other 2-D pairs) */
} ent_call_stats;

/* Tile shapes of the pair kernel (0 = keep the current value). */
typedef struct {
  uint32_t targets_per_warp[3]; /* per density dimension: d=1,2: 8 or 16;
                                   d=3: 4 or 8 (tile = 4 warps) */
  uint32_t cells_per_h;         /* d=2 strips: cells per bandwidth, 1..4 */
  uint32_t pair_variant;        /* pair body + 1, for every dimension:
                                   1 = min-based (packed sub/fma, 2 min),
                                   2 = saturating FMA, 3 = saturating at 5
                                   CTAs/SM, 4 = as 3 with 1.5x larger chunks,
                                   5 = symmetric (each unordered pair once,
                                   added to both points; support counts use
                                   3 instead; own tiles of 128/128/64
                                   targets), 6 = as 5 with tiles of
                                   64/64/32 targets; default 5 for
                                   dimension 3 (get reports dimension 2) */
  uint32_t pair_variant_by_dim[3]; /* the same per dimension (0 = keep);
                                      applied after pair_variant; for
                                      dimension 1 also 7 = range sums (no
                                      pair loop: each target's support is
                                      one range of the value-sorted points,
                                      summed from exact fixed-point prefix
                                      sums), the default for d = 1; for
                                      dimension 2 also 8 = strip moments
                                      (strips of h/4 inside a target's
                                      support summed from exact moment
                                      prefix sums, pairs only on its edge;
                                      the symmetric body runs instead when
                                      the device lacks the 128 B per point).
                                      Default for d = 2: chosen per
                                      instance, the moments for supports of
                                      6,000+ neighbours per target (sampled
                                      estimate), else the symmetric body;
                                      setting 8 explicitly gives every 2-D
                                      instance to the moments */
  uint32_t cells_per_h3;        /* d=3 strips: cells per bandwidth along
                                   dimensions 1 and 2, 1..2 (default 1) */
  uint32_t moment_cells_per_h;  /* d=2 strip-moment body: strips per
                                   bandwidth, 2..12 (default 4) */
} ent_tuning;

/* Context lifecycle. device < 0 selects the current device. */
int ent_create(ent_ctx** ctx, int device);
void ent_destroy(ent_ctx* ctx);
const char* ent_status_string(int status);
/* Message of the last failing call on ctx (empty if none). */
const char* ent_last_error(const ent_ctx* ctx);
int ent_last_stats(const ent_ctx* ctx, ent_call_stats* stats);
int ent_set_tuning(ent_ctx* ctx, const ent_tuning* tuning);
/* Diagnostic: out[i] = the FP64 natural log the per-point epilogues use
 * (a table-reduction log with few FP64 operations), on the device, for n
 * host values. No counterpart in the reference. */
int ent_log64_selftest(ent_ctx* ctx, const double* x, size_t n, double* out);
/*
 * Self-test of the log the strip-moment epilogue takes of a density's exact
 * 128-bit integer sum T (in 64-bit fixed point, FP32 arithmetic only): t holds
 * n values as (low, high) 64-bit word pairs; out[i] = log(T_i) 2^48 within
 * 8 (2^-45 absolute). No counterpart in the reference.
 */
int ent_ilog_selftest(ent_ctx* ctx, const uint64_t* t, size_t n, int64_t* out);
/* Diagnostic of the failure path: one device-side wait that nothing
 * completes runs into its bound (2 s) and the call returns ENT_ERR_TIMEOUT;
 * the context stays usable. No counterpart in the reference. */
int ent_wait_selftest(ent_ctx* ctx);
int ent_get_tuning(const ent_ctx* ctx, ent_tuning* tuning);

/*
 * Combined product-Epanechnikov densities of d = 1..3 selected, lagged
 * columns. Replaces
 *   std::vector<double> combined_densities(const float* coords,
 *       std::size_t n_rows, std::vector<unsigned> i_cols,
 *       std::vector<float> h, std::vector<unsigned> tau)
 * (densities_cuda.hpp:9-24, densities_cuda.cu:16-105; OpenMP form
 * densities_omp.cpp:163-233). tau may be NULL (all zero). Point i of the
 * result is the density at (x_{i_cols[0]}[i+tau[0]], ...), i < n_sel =
 * n_rows - max(tau):
 *   out[i] = 1/norm * sum_k prod_j 0.75 (1 - u_j^2)/h_j [u_j^2 <= 1],
 *   u_j = (x_j[i] - x_j[k]) / h_j,
 * norm = n_sel, or n_rows with ENT_COMPAT_NORM. *n_out receives n_sel.
 * coords, out: host memory (copies are part of the call).
 */
int ent_densities(ent_ctx* ctx, const float* coords, size_t n_rows,
                  size_t n_cols, const uint32_t* i_cols, const float* h,
                  const uint32_t* tau, uint32_t d, uint32_t flags, double* out,
                  size_t* n_out);
/* Same with coords and out in device memory of the context's device. */
int ent_densities_device(ent_ctx* ctx, const float* d_coords, size_t n_rows,
                         size_t n_cols, const uint32_t* i_cols, const float* h,
                         const uint32_t* tau, uint32_t d, uint32_t flags,
                         double* d_out, size_t* n_out);
/*
 * One share of one density's targets, for splitting a single large density
 * over GPUs as the reference's per-GPU driver splits its target rows
 * (density_1d.cuh:181-219, host reduction :94-104): of the n_sel targets,
 * in the library's sorted order, this call computes those at positions
 * [n_sel part / n_parts, n_sel (part + 1) / n_parts) against every source and
 * writes their densities to d_out (device, n_sel doubles, indexed by
 * original point); the other entries of d_out are left untouched, so shares
 * computed into zeroed buffers add up to the whole. logsum_out (nullable, on
 * the host) receives the sum of log p over the share's targets. Each share
 * runs the ordered pair kernel (every target summed fully in its own tile).
 * Same arguments and normalisation as ent_densities_device otherwise.
 */
int ent_densities_part_device(ent_ctx* ctx, const float* d_coords, size_t n_rows,
                              size_t n_cols, const uint32_t* i_cols, const float* h,
                              const uint32_t* tau, uint32_t d, uint32_t flags, uint32_t part,
                              uint32_t n_parts, double* d_out, size_t* n_out,
                              double* logsum_out);

/*
 * Number of (target, source) pairs inside the kernel support for the same
 * selection: out[i] = #{k : u_j^2 <= 1 for all j}. Used to report
 * pair-kernel evaluation rates; host memory.
 */
int ent_support_counts(ent_ctx* ctx, const float* coords, size_t n_rows,
                       size_t n_cols, const uint32_t* i_cols, const float* h,
                       const uint32_t* tau, uint32_t d, double* out,
                       size_t* n_out);

/* ------------------------------------------------------------ batches */

/*
 * A batched job runs as one batch (one persistent pair-kernel launch per
 * dimension over all its densities) when it fits one: at most 65535
 * densities and its workspace within the device's free memory. A larger job
 * runs as consecutive batches of as many densities as fit, with the same
 * results. ENT_MAX_BATCH_INSTANCES (1..65535) in the environment when a
 * context is created lowers the densities per batch of that context.
 */

/* flags for the batched entry points */
#define ENT_BATCH_SUPPORT_COUNTS 2u /* return in-support pair counts instead
                                       of entropies (pair-rate reporting) */
#define ENT_BATCH_DEVICE_INPUT 4u   /* ent_entropy_batch: coords are device
                                       pointers */

/*
 * All-pairs mutual information of n_cols coordinates in ONE batch: n_cols
 * 1-D marginal densities and n_cols(n_cols-1)/2 2-D joint densities, with
 * bandwidth h[j] for column j in every density it appears in (as
 * mi.cpp:38-52 reuses them). Replaces the per-pair combined_densities() loop
 * of Mi::main (mi.cpp:37-59). Resubstitution estimator in FP64:
 *   H_j = -1/n sum_i log p_j(x_i),  MI_ij = H_i + H_j - H_ij,
 * densities normalised by n_rows. mi_out: n_cols x n_cols row-major, zero
 * diagonal (as mi.cpp leaves it); h_out (nullable): the n_cols marginal
 * entropies. With ENT_BATCH_SUPPORT_COUNTS, mi_out[i][j] / h_out[i] instead
 * receive the number of in-support (target, source) pairs of each density.
 * coords: host memory, column-major n_rows x n_cols.
 */
int ent_mi_all_pairs(ent_ctx* ctx, const float* coords, size_t n_rows,
                     size_t n_cols, const float* h, uint32_t flags,
                     double* mi_out, double* h_out);
/* Same with coords in device memory (outputs stay on the host). */
int ent_mi_all_pairs_device(ent_ctx* ctx, const float* d_coords, size_t n_rows,
                            size_t n_cols, const float* h, uint32_t flags,
                            double* mi_out, double* h_out);

/*
 * All-ordered-pairs transfer entropy at every lag in taus, in ONE batch:
 *   TE_{j->i}(tau) = mean_t log[ p(y+, y, x) p(y) / (p(y, x) p(y+, y)) ]
 *                  = H(y,x) + H(y+,y) - H(y+,y,x) - H(y),
 * y = x_i[t], y+ = x_i[t+tau], x = x_j[t], t < n_rows - tau, bandwidth h[c]
 * for column c in every density (as transs.cpp:56-74 reuses them).
 * te_out: n_taus x n_cols x n_cols, te_out[q][i][j] = TE_{j->i}(taus[q]),
 * the reference's transs[i*n+j] layout (transs.cpp:75-113), zero diagonal.
 * Replaces the per-pair density loop of Transs::main (transs.cpp:39-115);
 * its own sum of p * h^3 * log(...) terms is the reference's formula, this
 * is the resubstitution estimator. With ENT_BATCH_SUPPORT_COUNTS, te_out
 * receives the in-support pair counts of the 3-D densities (diagonal: of
 * the 1-D ones). coords: host memory, column-major n_rows x n_cols.
 */
int ent_te_all_pairs(ent_ctx* ctx, const float* coords, size_t n_rows,
                     size_t n_cols, const float* h, const uint32_t* taus,
                     size_t n_taus, uint32_t flags, double* te_out);
/* Same with coords in device memory (te_out on the host). */
int ent_te_all_pairs_device(ent_ctx* ctx, const float* d_coords, size_t n_rows,
                            size_t n_cols, const float* h, const uint32_t* taus,
                            size_t n_taus, uint32_t flags, double* te_out);

/*
 * Entropies of a listed subset of the densities of the batches above, from
 * device coordinates: the unit one rank computes when one MI or TE job is
 * split over GPUs (the reference splits one density's target rows over its
 * GPUs instead, density_1d.cuh:181-219; here whole densities are dealt out
 * and each rank uploads the coordinate matrix once). items[q] is an index
 * into the batch order -- for MI: 0..n_cols-1 the 1-D marginals, then the
 * joints (i, j), i < j, in row order; for TE, per lag q in taus order:
 * [n_cols 1-D y][n_cols 2-D (y+, y)][n_cols(n_cols-1)/2 2-D (y_i, x_j), i < j]
 * [n_cols(n_cols-1) 3-D (y_i+, y_i, x_j), i != j, row order]. H_out[q]
 * receives -mean log p of item q (with ENT_BATCH_SUPPORT_COUNTS, its
 * in-support pair count). The listed densities run as one batch, and only
 * the coordinate views they use are sorted. Outputs on the host.
 */
int ent_mi_entropies_device(ent_ctx* ctx, const float* d_coords, size_t n_rows, size_t n_cols,
                            const float* h, const uint64_t* items, size_t n_items,
                            uint32_t flags, double* H_out);
int ent_te_entropies_device(ent_ctx* ctx, const float* d_coords, size_t n_rows, size_t n_cols,
                            const float* h, const uint32_t* taus, size_t n_taus,
                            const uint64_t* items, size_t n_items, uint32_t flags,
                            double* H_out);

/* One density instance of an uneven batch. */
typedef struct {
  const float* coords; /* column-major d x n: dimension j at coords[j*n + i] */
  uint64_t n;
  uint32_t d;          /* 1..3 */
  float h[3];
} ent_instance;

/*
 * Resubstitution entropies -mean(log p) of many independent instances of
 * uneven size and dimension, in ONE batch (one persistent launch per
 * dimension). Replaces sequential combined_densities() calls followed by
 * host reductions. h_out: n_inst values.
 */
int ent_entropy_batch(ent_ctx* ctx, const ent_instance* inst, size_t n_inst,
                      uint32_t flags, double* h_out);

/* ------------------------------------------------------------ autotuner */

#define ENT_TUNE_FORCE 1u /* re-time even if the cache holds the bucket */

/*
 * Autotuner of the pair kernel's tile shapes. Times every candidate pair
 * body and cell size for density dimension d (1..3) on the sample batch
 * (ent_entropy_batch with ENT_BATCH_DEVICE_INPUT in flags if the sample is
 * in device memory; device time of that dimension's pair kernel, best of 2)
 * and applies the fastest to the context, as ent_set_tuning would. The
 * choice is kept in the context's cache under (d, floor(log2 of the largest
 * sample instance of dimension d)); a later call for the same key applies the
 * cached choice without timing (unless ENT_TUNE_FORCE). chosen (nullable)
 * receives the context's tuning afterwards. The sample must contain an
 * instance of dimension d. No counterpart in the reference.
 */
int ent_autotune(ent_ctx* ctx, const ent_instance* sample, size_t n_sample,
                 uint32_t d, uint32_t flags, ent_tuning* chosen);
/* Number of entries in the context's autotune cache. */
size_t ent_autotune_cache_size(const ent_ctx* ctx);

/* ------------------------------------------------------ coordinate files */

/*
 * The reference's ASCII coordinate format (Tools::IO::read_coords,
 * tools.hxx:153-235): whitespace-separated values, one row per non-empty
 * line, n_cols = number of values on the first non-empty line. Read once and
 * parsed by all host threads (correctly rounded, as `ifs >> float`). A row
 * with another number of values, or a token that is not a number, is
 * ENT_ERR_IO (the reference reads across line ends instead). usecols
 * (nullable, n_usecols = 0: all columns) keep the file's column order, as the
 * reference does; an index >= n_cols is ENT_ERR_ARG.
 */
int ent_coords_file_shape(const char* path, size_t* n_rows, size_t* n_cols);
/* primary_index 'C': out[c * n_rows + r] (the reference's column-major
 * layout); 'R': out[r * n_cols_out + c]. n_rows / n_cols_out must match the
 * file and the selection. */
int ent_read_coords(const char* path, const size_t* usecols, size_t n_usecols,
                    char primary_index, float* out, size_t n_rows, size_t n_cols_out);
/* Same, column-major into device memory d_out of ctx's device: blocks of rows
 * are parsed into pinned buffers and copied with one 2-D copy per block while
 * the next block is parsed. */
int ent_load_coords_device(ent_ctx* ctx, const char* path, const size_t* usecols,
                           size_t n_usecols, float* d_out, size_t n_rows,
                           size_t n_cols_out);
/* Message of the last failing file call of this thread (empty if none). */
const char* ent_io_last_error(void);

/*
 * XTC trajectories, the format CoordsFile::open picks for names ending in
 * ".xtc" (coords_file/coords_file.cpp:137-145; XtcHandler :70-126, the
 * reference's vendored xdrfile codec). A frame is one row of 3 * natoms
 * values (x0, y0, z0, x1, ...), as XtcHandler::next returns it; reading stops
 * at the first frame that does not parse, as XtcHandler::next does.
 */
/* Frames and columns (3 natoms) of an XTC file (host only). */
int ent_xtc_file_shape(const char* path, size_t* n_frames, size_t* n_cols);
/* Decode the file on the device into the column-major n_rows x n_cols_out
 * matrix d_out (device memory of ctx's device): the file is indexed on the
 * host, copied to the device through pinned buffers, walked once per frame
 * (atom-group positions) and decoded by one thread per 64-atom segment.
 * usecols as for ent_read_coords (the file's column order). A malformed
 * compressed frame is ENT_ERR_IO naming the frame. */
int ent_load_xtc_device(ent_ctx* ctx, const char* path, const size_t* usecols,
                        size_t n_usecols, float* d_out, size_t n_rows, size_t n_cols_out);
/* Same into host memory: primary_index 'C' column-major, 'R' row-major (the
 * rows XtcHandler::next returns, one after another). */
int ent_read_xtc(ent_ctx* ctx, const char* path, const size_t* usecols, size_t n_usecols,
                 char primary_index, float* out, size_t n_rows, size_t n_cols_out);
/* Write n_rows frames of n_cols = 3 natoms columns (host memory, 'C' or 'R'
 * layout) as XtcHandler::write does (coords_file.cpp:112-126): frame r has
 * step r, time r, a zero box and the given precision (<= 0: 1000, the
 * handler's). The bytes equal the reference's writer's. Host only; frames are
 * encoded by all host threads. Coordinates that overflow 32-bit integers at
 * the precision, or atoms too far apart for the format's table, are
 * ENT_ERR_ARG (the reference writes a frame it cannot read back). */
int ent_write_xtc(const char* path, const float* coords, size_t n_rows, size_t n_cols,
                  char primary_index, float precision);
/* Message of the last failing host-only XTC call of this thread. */
const char* ent_xtc_last_error(void);

/* ------------------------------------ the reference's estimator formulas */

#define ENT_BATCH_DEVICE_OUTPUT 8u /* ent_dens_all: out is a device pointer */

#define ENT_REF_MI 1u      /* Mi::main, mi.cpp:37-59 */
#define ENT_REF_TRANSS 2u  /* Transs::main, transs.cpp:39-115 */
#define ENT_REF_AUTOENT 3u /* AutoEnt::main, autoent.cpp:39-58 */
#define ENT_REF_NEGS 4u    /* Negs::main, negs.cpp:36-47 */
#define ENT_REF_KLDIV 5u   /* KLDiv::main, kldiv.cpp:36-54 */

/*
 * One of the reference's estimators over all columns, with the reference's
 * own formula (not the resubstitution estimators above), as ONE batch: every
 * density it needs is an instance of one engine batch (marginals once), the
 * per-point densities stay in device memory and the sums run on the device in
 * FP64. Densities are normalised by n_rows as the reference's CUDA build does
 * (densities_cuda.cu:98-103); logs are the reference's float log, 0 at 0
 * (tools.cpp:18-37). Replaces the estimator main loops and their per-density
 * combined_densities() calls. out (host):
 *   ENT_REF_MI      n_cols x n_cols, out[i][j] = sum_k p_ij log(p_ij/p_i/p_j),
 *                   symmetric, zero diagonal
 *   ENT_REF_TRANSS  n_cols x n_cols, lag tau: out[i][j] (i < j) the
 *                   p(x_i, x_i+tau, x_j) term with weight h_i h_i h_j, out[j][i]
 *                   the p(x_i, x_j, x_j+tau) term with weight h_i h_j h_i, as
 *                   transs.cpp:75-104 (non-finite terms and p > 1 skipped)
 *   ENT_REF_AUTOENT n_cols, lag tau
 *   ENT_REF_NEGS    n_cols, -sum_k p~ log p~ with p~ = p / sum(p)
 *   ENT_REF_KLDIV   n_cols x n_cols, out[i][j] = sum_k p~_i log(p~_i / p~_j)
 * flags: ENT_BATCH_DEVICE_INPUT for device coordinates. No counterpart of
 * this batched form exists in the reference (its mains loop on the host).
 */
int ent_reference_estimator(ent_ctx* ctx, const float* coords, size_t n_rows,
                            size_t n_cols, const float* h, uint32_t estimator,
                            uint32_t tau, uint32_t flags, double* out);

/*
 * Dens::compute_densities_1d / _nd (dens.cpp:19-106) as ONE batch: the
 * sum-normalised densities of every column (dims = 1), every column pair
 * (dims = 2) or triple (dims = 3, the "dens -D 3" mode) in the reference's
 * order (i < j < k), each over lags taus[0..dims) (NULL: none; ignored for
 * dims = 1). out: *n_inst rows of *n_sel = n_rows - max(taus) values, host
 * memory, or device memory with ENT_BATCH_DEVICE_OUTPUT. Every density of
 * the call is held in device memory (*n_inst x *n_sel doubles).
 */
int ent_dens_all(ent_ctx* ctx, const float* coords, size_t n_rows, size_t n_cols,
                 const float* h, uint32_t dims, const uint32_t* taus,
                 uint32_t flags, double* out, size_t* n_inst, size_t* n_sel);

/* ---------------------------------------------------- neighbour search */

#define ENT_NB_WINDOW 0u /* reference boxes() windows (densities_omp.cpp:33-65) */
#define ENT_NB_BOXED 1u  /* Transs::BoxedSearch::Boxes (boxedsearch.cpp:15-62) */

/*
 * Neighbour search of one column of n values (host memory), bit-exact with
 * the reference's float arithmetic.
 * ENT_NB_WINDOW, width h: out_a[i] = first, out_b[i] = last index of the
 *   value-sorted column whose distance to x_i is below h (strict), i.e. the
 *   source range the reference density loop visits for point i.
 * ENT_NB_BOXED, box size h: out_a[i] = box of point i, out_b[i] = size of its
 *   neighbour list (own and adjacent boxes); *n_boxes = number of boxes.
 *   The reference's undefined cases are defined: the maximum is the true
 *   maximum, a box index equal to the box count joins the last box, and a
 *   zero-width range has one box.
 */
int ent_neighbor_counts(ent_ctx* ctx, const float* col, size_t n, float h,
                        uint32_t mode, uint64_t* out_a, uint64_t* out_b,
                        uint64_t* n_boxes);

/* ---------------------------------------------- bandwidth estimation */

/*
 * Convolution of the Epanechnikov kernel with itself over all pairs,
 *   out = 1/n^2 sum_i sum_j max(0, 4.5 - 2.25 |x_i - x_j| / h),
 * the AMISE helper of the reference. Replaces
 *   float epa_convolution(const std::vector<float>& sorted_coords, float h)
 * (densities_cuda.hpp:26-31; OpenMP form densities_omp.cpp:235-277).
 * Input need not be sorted. Host memory.
 */
int ent_epa_convolution(ent_ctx* ctx, const float* sorted_coords, size_t n,
                        float h, float* out);

/* modes of ent_hestimate */
#define ENT_HEST_THUMB 0u      /* h0 = n^(-1/7) sqrt(var) (hestimate.cpp:19-30) */
#define ENT_HEST_AMISE 1u      /* AMISE interval search (hestimate.cpp:41-104) */
#define ENT_HEST_AMISE_WARM 2u /* the same search entered skip_levels levels
                                  deep, at the bracket node containing h_init,
                                  with a full search for columns whose warm
                                  search ends against an inner node edge */

typedef struct {
  float h0;                /* rule-of-thumb start value */
  uint32_t conv_evals;     /* convolution evaluations spent */
  uint32_t levels_skipped; /* warm start: levels taken from h_init */
  uint32_t warm_converged; /* warm start: 1 if no full search was needed */
} ent_hest_stats;

/*
 * Per-column bandwidths of the selected columns cols[0..n_sel) (all columns
 * if cols is NULL), every column searched at once on the device (in passes
 * of at most 65535 columns, and of what the device's free memory holds,
 * when there are more; each column's result is independent of the others').
 * Replaces Hestimate::main<KRNL> (hestimate.hxx:6-26) with Thumb::Kernel or
 * AmiseMin::Kernel. h_init (warm mode): one start value per selected column.
 * stats (nullable): one entry per selected column. Host memory.
 */
int ent_hestimate(ent_ctx* ctx, const float* coords, size_t n_rows,
                  size_t n_cols, const uint32_t* cols, size_t n_sel,
                  uint32_t mode, const float* h_init, uint32_t skip_levels,
                  float* h_out, ent_hest_stats* stats);
/* Same with coords in device memory (h_init, h_out, stats on the host). */
int ent_hestimate_device(ent_ctx* ctx, const float* d_coords, size_t n_rows,
                         size_t n_cols, const uint32_t* cols, size_t n_sel,
                         uint32_t mode, const float* h_init,
                         uint32_t skip_levels, float* h_out,
                         ent_hest_stats* stats);

/*
 * Full AMISE search (ENT_HEST_AMISE) for every dimension of uneven
 * instances in one batch; h_out, stats: n_inst x 3 (slots beyond d zero).
 * flags: ENT_BATCH_DEVICE_INPUT for device coordinates.
 */
int ent_hestimate_batch(ent_ctx* ctx, const ent_instance* inst, size_t n_inst,
                        uint32_t flags, float* h_out, ent_hest_stats* stats);

/* ------------------------------------------- allocation-free density */

/* Largest input of ent_density_1d_noalloc. */
#define ENT_NOALLOC_MAX_N 65536u

/*
 * The 1-D density of ent_densities_device (one column, no lag, divided by
 * n) for callers that cannot allocate device memory -- for instance when
 * another framework owns the device memory pool, or in a service that must
 * not allocate after start-up. No counterpart in the reference, which
 * allocated and freed device memory on every call (density_1d.cuh:108-164).
 * All working memory is one fixed 2 MiB device array inside this library
 * (held on every device that loads it until the process exits), so n must
 * not exceed ENT_NOALLOC_MAX_N (ENT_ERR_TOO_LARGE otherwise). d_x (n floats)
 * and d_out (n doubles) are device memory of the current device; stream may
 * be NULL. The call is synchronous (it waits for its work on the stream
 * before returning) and calls no allocator. The first call on a device looks
 * up the array's device address; with CUDA's lazy module loading it also
 * loads this library's device code and the array, so a caller that must not
 * allocate after start-up makes one warm-up call then. Calls share the array: calls that overlap on the GPU
 * race and must be serialised by the caller.
 */
int ent_density_1d_noalloc(const float* d_x, size_t n, float h, double* d_out,
                           void* stream);

/* --------------------------------------- learned bandwidth warm start */

/*
 * A small MLP (32 -> 128 -> 128 -> 3, ReLU; 21,123 parameters) trained and
 * run by this library's own kernels: BF16 weights in the passes, FP32
 * accumulation, FP32 master weights and Adam moments on the device. It maps
 * 32 summary features of an instance (ent_features) to r_j =
 * log(h_j / h0_j) per dimension j, the AMISE bandwidth relative to the rule
 * of thumb, which warm-starts the AMISE search. No counterpart in the
 * reference beyond the search it shortens (hestimate.cpp:55-104).
 */
typedef struct ent_mlp ent_mlp;

size_t ent_mlp_param_count(void);
int ent_mlp_create(ent_ctx* ctx, uint64_t seed, ent_mlp** net);
void ent_mlp_destroy(ent_mlp* net);
/* Flat FP32 parameters [W1 128x32, b1, W2 128x128, b2, W3 3x128, b3] and
 * the feature normalisation (32 means, 32 scales); any pointer may be NULL. */
int ent_mlp_set_params(ent_mlp* net, const float* params, const float* feat_mu,
                       const float* feat_sd);
int ent_mlp_get_params(const ent_mlp* net, float* params, float* feat_mu,
                       float* feat_sd);
/* Y[B x 3] for raw (unnormalised) features X[B x 32]; host memory. */
int ent_mlp_forward(ent_ctx* ctx, ent_mlp* net, const float* X, size_t B,
                    float* Y);
/* Gradient of the masked mean-squared error sum(mask (Y - T)^2) / sum(mask)
 * with respect to the flat parameters (no update); host memory. */
int ent_mlp_gradients(ent_ctx* ctx, ent_mlp* net, const float* X,
                      const float* T, const float* mask, size_t B,
                      float* grads, float* loss);
/* One Adam step (beta 0.9 / 0.999) on a batch; *loss before the step. */
int ent_mlp_train_step(ent_ctx* ctx, ent_mlp* net, const float* X,
                       const float* T, const float* mask, size_t B, float lr,
                       float* loss);
/* The 32 features of every instance (feat: n_inst x 32); host memory. */
int ent_features(ent_ctx* ctx, const ent_instance* inst, size_t n_inst,
                 float* feat);
/*
 * Per-dimension AMISE bandwidths of every instance dimension, each search
 * entered skip_levels levels deep at the node of h0 * exp(r) predicted by
 * the network (features, network and search all on the device), falling
 * back to the full search where the warm search ends against an inner node
 * edge. h_out, stats: n_inst x 3 (slots beyond d are zero).
 * flags: ENT_BATCH_DEVICE_INPUT for device coordinates.
 */
int ent_hestimate_learned(ent_ctx* ctx, ent_mlp* net, const ent_instance* inst,
                          size_t n_inst, uint32_t flags, uint32_t skip_levels,
                          float* h_out, ent_hest_stats* stats);

#ifdef __cplusplus
}
#endif
#endif /* ENTROPICAL_GB300_H */
