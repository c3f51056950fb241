// Batched estimators: all-pairs mutual information and uneven entropy
// batches, each run as ONE engine batch, i.e. one persistent pair-kernel
// launch per dimension over every (instance, tile) work item (a job larger
// than one batch holds runs as several).
//
// Replaces the per-call loops of the reference estimators: Mi::main
// (mi.cpp:37-59) computes 1-D marginals inside its pair loop (M^2 1-D
// densities) and one 2-D density per pair, each a separate
// combined_densities() call with its own device allocation and copies.
// Here the M marginals and the M(M-1)/2 joints share one upload, one
// per-column sort and one launch, and the reductions stay on the device.
//
// Estimator (resubstitution, FP64): H = -mean_i log p(x_i),
// MI(X;Y) = H(X) + H(Y) - H(X,Y).
#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/entropical_gb300.h"
#include "api_internal.h"
#include "engine.h"

using namespace ent;

namespace {

struct EntropyRun {
  Ctx* c;
  const std::vector<InstSpec>* insts;
  bool counts;
  std::vector<double>* H;
};

// The log-sums (or counts) of one engine run, by instance.
int entropy_run_done(void* arg, size_t first, size_t count, const EngineOut& eo) {
  EntropyRun& r = *static_cast<EntropyRun*>(arg);
  Ctx& c = *r.c;
  std::vector<double> ls(count);
  cudaError_t e = cudaMemcpyAsync(ls.data(), eo.d_logsum_sorted, sizeof(double) * count,
                                  cudaMemcpyDeviceToHost, c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "read log-sums");
  e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "batch");
  for (size_t k = 0; k < count; ++k) {
    const size_t i = first + eo.slot_order[k];
    (*r.H)[i] = r.counts ? ls[k] : -ls[k] / (double)(*r.insts)[i].n;
  }
  return ENT_OK;
}

// Runs the engine in log-sum (or support-count) mode and returns, per
// instance, -mean(log p) (or the in-support pair count); as one batch, or as
// several for a job larger than one batch holds.
int run_entropies(Ctx& c, const std::vector<ViewSpec>& views,
                  std::vector<InstSpec>& insts, bool counts,
                  std::vector<double>* H) {
  const uint32_t mode = counts ? (DM_COUNT | DM_SUMV) : DM_LOGSUM;
  if (counts)
    for (auto& s : insts) s.norm = 1.0;
  H->assign(insts.size(), 0.0);
  EntropyRun r{&c, &insts, counts, H};
  return run_engine_batches(c, views, insts, mode, entropy_run_done, &r);
}

// The densities of an all-pairs MI in batch order: the n_cols 1-D
// marginals, then the joints (i, j), i < j, in row order.
void mi_build(const Ctx& c, const float* dc, size_t n_rows, size_t n_cols, const float* h,
              std::vector<ViewSpec>* views, std::vector<InstSpec>* insts) {
  views->resize(n_cols);
  for (size_t j = 0; j < n_cols; ++j) (*views)[j] = {dc + j * n_rows, (uint32_t)n_rows};
  insts->reserve(n_cols + n_cols * (n_cols - 1) / 2);
  for (size_t i = 0; i < n_cols; ++i) {
    InstSpec I;
    I.d = 1;
    I.n = (uint32_t)n_rows;
    I.view[0] = (uint32_t)i;
    I.h[0] = h[i];
    I.norm = (double)n_rows;
    I.S = c.strip_subdiv;
    insts->push_back(I);
  }
  for (size_t i = 0; i < n_cols; ++i)
    for (size_t j = i + 1; j < n_cols; ++j) {
      InstSpec I;
      I.d = 2;
      I.n = (uint32_t)n_rows;
      I.view[0] = (uint32_t)i;
      I.view[1] = (uint32_t)j;
      I.h[0] = h[i];
      I.h[1] = h[j];
      I.norm = (double)n_rows;
      I.S = c.strip_subdiv;
      insts->push_back(I);
    }
}

// The densities of an all-ordered-pairs TE over the lags in batch order:
// per lag [M 1-D y][M 2-D (y+, y)][M(M-1)/2 2-D (y_i, x_j), i < j]
// [M(M-1) 3-D (y+, y, x)].
void te_build(const Ctx& c, const float* dc, size_t n_rows, size_t M, const float* h,
              const uint32_t* taus, size_t n_taus, std::vector<ViewSpec>* views,
              std::vector<InstSpec>* insts) {
  const size_t per_tau = M + M + M * (M - 1) / 2 + M * (M - 1);
  insts->reserve(per_tau * n_taus);
  for (size_t q = 0; q < n_taus; ++q) {
    const uint32_t tau = taus[q];
    const uint32_t n = (uint32_t)(n_rows - tau);
    const uint32_t v0 = (uint32_t)views->size();
    for (size_t j = 0; j < M; ++j) views->push_back({dc + j * n_rows, n});        // x_j[t]
    for (size_t j = 0; j < M; ++j) views->push_back({dc + j * n_rows + tau, n});  // x_j[t+tau]
    auto mk = [&](uint32_t d, uint32_t a, uint32_t b, uint32_t cc, float ha, float hb,
                  float hc) {
      InstSpec I;
      I.d = d;
      I.n = n;
      I.view[0] = a;
      I.view[1] = b;
      I.view[2] = cc;
      I.h[0] = ha;
      I.h[1] = hb;
      I.h[2] = hc;
      I.norm = (double)n;
      I.S = c.strip_subdiv;
      insts->push_back(I);
    };
    for (size_t i = 0; i < M; ++i) mk(1, v0 + i, 0, 0, h[i], 1.f, 1.f);
    for (size_t i = 0; i < M; ++i) mk(2, v0 + M + i, v0 + i, 0, h[i], h[i], 1.f);
    for (size_t i = 0; i < M; ++i)
      for (size_t j = i + 1; j < M; ++j) mk(2, v0 + i, v0 + j, 0, h[i], h[j], 1.f);
    for (size_t i = 0; i < M; ++i)
      for (size_t j = 0; j < M; ++j)
        if (i != j) {
          // (x, y+, y): x sorted, cells of h in y+ and h/2 in y (3 x 5
          // strips). The same density as (y+, y, x), with y+ sorted and
          // cells in y and x, and the same candidates, but the 3-D kernel
          // on the 32 x 200k, 3-lag batch takes 740 ms against 770 ms (and
          // 751 ms with cells of h in both, 780 ms with h/2 in both).
          mk(3, v0 + j, v0 + M + i, v0 + i, h[j], h[i], h[i]);
          insts->back().S3[0] = 1;
          insts->back().S3[1] = 2;
        }
  }
}

// Keeps the listed instances (in the listed order) and the views they use.
int select_items(Ctx& c, const uint64_t* items, size_t n_items, std::vector<ViewSpec>* views,
                 std::vector<InstSpec>* insts) {
  std::vector<InstSpec> sel;
  sel.reserve(n_items);
  std::vector<uint32_t> remap(views->size(), UINT32_MAX);
  std::vector<ViewSpec> used;
  for (size_t q = 0; q < n_items; ++q) {
    if (items[q] >= insts->size()) return c.fail(ENT_ERR_ARG, "item index out of range");
    InstSpec I = (*insts)[items[q]];
    for (uint32_t j = 0; j < I.d; ++j) {
      uint32_t& r = remap[I.view[j]];
      if (r == UINT32_MAX) {
        r = (uint32_t)used.size();
        used.push_back((*views)[I.view[j]]);
      }
      I.view[j] = r;
    }
    sel.push_back(I);
  }
  *views = std::move(used);
  *insts = std::move(sel);
  return ENT_OK;
}

int mi_impl(ent_ctx* ctx, const float* coords, size_t n_rows, size_t n_cols,
            const float* h, uint32_t flags, double* mi_out, double* hx_out,
            bool device_in) {
  if (!ctx) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  if (!coords || !h || !mi_out) return c.fail(ENT_ERR_ARG, "null argument");
  if (n_cols < 1 || n_rows < 1) return c.fail(ENT_ERR_ARG, "empty input");
  if (n_rows > 0xffffff00ull) return c.fail(ENT_ERR_TOO_LARGE, "too many rows");
  for (size_t j = 0; j < n_cols; ++j)
    if (!(h[j] > 0.f) || !std::isfinite(h[j]))
      return c.fail(ENT_ERR_ARG, "bandwidth must be finite and positive");
  const float* dc = coords;
  if (!device_in) {
    float* p = static_cast<float*>(c.arena.alloc(4 * n_rows * n_cols));
    if (!p) return c.fail(ENT_ERR_CUDA, "out of device memory");
    cudaError_t e = cudaMemcpyAsync(p, coords, 4 * n_rows * n_cols,
                                    cudaMemcpyHostToDevice, c.stream);
    if (e != cudaSuccess) return c.cuda_fail(e, "copy coordinates");
    dc = p;
  }
  std::vector<ViewSpec> views;
  std::vector<InstSpec> insts;
  mi_build(c, dc, n_rows, n_cols, h, &views, &insts);
  std::vector<double> H;
  const bool counts = (flags & ENT_BATCH_SUPPORT_COUNTS) != 0;
  s = run_entropies(c, views, insts, counts, &H);
  if (s) return s;
  s = c.end_call();
  c.collect_kernel_stats();
  if (s) return s;
  size_t k = n_cols;
  for (size_t i = 0; i < n_cols; ++i) {
    if (hx_out) hx_out[i] = H[i];
    mi_out[i * n_cols + i] = counts ? H[i] : 0.0;
  }
  for (size_t i = 0; i < n_cols; ++i)
    for (size_t j = i + 1; j < n_cols; ++j, ++k) {
      const double v = counts ? H[k] : H[i] + H[j] - H[k];
      mi_out[i * n_cols + j] = v;
      mi_out[j * n_cols + i] = v;
    }
  return ENT_OK;
}

// TE_{j->i}(tau) = H(y_i, x_j) + H(y_i^+, y_i) - H(y_i^+, y_i, x_j) - H(y_i)
// over the n = N - tau samples t (y_i = x_i[t], y_i^+ = x_i[t + tau],
// x_j = x_j[t]); one batch over every lag and ordered pair.
int te_impl(ent_ctx* ctx, const float* coords, size_t n_rows, size_t n_cols, const float* h,
            const uint32_t* taus, size_t n_taus, uint32_t flags, double* te_out,
            bool device_in) {
  if (!ctx) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  if (!coords || !h || !taus || !te_out || n_taus == 0)
    return c.fail(ENT_ERR_ARG, "null argument");
  if (n_cols < 1) return c.fail(ENT_ERR_ARG, "empty input");
  if (n_rows > 0xffffff00ull) return c.fail(ENT_ERR_TOO_LARGE, "too many rows");
  for (size_t q = 0; q < n_taus; ++q)
    if (taus[q] == 0 || taus[q] >= n_rows) return c.fail(ENT_ERR_ARG, "lag out of range");
  for (size_t j = 0; j < n_cols; ++j)
    if (!(h[j] > 0.f) || !std::isfinite(h[j]))
      return c.fail(ENT_ERR_ARG, "bandwidth must be finite and positive");
  const float* dc = coords;
  if (!device_in) {
    float* p = static_cast<float*>(c.arena.alloc(4 * n_rows * n_cols));
    if (!p) return c.fail(ENT_ERR_CUDA, "out of device memory");
    cudaError_t e = cudaMemcpyAsync(p, coords, 4 * n_rows * n_cols, cudaMemcpyHostToDevice,
                                    c.stream);
    if (e != cudaSuccess) return c.cuda_fail(e, "copy coordinates");
    dc = p;
  }
  const size_t M = n_cols;
  const size_t per_tau = M + M + M * (M - 1) / 2 + M * (M - 1);
  std::vector<ViewSpec> views;
  std::vector<InstSpec> insts;
  te_build(c, dc, n_rows, M, h, taus, n_taus, &views, &insts);
  std::vector<double> H;
  const bool counts = (flags & ENT_BATCH_SUPPORT_COUNTS) != 0;
  s = run_entropies(c, views, insts, counts, &H);
  if (s) return s;
  s = c.end_call();
  c.collect_kernel_stats();
  if (s) return s;
  std::vector<size_t> pair_idx(M * M, 0);
  for (size_t i = 0, k = 0; i < M; ++i)
    for (size_t j = i + 1; j < M; ++j, ++k) pair_idx[i * M + j] = pair_idx[j * M + i] = k;
  for (size_t q = 0; q < n_taus; ++q) {
    const size_t b = q * per_tau;
    const size_t b2l = b + M, b2j = b + 2 * M, b3 = b + 2 * M + M * (M - 1) / 2;
    double* T = te_out + q * M * M;
    size_t k3 = 0;
    for (size_t i = 0; i < M; ++i)
      for (size_t j = 0; j < M; ++j) {
        if (i == j) {
          T[i * M + j] = counts ? H[b + i] : 0.0;
          continue;
        }
        const double h3 = H[b3 + k3++];
        T[i * M + j] = counts ? h3 : H[b2j + pair_idx[i * M + j]] + H[b2l + i] - h3 - H[b + i];
      }
  }
  return ENT_OK;
}

}  // namespace

extern "C" {

int ent_te_all_pairs(ent_ctx* ctx, const float* coords, size_t n_rows, size_t n_cols,
                     const float* h, const uint32_t* taus, size_t n_taus, uint32_t flags,
                     double* te_out) {
  return te_impl(ctx, coords, n_rows, n_cols, h, taus, n_taus, flags, te_out, false);
}

int ent_te_all_pairs_device(ent_ctx* ctx, const float* d_coords, size_t n_rows,
                            size_t n_cols, const float* h, const uint32_t* taus,
                            size_t n_taus, uint32_t flags, double* te_out) {
  return te_impl(ctx, d_coords, n_rows, n_cols, h, taus, n_taus, flags, te_out, true);
}


int ent_mi_all_pairs(ent_ctx* ctx, const float* coords, size_t n_rows,
                     size_t n_cols, const float* h, uint32_t flags,
                     double* mi_out, double* h_out) {
  return mi_impl(ctx, coords, n_rows, n_cols, h, flags, mi_out, h_out, false);
}

int ent_mi_all_pairs_device(ent_ctx* ctx, const float* d_coords, size_t n_rows,
                            size_t n_cols, const float* h, uint32_t flags,
                            double* mi_out, double* h_out) {
  return mi_impl(ctx, d_coords, n_rows, n_cols, h, flags, mi_out, h_out, true);
}

// Entropies (or support counts) of listed densities of the MI or TE batch.
static int items_impl(ent_ctx* ctx, bool te, const float* d_coords, size_t n_rows,
                      size_t n_cols, const float* h, const uint32_t* taus, size_t n_taus,
                      const uint64_t* items, size_t n_items, uint32_t flags, double* H_out) {
  if (!ctx) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  if (!d_coords || !h || (!items && n_items) || (!H_out && n_items) || (te && (!taus || !n_taus)))
    return c.fail(ENT_ERR_ARG, "null argument");
  if (n_cols < 1 || n_rows < 1) return c.fail(ENT_ERR_ARG, "empty input");
  if (n_rows > 0xffffff00ull) return c.fail(ENT_ERR_TOO_LARGE, "too many rows");
  for (size_t j = 0; j < n_cols; ++j)
    if (!(h[j] > 0.f) || !std::isfinite(h[j]))
      return c.fail(ENT_ERR_ARG, "bandwidth must be finite and positive");
  if (te)
    for (size_t q = 0; q < n_taus; ++q)
      if (taus[q] == 0 || taus[q] >= n_rows) return c.fail(ENT_ERR_ARG, "lag out of range");
  std::vector<ViewSpec> views;
  std::vector<InstSpec> insts;
  if (te) te_build(c, d_coords, n_rows, n_cols, h, taus, n_taus, &views, &insts);
  else mi_build(c, d_coords, n_rows, n_cols, h, &views, &insts);
  s = select_items(c, items, n_items, &views, &insts);
  if (s) return s;
  std::vector<double> H;
  if (n_items) {
    s = run_entropies(c, views, insts, (flags & ENT_BATCH_SUPPORT_COUNTS) != 0, &H);
    if (s) return s;
  }
  s = c.end_call();
  c.collect_kernel_stats();
  if (s) return s;
  for (size_t q = 0; q < n_items; ++q) H_out[q] = H[q];
  return ENT_OK;
}

int ent_mi_entropies_device(ent_ctx* ctx, const float* d_coords, size_t n_rows, size_t n_cols,
                            const float* h, const uint64_t* items, size_t n_items,
                            uint32_t flags, double* H_out) {
  return items_impl(ctx, false, d_coords, n_rows, n_cols, h, nullptr, 0, items, n_items, flags,
                    H_out);
}

int ent_te_entropies_device(ent_ctx* ctx, const float* d_coords, size_t n_rows, size_t n_cols,
                            const float* h, const uint32_t* taus, size_t n_taus,
                            const uint64_t* items, size_t n_items, uint32_t flags,
                            double* H_out) {
  return items_impl(ctx, true, d_coords, n_rows, n_cols, h, taus, n_taus, items, n_items, flags,
                    H_out);
}

int ent_entropy_batch(ent_ctx* ctx, const ent_instance* inst, size_t n_inst,
                      uint32_t flags, double* h_out) {
  if (!ctx) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  if (!inst || !h_out) return c.fail(ENT_ERR_ARG, "null argument");
  std::vector<ViewSpec> views;
  std::vector<InstSpec> insts(n_inst);
  for (size_t q = 0; q < n_inst; ++q) {
    const ent_instance& in = inst[q];
    if (in.d < 1 || in.d > 3) return c.fail(ENT_ERR_DIM, ent_status_string(ENT_ERR_DIM));
    if (!in.coords || in.n < 1) return c.fail(ENT_ERR_ARG, "empty instance");
    if (in.n > 0xffffff00ull) return c.fail(ENT_ERR_TOO_LARGE, "too many rows");
    const bool dev = (flags & ENT_BATCH_DEVICE_INPUT) != 0;
    const float* base = in.coords;
    if (!dev) {
      float* p = static_cast<float*>(c.arena.alloc(4 * in.n * in.d));
      if (!p) return c.fail(ENT_ERR_CUDA, "out of device memory");
      cudaError_t e = cudaMemcpyAsync(p, in.coords, 4 * in.n * in.d,
                                      cudaMemcpyHostToDevice, c.stream);
      if (e != cudaSuccess) return c.cuda_fail(e, "copy coordinates");
      base = p;
    }
    InstSpec& I = insts[q];
    I.d = in.d;
    I.n = (uint32_t)in.n;
    I.norm = (double)in.n;
    I.S = c.strip_subdiv;
    for (uint32_t j = 0; j < in.d; ++j) {
      if (!(in.h[j] > 0.f) || !std::isfinite(in.h[j]))
        return c.fail(ENT_ERR_ARG, "bandwidth must be finite and positive");
      I.h[j] = in.h[j];
      I.view[j] = (uint32_t)views.size();
      views.push_back({base + (size_t)j * in.n, (uint32_t)in.n});
    }
  }
  std::vector<double> H;
  s = run_entropies(c, views, insts, (flags & ENT_BATCH_SUPPORT_COUNTS) != 0, &H);
  if (s) return s;
  s = c.end_call();
  c.collect_kernel_stats();
  if (s) return s;
  for (size_t q = 0; q < n_inst; ++q) h_out[q] = H[q];
  return ENT_OK;
}

}  // extern "C"

// ------------------------------------------------------------ autotuner
namespace {

struct TuneCand {
  int variant, tile_r;
  uint32_t cells;
};

// Candidate shapes per density dimension: pair body (ent_tuning numbering
// minus one), targets per warp of the ordered bodies, cells per bandwidth
// (dimension 1 for d = 2, the strip-moment strips for PAIR_MOMENT,
// dimensions 1 and 2 for d = 3).
std::vector<TuneCand> tune_candidates(uint32_t d) {
  if (d == 1) return {{2, 16, 2}, {4, 16, 2}, {5, 16, 2}, {PAIR_RANGE, 16, 2}};
  if (d == 2)
    return {{2, 16, 2},           {4, 16, 1},           {4, 16, 2},          {4, 16, 3},
            {5, 16, 2},           {PAIR_MOMENT, 16, 3}, {PAIR_MOMENT, 16, 4}};
  return {{1, 8, 1}, {2, 8, 1}, {4, 8, 1}, {4, 8, 2}, {5, 8, 1}};
}

void apply_choice(Ctx& c, uint32_t d, int variant, int tile_r, uint32_t cells) {
  c.pair_variant[d - 1] = variant;
  if (d == 2) c.moment_auto = false;
  c.tile_r[d - 1] = tile_r;
  if (d == 2 && variant == PAIR_MOMENT) c.moment_cells = cells;
  else if (d == 2) c.strip_subdiv = cells;
  if (d == 3) c.strip_subdiv3 = cells;
}

}  // namespace

extern "C" {

int ent_autotune(ent_ctx* ctx, const ent_instance* sample, size_t n_sample, uint32_t d,
                 uint32_t flags, ent_tuning* chosen) {
  if (!ctx) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  if (d < 1 || d > 3) return c.fail(ENT_ERR_DIM, ent_status_string(ENT_ERR_DIM));
  if (!sample || n_sample == 0) return c.fail(ENT_ERR_ARG, "empty sample");
  uint64_t nmax = 0;
  for (size_t q = 0; q < n_sample; ++q)
    if (sample[q].d == d) nmax = std::max<uint64_t>(nmax, sample[q].n);
  if (nmax == 0) return c.fail(ENT_ERR_ARG, "no sample instance of dimension d");
  int bucket = 0;
  while ((2ull << bucket) <= nmax) ++bucket;
  const uint32_t key = (d << 8) | (uint32_t)bucket;
  auto it = c.tune_cache.find(key);
  if (it != c.tune_cache.end() && !(flags & ENT_TUNE_FORCE)) {
    apply_choice(c, d, it->second.variant, it->second.tile_r, it->second.cells);
  } else {
    const Ctx::TuneChoice keep{
        c.pair_variant[d - 1], c.tile_r[d - 1],
        d == 2 ? (c.pair_variant[1] == PAIR_MOMENT ? c.moment_cells : c.strip_subdiv)
               : c.strip_subdiv3};
    std::vector<double> h(n_sample);
    const uint32_t bflags = flags & ENT_BATCH_DEVICE_INPUT;
    float best = 0.f;
    Ctx::TuneChoice pick = keep;
    bool have = false;
    for (const TuneCand& t : tune_candidates(d)) {
      apply_choice(c, d, t.variant, t.tile_r, t.cells);
      float ms = 0.f;
      for (int rep = 0; rep < 3; ++rep) {  // first run warms up
        const int s = ent_entropy_batch(ctx, sample, n_sample, bflags, h.data());
        if (s) {
          apply_choice(c, d, keep.variant, keep.tile_r, keep.cells);
          return s;
        }
        const float m = c.stats.pair_kernel_ms_by_dim[d - 1];
        if (rep == 1 || (rep == 2 && m < ms)) ms = m;
      }
      if (!have || ms < best) {
        best = ms;
        pick = {t.variant, t.tile_r, t.cells};
        have = true;
      }
    }
    c.tune_cache[key] = pick;
    apply_choice(c, d, pick.variant, pick.tile_r, pick.cells);
  }
  if (chosen) return ent_get_tuning(ctx, chosen);
  return ENT_OK;
}

size_t ent_autotune_cache_size(const ent_ctx* ctx) {
  if (!ctx) return 0;
  return reinterpret_cast<const Ctx*>(ctx)->tune_cache.size();
}

}  // extern "C"

