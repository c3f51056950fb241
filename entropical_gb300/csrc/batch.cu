// Batched estimators: all-pairs mutual information and uneven entropy
// batches, each run as ONE engine batch, i.e. one persistent pair-kernel
// launch per dimension over every (instance, tile) work item.
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

// Runs the engine in log-sum (or support-count) mode and returns, per
// instance, -mean(log p) (or the in-support pair count).
int run_entropies(Ctx& c, const std::vector<ViewSpec>& views,
                  std::vector<InstSpec>& insts, bool counts,
                  std::vector<double>* H) {
  Engine eng;
  EngineOut eo;
  const uint32_t mode = counts ? (DM_COUNT | DM_SUMV) : DM_LOGSUM;
  if (counts)
    for (auto& s : insts) s.norm = 1.0;
  int s = eng.run(c, views, insts, mode, &eo);
  if (s) return s;
  std::vector<double> ls(insts.size());
  cudaError_t e = cudaMemcpyAsync(ls.data(), eo.d_logsum_sorted,
                                  sizeof(double) * insts.size(),
                                  cudaMemcpyDeviceToHost, c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "read log-sums");
  e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "batch");
  H->assign(insts.size(), 0.0);
  for (size_t r = 0; r < insts.size(); ++r) {
    const uint32_t i = eo.slot_order[r];
    if (counts) {
      (*H)[i] = ls[r];
    } else {
      (*H)[i] = -ls[r] / (double)insts[i].n;
    }
  }
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
  std::vector<ViewSpec> views(n_cols);
  for (size_t j = 0; j < n_cols; ++j) views[j] = {dc + j * n_rows, (uint32_t)n_rows};
  std::vector<InstSpec> insts;
  insts.reserve(n_cols + n_cols * (n_cols - 1) / 2);
  for (size_t i = 0; i < n_cols; ++i) {
    InstSpec I;
    I.d = 1;
    I.n = (uint32_t)n_rows;
    I.view[0] = (uint32_t)i;
    I.h[0] = h[i];
    I.norm = (double)n_rows;
    I.S = c.strip_subdiv;
    insts.push_back(I);
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
      insts.push_back(I);
    }
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

}  // namespace

extern "C" {

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
