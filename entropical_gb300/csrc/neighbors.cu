// Neighbour searches of the reference, on the device, bit-exact.
//
// * ENT_NB_WINDOW: boxes() (densities_omp.cpp:33-65). For every point x_i of
//   a column, against the value-sorted column s: lo_i = first k with
//   x_i - s_k < h, hi_i = last k with s_k - x_i < h (float subtraction and
//   strict compare, as the reference). Both predicates are monotone in k, so
//   a bisection finds exactly the element the reference's linear scans stop
//   at; the window size hi - lo + 1 is the number of sources the reference
//   density loop visits for that point.
// * ENT_NB_BOXED: Transs::BoxedSearch::Boxes (boxedsearch.cpp:15-62): boxes of
//   width `box` from the column minimum, box = floor((x - min) / box) in float,
//   neighbour list = own box and the adjacent ones. Its undefined cases are
//   defined (the maximum starts from the lowest float rather than the
//   smallest positive one, an index equal to the box count is clamped to the
//   last box, and a zero-width range has one box).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "../../include/entropical_gb300.h"
#include "api_internal.h"
#include "engine.h"

using namespace ent;

namespace {

__global__ void k_gather_values(const float* __restrict__ x, const uint32_t* __restrict__ perm,
                                float* __restrict__ s, uint32_t n) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    s[k] = x[perm[k]];
}

__global__ void k_windows(const float* __restrict__ x, const float* __restrict__ s, uint32_t n,
                          float h, uint64_t* __restrict__ lo, uint64_t* __restrict__ hi) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float r = x[i];
    uint32_t a = 0, b = n;  // first k with r - s[k] < h
    while (a < b) {
      const uint32_t m = a + (b - a) / 2;
      if (__fsub_rn(r, s[m]) < h) b = m; else a = m + 1;
    }
    lo[i] = a;
    a = 0;
    b = n;  // first k with s[k] - r >= h, minus one
    while (a < b) {
      const uint32_t m = a + (b - a) / 2;
      if (__fsub_rn(s[m], r) < h) a = m + 1; else b = m;
    }
    hi[i] = (uint64_t)a - 1;
  }
}

__global__ void k_boxes(const float* __restrict__ x, uint32_t n, float mn, float box,
                        uint64_t nb, uint64_t* __restrict__ box_of, uint32_t* __restrict__ cnt) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float q = __fdiv_rn(__fsub_rn(x[i], mn), box);
    uint64_t b = (uint64_t)floor((double)q);
    if (b >= nb) b = nb - 1;
    box_of[i] = b;
    atomicAdd(cnt + b, 1u);
  }
}

__global__ void k_box_neighbors(const uint64_t* __restrict__ box_of, uint32_t n, uint64_t nb,
                                const uint32_t* __restrict__ cnt, uint64_t* __restrict__ out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint64_t b = box_of[i];
    uint64_t c = cnt[b];
    if (b > 0) c += cnt[b - 1];
    if (b + 1 < nb) c += cnt[b + 1];
    out[i] = c;
  }
}

unsigned grid_for(uint32_t n) { return std::min<uint32_t>((n + 255) / 256, 4096u) + 1; }

}  // namespace

extern "C" int ent_neighbor_counts(ent_ctx* ctx, const float* col, size_t n, float h,
                                   uint32_t mode, uint64_t* out_a, uint64_t* out_b,
                                   uint64_t* n_boxes) {
  if (!ctx) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  if (!col || !out_a || !out_b || n == 0) return c.fail(ENT_ERR_ARG, "null argument");
  if (!(h > 0.f) || !std::isfinite(h)) return c.fail(ENT_ERR_ARG, "width must be finite and positive");
  if (n > 0xffffff00ull) return c.fail(ENT_ERR_TOO_LARGE, "too many rows");
  if (mode != ENT_NB_WINDOW && mode != ENT_NB_BOXED) return c.fail(ENT_ERR_ARG, "unknown mode");
  cudaError_t e;
  const uint32_t nn = (uint32_t)n;
  float* dx = static_cast<float*>(c.arena.alloc(4 * n));
  uint64_t* da = static_cast<uint64_t*>(c.arena.alloc(8 * n));
  uint64_t* db = static_cast<uint64_t*>(c.arena.alloc(8 * n));
  if (!dx || !da || !db) return c.fail(ENT_ERR_CUDA, "out of device memory");
  e = cudaMemcpyAsync(dx, col, 4 * n, cudaMemcpyHostToDevice, c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "copy column");
  std::vector<ViewSpec> views(1, ViewSpec{dx, nn});
  SortedViews sv;
  s = sort_views(c, views, &sv);  // also rejects non-finite input
  if (s) return s;
  uint64_t nb = 0;
  if (mode == ENT_NB_WINDOW) {
    float* ds = static_cast<float*>(c.arena.alloc(4 * n));
    if (!ds) return c.fail(ENT_ERR_CUDA, "out of device memory");
    k_gather_values<<<grid_for(nn), 256, 0, c.stream>>>(dx, sv.perm, ds, nn);
    k_windows<<<grid_for(nn), 256, 0, c.stream>>>(dx, ds, nn, h, da, db);
    c.stats.kernel_launches += 2;
  } else {
    const float mn = sv.stats[0].mn, mx = sv.stats[0].mx;
    const float range = mx - mn;
    nb = (uint64_t)std::ceil((double)(range / h));
    if (nb == 0) nb = 1;
    uint32_t* cnt = static_cast<uint32_t*>(c.arena.alloc(4 * nb));
    if (!cnt) return c.fail(ENT_ERR_CUDA, "out of device memory");
    cudaMemsetAsync(cnt, 0, 4 * nb, c.stream);
    k_boxes<<<grid_for(nn), 256, 0, c.stream>>>(dx, nn, mn, h, nb, da, cnt);
    k_box_neighbors<<<grid_for(nn), 256, 0, c.stream>>>(da, nn, nb, cnt, db);
    c.stats.kernel_launches += 2;
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return c.cuda_fail(e, "neighbour kernels");
  e = cudaMemcpyAsync(out_a, da, 8 * n, cudaMemcpyDeviceToHost, c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "copy results");
  e = cudaMemcpyAsync(out_b, db, 8 * n, cudaMemcpyDeviceToHost, c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "copy results");
  s = c.end_call();
  if (n_boxes) *n_boxes = nb;
  return s;
}
