// AMISE convolution sums and the hestimate bandwidth search on the device.
//
// Replaces epa_convolution (densities_omp.cpp:235-277; the CUDA form
// epa_conv.cuh:191-229 launches the density kernel instead, see the
// reference defect list) and the AmiseMin search (hestimate.cpp:41-104):
//
//   C(h) = 1/n^2 sum_i sum_j max(0, 4.5 - 2.25 |x_i - x_j| / h)
//   amise(h) = (0.04 / h^5 * C(h))^0.2 * 1.25 * 0.6^0.8 / n^0.8
//   bracket [0.1 h0, 2 h0], prec 0.01 h0: at each level evaluate amise at the
//   two quarter points and keep the half on the side of the smaller value.
//
// Columns are value-sorted once (radix sort of the engine). In a sorted
// column the support of target i is one contiguous index range, so C(h) is
// evaluated from FP64 prefix sums of the centred values: per target one
// binary search for the end of its range and a few FP64 operations
// (k_conv_range), O(n log n) per bandwidth instead of O(n * support). The
// per-column search state lives on the device; each level is conv (both
// pivots) -> per-column reduce -> decide, all columns at once, and the level
// sequence is captured into one CUDA graph.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <vector>

#include "../../include/entropical_gb300.h"
#include "api_internal.h"
#include "engine.h"
#include "staging.cuh"  // FULL_MASK

using namespace ent;

namespace {

struct ConvCol {
  const float* xs;      // value-sorted column (n + 8 floats)
  double* P;            // P[k] = sum_{j<k} (xs[j] - xs[n/2]), k = 0..n
  uint32_t n;
  uint32_t tile_base;   // first target block (slot) of the column
  uint32_t n_tiles;     // target blocks: ceil(n / CONV_TB)
  uint32_t chunk_base;  // first prefix chunk of the column
};

// Search state of one column (hestimate.cpp:55-86 recursion, unrolled).
struct HestState {
  float h0, lo, hi, prec;
  float glo, ghi;      // global bracket [0.1 h0, 2 h0]
  float node_lo, node_hi;  // warm start: bracket after the skipped levels
  float piv[2];        // pivots of the current level (or the single h)
  float result;
  int level, done, iter_max;
  int n_conv;
  int dirs;            // bit 0: a lower-half decision, bit 1: an upper-half one
  int warm, converged;
  uint32_t n;
};

// Sequential float sums in the reference's order give the reference's h0
// bit for bit (Boost lazy variance over float, hestimate.cpp:19-30). One warp
// per column: the lanes load 32 consecutive values at a time (coalesced, the
// next group in flight) and every lane adds them in element order from
// shuffles, so each lane holds the same sequential sums. With with_h0 = 0
// (a plain convolution) only n is recorded.
__global__ void k_thumb(const ConvCol* __restrict__ cols, const float* __restrict__ raw,
                        const uint64_t* __restrict__ raw_off, const double* __restrict__ pw,
                        HestState* __restrict__ st, uint32_t n_cols, int with_h0) {
  const uint32_t c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= n_cols) return;  // warp-uniform
  const uint32_t n = cols[c].n;
  if (!with_h0) {
    if (lane == 0) st[c].n = n;
    return;
  }
  const float* x = raw + raw_off[c];
  float s = 0.f, s2 = 0.f;
  float nxt = lane < n ? x[lane] : 0.f;
  for (uint32_t i0 = 0; i0 < n; i0 += 32) {
    const float cur = nxt;
    const uint32_t j = i0 + 32 + lane;
    nxt = j < n ? x[j] : 0.f;
    const uint32_t m = min(32u, n - i0);
    for (uint32_t k = 0; k < m; ++k) {
      const float v = __shfl_sync(0xffffffffu, cur, k);
      s = __fadd_rn(s, v);
      s2 = __fadd_rn(s2, __fmul_rn(v, v));
    }
  }
  if (lane == 0) {
    const float m2 = __fdiv_rn(s2, (float)n);
    const float m = __fdiv_rn(s, (float)n);
    const float var = __fsub_rn(m2, __fmul_rn(m, m));
    st[c].h0 = (float)(pw[c] * sqrt((double)var));
    st[c].n = n;
  }
}

// raw_off: offset of each column in the raw coordinates; perm_off: offset of
// its value order in the sort permutation (laid out by view, not by column).
__global__ void k_gather_sorted(const ConvCol* __restrict__ cols,
                                const float* __restrict__ raw,
                                const uint64_t* __restrict__ raw_off,
                                const uint32_t* __restrict__ perm,
                                const uint64_t* __restrict__ perm_off) {
  const ConvCol& C = cols[blockIdx.y];
  const float* x = raw + raw_off[blockIdx.y];
  const uint32_t* p = perm + perm_off[blockIdx.y];
  float* xs = const_cast<float*>(C.xs);
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < C.n + 8;
       k += gridDim.x * blockDim.x)
    xs[k] = k < C.n ? x[p[k]] : 0.f;
}

// Start a full search (hestimate.cpp:101-103) or a warm one: descend
// `skip` levels of the same dyadic bracket tree towards h_init without
// evaluating anything, then search from there.
__global__ void k_hest_init(HestState* __restrict__ st, uint32_t n_cols,
                            const float* __restrict__ h_init, int skip, int fixed_h,
                            const float* __restrict__ log_ratio) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_cols) return;
  HestState s = st[c];
  s.level = 0;
  s.done = 0;
  s.n_conv = 0;
  s.dirs = 0;
  s.iter_max = 20;
  s.converged = 1;
  s.warm = 0;
  if (fixed_h) {  // plain epa_convolution: one bandwidth, no search
    s.piv[0] = s.piv[1] = h_init[c];
    st[c] = s;
    return;
  }
  s.prec = (float)(0.01 * (double)s.h0);
  s.lo = (float)(0.1 * (double)s.h0);
  s.hi = 2.f * s.h0;
  s.glo = s.lo;
  s.ghi = s.hi;
  if ((h_init || log_ratio) && skip > 0) {
    s.warm = 1;
    // start value: given, or h0 * exp(r) from the learned log-ratio
    const float t = log_ratio ? s.h0 * expf(log_ratio[c]) : h_init[c];
    for (int k = 0; k < skip; ++k) {
      const float delta = s.hi - s.lo;
      const float pivot = (float)((double)s.lo + 0.5 * (double)delta);
      if (s.iter_max == 0 || delta <= s.prec) break;
      if (t < pivot) s.hi = pivot; else s.lo = pivot;
      s.iter_max -= 1;
      s.level += 1;
    }
  }
  s.node_lo = s.lo;
  s.node_hi = s.hi;
  const float delta = s.hi - s.lo;
  const float pivot = (float)((double)s.lo + 0.5 * (double)delta);
  if (s.iter_max == 0 || delta <= s.prec) {
    s.done = 1;
    s.result = pivot;
  } else {
    s.piv[0] = (float)((double)pivot - 0.25 * (double)delta);
    s.piv[1] = (float)((double)pivot + 0.25 * (double)delta);
  }
  st[c] = s;
}

// ---------------------------------------------------------------- prefix
// P[k] = sum_{j<k} (xs[j] - mu) in FP64 for every column, mu = xs[n/2]:
// centring keeps the partial sums near the spread of the data, so the range
// sums below lose few bits. Three passes: chunk totals, one warp scanning
// each column's chunk totals, chunk-local scans from the chunk offsets. Every
// sum runs in a fixed order, so P is deterministic.
constexpr uint32_t CONV_TB = 256;                // targets per block of k_conv_range
constexpr uint32_t PF_E = 8;                     // prefix values per thread
constexpr uint32_t PF_CHUNK = CONV_TB * PF_E;    // prefix values per block

__device__ __forceinline__ double col_centre(const ConvCol& C) {
  return (double)C.xs[C.n / 2];
}

__global__ void __launch_bounds__(CONV_TB)
    k_prefix_totals(const ConvCol* __restrict__ cols, double* __restrict__ chunk_tot) {
  __shared__ double sw[CONV_TB / 32];
  const ConvCol& C = cols[blockIdx.y];
  const uint64_t b0 = (uint64_t)blockIdx.x * PF_CHUNK;
  if (b0 >= C.n) return;  // block-uniform
  const double mu = col_centre(C);
  const uint64_t k0 = b0 + (uint64_t)threadIdx.x * PF_E;
  double a = 0.0;
#pragma unroll
  for (uint32_t e = 0; e < PF_E; ++e)
    if (k0 + e < C.n) a += (double)C.xs[k0 + e] - mu;
  for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(FULL_MASK, a, o);
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (uint32_t w = 0; w < CONV_TB / 32; ++w) t += sw[w];
    chunk_tot[C.chunk_base + blockIdx.x] = t;
  }
}

// One warp per column: exclusive scan of its chunk totals, in place.
__global__ void k_prefix_chunks(const ConvCol* __restrict__ cols, uint32_t n_cols,
                                double* __restrict__ chunk_tot) {
  const uint32_t c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= n_cols) return;  // warp-uniform
  const uint32_t nch = (cols[c].n + PF_CHUNK - 1) / PF_CHUNK;
  double* t = chunk_tot + cols[c].chunk_base;
  double run = 0.0;
  for (uint32_t b = 0; b < nch; b += 32) {
    const double v = b + lane < nch ? t[b + lane] : 0.0;
    double inc = v;
    for (int o = 1; o < 32; o <<= 1) {
      const double u = __shfl_up_sync(FULL_MASK, inc, o);
      if (lane >= o) inc += u;
    }
    double exc = __shfl_up_sync(FULL_MASK, inc, 1);
    if (lane == 0) exc = 0.0;
    if (b + lane < nch) t[b + lane] = run + exc;
    run += __shfl_sync(FULL_MASK, inc, 31);
  }
}

__global__ void __launch_bounds__(CONV_TB)
    k_prefix_write(const ConvCol* __restrict__ cols, const double* __restrict__ chunk_off) {
  __shared__ double sw[CONV_TB / 32];
  const ConvCol& C = cols[blockIdx.y];
  const uint64_t b0 = (uint64_t)blockIdx.x * PF_CHUNK;
  if (b0 >= C.n) return;  // block-uniform
  const double mu = col_centre(C);
  const uint64_t k0 = b0 + (uint64_t)threadIdx.x * PF_E;
  double v[PF_E];
  double tot = 0.0;
#pragma unroll
  for (uint32_t e = 0; e < PF_E; ++e) {
    if (k0 + e < C.n) tot += (double)C.xs[k0 + e] - mu;
    v[e] = tot;  // inclusive within the thread
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double inc = tot;
  for (int o = 1; o < 32; o <<= 1) {
    const double u = __shfl_up_sync(FULL_MASK, inc, o);
    if (lane >= o) inc += u;
  }
  if (lane == 31) sw[warp] = inc;
  __syncthreads();
  double base = chunk_off[C.chunk_base + blockIdx.x];
  for (int w = 0; w < warp; ++w) base += sw[w];
  double exc = __shfl_up_sync(FULL_MASK, inc, 1);
  if (lane == 0) exc = 0.0;
  base += exc;
  double* P = C.P;
  if (b0 == 0 && threadIdx.x == 0) P[0] = 0.0;
#pragma unroll
  for (uint32_t e = 0; e < PF_E; ++e)
    if (k0 + e < C.n) P[k0 + e + 1] = base + v[e];
}

// --------------------------------------------------------- convolution
// C(h) n^2 = sum_i sum_j K_ij with K_ij = 4.5 - 2.25 |x_i - x_j| / h on the
// support |x_i - x_j| <= 2h. The support is symmetric and, in a sorted
// column, contiguous: for target i the partners j > i are i+1 .. e_i - 1,
// e_i the first index with fl(x_j - x_i) > 2h (a monotone predicate, found
// by binary search). With c_i = e_i - 1 - i partners and
// S_i = sum_{j=i+1}^{e_i-1} (x_j - x_i) = (P[e_i] - P[i+1]) - c_i (x_i - mu),
//   sum_j K_ij over j > i = 4.5 c_i - 2.25 S_i / h,
// and the double sum is 4.5 n + 2 sum_i (4.5 c_i - 2.25 S_i / h): exact
// arithmetic on the same support as the reference's per-pair loop
// (densities_omp.cpp:247-272), O(log n) per target instead of O(support).
// One thread per target, CONV_TB targets per block; NP bandwidths per pass
// (1: plain epa_convolution, 2: both pivots of a search level). Each block
// writes its partial double sums to its slot; k_conv_reduce adds the slots
// of a column in a fixed order.
template <int NP>
__global__ void __launch_bounds__(CONV_TB)
    k_conv_range(const ConvCol* __restrict__ cols, uint32_t n_cols,
                 const uint32_t* __restrict__ col_tile_base, const HestState* __restrict__ st,
                 double* __restrict__ tile_sum) {
  __shared__ double sA[NP][CONV_TB / 32];
  __shared__ unsigned long long sC[NP][CONV_TB / 32];
  const uint32_t g = blockIdx.x;
  uint32_t lo = 0, hi = n_cols;
  while (hi - lo > 1) {
    const uint32_t m = (lo + hi) / 2;
    if (col_tile_base[m] <= g) lo = m; else hi = m;
  }
  const ConvCol& C = cols[lo];
  if (st[lo].done) {  // block-uniform
    if (threadIdx.x == 0) tile_sum[2 * (size_t)g] = tile_sum[2 * (size_t)g + 1] = 0.0;
    return;
  }
  const uint32_t n = C.n;
  const uint32_t blk = g - C.tile_base;
  const uint32_t i = blk * CONV_TB + threadIdx.x;
  const float* __restrict__ xs = C.xs;
  const double* __restrict__ P = C.P;
  float w[NP];
#pragma unroll
  for (int k = 0; k < NP; ++k) w[k] = 2.f * st[lo].piv[k];
  double A[NP];
  unsigned long long cnt[NP];
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    A[k] = 0.0;
    cnt[k] = 0ull;
  }
  if (i < n) {
    const float xi = xs[i];
    const double xc = (double)xi - col_centre(C);
    const double p1 = P[i + 1];
#pragma unroll
    for (int k = 0; k < NP; ++k) {
      uint32_t a = i + 1, b = n;  // first j > i with fl(x_j - x_i) > 2h
      while (a < b) {
        const uint32_t m = a + ((b - a) >> 1);
        if (__fsub_rn(xs[m], xi) > w[k]) b = m; else a = m + 1;
      }
      const uint32_t c = a - 1 - i;
      A[k] = fma(-(double)c, xc, P[a] - p1);
      cnt[k] = c;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    for (int o = 16; o; o >>= 1) {
      A[k] += __shfl_xor_sync(FULL_MASK, A[k], o);
      cnt[k] += __shfl_xor_sync(FULL_MASK, cnt[k], o);
    }
    if (lane == 0) {
      sA[k][warp] = A[k];
      sC[k][warp] = cnt[k];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t nb = min(CONV_TB, n - blk * CONV_TB);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      double t = 0.0;
      if (k < NP) {
        double sa = 0.0;
        unsigned long long sc = 0ull;
        for (uint32_t q = 0; q < CONV_TB / 32; ++q) {
          sa += sA[k][q];
          sc += sC[k][q];
        }
        t = 4.5 * (double)nb + 9.0 * (double)sc - (4.5 / (double)st[lo].piv[k]) * sa;
      }
      tile_sum[2 * (size_t)g + k] = t;
    }
  }
}

__global__ void __launch_bounds__(256)
    k_conv_reduce(const ConvCol* __restrict__ cols, const double* __restrict__ tile_sum,
                  double* __restrict__ col_sum) {
  __shared__ double sw[8][2];
  const ConvCol& C = cols[blockIdx.x];
  double a0 = 0.0, a1 = 0.0;
  for (uint32_t t = threadIdx.x; t < C.n_tiles; t += blockDim.x) {
    a0 += tile_sum[2 * (size_t)(C.tile_base + t)];
    a1 += tile_sum[2 * (size_t)(C.tile_base + t) + 1];
  }
  for (int o = 16; o; o >>= 1) {
    a0 += __shfl_xor_sync(FULL_MASK, a0, o);
    a1 += __shfl_xor_sync(FULL_MASK, a1, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sw[threadIdx.x >> 5][0] = a0;
    sw[threadIdx.x >> 5][1] = a1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0.0, t1 = 0.0;
    for (int w = 0; w < 8; ++w) {
      t0 += sw[w][0];
      t1 += sw[w][1];
    }
    col_sum[2 * blockIdx.x] = t0;
    col_sum[2 * blockIdx.x + 1] = t1;
  }
}

// AmiseMin::_amise (hestimate.cpp:41-53) in the reference's float/double mix.
__device__ float amise_of(float conv, float h, uint32_t n) {
  float a = (float)(0.04 * 1 / pow((double)h, 5.0) * (double)conv);
  a = (float)pow((double)a, 0.2);
  a = (float)((double)a * 1.25 * pow(0.6, 0.8) / pow((double)(float)n, 0.8));
  return a;
}

__device__ __forceinline__ float conv_value(double sum, uint32_t n) {
  // kahan_sum(outer) / (n_rows * n_rows) in float (densities_omp.cpp:276)
  return __fdiv_rn((float)sum, (float)((unsigned long long)n * n));
}

// One level of the interval search (hestimate.cpp:55-86) for every column.
__global__ void k_hest_level(HestState* __restrict__ st, uint32_t n_cols,
                             const double* __restrict__ col_sum,
                             float* __restrict__ conv_out) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_cols) return;
  HestState s = st[c];
  if (s.done) return;
  const float cl = conv_value(col_sum[2 * c], s.n);
  const float ch = conv_value(col_sum[2 * c + 1], s.n);
  if (conv_out) {
    conv_out[2 * c] = cl;
    conv_out[2 * c + 1] = ch;
  }
  const float al = amise_of(cl, s.piv[0], s.n);
  const float ah = amise_of(ch, s.piv[1], s.n);
  s.n_conv += 2;
  const float delta0 = s.hi - s.lo;
  const float pivot0 = (float)((double)s.lo + 0.5 * (double)delta0);
  if (al < ah) {
    s.hi = pivot0;
    s.dirs |= 1;
  } else {
    s.lo = pivot0;
    s.dirs |= 2;
  }
  s.iter_max -= 1;
  s.level += 1;
  const float delta = s.hi - s.lo;
  const float pivot = (float)((double)s.lo + 0.5 * (double)delta);
  if (s.iter_max == 0 || delta <= s.prec) {
    s.done = 1;
    s.result = pivot;
    // A warm search whose every decision pointed towards the same edge of
    // its starting node, where that edge is not the global bracket's, may
    // have left the optimum outside the node: report it for a full search.
    if (s.warm) {
      if ((s.dirs == 2 && s.node_hi < s.ghi) || (s.dirs == 1 && s.node_lo > s.glo))
        s.converged = 0;
    }
  } else {
    s.piv[0] = (float)((double)pivot - 0.25 * (double)delta);
    s.piv[1] = (float)((double)pivot + 0.25 * (double)delta);
  }
  st[c] = s;
}

__global__ void k_conv_single_out(const HestState* __restrict__ st, uint32_t n_cols,
                                  const double* __restrict__ col_sum, float* __restrict__ out) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n_cols) out[c] = conv_value(col_sum[2 * c], st[c].n);
}

__global__ void k_pick(const float* __restrict__ y, const uint32_t* __restrict__ map,
                       float* __restrict__ out, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = y[map[i]];
}

template <class T>
T* upload(Ctx& c, const std::vector<T>& v, cudaError_t* e) {
  T* p = static_cast<T*>(c.arena.alloc(sizeof(T) * std::max<size_t>(v.size(), 1)));
  if (!p) {
    *e = cudaErrorMemoryAllocation;
    return nullptr;
  }
  *e = v.empty() ? cudaSuccess
                 : cudaMemcpyAsync(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice,
                                   c.stream);
  return p;
}


}  // namespace

// Shared implementation of ent_epa_convolution / ent_hestimate. `raw` holds
// n_cols device columns back to back (raw_off offsets). mode: 0 = fixed
// bandwidths h_fixed (convolution only), 1 = full search, 2 = warm search.
namespace {

// One pass of the search over at most kHestMaxCols columns, all held at once.
int hestimate_pass(Ctx& c, const float* raw, const std::vector<uint64_t>& raw_off,
                   const std::vector<uint32_t>& lens, int mode, const float* h_fixed_or_init,
                   int skip, float* h_out, float* conv_out, ent_hest_stats* stats,
                   const float* d_log_ratio) {
  cudaError_t e;
  const cudaStream_t s = c.stream;
  const uint32_t nc = (uint32_t)lens.size();
  if (nc == 0) return ENT_OK;
  // value sort of every column through the engine's radix sort
  std::vector<ViewSpec> views(nc);
  for (uint32_t i = 0; i < nc; ++i) views[i] = {raw + raw_off[i], lens[i]};
  SortedViews sv;
  int rs = sort_views(c, views, &sv);
  if (rs) return rs;
  std::vector<ConvCol> hc(nc);
  uint32_t slots = 0, chunks = 0;
  std::vector<uint32_t> base(nc);
  std::vector<double> pw(nc);
  for (uint32_t i = 0; i < nc; ++i) {
    hc[i].n = lens[i];
    hc[i].xs = static_cast<float*>(c.arena.alloc(4 * ((size_t)lens[i] + 8)));
    hc[i].P = static_cast<double*>(c.arena.alloc(8 * ((size_t)lens[i] + 1)));
    if (!hc[i].xs || !hc[i].P) return c.fail(ENT_ERR_CUDA, "out of device memory");
    hc[i].n_tiles = (lens[i] + CONV_TB - 1) / CONV_TB;
    hc[i].tile_base = slots;
    hc[i].chunk_base = chunks;
    base[i] = slots;
    slots += hc[i].n_tiles;
    chunks += (lens[i] + PF_CHUNK - 1) / PF_CHUNK;
    pw[i] = std::pow((double)lens[i], -1.0 / 7.0);  // std::pow(n_rows, -1/7)
  }
  ConvCol* dcols = upload(c, hc, &e);
  if (e != cudaSuccess) return c.cuda_fail(e, "upload columns");
  uint64_t* doff = upload(c, raw_off, &e);
  if (e != cudaSuccess) return c.cuda_fail(e, "upload offsets");
  uint64_t* dpoff = upload(c, sv.off, &e);
  if (e != cudaSuccess) return c.cuda_fail(e, "upload permutation offsets");
  double* dpw = upload(c, pw, &e);
  if (e != cudaSuccess) return c.cuda_fail(e, "upload powers");
  uint32_t* dbase = upload(c, base, &e);
  if (e != cudaSuccess) return c.cuda_fail(e, "upload tile bases");
  std::vector<float> hin(nc, 1.f);
  if (h_fixed_or_init) hin.assign(h_fixed_or_init, h_fixed_or_init + nc);
  float* dhin = upload(c, hin, &e);
  if (e != cudaSuccess) return c.cuda_fail(e, "upload bandwidths");
  HestState* dst = static_cast<HestState*>(c.arena.alloc(sizeof(HestState) * nc));
  double* tsum = static_cast<double*>(c.arena.alloc(16 * (size_t)std::max(slots, 1u)));
  double* csum = static_cast<double*>(c.arena.alloc(16 * (size_t)nc));
  double* ctot = static_cast<double*>(c.arena.alloc(8 * (size_t)std::max(chunks, 1u)));
  float* dconv = static_cast<float*>(c.arena.alloc(8 * (size_t)nc * 24));
  if (!dst || !tsum || !csum || !ctot || !dconv)
    return c.fail(ENT_ERR_CUDA, "out of device memory");
  cudaMemsetAsync(dst, 0, sizeof(HestState) * nc, s);

  const unsigned gx = std::min<uint32_t>((std::max(sv.max_n, 1u) + 255) / 256 + 1, 1024);
  const unsigned gc = (std::max(sv.max_n, 1u) + PF_CHUNK - 1) / PF_CHUNK;
  k_gather_sorted<<<dim3(gx, nc), 256, 0, s>>>(dcols, raw, doff, sv.perm, dpoff);
  k_thumb<<<(nc + 3) / 4, 128, 0, s>>>(dcols, raw, doff, dpw, dst, nc, mode == 0 ? 0 : 1);
  k_hest_init<<<(nc + 63) / 64, 64, 0, s>>>(
      dst, nc, (mode == 0 || (mode == 2 && !d_log_ratio)) ? dhin : nullptr,
      mode == 2 ? skip : 0, mode == 0 ? 1 : 0, mode == 2 ? d_log_ratio : nullptr);
  k_prefix_totals<<<dim3(gc, nc), CONV_TB, 0, s>>>(dcols, ctot);
  k_prefix_chunks<<<(nc + 3) / 4, 128, 0, s>>>(dcols, nc, ctot);
  k_prefix_write<<<dim3(gc, nc), CONV_TB, 0, s>>>(dcols, ctot);
  c.stats.kernel_launches += 6;
  if ((e = cudaGetLastError()) != cudaSuccess) return c.cuda_fail(e, "hestimate setup");

  cudaEventRecord(c.ev_k0, s);
  if (mode == 0) {
    k_conv_range<1><<<slots, CONV_TB, 0, s>>>(dcols, nc, dbase, dst, tsum);
    k_conv_reduce<<<nc, 256, 0, s>>>(dcols, tsum, csum);
    k_conv_single_out<<<(nc + 63) / 64, 64, 0, s>>>(dst, nc, csum, dconv);
    c.stats.kernel_launches += 3;
    if ((e = cudaGetLastError()) != cudaSuccess) return c.cuda_fail(e, "convolution kernel");
  } else {
    // The level loop (at most 20 levels; 8 for every finite h0 > 0) runs as
    // one captured CUDA graph of conv -> reduce -> decide per level.
    const int max_levels = 9 - (mode == 2 ? std::min(skip, 8) : 0);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return c.cuda_fail(e, "begin capture");
    for (int L = 0; L < max_levels; ++L) {
      k_conv_range<2><<<slots, CONV_TB, 0, s>>>(dcols, nc, dbase, dst, tsum);
      k_conv_reduce<<<nc, 256, 0, s>>>(dcols, tsum, csum);
      k_hest_level<<<(nc + 63) / 64, 64, 0, s>>>(dst, nc, csum, dconv + 2 * (size_t)nc * L);
    }
    e = cudaStreamEndCapture(s, &graph);
    if (e != cudaSuccess) return c.cuda_fail(e, "end capture");
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(graph);
      return c.cuda_fail(e, "graph instantiate");
    }
    e = cudaGraphLaunch(exec, s);
    cudaStreamSynchronize(s);
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return c.cuda_fail(e, "graph launch");
    c.stats.kernel_launches += 3 * max_levels;
  }
  cudaEventRecord(c.ev_k1, s);
  c.ran_k = true;

  std::vector<HestState> hs(nc);
  e = cudaMemcpyAsync(hs.data(), dst, sizeof(HestState) * nc, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return c.cuda_fail(e, "read search state");
  if (mode == 0 && conv_out) {
    e = cudaMemcpyAsync(conv_out, dconv, 4 * (size_t)nc, cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return c.cuda_fail(e, "read convolution");
  }
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return c.cuda_fail(e, "hestimate");
  if (mode != 0) {
    std::vector<uint32_t> redo;
    for (uint32_t i = 0; i < nc; ++i) {
      if (!hs[i].done) return c.fail(ENT_ERR_STATE, "bandwidth search did not finish");
      h_out[i] = hs[i].result;
      if (stats) {
        stats[i].h0 = hs[i].h0;
        stats[i].conv_evals = (uint32_t)hs[i].n_conv;
        stats[i].levels_skipped = mode == 2 ? (uint32_t)skip : 0u;
        stats[i].warm_converged = mode == 2 ? (uint32_t)hs[i].converged : 0u;
      }
      if (mode == 2 && !hs[i].converged) redo.push_back(i);
    }
    if (!redo.empty()) {
      // fall back to the full search for the columns the warm start missed
      std::vector<uint64_t> off2;
      std::vector<uint32_t> len2;
      for (uint32_t i : redo) {
        off2.push_back(raw_off[i]);
        len2.push_back(lens[i]);
      }
      std::vector<float> h2(redo.size());
      std::vector<ent_hest_stats> st2(redo.size());
      int r2 = hestimate_pass(c, raw, off2, len2, 1, nullptr, 0, h2.data(), nullptr,
                              st2.data(), nullptr);
      if (r2) return r2;
      for (size_t q = 0; q < redo.size(); ++q) {
        h_out[redo[q]] = h2[q];
        if (stats) stats[redo[q]].conv_evals += st2[q].conv_evals;
      }
    }
  }
  return ENT_OK;
}

// Columns of one pass: the per-column kernels index columns by the grid's y
// dimension. Device bytes per point of a column in a pass (its sort keys and
// order with their ping-pong buffers, the sorted copy, the FP64 prefix sums)
// and per column (search state, tile sums, convolution values).
constexpr uint32_t kHestMaxCols = 65535;
constexpr size_t kHestBytesPerPoint = 28;
constexpr size_t kHestBytesPerCol = 1024;

}  // namespace

// A search over more columns than one pass takes, or than the device's free
// memory holds at once, runs as consecutive passes over groups of columns,
// the workspace rewound after each (every pass ends synchronised).
int hestimate_engine(Ctx& c, const float* raw, const std::vector<uint64_t>& raw_off,
                     const std::vector<uint32_t>& lens, int mode, const float* h_fixed_or_init,
                     int skip, float* h_out, float* conv_out, ent_hest_stats* stats,
                     const float* d_log_ratio) {
  const size_t nc = lens.size();
  size_t est = 0;
  for (uint32_t n : lens) est += kHestBytesPerPoint * n + kHestBytesPerCol;
  size_t budget = SIZE_MAX;
  if (nc > kHestMaxCols || est > c.arena.spare()) budget = device_budget(c);
  if (nc <= kHestMaxCols && est <= budget)
    return hestimate_pass(c, raw, raw_off, lens, mode, h_fixed_or_init, skip, h_out, conv_out,
                          stats, d_log_ratio);
  const Arena::Mark base = c.arena.mark();
  for (size_t q0 = 0; q0 < nc;) {
    size_t q = q0, bytes = 0;
    for (; q < nc; ++q) {
      const size_t add = kHestBytesPerPoint * lens[q] + kHestBytesPerCol;
      if (q > q0 && (bytes + add > budget || q - q0 >= kHestMaxCols)) break;
      bytes += add;
    }
    const std::vector<uint64_t> off(raw_off.begin() + (std::ptrdiff_t)q0,
                                    raw_off.begin() + (std::ptrdiff_t)q);
    const std::vector<uint32_t> len(lens.begin() + (std::ptrdiff_t)q0,
                                    lens.begin() + (std::ptrdiff_t)q);
    int s = hestimate_pass(c, raw, off, len, mode, h_fixed_or_init ? h_fixed_or_init + q0 : nullptr,
                           skip, h_out + q0, conv_out ? conv_out + q0 : nullptr,
                           stats ? stats + q0 : nullptr, d_log_ratio ? d_log_ratio + q0 : nullptr);
    if (s) return s;
    const cudaError_t e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return c.cuda_fail(e, "hestimate");
    c.collect_kernel_stats();
    c.arena.rewind(base);
    q0 = q;
  }
  return ENT_OK;
}

static int hest_common(ent_ctx* ctx, const float* coords, size_t n_rows, size_t n_cols,
                       const uint32_t* cols, size_t n_sel, uint32_t mode, const float* h_init,
                       uint32_t skip, float* h_out, ent_hest_stats* stats, bool device_in) {
  if (!ctx) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  if (!coords || !h_out || n_sel == 0) return c.fail(ENT_ERR_ARG, "null argument");
  if (mode > ENT_HEST_AMISE_WARM) return c.fail(ENT_ERR_ARG, "unknown hestimate mode");
  if (mode == ENT_HEST_AMISE_WARM && !h_init) return c.fail(ENT_ERR_ARG, "warm start needs h_init");
  if (n_rows < 2 || n_rows > 0xffffff00ull) return c.fail(ENT_ERR_ARG, "bad row count");
  std::vector<uint64_t> off(n_sel);
  std::vector<uint32_t> lens(n_sel, (uint32_t)n_rows);
  const float* raw = coords;
  for (size_t q = 0; q < n_sel; ++q) {
    const uint32_t col = cols ? cols[q] : (uint32_t)q;
    if (col >= n_cols) return c.fail(ENT_ERR_ARG, "column index out of range");
    off[q] = (uint64_t)col * n_rows;
  }
  if (!device_in) {
    float* p = static_cast<float*>(c.arena.alloc(4 * n_rows * n_sel));
    if (!p) return c.fail(ENT_ERR_CUDA, "out of device memory");
    for (size_t q = 0; q < n_sel; ++q) {
      cudaError_t e = cudaMemcpyAsync(p + q * n_rows, coords + off[q], 4 * n_rows,
                                      cudaMemcpyHostToDevice, c.stream);
      if (e != cudaSuccess) return c.cuda_fail(e, "copy coordinates");
      off[q] = q * n_rows;
    }
    raw = p;
  }
  if (mode == ENT_HEST_THUMB) {
    // h0 only: a zero-level search reports it
    std::vector<float> dummy(n_sel);
    std::vector<ent_hest_stats> st(n_sel);
    s = hestimate_engine(c, raw, off, lens, 2, h_out, 64, dummy.data(), nullptr, st.data(),
                         nullptr);
    if (s) return s;
    for (size_t q = 0; q < n_sel; ++q) {
      h_out[q] = st[q].h0;
      if (stats) {
        stats[q] = st[q];
        stats[q].conv_evals = 0;
      }
    }
  } else {
    s = hestimate_engine(c, raw, off, lens, (int)mode, h_init, (int)skip, h_out, nullptr, stats,
                         nullptr);
    if (s) return s;
  }
  s = c.end_call();
  c.collect_kernel_stats();
  return s;
}

extern "C" {

int ent_epa_convolution(ent_ctx* ctx, const float* sorted, size_t n, float h, float* out) {
  if (!ctx) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  if (!sorted || !out || n == 0) return c.fail(ENT_ERR_ARG, "null argument");
  if (!(h > 0.f) || !std::isfinite(h)) return c.fail(ENT_ERR_ARG, "bandwidth must be finite and positive");
  if (n > 0xffffff00ull) return c.fail(ENT_ERR_TOO_LARGE, "too many rows");
  float* p = static_cast<float*>(c.arena.alloc(4 * n));
  if (!p) return c.fail(ENT_ERR_CUDA, "out of device memory");
  cudaError_t e = cudaMemcpyAsync(p, sorted, 4 * n, cudaMemcpyHostToDevice, c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "copy coordinates");
  std::vector<uint64_t> off(1, 0);
  std::vector<uint32_t> lens(1, (uint32_t)n);
  float hv = h, dummy = 0.f;
  s = hestimate_engine(c, p, off, lens, 0, &hv, 0, &dummy, out, nullptr, nullptr);
  if (s) return s;
  s = c.end_call();
  c.collect_kernel_stats();
  return s;
}

int ent_hestimate(ent_ctx* ctx, const float* coords, size_t n_rows, size_t n_cols,
                  const uint32_t* cols, size_t n_sel, uint32_t mode, const float* h_init,
                  uint32_t skip_levels, float* h_out, ent_hest_stats* stats) {
  return hest_common(ctx, coords, n_rows, n_cols, cols, n_sel, mode, h_init, skip_levels,
                     h_out, stats, false);
}

int ent_hestimate_device(ent_ctx* ctx, const float* d_coords, size_t n_rows, size_t n_cols,
                         const uint32_t* cols, size_t n_sel, uint32_t mode,
                         const float* h_init, uint32_t skip_levels, float* h_out,
                         ent_hest_stats* stats) {
  return hest_common(ctx, d_coords, n_rows, n_cols, cols, n_sel, mode, h_init, skip_levels,
                     h_out, stats, true);
}

// Bandwidth search over every dimension of uneven instances: the full AMISE
// search (net == nullptr) or the learned warm start.
static int hest_instances(ent_ctx* ctx, ent_mlp* net, const ent_instance* inst, size_t n_inst,
                          uint32_t flags, uint32_t skip_levels, float* h_out,
                          ent_hest_stats* stats) {
  if (!ctx || !inst || !h_out || n_inst == 0) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  const bool dev = (flags & ENT_BATCH_DEVICE_INPUT) != 0;
  std::vector<const float*> base(n_inst);
  std::vector<uint32_t> nn(n_inst), dd(n_inst);
  std::vector<uint64_t> off;
  std::vector<uint32_t> lens;
  std::vector<uint32_t> col_inst, col_dim;
  // all instance dimensions are columns of one device buffer region each
  const float* raw0 = nullptr;
  for (size_t q = 0; q < n_inst; ++q) {
    if (inst[q].d < 1 || inst[q].d > 3) return c.fail(ENT_ERR_DIM, ent_status_string(ENT_ERR_DIM));
    if (inst[q].n < 2 || inst[q].n > 0xffffff00ull) return c.fail(ENT_ERR_ARG, "bad size");
    const float* p = inst[q].coords;
    if (!dev) {
      float* d = static_cast<float*>(c.arena.alloc(4 * inst[q].n * inst[q].d));
      if (!d) return c.fail(ENT_ERR_CUDA, "out of device memory");
      cudaError_t e = cudaMemcpyAsync(d, inst[q].coords, 4 * inst[q].n * inst[q].d,
                                      cudaMemcpyHostToDevice, c.stream);
      if (e != cudaSuccess) return c.cuda_fail(e, "copy coordinates");
      p = d;
    }
    base[q] = p;
    nn[q] = (uint32_t)inst[q].n;
    dd[q] = inst[q].d;
  }
  // offsets relative to the lowest address so one raw pointer covers all
  raw0 = *std::min_element(base.begin(), base.end());
  for (size_t q = 0; q < n_inst; ++q)
    for (uint32_t j = 0; j < dd[q]; ++j) {
      off.push_back((uint64_t)(base[q] - raw0) + (uint64_t)j * nn[q]);
      lens.push_back(nn[q]);
      col_inst.push_back((uint32_t)q);
      col_dim.push_back(j);
    }
  std::vector<float> hc(lens.size());
  std::vector<ent_hest_stats> sc(lens.size());
  if (net) {
    float* df = static_cast<float*>(c.arena.alloc(4 * 32 * n_inst));
    float* dy = static_cast<float*>(c.arena.alloc(4 * 3 * n_inst));
    float* dr = static_cast<float*>(c.arena.alloc(4 * lens.size()));
    if (!df || !dy || !dr) return c.fail(ENT_ERR_CUDA, "out of device memory");
    s = mlp_features_device(c, base, nn, dd, df);
    if (s) return s;
    s = mlp_forward_device(c, net, df, n_inst, dy);
    if (s) return s;
    // per column: r = y[inst][dim]
    std::vector<uint32_t> map(lens.size());
    for (size_t k = 0; k < lens.size(); ++k) map[k] = col_inst[k] * 3 + col_dim[k];
    cudaError_t e;
    uint32_t* dmap = upload(c, map, &e);
    if (e != cudaSuccess) return c.cuda_fail(e, "upload map");
    k_pick<<<(unsigned)((lens.size() + 127) / 128), 128, 0, c.stream>>>(dy, dmap, dr,
                                                                       (uint32_t)lens.size());
    c.stats.kernel_launches += 1;
    s = hestimate_engine(c, raw0, off, lens, 2, nullptr, (int)skip_levels, hc.data(), nullptr,
                         sc.data(), dr);
  } else {
    s = hestimate_engine(c, raw0, off, lens, 1, nullptr, 0, hc.data(), nullptr, sc.data(),
                         nullptr);
  }
  if (s) return s;
  for (size_t q = 0; q < n_inst; ++q)
    for (int j = 0; j < 3; ++j) h_out[3 * q + j] = 0.f;
  for (size_t k = 0; k < lens.size(); ++k) {
    h_out[3 * col_inst[k] + col_dim[k]] = hc[k];
    if (stats) stats[3 * col_inst[k] + col_dim[k]] = sc[k];
  }
  s = c.end_call();
  c.collect_kernel_stats();
  return s;
}

int ent_hestimate_learned(ent_ctx* ctx, ent_mlp* net, const ent_instance* inst, size_t n_inst,
                          uint32_t flags, uint32_t skip_levels, float* h_out,
                          ent_hest_stats* stats) {
  if (!net) return ENT_ERR_ARG;
  return hest_instances(ctx, net, inst, n_inst, flags, skip_levels, h_out, stats);
}

int ent_hestimate_batch(ent_ctx* ctx, const ent_instance* inst, size_t n_inst, uint32_t flags,
                        float* h_out, ent_hest_stats* stats) {
  return hest_instances(ctx, nullptr, inst, n_inst, flags, 0, h_out, stats);
}

}  // extern "C"
