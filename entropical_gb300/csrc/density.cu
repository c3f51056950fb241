// Product-Epanechnikov density sums on device-built cell lists (sm_103a).
//
// Replaces the reference density backends: the dense all-pairs CUDA kernels
// density_{1,2,3}d_krnl (density_1d.cuh:51-90, density_2d.cuh:57-100,
// density_3d.cuh:61-108) and the OpenMP window loops
// (densities_omp.cpp:33-159). For every target point t
//     S_t = sum_s prod_j max(0, g_j^2 - (y_tj - y_sj)^2),   y_j = x_j 2^k_j,
//     p_t = 0.75^d / (norm * prod_j h_j g_j^2) * S_t,
// with 2^k_j an exact power of two such that g_j = h_j 2^k_j lies in [1, 2).
// Since (y_t - y_s)/g = (x_t - x_s)/h exactly, this equals the reference's
// sum of 0.75 (1-u^2)/h products, and the coordinate differences carry the
// precision of the raw float data, as in the reference's (ref - val)/h.
//
// Cell lists ("strips"): points are sorted on dimension 0; dimensions 1..d-1
// are binned into cells of width h/S, and a stable partition by cell keeps
// dimension-0 order inside each strip. A target tile (up to TT consecutive
// points of one strip) then sees all of its in-support sources inside
// (2S+1)^(d-1) contiguous runs: one per neighbouring strip, clipped by
// binary search to [y0_first - g0, y0_last + g0]. This is the device form of
// the reference's sorted-window search boxes() (densities_omp.cpp:33-65) and
// of the cell boxes of Transs::BoxedSearch (boxedsearch.cpp:15-62).
//
// The pair kernel is a persistent CTA loop over an atomic work queue of
// tiles. Source runs are staged into shared memory in double-buffered chunks
// with cp.async.bulk (TMA bulk copies) completing on mbarriers; four warps
// each own R register-resident targets and stride the chunk with their 32
// lanes. The pair body is branchless FP32 on the CUDA cores using packed
// f32x2 sub/fma: for d = 2 one pair is sub.f32x2, fma.f32x2, 2 min, 1 fma.
// Per-lane chunk partials are folded into Kahan-compensated FP32 sums; the
// per-point scale, log and entropy sums are FP64.
#include <cfloat>

#include "engine.h"
#include "staging.cuh"

namespace ent {

namespace {

constexpr unsigned FULL = 0xffffffffu;

// ------------------------------------------------------------ column stats
__global__ void __launch_bounds__(1024)
    k_colstats(const ViewDev* __restrict__ views, ViewStats* __restrict__ stats) {
  __shared__ float smn[32], smx[32];
  __shared__ uint32_t sbad[32];
  const ViewDev v = views[blockIdx.x];
  float mn = FLT_MAX, mx = -FLT_MAX;
  uint32_t bad = 0;
  for (uint32_t i = threadIdx.x; i < v.n; i += blockDim.x) {
    const float f = v.x[i];
    if (!isfinite(f)) {
      bad = 1;
      continue;
    }
    mn = fminf(mn, f);
    mx = fmaxf(mx, f);
  }
  for (int o = 16; o; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(FULL, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(FULL, mx, o));
    bad |= __shfl_xor_sync(FULL, bad, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    smn[warp] = mn;
    smx[warp] = mx;
    sbad[warp] = bad;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    mn = lane < nw ? smn[lane] : FLT_MAX;
    mx = lane < nw ? smx[lane] : -FLT_MAX;
    bad = lane < nw ? sbad[lane] : 0u;
    for (int o = 16; o; o >>= 1) {
      mn = fminf(mn, __shfl_xor_sync(FULL, mn, o));
      mx = fmaxf(mx, __shfl_xor_sync(FULL, mx, o));
      bad |= __shfl_xor_sync(FULL, bad, o);
    }
    if (lane == 0) {
      ViewStats r;
      r.mn = mn;
      r.mx = mx;
      r.nonfinite = bad;
      r.pad = 0;
      stats[blockIdx.x] = r;
    }
  }
}

// ---------------------------------------------------------- sort keys
__global__ void k_view_keys(const ViewDev* __restrict__ views,
                            const uint64_t* __restrict__ view_off,
                            uint32_t* __restrict__ keys,
                            uint32_t* __restrict__ vals) {
  const ViewDev v = views[blockIdx.y];
  const uint64_t base = view_off[blockIdx.y];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < v.n;
       i += gridDim.x * blockDim.x) {
    keys[base + i] = float_key(v.x[i]);
    vals[base + i] = i;
  }
}

// Cell index in FP32 (the FP64 pipe of this GPU is slow): a = fl(fl(x - lo)
// inv_w) is within 3 2^-24 a of the exact (x - lo)/w, i.e. within 1.8e-7 ncell
// cells; the host widens the cells by at least 6e-7 ncell / S so that two
// points within h never land more than S cells apart. x >= lo (the view's
// minimum), so a >= 0 and truncation is floor.
__device__ __forceinline__ uint32_t cell_of(float x, float lo, float inv_w, uint32_t ncell) {
  const float a = __fmul_rn(__fsub_rn(x, lo), inv_w);
  if (!(a < (float)ncell)) return ncell - 1;
  return a > 0.f ? (uint32_t)a : 0u;
}

// Four points per thread per step, their loads issued together (the
// coordinate reads are gathers through the sorted order).
constexpr uint32_t CL_ITEMS = 4;

__global__ void k_strip_keys(const InstDev* __restrict__ insts,
                             const uint32_t* __restrict__ inst_ids,
                             const uint64_t* __restrict__ seg_off,
                             uint32_t* __restrict__ keys,
                             uint32_t* __restrict__ vals) {
  const InstDev& I = insts[inst_ids[blockIdx.y]];
  const uint64_t base = seg_off[blockIdx.y];
  const uint32_t n = I.n, stride = gridDim.x * blockDim.x;
  const uint32_t* __restrict__ perm0 = I.perm0;
  const float* __restrict__ x1 = I.x[1];
  const float* __restrict__ x2 = I.x[2];
  for (uint32_t k0 = blockIdx.x * blockDim.x + threadIdx.x; k0 < n; k0 += CL_ITEMS * stride) {
    uint32_t j[CL_ITEMS];
    float a[CL_ITEMS], b[CL_ITEMS];
#pragma unroll
    for (uint32_t u = 0; u < CL_ITEMS; ++u) {
      const uint32_t k = k0 + u * stride;
      j[u] = k < n ? perm0[k] : 0u;
    }
#pragma unroll
    for (uint32_t u = 0; u < CL_ITEMS; ++u) {
      const uint32_t k = k0 + u * stride;
      a[u] = k < n ? x1[j[u]] : 0.f;
      b[u] = (k < n && I.d == 3) ? x2[j[u]] : 0.f;
    }
#pragma unroll
    for (uint32_t u = 0; u < CL_ITEMS; ++u) {
      const uint32_t k = k0 + u * stride;
      if (k >= n) break;
      uint32_t key = cell_of(a[u], I.lo1, I.inv_w1, I.ncell1);
      if (I.d == 3) key = key * I.ncell2 + cell_of(b[u], I.lo2, I.inv_w2, I.ncell2);
      keys[base + k] = key;
      vals[base + k] = j[u];
    }
  }
}

// strip_start[s] = the first sorted position whose strip key is >= s, for
// s = 0 .. n_strips: one lower-bound search per strip (a few hundred strips
// per instance) instead of a pass over every point.
__global__ void k_strip_bounds(const InstDev* __restrict__ insts) {
  const InstDev& I = insts[blockIdx.y];
  const uint32_t n = I.n, L = I.n_strips;
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s <= L;
       s += gridDim.x * blockDim.x) {
    if (I.d == 1) {  // one strip
      I.strip_start[s] = s ? n : 0u;
      continue;
    }
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
      const uint32_t m = lo + ((hi - lo) >> 1);
      if (I.skeys[m] < s) lo = m + 1; else hi = m;
    }
    I.strip_start[s] = lo;
  }
}

// Exclusive scan of tiles-per-strip, one block per instance.
__global__ void __launch_bounds__(1024) k_tile_offsets(const InstDev* __restrict__ insts) {
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t carry_s;
  const InstDev& I = insts[blockIdx.x];
  const uint32_t L = I.n_strips;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  for (uint32_t base = 0; base < L; base += 1024) {
    const uint32_t i = base + threadIdx.x;
    uint32_t v = 0;
    if (i < L) {
      const uint32_t len = I.strip_start[i + 1] - I.strip_start[i];
      v = (len + I.tt - 1) / I.tt;
    }
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(FULL, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = warp_tot[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, w, o);
        if (lane >= o) w += y;
      }
      warp_tot[lane] = w;
    }
    __syncthreads();
    const uint32_t carry = carry_s;
    if (i < L) I.tile_off[i] = carry + (warp ? warp_tot[warp - 1] : 0u) + x - v;
    __syncthreads();
    if (threadIdx.x == 0) carry_s = carry + warp_tot[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) I.tile_off[L] = carry_s;
}

__global__ void k_gather_pts(const InstDev* __restrict__ insts) {
  const InstDev& I = insts[blockIdx.y];
  const uint32_t n = I.n, stride = gridDim.x * blockDim.x;
  const int d = (int)I.d;
  const uint32_t* __restrict__ perm = I.perm;
  for (uint32_t k0 = blockIdx.x * blockDim.x + threadIdx.x; k0 < n; k0 += CL_ITEMS * stride) {
    uint32_t j[CL_ITEMS];
    float v[CL_ITEMS][3];
#pragma unroll
    for (uint32_t u = 0; u < CL_ITEMS; ++u) {
      const uint32_t k = k0 + u * stride;
      j[u] = k < n ? perm[k] : 0u;
    }
#pragma unroll
    for (uint32_t u = 0; u < CL_ITEMS; ++u) {
      const bool in = k0 + u * stride < n;
#pragma unroll
      for (int c = 0; c < 3; ++c) v[u][c] = (in && c < d) ? I.x[c][j[u]] : 0.f;
    }
#pragma unroll
    for (uint32_t u = 0; u < CL_ITEMS; ++u) {
      const uint32_t k = k0 + u * stride;
      if (k >= n) break;
      // multiplication by a power of two is exact
      const float y0 = v[u][0] * I.sc[0];
      if (d == 1) {
        reinterpret_cast<float*>(I.pts)[k] = y0;
      } else if (d == 2) {
        reinterpret_cast<float2*>(I.pts)[k] = make_float2(y0, v[u][1] * I.sc[1]);
      } else {
        reinterpret_cast<float4*>(I.pts)[k] =
            make_float4(y0, v[u][1] * I.sc[1], v[u][2] * I.sc[2], 0.f);
      }
    }
  }
}

// ------------------------------------------------------------- tile plan
__device__ __forceinline__ float y0_at(const void* pts, int d, uint32_t k) {
  if (d == 1) return reinterpret_cast<const float*>(pts)[k];
  if (d == 2) return reinterpret_cast<const float2*>(pts)[k].x;
  return reinterpret_cast<const float4*>(pts)[k].x;
}

// first k in [a, b) with y0(k) >= v
__device__ uint32_t lower_y(const void* pts, int d, uint32_t a, uint32_t b, float v) {
  while (a < b) {
    const uint32_t m = a + (b - a) / 2;
    if (y0_at(pts, d, m) < v) a = m + 1; else b = m;
  }
  return a;
}
// first k in [a, b) with y0(k) > v
__device__ uint32_t upper_y(const void* pts, int d, uint32_t a, uint32_t b, float v) {
  while (a < b) {
    const uint32_t m = a + (b - a) / 2;
    if (y0_at(pts, d, m) <= v) a = m + 1; else b = m;
  }
  return a;
}

// The plan of slot g: its tile descriptor; returns the slot's candidate
// pairs (sources x targets) and its dimension in *d_out (left 0 for an empty
// slot).
__device__ __forceinline__ unsigned long long plan_slot(const InstDev* __restrict__ insts,
                                                        uint32_t n_inst,
                                                        const uint32_t* __restrict__ inst_tile_base,
                                                        TileDesc* __restrict__ tiles, uint32_t g,
                                                        int* d_out) {
  uint32_t lo = 0, hi = n_inst;
  while (hi - lo > 1) {
    const uint32_t m = (lo + hi) / 2;
    if (inst_tile_base[m] <= g) lo = m; else hi = m;
  }
  const InstDev& I = insts[lo];
  TileDesc td;
  td.inst = lo;
  td.t_begin = 0;
  td.t_count = 0;
  td.n_runs = 0;
  td.pad = 0;
  // slot -> (tile, share of its sources)
  const uint32_t parts = max(I.parts, 1u);
  const uint32_t t = (g - I.tile_base) / parts;
  td.part = (g - I.tile_base) % parts;
  const uint32_t total = I.tile_off[I.n_strips];
  if (t >= total) {
    tiles[g] = td;
    return 0ull;
  }
  uint32_t a = 0, b = I.n_strips;
  while (b - a > 1) {
    const uint32_t m = (a + b) / 2;
    if (I.tile_off[m] <= t) a = m; else b = m;
  }
  const uint32_t s = a;
  const int d = (int)I.d;
  // the tile's targets, clipped to the instance's share [t_lo, t_hi)
  const uint32_t tb0 = I.strip_start[s] + (t - I.tile_off[s]) * I.tt;
  const uint32_t te0 = min(tb0 + I.tt, I.strip_start[s + 1]);
  const uint32_t tb = max(tb0, I.t_lo), te = min(te0, I.t_hi);
  if (te <= tb) {  // outside the share
    tiles[g] = td;
    return 0ull;
  }
  const uint32_t tc = te - tb;
  const float yf = y0_at(I.pts, d, tb);
  const float yl = y0_at(I.pts, d, tb + tc - 1);
  // half-width g0 = sqrt(g0^2), widened so that rounding can only add
  // candidates (an out-of-support candidate contributes exactly 0)
  const float g0 = sqrtf(I.g2[0]);
  const float eps = 1e-5f * (g0 + fmaxf(fabsf(yf), fabsf(yl)));
  const float vlo = yf - g0 - eps, vhi = yl + g0 + eps;
  td.t_begin = tb;
  td.t_count = tc;
  uint32_t nr = 0;
  unsigned long long nsrc = 0;
  auto add_strip = [&](uint32_t sp) {
    const uint32_t a0 = I.strip_start[sp], b0 = I.strip_start[sp + 1];
    if (a0 == b0) return;
    // symmetric mode: sources before the tile's first target are skipped
    // (their tiles evaluate those pairs)
    if (I.sym && b0 <= tb) return;
    uint32_t l = lower_y(I.pts, d, a0, b0, vlo);
    if (I.sym) l = max(l, tb);
    const uint32_t h = upper_y(I.pts, d, l, b0, vhi);
    if (h <= l) return;
    if (nr > 0 && td.lo[nr - 1] + td.len[nr - 1] == l) {
      td.len[nr - 1] += h - l;
    } else {
      td.lo[nr] = l;
      td.len[nr] = h - l;
      ++nr;
    }
    nsrc += h - l;
  };
  if (d == 1) {
    add_strip(0);
  } else if (d == 2) {
    const int S = (int)I.S;
    const int c1 = (int)s;
    if (I.fused) {
      // strip moments: the tile's only run is the strip S above it, where
      // the y edge of its targets' support falls (the one S below is the run
      // of that strip's own tiles, so each edge pair is evaluated once)
      if (c1 + S < (int)I.ncell1) add_strip((uint32_t)(c1 + S));
    } else {
      for (int c = max(0, c1 - S); c <= min((int)I.ncell1 - 1, c1 + S); ++c)
        add_strip((uint32_t)c);
    }
  } else {
    const int S = (int)I.S, S2 = (int)I.S2;
    const int c1 = (int)(s / I.ncell2), c2 = (int)(s % I.ncell2);
    for (int u = max(0, c1 - S); u <= min((int)I.ncell1 - 1, c1 + S); ++u)
      for (int v = max(0, c2 - S2); v <= min((int)I.ncell2 - 1, c2 + S2); ++v)
        add_strip((uint32_t)u * I.ncell2 + (uint32_t)v);
  }
  td.n_runs = nr;
  if (parts > 1) {
    // this slot's share [a, b) of the concatenated source runs (symmetric
    // kernel only: its target sums are atomic, so shares may run anywhere)
    const unsigned long long a = nsrc * td.part / parts, b = nsrc * (td.part + 1) / parts;
    unsigned long long pre = 0;
    uint32_t n2 = 0;
    for (uint32_t r = 0; r < nr; ++r) {
      const uint32_t rlo = td.lo[r], rlen = td.len[r];  // before n2 <= r overwrites
      const unsigned long long s0 = max(a, pre), s1 = min(b, pre + rlen);
      if (s1 > s0) {
        td.lo[n2] = rlo + (uint32_t)(s0 - pre);
        td.len[n2] = (uint32_t)(s1 - s0);
        ++n2;
      }
      pre += rlen;
    }
    td.n_runs = n2;
    nsrc = b - a;
  }
  tiles[g] = td;
  *d_out = d;
  return nsrc * (unsigned long long)tc;
}

// One thread per slot. The candidate-pair totals are summed per warp and
// dimension first: one atomic per warp, not one per slot on one address.
__global__ void k_plan(const InstDev* __restrict__ insts, uint32_t n_inst,
                       const uint32_t* __restrict__ inst_tile_base,
                       TileDesc* __restrict__ tiles, uint32_t n_slots,
                       unsigned long long* __restrict__ n_src_total) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  int d = 0;
  const unsigned long long c =
      g < n_slots ? plan_slot(insts, n_inst, inst_tile_base, tiles, g, &d) : 0ull;
  if (!n_src_total) return;  // grid-uniform
  for (int dd = 1; dd <= 3; ++dd) {
    unsigned long long v = d == dd ? c : 0ull;
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(n_src_total + (dd - 1), v);
  }
}

// ------------------------------------------------------- pair kernel
// Pair-body variants V: 0 min-based; 1 saturating FMA; 2 saturating FMA at
// 5 resident CTAs per SM; 3 as 2 with 1.5x larger staged chunks. (The
// symmetric bodies PAIR_SYM and PAIR_SYM + 1 are k_density_sym,
// density_sym.cu.)
template <int V>
struct VariantTraits {
  static constexpr int MINB = V >= 2 ? 5 : 1;
  static constexpr int CHX_D1 = V == 3 ? 6144 : 0;
  static constexpr int CHX_D2 = V == 3 ? 3072 : 0;
  static constexpr int CHX_D3 = V == 3 ? 1536 : 0;
};

template <int D, int V>
__host__ __device__ constexpr int chunk_of() {
  return D == 1 ? VariantTraits<V>::CHX_D1
                : (D == 2 ? VariantTraits<V>::CHX_D2 : VariantTraits<V>::CHX_D3);
}

template <int D, int R, int V>
__global__ void __launch_bounds__(128, VariantTraits<V>::MINB)
    k_density(const TileDesc* __restrict__ tiles, uint32_t n_slots,
              const InstDev* __restrict__ insts, uint32_t* work_counter,
              uint32_t* err, double* tile_logsum, uint32_t mode) {
  typedef Cfg<D, R, chunk_of<D, V>()> C;
  typedef typename C::P P;
  extern __shared__ __align__(128) unsigned char dsm[];
  P* bufs = reinterpret_cast<P*>(dsm);
  __shared__ __align__(8) uint64_t full[2];
  __shared__ Piece ptab[2][C::MAXP];
  __shared__ uint32_t npc[2];
  __shared__ uint32_t run_lo[MAX_RUNS], run_pre[MAX_RUNS + 1];
  __shared__ uint32_t s_g, s_nr, s_tb, s_tc, s_inst;
  __shared__ double s_lsum[C::NW];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  uint32_t q = 0;

  for (;;) {
    if (tid == 0) {
      const uint32_t g = atomicAdd(work_counter, 1u);
      s_g = g;
      if (g < n_slots) {
        const TileDesc* T = tiles + g;
        const uint32_t nr = T->n_runs;
        s_tb = T->t_begin;
        s_tc = T->t_count;
        s_inst = T->inst;
        s_nr = nr;
        run_pre[0] = 0;
        for (uint32_t r = 0; r < nr; ++r) {
          run_lo[r] = T->lo[r];
          run_pre[r + 1] = run_pre[r] + T->len[r];
        }
      }
    }
    __syncthreads();
    const uint32_t g = s_g;
    if (g >= n_slots) break;
    const uint32_t tc = s_tc;
    if (tc == 0) {
      if (tid == 0 && (mode & (DM_LOGSUM | DM_SUMV))) tile_logsum[g] = 0.0;
      __syncthreads();
      continue;
    }
    const InstDev* I = insts + s_inst;
    const P* __restrict__ pts = reinterpret_cast<const P*>(I->pts);
    const uint32_t nr = s_nr, nsrc = run_pre[nr], tb = s_tb;
    // -g^2 per dimension: v = d^2 - g^2 <= 0 inside the support
    const float ng0 = -I->g2[0], ng1 = -I->g2[D > 1 ? 1 : 0], ng2 = -I->g2[D > 2 ? 2 : 0];
    const f32x2 M1 = (D == 1) ? pk2(ng0, ng0) : pk2(ng0, ng1);
    const uint32_t nch = (nsrc + C::CH - 1) / C::CH;
    if (tid == 0 && nch > 0)
      issue_chunk<C>(0, q & 1u, nsrc, nr, run_lo, run_pre, pts, bufs, ptab, npc, full);

    // Register-resident targets of this warp; missing ones sit far away.
    float ks[R], kc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      ks[r] = 0.f;
      kc[r] = 0.f;
    }
    const float FAR = __int_as_float(0x7f800000);  // +inf: every term is 0
    f32x2 T01[R];
    float T2[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const uint32_t li = warp * R + r;
      P p;
      if (li < tc) {
        p = pts[tb + li];
      } else {
        if constexpr (D == 1) p = FAR;
        else if constexpr (D == 2) p = make_float2(FAR, FAR);
        else p = make_float4(FAR, FAR, FAR, 0.f);
      }
      if constexpr (D == 1) {
        T2[r] = p;
      } else if constexpr (D == 2) {
        T01[r] = pk2(p.x, p.y);
      } else {
        T01[r] = pk2(p.x, p.y);
        T2[r] = p.z;
      }
    }

    bool aborted = false;
    uint32_t ab_q = 0;
    bool ab_next = false;
    for (uint32_t c = 0; c < nch; ++c) {
      const uint32_t qq = q + c, b = qq & 1u;
      if (tid == 0 && c + 1 < nch)
        issue_chunk<C>(c + 1, (qq + 1) & 1u, nsrc, nr, run_lo, run_pre, pts, bufs, ptab,
                       npc, full);
      const bool ok = mbar_wait(&full[b], (qq >> 1) & 1u);
      if (ok) {
        const P* B = bufs + (size_t)b * C::CAP;
        const uint32_t np = npc[b];
        for (uint32_t pi = 0; pi < np; ++pi) {
          const uint32_t s0 = ptab[b][pi].s0, n = ptab[b][pi].n;
          if (mode & DM_COUNT) {
            // Same support test as the sum loops: fma(d, d, -1) <= 0 per dim.
            float acc[R];
#pragma unroll
            for (int r = 0; r < R; ++r) acc[r] = 0.f;
            for (uint32_t k = lane; k < n; k += 32) {
              const P s = B[s0 + k];
#pragma unroll
              for (int r = 0; r < R; ++r) {
                bool in;
                if constexpr (D == 1) {
                  const float dd = __fsub_rn(T2[r], s);
                  in = fmaf(dd, dd, ng0) <= 0.f;
                } else {
                  float tx, ty;
                  upk2(T01[r], tx, ty);
                  const float dx = __fsub_rn(tx, s.x), dy = __fsub_rn(ty, s.y);
                  in = fmaf(dx, dx, ng0) <= 0.f && fmaf(dy, dy, ng1) <= 0.f;
                  if constexpr (D == 3) {
                    const float dz = __fsub_rn(T2[r], s.z);
                    in = in && fmaf(dz, dz, ng2) <= 0.f;
                  }
                }
                acc[r] += in ? 1.f : 0.f;
              }
            }
#pragma unroll
            for (int r = 0; r < R; ++r) kahan_add(ks[r], kc[r], acc[r]);
          } else if constexpr (V >= 1) {
            // saturating body: (g^2 - d^2)^+ = sat(fma(-d, d, g^2)) because
            // g^2 < 1; all work on the FMA pipe, no min on the ALU
            const float g2a = -ng0, g2b = -ng1, g2c = -ng2;
            if constexpr (D == 1) {
              f32x2 acc[R / 2];
              f32x2 T[R / 2];
#pragma unroll
              for (int i = 0; i < R / 2; ++i) {
                acc[i] = pk2(0.f, 0.f);
                T[i] = pk2(T2[2 * i], T2[2 * i + 1]);
              }
#pragma unroll 2
              for (uint32_t k = lane; k < n; k += 32) {
                const float s = B[s0 + k];
                const f32x2 S = pk2(s, s);
#pragma unroll
                for (int i = 0; i < R / 2; ++i) {
                  float da, db;
                  upk2(sub2(T[i], S), da, db);
                  acc[i] = add2(acc[i], pk2(__saturatef(__fmaf_rn(-da, da, g2a)),
                                            __saturatef(__fmaf_rn(-db, db, g2a))));
                }
              }
#pragma unroll
              for (int i = 0; i < R / 2; ++i) {
                float a0, a1;
                upk2(acc[i], a0, a1);
                kahan_add(ks[2 * i], kc[2 * i], a0);
                kahan_add(ks[2 * i + 1], kc[2 * i + 1], a1);
              }
            } else {
              float acc[R];
#pragma unroll
              for (int r = 0; r < R; ++r) acc[r] = 0.f;
#pragma unroll 2
              for (uint32_t k = lane; k < n; k += 32) {
                const P s = B[s0 + k];
                const f32x2 S = pk2(s.x, s.y);
#pragma unroll
                for (int r = 0; r < R; ++r) {
                  float dx, dy;
                  upk2(sub2(T01[r], S), dx, dy);
                  const float wx = __saturatef(__fmaf_rn(-dx, dx, g2a));
                  const float wy = __saturatef(__fmaf_rn(-dy, dy, g2b));
                  if constexpr (D == 2) {
                    acc[r] = __fmaf_rn(wx, wy, acc[r]);
                  } else {
                    const float dz = T2[r] - s.z;
                    const float wz = __saturatef(__fmaf_rn(-dz, dz, g2c));
                    acc[r] = __fmaf_rn(wx * wy, wz, acc[r]);
                  }
                }
              }
#pragma unroll
              for (int r = 0; r < R; ++r) kahan_add(ks[r], kc[r], acc[r]);
            }
          } else if constexpr (D == 1) {
            f32x2 acc[R / 2];
            f32x2 T[R / 2];
#pragma unroll
            for (int i = 0; i < R / 2; ++i) {
              acc[i] = pk2(0.f, 0.f);
              T[i] = pk2(T2[2 * i], T2[2 * i + 1]);
            }
#pragma unroll 2
            for (uint32_t k = lane; k < n; k += 32) {
              const float s = B[s0 + k];
              const f32x2 S = pk2(s, s);
#pragma unroll
              for (int i = 0; i < R / 2; ++i) {
                const f32x2 dd = sub2(T[i], S);
                const f32x2 v = fma2(dd, dd, M1);
                float va, vb;
                upk2(v, va, vb);
                acc[i] = add2(acc[i], pk2(fminf(va, 0.f), fminf(vb, 0.f)));
              }
            }
#pragma unroll
            for (int i = 0; i < R / 2; ++i) {
              float a0, a1;
              upk2(acc[i], a0, a1);
              kahan_add(ks[2 * i], kc[2 * i], -a0);
              kahan_add(ks[2 * i + 1], kc[2 * i + 1], -a1);
            }
          } else if constexpr (D == 2) {
            float acc[R];
#pragma unroll
            for (int r = 0; r < R; ++r) acc[r] = 0.f;
#pragma unroll 2
            for (uint32_t k = lane; k < n; k += 32) {
              const float2 s = B[s0 + k];
              const f32x2 S = pk2(s.x, s.y);
#pragma unroll
              for (int r = 0; r < R; ++r) {
                const f32x2 dd = sub2(T01[r], S);
                const f32x2 v = fma2(dd, dd, M1);
                float vx, vy;
                upk2(v, vx, vy);
                acc[r] = fmaf(fminf(vx, 0.f), fminf(vy, 0.f), acc[r]);
              }
            }
#pragma unroll
            for (int r = 0; r < R; ++r) kahan_add(ks[r], kc[r], acc[r]);
          } else {
            float acc[R];
#pragma unroll
            for (int r = 0; r < R; ++r) acc[r] = 0.f;
#pragma unroll 2
            for (uint32_t k = lane; k < n; k += 32) {
              const float4 s = B[s0 + k];
              const f32x2 S = pk2(s.x, s.y);
#pragma unroll
              for (int r = 0; r < R; ++r) {
                const f32x2 dd = sub2(T01[r], S);
                const float dz = T2[r] - s.z;
                const f32x2 v = fma2(dd, dd, M1);
                const float vz = fmaf(dz, dz, ng2);
                float vx, vy;
                upk2(v, vx, vy);
                const float pxy = fminf(vx, 0.f) * fminf(vy, 0.f);
                acc[r] = fmaf(pxy, fminf(vz, 0.f), acc[r]);
              }
            }
#pragma unroll
            for (int r = 0; r < R; ++r) kahan_add(ks[r], kc[r], -acc[r]);
          }
        }
      }
      if (__syncthreads_or(!ok)) {
        aborted = true;
        ab_q = qq;
        ab_next = c + 1 < nch;
        break;
      }
    }
    if (aborted) {
      // Let any copy still in flight land before this CTA's shared memory
      // is released, then report and stop.
      if (tid == 0) {
        atomicOr(err, EF_TIMEOUT);
        mbar_wait(&full[ab_q & 1u], (ab_q >> 1) & 1u);
        if (ab_next) mbar_wait(&full[(ab_q + 1) & 1u], ((ab_q + 1) >> 1) & 1u);
      }
      __syncthreads();
      return;
    }
    q += nch;

    // Epilogue: combine lanes, scale in FP64, write / log-sum.
    float v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = ks[r] - kc[r];
    const float tot = warp_transpose_sum<R>(v, lane);
    const int tgt = lane >> (5 - Log2<R>::v);
    const bool writer = (lane & ((32 / R) - 1)) == 0;
    const uint32_t li = warp * R + tgt;
    double lsum = 0.0;
    if (writer && li < tc) {
      const double dens = I->scale * (double)tot;
      if (mode & DM_WRITE_F64) I->out[I->perm[tb + li]] = dens;
      if (mode & DM_LOGSUM) lsum = log(dens);
      else if (mode & DM_SUMV) lsum = dens;
    }
    if (mode & (DM_LOGSUM | DM_SUMV)) {
      for (int o = 16; o; o >>= 1) lsum += __shfl_xor_sync(FULL, lsum, o);
      if (lane == 0) s_lsum[warp] = lsum;
    }
    __syncthreads();
    if (tid == 0 && (mode & (DM_LOGSUM | DM_SUMV))) {
      double t = 0.0;
#pragma unroll
      for (int w = 0; w < C::NW; ++w) t += s_lsum[w];
      tile_logsum[g] = t;
    }
  }
}

template <int D, int R, int V>
cudaError_t launch_density_t(cudaStream_t st, const TileDesc* tiles,
                             uint32_t n_slots, const InstDev* insts,
                             uint32_t* work_counter, uint32_t* err,
                             double* tile_logsum, uint32_t mode, int n_sms,
                             int* launched) {
  typedef Cfg<D, R, chunk_of<D, V>()> C;
  auto kern = k_density<D, R, V>;
  cudaError_t e = cudaFuncSetAttribute(
      kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, C::NT,
                                                    C::SMEM);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  uint64_t grid = (uint64_t)per_sm * (uint64_t)n_sms;
  if (grid > n_slots) grid = n_slots;
  if (grid == 0) grid = 1;
  e = cudaMemsetAsync(work_counter, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  kern<<<(unsigned)grid, C::NT, C::SMEM, st>>>(tiles, n_slots, insts,
                                               work_counter, err, tile_logsum,
                                               mode);
  if (launched) *launched = (int)grid;
  return cudaGetLastError();
}

// Deterministic per-instance sum of the tile log-sums.
__global__ void __launch_bounds__(256)
    k_inst_logsum(const InstDev* __restrict__ insts,
                  const double* __restrict__ tile_logsum, double* out) {
  __shared__ double sw[8];
  const InstDev& I = insts[blockIdx.x];
  const uint32_t n = I.tile_cap;
  double a = 0.0;
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
    a += tile_logsum[I.tile_base + i];
  for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(FULL, a, o);
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += sw[w];
    out[blockIdx.x] = t;
  }
}

}  // namespace

// Targets per warp: the tunable variants of each dimension (tile = 4 warps).
int density_variant_supported(int d, int r, int v) {
  if (v == 0) return density_r_supported(d, r);
  if (pair_is_sym(v)) return d >= 1 && d <= 3;  // own tile shape, sym_tile_r
  if (v == PAIR_RANGE) return d == 1;            // range sums: tiles only finish
  if (v == PAIR_MOMENT) return d == 2;           // strip moments: the same
  return v >= 1 && v <= 3 && r == (d == 3 ? 8 : 16);
}

int density_r_supported(int d, int r) {
  if (d == 1 || d == 2) return r == 8 || r == 16;
  if (d == 3) return r == 4 || r == 8;
  return 0;
}

int density_tile_targets(int /*d*/, int r) { return 4 * r; }

cudaError_t launch_colstats(cudaStream_t st, const ViewDev* views,
                            uint32_t n_views, ViewStats* stats) {
  if (n_views == 0) return cudaSuccess;
  k_colstats<<<n_views, 1024, 0, st>>>(views, stats);
  return cudaGetLastError();
}

static unsigned grid_x_for(uint32_t max_n) {
  uint32_t g = (max_n + 255) / 256;
  if (g > 1024) g = 1024;
  return g ? g : 1;
}

cudaError_t launch_view_keys(cudaStream_t st, const ViewDev* views,
                             const uint64_t* view_off, uint32_t n_views,
                             uint32_t max_n, uint32_t* keys, uint32_t* vals) {
  if (n_views == 0) return cudaSuccess;
  k_view_keys<<<dim3(grid_x_for(max_n), n_views), 256, 0, st>>>(views, view_off,
                                                               keys, vals);
  return cudaGetLastError();
}

cudaError_t launch_strip_keys(cudaStream_t st, const InstDev* insts,
                              const uint32_t* inst_ids, const uint64_t* seg_off,
                              uint32_t n_seg, uint32_t max_n, uint32_t* keys,
                              uint32_t* vals) {
  if (n_seg == 0) return cudaSuccess;
  k_strip_keys<<<dim3(grid_x_for((max_n + CL_ITEMS - 1) / CL_ITEMS), n_seg), 256, 0, st>>>(
      insts, inst_ids, seg_off, keys, vals);
  return cudaGetLastError();
}

cudaError_t launch_strip_bounds(cudaStream_t st, const InstDev* insts,
                                uint32_t n_inst, uint32_t max_strips) {
  if (n_inst == 0) return cudaSuccess;
  k_strip_bounds<<<dim3(grid_x_for(max_strips + 1), n_inst), 256, 0, st>>>(insts);
  return cudaGetLastError();
}

cudaError_t launch_tile_offsets(cudaStream_t st, const InstDev* insts,
                                uint32_t n_inst) {
  if (n_inst == 0) return cudaSuccess;
  k_tile_offsets<<<n_inst, 1024, 0, st>>>(insts);
  return cudaGetLastError();
}

cudaError_t launch_gather_pts(cudaStream_t st, const InstDev* insts,
                              uint32_t n_inst, uint32_t max_n) {
  if (n_inst == 0) return cudaSuccess;
  k_gather_pts<<<dim3(grid_x_for((max_n + CL_ITEMS - 1) / CL_ITEMS), n_inst), 256, 0, st>>>(
      insts);
  return cudaGetLastError();
}

cudaError_t launch_plan(cudaStream_t st, const InstDev* insts, uint32_t n_inst,
                        const uint32_t* inst_tile_base, TileDesc* tiles,
                        uint32_t n_slots, uint64_t* n_src_total) {
  if (n_slots == 0) return cudaSuccess;
  k_plan<<<(n_slots + 127) / 128, 128, 0, st>>>(
      insts, n_inst, inst_tile_base, tiles, n_slots,
      reinterpret_cast<unsigned long long*>(n_src_total));
  return cudaGetLastError();
}

cudaError_t launch_density(cudaStream_t st, int d, int r, int v, const TileDesc* tiles,
                           uint32_t n_slots, const InstDev* insts,
                           uint32_t* work_counter, uint32_t* err,
                           double* tile_logsum, uint32_t mode, int n_sms,
                           int* launched) {
  if (pair_is_sym(v))
    return launch_density_sym(st, d, v, tiles, n_slots, insts, work_counter, err, n_sms,
                              launched);
#define ENT_LAUNCH(D, R, V)                                                         \
  if (d == D && r == R && v == V)                                                   \
    return launch_density_t<D, R, V>(st, tiles, n_slots, insts, work_counter, err,  \
                                     tile_logsum, mode, n_sms, launched);
  ENT_LAUNCH(1, 8, 0)
  ENT_LAUNCH(1, 16, 0)
  ENT_LAUNCH(1, 16, 1)
  ENT_LAUNCH(1, 16, 2)
  ENT_LAUNCH(1, 16, 3)
  ENT_LAUNCH(2, 8, 0)
  ENT_LAUNCH(2, 16, 0)
  ENT_LAUNCH(2, 16, 1)
  ENT_LAUNCH(2, 16, 2)
  ENT_LAUNCH(2, 16, 3)
  ENT_LAUNCH(3, 4, 0)
  ENT_LAUNCH(3, 8, 0)
  ENT_LAUNCH(3, 8, 1)
  ENT_LAUNCH(3, 8, 2)
  ENT_LAUNCH(3, 8, 3)
#undef ENT_LAUNCH
  return cudaErrorInvalidValue;
}

cudaError_t launch_density(cudaStream_t st, int d, int r, const TileDesc* tiles,
                           uint32_t n_slots, const InstDev* insts,
                           uint32_t* work_counter, uint32_t* err,
                           double* tile_logsum, uint32_t mode, int n_sms,
                           int* launched) {
  return launch_density(st, d, r, 0, tiles, n_slots, insts, work_counter, err, tile_logsum,
                        mode, n_sms, launched);
}

cudaError_t launch_inst_logsum(cudaStream_t st, const InstDev* insts,
                               uint32_t n_inst, const double* tile_logsum,
                               double* inst_logsum) {
  if (n_inst == 0) return cudaSuccess;
  k_inst_logsum<<<n_inst, 256, 0, st>>>(insts, tile_logsum, inst_logsum);
  return cudaGetLastError();
}

}  // namespace ent
