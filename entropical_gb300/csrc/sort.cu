// Segmented, stable LSD radix sort of (uint32 key, uint32 value) pairs.
//
// Used for two things on the density path:
//   * sorting each coordinate column by value (orderable float keys, four
//     8-bit passes) -- the device replacement of Tools::dim1_sorted_coords
//     (tools.hxx:113-150);
//   * partitioning an already value-sorted sequence into strips (cell ids of
//     the remaining dimensions as keys, 1-3 passes). Because every pass is
//     stable, points stay sorted on dimension 0 inside each strip.
//
// One pass = histogram (per block, per digit) -> per-segment exclusive scan
// in digit-major order -> stable scatter (warp match + per-warp digit counts
// combined in warp order). Deterministic: the output order is a pure
// function of the input.
#include "engine.h"

namespace ent {

namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 8;
constexpr int RS_CHUNK = RS_THREADS * RS_ITEMS;  // elements per block
constexpr int RS_WARPS = RS_THREADS / 32;

__global__ void __launch_bounds__(RS_THREADS)
    k_radix_hist(const uint32_t* __restrict__ keys, int shift, SegTableDev t) {
  __shared__ uint32_t cnt[256];
  const uint32_t b = blockIdx.x;
  const uint32_t s = t.blk_seg[b];
  const uint32_t j = b - t.seg_blk0[s];
  const uint32_t nb = t.seg_blk0[s + 1] - t.seg_blk0[s];
  const uint64_t base = t.seg_off[s];
  const uint32_t len = t.seg_len[s];
  const uint32_t e0 = j * RS_CHUNK;
  const uint32_t e1 = min(e0 + RS_CHUNK, len);
  cnt[threadIdx.x] = 0;
  __syncthreads();
  for (uint32_t e = e0 + threadIdx.x; e < e1; e += RS_THREADS)
    atomicAdd(&cnt[(keys[base + e] >> shift) & 255u], 1u);
  __syncthreads();
  t.hist[(uint64_t)t.seg_blk0[s] * 256 + (uint64_t)threadIdx.x * nb + j] =
      cnt[threadIdx.x];
}

// Exclusive scan of one segment's 256*nb histogram entries (digit-major).
__global__ void __launch_bounds__(1024) k_radix_scan(SegTableDev t) {
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t carry_s;
  const uint32_t s = blockIdx.x;
  const uint32_t nb = t.seg_blk0[s + 1] - t.seg_blk0[s];
  uint32_t* a = t.hist + (uint64_t)t.seg_blk0[s] * 256;
  const uint32_t L = 256 * nb;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  for (uint32_t base = 0; base < L; base += 1024) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < L ? a[i] : 0u;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      warp_tot[lane] = w;  // inclusive
    }
    __syncthreads();
    const uint32_t carry = carry_s;
    const uint32_t wprev = warp ? warp_tot[warp - 1] : 0u;
    if (i < L) a[i] = carry + wprev + x - v;
    __syncthreads();
    if (threadIdx.x == 0) carry_s = carry + warp_tot[31];
    __syncthreads();
  }
}

// Stable scatter of one block's chunk (RS_CHUNK elements; warp w owns the
// RS_ITEMS * 32 consecutive elements from w * RS_ITEMS * 32). Each warp ranks
// its elements per digit with warp matches and warp-private digit counts (in
// element order); one block-wide scan over (digit, warp) turns the counts
// into positions in the chunk sorted by digit; the chunk is reordered in
// shared memory and its digit runs are written out contiguously (coalesced).
// Four block barriers per chunk.
__global__ void __launch_bounds__(RS_THREADS)
    k_radix_scatter(const uint32_t* __restrict__ kin,
                    const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
                    uint32_t* __restrict__ vout, int shift, SegTableDev t) {
  __shared__ uint32_t off[256];     // global start of each digit for this block
  __shared__ uint32_t lstart[256];  // start of each digit in the reordered chunk
  __shared__ uint32_t wcnt[RS_WARPS][256];
  __shared__ uint32_t wtot[RS_WARPS];
  __shared__ uint32_t sk[RS_CHUNK], sv[RS_CHUNK];
  const uint32_t b = blockIdx.x;
  const uint32_t s = t.blk_seg[b];
  const uint32_t j = b - t.seg_blk0[s];
  const uint32_t nb = t.seg_blk0[s + 1] - t.seg_blk0[s];
  const uint64_t base = t.seg_off[s];
  const uint32_t len = t.seg_len[s];
  const uint32_t e0 = j * RS_CHUNK;
  const uint32_t ne = min((uint32_t)RS_CHUNK, len - e0);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  off[threadIdx.x] =
      t.hist[(uint64_t)t.seg_blk0[s] * 256 + (uint64_t)threadIdx.x * nb + j];
#pragma unroll
  for (int w = 0; w < RS_WARPS; ++w) wcnt[w][threadIdx.x] = 0;
  __syncthreads();
  // 1. per warp: rank of every element among the warp's elements of its digit
  const uint32_t lt_mask = (1u << lane) - 1u;
  uint32_t key[RS_ITEMS], val[RS_ITEMS], rnk[RS_ITEMS];
  uint32_t* myc = wcnt[warp];
#pragma unroll
  for (int it = 0; it < RS_ITEMS; ++it) {
    const uint32_t e = (uint32_t)warp * (RS_ITEMS * 32) + it * 32 + lane;
    const bool valid = e < ne;
    uint32_t digit = 256;
    key[it] = 0;
    val[it] = 0;
    if (valid) {
      key[it] = kin[base + e0 + e];
      val[it] = vin[base + e0 + e];
      digit = (key[it] >> shift) & 255u;
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, digit);
    const uint32_t r = __popc(peers & lt_mask);
    const uint32_t prior = valid ? myc[digit] : 0u;
    __syncwarp();
    if (valid && r == 0) myc[digit] = prior + __popc(peers);
    __syncwarp();
    rnk[it] = prior + r;
  }
  __syncthreads();
  // 2. thread d: digit d's total and per-warp starts; block scan over digits
  const uint32_t d = threadIdx.x;
  uint32_t tot = 0;
#pragma unroll
  for (int w = 0; w < RS_WARPS; ++w) {
    const uint32_t c = wcnt[w][d];
    wcnt[w][d] = tot;
    tot += c;
  }
  uint32_t x = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wtot[warp] = x;
  __syncthreads();
  uint32_t wp = 0;
  for (int w = 0; w < warp; ++w) wp += wtot[w];
  const uint32_t start = wp + x - tot;
  lstart[d] = start;
#pragma unroll
  for (int w = 0; w < RS_WARPS; ++w) wcnt[w][d] += start;
  __syncthreads();
  // 3. reorder the chunk by digit in shared memory
#pragma unroll
  for (int it = 0; it < RS_ITEMS; ++it) {
    const uint32_t e = (uint32_t)warp * (RS_ITEMS * 32) + it * 32 + lane;
    if (e < ne) {
      const uint32_t dg = (key[it] >> shift) & 255u;
      const uint32_t lp = myc[dg] + rnk[it];
      sk[lp] = key[it];
      sv[lp] = val[it];
    }
  }
  __syncthreads();
  // 4. digit runs to their global positions, consecutive elements together
  for (uint32_t i = threadIdx.x; i < ne; i += RS_THREADS) {
    const uint32_t k = sk[i];
    const uint32_t dg = (k >> shift) & 255u;
    const uint32_t pos = off[dg] + (i - lstart[dg]);
    kout[base + pos] = k;
    vout[base + pos] = sv[i];
  }
}

}  // namespace

uint32_t radix_blocks_for(uint32_t len) {
  return (len + RS_CHUNK - 1) / RS_CHUNK;
}

cudaError_t seg_radix_sort(cudaStream_t st, const SegTableDev& t,
                           uint32_t n_seg, uint32_t total_blocks,
                           uint32_t*& keys, uint32_t*& vals, uint32_t*& ktmp,
                           uint32_t*& vtmp, int begin_bit, int end_bit) {
  for (int shift = begin_bit; shift < end_bit; shift += 8) {
    if (total_blocks == 0) break;
    k_radix_hist<<<total_blocks, RS_THREADS, 0, st>>>(keys, shift, t);
    k_radix_scan<<<n_seg, 1024, 0, st>>>(t);
    k_radix_scatter<<<total_blocks, RS_THREADS, 0, st>>>(keys, vals, ktmp, vtmp,
                                                         shift, t);
    uint32_t* a = keys;
    keys = ktmp;
    ktmp = a;
    a = vals;
    vals = vtmp;
    vtmp = a;
  }
  return cudaGetLastError();
}

}  // namespace ent
