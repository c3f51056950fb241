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

// Stable scatter of one block's chunk: every element's rank among the
// chunk's elements of its digit is found with warp matches and per-warp
// digit counts (in element order), the chunk is reordered by digit in shared
// memory, and the digit runs are written out contiguously (coalesced).
__global__ void __launch_bounds__(RS_THREADS)
    k_radix_scatter(const uint32_t* __restrict__ kin,
                    const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
                    uint32_t* __restrict__ vout, int shift, SegTableDev t) {
  __shared__ uint32_t off[256];    // global start of each digit for this block
  __shared__ uint32_t lstart[256]; // start of each digit in the block's chunk
  __shared__ uint32_t run[256];
  __shared__ uint32_t wcnt[RS_WARPS][256];
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
  // digit counts of the chunk -> local digit starts (exclusive scan)
  run[threadIdx.x] = 0;
  __syncthreads();
  for (uint32_t e = threadIdx.x; e < ne; e += RS_THREADS)
    atomicAdd(&run[(kin[base + e0 + e] >> shift) & 255u], 1u);
  __syncthreads();
  {
    const uint32_t c = run[threadIdx.x];
    uint32_t x = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wcnt[0][warp] = x;
    __syncthreads();
    uint32_t wp = 0;
    for (int w = 0; w < warp; ++w) wp += wcnt[0][w];
    lstart[threadIdx.x] = wp + x - c;
    __syncthreads();
  }
  run[threadIdx.x] = 0;
  const uint32_t lt_mask = (1u << lane) - 1u;
  for (int it = 0; it < RS_ITEMS; ++it) {
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) wcnt[w][threadIdx.x] = 0;
    __syncthreads();
    const uint32_t e = e0 + it * RS_THREADS + threadIdx.x;
    const bool valid = e < len;
    uint32_t key = 0, val = 0, digit = 256;
    if (valid) {
      key = kin[base + e];
      val = vin[base + e];
      digit = (key >> shift) & 255u;
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, digit);
    const uint32_t rank = __popc(peers & lt_mask);
    if (valid && rank == 0) wcnt[warp][digit] = __popc(peers);
    __syncthreads();
    {  // exclusive scan over warps, per digit, continuing the running count
      uint32_t r = run[threadIdx.x];
#pragma unroll
      for (int w = 0; w < RS_WARPS; ++w) {
        const uint32_t c = wcnt[w][threadIdx.x];
        wcnt[w][threadIdx.x] = r;
        r += c;
      }
      run[threadIdx.x] = r;
    }
    __syncthreads();
    if (valid) {
      const uint32_t lp = lstart[digit] + wcnt[warp][digit] + rank;
      sk[lp] = key;
      sv[lp] = val;
    }
    __syncthreads();
  }
  // chunk in digit order: consecutive elements of a digit go to consecutive
  // global positions
  for (uint32_t i = threadIdx.x; i < ne; i += RS_THREADS) {
    const uint32_t key = sk[i];
    const uint32_t d = (key >> shift) & 255u;
    const uint32_t pos = off[d] + (i - lstart[d]);
    kout[base + pos] = key;
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
