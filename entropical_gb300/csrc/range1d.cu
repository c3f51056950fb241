// One-dimensional density sums from exact prefix sums (pair body PAIR_RANGE).
//
// The 1-D density at target k is sum_j max(0, g^2 - (y_j - y_k)^2) over the
// value-sorted scaled points y (the reference's densities_1d loop,
// densities_omp.cpp:67-94, and density_1d.cuh: one term per pair). In a sorted
// column the support of k is one index range [s_k, e_k): both ends come from
// binary searches with the pair kernels' own test fma(-d, d, g^2) > 0,
// d = fl(y_j - y_k), which is monotone in |d|. On the range
//   sum_j (g^2 - (y_j - y_k)^2) = c g^2 - sum_j (y_j - y_k)^2,   c = e_k - s_k,
// and with prefix sums SY, SY2 of Y = y 2^46 and Y^2
//   sum_j (Y_j - Y_k)^2 = SY2 - 2 Y_k SY + c Y_k^2.
// Y is the fixed-point image of y (exact for |y| >= 2^-23 in units of g,
// rounded below), and every sum and product is taken modulo 2^128 in integer
// arithmetic: the identity holds in the integers, reduction modulo 2^128 is a
// ring map, and the true value is below c (2^46 + 1)^2 < 2^124, so the
// modular result IS the exact integer. No cancellation, no dependence on the
// data's offset or spread, and any summation order gives the same bits. The
// per-target cost is two binary searches and a few 128-bit operations instead
// of a pass over its support; the result is exact up to the fixed-point
// rounding of |y| < 2^-23 g (error < 2^-45 g^2 per pair).
//
// Output: InstDev::acc[k] (unscaled sums, sorted positions), finished by
// launch_sym_finish exactly as the symmetric pair kernels' sums.
#include <algorithm>

#include "engine.h"
#include "staging.cuh"  // FULL_MASK

namespace ent {
namespace {

typedef unsigned __int128 u128;

constexpr uint32_t R1_TB = 256;               // targets per block
constexpr uint32_t R1_E = 8;                  // prefix values per thread
constexpr uint32_t R1_CHUNK = R1_TB * R1_E;   // prefix values per block

// round(y 2^46) modulo 2^128 (two's complement), y finite.
__device__ __forceinline__ u128 quant46(float y) {
  const uint32_t b = __float_as_uint(y);
  const int e = (int)((b >> 23) & 0xffu);
  if (e == 0) return 0;  // zero or subnormal
  const uint64_t m = (uint64_t)((b & 0x7fffffu) | 0x800000u);
  const int sh = e - 104;  // y 2^46 = m 2^(e - 150 + 46)
  u128 v;
  if (sh >= 128) {
    v = 0;
  } else if (sh >= 0) {
    v = (u128)m << sh;
  } else if (sh > -25) {
    v = (u128)((m + (1ull << (-sh - 1))) >> (-sh));
  } else {
    v = 0;
  }
  return (b & 0x80000000u) ? (u128)0 - v : v;
}

__device__ __forceinline__ u128 shfl_up128(u128 v, int o) {
  const unsigned long long lo = __shfl_up_sync(FULL_MASK, (unsigned long long)v, o);
  const unsigned long long hi = __shfl_up_sync(FULL_MASK, (unsigned long long)(v >> 64), o);
  return ((u128)hi << 64) | lo;
}
__device__ __forceinline__ u128 shfl_idx128(u128 v, int l) {
  const unsigned long long lo = __shfl_sync(FULL_MASK, (unsigned long long)v, l);
  const unsigned long long hi = __shfl_sync(FULL_MASK, (unsigned long long)(v >> 64), l);
  return ((u128)hi << 64) | lo;
}
__device__ __forceinline__ u128 shfl_xor128(u128 v, int o) {
  const unsigned long long lo = __shfl_xor_sync(FULL_MASK, (unsigned long long)v, o);
  const unsigned long long hi = __shfl_xor_sync(FULL_MASK, (unsigned long long)(v >> 64), o);
  return ((u128)hi << 64) | lo;
}

__device__ __forceinline__ double u128_to_double(u128 v) {
  return __ull2double_rn((unsigned long long)(v >> 64)) * 18446744073709551616.0 +
         __ull2double_rn((unsigned long long)v);
}

// chunk totals {sum Y, sum Y^2} of every chunk of every instance
__global__ void __launch_bounds__(R1_TB)
    k_r1_totals(const Range1D* __restrict__ rs, u128* __restrict__ tot) {
  __shared__ u128 sw[2][R1_TB / 32];
  const Range1D& R = rs[blockIdx.y];
  const uint64_t b0 = (uint64_t)blockIdx.x * R1_CHUNK;
  if (b0 >= R.n) return;  // block-uniform
  const uint64_t k0 = b0 + (uint64_t)threadIdx.x * R1_E;
  u128 s1 = 0, s2 = 0;
#pragma unroll
  for (uint32_t e = 0; e < R1_E; ++e)
    if (k0 + e < R.n) {
      const u128 Y = quant46(R.y[k0 + e]);
      s1 += Y;
      s2 += Y * Y;
    }
  for (int o = 16; o; o >>= 1) {
    s1 += shfl_xor128(s1, o);
    s2 += shfl_xor128(s2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sw[0][threadIdx.x >> 5] = s1;
    sw[1][threadIdx.x >> 5] = s2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    u128 a = 0, b = 0;
    for (uint32_t w = 0; w < R1_TB / 32; ++w) {
      a += sw[0][w];
      b += sw[1][w];
    }
    tot[2 * ((size_t)R.chunk_base + blockIdx.x)] = a;
    tot[2 * ((size_t)R.chunk_base + blockIdx.x) + 1] = b;
  }
}

// one warp per instance: exclusive scan of its chunk totals, in place
__global__ void k_r1_chunks(const Range1D* __restrict__ rs, uint32_t n_inst,
                            u128* __restrict__ tot) {
  const uint32_t q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= n_inst) return;  // warp-uniform
  const uint32_t nch = (rs[q].n + R1_CHUNK - 1) / R1_CHUNK;
  u128* t = tot + 2 * (size_t)rs[q].chunk_base;
  u128 run1 = 0, run2 = 0;
  for (uint32_t b = 0; b < nch; b += 32) {
    const bool in = b + lane < nch;
    const u128 v1 = in ? t[2 * (b + lane)] : (u128)0;
    const u128 v2 = in ? t[2 * (b + lane) + 1] : (u128)0;
    u128 i1 = v1, i2 = v2;
    for (int o = 1; o < 32; o <<= 1) {
      const u128 u1 = shfl_up128(i1, o), u2 = shfl_up128(i2, o);
      if (lane >= o) {
        i1 += u1;
        i2 += u2;
      }
    }
    if (in) {  // exclusive = inclusive - own (exact modulo 2^128)
      t[2 * (b + lane)] = run1 + i1 - v1;
      t[2 * (b + lane) + 1] = run2 + i2 - v2;
    }
    run1 += shfl_idx128(i1, 31);
    run2 += shfl_idx128(i2, 31);
  }
}

// P[k] = {sum_{j<k} Y_j, sum_{j<k} Y_j^2}, k = 0..n
__global__ void __launch_bounds__(R1_TB)
    k_r1_write(const Range1D* __restrict__ rs, const u128* __restrict__ off) {
  __shared__ u128 sw[2][R1_TB / 32];
  const Range1D& R = rs[blockIdx.y];
  const uint64_t b0 = (uint64_t)blockIdx.x * R1_CHUNK;
  if (b0 >= R.n) return;  // block-uniform
  const uint64_t k0 = b0 + (uint64_t)threadIdx.x * R1_E;
  u128 a1[R1_E], a2[R1_E];
  u128 s1 = 0, s2 = 0;
#pragma unroll
  for (uint32_t e = 0; e < R1_E; ++e) {
    if (k0 + e < R.n) {
      const u128 Y = quant46(R.y[k0 + e]);
      s1 += Y;
      s2 += Y * Y;
    }
    a1[e] = s1;
    a2[e] = s2;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  u128 i1 = s1, i2 = s2;
  for (int o = 1; o < 32; o <<= 1) {
    const u128 u1 = shfl_up128(i1, o), u2 = shfl_up128(i2, o);
    if (lane >= o) {
      i1 += u1;
      i2 += u2;
    }
  }
  if (lane == 31) {
    sw[0][warp] = i1;
    sw[1][warp] = i2;
  }
  __syncthreads();
  u128 base1 = off[2 * ((size_t)R.chunk_base + blockIdx.x)] + i1 - s1;
  u128 base2 = off[2 * ((size_t)R.chunk_base + blockIdx.x) + 1] + i2 - s2;
  for (int w = 0; w < warp; ++w) {
    base1 += sw[0][w];
    base2 += sw[1][w];
  }
  u128* P = static_cast<u128*>(R.P);
  if (b0 == 0 && threadIdx.x == 0) P[0] = P[1] = 0;
#pragma unroll
  for (uint32_t e = 0; e < R1_E; ++e)
    if (k0 + e < R.n) {
      P[2 * (k0 + e + 1)] = base1 + a1[e];
      P[2 * (k0 + e + 1) + 1] = base2 + a2[e];
    }
}

__device__ __forceinline__ bool in_support(float yj, float yk, float g2) {
  const float d = __fsub_rn(yj, yk);
  return __fmaf_rn(-d, d, g2) > 0.f;
}

// one thread per target: its range, then the sum from the prefix sums
__global__ void __launch_bounds__(R1_TB)
    k_r1_density(const Range1D* __restrict__ rs, uint32_t n_inst,
                 const uint32_t* __restrict__ blk_base) {
  const uint32_t g = blockIdx.x;
  uint32_t lo = 0, hi = n_inst;
  while (hi - lo > 1) {
    const uint32_t m = (lo + hi) / 2;
    if (blk_base[m] <= g) lo = m; else hi = m;
  }
  const Range1D& R = rs[lo];
  const uint32_t k = (g - R.blk_base) * R1_TB + threadIdx.x;
  const uint32_t n = R.n;
  if (k >= n) return;
  const float* __restrict__ y = R.y;
  const float yk = y[k], g2 = R.g2;
  uint32_t a = 0, b = k;  // first j <= k in the support
  while (a < b) {
    const uint32_t m = a + ((b - a) >> 1);
    if (in_support(yk, y[m], g2)) b = m; else a = m + 1;
  }
  const uint32_t s = a;
  a = k + 1;
  b = n;  // first j > k outside the support
  while (a < b) {
    const uint32_t m = a + ((b - a) >> 1);
    if (in_support(y[m], yk, g2)) a = m + 1; else b = m;
  }
  const uint32_t e = a;
  const u128* __restrict__ P = static_cast<const u128*>(R.P);
  const u128 sy = P[2 * (size_t)e] - P[2 * (size_t)s];
  const u128 sy2 = P[2 * (size_t)e + 1] - P[2 * (size_t)s + 1];
  const u128 Yk = quant46(yk);
  const uint32_t c = e - s;
  const u128 q = sy2 - 2 * Yk * sy + (u128)c * (Yk * Yk);
  // 2^-92 converts the fixed-point squares back to units of y^2
  R.acc[k] = (double)c * (double)g2 - u128_to_double(q) * 0x1p-92;
}

}  // namespace

uint32_t range1d_chunks(uint32_t n) { return (n + R1_CHUNK - 1) / R1_CHUNK; }
uint32_t range1d_blocks(uint32_t n) { return (n + R1_TB - 1) / R1_TB; }
size_t range1d_prefix_bytes(uint32_t n) { return 32 * ((size_t)n + 1); }

cudaError_t launch_range1d(cudaStream_t st, const Range1D* rs, uint32_t n_inst, uint32_t max_n,
                           const uint32_t* blk_base, uint32_t n_blocks, void* chunk_tot) {
  if (n_inst == 0 || n_blocks == 0) return cudaSuccess;
  u128* tot = static_cast<u128*>(chunk_tot);
  const dim3 gc(range1d_chunks(std::max(max_n, 1u)), n_inst);
  k_r1_totals<<<gc, R1_TB, 0, st>>>(rs, tot);
  k_r1_chunks<<<(n_inst + 3) / 4, 128, 0, st>>>(rs, n_inst, tot);
  k_r1_write<<<gc, R1_TB, 0, st>>>(rs, tot);
  k_r1_density<<<n_blocks, R1_TB, 0, st>>>(rs, n_inst, blk_base);
  return cudaGetLastError();
}

}  // namespace ent
