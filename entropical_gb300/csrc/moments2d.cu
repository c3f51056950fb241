// Two-dimensional density sums from exact strip moments (pair body
// PAIR_MOMENT).
//
// The 2-D density at target t is sum_s wx(t,s) wy(t,s) with
// w = max(0, g^2 - d^2) per dimension in scaled units (the reference's
// densities_2d loop, densities_omp.cpp:97-126, and density_2d.cuh). The
// points are strip-major: strips of width h/S along dimension 1, sorted by
// dimension 0 inside each strip. For one target and one strip:
//  * the sources in x-support form one index range [l, r) of the strip,
//    found by two binary searches with the pair kernels' own test
//    fma(-d, d, g^2) > 0 (monotone in |d|);
//  * if the strip's smallest and largest y both pass the y test, every
//    source of the strip does (|fl(y - t_y)| lies between the two), and on
//    [l, r) the sum is a polynomial in the sources' coordinates:
//      sum (G1 - (TX - X)^2)(G2 - (TY - Y)^2)
//        = sum_{a,b <= 2} c_a(TX) d_b(TY) M_ab,   M_ab = sum X^a Y^b,
//    with X = x 2^23, Y = y 2^23 fixed point and G = g^2 2^46. The moments
//    come from prefix sums over the strip-major order taken modulo 2^128;
//    the identity holds in the integers, reduction modulo 2^128 is a ring
//    map and the true value lies in (-2^124, 2^124), so the signed modular
//    result IS the exact integer: no cancellation whatever the offset or
//    spread of the data;
//  * the strips at distance exactly S from the target's own (where the edge
//    of its y-support falls) are summed pair by pair by the symmetric pair
//    kernel, each pair once for both points (the plan gives every strip one
//    tile run: the strip S above it); strips nearer than S whose y extent
//    still crosses the support (rounding at the widened cell edges) are
//    summed pair by pair here.
// Fixed-point rounding of the coordinates (2^-23 g) changes a kernel value
// by less than 2^-21 g^2 per dimension, far below the 1e-5 density bar.
//
// The epilogue (scale, per-point output, log and per-block sums) runs in the
// same kernel; the symmetric kernel's finish skips these instances. The log
// of each target's exact sum is taken in 64-bit fixed point (ilog_fx48) and
// the block sums are exact integer sums.
#include <algorithm>

#include "engine.h"
#include "staging.cuh"  // FULL_MASK

namespace ent {
namespace {

typedef unsigned __int128 u128;

constexpr uint32_t M2_TB = 128;               // targets per block
constexpr uint32_t M2_PT = 256;               // prefix threads per block
constexpr uint32_t M2_E = 8;                  // prefix values per thread
constexpr uint32_t M2_CHUNK = M2_PT * M2_E;   // prefix values per block
constexpr int NM = 8;  // X, Y, X^2, XY, Y^2, X^2 Y, X Y^2, X^2 Y^2

// round(v 2^F) modulo 2^128 (two's complement), v finite.
template <int F>
__device__ __forceinline__ u128 quant(float v) {
  const uint32_t b = __float_as_uint(v);
  const int e = (int)((b >> 23) & 0xffu);
  if (e == 0) return 0;  // zero or subnormal
  const uint64_t m = (uint64_t)((b & 0x7fffffu) | 0x800000u);
  const int sh = e - 150 + F;
  u128 q;
  if (sh >= 128) {
    q = 0;
  } else if (sh >= 0) {
    q = (u128)m << sh;
  } else if (sh > -25) {
    q = (u128)((m + (1ull << (-sh - 1))) >> (-sh));
  } else {
    q = 0;
  }
  return (b & 0x80000000u) ? (u128)0 - q : q;
}

// quant<23> of a value below 2^8 in magnitude (|result| < 2^31), with the
// same rounding (half away from zero).
__device__ __forceinline__ int32_t quant23_narrow(float v) {
  const uint32_t b = __float_as_uint(v);
  const int e = (int)((b >> 23) & 0xffu);
  const uint32_t m = (b & 0x7fffffu) | 0x800000u;
  const int sh = e - 127;  // <= 7
  uint32_t q;
  if (e == 0) q = 0;
  else if (sh >= 0) q = m << sh;
  else if (sh > -25) q = (m + (1u << (-sh - 1))) >> (-sh);
  else q = 0;
  return (b & 0x80000000u) ? -(int32_t)q : (int32_t)q;
}

// both coordinates below 2^8 in magnitude (scaled units)
__device__ __forceinline__ bool narrow2(float2 p) {
  return ((__float_as_uint(p.x) >> 23) & 0xffu) < 135u &&
         ((__float_as_uint(p.y) >> 23) & 0xffu) < 135u;
}

__device__ __forceinline__ u128 u128_of(int64_t hi, uint64_t lo) {
  return ((u128)(uint64_t)hi << 64) | lo;
}

// The eight moments of one point modulo 2^128. Points whose scaled
// coordinates lie below 2^8 in magnitude (all of them for data within a few
// hundred bandwidths of zero) take 32-bit coordinates and 64 x 64 -> 128-bit
// products; the others the general 128-bit form. Both give the same residues.
__device__ __forceinline__ void moments(float2 p, u128 (&m)[NM]) {
  if (narrow2(p)) {
    const int32_t x = quant23_narrow(p.x), y = quant23_narrow(p.y);
    const int64_t X2 = (int64_t)x * x, Y2 = (int64_t)y * y, XY = (int64_t)x * y;
    const int64_t X = x, Y = y;
    m[0] = (u128)(__int128)x;
    m[1] = (u128)(__int128)y;
    m[2] = (u128)(uint64_t)X2;
    m[3] = (u128)(__int128)XY;
    m[4] = (u128)(uint64_t)Y2;
    m[5] = u128_of(__mul64hi(X2, Y), (uint64_t)X2 * (uint64_t)Y);
    m[6] = u128_of(__mul64hi(X, Y2), (uint64_t)X * (uint64_t)Y2);
    m[7] = u128_of((int64_t)__umul64hi((uint64_t)X2, (uint64_t)Y2),
                   (uint64_t)X2 * (uint64_t)Y2);
    return;
  }
  const u128 X = quant<23>(p.x), Y = quant<23>(p.y);
  const u128 X2 = X * X, Y2 = Y * Y;
  m[0] = X;
  m[1] = Y;
  m[2] = X2;
  m[3] = X * Y;
  m[4] = Y2;
  m[5] = X2 * Y;
  m[6] = X * Y2;
  m[7] = X2 * Y2;
}

// The M2_E points of one prefix thread, loaded at once (16-byte loads when
// all are present: pts is 256-byte aligned and k0 a multiple of 8); returns
// how many are present.
__device__ __forceinline__ uint32_t load_points8(const float2* __restrict__ pts, uint64_t k0,
                                                 uint32_t n, float2 (&p)[M2_E]) {
  static_assert(M2_E == 8, "four 16-byte loads per thread");
  if (k0 + M2_E <= n) {
    const float4* q = reinterpret_cast<const float4*>(pts + k0);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float4 v = q[i];
      p[2 * i] = make_float2(v.x, v.y);
      p[2 * i + 1] = make_float2(v.z, v.w);
    }
    return M2_E;
  }
  const uint32_t ne = k0 < n ? (uint32_t)(n - k0) : 0u;
#pragma unroll
  for (uint32_t e = 0; e < M2_E; ++e) p[e] = e < ne ? pts[k0 + e] : make_float2(0.f, 0.f);
  return ne;
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

__device__ __forceinline__ double s128_to_double(u128 v) {
  const bool neg = (v >> 127) != 0;
  if (neg) v = (u128)0 - v;
  const double d = __ull2double_rn((unsigned long long)(v >> 64)) * 18446744073709551616.0 +
                   __ull2double_rn((unsigned long long)v);
  return neg ? -d : d;
}

// ---------------------------------------------- log of an exact 128-bit sum
// The per-point log of the strip-moment epilogue without the FP64 pipe (it
// runs at a small fraction of the FP32 rate on this GPU): the target's sum is
// one exact nonnegative integer T (units of 2^-92 g^4), and log T is formed in
// 64-bit fixed point with 2^-48 resolution. T = m 2^p with m in [1, 2) taken
// from T's top 48 bits; the top 8 bits of m after the leading one pick a table
// entry {inv ~ 1/c, log(1/inv) in 2^-56 fixed point}, c = 1 + (k + 1/2)/256
// (the table is made on the host with its libm); r = m inv - 1 is formed
// exactly as a float-float pair rh + rl (|r| < 2^-8, |rl| < 2^-22),
// log1p(r) = r - r^2/2 + r^3/3 - r^4/4 + r^5/5 with rh^2 as an exact FP32
// product pair and the rl cross terms to r^3, and
//   log T = p ln 2 + log(1/inv) + log1p(r),
// every part added in fixed point. Error below 2^-45 (2.9e-14) absolute: the
// 48-bit truncation of T, the rounding of rl and of the fixed-point parts.
constexpr int64_t LN2_FX56 = 49946518145322874LL;  // round(ln 2 * 2^56)

// round(x 2^48) of a float with |x| < 1
__device__ __forceinline__ int64_t f32_to_fx48(float x) {
  const uint32_t b = __float_as_uint(x);
  const int e = (int)((b >> 23) & 0xffu);
  if (e == 0) return 0;
  const int64_t m = (int64_t)((b & 0x7fffffu) | 0x800000u);
  const int sh = e - 102;  // x 2^48 = m 2^(e - 150 + 48)
  int64_t q;
  if (sh >= 0) q = m << sh;
  else if (sh > -25) q = (m + (1LL << (-sh - 1))) >> (-sh);
  else q = 0;
  return (b & 0x80000000u) ? -q : q;
}

// (hi, lo) += m 2^sh rounded to an integer, m < 2^53 (the fixed-point image
// of a nonnegative float or double; two 64-bit words, no 128-bit shifts)
__device__ __forceinline__ void add_shifted(uint64_t m, int sh, uint64_t& lo, uint64_t& hi) {
  uint64_t a = 0, b = 0;  // low and high word of the addend
  if (sh >= 64) {
    b = m << (sh - 64);
  } else if (sh > 0) {
    a = m << sh;
    b = m >> (64 - sh);
  } else if (sh == 0) {
    a = m;
  } else if (sh > -54) {
    a = (m + (1ull << (-sh - 1))) >> (-sh);
  }
  lo += a;
  hi += b + (lo < a ? 1ull : 0ull);
}

// += round(v 2^92) for a finite float v >= 0 below 2^30
__device__ __forceinline__ void add_fx92_f32(float v, uint64_t& lo, uint64_t& hi) {
  const uint32_t b = __float_as_uint(v);
  const int e = (int)((b >> 23) & 0xffu);
  if (e == 0 || (b >> 31)) return;
  add_shifted((uint64_t)((b & 0x7fffffu) | 0x800000u), e - 150 + 92, lo, hi);
}

// += round(v 2^92) for a finite double v >= 0 below 2^30
__device__ __forceinline__ void add_fx92_f64(double v, uint64_t& lo, uint64_t& hi) {
  const uint64_t b = (uint64_t)__double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ffu);
  if (e == 0 || (b >> 63)) return;
  add_shifted((b & 0xfffffffffffffull) | (1ull << 52), e - 1075 + 92, lo, hi);
}

// log(T) in 2^-48 fixed point of T = hi 2^64 + lo > 0
__device__ __forceinline__ int64_t ilog_fx48(uint64_t lo, uint64_t hi,
                                             const ILogEntry* __restrict__ tab) {
  if ((lo | hi) == 0) return -(1LL << 62);  // never for a density: its own term is > 0
  const int p = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);
  const int s = p - 47;  // m48 = floor(T / 2^s), in [2^47, 2^48)
  uint64_t m48;
  if (s >= 64) m48 = hi >> (s - 64);
  else if (s > 0) m48 = (hi << (64 - s)) | (lo >> s);
  else m48 = lo << (-s);
  const uint32_t k = (uint32_t)(m48 >> 39) & 255u;
  const ILogEntry t = tab[k];
  // m = mh + ml exactly (24 + 24 bits)
  const float mh = __uint_as_float(0x3f800000u | (uint32_t)((m48 >> 24) & 0x7fffffu));
  const float ml = __fmul_rn(__uint2float_rn((uint32_t)(m48 & 0xffffffu)), 0x1p-47f);
  const float p1 = __fmul_rn(mh, t.inv);
  const float e1 = __fmaf_rn(mh, t.inv, -p1);  // mh inv = p1 + e1 exactly
  const float rh = __fsub_rn(p1, 1.0f);        // exact: p1 in [1/2, 2]
  const float rl = __fmaf_rn(ml, t.inv, e1);
  const float qh = __fmul_rn(rh, rh);
  const float qe = __fmaf_rn(rh, rh, -qh);     // rh^2 = qh + qe exactly
  // two-sum of rh and -qh/2
  const float b2 = __fmul_rn(-0.5f, qh);
  const float sh = __fadd_rn(rh, b2);
  const float bb = __fsub_rn(sh, rh);
  const float err = __fadd_rn(__fsub_rn(rh, __fsub_rn(sh, bb)), __fsub_rn(b2, bb));
  const float h3 = __fmul_rn(__fmul_rn(rh, qh),
                             __fmaf_rn(rh, __fmaf_rn(rh, 0.2f, -0.25f), 1.0f / 3.0f));
  // the small rest: rounding of the two-sum and the cross terms of r^2/2 and
  // r^3/3 with rl (-rh rl + rh^2 rl); rl itself is added on its own
  const float rest = __fadd_rn(__fadd_rn(err, __fmaf_rn(-0.5f, qe, h3)),
                               __fmul_rn(rl, __fsub_rn(qh, rh)));
  int64_t fx = ((int64_t)p * LN2_FX56 + 128) >> 8;
  fx += (t.l56 + 128) >> 8;
  fx += f32_to_fx48(sh) + f32_to_fx48(rl) + f32_to_fx48(rest);
  return fx;
}

// y extent (smallest, largest scaled y) of every strip: one warp per strip
__global__ void k_m2_ybounds(const Mom2D* __restrict__ ms) {
  const Mom2D& M = ms[blockIdx.y];
  const uint32_t s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (s >= M.n_strips) return;  // warp-uniform
  const uint32_t a = M.strip_start[s], b = M.strip_start[s + 1];
  float lo = 3.4e38f, hi = -3.4e38f;
  for (uint32_t k = a + lane; k < b; k += 32) {
    const float y = M.pts[k].y;
    lo = fminf(lo, y);
    hi = fmaxf(hi, y);
  }
  for (int o = 16; o; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(FULL_MASK, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(FULL_MASK, hi, o));
  }
  if (lane == 0) M.ybound[s] = make_float2(lo, hi);
}

// Block scan helper: exclusive prefix of v (per thread) over the block, and
// the block total; sw holds NM u128 per warp.
__device__ __forceinline__ void block_scan8(u128 (&v)[NM], u128 (&excl)[NM],
                                            u128 (*sw)[NM]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  u128 inc[NM];
#pragma unroll
  for (int m = 0; m < NM; ++m) inc[m] = v[m];
  for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
    for (int m = 0; m < NM; ++m) {
      const u128 u = shfl_up128(inc[m], o);
      if (lane >= o) inc[m] += u;
    }
  }
  if (lane == 31)
#pragma unroll
    for (int m = 0; m < NM; ++m) sw[warp][m] = inc[m];
  __syncthreads();
#pragma unroll
  for (int m = 0; m < NM; ++m) {
    u128 base = inc[m] - v[m];
    for (int w = 0; w < warp; ++w) base += sw[w][m];
    excl[m] = base;
  }
}

// chunk totals of the eight moments
__global__ void __launch_bounds__(M2_PT)
    k_m2_totals(const Mom2D* __restrict__ ms, u128* __restrict__ tot) {
  __shared__ u128 sw[M2_PT / 32][NM];
  const Mom2D& M = ms[blockIdx.y];
  const uint64_t b0 = (uint64_t)blockIdx.x * M2_CHUNK;
  if (b0 >= M.n) return;  // block-uniform
  const uint64_t k0 = b0 + (uint64_t)threadIdx.x * M2_E;
  float2 pt[M2_E];
  const uint32_t ne = load_points8(M.pts, k0, M.n, pt);
  u128 s[NM];
#pragma unroll
  for (int m = 0; m < NM; ++m) s[m] = 0;
#pragma unroll
  for (uint32_t e = 0; e < M2_E; ++e)
    if (e < ne) {
      u128 q[NM];
      moments(pt[e], q);
#pragma unroll
      for (int m = 0; m < NM; ++m) s[m] += q[m];
    }
  // block total: warp sums, then the warps in order
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int m = 0; m < NM; ++m) {
    for (int o = 16; o; o >>= 1) {
      const unsigned long long lo = __shfl_xor_sync(FULL_MASK, (unsigned long long)s[m], o);
      const unsigned long long hi = __shfl_xor_sync(FULL_MASK, (unsigned long long)(s[m] >> 64), o);
      s[m] += ((u128)hi << 64) | lo;
    }
    if (lane == 0) sw[warp][m] = s[m];
  }
  __syncthreads();
  if (threadIdx.x < NM) {
    u128 t = 0;
    for (uint32_t w = 0; w < M2_PT / 32; ++w) t += sw[w][threadIdx.x];
    tot[NM * ((size_t)M.chunk_base + blockIdx.x) + threadIdx.x] = t;
  }
}

// one warp per instance: exclusive scan of its chunk totals, in place
__global__ void k_m2_chunks(const Mom2D* __restrict__ ms, uint32_t n_inst,
                            u128* __restrict__ tot) {
  const uint32_t q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= n_inst) return;  // warp-uniform
  const uint32_t nch = (ms[q].n + M2_CHUNK - 1) / M2_CHUNK;
  u128* t = tot + NM * (size_t)ms[q].chunk_base;
  for (int m = 0; m < NM; ++m) {
    u128 run = 0;
    for (uint32_t b = 0; b < nch; b += 32) {
      const bool in = b + lane < nch;
      const u128 v = in ? t[NM * (b + lane) + m] : (u128)0;
      u128 inc = v;
      for (int o = 1; o < 32; o <<= 1) {
        const u128 u = shfl_up128(inc, o);
        if (lane >= o) inc += u;
      }
      if (in) t[NM * (b + lane) + m] = run + inc - v;
      run += shfl_idx128(inc, 31);
    }
  }
}

// P[k] = sum_{j<k} moments(pts[j]), k = 0..n. Each thread sums M2_E
// consecutive points; the rows of one e (point k0 + e of every lane) pass
// through shared memory, so that every store instruction writes four whole
// 128-byte rows instead of 16 bytes into each of 32 rows.
__global__ void __launch_bounds__(M2_PT)
    k_m2_write(const Mom2D* __restrict__ ms, const u128* __restrict__ off) {
  __shared__ u128 sw[M2_PT / 32][NM];
  __shared__ u128 stage[M2_PT / 32][32 * NM];  // one row per lane, chunks swizzled
  const Mom2D& M = ms[blockIdx.y];
  const uint64_t b0 = (uint64_t)blockIdx.x * M2_CHUNK;
  if (b0 >= M.n) return;  // block-uniform
  const uint64_t k0 = b0 + (uint64_t)threadIdx.x * M2_E;
  u128 s[NM], run[NM];
#pragma unroll
  for (int m = 0; m < NM; ++m) s[m] = 0;
  for (uint32_t e = 0; e < M2_E; ++e)
    if (k0 + e < M.n) {
      u128 q[NM];
      moments(M.pts[k0 + e], q);
#pragma unroll
      for (int m = 0; m < NM; ++m) s[m] += q[m];
    }
  block_scan8(s, run, sw);
  const u128* o = off + NM * ((size_t)M.chunk_base + blockIdx.x);
#pragma unroll
  for (int m = 0; m < NM; ++m) run[m] += o[m];
  u128* P = static_cast<u128*>(M.P);
  if (b0 == 0 && threadIdx.x == 0)
#pragma unroll
    for (int m = 0; m < NM; ++m) P[m] = 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  u128* st = stage[warp];
  // the warp's first point; lane r's rows are points wk0 + 8 r + e
  const uint64_t wk0 = b0 + (uint64_t)(warp * 32) * M2_E;
  for (uint32_t e = 0; e < M2_E; ++e) {
    if (k0 + e < M.n) {
      u128 q[NM];
      moments(M.pts[k0 + e], q);
#pragma unroll
      for (int m = 0; m < NM; ++m) {
        run[m] += q[m];
        st[lane * NM + (m ^ (lane & 7))] = run[m];
      }
    }
    __syncwarp();
    // 8 lanes per row: chunk c of row r = 4 i + lane / 8
    const int c = lane & 7;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = 4 * i + (lane >> 3);
      const uint64_t k = wk0 + (uint64_t)r * M2_E + e;
      if (k < M.n) P[NM * (k + 1) + c] = st[r * NM + (c ^ (r & 7))];
    }
    __syncwarp();
  }
}

__device__ __forceinline__ bool insup(float a, float b, float g2) {
  const float d = __fsub_rn(a, b);
  return __fmaf_rn(-d, d, g2) > 0.f;
}

// acc + wx wy for one source p of target t (x inside the support)
__device__ __forceinline__ float pair_term(float2 p, float2 t, float g1, float g2, float acc) {
  const float dx = __fsub_rn(p.x, t.x), dy = __fsub_rn(p.y, t.y);
  const float wy = __saturatef(__fmaf_rn(-dy, dy, g2));
  return __fmaf_rn(__fmaf_rn(-dx, dx, g1), wy, acc);
}

// x-support of a target at tx in the x-sorted points of one strip, searched
// in [lo, hi) with the pair kernels' own test (monotone in the position and
// in tx): the first position not left of the support, and the first one
// right of it.
__device__ __forceinline__ uint32_t first_not_left(const float2* __restrict__ pts, uint32_t lo,
                                                   uint32_t hi, float tx, float g1) {
  while (lo < hi) {
    const uint32_t m = lo + ((hi - lo) >> 1);
    const float xm = pts[m].x;
    if (xm < tx && !insup(xm, tx, g1)) lo = m + 1; else hi = m;
  }
  return lo;
}
__device__ __forceinline__ uint32_t first_right(const float2* __restrict__ pts, uint32_t lo,
                                                uint32_t hi, float tx, float g1) {
  while (lo < hi) {
    const uint32_t m = lo + ((hi - lo) >> 1);
    const float xm = pts[m].x;
    if (xm > tx && !insup(xm, tx, g1)) hi = m; else lo = m + 1;
  }
  return lo;
}

constexpr int M2_MAX_IN = 23;  // inside strips per target: 2S - 1, S <= 12

// One thread per target; a warp holds 32 consecutive sorted positions. The
// strips within S - 1 of the target's own strip are inside its y-support
// (checked per strip against the strip's y extent); the two strips at
// distance S, where the support's y edge falls, are summed pair by pair by
// the symmetric pair kernel beforehand (its FP64 sums arrive in M.acc).
//
// Searches. When the warp's 32 targets lie in one strip they are x-sorted,
// and the support bounds in any other strip are monotone in the target's x.
// The warp first finds, for every inside strip at once (one bisection per
// lane), the bounds of its first and last target; each lane then searches
// only between them -- a range of about as many points as the warp's x-span
// holds, instead of the whole strip. Other warps (strip boundaries, the end
// of an instance) search each strip in full.
//
// Sums. The moment rows of all inside strips are added first (128-bit, in
// registers) and combined with the target's coefficients once; strips whose
// y extent crosses the support (rounding at the widened cell edges only)
// are summed pair by pair.
//
// Epilogue as the other bodies' finish kernel: density = scale x sum,
// written by original index and/or logged (FP64) and summed per block of
// targets in a fixed order into the instance's slots of tile_logsum.
// LOGONLY: the log-sum epilogue alone (mode == DM_LOGSUM, the estimator
// batches), compiled without the FP64 density path of the other modes.
template <bool LOGONLY>
__global__ void __launch_bounds__(M2_TB, 10)
    k_m2_density(const Mom2D* __restrict__ ms, uint32_t n_inst,
                 const uint32_t* __restrict__ blk_base, const ILogEntry* __restrict__ ilog,
                 double* __restrict__ tile_logsum, uint32_t mode) {
  __shared__ double s_part[M2_TB / 32];
  __shared__ long long s_fx[M2_TB / 32];
  __shared__ uint32_t s_br[M2_TB / 32][4 * M2_MAX_IN];
  const uint32_t gb = blockIdx.x;
  uint32_t lo = 0, hi = n_inst;
  while (hi - lo > 1) {
    const uint32_t m = (lo + hi) / 2;
    if (blk_base[m] <= gb) lo = m; else hi = m;
  }
  const Mom2D& M = ms[lo];
  const uint32_t blk = gb - M.blk_base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t k = blk * M2_TB + threadIdx.x;
  const bool valid = k < M.n;
  const float2* __restrict__ pts = M.pts;
  const uint32_t* __restrict__ ss = M.strip_start;
  const u128* __restrict__ P = static_cast<const u128*>(M.P);
  const float g1 = M.g2[0], g2 = M.g2[1];
  const int S = (int)M.S, n_strips = (int)M.n_strips;
  const float2 t = pts[valid ? k : M.n - 1];
  const int s = (int)M.skeys[valid ? k : M.n - 1];
  const int s0 = __shfl_sync(FULL_MASK, s, 0);
  const bool uni = __all_sync(FULL_MASK, valid && s == s0);
  if (uni) {
    // bounds of the warp's first and last target in every inside strip
    const float tmin = __shfl_sync(FULL_MASK, t.x, 0), tmax = __shfl_sync(FULL_MASK, t.x, 31);
    for (int q = lane; q < 4 * (2 * S - 1); q += 32) {
      const int sp = s0 + q / 4 - (S - 1);
      uint32_t res = 0;
      if (sp >= 0 && sp < n_strips) {
        const uint32_t a = ss[sp], b = ss[sp + 1];
        const float tq = (q & 1) ? tmax : tmin;
        res = (q & 2) ? first_right(pts, a, b, tq, g1) : first_not_left(pts, a, b, tq, g1);
      }
      s_br[warp][q] = res;
    }
    __syncwarp();
  }
  u128 mo[NM];
#pragma unroll
  for (int m = 0; m < NM; ++m) mo[m] = 0;
  uint32_t cnt = 0;
  float fs = 0.f;
  for (int o = -(S - 1); o <= S - 1; ++o) {
    const int sp = s + o;
    if (sp < 0 || sp >= n_strips) continue;
    const uint32_t a = ss[sp], b = ss[sp + 1];
    if (a == b) continue;
    const float2 yb = M.ybound[sp];
    const bool in_lo = insup(yb.x, t.y, g2), in_hi = insup(yb.y, t.y, g2);
    if ((!in_lo && yb.x >= t.y) || (!in_hi && yb.y <= t.y)) continue;  // all out
    uint32_t llo = a, lhi = b, rlo = a, rhi = b;
    if (uni) {
      const uint32_t* br = s_br[warp] + 4 * (o + S - 1);
      llo = br[0];
      lhi = br[1];
      rlo = br[2];
      rhi = br[3];
    }
    const uint32_t l = first_not_left(pts, llo, lhi, t.x, g1);
    const uint32_t r = first_right(pts, max(rlo, l), rhi, t.x, g1);
    if (l >= r) continue;
    if (in_lo && in_hi) {
      const u128* pl = P + NM * (size_t)l;
      const u128* pr = P + NM * (size_t)r;
#pragma unroll
      for (int m = 0; m < NM; ++m) mo[m] += pr[m] - pl[m];
      cnt += r - l;
    } else {
      float a0 = 0.f, a1 = 0.f;
      uint32_t j = l;
      for (; j + 2 <= r; j += 2) {
        a0 = pair_term(pts[j], t, g1, g2, a0);
        a1 = pair_term(pts[j + 1], t, g1, g2, a1);
      }
      if (j < r) a0 = pair_term(pts[j], t, g1, g2, a0);
      fs += a0 + a1;
    }
  }
  double v = 0.0;     // DM_SUMV: this target's density
  long long fx = 0;   // DM_LOGSUM: log of this target's sum, 2^-48 fixed point
  if (valid) {
    // sum_b d_b M_ab for a = 0, 1, 2 (d_2 = -1), then sum_a c_a (.) (c_2 = -1)
    const u128 TX = quant<23>(t.x), TY = quant<23>(t.y);
    const u128 c0 = quant<46>(g1) - TX * TX, c1 = TX + TX;
    const u128 d0 = quant<46>(g2) - TY * TY, d1 = TY + TY;
    const u128 e0 = d0 * (u128)cnt + d1 * mo[1] - mo[4];
    const u128 e1 = d0 * mo[0] + d1 * mo[3] - mo[6];
    const u128 e2 = d0 * mo[2] + d1 * mo[5] - mo[7];
    // the whole sum in units of 2^-92 g^4: the exact moment part, the
    // partial strips' and the edge strips' sums in fixed point
    const u128 T = c0 * e0 + c1 * e1 - e2;
    uint64_t tlo = (uint64_t)T, thi = (uint64_t)(T >> 64);
    if (fs != 0.f) add_fx92_f32(fs, tlo, thi);
    if (M.acc) add_fx92_f64(M.acc[k], tlo, thi);
    if (!LOGONLY && (mode & (DM_WRITE_F64 | DM_SUMV))) {
      const double dens = M.scale * (s128_to_double(((u128)thi << 64) | tlo) * 0x1p-92);
      if (mode & DM_WRITE_F64) M.out[M.perm[k]] = dens;
      v = dens;
    }
    if (mode & DM_LOGSUM) fx = ilog_fx48(tlo, thi, ilog);
  }
  if (mode & DM_LOGSUM) {  // block-uniform: exact integer block sum
    for (int o = 16; o; o >>= 1) fx += __shfl_xor_sync(FULL_MASK, fx, o);
    if (lane == 0) s_fx[warp] = fx;
    __syncthreads();
    if (threadIdx.x == 0) {
      long long tsum = 0;
      for (uint32_t w = 0; w < M2_TB / 32; ++w) tsum += s_fx[w];
      const uint32_t nv = min(M2_TB, M.n - blk * M2_TB);
      // log density = log T + log(scale) - 92 log 2 = log T + M.logc
      tile_logsum[M.slot_base + blk] = (double)tsum * 0x1p-48 + (double)nv * M.logc;
    }
  } else if (!LOGONLY && (mode & DM_SUMV)) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
    if (lane == 0) s_part[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tsum = 0.0;
      for (uint32_t w = 0; w < M2_TB / 32; ++w) tsum += s_part[w];
      tile_logsum[M.slot_base + blk] = tsum;
    }
  }
}

// Self-test of ilog_fx48 on 128-bit inputs given as (low, high) words.
__global__ void k_ilog_test(const unsigned long long* __restrict__ t, size_t n,
                            const ILogEntry* __restrict__ tab, long long* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = ilog_fx48(t[2 * i], t[2 * i + 1], tab);
}

// One warp per instance; lane l samples the target at quantile (2l+1)/64 of
// dimension 0.
__global__ void k_support_est(const SupportEst* __restrict__ in, uint32_t n_inst,
                              float* __restrict__ est) {
  const uint32_t q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= n_inst) return;  // warp-uniform
  const SupportEst& E = in[q];
  const uint32_t n = E.n;
  const uint32_t pos = (uint32_t)(((2ull * lane + 1) * n) / 64);
  const float xt = key_float(E.keys0[pos]);
  const float yt = E.y1[E.perm0[pos]];
  // window [lo, hi) of dimension 0 within h0 of xt
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t m = lo + ((hi - lo) >> 1);
    if (key_float(E.keys0[m]) <= xt - E.h0) lo = m + 1; else hi = m;
  }
  uint32_t a = lo, b = n;
  while (a < b) {
    const uint32_t m = a + ((b - a) >> 1);
    if (key_float(E.keys0[m]) < xt + E.h0) a = m + 1; else b = m;
  }
  const uint32_t c = a - lo;
  const uint32_t ns = min(c, 32u);
  uint32_t in_y = 0;
  for (uint32_t s = 0; s < ns; ++s) {
    const uint32_t p = lo + (uint32_t)(((uint64_t)s * c) / ns);
    in_y += fabsf(E.y1[E.perm0[p]] - yt) < E.h1 ? 1u : 0u;
  }
  float k = ns ? (float)c * (float)in_y / (float)ns : 0.f;
  for (int o = 16; o; o >>= 1) k += __shfl_xor_sync(FULL_MASK, k, o);
  if (lane == 0) est[q] = k / 32.f;
}

}  // namespace

cudaError_t launch_support_est(cudaStream_t st, const SupportEst* in, uint32_t n_inst,
                               float* est) {
  if (n_inst == 0) return cudaSuccess;
  k_support_est<<<(n_inst + 3) / 4, 128, 0, st>>>(in, n_inst, est);
  return cudaGetLastError();
}

uint32_t moments2d_chunks(uint32_t n) { return (n + M2_CHUNK - 1) / M2_CHUNK; }
uint32_t moments2d_blocks(uint32_t n) { return (n + M2_TB - 1) / M2_TB; }
uint32_t moments2d_block_targets() { return M2_TB; }
size_t moments2d_prefix_bytes(uint32_t n) { return (size_t)NM * 16 * ((size_t)n + 1); }

cudaError_t launch_moments2d_prefix(cudaStream_t st, const Mom2D* ms, uint32_t n_inst,
                                    uint32_t max_n, uint32_t max_strips, void* chunk_tot) {
  if (n_inst == 0) return cudaSuccess;
  u128* tot = static_cast<u128*>(chunk_tot);
  k_m2_ybounds<<<dim3((max_strips + 7) / 8, n_inst), 256, 0, st>>>(ms);
  const dim3 gc(moments2d_chunks(std::max(max_n, 1u)), n_inst);
  k_m2_totals<<<gc, M2_PT, 0, st>>>(ms, tot);
  k_m2_chunks<<<(n_inst + 3) / 4, 128, 0, st>>>(ms, n_inst, tot);
  k_m2_write<<<gc, M2_PT, 0, st>>>(ms, tot);
  return cudaGetLastError();
}

cudaError_t launch_moments2d_targets(cudaStream_t st, const Mom2D* ms, uint32_t n_inst,
                                     const uint32_t* blk_base, uint32_t n_blocks,
                                     const ILogEntry* ilog, double* tile_logsum, uint32_t mode) {
  if (n_inst == 0 || n_blocks == 0) return cudaSuccess;
  if (mode == DM_LOGSUM)
    k_m2_density<true><<<n_blocks, M2_TB, 0, st>>>(ms, n_inst, blk_base, ilog, tile_logsum,
                                                   mode);
  else
    k_m2_density<false><<<n_blocks, M2_TB, 0, st>>>(ms, n_inst, blk_base, ilog, tile_logsum,
                                                    mode);
  return cudaGetLastError();
}

cudaError_t launch_ilog_test(cudaStream_t st, const unsigned long long* t, size_t n,
                             const ILogEntry* tab, long long* out) {
  if (n == 0) return cudaSuccess;
  const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 4096);
  k_ilog_test<<<blocks, 256, 0, st>>>(t, n, tab, out);
  return cudaGetLastError();
}

}  // namespace ent
