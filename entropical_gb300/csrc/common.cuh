// Shared device helpers for the entropical GB300 kernels (sm_103a only).
//
// - mbarrier + cp.async.bulk (TMA bulk copy) wrappers with bounded waits:
//   every wait gives up after ENT_WAIT_NS nanoseconds, raises a bit in the
//   device error word and lets the kernel drain and return, so a stuck copy
//   can never hang the GPU.
// - packed f32x2 arithmetic (add/sub/fma .f32x2, sm_100+ family): two FP32
//   lanes per instruction, used to halve issue slots in the pair loops.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#ifndef __CUDACC__
#error "compile with nvcc"
#endif

namespace ent {

// Device error word bits (read back by the host after each call).
enum : uint32_t {
  EF_TIMEOUT = 1u,     // a bounded mbarrier / queue wait gave up
  EF_NONFINITE = 2u,   // NaN or Inf met in an input coordinate
  EF_CAPACITY = 4u,    // a tile needed more run slots than allocated
};

constexpr unsigned long long ENT_WAIT_NS = 2000000000ull;  // 2 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar,
                                                      uint32_t bytes) {
  asm volatile(
      "{ .reg .b64 st; mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], "
      "%1; }" ::"r"(smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; "
      "selp.u32 %0, 1, 0, p; }"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for the phase with the given parity to complete, for at most
// ENT_WAIT_NS. Returns false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer();
  for (uint32_t it = 0; it < (1u << 26); ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 255u && globaltimer() - t0 > ENT_WAIT_NS) return false;
  }
  return false;
}

// Bulk (non-tensor) TMA copy global -> shared, completion counted on `bar`.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src,
                                         uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], "
      "[%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// ---------------------------------------------------------------- f32x2
typedef unsigned long long f32x2;

__device__ __forceinline__ f32x2 pk2(float a, float b) {
  f32x2 r;
  asm("mov.b64 %0, {%1,%2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void upk2(f32x2 v, float& a, float& b) {
  asm("mov.b64 {%0,%1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}

// Kahan-compensated FP32 accumulation of a partial sum x into (s, c).
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

// float -> double by re-biasing the IEEE-754 fields on the integer pipes
// (exact for normal floats; zero and subnormals give 0). The FP64 pipe of
// this GPU runs at a small fraction of the FP32 rate, so conversions on the
// hot path avoid it. Inputs must be finite.
__device__ __forceinline__ double f32_to_f64_int(float v) {
  const uint32_t b = __float_as_uint(v);
  const uint32_t e = (b >> 23) & 0xffu;
  if (e == 0) return 0.0;
  const uint64_t r = ((uint64_t)(b & 0x80000000u) << 32) |
                     ((uint64_t)(e + (1023u - 127u)) << 52) |
                     ((uint64_t)(b & 0x7fffffu) << 29);
  return __longlong_as_double((long long)r);
}

// Natural log in FP64 for the per-point epilogues, with few FP64 operations
// (the FP64 pipe of this GPU runs at a small fraction of the FP32 rate).
// Table reduction (Tang's method): x = m 2^e with m in [1, 2); the top 8 bits
// of m pick c = 1 + (k + 1/2)/256 with FP64 entries {1/c, log c} (computed on
// the host, LOG64_TABLE_ENTRIES = 256 + 1: the last one holds log 2 split in a
// high part with 32 zero low bits, exact in e * hi, and the remainder); then
// r = m/c - 1 in [-2^-9, 2^-9] and log1p(r) = r - r^2/2 + ... + r^7/7 (the
// first omitted term is below 2^-66). log x = (e*ln2_hi + log c) +
// (e*ln2_lo + log1p(r)). Non-normal or non-positive x fall back to log().
constexpr int LOG64_TABLE_ENTRIES = 257;
__device__ __forceinline__ double log_fp64(double x, const double2* __restrict__ tab) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned ex = (unsigned)(b >> 52);  // sign and biased exponent
  if (ex == 0u || ex >= 0x7ffu) return log(x);
  const int e = (int)ex - 1023;
  const unsigned k = (unsigned)(b >> 44) & 0xffu;
  const double m = __longlong_as_double((long long)((b & 0x000fffffffffffffull) |
                                                    0x3ff0000000000000ull));
  const double2 t = __ldg(tab + k);  // {1/c, log c}
  const double2 l2 = __ldg(tab + 256);
  const double r = fma(m, t.x, -1.0);
  double p = fma(r, 1.0 / 7.0, -1.0 / 6.0);
  p = fma(r, p, 1.0 / 5.0);
  p = fma(r, p, -1.0 / 4.0);
  p = fma(r, p, 1.0 / 3.0);
  p = fma(r, p, -0.5);
  p = fma(r * r, p, r);
  const double de = (double)e;
  return fma(de, l2.x, t.y) + fma(de, l2.y, p);
}

// Orderable 32-bit key of a float: unsigned compare == float compare
// (-0.0 sorts just before +0.0; NaN never reaches here).
__device__ __forceinline__ uint32_t float_key(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_float(uint32_t k) {
  uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  return __uint_as_float(u);
}

}  // namespace ent
