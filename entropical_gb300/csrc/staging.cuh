// Shared-memory staging of candidate-source runs for the persistent pair
// kernels (density and AMISE convolution): chunking of up to MAX_RUNS
// contiguous runs, 16-byte aligned cp.async.bulk copies completing on an
// mbarrier, and the warp-transposed lane reduction of R per-target sums.
#pragma once

#include "engine.h"

namespace ent {

constexpr unsigned FULL_MASK = 0xffffffffu;

// ------------------------------------------------------- pair kernel
template <int D> struct PtType;
template <> struct PtType<1> { typedef float T; };
template <> struct PtType<2> { typedef float2 T; };
template <> struct PtType<3> { typedef float4 T; };

// CHX: elements per staged chunk (0 = default for the dimension); NWX warps
template <int D, int R, int CHX = 0, int NWX = 4>
struct Cfg {
  static constexpr int NW = NWX;
  static constexpr int NT = NW * 32;
  static constexpr int TT = NW * R;
  typedef typename PtType<D>::T P;
  static constexpr int E = sizeof(P);
  static constexpr int A = 16 / E;  // 16-byte alignment, in elements
  static constexpr int CH = CHX ? CHX : ((D == 1) ? 4096 : (D == 2 ? 2048 : 1024));
  static constexpr int MAXP = MAX_RUNS + 1;
  static constexpr int CAP = CH + 2 * A * MAXP;
  static constexpr size_t SMEM = 2 * (size_t)CAP * E;
};

struct Piece {
  uint32_t s0;   // shared-memory element index of the first exact element
  uint32_t n;    // exact elements
  uint32_t g0;   // first copied element (16-byte aligned) in the points array
  uint32_t cnt;  // copied elements
  uint32_t o;    // shared-memory element offset of the copy
};

template <class C>
__device__ __forceinline__ void issue_chunk(
    uint32_t c, uint32_t b, uint32_t nsrc, uint32_t nr, const uint32_t* run_lo,
    const uint32_t* run_pre, const typename C::P* pts, typename C::P* bufs,
    Piece (*ptab)[C::MAXP], uint32_t* npc, uint64_t* full) {
  const uint32_t begin = c * C::CH;
  const uint32_t end = min(begin + (uint32_t)C::CH, nsrc);
  uint32_t np = 0, o = 0, bytes = 0;
  for (uint32_t r = 0; r < nr; ++r) {
    const uint32_t rb = run_pre[r], re = run_pre[r + 1];
    if (re <= begin || rb >= end) continue;
    const uint32_t a = run_lo[r] + (max(begin, rb) - rb);
    const uint32_t e = run_lo[r] + (min(end, re) - rb);
    const uint32_t a0 = a & ~(uint32_t)(C::A - 1);
    const uint32_t e0 = (e + C::A - 1) & ~(uint32_t)(C::A - 1);
    Piece p;
    p.s0 = o + (a - a0);
    p.n = e - a;
    p.g0 = a0;
    p.cnt = e0 - a0;
    p.o = o;
    ptab[b][np++] = p;
    o += e0 - a0;
    bytes += (e0 - a0) * C::E;
  }
  npc[b] = np;
  fence_proxy_async_smem();
  mbar_arrive_expect_tx(&full[b], bytes);
  typename C::P* dst = bufs + (size_t)b * C::CAP;
  for (uint32_t i = 0; i < np; ++i) {
    const Piece p = ptab[b][i];
    bulk_g2s(dst + p.o, pts + p.g0, p.cnt * C::E, &full[b]);
  }
}

// Sum v[0..R) over the 32 lanes so that lane l ends with the total of
// target (l >> (5 - log2 R)); 2R-2 + (5 - log2 R) shuffles.
template <int R>
__device__ __forceinline__ float warp_transpose_sum(float (&v)[R], int lane) {
#pragma unroll
  for (int cnt = R, mask = 16; cnt > 1; cnt >>= 1, mask >>= 1) {
    const bool up = (lane & mask) != 0;
#pragma unroll
    for (int i = 0; i < cnt / 2; ++i) {
      const float send = up ? v[i] : v[i + cnt / 2];
      const float keep = up ? v[i + cnt / 2] : v[i];
      v[i] = keep + __shfl_xor_sync(FULL_MASK, send, mask);
    }
  }
  float x = v[0];
#pragma unroll
  for (int mask = 32 / R / 2; mask >= 1; mask >>= 1)
    x += __shfl_xor_sync(FULL_MASK, x, mask);
  return x;
}

template <int R>
struct Log2 {
  static constexpr int v = (R <= 1) ? 0 : 1 + Log2<R / 2>::v;
};
template <>
struct Log2<1> {
  static constexpr int v = 0;
};


}  // namespace ent
