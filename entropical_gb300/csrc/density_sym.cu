// Symmetric pair kernel: every unordered (target, source) pair inside the
// candidate runs is evaluated once and added to both points.
//
// The reference sums, for every target i, K(x_i - x_k) over all k
// (densities_omp.cpp:67-159, density_2d.cuh:34-100); the product kernel is
// symmetric, K(x_i - x_k) == K(x_k - x_i) bit for bit (x_i - x_k is the exact
// negation of x_k - x_i), so each pair can serve both sums. The tile plan
// (k_plan with InstDev::sym) keeps, for a tile of targets [tb, tb + tc) in
// strip-major order, only the sources at positions >= tb:
//   * sources in [tb, tb + tc) (the tile itself) are evaluated in both orders
//     and added on the target side only;
//   * sources at >= tb + tc are added to the target (registers) and to the
//     source: each warp stores its per-source sum over its R targets in its
//     own shared-memory row (one float per staged element); once per chunk
//     the four rows are added in a fixed order and flushed into the FP64
//     sums InstDev::acc, so the FP32 part of every sum is deterministic;
//   * a source before tb belongs to an earlier tile, which evaluates the pair.
// Target-side sums are flushed into the same FP64 array once per chunk (warp
// transpose-sum, one FP64 atomic per target), so no per-target compensation
// state is carried and a warp can hold 32 targets. k_sym_finish scales the
// sums and writes densities or per-tile log-sums.
//
// Every mbarrier wait is bounded; on expiry the kernel reports EF_TIMEOUT,
// waits (bounded) for its own copies in flight and returns.
#include <algorithm>

#include "staging.cuh"

namespace ent {
namespace {

constexpr unsigned FULL = 0xffffffffu;

// Staged elements per chunk; shared memory per CTA = chunk buffers x 2 plus
// one float row per warp (NW x CAP floats). 4 warps: 51 KB (d = 1, 2) and
// 38 KB (d = 3), 4 resp. 5 CTAs per SM; 8 warps: 44 / 51 / 34 KB, 3 CTAs.
template <int D, int NW>
struct SymChunk {
  static constexpr int CH = NW == 4 ? (D == 1 ? 2048 : (D == 2 ? 1536 : 768))
                                    : (D == 1 ? 1024 : (D == 2 ? 1024 : 512));
};

template <int D, int R, int MINB, int NW>
__global__ void __launch_bounds__(NW * 32, MINB)
    k_density_sym(const TileDesc* __restrict__ tiles, uint32_t n_slots,
                  const InstDev* __restrict__ insts, uint32_t* work_counter,
                  uint32_t* err) {
  typedef Cfg<D, R, SymChunk<D, NW>::CH, NW> C;
  typedef typename C::P P;
  static_assert(R <= 32 && (R & (R - 1)) == 0, "R: power of two <= 32");
  extern __shared__ __align__(128) unsigned char dsm[];
  P* bufs = reinterpret_cast<P*>(dsm);
  float* srow = reinterpret_cast<float*>(dsm + C::SMEM);  // C::NW rows of CAP floats
  __shared__ __align__(8) uint64_t full[2];
  __shared__ Piece ptab[2][C::MAXP];
  __shared__ uint32_t npc[2];
  __shared__ uint32_t run_lo[MAX_RUNS], run_pre[MAX_RUNS + 1];
  __shared__ uint32_t s_g, s_nr, s_tb, s_tc, s_inst;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  float* myrow = srow + (size_t)warp * C::CAP;
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
      __syncthreads();
      continue;
    }
    const InstDev* I = insts + s_inst;
    const P* __restrict__ pts = reinterpret_cast<const P*>(I->pts);
    double* __restrict__ acc64 = I->acc;
    const uint32_t nr = s_nr, nsrc = run_pre[nr], tb = s_tb, tend = tb + tc;
    const float g2a = I->g2[0], g2b = I->g2[D > 1 ? 1 : 0], g2c = I->g2[D > 2 ? 2 : 0];
    const uint32_t nch = (nsrc + C::CH - 1) / C::CH;
    if (tid == 0 && nch > 0)
      issue_chunk<C>(0, q & 1u, nsrc, nr, run_lo, run_pre, pts, bufs, ptab, npc, full);

    // Register-resident targets of this warp; missing ones sit at +inf, where
    // every term is 0.
    const float FAR = __int_as_float(0x7f800000);
    f32x2 T01[D == 1 ? 1 : R];
    float T2[D == 2 ? 1 : R];
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
    const int tgt = lane >> (5 - Log2<R>::v);
    const bool writer = (lane & ((32 / R) - 1)) == 0;
    const uint32_t my_li = warp * R + tgt;

    bool aborted = false;
    uint32_t ab_q = 0;
    bool ab_next = false;
    for (uint32_t c = 0; c < nch; ++c) {
      const uint32_t qq = q + c, b = qq & 1u;
      if (tid == 0 && c + 1 < nch)
        issue_chunk<C>(c + 1, (qq + 1) & 1u, nsrc, nr, run_lo, run_pre, pts, bufs, ptab,
                       npc, full);
      const bool ok = mbar_wait(&full[b], (qq >> 1) & 1u);
      float acc[R];
#pragma unroll
      for (int r = 0; r < R; ++r) acc[r] = 0.f;
      if (ok) {
        const P* B = bufs + (size_t)b * C::CAP;
        const uint32_t np = npc[b];
        for (uint32_t pi = 0; pi < np; ++pi) {
          const uint32_t s0 = ptab[b][pi].s0, n = ptab[b][pi].n;
          if constexpr (D == 1) {
            f32x2 accp[R / 2];
            f32x2 T[R / 2];
#pragma unroll
            for (int i = 0; i < R / 2; ++i) {
              accp[i] = pk2(0.f, 0.f);
              T[i] = pk2(T2[2 * i], T2[2 * i + 1]);
            }
#pragma unroll 2
            for (uint32_t k = lane; k < n; k += 32) {
              const float s = B[s0 + k];
              const f32x2 S = pk2(s, s);
              f32x2 src0 = pk2(0.f, 0.f), src1 = pk2(0.f, 0.f);
#pragma unroll
              for (int i = 0; i < R / 2; ++i) {
                float da, db;
                upk2(sub2(T[i], S), da, db);
                const f32x2 w = pk2(__saturatef(__fmaf_rn(-da, da, g2a)),
                                    __saturatef(__fmaf_rn(-db, db, g2a)));
                accp[i] = add2(accp[i], w);
                if (i & 1) src1 = add2(src1, w);
                else src0 = add2(src0, w);
              }
              float u0, u1, u2, u3;
              upk2(src0, u0, u1);
              upk2(src1, u2, u3);
              myrow[s0 + k] = (u0 + u1) + (u2 + u3);
            }
#pragma unroll
            for (int i = 0; i < R / 2; ++i) {
              float a0, a1;
              upk2(accp[i], a0, a1);
              acc[2 * i] += a0;
              acc[2 * i + 1] += a1;
            }
          } else {
#pragma unroll 2
            for (uint32_t k = lane; k < n; k += 32) {
              const P s = B[s0 + k];
              const f32x2 S = pk2(s.x, s.y);
              // source-side sum over the warp's R targets in 4 interleaved
              // partials (short rounding and dependency chains)
              float src[4] = {0.f, 0.f, 0.f, 0.f};
              if constexpr (D == 3) {
                // two targets per step, their chains interleaved
#pragma unroll
                for (int r = 0; r < R / 2; ++r) {
                  const int q = r + R / 2;
                  float dxa, dya, dxb, dyb;
                  upk2(sub2(T01[r], S), dxa, dya);
                  upk2(sub2(T01[q], S), dxb, dyb);
                  const float dza = T2[r] - s.z, dzb = T2[q] - s.z;
                  const float wxa = __saturatef(__fmaf_rn(-dxa, dxa, g2a));
                  const float wxb = __saturatef(__fmaf_rn(-dxb, dxb, g2a));
                  const float wya = __saturatef(__fmaf_rn(-dya, dya, g2b));
                  const float wyb = __saturatef(__fmaf_rn(-dyb, dyb, g2b));
                  const float wza = __saturatef(__fmaf_rn(-dza, dza, g2c));
                  const float wzb = __saturatef(__fmaf_rn(-dzb, dzb, g2c));
                  const float pa = wxa * wya, pb = wxb * wyb;
                  acc[r] = __fmaf_rn(pa, wza, acc[r]);
                  acc[q] = __fmaf_rn(pb, wzb, acc[q]);
                  src[r & 3] = __fmaf_rn(pa, wza, src[r & 3]);
                  src[q & 3] = __fmaf_rn(pb, wzb, src[q & 3]);
                }
              }
              if constexpr (D == 2) {
                // two targets per step, their chains interleaved
#pragma unroll
                for (int r = 0; r < R / 2; ++r) {
                  const int q = r + R / 2;
                  float dxa, dya, dxb, dyb;
                  upk2(sub2(T01[r], S), dxa, dya);
                  upk2(sub2(T01[q], S), dxb, dyb);
                  const float wxa = __saturatef(__fmaf_rn(-dxa, dxa, g2a));
                  const float wxb = __saturatef(__fmaf_rn(-dxb, dxb, g2a));
                  const float wya = __saturatef(__fmaf_rn(-dya, dya, g2b));
                  const float wyb = __saturatef(__fmaf_rn(-dyb, dyb, g2b));
                  acc[r] = __fmaf_rn(wxa, wya, acc[r]);
                  acc[q] = __fmaf_rn(wxb, wyb, acc[q]);
                  src[r & 3] = __fmaf_rn(wxa, wya, src[r & 3]);
                  src[q & 3] = __fmaf_rn(wxb, wyb, src[q & 3]);
                }
              }
              myrow[s0 + k] = (src[0] + src[1]) + (src[2] + src[3]);
            }
          }
        }
      }
      if (__syncthreads_or(!ok)) {
        aborted = true;
        ab_q = qq;
        ab_next = c + 1 < nch;
        break;
      }
      // Target side of this chunk: lanes combined, one FP64 add per target.
      const float tot = warp_transpose_sum<R>(acc, lane);
      if (writer && my_li < tc && tot != 0.f)
        atomicAdd(acc64 + tb + my_li, f32_to_f64_int(tot));
      // Source side: every warp wrote every staged element of this chunk
      // into its row; the tile's own targets are complete on the target side.
      const uint32_t np = npc[b];
      for (uint32_t pi = 0; pi < np; ++pi) {
        const Piece p = ptab[b][pi];
        const uint32_t a = p.g0 + (p.s0 - p.o);
        for (uint32_t k = tid; k < p.n; k += C::NT) {
          if (a + k < tend) continue;
          const uint32_t e = p.s0 + k;
          float v = srow[e];
#pragma unroll
          for (int w = 1; w < NW; ++w) v += srow[(size_t)w * C::CAP + e];
          if (v != 0.f) atomicAdd(acc64 + a + k, f32_to_f64_int(v));
        }
      }
      __syncthreads();
    }
    if (aborted) {
      if (tid == 0) {
        atomicOr(err, EF_TIMEOUT);
        mbar_wait(&full[ab_q & 1u], (ab_q >> 1) & 1u);
        if (ab_next) mbar_wait(&full[(ab_q + 1) & 1u], ((ab_q + 1) >> 1) & 1u);
      }
      __syncthreads();
      return;
    }
    q += nch;
  }
}

template <int D, int R, int MINB, int NW>
cudaError_t launch_sym_t(cudaStream_t st, const TileDesc* tiles, uint32_t n_slots,
                         const InstDev* insts, uint32_t* work_counter, uint32_t* err,
                         int n_sms, int* launched) {
  typedef Cfg<D, R, SymChunk<D, NW>::CH, NW> C;
  auto kern = k_density_sym<D, R, MINB, NW>;
  const size_t smem = C::SMEM + (size_t)C::NW * C::CAP * sizeof(float);
  cudaError_t e =
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, C::NT, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  uint64_t grid = (uint64_t)per_sm * (uint64_t)n_sms;
  if (grid > n_slots) grid = n_slots;
  if (grid == 0) grid = 1;
  e = cudaMemsetAsync(work_counter, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  kern<<<(unsigned)grid, C::NT, smem, st>>>(tiles, n_slots, insts, work_counter, err);
  if (launched) *launched = (int)grid;
  return cudaGetLastError();
}

// Symmetric epilogue: one warp per tile slot turns the FP64 sums of its
// targets into densities (scale), written by original index and/or summed
// (log or value) into the slot's tile_logsum.
__global__ void __launch_bounds__(256)
    k_sym_finish(const TileDesc* __restrict__ tiles, uint32_t n_slots,
                 const InstDev* __restrict__ insts, const double2* __restrict__ logtab,
                 double* tile_logsum, uint32_t mode) {
  const uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (g >= n_slots) return;  // warp-uniform
  const TileDesc& T = tiles[g];
  // the strip-moment kernel writes the slots of the instances it owns
  if (insts[T.inst].fused) return;  // warp-uniform
  const uint32_t tc = T.part == 0 ? T.t_count : 0u;  // one slot per tile finishes it
  double ls = 0.0;
  if (tc) {
    const InstDev& I = insts[T.inst];
    for (uint32_t li = lane; li < tc; li += 32) {
      const uint32_t k = T.t_begin + li;
      const double dens = I.scale * I.acc[k];
      if (mode & DM_WRITE_F64) I.out[I.perm[k]] = dens;
      if (mode & DM_LOGSUM) ls += log_fp64(dens, logtab);
      else if (mode & DM_SUMV) ls += dens;
    }
  }
  if (mode & (DM_LOGSUM | DM_SUMV)) {
    for (int o = 16; o; o >>= 1) ls += __shfl_xor_sync(FULL, ls, o);
    if (lane == 0) tile_logsum[g] = ls;
  }
}

// One bounded wait on an mbarrier whose expected bytes never arrive: the
// wait gives up after ENT_WAIT_NS and the kernel reports EF_TIMEOUT (no copy
// is in flight, so the CTA may exit).
__global__ void k_wait_test(uint32_t* err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    mbar_arrive_expect_tx(&bar, 16);
    if (!mbar_wait(&bar, 0)) atomicOr(err, EF_TIMEOUT);
  }
}

__global__ void k_log64_test(const double* __restrict__ x, size_t n,
                             const double2* __restrict__ logtab, double* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = log_fp64(x[i], logtab);
}

}  // namespace

// Shapes of the symmetric bodies: PAIR_SYM 4 warps of 32 targets (d = 1, 2;
// 4 CTAs per SM) / 16 (d = 3; 5 CTAs per SM); PAIR_SYM + 1 8 warps of 16 /
// 8 targets, 3 CTAs per SM. Tiles: 128 targets (d = 1, 2), 64 (d = 3).
int sym_tile_r(int d, int v) {
  if (v == PAIR_SYM) return d == 3 ? 16 : 32;
  return d == 3 ? 8 : 16;
}

int sym_tile_targets(int d, int v) { return (v == PAIR_SYM ? 4 : 8) * sym_tile_r(d, v); }

cudaError_t launch_density_sym(cudaStream_t st, int d, int v, const TileDesc* tiles,
                               uint32_t n_slots, const InstDev* insts,
                               uint32_t* work_counter, uint32_t* err, int n_sms,
                               int* launched) {
  const int r = sym_tile_r(d, v);
  const int nw = v == PAIR_SYM ? 4 : 8;
#define ENT_SYM(D, R, M, W)                                                               \
  if (d == D && r == R && nw == W)                                                        \
    return launch_sym_t<D, R, M, W>(st, tiles, n_slots, insts, work_counter, err, n_sms, \
                                    launched);
  ENT_SYM(1, 32, 4, 4)
  ENT_SYM(1, 16, 3, 8)
  ENT_SYM(2, 32, 4, 4)
  ENT_SYM(2, 16, 3, 8)
  ENT_SYM(3, 16, 5, 4)
  ENT_SYM(3, 8, 3, 8)
#undef ENT_SYM
  return cudaErrorInvalidValue;
}

cudaError_t launch_sym_finish(cudaStream_t st, const TileDesc* tiles,
                              uint32_t n_slots, const InstDev* insts,
                              const double2* logtab, double* tile_logsum, uint32_t mode) {
  if (n_slots == 0) return cudaSuccess;
  const uint64_t blocks = ((uint64_t)n_slots * 32 + 255) / 256;
  k_sym_finish<<<(unsigned)blocks, 256, 0, st>>>(tiles, n_slots, insts, logtab, tile_logsum,
                                                  mode);
  return cudaGetLastError();
}

cudaError_t launch_wait_test(cudaStream_t st, uint32_t* err) {
  k_wait_test<<<1, 32, 0, st>>>(err);
  return cudaGetLastError();
}

cudaError_t launch_log64_test(cudaStream_t st, const double* x, size_t n,
                              const double2* logtab, double* out) {
  if (n == 0) return cudaSuccess;
  const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 4096);
  k_log64_test<<<blocks, 256, 0, st>>>(x, n, logtab, out);
  return cudaGetLastError();
}

}  // namespace ent
