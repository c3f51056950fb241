// C ABI and host orchestration of the entropical GB300 density path.
//
// A context (ent_ctx) owns one stream, a grow-only device workspace and the
// statistics of the last call. Every density request is expressed as a batch
// of instances over column views and run by Engine::run:
//
//   views  --colstats-->  min/max/moments (one host sync)
//          --radix sort--> dimension-0 order per view
//   insts  --strip keys + stable radix--> strip-major order, strip starts
//          --tile offsets, gather, plan--> tile descriptors
//          --persistent pair kernel (per d)--> densities / log-sums
//
// The plain combined_densities() replacement is a batch of one instance;
// the batched estimators (mi, transs, uneven entropy batches) submit all of
// their instances at once so that one persistent launch per dimension covers
// every (instance, tile) work item.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/entropical_gb300.h"
#include "api_internal.h"
#include "engine.h"

using namespace ent;

// ------------------------------------------------------------------ arena
void* Arena::alloc(size_t bytes) {
  bytes = (bytes + 255) & ~(size_t)255;
  if (bytes == 0) bytes = 256;
  if (!blocks.empty() && used_in_last + bytes <= blocks.back().size) {
    void* p = static_cast<char*>(blocks.back().ptr) + used_in_last;
    used_in_last += bytes;
    total_used += bytes;
    peak = std::max(peak, total_used);
    return p;
  }
  size_t sz = std::max(bytes, blocks.empty() ? (size_t)64 << 20
                                             : blocks.back().size * 2);
  void* p = nullptr;
  if (cudaMalloc(&p, sz) != cudaSuccess) {
    cudaGetLastError();
    sz = bytes;
    if (cudaMalloc(&p, sz) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
  }
  blocks.push_back({p, sz});
  used_in_last = bytes;
  total_used += bytes;
  peak = std::max(peak, total_used);
  return p;
}

void Arena::coalesce() {
  if (blocks.size() > 1) {
    size_t want = std::max(peak, (size_t)64 << 20);
    for (auto& b : blocks) cudaFree(b.ptr);
    blocks.clear();
    void* p = nullptr;
    if (cudaMalloc(&p, want) == cudaSuccess) blocks.push_back({p, want});
    else cudaGetLastError();
  }
}

void Arena::reset() {
  coalesce();
  used_in_last = 0;
  total_used = 0;
  peak = 0;
}

// Allocations come from the last block only (the tails of earlier ones stay
// unused until the blocks are coalesced).
size_t Arena::spare() const { return blocks.empty() ? 0 : blocks.back().size - used_in_last; }

void Arena::rewind(const Mark& m) {
  if (blocks.size() > m.n_blocks) {
    const Block last = blocks.back();
    for (size_t i = m.n_blocks; i + 1 < blocks.size(); ++i) cudaFree(blocks[i].ptr);
    blocks.resize(m.n_blocks);
    blocks.push_back(last);
    used_in_last = 0;
  } else {
    used_in_last = m.used_in_last;
  }
  total_used = m.total_used;
}

void Arena::release() {
  for (auto& b : blocks) cudaFree(b.ptr);
  blocks.clear();
  used_in_last = total_used = peak = 0;
}

// ---------------------------------------------------------------- context
int Ctx::fail(int status, const std::string& msg) {
  last_error = msg;
  return status;
}

int Ctx::cuda_fail(cudaError_t e, const char* where) {
  last_error = std::string("CUDA error: ") + where + "\n" + cudaGetErrorString(e);
  return ENT_ERR_CUDA;
}

int Ctx::begin_call() {
  last_error.clear();
  stats = ent_call_stats{};
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return cuda_fail(e, "stream sync");
  arena.reset();
  e = cudaMemsetAsync(d_err, 0, sizeof(uint32_t), stream);
  if (e != cudaSuccess) return cuda_fail(e, "memset err");
  cudaEventRecord(ev_call0, stream);
  return ENT_OK;
}

int Ctx::ensure_staging(size_t bytes) {
  if (stage_bytes >= bytes) return ENT_OK;
  for (int k = 0; k < 2; ++k) {
    if (h_stage[k]) cudaFreeHost(h_stage[k]);
    h_stage[k] = nullptr;
  }
  stage_bytes = 0;
  for (int k = 0; k < 2; ++k) {
    cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(&h_stage[k]), bytes,
                                  cudaHostAllocDefault);
    if (e == cudaSuccess && !ev_stage[k])
      e = cudaEventCreateWithFlags(&ev_stage[k], cudaEventDisableTiming);
    if (e != cudaSuccess) {
      if (h_stage[k]) cudaFreeHost(h_stage[k]);
      h_stage[k] = nullptr;
      return cuda_fail(e, "pinned staging");
    }
  }
  stage_bytes = bytes;
  return ENT_OK;
}

int Ctx::end_call() {
  cudaEventRecord(ev_call1, stream);
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return cuda_fail(e, "kernel execution");
  // A call that outgrew the workspace left it in several blocks; join them
  // now, while the work is done, so the next call starts from one block.
  arena.coalesce();
  uint32_t err = 0;
  e = cudaMemcpy(&err, d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "read error word");
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, ev_call0, ev_call1) == cudaSuccess)
    stats.total_ms = ms;
  cudaGetLastError();
  if (err & EF_TIMEOUT)
    return fail(ENT_ERR_TIMEOUT, "a bounded device-side wait expired");
  if (err & EF_NONFINITE)
    return fail(ENT_ERR_NONFINITE, "non-finite coordinate in the selection");
  return ENT_OK;
}

// Table of log_fp64 (common.cuh), computed with the host's libm.
cudaError_t init_log_table(double2** out) {
  std::vector<double2> t(LOG64_TABLE_ENTRIES);
  for (int k = 0; k < 256; ++k) {
    const long double c = 1.0L + ((long double)k + 0.5L) / 256.0L;
    t[k].x = (double)(1.0L / c);
    t[k].y = (double)std::log(c);
  }
  const long double ln2 = std::log(2.0L);
  const double hi = (double)ln2;
  unsigned long long hb;
  std::memcpy(&hb, &hi, sizeof(hb));
  hb &= 0xffffffff00000000ull;
  double hi32;
  std::memcpy(&hi32, &hb, sizeof(hi32));
  t[256].x = hi32;
  t[256].y = (double)(ln2 - (long double)hi32);
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(out), sizeof(double2) * t.size());
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*out, t.data(), sizeof(double2) * t.size(), cudaMemcpyHostToDevice);
}

// Table of the strip-moment epilogue's log (ilog_fx48, moments2d.cu): per
// k, inv = 1/c rounded to FP32 for c = 1 + (k + 1/2)/256, and log(1/inv)
// rounded to 2^-56, computed with the host's libm in long double.
cudaError_t init_ilog_table(ILogEntry** out) {
  std::vector<ILogEntry> t(ILOG_TABLE_ENTRIES);
  for (int k = 0; k < ILOG_TABLE_ENTRIES; ++k) {
    const long double c = 1.0L + ((long double)k + 0.5L) / 256.0L;
    t[k].inv = (float)(1.0L / c);
    t[k].pad = 0.f;
    t[k].l56 = (long long)std::llround(-std::log((long double)t[k].inv) * 0x1p56L);
  }
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(out), sizeof(ILogEntry) * t.size());
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*out, t.data(), sizeof(ILogEntry) * t.size(), cudaMemcpyHostToDevice);
}

// ----------------------------------------------------------------- engine
namespace {

template <class T>
T* arena_upload(Ctx& c, const std::vector<T>& v, cudaError_t* e) {
  T* p = static_cast<T*>(c.arena.alloc(sizeof(T) * std::max<size_t>(v.size(), 1)));
  if (!p) {
    *e = cudaErrorMemoryAllocation;
    return nullptr;
  }
  if (!v.empty())
    *e = cudaMemcpyAsync(p, v.data(), sizeof(T) * v.size(),
                         cudaMemcpyHostToDevice, c.stream);
  else
    *e = cudaSuccess;
  return p;
}

// Segment table for the segmented radix sort over (offset, length) pairs.
struct SegBuild {
  std::vector<uint64_t> off;
  std::vector<uint32_t> len, blk0, blk_seg;
  uint32_t total_blocks = 0;
  void add(uint64_t o, uint32_t n) {
    off.push_back(o);
    len.push_back(n);
    blk0.push_back(total_blocks);
    const uint32_t nb = radix_blocks_for(n);
    for (uint32_t i = 0; i < nb; ++i) blk_seg.push_back((uint32_t)len.size() - 1);
    total_blocks += nb;
  }
  int upload(Ctx& c, SegTableDev* t) {
    cudaError_t e;
    blk0.push_back(total_blocks);
    t->seg_off = arena_upload(c, off, &e);
    if (e != cudaSuccess) return c.cuda_fail(e, "upload seg_off");
    t->seg_len = arena_upload(c, len, &e);
    if (e != cudaSuccess) return c.cuda_fail(e, "upload seg_len");
    t->seg_blk0 = arena_upload(c, blk0, &e);
    if (e != cudaSuccess) return c.cuda_fail(e, "upload seg_blk0");
    t->blk_seg = arena_upload(c, blk_seg, &e);
    if (e != cudaSuccess) return c.cuda_fail(e, "upload blk_seg");
    t->hist = static_cast<uint32_t*>(
        c.arena.alloc(sizeof(uint32_t) * 256 * (size_t)std::max(total_blocks, 1u)));
    if (!t->hist) return c.fail(ENT_ERR_CUDA, "out of device memory");
    return ENT_OK;
  }
};

int bits_for(uint32_t max_key) {
  int b = 0;
  while (b < 32 && (max_key >> b) != 0) ++b;
  return ((b + 7) / 8) * 8;
}

}  // namespace

int sort_views(Ctx& c, const std::vector<ViewSpec>& views, SortedViews* out) {
  cudaError_t e;
  const cudaStream_t st = c.stream;
  const uint32_t nv = (uint32_t)views.size();
  std::vector<ViewDev> hv(nv);
  out->max_n = 0;
  out->off.assign(nv, 0);
  uint64_t vtot = 0;
  for (uint32_t v = 0; v < nv; ++v) {
    hv[v].x = views[v].x;
    hv[v].n = views[v].n;
    hv[v].pad = 0;
    out->off[v] = vtot;
    vtot += views[v].n;
    out->max_n = std::max(out->max_n, views[v].n);
  }
  ViewDev* dv = arena_upload(c, hv, &e);
  if (e != cudaSuccess) return c.cuda_fail(e, "upload views");
  ViewStats* dstats = static_cast<ViewStats*>(c.arena.alloc(sizeof(ViewStats) * nv));
  if (!dstats) return c.fail(ENT_ERR_CUDA, "out of device memory");
  e = launch_colstats(st, dv, nv, dstats);
  if (e != cudaSuccess) return c.cuda_fail(e, "colstats");
  c.stats.kernel_launches += 1;
  out->stats.assign(nv, ViewStats{});
  uint64_t* dvoff = arena_upload(c, out->off, &e);
  if (e != cudaSuccess) return c.cuda_fail(e, "upload view offsets");
  uint32_t* vk = static_cast<uint32_t*>(c.arena.alloc(4 * vtot));
  uint32_t* vvals = static_cast<uint32_t*>(c.arena.alloc(4 * vtot));
  uint32_t* vk2 = static_cast<uint32_t*>(c.arena.alloc(4 * vtot));
  uint32_t* vv2 = static_cast<uint32_t*>(c.arena.alloc(4 * vtot));
  if (!vk || !vvals || !vk2 || !vv2) return c.fail(ENT_ERR_CUDA, "out of device memory");
  e = launch_view_keys(st, dv, dvoff, nv, out->max_n, vk, vvals);
  if (e != cudaSuccess) return c.cuda_fail(e, "view keys");
  c.stats.kernel_launches += 1;
  {
    SegBuild sb;
    for (uint32_t v = 0; v < nv; ++v) sb.add(out->off[v], views[v].n);
    SegTableDev t;
    int s = sb.upload(c, &t);
    if (s) return s;
    e = seg_radix_sort(st, t, nv, sb.total_blocks, vk, vvals, vk2, vv2, 0, 32);
    if (e != cudaSuccess) return c.cuda_fail(e, "view sort");
    c.stats.kernel_launches += 12;
  }
  // the statistics are needed on the host to plan cell grids
  e = cudaMemcpyAsync(out->stats.data(), dstats, sizeof(ViewStats) * nv,
                      cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return c.cuda_fail(e, "read stats");
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return c.cuda_fail(e, "colstats/sort");
  for (uint32_t v = 0; v < nv; ++v)
    if (out->stats[v].nonfinite)
      return c.fail(ENT_ERR_NONFINITE, "non-finite coordinate in the selection");
  out->perm = vvals;
  out->keys = vk;
  return ENT_OK;
}

int Engine::run(Ctx& c, const std::vector<ViewSpec>& views,
                const std::vector<InstSpec>& insts, uint32_t mode, EngineOut* out) {
  cudaError_t e;
  const cudaStream_t st = c.stream;
  const uint32_t nv = (uint32_t)views.size();
  const uint32_t ni = (uint32_t)insts.size();
  if (nv == 0 || ni == 0) return ENT_OK;
  if (nv > 65535 || ni > 65535)
    return c.fail(ENT_ERR_TOO_LARGE, "more than 65535 views or instances in one batch");

  // 1-2. column statistics and value sort of every view
  SortedViews sv;
  int rs = sort_views(c, views, &sv);
  if (rs) return rs;
  const std::vector<ViewStats>& vs = sv.stats;
  const std::vector<uint64_t>& voff = sv.off;
  uint32_t* vvals = sv.perm;

  // 3. host plan of every instance
  std::vector<InstDev> hi(ni);
  std::vector<uint32_t> order;  // instances grouped by dimension
  for (int d = 1; d <= 3; ++d)
    for (uint32_t i = 0; i < ni; ++i)
      if ((int)insts[i].d == d) order.push_back(i);
  uint32_t slot = 0;
  uint32_t max_n = 0;
  uint32_t max_strips = 1;
  // pair body per dimension; the symmetric body has no counting mode
  int var_d[4] = {0, 0, 0, 0};
  bool sym_d[4] = {false, false, false, false};
  bool share = false;  // an instance computes a share of its targets only
  for (uint32_t i = 0; i < ni; ++i) share = share || insts[i].n_parts > 1;
  for (int d = 1; d <= 3; ++d) {
    int v = c.pair_variant[d - 1];
    if (!density_variant_supported(d, c.tile_r[d - 1], v)) v = 0;
    if (pair_uses_acc(v) && ((mode & DM_COUNT) || share)) v = 2;
    if (v == 2 && !density_variant_supported(d, c.tile_r[d - 1], v)) v = 0;
    var_d[d] = v;
  }
  // 2-D under PAIR_MOMENT: which instances the strip moments take. Chosen
  // explicitly: all. By default: those with at least MOMENT_MIN_SUPPORT
  // in-support neighbours per target (a sampled estimate on the sorted views),
  // if they hold MOMENT_MIN_POINTS points together; the symmetric pair kernel
  // takes the rest (it is faster on small supports and on small calls).
  std::vector<char> fused(ni, 0);
  if (var_d[2] == PAIR_MOMENT) {
    uint64_t pts2 = 0;
    for (uint32_t i = 0; i < ni; ++i)
      if (insts[i].d == 2) pts2 += insts[i].n;
    if (!c.moment_auto) {
      for (uint32_t i = 0; i < ni; ++i) fused[i] = insts[i].d == 2;
    } else if (pts2 >= MOMENT_MIN_POINTS) {
      std::vector<SupportEst> se;
      std::vector<uint32_t> se_inst;
      for (uint32_t i = 0; i < ni; ++i) {
        if (insts[i].d != 2) continue;
        const InstSpec& q = insts[i];
        se.push_back({sv.keys + voff[q.view[0]], vvals + voff[q.view[0]], views[q.view[1]].x,
                      q.n, q.h[0], q.h[1]});
        se_inst.push_back(i);
      }
      SupportEst* dse = arena_upload(c, se, &e);
      if (e != cudaSuccess) return c.cuda_fail(e, "upload support estimate");
      float* dest = static_cast<float*>(c.arena.alloc(4 * se.size()));
      if (!dest) return c.fail(ENT_ERR_CUDA, "out of device memory");
      std::vector<float> est(se.size());
      e = launch_support_est(st, dse, (uint32_t)se.size(), dest);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(est.data(), dest, 4 * est.size(), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) return c.cuda_fail(e, "support estimate");
      c.stats.kernel_launches += 1;
      uint64_t pts_m = 0;
      for (size_t q = 0; q < se.size(); ++q)
        if (est[q] >= MOMENT_MIN_SUPPORT) {
          fused[se_inst[q]] = 1;
          pts_m += insts[se_inst[q]].n;
        }
      if (pts_m < MOMENT_MIN_POINTS) std::fill(fused.begin(), fused.end(), 0);
    }
    // The moment prefix sums take 128 B per point; where the device cannot
    // hold them with room to spare, the symmetric pair body runs.
    size_t need = 0;
    for (uint32_t i = 0; i < ni; ++i)
      if (fused[i]) need += moments2d_prefix_bytes(insts[i].n) + 8 * (size_t)insts[i].n;
    const size_t want = need + (need >> 3);
    if (need && want > c.arena.spare()) {  // the device query only when the arena lacks room
      size_t free_b = 0, total_b = 0;
      if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        free_b = 0;
      }
      if (want + ((size_t)1 << 30) > free_b + c.arena.spare())
        std::fill(fused.begin(), fused.end(), 0);
    }
    if (std::find(fused.begin(), fused.end(), 1) == fused.end()) var_d[2] = PAIR_SYM;
  }
  bool sym2 = false;  // a 2-D instance on the symmetric pair kernel
  for (uint32_t i = 0; i < ni; ++i) sym2 = sym2 || (insts[i].d == 2 && !fused[i]);
  for (int d = 1; d <= 3; ++d) sym_d[d] = pair_uses_acc(var_d[d]);
  uint64_t sym_points = 0;
  for (int d = 1; d <= 3; ++d) {
    group_base[d] = slot;
    for (uint32_t i : order) {
      const InstSpec& s = insts[i];
      if ((int)s.d != d) continue;
      InstDev& I = hi[i];
      std::memset(&I, 0, sizeof(I));
      I.n = s.n;
      I.d = s.d;
      const uint32_t np = std::max(s.n_parts, 1u);
      I.t_lo = (uint32_t)((uint64_t)s.n * std::min(s.part, np) / np);
      I.t_hi = (uint32_t)((uint64_t)s.n * std::min(s.part + 1, np) / np);
      max_n = std::max(max_n, s.n);
      double prod_hg2 = 1.0;
      for (uint32_t j = 0; j < s.d; ++j) {
        const ViewStats& st_j = vs[s.view[j]];
        I.x[j] = views[s.view[j]].x;
        // exact power-of-two scale with g = h 2^k in [1, 2), limited so that
        // no scaled coordinate can overflow
        int k = -std::ilogb(s.h[j]) - 1;  // g in [0.5, 1): g^2 - d^2 < 1
        const double amax = std::max(std::fabs((double)st_j.mn), std::fabs((double)st_j.mx));
        while (k > -126 && amax * std::ldexp(1.0, k) > 1e37) --k;
        k = std::max(-126, std::min(126, k));
        I.sc[j] = std::ldexp(1.0f, k);
        const float g = s.h[j] * I.sc[j];
        I.g2[j] = g * g;
        prod_hg2 *= (double)s.h[j] * (double)I.g2[j];
      }
      I.perm0 = vvals + voff[s.view[0]];
      I.S = s.d == 2 ? (fused[i] ? c.moment_cells
                                                : std::max(1u, std::min(4u, s.S)))
                     : (s.d == 3 ? std::max(1u, std::min(2u, s.S3[0] ? s.S3[0] : c.strip_subdiv3))
                                 : 1u);
      I.S2 = s.d == 3 ? std::max(1u, std::min(2u, s.S3[1] ? s.S3[1] : c.strip_subdiv3)) : 1u;
      I.ncell1 = I.ncell2 = 1;
      // Cells of width h/S, widened so that the FP32 cell index (cell_of:
      // error below 1.8e-7 cells per cell of range) keeps two points within
      // h at most S cells apart. Capping the cell count only merges far
      // cells (more candidates, never fewer in-support sources).
      auto cells = [](const ViewStats& v, float hh, uint32_t S, double cap, float* inv_w,
                      uint32_t* ncell) {
        const double range = (double)v.mx - (double)v.mn;
        double w = (double)hh / S * (1.0 + 1e-4);
        const double nc0 = std::min(std::floor(range / w) + 1.0, cap);
        w = (double)hh / S * (1.0 + std::max(1e-4, 6e-7 * nc0 / S));
        *inv_w = (float)(1.0 / w);
        *ncell = (uint32_t)std::min(std::floor(range / w) + 1.0, cap);
      };
      if (s.d >= 2) {
        I.lo1 = vs[s.view[1]].mn;
        cells(vs[s.view[1]], s.h[1], I.S, s.d == 2 ? (1u << 16) : (1u << 10), &I.inv_w1,
              &I.ncell1);
      }
      if (s.d == 3) {
        I.lo2 = vs[s.view[2]].mn;
        cells(vs[s.view[2]], s.h[2], I.S2, 1u << 10, &I.inv_w2, &I.ncell2);
      }
      I.n_strips = I.ncell1 * I.ncell2;
      max_strips = std::max(max_strips, I.n_strips);
      I.scale = (mode & DM_COUNT) ? 1.0 : std::pow(0.75, (double)s.d) / (s.norm * prod_hg2);
      I.out = s.out;
      if (fused[i]) {
        // Edge tiles for the symmetric pair kernel (one run each: the strip S
        // above); its FP64 sums go to acc. The moment kernel runs its own
        // epilogue and writes one slot per block of targets, within tile_cap.
        I.fused = 1;
        I.sym = 1;
        I.tt = (uint32_t)sym_tile_targets(2, PAIR_SYM);
        I.tile_cap = std::max((s.n + I.tt - 1) / I.tt + std::min(I.n_strips, s.n),
                              moments2d_blocks(s.n));
        sym_points += s.n;
      } else {
        // 2-D instances beside strip moments run the symmetric pair kernel
        const int body = (d == 2 && var_d[2] == PAIR_MOMENT) ? PAIR_SYM : var_d[d];
        I.tt = (uint32_t)(sym_d[d] ? sym_tile_targets(d, body)
                                   : density_tile_targets((int)s.d, c.tile_r[s.d - 1]));
        I.tile_cap = (s.n + I.tt - 1) / I.tt + std::min(I.n_strips, s.n);  // tiles
        I.sym = sym_d[d] ? 1u : 0u;
        if (I.sym) sym_points += s.n;
      }
    }
    // Work items: a batch with few tiles for the persistent grid (a single
    // density, say) splits every tile's sources into up to 8 shares so that
    // all CTAs get work; only the symmetric kernel adds its target sums
    // atomically and can take shares.
    uint64_t tiles_d = 0;
    for (uint32_t i : order)
      if ((int)insts[i].d == d) tiles_d += hi[i].tile_cap;
    uint32_t parts = 1;
    const uint64_t want = 16ull * (uint64_t)c.n_sms;
    if (pair_is_sym(var_d[d]) && tiles_d > 0 && tiles_d < want)
      parts = (uint32_t)std::min<uint64_t>(8, (want + tiles_d - 1) / tiles_d);
    for (uint32_t i : order) {
      if ((int)insts[i].d != d) continue;
      InstDev& I = hi[i];
      I.parts = parts;
      I.tile_cap *= parts;
      I.tile_base = slot;
      slot += I.tile_cap;
    }
    group_slots[d] = slot - group_base[d];
  }
  const uint32_t n_slots = slot;

  // buffers per instance
  std::vector<uint32_t> seg_inst;  // d >= 2 instances (strip sort segments)
  std::vector<uint64_t> seg_off;
  uint64_t seg_tot = 0;
  for (uint32_t i = 0; i < ni; ++i) {
    InstDev& I = hi[i];
    const size_t esz = I.d == 1 ? 4 : (I.d == 2 ? 8 : 16);
    I.pts = c.arena.alloc(esz * ((size_t)I.n + 8));
    I.strip_start = static_cast<uint32_t*>(c.arena.alloc(4 * ((size_t)I.n_strips + 1)));
    I.tile_off = static_cast<uint32_t*>(c.arena.alloc(4 * ((size_t)I.n_strips + 1)));
    if (!I.pts || !I.strip_start || !I.tile_off)
      return c.fail(ENT_ERR_CUDA, "out of device memory");
    if (I.d == 1) {
      I.perm = const_cast<uint32_t*>(I.perm0);
    } else {
      seg_inst.push_back(i);
      seg_off.push_back(seg_tot);
      seg_tot += I.n;
    }
  }
  // FP64 sums of the symmetric instances, one block zeroed in the sequence
  double* sym_acc = nullptr;
  if (sym_points) {
    sym_acc = static_cast<double*>(c.arena.alloc(sizeof(double) * sym_points));
    if (!sym_acc) return c.fail(ENT_ERR_CUDA, "out of device memory");
    uint64_t o = 0;
    for (uint32_t i = 0; i < ni; ++i)
      if (hi[i].sym) {
        hi[i].acc = sym_acc + o;
        o += hi[i].n;
      }
  }
  // 1-D instances on the range-sum body: prefix sums and target blocks
  std::vector<Range1D> r1;
  std::vector<uint32_t> r1_blk;
  uint32_t r1_chunks = 0, r1_blocks = 0, r1_max_n = 0;
  if (var_d[1] == PAIR_RANGE) {
    for (uint32_t i : order) {
      if (hi[i].d != 1) continue;
      Range1D r;
      r.y = static_cast<const float*>(hi[i].pts);
      r.acc = hi[i].acc;
      r.P = c.arena.alloc(range1d_prefix_bytes(hi[i].n));
      if (!r.P) return c.fail(ENT_ERR_CUDA, "out of device memory");
      r.n = hi[i].n;
      r.g2 = hi[i].g2[0];
      r.chunk_base = r1_chunks;
      r.blk_base = r1_blocks;
      r1_chunks += range1d_chunks(r.n);
      r1_blocks += range1d_blocks(r.n);
      r1_max_n = std::max(r1_max_n, r.n);
      r1.push_back(r);
      r1_blk.push_back(r.blk_base);
    }
    if (r1.size() > 65535u) return c.fail(ENT_ERR_TOO_LARGE, "too many 1-D instances in one batch");
  }
  Range1D* dr1 = nullptr;
  uint32_t* dr1_blk = nullptr;
  void* r1_tot = nullptr;
  if (!r1.empty()) {
    dr1 = arena_upload(c, r1, &e);
    if (e != cudaSuccess) return c.cuda_fail(e, "upload 1-D ranges");
    dr1_blk = arena_upload(c, r1_blk, &e);
    if (e != cudaSuccess) return c.cuda_fail(e, "upload 1-D blocks");
    r1_tot = c.arena.alloc(32 * (size_t)r1_chunks);
    if (!r1_tot) return c.fail(ENT_ERR_CUDA, "out of device memory");
  }
  uint32_t *sk = nullptr, *svals = nullptr, *sk2 = nullptr, *sv2 = nullptr;
  int strip_bits = bits_for(max_strips);
  if (!seg_inst.empty()) {
    sk = static_cast<uint32_t*>(c.arena.alloc(4 * seg_tot));
    svals = static_cast<uint32_t*>(c.arena.alloc(4 * seg_tot));
    sk2 = static_cast<uint32_t*>(c.arena.alloc(4 * seg_tot));
    sv2 = static_cast<uint32_t*>(c.arena.alloc(4 * seg_tot));
    if (!sk || !svals || !sk2 || !sv2) return c.fail(ENT_ERR_CUDA, "out of device memory");
    const int passes = strip_bits / 8;
    uint32_t* rk = (passes % 2) ? sk2 : sk;
    uint32_t* rv = (passes % 2) ? sv2 : svals;
    for (size_t q = 0; q < seg_inst.size(); ++q) {
      hi[seg_inst[q]].perm = rv + seg_off[q];
      hi[seg_inst[q]].skeys = rk + seg_off[q];
    }
  }
  // 2-D instances on the strip-moment body: strip extents, moment prefix
  // sums and target blocks
  std::vector<Mom2D> m2;
  std::vector<uint32_t> m2_blk;
  uint32_t m2_chunks = 0, m2_blocks = 0, m2_max_n = 0, m2_max_strips = 1;
  if (var_d[2] == PAIR_MOMENT) {
    for (uint32_t i : order) {
      if (!fused[i]) continue;
      Mom2D m;
      m.pts = static_cast<const float2*>(hi[i].pts);
      m.skeys = hi[i].skeys;
      m.strip_start = hi[i].strip_start;
      m.ybound = static_cast<float2*>(c.arena.alloc(8 * (size_t)hi[i].n_strips));
      m.perm = hi[i].perm;
      m.out = hi[i].out;
      m.acc = hi[i].acc;
      m.scale = hi[i].scale;
      m.logc = std::log(hi[i].scale) - 92.0 * std::log(2.0);
      m.slot_base = hi[i].tile_base;
      m.P = c.arena.alloc(moments2d_prefix_bytes(hi[i].n));
      if (!m.ybound || !m.P) return c.fail(ENT_ERR_CUDA, "out of device memory");
      m.n = hi[i].n;
      m.n_strips = hi[i].n_strips;
      m.S = hi[i].S;
      m.g2[0] = hi[i].g2[0];
      m.g2[1] = hi[i].g2[1];
      m.chunk_base = m2_chunks;
      m.blk_base = m2_blocks;
      m2_chunks += moments2d_chunks(m.n);
      m2_blocks += moments2d_blocks(m.n);
      m2_max_n = std::max(m2_max_n, m.n);
      m2_max_strips = std::max(m2_max_strips, m.n_strips);
      m2.push_back(m);
      m2_blk.push_back(m.blk_base);
    }
    if (m2.size() > 65535u) return c.fail(ENT_ERR_TOO_LARGE, "too many 2-D instances in one batch");
  }
  Mom2D* dm2 = nullptr;
  uint32_t* dm2_blk = nullptr;
  void* m2_tot = nullptr;
  if (!m2.empty()) {
    dm2 = arena_upload(c, m2, &e);
    if (e != cudaSuccess) return c.cuda_fail(e, "upload 2-D moments");
    dm2_blk = arena_upload(c, m2_blk, &e);
    if (e != cudaSuccess) return c.cuda_fail(e, "upload 2-D blocks");
    m2_tot = c.arena.alloc(128 * (size_t)m2_chunks);
    if (!m2_tot) return c.fail(ENT_ERR_CUDA, "out of device memory");
  }
  InstDev* di = arena_upload(c, hi, &e);
  if (e != cudaSuccess) return c.cuda_fail(e, "upload instances");

  // Every upload and allocation happens before the kernel sequence, which is
  // captured into one CUDA graph and launched once.
  uint32_t* dseg_inst = nullptr;
  uint64_t* dseg_off = nullptr;
  SegBuild sb;
  SegTableDev segt{};
  if (!seg_inst.empty()) {
    dseg_inst = arena_upload(c, seg_inst, &e);
    if (e != cudaSuccess) return c.cuda_fail(e, "upload seg inst");
    dseg_off = arena_upload(c, seg_off, &e);
    if (e != cudaSuccess) return c.cuda_fail(e, "upload seg off");
    for (size_t q = 0; q < seg_inst.size(); ++q) sb.add(seg_off[q], hi[seg_inst[q]].n);
    int s = sb.upload(c, &segt);
    if (s) return s;
  }
  // instance index for every slot: inst_tile_base must be ascending, so the
  // plan kernel searches the instances in slot order.
  std::vector<uint32_t> slot_order(ni);
  for (uint32_t i = 0; i < ni; ++i) slot_order[i] = i;
  std::sort(slot_order.begin(), slot_order.end(),
            [&](uint32_t a, uint32_t b) { return hi[a].tile_base < hi[b].tile_base; });
  std::vector<InstDev> hi_sorted(ni);
  std::vector<uint32_t> inst_base(ni);
  for (uint32_t r = 0; r < ni; ++r) {
    hi_sorted[r] = hi[slot_order[r]];
    inst_base[r] = hi[slot_order[r]].tile_base;
  }
  InstDev* di_sorted = arena_upload(c, hi_sorted, &e);
  if (e != cudaSuccess) return c.cuda_fail(e, "upload sorted instances");
  uint32_t* dbase = arena_upload(c, inst_base, &e);
  if (e != cudaSuccess) return c.cuda_fail(e, "upload tile bases");
  TileDesc* tiles = static_cast<TileDesc*>(c.arena.alloc(sizeof(TileDesc) * (size_t)n_slots));
  uint64_t* dnsrc = static_cast<uint64_t*>(c.arena.alloc(sizeof(uint64_t) * 3));
  double* tile_ls = static_cast<double*>(c.arena.alloc(sizeof(double) * (size_t)n_slots));
  uint32_t* wc = static_cast<uint32_t*>(c.arena.alloc(sizeof(uint32_t) * 4));
  double* dls = static_cast<double*>(c.arena.alloc(sizeof(double) * ni));
  if (!tiles || !dnsrc || !tile_ls || !wc || !dls)
    return c.fail(ENT_ERR_CUDA, "out of device memory");

  // capture pays off for batches; a call of a few instances launches
  // directly (capture + instantiate cost ~40 us, ~5 % of a 100k-point call)
  const bool graph = c.use_graphs && ni > 4;
  auto rec = [&](cudaEvent_t ev) {
    return graph ? cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal)
                 : cudaEventRecord(ev, st);
  };
  uint32_t launches = 0;
  auto sequence = [&]() -> cudaError_t {
    cudaError_t r;
    // 4. strip partition (stable, keeps dimension-0 order inside strips)
    if (!seg_inst.empty()) {
      r = launch_strip_keys(st, di, dseg_inst, dseg_off, (uint32_t)seg_inst.size(), max_n, sk,
                            svals);
      if (r != cudaSuccess) return r;
      uint32_t *k0 = sk, *v0 = svals, *k1 = sk2, *v1 = sv2;
      r = seg_radix_sort(st, segt, (uint32_t)seg_inst.size(), sb.total_blocks, k0, v0, k1, v1,
                         0, strip_bits);
      if (r != cudaSuccess) return r;
      launches += 1 + 3 * (strip_bits / 8);
    }
    // 5. strips, tiles, points, plan
    if ((r = launch_strip_bounds(st, di, ni, max_strips)) != cudaSuccess) return r;
    if ((r = launch_tile_offsets(st, di, ni)) != cudaSuccess) return r;
    if ((r = launch_gather_pts(st, di, ni, max_n)) != cudaSuccess) return r;
    if ((r = cudaMemsetAsync(dnsrc, 0, sizeof(uint64_t) * 3, st)) != cudaSuccess) return r;
    if (sym_acc &&
        (r = cudaMemsetAsync(sym_acc, 0, sizeof(double) * sym_points, st)) != cudaSuccess)
      return r;
    if ((r = launch_plan(st, di_sorted, ni, dbase, tiles, n_slots, dnsrc)) != cudaSuccess) return r;
    launches += 4;
    // 6. pair kernel, one persistent launch per dimension present; the tile
    // descriptors carry indices into the slot-sorted instance array
    rec(c.ev_k0);
    for (int d = 1; d <= 3; ++d) {
      if (group_slots[d] == 0) continue;
      int launched = 0;
      rec(c.ev_d[d - 1][0]);
      if (d == 1 && var_d[1] == PAIR_RANGE) {
        r = launch_range1d(st, dr1, (uint32_t)r1.size(), r1_max_n, dr1_blk, r1_blocks, r1_tot);
        launches += 3;
      } else if (d == 2 && var_d[2] == PAIR_MOMENT) {
        // The symmetric kernel first: the edge strips of the moment instances
        // and every pair of the other 2-D instances. Then the moments, which
        // add the edge sums and write the slots of their instances (the rest
        // of those instances' slots stay zero).
        r = cudaMemsetAsync(tile_ls + group_base[2], 0, sizeof(double) * group_slots[2], st);
        if (r == cudaSuccess) r = rec(c.ev_m[0][0]);
        if (r == cudaSuccess)
          r = launch_density(st, 2, c.tile_r[1], PAIR_SYM, tiles + group_base[2],
                             group_slots[2], di_sorted, wc + 2, c.d_err,
                             tile_ls + group_base[2], mode, c.n_sms, &launched);
        if (r == cudaSuccess) r = rec(c.ev_m[0][1]);
        if (r == cudaSuccess)
          r = launch_moments2d_prefix(st, dm2, (uint32_t)m2.size(), m2_max_n, m2_max_strips,
                                      m2_tot);
        if (r == cudaSuccess) r = rec(c.ev_m[1][0]);
        if (r == cudaSuccess)
          r = launch_moments2d_targets(st, dm2, (uint32_t)m2.size(), dm2_blk, m2_blocks,
                                       c.d_ilogtab, tile_ls, mode);
        if (r == cudaSuccess) r = rec(c.ev_m[1][1]);
        c.ran_m = true;
        launches += 5;
      } else {
        r = launch_density(st, d, c.tile_r[d - 1], var_d[d], tiles + group_base[d],
                           group_slots[d], di_sorted, wc + d, c.d_err, tile_ls + group_base[d],
                           mode, c.n_sms, &launched);
      }
      if (r != cudaSuccess) return r;
      rec(c.ev_d[d - 1][1]);
      c.ran_d[d - 1] = true;
      launches += 1;
      if (sym_d[d] && (d != 2 || var_d[2] != PAIR_MOMENT || sym2)) {
        r = launch_sym_finish(st, tiles + group_base[d], group_slots[d], di_sorted, c.d_logtab,
                              tile_ls + group_base[d], mode);
        if (r != cudaSuccess) return r;
        launches += 1;
      }
    }
    rec(c.ev_k1);
    c.ran_k = true;
    if (mode & (DM_LOGSUM | DM_SUMV)) {
      if ((r = launch_inst_logsum(st, di_sorted, ni, tile_ls, dls)) != cudaSuccess) return r;
      launches += 1;
    }
    return cudaSuccess;
  };
  if (graph) {
    e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return c.cuda_fail(e, "begin capture");
    cudaError_t es = sequence();
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(st, &g);
    if (es != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return c.cuda_fail(es, "batch kernels");
    }
    if (e != cudaSuccess) return c.cuda_fail(e, "end capture");
    if (c.graph_exec) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(c.graph_exec, g, &info) == cudaSuccess) {
        ++c.graph_updates;
      } else {  // another shape: instantiate this one
        cudaGetLastError();
        cudaGraphExecDestroy(c.graph_exec);
        c.graph_exec = nullptr;
      }
    }
    if (!c.graph_exec) {
      e = cudaGraphInstantiate(&c.graph_exec, g, 0);
      if (e != cudaSuccess) {
        c.graph_exec = nullptr;
        cudaGraphDestroy(g);
        return c.cuda_fail(e, "graph instantiate");
      }
      ++c.graph_instantiations;
    }
    cudaGraphDestroy(g);
    e = cudaGraphLaunch(c.graph_exec, st);
    if (e != cudaSuccess) return c.cuda_fail(e, "graph launch");
  } else {
    e = sequence();
    if (e != cudaSuccess) return c.cuda_fail(e, "batch kernels");
  }
  c.stats.kernel_launches += launches;
  if ((mode & (DM_LOGSUM | DM_SUMV)) && out) {
    out->d_logsum_sorted = dls;
    out->slot_order = slot_order;
  }
  e = cudaMemcpyAsync(c.h_nsrc_d, dnsrc, sizeof(uint64_t) * 3, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return c.cuda_fail(e, "read pair count");
  c.stats.instances += ni;
  c.stats.tiles += n_slots;
  c.pending_pairs = true;
  return ENT_OK;
}

namespace {

// Device bytes an engine run takes per point of an instance (sorted points,
// strip order and its sort buffers, FP64 sums, the 1-D range and 2-D moment
// prefix rows) and per point of a sorted view, rounded up from the MI and TE
// batches' workspace (174 B per 2-D point with the moment rows, under 64 B
// per 1-D or 3-D point), plus the per-instance tables.
constexpr size_t kBatchBytesPerPoint[4] = {0, 64, 192, 64};
constexpr size_t kBatchBytesPerViewPoint = 16;
constexpr size_t kBatchBytesPerInstance = 4096;
constexpr size_t kBatchMaxViews = 65535;

size_t inst_bytes(const InstSpec& s) {
  return (size_t)s.n * kBatchBytesPerPoint[std::min(s.d, 3u)] + kBatchBytesPerInstance;
}

}  // namespace

size_t device_budget(Ctx& c) {
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    cudaGetLastError();
    free_b = 0;
  }
  const size_t avail = free_b + c.arena.spare();
  const size_t reserve = std::max(avail / 8, (size_t)2 << 30);
  return avail > reserve ? avail - reserve : avail / 2;
}

int run_engine_batches(Ctx& c, const std::vector<ViewSpec>& views,
                       const std::vector<InstSpec>& insts, uint32_t mode, BatchDone done,
                       void* arg) {
  if (insts.empty()) return ENT_OK;
  size_t est = 0;
  for (const auto& q : insts) est += inst_bytes(q);
  for (const auto& v : views) est += (size_t)v.n * kBatchBytesPerViewPoint;
  const bool one_run = insts.size() <= c.max_batch_instances && views.size() <= kBatchMaxViews;
  size_t budget = SIZE_MAX;
  if (!one_run || est > c.arena.spare()) budget = device_budget(c);
  if (one_run && est <= budget) {
    Engine eng;
    EngineOut eo;
    int s = eng.run(c, views, insts, mode, &eo);
    if (s) return s;
    return done ? done(arg, 0, insts.size(), eo) : ENT_OK;
  }
  // consecutive runs of as many instances as fit (at least one)
  const Arena::Mark base = c.arena.mark();
  std::vector<uint32_t> remap(views.size(), UINT32_MAX);
  for (size_t q0 = 0; q0 < insts.size();) {
    std::vector<ViewSpec> cv;
    std::vector<InstSpec> ci;
    std::vector<uint32_t> used;  // views mapped for this run
    size_t bytes = 0, q = q0;
    for (; q < insts.size(); ++q) {
      InstSpec I = insts[q];
      size_t add = inst_bytes(I), new_views = 0;
      for (uint32_t j = 0; j < I.d; ++j) {
        bool seen = remap[I.view[j]] != UINT32_MAX;
        for (uint32_t k = 0; k < j; ++k) seen = seen || I.view[k] == I.view[j];
        if (!seen) {
          ++new_views;
          add += (size_t)views[I.view[j]].n * kBatchBytesPerViewPoint;
        }
      }
      if (q > q0 && (bytes + add > budget || ci.size() + 1 > c.max_batch_instances ||
                     cv.size() + new_views > kBatchMaxViews))
        break;
      for (uint32_t j = 0; j < I.d; ++j) {
        uint32_t& r = remap[I.view[j]];
        if (r == UINT32_MAX) {
          r = (uint32_t)cv.size();
          cv.push_back(views[I.view[j]]);
          used.push_back(I.view[j]);
        }
        I.view[j] = r;
      }
      ci.push_back(I);
      bytes += add;
    }
    Engine eng;
    EngineOut eo;
    int s = eng.run(c, cv, ci, mode, &eo);
    if (s == ENT_OK && done) s = done(arg, q0, ci.size(), eo);
    if (s) return s;
    cudaError_t e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return c.cuda_fail(e, "batch");
    c.collect_kernel_stats();
    c.arena.rewind(base);
    for (uint32_t v : used) remap[v] = UINT32_MAX;
    q0 = q;
  }
  return ENT_OK;
}

unsigned Ctx::persistent_grid(uint32_t n_work, const void* kern, int threads, size_t smem) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) !=
      cudaSuccess) {
    cudaGetLastError();
    per_sm = 1;
  }
  uint64_t g = (uint64_t)std::max(per_sm, 1) * (uint64_t)n_sms;
  g = std::min<uint64_t>(g, std::max<uint32_t>(n_work, 1));
  return (unsigned)g;
}

// Adds the kernel times of the runs since the last collection (one engine
// run, or one per batch of a job split into several) to the call's stats.
void Ctx::collect_kernel_stats() {
  float ms = 0.f;
  if (ran_k && cudaEventElapsedTime(&ms, ev_k0, ev_k1) == cudaSuccess) stats.pair_kernel_ms += ms;
  ran_k = false;
  if (ran_m) {
    if (cudaEventElapsedTime(&ms, ev_m[0][0], ev_m[0][1]) == cudaSuccess)
      stats.moment_edge_ms += ms;
    if (cudaEventElapsedTime(&ms, ev_m[1][0], ev_m[1][1]) == cudaSuccess)
      stats.moment_target_ms += ms;
    ran_m = false;
  }
  for (int d = 0; d < 3; ++d) {
    if (ran_d[d] && cudaEventElapsedTime(&ms, ev_d[d][0], ev_d[d][1]) == cudaSuccess)
      stats.pair_kernel_ms_by_dim[d] += ms;
    ran_d[d] = false;
    if (pending_pairs) {
      stats.candidate_pairs_by_dim[d] += h_nsrc_d[d];
      stats.candidate_pairs += h_nsrc_d[d];
    }
  }
  cudaGetLastError();
  pending_pairs = false;
}

// ------------------------------------------------------------------ C ABI
extern "C" {

int ent_create(ent_ctx** out, int device) {
  if (!out) return ENT_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return ENT_ERR_NO_DEVICE;
  }
  if (device < 0) {
    if (cudaGetDevice(&device) != cudaSuccess) return ENT_ERR_CUDA;
  }
  if (device >= n) return ENT_ERR_ARG;
  Ctx* c = new Ctx();
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&c->d_err, 16) != cudaSuccess ||
      cudaEventCreate(&c->ev_call0) != cudaSuccess ||
      cudaEventCreate(&c->ev_call1) != cudaSuccess ||
      cudaEventCreate(&c->ev_k0) != cudaSuccess ||
      cudaEventCreate(&c->ev_k1) != cudaSuccess ||
      cudaEventCreate(&c->ev_d[0][0]) != cudaSuccess ||
      cudaEventCreate(&c->ev_d[0][1]) != cudaSuccess ||
      cudaEventCreate(&c->ev_d[1][0]) != cudaSuccess ||
      cudaEventCreate(&c->ev_d[1][1]) != cudaSuccess ||
      cudaEventCreate(&c->ev_d[2][0]) != cudaSuccess ||
      cudaEventCreate(&c->ev_d[2][1]) != cudaSuccess ||
      cudaEventCreate(&c->ev_m[0][0]) != cudaSuccess ||
      cudaEventCreate(&c->ev_m[0][1]) != cudaSuccess ||
      cudaEventCreate(&c->ev_m[1][0]) != cudaSuccess ||
      cudaEventCreate(&c->ev_m[1][1]) != cudaSuccess ||
      cudaDeviceGetAttribute(&c->n_sms, cudaDevAttrMultiProcessorCount, device) !=
          cudaSuccess) {
    cudaGetLastError();
    delete c;
    return ENT_ERR_CUDA;
  }
  if (const char* g = std::getenv("ENT_NO_GRAPHS")) c->use_graphs = (g[0] == '0');
  if (const char* m = std::getenv("ENT_MAX_BATCH_INSTANCES")) {
    const long v = std::strtol(m, nullptr, 10);
    if (v >= 1 && v <= 65535) c->max_batch_instances = (uint32_t)v;
  }
  if (init_log_table(&c->d_logtab) != cudaSuccess) {
    cudaGetLastError();
    ent_destroy(reinterpret_cast<ent_ctx*>(c));
    return ENT_ERR_CUDA;
  }
  if (init_ilog_table(&c->d_ilogtab) != cudaSuccess) {
    cudaGetLastError();
    ent_destroy(reinterpret_cast<ent_ctx*>(c));
    return ENT_ERR_CUDA;
  }
  *out = reinterpret_cast<ent_ctx*>(c);
  return ENT_OK;
}

void ent_destroy(ent_ctx* ctx) {
  if (!ctx) return;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  c->arena.release();
  cudaFree(c->d_err);
  if (c->d_logtab) cudaFree(c->d_logtab);
  if (c->d_ilogtab) cudaFree(c->d_ilogtab);
  cudaEventDestroy(c->ev_call0);
  cudaEventDestroy(c->ev_call1);
  cudaEventDestroy(c->ev_k0);
  cudaEventDestroy(c->ev_k1);
  for (int d = 0; d < 3; ++d) {
    cudaEventDestroy(c->ev_d[d][0]);
    cudaEventDestroy(c->ev_d[d][1]);
  }
  for (int k = 0; k < 2; ++k) {
    cudaEventDestroy(c->ev_m[k][0]);
    cudaEventDestroy(c->ev_m[k][1]);
  }
  for (int k = 0; k < 2; ++k) {
    if (c->h_stage[k]) cudaFreeHost(c->h_stage[k]);
    if (c->ev_stage[k]) cudaEventDestroy(c->ev_stage[k]);
  }
  cudaStreamDestroy(c->stream);
  delete c;
}

const char* ent_status_string(int s) {
  switch (s) {
    case ENT_OK: return "ok";
    case ENT_ERR_DIM: return "can only compute combined probabilities in 1, 2 or 3 dimensions";
    case ENT_ERR_H_COUNT: return "number of bandwidth parameters does not match number of selected columns";
    case ENT_ERR_TAU_COUNT: return "number of lagtimes (tau) does not match number of selected dimensions";
    case ENT_ERR_ARG: return "invalid argument";
    case ENT_ERR_NONFINITE: return "non-finite coordinate";
    case ENT_ERR_CUDA: return "CUDA error";
    case ENT_ERR_NO_DEVICE: return "no CUDA-compatible GPUs found";
    case ENT_ERR_TIMEOUT: return "device-side wait timed out";
    case ENT_ERR_TOO_LARGE: return "input too large";
    case ENT_ERR_STATE: return "invalid state";
    case ENT_ERR_IO: return "coordinate file unreadable or malformed";
  }
  return "unknown status";
}

int ent_wait_selftest(ent_ctx* ctx) {
  if (!ctx) return ENT_ERR_ARG;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  int s = c->begin_call();
  if (s) return s;
  cudaError_t e = launch_wait_test(c->stream, c->d_err);
  if (e != cudaSuccess) return c->cuda_fail(e, "wait self-test");
  return c->end_call();
}

int ent_log64_selftest(ent_ctx* ctx, const double* x, size_t n, double* out) {
  if (!ctx || (n && (!x || !out))) return ENT_ERR_ARG;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  int s = c->begin_call();
  if (s) return s;
  if (n == 0) return c->end_call();
  double* d = static_cast<double*>(c->arena.alloc(2 * sizeof(double) * n));
  if (!d) return c->fail(ENT_ERR_CUDA, "out of device memory");
  cudaError_t e = cudaMemcpyAsync(d, x, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = launch_log64_test(c->stream, d, n, c->d_logtab, d + n);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return c->cuda_fail(e, "log self-test");
  return c->end_call();
}

int ent_ilog_selftest(ent_ctx* ctx, const uint64_t* t, size_t n, int64_t* out) {
  if (!ctx || (n && (!t || !out))) return ENT_ERR_ARG;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  int s = c->begin_call();
  if (s) return s;
  if (n == 0) return c->end_call();
  unsigned long long* d = static_cast<unsigned long long*>(c->arena.alloc(24 * n));
  if (!d) return c->fail(ENT_ERR_CUDA, "out of device memory");
  long long* dout = reinterpret_cast<long long*>(d + 2 * n);
  cudaError_t e = cudaMemcpyAsync(d, t, 16 * n, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = launch_ilog_test(c->stream, d, n, c->d_ilogtab, dout);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, dout, 8 * n, cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return c->cuda_fail(e, "ilog self-test");
  return c->end_call();
}

int ent_set_tuning(ent_ctx* ctx, const ent_tuning* t) {
  if (!ctx || !t) return ENT_ERR_ARG;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  for (int d = 1; d <= 3; ++d)
    if (t->targets_per_warp[d - 1] && !density_r_supported(d, (int)t->targets_per_warp[d - 1]))
      return c->fail(ENT_ERR_ARG, "unsupported targets_per_warp");
  if (t->cells_per_h > 4) return c->fail(ENT_ERR_ARG, "cells_per_h must be 1..4");
  if (t->cells_per_h3 > 2) return c->fail(ENT_ERR_ARG, "cells_per_h3 must be 1..2");
  if (t->moment_cells_per_h == 1 || t->moment_cells_per_h > 12)
    return c->fail(ENT_ERR_ARG, "moment_cells_per_h must be 2..12");
  if (t->pair_variant > PAIR_SYM + 2) return c->fail(ENT_ERR_ARG, "pair_variant must be 0..6");
  for (int d = 0; d < 3; ++d)
    if (t->pair_variant_by_dim[d] >
        (d == 0 ? PAIR_RANGE + 1 : (d == 1 ? PAIR_MOMENT + 1 : PAIR_SYM + 2)) ||
        (d == 1 && t->pair_variant_by_dim[d] == PAIR_RANGE + 1))
      return c->fail(ENT_ERR_ARG, d == 0   ? "pair_variant_by_dim[0] must be 0..7"
                                  : d == 1 ? "pair_variant_by_dim[1] must be 0..6 or 8"
                                           : "pair_variant_by_dim[2] must be 0..6");
  if (t->pair_variant) {
    for (int d = 0; d < 3; ++d) c->pair_variant[d] = (int)t->pair_variant - 1;
    c->moment_auto = false;
  }
  if (t->pair_variant_by_dim[1]) c->moment_auto = false;
  for (int d = 0; d < 3; ++d)
    if (t->pair_variant_by_dim[d]) c->pair_variant[d] = (int)t->pair_variant_by_dim[d] - 1;
  for (int d = 1; d <= 3; ++d)
    if (t->targets_per_warp[d - 1]) c->tile_r[d - 1] = (int)t->targets_per_warp[d - 1];
  if (t->cells_per_h) c->strip_subdiv = t->cells_per_h;
  if (t->cells_per_h3) c->strip_subdiv3 = t->cells_per_h3;
  if (t->moment_cells_per_h) c->moment_cells = t->moment_cells_per_h;
  return ENT_OK;
}

int ent_get_tuning(const ent_ctx* ctx, ent_tuning* t) {
  if (!ctx || !t) return ENT_ERR_ARG;
  const Ctx* c = reinterpret_cast<const Ctx*>(ctx);
  for (int d = 0; d < 3; ++d) t->targets_per_warp[d] = (uint32_t)c->tile_r[d];
  t->cells_per_h = c->strip_subdiv;
  t->cells_per_h3 = c->strip_subdiv3;
  t->moment_cells_per_h = c->moment_cells;
  t->pair_variant = (uint32_t)c->pair_variant[1] + 1;
  for (int d = 0; d < 3; ++d) t->pair_variant_by_dim[d] = (uint32_t)c->pair_variant[d] + 1;
  return ENT_OK;
}

const char* ent_last_error(const ent_ctx* ctx) {
  if (!ctx) return "";
  return reinterpret_cast<const Ctx*>(ctx)->last_error.c_str();
}

int ent_last_stats(const ent_ctx* ctx, ent_call_stats* s) {
  if (!ctx || !s) return ENT_ERR_ARG;
  *s = reinterpret_cast<const Ctx*>(ctx)->stats;
  return ENT_OK;
}

}  // extern "C"

// Validation shared by the density entry points (densities_common.hxx:7-49).
int validate_selection(Ctx& c, size_t n_rows, size_t n_cols,
                       const uint32_t* i_cols, const float* h,
                       const uint32_t* tau, uint32_t d, size_t* n_sel) {
  if (d < 1 || d > 3)
    return c.fail(ENT_ERR_DIM, ent_status_string(ENT_ERR_DIM));
  if (!i_cols || !h) return c.fail(ENT_ERR_ARG, "null column or bandwidth array");
  uint32_t tmax = 0;
  for (uint32_t j = 0; j < d; ++j) {
    if (i_cols[j] >= n_cols) return c.fail(ENT_ERR_ARG, "column index out of range");
    if (!(h[j] > 0.f) || !std::isfinite(h[j]))
      return c.fail(ENT_ERR_ARG, "bandwidth must be finite and positive");
    if (tau) tmax = std::max(tmax, tau[j]);
  }
  if ((size_t)tmax >= n_rows) return c.fail(ENT_ERR_ARG, "lag not smaller than n_rows");
  if (n_rows > 0xffffff00ull) return c.fail(ENT_ERR_TOO_LARGE, "too many rows");
  *n_sel = n_rows - tmax;
  return ENT_OK;
}

static int densities_impl(ent_ctx* ctx, const float* coords, size_t n_rows,
                          size_t n_cols, const uint32_t* i_cols, const float* h,
                          const uint32_t* tau, uint32_t d, uint32_t flags,
                          double* out, size_t* n_out, bool device_io,
                          bool counts, uint32_t part = 0, uint32_t n_parts = 1,
                          double* logsum_out = nullptr) {
  if (!ctx) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  size_t n_sel = 0;
  s = validate_selection(c, n_rows, n_cols, i_cols, h, tau, d, &n_sel);
  if (s) return s;
  if (n_out) *n_out = n_sel;
  if (!coords || !out) return c.fail(ENT_ERR_ARG, "null coords or output");
  cudaError_t e;
  std::vector<ViewSpec> views(d);
  for (uint32_t j = 0; j < d; ++j) {
    const size_t off = (size_t)i_cols[j] * n_rows + (tau ? tau[j] : 0);
    if (device_io) {
      views[j].x = coords + off;
    } else {
      float* p = static_cast<float*>(c.arena.alloc(4 * n_sel));
      if (!p) return c.fail(ENT_ERR_CUDA, "out of device memory");
      e = cudaMemcpyAsync(p, coords + off, 4 * n_sel, cudaMemcpyHostToDevice, c.stream);
      if (e != cudaSuccess) return c.cuda_fail(e, "copy coordinates");
      views[j].x = p;
    }
    views[j].n = (uint32_t)n_sel;
  }
  double* dout = out;
  if (!device_io) {
    dout = static_cast<double*>(c.arena.alloc(8 * n_sel));
    if (!dout) return c.fail(ENT_ERR_CUDA, "out of device memory");
  }
  std::vector<InstSpec> insts(1);
  InstSpec& I = insts[0];
  I.d = d;
  I.n = (uint32_t)n_sel;
  for (uint32_t j = 0; j < d; ++j) {
    I.view[j] = j;
    I.h[j] = h[j];
  }
  I.norm = counts ? 1.0 : ((flags & ENT_COMPAT_NORM) ? (double)n_rows : (double)n_sel);
  I.out = dout;
  I.S = c.strip_subdiv;
  I.part = part;
  I.n_parts = n_parts;
  Engine eng;
  EngineOut eo;
  const bool want_ls = logsum_out && !counts;
  s = eng.run(c, views, insts, DM_WRITE_F64 | (counts ? DM_COUNT : 0u) | (want_ls ? DM_LOGSUM : 0u),
              want_ls ? &eo : nullptr);
  if (s) return s;
  if (want_ls) {
    e = cudaMemcpyAsync(logsum_out, eo.d_logsum_sorted, sizeof(double), cudaMemcpyDeviceToHost,
                        c.stream);
    if (e != cudaSuccess) return c.cuda_fail(e, "copy log-sum");
  }
  if (!device_io) {
    e = cudaMemcpyAsync(out, dout, 8 * n_sel, cudaMemcpyDeviceToHost, c.stream);
    if (e != cudaSuccess) return c.cuda_fail(e, "copy densities");
  }
  s = c.end_call();
  c.collect_kernel_stats();
  return s;
}

extern "C" {

int ent_densities(ent_ctx* ctx, const float* coords, size_t n_rows,
                  size_t n_cols, const uint32_t* i_cols, const float* h,
                  const uint32_t* tau, uint32_t d, uint32_t flags, double* out,
                  size_t* n_out) {
  return densities_impl(ctx, coords, n_rows, n_cols, i_cols, h, tau, d, flags,
                        out, n_out, false, false);
}

int ent_densities_device(ent_ctx* ctx, const float* d_coords, size_t n_rows,
                         size_t n_cols, const uint32_t* i_cols, const float* h,
                         const uint32_t* tau, uint32_t d, uint32_t flags,
                         double* d_out, size_t* n_out) {
  return densities_impl(ctx, d_coords, n_rows, n_cols, i_cols, h, tau, d, flags,
                        d_out, n_out, true, false);
}

int ent_densities_part_device(ent_ctx* ctx, const float* d_coords, size_t n_rows,
                              size_t n_cols, const uint32_t* i_cols, const float* h,
                              const uint32_t* tau, uint32_t d, uint32_t flags, uint32_t part,
                              uint32_t n_parts, double* d_out, size_t* n_out,
                              double* logsum_out) {
  if (!ctx) return ENT_ERR_ARG;
  if (n_parts == 0 || part >= n_parts) {
    Ctx& c = *reinterpret_cast<Ctx*>(ctx);
    return c.fail(ENT_ERR_ARG, "share index out of range");
  }
  return densities_impl(ctx, d_coords, n_rows, n_cols, i_cols, h, tau, d, flags, d_out, n_out,
                        true, false, part, n_parts, logsum_out);
}

int ent_support_counts(ent_ctx* ctx, const float* coords, size_t n_rows,
                       size_t n_cols, const uint32_t* i_cols, const float* h,
                       const uint32_t* tau, uint32_t d, double* out,
                       size_t* n_out) {
  return densities_impl(ctx, coords, n_rows, n_cols, i_cols, h, tau, d, 0u, out,
                        n_out, false, true);
}

}  // extern "C"
