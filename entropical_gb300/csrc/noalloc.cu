// An allocation-free form of the 1-D density (combined_densities with one
// column and no lag) for callers that cannot allocate device memory: hosts
// whose device memory is owned by another framework's pool, long-running
// services that forbid allocation after start-up to avoid latency spikes and
// fragmentation, or plugins that are handed fixed buffers and nothing else.
//
// Every working buffer of the computation -- radix-sort keys and histograms,
// the sorted points, the tile plan, counters -- lives in one file-scope
// device array of NOALLOC_SCRATCH_BYTES, which is why the input size is
// capped at ENT_NOALLOC_MAX_N points. The caller passes the input column and
// the output densities in device memory. This entry point calls no
// cudaMalloc / cudaFree and allocates no host memory either.
//
// Because every call shares the one array, calls that overlap on the GPU
// (two host threads, or two streams in flight at once) race on it and must
// be serialised by the caller. The array keeps the last call's contents; the
// counters that must start at zero are cleared at the start of every call.
//
// The device address of the array is looked up once per device, by the
// first call made with that device current (cudaGetSymbolAddress), and
// cached. With CUDA's lazy module loading (the default) that first call also loads this
// library's device code and the array onto the device, so a service that
// must not allocate after start-up should make one warm-up call then. Every
// call is synchronous: it copies a few small tables from its own stack and
// waits for its work on the stream before it returns.
#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/entropical_gb300.h"
#include "engine.h"

using namespace ent;

namespace {

constexpr uint32_t MAX_N = ENT_NOALLOC_MAX_N;
constexpr uint32_t CHUNK = 2048;  // elements per radix block (sort.cu)
constexpr uint32_t MAX_BLOCKS = (MAX_N + CHUNK - 1) / CHUNK;
constexpr uint32_t R1 = 16, TT = 4 * R1;  // the default 1-D tile shape
constexpr uint32_t MAX_TILES = (MAX_N + TT - 1) / TT + 1;
constexpr size_t NOALLOC_SCRATCH_BYTES = 2u << 20;  // 2 MiB

// Layout of the scratch array (byte offsets, 256-byte aligned).
constexpr size_t al(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t O_KEYS = 0;
constexpr size_t O_VALS = al(O_KEYS + 4ull * MAX_N);
constexpr size_t O_KEYS2 = al(O_VALS + 4ull * MAX_N);
constexpr size_t O_VALS2 = al(O_KEYS2 + 4ull * MAX_N);
constexpr size_t O_HIST = al(O_VALS2 + 4ull * MAX_N);
constexpr size_t O_SEGOFF = al(O_HIST + 4ull * 256 * MAX_BLOCKS);
constexpr size_t O_SEGLEN = al(O_SEGOFF + 8);
constexpr size_t O_SEGBLK0 = al(O_SEGLEN + 4);
constexpr size_t O_BLKSEG = al(O_SEGBLK0 + 8);
constexpr size_t O_VIEW = al(O_BLKSEG + 4ull * MAX_BLOCKS);
constexpr size_t O_VIEWOFF = al(O_VIEW + sizeof(ViewDev));
constexpr size_t O_STATS = al(O_VIEWOFF + 8);
constexpr size_t O_PTS = al(O_STATS + sizeof(ViewStats));
constexpr size_t O_STRIP = al(O_PTS + 4ull * (MAX_N + 8));
constexpr size_t O_TILEOFF = al(O_STRIP + 8);
constexpr size_t O_INST = al(O_TILEOFF + 8);
constexpr size_t O_BASE = al(O_INST + sizeof(InstDev));
constexpr size_t O_TILES = al(O_BASE + 4);
constexpr size_t O_COUNTERS = al(O_TILES + sizeof(TileDesc) * MAX_TILES);
constexpr size_t O_END = al(O_COUNTERS + 64);
static_assert(O_END <= NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the array");

static __device__ __align__(256) unsigned char g_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
unsigned char* g_addr[MAX_DEVICES] = {};

// Device address of the scratch array on the current device (looked up once).
int scratch_address(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (dev < 0 || dev >= MAX_DEVICES) return ENT_ERR_ARG;
  if (!g_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      return ENT_ERR_CUDA;
    }
    g_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_addr[dev];
  return ENT_OK;
}

// A failed CUDA call: clear the error state so it does not surface in the
// caller's next check, and report ENT_ERR_CUDA.
int cuda_error() {
  cudaGetLastError();
  return ENT_ERR_CUDA;
}

}  // namespace

extern "C" int ent_density_1d_noalloc(const float* d_x, size_t n, float h, double* d_out,
                                      void* stream) {
  if (!d_x || !d_out || n == 0) return ENT_ERR_ARG;
  if (n > MAX_N) return ENT_ERR_TOO_LARGE;
  if (!(h > 0.f) || !std::isfinite(h)) return ENT_ERR_ARG;
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return ENT_ERR_NO_DEVICE;
  }
  unsigned char* S = nullptr;
  int rs = scratch_address(dev, &S);
  if (rs) return rs;
  int n_sms = 1;
  if (cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return cuda_error();
  const uint32_t nn = (uint32_t)n;
  uint32_t* keys = reinterpret_cast<uint32_t*>(S + O_KEYS);
  uint32_t* vals = reinterpret_cast<uint32_t*>(S + O_VALS);
  uint32_t* keys2 = reinterpret_cast<uint32_t*>(S + O_KEYS2);
  uint32_t* vals2 = reinterpret_cast<uint32_t*>(S + O_VALS2);
  uint32_t* counters = reinterpret_cast<uint32_t*>(S + O_COUNTERS);
  uint32_t* err = counters;        // error word
  uint32_t* work = counters + 4;   // persistent-kernel work queue
  uint64_t* nsrc = reinterpret_cast<uint64_t*>(counters + 8);

  // Small tables, staged from the host stack.
  const uint32_t nb = (nn + CHUNK - 1) / CHUNK;
  uint64_t seg_off = 0;
  uint32_t seg_len = nn;
  uint32_t seg_blk0[2] = {0, nb};
  uint32_t blk_seg[MAX_BLOCKS];
  for (uint32_t b = 0; b < nb; ++b) blk_seg[b] = 0;
  ViewDev view;
  view.x = d_x;
  view.n = nn;
  view.pad = 0;
  uint64_t view_off = 0;
  cudaError_t e = cudaSuccess;
  e = cudaMemsetAsync(counters, 0, 64, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S + O_SEGOFF, &seg_off, 8, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S + O_SEGLEN, &seg_len, 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S + O_SEGBLK0, seg_blk0, 8, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(S + O_BLKSEG, blk_seg, 4ull * nb, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S + O_VIEW, &view, sizeof(view), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S + O_VIEWOFF, &view_off, 8, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_error();

  // Column statistics: non-finite input and the range for the exact scale.
  const ViewDev* dview = reinterpret_cast<const ViewDev*>(S + O_VIEW);
  ViewStats* dstats = reinterpret_cast<ViewStats*>(S + O_STATS);
  if (launch_colstats(st, dview, 1, dstats) != cudaSuccess) return cuda_error();
  ViewStats vs;
  if (cudaMemcpyAsync(&vs, dstats, sizeof(vs), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return cuda_error();
  if (vs.nonfinite) return ENT_ERR_NONFINITE;

  // Value sort (stable radix sort of orderable keys), in the scratch array.
  if (launch_view_keys(st, dview, reinterpret_cast<const uint64_t*>(S + O_VIEWOFF), 1, nn, keys,
                       vals) != cudaSuccess)
    return cuda_error();
  SegTableDev t;
  t.seg_off = reinterpret_cast<const uint64_t*>(S + O_SEGOFF);
  t.seg_len = reinterpret_cast<const uint32_t*>(S + O_SEGLEN);
  t.seg_blk0 = reinterpret_cast<const uint32_t*>(S + O_SEGBLK0);
  t.blk_seg = reinterpret_cast<const uint32_t*>(S + O_BLKSEG);
  t.hist = reinterpret_cast<uint32_t*>(S + O_HIST);
  if (seg_radix_sort(st, t, 1, nb, keys, vals, keys2, vals2, 0, 32) != cudaSuccess)
    return cuda_error();

  // One 1-D instance: exact power-of-two scale, one strip, tiles of TT.
  InstDev I;
  std::memset(&I, 0, sizeof(I));
  I.x[0] = d_x;
  I.n = nn;
  I.d = 1;
  I.S = 1;
  I.n_strips = 1;
  I.ncell1 = I.ncell2 = 1;
  // g = h 2^k in [0.5, 1), as the library's other entry points scale it
  // (the saturating pair bodies need g^2 < 1; this one uses the min-based body)
  int k = -std::ilogb(h) - 1;
  const double amax = std::fmax(std::fabs((double)vs.mn), std::fabs((double)vs.mx));
  while (k > -126 && amax * std::ldexp(1.0, k) > 1e37) --k;
  k = k < -126 ? -126 : (k > 126 ? 126 : k);
  I.sc[0] = std::ldexp(1.0f, k);
  const float g = h * I.sc[0];
  I.g2[0] = g * g;
  I.perm0 = vals;
  I.perm = vals;
  I.skeys = nullptr;
  I.pts = S + O_PTS;
  I.strip_start = reinterpret_cast<uint32_t*>(S + O_STRIP);
  I.tile_off = reinterpret_cast<uint32_t*>(S + O_TILEOFF);
  I.tt = TT;
  I.tile_cap = (nn + TT - 1) / TT + 1;
  I.t_lo = 0;  // every target
  I.t_hi = nn;
  I.tile_base = 0;
  I.scale = 0.75 / ((double)nn * (double)h * (double)I.g2[0]);
  I.out = d_out;
  uint32_t base0 = 0;
  InstDev* dinst = reinterpret_cast<InstDev*>(S + O_INST);
  if (cudaMemcpyAsync(dinst, &I, sizeof(I), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(S + O_BASE, &base0, 4, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return cuda_error();
  TileDesc* tiles = reinterpret_cast<TileDesc*>(S + O_TILES);
  if (launch_strip_bounds(st, dinst, 1, I.n_strips) != cudaSuccess ||
      launch_tile_offsets(st, dinst, 1) != cudaSuccess ||
      launch_gather_pts(st, dinst, 1, nn) != cudaSuccess ||
      launch_plan(st, dinst, 1, reinterpret_cast<const uint32_t*>(S + O_BASE), tiles, I.tile_cap,
                  nsrc) != cudaSuccess)
    return cuda_error();
  int launched = 0;
  if (launch_density(st, 1, (int)R1, tiles, I.tile_cap, dinst, work, err, nullptr, DM_WRITE_F64,
                     n_sms, &launched) != cudaSuccess)
    return cuda_error();
  uint32_t herr = 0;
  if (cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return cuda_error();
  if (herr & EF_TIMEOUT) return ENT_ERR_TIMEOUT;
  return ENT_OK;
}
