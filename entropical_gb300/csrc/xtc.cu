// XTC trajectories: the second format behind the reference's coordinate
// files. CoordsFile::open (coords_file/coords_file.cpp:137-145) gives a name
// ending in ".xtc" to XtcHandler, whose next() returns one frame as a row of
// 3 * natoms floats (x0, y0, z0, x1, ...; coords_file.cpp:90-110) and whose
// write() appends one such row as a frame (precision 1000, zero box, step and
// time = the row number; coords_file.cpp:112-126). The codec is GROMACS'
// XTC, vendored by the reference as xdrfile (Frans van Hoesel's coordinate
// compression: xdrfile.c:761-961 decodes, :963-1255 encodes).
//
// Reading, GB300-first: the file is indexed on the host (one pass over the
// frame headers) and copied whole to device memory through pinned staging
// buffers filled by all host threads; what crosses the host link is the
// compressed file, not the floats. Each frame is one serial bit stream (the
// position of every atom group follows from the groups before it), so the
// device decodes in two passes: a walk per frame reads only the flag and run
// bits, validates the frame and records the decoder's state at every 64th
// atom; then one thread per 64-atom segment decodes the packed values
// straight into the column-major coordinate matrix the density calls take
// (column 3a + c holds coordinate c of atom a over all frames; threads of
// consecutive frames write neighbouring addresses).
//
// Frame layout (XDR: big-endian 4-byte units): magic 1995, natoms, step,
// time, box[9], natoms again; natoms <= 9: 3 * natoms raw floats; else
// precision, minint[3], maxint[3], smallidx, byte count and the compressed
// bits (byte count bytes, zero-padded to a multiple of 4).
//
// Reading stops at the first frame that does not parse (wrong magic, another
// atom count, truncated), as XtcHandler::next stops at the first failing
// read_xtc. Differences from the reference, all on input the reference
// mishandles: a compressed body that decodes past its byte count, into more
// atoms than the frame has, or with a table index or range outside the
// format's is ENT_ERR_IO (the reference reads on or divides by zero); the
// writer refuses coordinates that overflow 32-bit integers at the precision
// and atoms so far apart that the format's table runs out (the reference
// prints a warning and writes a frame it cannot read back).
#include <cuda_runtime.h>
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/entropical_gb300.h"
#include "api_internal.h"

namespace {

// The format's table of small-integer ranges (xdrfile.c:743-753): entry k is
// about 2^(k/3), so three values below entry k fit in k bits; entries 0..8
// are unused. The values, including the irregular ones, are part of the
// format and must match every other XTC codec.
#define XTC_RANGES                                                                          \
  {0,       0,       0,        0,        0,       0,       0,       0,       0,       8,      \
   10,      12,      16,       20,       25,      32,      40,      50,      64,      80,     \
   101,     128,     161,      203,      256,     322,     406,     512,     645,     812,    \
   1024,    1290,    1625,     2048,     2580,    3250,    4096,    5060,    6501,    8192,   \
   10321,   13003,   16384,    20642,    26007,   32768,   41285,   52015,   65536,   82570,  \
   104031,  131072,  165140,   208063,   262144,  330280,  416127,  524287,  660561,  832255, \
   1048576, 1321122, 1664510,  2097152,  2642245, 3329021, 4194304, 5284491, 6658042, 8388607, \
   10568983, 13316085, 16777216}
constexpr int XTC_FIRST = 9;
constexpr int XTC_LAST = 73;  // entries
constexpr int XTC_MAGIC = 1995;
constexpr size_t XTC_HEAD = 56;     // magic .. second natoms
constexpr size_t XTC_CHEAD = 92;    // .. byte count, compressed frames
constexpr uint32_t XTC_DECODE_THREADS = 128;

const int h_ranges[XTC_LAST] = XTC_RANGES;
__constant__ int c_ranges[XTC_LAST] = XTC_RANGES;

thread_local std::string g_xtc_error;

inline uint32_t be32(const uint8_t* p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}
inline void put_be32(std::vector<uint8_t>& o, uint32_t v) {
  o.push_back((uint8_t)(v >> 24));
  o.push_back((uint8_t)(v >> 16));
  o.push_back((uint8_t)(v >> 8));
  o.push_back((uint8_t)v);
}
inline uint32_t f2u(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}

unsigned host_threads() {
  const unsigned t = std::thread::hardware_concurrency();
  return std::max(1u, std::min(t, 64u));
}

// ------------------------------------------------------------ file index

struct XtcIndex {
  uint32_t natoms = 0;
  std::vector<uint64_t> frame;  // byte offset of each frame
  uint64_t end = 0;             // one past the last frame read
};

struct Fd {
  int fd = -1;
  ~Fd() {
    if (fd >= 0) close(fd);
  }
};

bool pread_all(int fd, uint8_t* dst, size_t len, uint64_t off) {
  while (len) {
    const ssize_t r = pread(fd, dst, len, (off_t)off);
    if (r <= 0) return false;
    dst += r;
    len -= (size_t)r;
    off += (uint64_t)r;
  }
  return true;
}

// Walks the frame headers through a read-only mapping of the file: one
// header read per frame, no system call per frame.
bool index_xtc(const char* path, XtcIndex* ix, std::string* err) {
  Fd f;
  f.fd = open(path, O_RDONLY);
  if (f.fd < 0) {
    *err = std::string("cannot open ") + path;
    return false;
  }
  struct stat st;
  if (fstat(f.fd, &st) != 0) {
    *err = "cannot stat the file";
    return false;
  }
  const uint64_t size = (uint64_t)st.st_size;
  const uint8_t* m = nullptr;
  if (size >= XTC_HEAD) {
    void* p = mmap(nullptr, (size_t)size, PROT_READ, MAP_PRIVATE, f.fd, 0);
    if (p == MAP_FAILED) {
      *err = "cannot map the file";
      return false;
    }
    m = static_cast<const uint8_t*>(p);
  }
  uint64_t off = 0;
  while (m && off + XTC_HEAD <= size) {
    const uint8_t* h = m + off;
    const int32_t magic = (int32_t)be32(h), natoms = (int32_t)be32(h + 4);
    const int32_t lsize = (int32_t)be32(h + 52);
    if (magic != XTC_MAGIC || natoms <= 0 || lsize != natoms) break;
    if (ix->natoms == 0) ix->natoms = (uint32_t)natoms;
    if ((uint32_t)natoms != ix->natoms) break;
    uint64_t len;
    if (natoms <= 9) {
      len = XTC_HEAD + 12ull * (uint64_t)natoms;
    } else {
      if (off + XTC_CHEAD > size) break;
      len = XTC_CHEAD + (((uint64_t)be32(h + XTC_CHEAD - 4) + 3) & ~3ull);
    }
    if (off + len > size) break;
    ix->frame.push_back(off);
    off += len;
  }
  if (m) munmap(const_cast<uint8_t*>(m), (size_t)size);
  ix->end = off;
  if (ix->frame.empty()) {
    *err = std::string(path) + ": no XTC frame";
    return false;
  }
  if (ix->frame.size() > 0xffffff00ull) {
    *err = "too many frames";
    return false;
  }
  return true;
}

// ----------------------------------------------------------- device decode

// Most-significant-first bit reader over one frame's compressed words,
// started at any bit position. The word after the one being consumed is
// already loaded, so its latency runs under the decoding of the current
// word's bits. Words past the frame's data read as zero.
struct BitReader {
  const uint32_t* w;  // next word to load
  const uint32_t* wend;
  uint64_t acc;  // unread bits, MSB-aligned
  int nacc;
  uint32_t next;  // the next word, loaded ahead (raw byte order)
  uint64_t pos;   // bits consumed from the start of the data

  __device__ __forceinline__ void start(const uint32_t* data, const uint32_t* end,
                                        uint64_t bitpos) {
    w = data + (bitpos >> 5);
    wend = end;
    pos = bitpos;
    const uint32_t first = w < wend ? __byte_perm(__ldg(w), 0, 0x0123) : 0u;
    ++w;
    const int skip = (int)(bitpos & 31u);
    acc = ((uint64_t)first << 32) << skip;
    nacc = 32 - skip;
    next = w < wend ? __ldg(w) : 0u;
    ++w;
  }
  __device__ __forceinline__ uint32_t get(int n) {  // 1 <= n <= 32
    if (nacc < n) {
      const uint32_t v = __byte_perm(next, 0, 0x0123);
      next = w < wend ? __ldg(w) : 0u;
      ++w;
      acc |= (uint64_t)v << (32 - nacc);
      nacc += 32;
    }
    const uint32_t v = (uint32_t)(acc >> (64 - n));
    acc <<= n;
    nacc -= n;
    pos += (uint64_t)n;
    return v;
  }
};

// Reciprocals m(s) = floor((2^64 - 1) / s) of the table's ranges, for
// division by multiplication (Granlund and Montgomery, "Division by invariant
// integers using multiplication", PLDI 1994).
struct RangeInv {
  uint64_t v[XTC_LAST];
};
constexpr RangeInv make_range_inv() {
  RangeInv r{};
  const int t[XTC_LAST] = XTC_RANGES;
  for (int k = 0; k < XTC_LAST; ++k) r.v[k] = t[k] ? ~0ull / (uint64_t)t[k] : 0ull;
  return r;
}
__constant__ RangeInv c_range_inv = make_range_inv();

// q = t / s, returns t % s, for t < s 2^32 (so t < 2^56 and q < 2^32) and
// m = floor((2^64 - 1) / s): the product estimate is q or q - 1.
__device__ __forceinline__ uint32_t divrem_step(uint64_t t, uint32_t s, uint64_t m,
                                                uint32_t* q) {
  uint64_t qq = __umul64hi(t, m);
  uint64_t r = t - qq * s;
  if (r >= s) {
    ++qq;
    r -= s;
  }
  *q = (uint32_t)qq;
  return (uint32_t)r;
}

// v = hi:mid:lo becomes v / s; returns v % s (1 <= s < 2^24, m as above).
__device__ __forceinline__ uint32_t divmod96(uint32_t& hi, uint32_t& mid, uint32_t& lo,
                                             uint32_t s, uint64_t m) {
  uint32_t r = 0;
  if (hi) r = divrem_step(hi, s, m, &hi);
  if (hi | mid) r = divrem_step(((uint64_t)r << 32) | mid, s, m, &mid);
  return divrem_step(((uint64_t)r << 32) | lo, s, m, &lo);
}

// Three integers packed as N = (n0 s1 + n1) s2 + n2 in nbits bits, stored as
// byte chunks least significant first, the last chunk holding what is left
// of nbits (decodeints, xdrfile.c:708-741; n0 is the low 32 bits of the last
// quotient). Up to 64 bits the chunks are read with two reads and put in
// order with a byte reversal; longer numbers chunk by chunk. nbits <= 96.
__device__ __forceinline__ void get_triple(BitReader& b, int nbits, uint32_t s1, uint64_t m1,
                                           uint32_t s2, uint64_t m2, int32_t* n) {
  uint32_t limb[3] = {0u, 0u, 0u};
  if (nbits <= 64) {
    const int k = (nbits - 1) >> 3;  // full byte chunks
    const int r = nbits - 8 * k;     // bits of the last chunk, 1..8
    uint64_t y = 0;                  // the k full chunks, first chunk most significant
    if (k > 4) {
      y = (uint64_t)b.get(32) << (8 * k - 32);
      y |= b.get(8 * k - 32);
    } else if (k > 0) {
      y = b.get(8 * k);
    }
    const uint64_t last = b.get(r);
    // reverse the chunk order: first chunk least significant
    const uint64_t rev = ((uint64_t)__byte_perm((uint32_t)y, 0, 0x0123) << 32) |
                         __byte_perm((uint32_t)(y >> 32), 0, 0x0123);
    const uint64_t v = (k ? rev >> (64 - 8 * k) : 0ull) | (last << (8 * k));
    limb[0] = (uint32_t)v;
    limb[1] = (uint32_t)(v >> 32);
  } else {
    int shift = 0;
    while (nbits > 8) {
      limb[shift >> 5] |= b.get(8) << (shift & 31);
      shift += 8;
      nbits -= 8;
    }
    limb[shift >> 5] |= b.get(nbits) << (shift & 31);
  }
  n[2] = (int32_t)divmod96(limb[2], limb[1], limb[0], s2, m2);
  n[1] = (int32_t)divmod96(limb[2], limb[1], limb[0], s1, m1);
  n[0] = (int32_t)limb[0];
}

__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) {
  return (int32_t)((uint32_t)a + (uint32_t)b);
}

struct DecodeOut {
  float* out;
  size_t col_stride, row_stride;
  const int32_t* col_map;  // 3 natoms entries: output column or -1 (null: identity)
  __device__ __forceinline__ void put(uint32_t f, uint32_t a, const int32_t* v, float inv) const {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int32_t col = col_map ? __ldg(col_map + 3 * a + c) : (int32_t)(3 * a + c);
      if (col >= 0)
        out[(size_t)col * col_stride + (size_t)f * row_stride] =
            __fmul_rn(__int2float_rn(v[c]), inv);
    }
  }
};

enum : uint32_t {
  XERR_NONE = 0,
  XERR_INDEX = 1,    // table index outside the format's
  XERR_RANGE = 2,    // empty or 32-bit coordinate range
  XERR_ATOMS = 3,    // a run past the frame's atom count
  XERR_OVERRUN = 4,  // decoded past the byte count
  XERR_BIG = 5,      // a compressed frame of 256 MB or more
};

__device__ void xtc_fail(uint32_t* err, uint32_t code, uint32_t frame) {
  if (atomicCAS(err, 0u, code) == 0u) err[1] = frame;
}

// Atoms per decoding segment: the walk records the decoder's state at the
// first atom group that starts at or after every multiple of XTC_SEG_ATOMS.
constexpr uint32_t XTC_SEG_ATOMS = 64;

// Decoder state at the start of an atom group: the bit position, the atom
// index, the small-integer table index and the run length (which carries
// over groups whose flag bit is 0). Nothing else crosses groups: the group's
// large atom resets the previous coordinates.
struct XtcCheckpoint {
  uint64_t pos;
  uint32_t atom;
  uint16_t smallidx;
  uint16_t run;
};

// The constants of one compressed frame (xdrfile.c:761-840).
struct FrameHead {
  const uint32_t* data;
  const uint32_t* dend;
  uint32_t n_bytes;
  int32_t minint[3];
  uint32_t size[3];
  uint64_t m1, m2;  // reciprocals of size[1], size[2]
  int bits_d[3];    // large ranges: bits per coordinate
  int bitsize;      // else: bits of the packed triple
  bool large;
  float inv;
  int smallidx;
};

__device__ __forceinline__ uint32_t be_word(const uint32_t* p) {
  return __byte_perm(__ldg(p), 0, 0x0123);
}

// Header of frame f (natoms > 9); false (and err set) for a malformed one.
// file_end: one past the uploaded file's last word. The host's index already
// keeps every frame inside the file; the checks here keep the kernels inside
// the buffer even if the file changed between the index and the copy.
__device__ bool parse_head(const uint32_t* fw, uint32_t f, FrameHead& h, uint32_t* err,
                           const uint32_t* file_end) {
  if (fw + 23 > file_end) {
    xtc_fail(err, XERR_OVERRUN, f);
    return false;
  }
  const float precision = __uint_as_float(be_word(fw + 14));
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    h.minint[d] = (int32_t)be_word(fw + 15 + d);
    h.size[d] = be_word(fw + 18 + d) - (uint32_t)h.minint[d] + 1u;
  }
  h.smallidx = (int32_t)be_word(fw + 21);
  h.n_bytes = be_word(fw + 22);
  h.data = fw + 23;
  h.dend = h.data + ((h.n_bytes + 3u) >> 2);
  if (h.dend > file_end || h.dend < h.data) h.dend = file_end;
  if (h.smallidx < XTC_FIRST || h.smallidx >= XTC_LAST) {
    xtc_fail(err, XERR_INDEX, f);
    return false;
  }
  h.large = (h.size[0] | h.size[1] | h.size[2]) > 0xffffffu;
  h.bitsize = 0;
  h.m1 = h.m2 = 0;
#pragma unroll
  for (int d = 0; d < 3; ++d) h.bits_d[d] = 0;
  if (h.large) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      h.bits_d[d] = 32 - __clz(h.size[d]);  // smallest b with size < 2^b
      if (h.bits_d[d] >= 32) {
        xtc_fail(err, XERR_RANGE, f);
        return false;
      }
    }
  } else {
    if (h.size[0] == 0u || h.size[1] == 0u || h.size[2] == 0u) {
      xtc_fail(err, XERR_RANGE, f);
      return false;
    }
    // bit length of size0 size1 size2 (< 2^72)
    const uint64_t p01 = (uint64_t)h.size[0] * h.size[1];
    const uint64_t lo = p01 * h.size[2];
    const uint64_t hi = __umul64hi(p01, h.size[2]);
    h.bitsize = hi ? 128 - __clzll(hi) : 64 - __clzll(lo);
    h.m1 = ~0ull / h.size[1];
    h.m2 = ~0ull / h.size[2];
  }
  h.inv = __double2float_rn(__ddiv_rn(1.0, (double)precision));
  return true;
}

// Pass 1, one walk per frame: goes over the atom groups reading only what
// decides the next group's position (the flag and run bits; the packed
// values are passed over by their bit lengths), validates the frame and
// records a checkpoint at the first group starting at or after every
// multiple of XTC_SEG_ATOMS atoms. xdrfile_decompress_coord_float
// (xdrfile.c:761-961) restated, without the arithmetic.
// stride: threads per frame, 1 or 32. A warp's lanes wait for each other at
// every step, and every step of a walk waits on its own load, so with few
// frames each walk gets a warp of its own (stride 32: lane 0 walks) and waits
// only for its own cache misses; with many frames the warps of 32 walks
// hide each other's waits.
__global__ void __launch_bounds__(XTC_DECODE_THREADS)
    k_xtc_walk(const uint8_t* __restrict__ file, const uint64_t* __restrict__ frame_off,
               uint32_t n_frames, uint32_t natoms, uint32_t max_seg, uint32_t stride,
               const uint32_t* file_end, XtcCheckpoint* __restrict__ cps,
               uint32_t* __restrict__ n_seg, uint32_t* err) {
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid % stride) return;
  const uint64_t fl = tid / stride;
  if (fl >= n_frames) return;
  const uint32_t f = (uint32_t)fl;
  n_seg[f] = 0;
  XtcCheckpoint* cp = cps + (size_t)f * max_seg;
  if (natoms <= 9) {  // raw floats: one segment
    const uint32_t* fw = reinterpret_cast<const uint32_t*>(file + frame_off[f]);
    if (fw + 14 + 3 * natoms > file_end) return xtc_fail(err, XERR_OVERRUN, f);
    cp[0] = XtcCheckpoint{0, 0, 0, 0};
    n_seg[f] = 1;
    return;
  }
  const uint32_t* fw = reinterpret_cast<const uint32_t*>(file + frame_off[f]);
  FrameHead h;
  if (!parse_head(fw, f, h, err, file_end)) return;
  const uint32_t big_bits =
      h.large ? (uint32_t)(h.bits_d[0] + h.bits_d[1] + h.bits_d[2]) : (uint32_t)h.bitsize;
  const uint32_t n_words = (uint32_t)(h.dend - h.data);
  if (n_words >= (1u << 26)) return xtc_fail(err, XERR_BIG, f);  // bit positions < 2^31
  // A serial chain per frame: every instruction waits for the one before,
  // so the loop keeps to 32-bit positions, one funnel shift for the flag and
  // run bits, and v / 3 as (11 v) >> 5 (exact for v < 32).
  uint32_t pos = 0;
  int smallidx = h.smallidx;
  uint32_t n_small = 0;     // atoms of the current run (carried while the flag is 0)
  uint32_t small_bits = 0;  // their bits: n_small * smallidx
  uint32_t i = 0, seg = 0, next_cp = 0;
  while (i < natoms) {
    if (i >= next_cp) {
      if (seg >= max_seg) return xtc_fail(err, XERR_ATOMS, f);  // cannot happen
      cp[seg++] = XtcCheckpoint{pos, i, (uint16_t)smallidx, (uint16_t)(3u * n_small)};
      next_cp = (i / XTC_SEG_ATOMS + 1) * XTC_SEG_ATOMS;
    }
    pos += big_bits;  // the group's large atom
    const uint32_t wi = pos >> 5;
    const uint32_t a = wi < n_words ? be_word(h.data + wi) : 0u;
    const uint32_t b = wi + 1u < n_words ? be_word(h.data + wi + 1u) : 0u;
    const uint32_t top = __funnelshift_l(b, a, pos & 31u);  // bits from pos on
    int is_smaller = 0;
    if (top >> 31) {  // flag: a new run length follows in 5 bits
      const uint32_t v = (top >> 26) & 31u;
      const uint32_t q = (v * 11u) >> 5;  // v / 3
      is_smaller = (int)(v - 3u * q) - 1;
      n_small = q;
      small_bits = q * (uint32_t)smallidx;
      pos += 6;
    } else {
      pos += 1;
    }
    if (i + 1u + n_small > natoms) return xtc_fail(err, XERR_ATOMS, f);
    pos += small_bits;  // the group's small atoms
    i += 1u + n_small;
    if (is_smaller != 0) {
      smallidx += is_smaller;
      if (smallidx < XTC_FIRST || smallidx >= XTC_LAST) return xtc_fail(err, XERR_INDEX, f);
      small_bits = n_small * (uint32_t)smallidx;
    }
  }
  if ((uint64_t)pos > 8ull * h.n_bytes) return xtc_fail(err, XERR_OVERRUN, f);
  n_seg[f] = seg;
}

// Pass 2, one thread per (segment, frame), frames fastest: decodes the atom
// groups from its checkpoint to the next one and writes their atoms.
__global__ void __launch_bounds__(XTC_DECODE_THREADS)
    k_xtc_decode(const uint8_t* __restrict__ file, const uint64_t* __restrict__ frame_off,
                 uint32_t n_frames, uint32_t natoms, uint32_t max_seg,
                 const uint32_t* file_end, const XtcCheckpoint* __restrict__ cps,
                 const uint32_t* __restrict__ n_seg, DecodeOut o, uint32_t* err) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (uint64_t)n_frames * max_seg) return;
  const uint32_t f = (uint32_t)(t % n_frames), seg = (uint32_t)(t / n_frames);
  const uint32_t ns = n_seg[f];
  if (seg >= ns) return;
  const uint32_t* fw = reinterpret_cast<const uint32_t*>(file + frame_off[f]);
  if (natoms <= 9) {
    for (uint32_t a = 0; a < natoms; ++a) {
      for (int c = 0; c < 3; ++c) {
        const int32_t col = o.col_map ? __ldg(o.col_map + 3 * a + c) : (int32_t)(3 * a + c);
        if (col >= 0)
          o.out[(size_t)col * o.col_stride + (size_t)f * o.row_stride] =
              __uint_as_float(be_word(fw + 14 + 3 * a + c));
      }
    }
    return;
  }
  FrameHead h;
  if (!parse_head(fw, f, h, err, file_end)) return;
  const XtcCheckpoint cp = cps[(size_t)f * max_seg + seg];
  const uint32_t end = seg + 1 < ns ? cps[(size_t)f * max_seg + seg + 1].atom : natoms;
  BitReader b;
  b.start(h.data, h.dend, cp.pos);
  int smallidx = cp.smallidx;
  int smallnum = c_ranges[smallidx] / 2;
  int run = cp.run;
  uint32_t i = cp.atom;
  while (i < end) {
    int32_t big[3];
    if (h.large) {
#pragma unroll
      for (int d = 0; d < 3; ++d) big[d] = h.bits_d[d] ? (int32_t)b.get(h.bits_d[d]) : 0;
    } else {
      get_triple(b, h.bitsize, h.size[1], h.m1, h.size[2], h.m2, big);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) big[d] = wadd(big[d], h.minint[d]);
    int is_smaller = 0;
    if (b.get(1)) {
      const int v = (int)b.get(5);
      is_smaller = v % 3 - 1;
      run = v - v % 3;
    }
    const uint32_t n_small = (uint32_t)run / 3u;
    if (i + 1u + n_small > natoms) return xtc_fail(err, XERR_ATOMS, f);
    if (n_small == 0) {
      o.put(f, i, big, h.inv);
      ++i;
    } else {
      const uint32_t ss = (uint32_t)c_ranges[smallidx];
      const uint64_t ms = c_range_inv.v[smallidx];
      int32_t prev[3] = {big[0], big[1], big[2]};
      for (uint32_t k = 0; k < n_small; ++k) {
        int32_t sv[3];
        get_triple(b, smallidx, ss, ms, ss, ms, sv);
#pragma unroll
        for (int d = 0; d < 3; ++d) sv[d] = wadd(wadd(sv[d], prev[d]), -smallnum);
        // the first small atom comes before the large one (the encoder
        // swapped the two: water-like groups compress better)
        o.put(f, i, sv, h.inv);
        if (k == 0) {
          o.put(f, i + 1, big, h.inv);
          i += 2;
        } else {
          i += 1;
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) prev[d] = sv[d];
      }
    }
    if (is_smaller != 0) {
      smallidx += is_smaller;
      if (smallidx < XTC_FIRST || smallidx >= XTC_LAST) return xtc_fail(err, XERR_INDEX, f);
      smallnum = c_ranges[smallidx] / 2;  // as the reference's smaller/smallnum updates give
    }
  }
}

const char* xerr_text(uint32_t code) {
  switch (code) {
    case XERR_INDEX: return "small-integer table index outside the format";
    case XERR_RANGE: return "empty or 32-bit coordinate range";
    case XERR_ATOMS: return "run of small atoms past the atom count";
    case XERR_OVERRUN: return "compressed bits past the byte count";
    case XERR_BIG: return "compressed frame of 256 MB or more";
    default: return "malformed compressed frame";
  }
}

// ------------------------------------------------------------------ encode

// Most-significant-first bit writer (encodebits, xdrfile.c:542-592).
struct BitWriter {
  std::vector<uint8_t> bytes;
  uint64_t acc = 0;  // pending bits in the low nacc bits
  int nacc = 0;
  void put(uint32_t v, int n) {  // 0 <= n <= 32, v < 2^n
    if (n == 0) return;
    acc = (acc << n) | v;
    nacc += n;
    while (nacc >= 8) {
      nacc -= 8;
      bytes.push_back((uint8_t)(acc >> nacc));
    }
    acc &= (1ull << nacc) - 1ull;
  }
  void flush() {
    if (nacc) bytes.push_back((uint8_t)(acc << (8 - nacc)));
    acc = 0;
    nacc = 0;
  }
};

// N = (n0 s1 + n1) s2 + n2 in nbits bits, byte chunks least significant
// first (encodeints, xdrfile.c:594-658).
void put_triple(BitWriter& w, int nbits, const uint32_t* s, const uint32_t* n) {
  unsigned __int128 N = ((unsigned __int128)n[0] * s[1] + n[1]) * s[2] + n[2];
  while (nbits > 8) {
    w.put((uint32_t)(N & 0xffu), 8);
    N >>= 8;
    nbits -= 8;
  }
  w.put((uint32_t)(N & ((1u << nbits) - 1u)), nbits);
}

inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
inline int32_t wabs(int32_t a) { return a < 0 ? (int32_t)(0u - (uint32_t)a) : a; }
inline int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }

// One frame of XtcHandler::write (coords_file.cpp:112-126 -> write_xtc,
// xdrfile_xtc.c:97-108 -> xdrfile_compress_coord_float, xdrfile.c:963-1255).
// x: 3 natoms floats, atom-major.
bool encode_frame(const float* x, uint32_t natoms, int32_t step, float time, float precision,
                  std::vector<uint8_t>* o, std::string* err) {
  put_be32(*o, (uint32_t)XTC_MAGIC);
  put_be32(*o, natoms);
  put_be32(*o, (uint32_t)step);
  put_be32(*o, f2u(time));
  for (int k = 0; k < 9; ++k) put_be32(*o, 0u);  // box
  put_be32(*o, natoms);
  if (natoms <= 9) {
    for (uint32_t k = 0; k < 3 * natoms; ++k) put_be32(*o, f2u(x[k]));
    return true;
  }
  if (precision <= 0.f) precision = 1000.f;
  put_be32(*o, f2u(precision));
  std::vector<int32_t> q(3 * (size_t)natoms);
  int32_t minint[3] = {INT_MAX, INT_MAX, INT_MAX}, maxint[3] = {INT_MIN, INT_MIN, INT_MIN};
  int32_t mindiff = INT_MAX;
  int32_t old[3] = {0, 0, 0};
  for (uint32_t a = 0; a < natoms; ++a) {
    for (int d = 0; d < 3; ++d) {
      const float v = x[3 * a + d];
      if (!std::isfinite(v)) {
        *err = "non-finite coordinate";
        return false;
      }
      // nearest integer as the reference rounds: float product, then +-0.5
      // in double, stored back to float and truncated
      const float prod = v * precision;
      const float lf = (float)(v >= 0.f ? (double)prod + 0.5 : (double)prod - 0.5);
      if (std::fabs(lf) > (float)(INT_MAX - 2)) {
        *err = "coordinate too large for 32-bit integers at this precision";
        return false;
      }
      const int32_t li = (int32_t)lf;
      q[3 * a + d] = li;
      minint[d] = std::min(minint[d], li);
      maxint[d] = std::max(maxint[d], li);
    }
    const int32_t* c = &q[3 * a];
    const int32_t diff =
        (int32_t)((uint32_t)wabs(wsub(old[0], c[0])) + (uint32_t)wabs(wsub(old[1], c[1])) +
                  (uint32_t)wabs(wsub(old[2], c[2])));
    if (a >= 1 && diff < mindiff) mindiff = diff;
    for (int d = 0; d < 3; ++d) old[d] = c[d];
  }
  for (int d = 0; d < 3; ++d) put_be32(*o, (uint32_t)minint[d]);
  for (int d = 0; d < 3; ++d) put_be32(*o, (uint32_t)maxint[d]);
  for (int d = 0; d < 3; ++d)
    if ((float)maxint[d] - (float)minint[d] >= (float)(INT_MAX - 2)) {
      *err = "coordinate range too large for 32-bit integers at this precision";
      return false;
    }
  uint32_t size[3];
  for (int d = 0; d < 3; ++d) size[d] = (uint32_t)maxint[d] - (uint32_t)minint[d] + 1u;
  const bool large = (size[0] | size[1] | size[2]) > 0xffffffu;
  int bits_d[3] = {0, 0, 0}, bitsize = 0;
  if (large) {
    for (int d = 0; d < 3; ++d) {
      int b = 0;
      while (b < 32 && (1ull << b) <= size[d]) ++b;
      bits_d[d] = b;
    }
  } else {
    unsigned __int128 P = (unsigned __int128)size[0] * size[1] * size[2];
    while (P) {
      ++bitsize;
      P >>= 1;
    }
  }
  int smallidx = XTC_FIRST;
  while (smallidx < XTC_LAST && h_ranges[smallidx] < mindiff) ++smallidx;
  const int maxidx = std::min(XTC_LAST, smallidx + 8);
  if (maxidx >= XTC_LAST) {
    *err = "atoms too far apart for the XTC table at this precision";
    return false;
  }
  put_be32(*o, (uint32_t)smallidx);
  const int minidx = maxidx - 8;
  int smaller = h_ranges[std::max(XTC_FIRST, smallidx - 1)] / 2;
  int smallnum = h_ranges[smallidx] / 2;
  uint32_t sizesmall = (uint32_t)h_ranges[smallidx];
  const int larger = h_ranges[maxidx] / 2;
  BitWriter w;
  int32_t prev[3] = {0, 0, 0};
  int prevrun = -1;
  uint32_t i = 0;
  uint32_t small[30];
  while (i < natoms) {
    int32_t* c = &q[3 * (size_t)i];
    int is_smaller;
    if (smallidx < maxidx && i >= 1 && wabs(wsub(c[0], prev[0])) < larger &&
        wabs(wsub(c[1], prev[1])) < larger && wabs(wsub(c[2], prev[2])) < larger)
      is_smaller = 1;
    else if (smallidx > minidx)
      is_smaller = -1;
    else
      is_smaller = 0;
    bool is_small = false;
    if (i + 1 < natoms && wabs(wsub(c[0], c[3])) < smallnum &&
        wabs(wsub(c[1], c[4])) < smallnum && wabs(wsub(c[2], c[5])) < smallnum) {
      // the next atom is close: code it first, this one as its small follower
      for (int d = 0; d < 3; ++d) std::swap(c[d], c[3 + d]);
      is_small = true;
    }
    uint32_t t[3];
    for (int d = 0; d < 3; ++d) t[d] = (uint32_t)c[d] - (uint32_t)minint[d];
    if (large) {
      for (int d = 0; d < 3; ++d) w.put(t[d], bits_d[d]);
    } else {
      put_triple(w, bitsize, size, t);
    }
    for (int d = 0; d < 3; ++d) prev[d] = c[d];
    ++i;
    int run = 0;
    if (!is_small && is_smaller == -1) is_smaller = 0;
    while (is_small && run < 24) {
      int32_t* nc = &q[3 * (size_t)i];
      int32_t sum = 0;
      for (int d = 0; d < 3; ++d) {
        const int32_t dd = wsub(nc[d], prev[d]);
        sum = (int32_t)((uint32_t)sum + (uint32_t)wmul(dd, dd));
      }
      if (is_smaller == -1 && sum >= wmul(smaller, smaller)) is_smaller = 0;
      for (int d = 0; d < 3; ++d) {
        small[run++] = (uint32_t)(wsub(nc[d], prev[d])) + (uint32_t)smallnum;
        prev[d] = nc[d];
      }
      ++i;
      is_small = false;
      if (i < natoms) {
        const int32_t* n2 = &q[3 * (size_t)i];
        is_small = wabs(wsub(n2[0], prev[0])) < smallnum && wabs(wsub(n2[1], prev[1])) < smallnum &&
                   wabs(wsub(n2[2], prev[2])) < smallnum;
      }
    }
    if (run != prevrun || is_smaller != 0) {
      prevrun = run;
      w.put(1, 1);
      w.put((uint32_t)(run + is_smaller + 1), 5);
    } else {
      w.put(0, 1);
    }
    const uint32_t ss[3] = {sizesmall, sizesmall, sizesmall};
    for (int k = 0; k < run; k += 3) put_triple(w, smallidx, ss, small + k);
    if (is_smaller != 0) {
      smallidx += is_smaller;
      if (is_smaller < 0) {
        smallnum = smaller;
        smaller = h_ranges[smallidx - 1] / 2;
      } else {
        smaller = smallnum;
        smallnum = h_ranges[smallidx] / 2;
      }
      sizesmall = (uint32_t)h_ranges[smallidx];
    }
  }
  w.flush();
  put_be32(*o, (uint32_t)w.bytes.size());
  o->insert(o->end(), w.bytes.begin(), w.bytes.end());
  while (o->size() & 3u) o->push_back(0);
  return true;
}

// ---------------------------------------------------------------- helpers

int column_map_xtc(uint32_t natoms, const size_t* usecols, size_t n_usecols,
                   std::vector<int32_t>* map, size_t* n_use, std::string* err) {
  const size_t n_cols = 3 * (size_t)natoms;
  map->clear();
  if (!usecols || n_usecols == 0) {
    *n_use = n_cols;
    return ENT_OK;
  }
  map->assign(n_cols, -1);
  for (size_t k = 0; k < n_usecols; ++k) {
    if (usecols[k] >= n_cols) {
      *err = "column index beyond the file's columns";
      return ENT_ERR_ARG;
    }
    (*map)[usecols[k]] = 0;
  }
  // the file's column order, as read_coords keeps it
  size_t u = 0;
  for (size_t c = 0; c < n_cols; ++c)
    if ((*map)[c] == 0) (*map)[c] = (int32_t)u++;
  *n_use = u;
  return ENT_OK;
}

// Copies [0, len) of the file to device memory d_file through the context's
// two pinned staging buffers; each buffer is filled by all host threads
// (pread) while the other one's copy runs.
int upload_file(Ctx& c, const char* path, uint64_t len, uint8_t* d_file) {
  Fd f;
  f.fd = open(path, O_RDONLY);
  if (f.fd < 0) return c.fail(ENT_ERR_IO, std::string("cannot open ") + path);
  const size_t CH = (size_t)std::min<uint64_t>(len, 32ull << 20);
  int rc = c.ensure_staging(CH);
  if (rc) return rc;
  const unsigned T = host_threads();
  uint64_t blk = 0;
  for (uint64_t off = 0; rc == ENT_OK && off < len; off += CH, ++blk) {
    const size_t n = (size_t)std::min<uint64_t>(CH, len - off);
    const int b = (int)(blk & 1);
    uint8_t* stage = c.h_stage[b];
    if (blk >= 2 && cudaEventSynchronize(c.ev_stage[b]) != cudaSuccess) {
      rc = c.cuda_fail(cudaGetLastError(), "staging reuse");
      break;
    }
    const unsigned nt = (unsigned)std::min<size_t>(T, std::max<size_t>(1, n >> 20));
    std::vector<std::thread> th;
    std::vector<char> ok(nt, 1);
    for (unsigned t = 1; t < nt; ++t) {
      const size_t a = n * t / nt, e = n * (t + 1) / nt;
      th.emplace_back([&, a, e, t] { ok[t] = pread_all(f.fd, stage + a, e - a, off + a); });
    }
    ok[0] = pread_all(f.fd, stage, n / nt, off);
    for (auto& x : th) x.join();
    if (std::find(ok.begin(), ok.end(), 0) != ok.end()) {
      rc = c.fail(ENT_ERR_IO, "read failed");
      break;
    }
    cudaError_t e = cudaMemcpyAsync(d_file + off, stage, n, cudaMemcpyHostToDevice, c.stream);
    if (e == cudaSuccess) e = cudaEventRecord(c.ev_stage[b], c.stream);
    if (e != cudaSuccess) rc = c.cuda_fail(e, "copy file block");
  }
  if (cudaStreamSynchronize(c.stream) != cudaSuccess && rc == ENT_OK)
    rc = c.cuda_fail(cudaGetLastError(), "copy file");
  return rc;
}

// Decodes the file into out (device): value (frame f, output column u) at
// out[u * col_stride + f * row_stride].
int decode_to_device(Ctx& c, const char* path, const size_t* usecols, size_t n_usecols,
                     size_t n_rows, size_t n_cols_out, float* d_out, size_t col_stride,
                     size_t row_stride) {
  XtcIndex ix;
  std::string err;
  if (!index_xtc(path, &ix, &err)) return c.fail(ENT_ERR_IO, err);
  std::vector<int32_t> map;
  size_t n_use = 0;
  int s = column_map_xtc(ix.natoms, usecols, n_usecols, &map, &n_use, &err);
  if (s) return c.fail(s, err);
  if (n_rows != ix.frame.size() || n_cols_out != n_use)
    return c.fail(ENT_ERR_ARG, "output shape does not match the file");
  const uint32_t n_frames = (uint32_t)ix.frame.size();
  uint8_t* d_file = static_cast<uint8_t*>(c.arena.alloc((ix.end + 15) & ~15ull));
  uint64_t* d_off = static_cast<uint64_t*>(c.arena.alloc(8ull * n_frames));
  int32_t* d_map = map.empty() ? nullptr
                               : static_cast<int32_t*>(c.arena.alloc(4 * map.size()));
  uint32_t* d_xerr = static_cast<uint32_t*>(c.arena.alloc(16));
  // decoding segments: a checkpoint per XTC_SEG_ATOMS atoms of every frame
  const uint32_t max_seg = std::max<uint32_t>(1, (ix.natoms + XTC_SEG_ATOMS - 1) / XTC_SEG_ATOMS);
  const uint64_t n_threads2 = (uint64_t)n_frames * max_seg;
  if (n_threads2 > (uint64_t)UINT32_MAX * XTC_DECODE_THREADS)
    return c.fail(ENT_ERR_TOO_LARGE, "trajectory too large for one call");
  XtcCheckpoint* d_cp =
      static_cast<XtcCheckpoint*>(c.arena.alloc(sizeof(XtcCheckpoint) * n_threads2));
  uint32_t* d_nseg = static_cast<uint32_t*>(c.arena.alloc(4ull * n_frames));
  if (!d_file || !d_off || (!map.empty() && !d_map) || !d_xerr || !d_cp || !d_nseg)
    return c.fail(ENT_ERR_CUDA, "out of device memory");
  s = upload_file(c, path, ix.end, d_file);
  if (s) return s;
  cudaError_t e = cudaMemcpyAsync(d_off, ix.frame.data(), 8ull * n_frames,
                                  cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess && d_map)
    e = cudaMemcpyAsync(d_map, map.data(), 4 * map.size(), cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_xerr, 0, 16, c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "copy frame index");
  if (n_use == 0) return ENT_OK;
  DecodeOut o{d_out, col_stride, row_stride, d_map};
  const uint32_t* file_end = reinterpret_cast<const uint32_t*>(d_file + (ix.end & ~3ull));
  cudaEventRecord(c.ev_k0, c.stream);
  // one walk per warp while the frames fill fewer than 8 warps per SM
  const uint32_t stride = (uint64_t)n_frames < 8ull * 32 * (uint64_t)c.n_sms ? 32u : 1u;
  const uint64_t n_threads1 = (uint64_t)n_frames * stride;
  k_xtc_walk<<<(unsigned)((n_threads1 + XTC_DECODE_THREADS - 1) / XTC_DECODE_THREADS),
               XTC_DECODE_THREADS, 0, c.stream>>>(d_file, d_off, n_frames, ix.natoms, max_seg,
                                                  stride, file_end, d_cp, d_nseg, d_xerr);
  e = cudaGetLastError();
  if (e == cudaSuccess) {
    k_xtc_decode<<<(unsigned)((n_threads2 + XTC_DECODE_THREADS - 1) / XTC_DECODE_THREADS),
                   XTC_DECODE_THREADS, 0, c.stream>>>(d_file, d_off, n_frames, ix.natoms, max_seg,
                                                      file_end, d_cp, d_nseg, o, d_xerr);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return c.cuda_fail(e, "decode launch");
  cudaEventRecord(c.ev_k1, c.stream);
  uint32_t herr[2] = {0, 0};
  e = cudaMemcpyAsync(herr, d_xerr, 8, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "decode");
  if (herr[0] != XERR_NONE)
    return c.fail(ENT_ERR_IO, std::string(path) + ": frame " + std::to_string(herr[1]) + ": " +
                                  xerr_text(herr[0]));
  c.stats.kernel_launches = 2;
  c.stats.instances = n_frames;
  return ENT_OK;
}

int finish(Ctx& c) {
  const int s = c.end_call();
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, c.ev_k0, c.ev_k1) == cudaSuccess) c.stats.pair_kernel_ms = ms;
  cudaGetLastError();
  return s;
}

}  // namespace

extern "C" {

int ent_xtc_file_shape(const char* path, size_t* n_frames, size_t* n_cols) {
  g_xtc_error.clear();
  if (!path || !n_frames || !n_cols) return ENT_ERR_ARG;
  XtcIndex ix;
  if (!index_xtc(path, &ix, &g_xtc_error)) return ENT_ERR_IO;
  *n_frames = ix.frame.size();
  *n_cols = 3 * (size_t)ix.natoms;
  return ENT_OK;
}

int ent_load_xtc_device(ent_ctx* ctx, const char* path, const size_t* usecols,
                        size_t n_usecols, float* d_out, size_t n_rows, size_t n_cols_out) {
  if (!ctx) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  if (!path || !d_out) return c.fail(ENT_ERR_ARG, "null argument");
  s = decode_to_device(c, path, usecols, n_usecols, n_rows, n_cols_out, d_out, n_rows, 1);
  if (s) return s;
  return finish(c);
}

int ent_read_xtc(ent_ctx* ctx, const char* path, const size_t* usecols, size_t n_usecols,
                 char primary_index, float* out, size_t n_rows, size_t n_cols_out) {
  if (!ctx) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  if (!path || !out || (primary_index != 'C' && primary_index != 'R'))
    return c.fail(ENT_ERR_ARG, "null argument or primary index not 'C'/'R'");
  const size_t bytes = 4 * n_rows * n_cols_out;
  float* d = static_cast<float*>(c.arena.alloc(std::max<size_t>(bytes, 16)));
  if (!d) return c.fail(ENT_ERR_CUDA, "out of device memory");
  const bool col_major = primary_index == 'C';
  s = decode_to_device(c, path, usecols, n_usecols, n_rows, n_cols_out, d,
                       col_major ? n_rows : 1, col_major ? 1 : n_cols_out);
  if (s) return s;
  if (bytes) {
    cudaError_t e = cudaMemcpyAsync(out, d, bytes, cudaMemcpyDeviceToHost, c.stream);
    if (e != cudaSuccess) return c.cuda_fail(e, "copy coordinates");
  }
  return finish(c);
}

int ent_write_xtc(const char* path, const float* coords, size_t n_rows, size_t n_cols,
                  char primary_index, float precision) {
  g_xtc_error.clear();
  if (!path || (!coords && n_rows != 0 && n_cols != 0) ||
      (primary_index != 'C' && primary_index != 'R'))
    return ENT_ERR_ARG;
  if (n_cols == 0 || n_cols % 3 != 0 || n_cols / 3 > (size_t)INT_MAX || n_rows > (size_t)INT_MAX) {
    g_xtc_error = "columns must be a positive multiple of 3 (x, y, z per atom)";
    return ENT_ERR_ARG;
  }
  const uint32_t natoms = (uint32_t)(n_cols / 3);
  const bool col_major = primary_index == 'C';
  // frames are independent: every host thread encodes a contiguous range
  const unsigned T = (unsigned)std::min<size_t>(host_threads(), std::max<size_t>(n_rows, 1));
  std::vector<std::vector<uint8_t>> part(T);
  std::vector<std::string> errs(T);
  std::vector<char> ok(T, 1);
  std::vector<std::thread> th;
  for (unsigned t = 0; t < T; ++t) {
    th.emplace_back([&, t] {
      const size_t r0 = n_rows * t / T, r1 = n_rows * (t + 1) / T;
      std::vector<float> row(n_cols);
      for (size_t r = r0; r < r1 && ok[t]; ++r) {
        for (size_t k = 0; k < n_cols; ++k)
          row[k] = col_major ? coords[k * n_rows + r] : coords[r * n_cols + k];
        if (!encode_frame(row.data(), natoms, (int32_t)r, (float)r, precision, &part[t],
                          &errs[t])) {
          errs[t] = "row " + std::to_string(r) + ": " + errs[t];
          ok[t] = 0;
        }
      }
    });
  }
  for (auto& x : th) x.join();
  for (unsigned t = 0; t < T; ++t)
    if (!ok[t]) {
      g_xtc_error = errs[t];
      return ENT_ERR_ARG;
    }
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    g_xtc_error = std::string("cannot create ") + path;
    return ENT_ERR_IO;
  }
  bool good = true;
  for (auto& p : part)
    if (!p.empty()) good = good && std::fwrite(p.data(), 1, p.size(), f) == p.size();
  good = (std::fclose(f) == 0) && good;
  if (!good) {
    g_xtc_error = "write failed";
    return ENT_ERR_IO;
  }
  return ENT_OK;
}

const char* ent_xtc_last_error(void) { return g_xtc_error.c_str(); }

}  // extern "C"
