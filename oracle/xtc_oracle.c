/*
 * xtc_oracle.c -- CPU oracle for the XTC trajectory reader.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/ and the CPU-baseline leg of
 * bench.py as the checker of the library's device XTC decoder, never by the
 * product.
 *
 * Restates the reading side of the reference's XTC handler: CoordsFile::
 * XtcHandler::next (coords_file/coords_file.cpp:90-110) calls read_xtc
 * (coords_file/xdrfile/xdrfile_xtc.c:83-95: frame header, box, then
 * xdrfile_decompress_coord_float, xdrfile.c:761-961) and returns the frame as
 * one row of 3 * natoms floats (x0, y0, z0, x1, ...). The reference vendors
 * xdrfile (GROMACS' XTC codec, Frans van Hoesel's coordinate compression);
 * this file is pinned against those sources compiled in place
 * (oracle/Makefile, target xdr) and against committed fixtures written by
 * them (tests/golden/xtc_*).
 *
 * Frame layout (XDR: big-endian 4-byte units):
 *   magic 1995, natoms, step, time, box[9], natoms again,
 *   natoms <= 9: 3 * natoms raw floats;
 *   else: precision, minint[3], maxint[3], smallidx, byte count, the
 *         compressed bits (byte count bytes, zero-padded to 4).
 * Reading stops at the first frame that does not parse, as XtcHandler::next
 * stops at the first failing read_xtc.
 */
#include "ent_oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* The format's table of small-integer ranges (xdrfile.c:743-753): entry k is
 * about 2^(k/3); three values below entry k fit in k bits. Entries 0..8 are
 * unused. The values, including their irregular ones, are part of the
 * format. */
static const int orc_xtc_ranges[73] = {
    0,       0,       0,       0,       0,       0,       0,       0,       0,
    8,       10,      12,      16,      20,      25,      32,      40,      50,
    64,      80,      101,     128,     161,     203,     256,     322,     406,
    512,     645,     812,     1024,    1290,    1625,    2048,    2580,    3250,
    4096,    5060,    6501,    8192,    10321,   13003,   16384,   20642,   26007,
    32768,   41285,   52015,   65536,   82570,   104031,  131072,  165140,  208063,
    262144,  330280,  416127,  524287,  660561,  832255,  1048576, 1321122, 1664510,
    2097152, 2642245, 3329021, 4194304, 5284491, 6658042, 8388607, 10568983, 13316085,
    16777216};
#define ORC_XTC_FIRST 9
#define ORC_XTC_LAST 73

static uint32_t be32(const unsigned char* p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}
static float be_float(const unsigned char* p) {
  uint32_t u = be32(p);
  float f;
  memcpy(&f, &u, 4);
  return f;
}

typedef struct {
  const unsigned char* p;
  size_t n_bits;
  size_t pos;
} orc_bits;

/* Next n (<= 32) bits, most significant first (decodebits, xdrfile.c:660-700).
 * Bits past the data read as zero; the caller checks pos against n_bits. */
static uint32_t get_bits(orc_bits* b, int n) {
  uint64_t v = 0;
  int got = 0;
  while (got < n) {
    const size_t byte = b->pos >> 3;
    const int off = (int)(b->pos & 7);
    int take = 8 - off;
    if (take > n - got) take = n - got;
    const unsigned cur = byte < (b->n_bits >> 3) ? b->p[byte] : 0u;
    v = (v << take) | ((cur >> (8 - off - take)) & ((1u << take) - 1u));
    got += take;
    b->pos += take;
  }
  return (uint32_t)v;
}

/* Three integers packed as one number N = (n0 * s1 + n1) * s2 + n2 stored in
 * nbits bits as byte chunks, least significant chunk first (decodeints,
 * xdrfile.c:708-741; n0 is taken as the low 32 bits of the last quotient). */
static void get_triple(orc_bits* b, int nbits, const uint32_t s[3], int32_t out[3]) {
  unsigned __int128 N = 0;
  int shift = 0;
  while (nbits > 8) {
    N |= (unsigned __int128)get_bits(b, 8) << shift;
    shift += 8;
    nbits -= 8;
  }
  if (nbits > 0) N |= (unsigned __int128)get_bits(b, nbits) << shift;
  out[2] = (int32_t)(uint32_t)(N % s[2]);
  N /= s[2];
  out[1] = (int32_t)(uint32_t)(N % s[1]);
  N /= s[1];
  out[0] = (int32_t)(uint32_t)N;
}

/* Bit length of s0*s1*s2 (sizeofints, xdrfile.c:498-530). */
static int product_bits(const uint32_t s[3]) {
  unsigned __int128 P = (unsigned __int128)s[0] * s[1] * s[2];
  int bits = 0;
  while (P) {
    ++bits;
    P >>= 1;
  }
  return bits;
}

/* Smallest b with v < 2^b, at most 32 (sizeofint, xdrfile.c:473-483). */
static int value_bits(uint32_t v) {
  int b = 0;
  while (b < 32 && ((uint64_t)1 << b) <= v) ++b;
  return b;
}

static int32_t wrap_add(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }

/* Decode one compressed frame body: data = the compressed bytes, hdr = the
 * 36 bytes precision .. byte count. Row layout x0 y0 z0 x1 ... into row[]. */
static int decode_body(const unsigned char* hdr, const unsigned char* data, uint32_t n_bytes,
                       int natoms, float* row) {
  const float precision = be_float(hdr);
  int32_t minint[3], maxint[3];
  for (int d = 0; d < 3; ++d) {
    minint[d] = (int32_t)be32(hdr + 4 + 4 * d);
    maxint[d] = (int32_t)be32(hdr + 16 + 4 * d);
  }
  int smallidx = (int32_t)be32(hdr + 28);
  if (smallidx < ORC_XTC_FIRST || smallidx >= ORC_XTC_LAST) return -2;
  uint32_t sizeint[3];
  for (int d = 0; d < 3; ++d) sizeint[d] = (uint32_t)maxint[d] - (uint32_t)minint[d] + 1u;
  const int large = (sizeint[0] | sizeint[1] | sizeint[2]) > 0xffffffu;
  int bitsizeint[3] = {0, 0, 0}, bitsize = 0;
  if (large) {
    for (int d = 0; d < 3; ++d) {
      bitsizeint[d] = value_bits(sizeint[d]);
      if (bitsizeint[d] >= 32) return -2;
    }
  } else {
    if (!sizeint[0] || !sizeint[1] || !sizeint[2]) return -2;
    bitsize = product_bits(sizeint);
  }
  const float inv = (float)(1.0 / (double)precision);
  orc_bits b = {data, 8 * (size_t)n_bytes, 0};
  int smallnum = orc_xtc_ranges[smallidx] / 2;
  int smaller = orc_xtc_ranges[smallidx - 1 > ORC_XTC_FIRST ? smallidx - 1 : ORC_XTC_FIRST] / 2;
  int run = 0;
  int i = 0;
  while (i < natoms) {
    int32_t big[3];
    if (large) {
      for (int d = 0; d < 3; ++d) big[d] = (int32_t)get_bits(&b, bitsizeint[d]);
    } else {
      get_triple(&b, bitsize, sizeint, big);
    }
    for (int d = 0; d < 3; ++d) big[d] = wrap_add(big[d], minint[d]);
    int is_smaller = 0;
    if (get_bits(&b, 1)) {
      const int v = (int)get_bits(&b, 5);
      is_smaller = v % 3 - 1;
      run = v - v % 3;
    }
    const int n_small = run / 3;
    if (i + 1 + n_small > natoms) return -2;
    if (n_small == 0) {
      for (int d = 0; d < 3; ++d) row[3 * i + d] = (float)big[d] * inv;
      ++i;
    } else {
      /* The first small atom precedes the large one in the row (the
       * encoder swapped them; water-like triples compress better). */
      const uint32_t ss[3] = {(uint32_t)orc_xtc_ranges[smallidx],
                              (uint32_t)orc_xtc_ranges[smallidx],
                              (uint32_t)orc_xtc_ranges[smallidx]};
      int32_t prev[3] = {big[0], big[1], big[2]};
      for (int k = 0; k < n_small; ++k) {
        int32_t s[3];
        get_triple(&b, smallidx, ss, s);
        for (int d = 0; d < 3; ++d) s[d] = wrap_add(wrap_add(s[d], prev[d]), -smallnum);
        if (k == 0) {
          for (int d = 0; d < 3; ++d) {
            row[3 * i + d] = (float)s[d] * inv;
            row[3 * (i + 1) + d] = (float)big[d] * inv;
          }
          i += 2;
        } else {
          for (int d = 0; d < 3; ++d) row[3 * i + d] = (float)s[d] * inv;
          i += 1;
        }
        for (int d = 0; d < 3; ++d) prev[d] = s[d];
      }
    }
    if (is_smaller != 0) {
      smallidx += is_smaller;
      if (smallidx < ORC_XTC_FIRST || smallidx >= ORC_XTC_LAST) return -2;
      if (is_smaller < 0) {
        smallnum = smaller;
        smaller = smallidx > ORC_XTC_FIRST ? orc_xtc_ranges[smallidx - 1] / 2 : 0;
      } else {
        smaller = smallnum;
        smallnum = orc_xtc_ranges[smallidx] / 2;
      }
    }
  }
  return b.pos <= 8 * (size_t)n_bytes ? 0 : -2;
}

/* Reads one frame at the file position: 0 ok (row filled when row != NULL),
 * 1 no further frame (end of file or a frame that does not parse), <0 a
 * malformed compressed body. natoms_io: the file's atom count (set from the
 * first frame when *natoms_io == 0). */
static int read_frame(FILE* f, int* natoms_io, float* row, unsigned char** buf, size_t* cap) {
  unsigned char h[56];
  if (fread(h, 1, 56, f) != 56) return 1;
  if ((int32_t)be32(h) != 1995) return 1;
  const int natoms = (int32_t)be32(h + 4);
  const int lsize = (int32_t)be32(h + 52);
  if (natoms <= 0 || lsize != natoms) return 1;
  if (*natoms_io == 0) *natoms_io = natoms;
  if (natoms != *natoms_io) return 1;
  if (natoms <= 9) {
    unsigned char raw[108];
    if (fread(raw, 1, 12 * (size_t)natoms, f) != 12 * (size_t)natoms) return 1;
    if (row)
      for (int k = 0; k < 3 * natoms; ++k) row[k] = be_float(raw + 4 * k);
    return 0;
  }
  unsigned char hdr[36];
  if (fread(hdr, 1, 36, f) != 36) return 1;
  const uint32_t n_bytes = be32(hdr + 32);
  const size_t padded = ((size_t)n_bytes + 3) & ~(size_t)3;
  if (padded > *cap) {
    unsigned char* nb = (unsigned char*)realloc(*buf, padded);
    if (!nb) return -1;
    *buf = nb;
    *cap = padded;
  }
  if (fread(*buf, 1, padded, f) != padded) return 1; /* truncated: the end */
  if (!row) return 0;
  return decode_body(hdr, *buf, n_bytes, natoms, row) == 0 ? 0 : -2;
}

int orc_xtc_shape(const char* path, size_t* n_frames, size_t* n_atoms) {
  FILE* f = fopen(path, "rb");
  if (!f) return -1;
  int natoms = 0;
  size_t n = 0;
  unsigned char* buf = NULL;
  size_t cap = 0;
  while (read_frame(f, &natoms, NULL, &buf, &cap) == 0) ++n;
  fclose(f);
  free(buf);
  *n_frames = n;
  *n_atoms = (size_t)natoms;
  return n ? 0 : -2;
}

long orc_read_xtc(const char* path, size_t f0, size_t f1, float* out, size_t n_out_rows) {
  FILE* f = fopen(path, "rb");
  if (!f) return -1;
  unsigned char h[8];
  if (fread(h, 1, 8, f) != 8 || (int32_t)be32(h) != 1995 || (int32_t)be32(h + 4) <= 0) {
    fclose(f);
    return -2;
  }
  int natoms = (int32_t)be32(h + 4);
  rewind(f);
  unsigned char* buf = NULL;
  size_t cap = 0;
  float* row = (float*)malloc(sizeof(float) * 3 * (size_t)natoms);
  long done = row ? 0 : -1;
  for (size_t fr = 0; row && fr < f1; ++fr) {
    const int r = read_frame(f, &natoms, fr >= f0 ? row : NULL, &buf, &cap);
    if (r == 1) break;
    if (r < 0) {
      done = r;
      break;
    }
    if (fr < f0) continue;
    for (int k = 0; k < 3 * natoms; ++k) out[(size_t)k * n_out_rows + (fr - f0)] = row[k];
    ++done;
  }
  fclose(f);
  free(buf);
  free(row);
  return done;
}
