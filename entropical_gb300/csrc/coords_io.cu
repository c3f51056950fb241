// Coordinate files: the reference's ASCII format, read in parallel.
//
// Tools::IO::read_coords (tools.hxx:153-235) reads a whitespace-separated
// text matrix with a two-pass std::ifstream parser: the first non-empty line
// gives n_cols, the number of non-empty lines gives n_rows, then every value
// is read with `ifs >> float` into a row-major ('R') or column-major ('C')
// buffer, keeping only the requested columns. Here a regular file is mapped
// read-only (other files are read into memory), the starts of the non-empty
// lines are found by all host threads, and rows are parsed in parallel with
// std::from_chars (correctly rounded, like the strtof behind `ifs >> float`).
// ent_load_coords_device parses blocks of rows into pinned staging buffers
// and copies each block to its place in a column-major device matrix with one
// 2-D copy while the next block is being parsed.
//
// Differences from the reference, all on malformed input: a row with a
// different number of values than the first is an error (the reference reads
// values across line ends and silently shifts the matrix); a value that is
// not a number is an error (the reference leaves it unread); a value above
// the float range is +-infinity, as strtof gives it (the reference stores
// +-FLT_MAX there and reads nothing after it: every later value of the matrix
// repeats it). A leading '+' is accepted, as `ifs >> float` does.
#include <cuda_runtime.h>
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/entropical_gb300.h"
#include "api_internal.h"

namespace {

// The file's bytes: a read-only mapping of a regular file (no copy; the
// pages are faulted in by the threads that scan them), else the whole stream
// read into memory (pipes, files that cannot be mapped). As with any mapped
// reader, a file truncated by another process while it is being read ends
// this one with SIGBUS.
struct TextFile {
  const char* data = nullptr;
  size_t size = 0;
  void* map = nullptr;
  std::vector<char> owned;
  std::vector<size_t> line_start;  // non-empty lines
  std::vector<size_t> line_end;
  size_t n_cols = 0;
  std::string error;
  TextFile() = default;
  TextFile(const TextFile&) = delete;
  TextFile& operator=(const TextFile&) = delete;
  ~TextFile() {
    if (map) munmap(map, size);
  }
};

unsigned n_threads() {
  const unsigned t = std::thread::hardware_concurrency();
  return std::max(1u, std::min(t, 64u));
}

template <class F>
void parallel_for(size_t n, F f) {
  const unsigned T = (unsigned)std::min<size_t>(n_threads(), std::max<size_t>(n, 1));
  if (T <= 1) {
    f(0, n, 0u);
    return;
  }
  std::vector<std::thread> th;
  for (unsigned t = 0; t < T; ++t) {
    const size_t a = n * t / T, b = n * (t + 1) / T;
    th.emplace_back([=] { f(a, b, t); });
  }
  for (auto& x : th) x.join();
}

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// Maps (or reads) the file and indexes its non-empty lines (a line of spaces
// counts, as a non-empty std::getline result does in the reference; a last
// line without a line break counts too).
bool load_text(const char* path, TextFile* tf) {
  const int fd = open(path, O_RDONLY | O_CLOEXEC);
  if (fd < 0) {
    tf->error = std::string("cannot open ") + path;
    return false;
  }
  struct stat st;
  const bool regular = fstat(fd, &st) == 0 && S_ISREG(st.st_mode);
  if (regular && st.st_size > 0) {
    void* m = mmap(nullptr, (size_t)st.st_size, PROT_READ, MAP_PRIVATE, fd, 0);
    if (m != MAP_FAILED) {
      tf->map = m;
      tf->data = static_cast<const char*>(m);
      tf->size = (size_t)st.st_size;
    }
  }
  if (!tf->map) {  // also files that report no size (procfs)
    size_t got = 0;
    tf->owned.resize(std::max<size_t>(regular ? (size_t)st.st_size : 0, (size_t)1 << 16));
    while (true) {
      if (got == tf->owned.size()) tf->owned.resize(2 * got);
      const ssize_t r = read(fd, tf->owned.data() + got, tf->owned.size() - got);
      if (r < 0 && errno == EINTR) continue;
      if (r < 0) {
        close(fd);
        tf->error = std::string("cannot read ") + path;
        return false;
      }
      if (r == 0) break;
      got += (size_t)r;
    }
    tf->data = tf->owned.data();
    tf->size = got;
  }
  close(fd);
  const char* b = tf->data;
  const size_t n = tf->size;
  // per-thread line scan over byte ranges split at line ends
  const unsigned T = (unsigned)std::min<size_t>(n_threads(), std::max<size_t>(1, n >> 16));
  std::vector<size_t> cut(T + 1, 0);
  cut[T] = n;
  for (unsigned t = 1; t < T; ++t) {
    size_t p = n * t / T;
    while (p > 0 && p < n && b[p - 1] != '\n') ++p;
    cut[t] = std::max(p, cut[t - 1]);
  }
  std::vector<std::vector<size_t>> s(T), e(T);
  parallel_for(T, [&](size_t a, size_t bb, unsigned) {
    for (size_t t = a; t < bb; ++t) {
      size_t p = cut[t];
      while (p < cut[t + 1]) {
        const char* q = static_cast<const char*>(std::memchr(b + p, '\n', cut[t + 1] - p));
        const size_t end = q ? (size_t)(q - b) : cut[t + 1];
        if (end > p) {
          s[t].push_back(p);
          e[t].push_back(end);
        }
        p = end + 1;
      }
    }
  });
  for (unsigned t = 0; t < T; ++t) {
    tf->line_start.insert(tf->line_start.end(), s[t].begin(), s[t].end());
    tf->line_end.insert(tf->line_end.end(), e[t].begin(), e[t].end());
  }
  if (!tf->line_start.empty()) {
    size_t p = tf->line_start[0], q = tf->line_end[0], c = 0;
    while (p < q) {
      while (p < q && is_space(b[p])) ++p;
      if (p >= q) break;
      ++c;
      while (p < q && !is_space(b[p])) ++p;
    }
    tf->n_cols = c;
  }
  return true;
}

// Whether a decimal token that does not fit a float lies below its range
// (else above it): the power of ten of its first nonzero digit, the explicit
// exponent included, is negative ("0.000...1" as well as "1e-50").
bool below_float_range(const char* p, const char* end) {
  if (p < end && *p == '-') ++p;
  long int_sig = 0, frac_zeros = 0;  // integer digits from the first nonzero; zeros after '.'
  bool dot = false, nz = false;
  for (; p < end && *p != 'e' && *p != 'E'; ++p) {
    if (*p == '.') {
      dot = true;
    } else if (!dot) {
      nz = nz || *p != '0';
      int_sig += nz;
    } else if (!nz) {
      if (*p != '0') break;
      ++frac_zeros;
    }
  }
  long e10 = int_sig > 0 ? int_sig - 1 : -(frac_zeros + 1);
  while (p < end && *p != 'e' && *p != 'E') ++p;
  if (p < end) {  // the explicit exponent, saturated
    ++p;
    const bool eneg = p < end && *p == '-';
    if (p < end && (*p == '-' || *p == '+')) ++p;
    long ev = 0;
    for (; p < end && *p >= '0' && *p <= '9'; ++p) ev = std::min(10 * ev + (*p - '0'), 1000000L);
    e10 += eneg ? -ev : ev;
  }
  return e10 < 0;
}

// Parses rows [r0, r1) into dst: element (row r, used column u) at
// dst[u * col_stride + (r - r0) * row_stride]. Returns false on a malformed
// row (message in err).
bool parse_rows(const TextFile& tf, size_t r0, size_t r1, const std::vector<int>& use,
                float* dst, size_t col_stride, size_t row_stride, std::string* err) {
  const char* b = tf.data;
  const size_t nc = tf.n_cols;
  for (size_t r = r0; r < r1; ++r) {
    const char* p = b + tf.line_start[r];
    const char* q = b + tf.line_end[r];
    size_t c = 0;
    while (true) {
      while (p < q && is_space(*p)) ++p;
      if (p >= q) break;
      if (c >= nc) {
        *err = "row " + std::to_string(r + 1) + " has more than " + std::to_string(nc) + " values";
        return false;
      }
      const char* tok = p;
      if (*tok == '+') ++tok;
      float v = 0.f;
      const auto res = std::from_chars(tok, q, v);
      if (res.ec == std::errc::invalid_argument || (res.ptr < q && !is_space(*res.ptr))) {
        *err = "row " + std::to_string(r + 1) + ": not a number";
        return false;
      }
      // out-of-range values saturate as strtof does
      if (res.ec == std::errc::result_out_of_range) {
        const bool neg = *tok == '-';
        const bool tiny = below_float_range(tok, res.ptr);
        v = tiny ? (neg ? -0.f : 0.f) : (neg ? -HUGE_VALF : HUGE_VALF);
      }
      if (use[c] >= 0) dst[(size_t)use[c] * col_stride + (r - r0) * row_stride] = v;
      ++c;
      p = res.ptr;
    }
    if (c != nc) {
      *err = "row " + std::to_string(r + 1) + " has " + std::to_string(c) + " values, expected " +
             std::to_string(nc);
      return false;
    }
  }
  return true;
}

bool parallel_parse(const TextFile& tf, size_t r0, size_t r1, const std::vector<int>& use,
                    float* dst, size_t col_stride, size_t row_stride, std::string* err) {
  std::atomic<bool> ok{true};
  std::vector<std::string> errs(n_threads());
  parallel_for(r1 - r0, [&](size_t a, size_t b, unsigned t) {
    if (!parse_rows(tf, r0 + a, r0 + b, use, dst + a * row_stride, col_stride, row_stride,
                    &errs[t]))
      ok = false;
  });
  if (!ok)
    for (auto& e : errs)
      if (!e.empty()) {
        *err = e;
        break;
      }
  return ok;
}

int column_map(const TextFile& tf, const size_t* usecols, size_t n_use, std::vector<int>* use,
               std::string* err) {
  use->assign(tf.n_cols, -1);
  if (!usecols || n_use == 0) {
    for (size_t i = 0; i < tf.n_cols; ++i) (*use)[i] = (int)i;
    return ENT_OK;
  }
  // as the reference: the used columns keep the file's order
  std::vector<char> on(tf.n_cols, 0);
  for (size_t k = 0; k < n_use; ++k) {
    if (usecols[k] >= tf.n_cols) {
      *err = "given column index is not compatible with available number of columns (" +
             std::to_string(tf.n_cols) + ")";
      return ENT_ERR_ARG;
    }
    on[usecols[k]] = 1;
  }
  int u = 0;
  for (size_t i = 0; i < tf.n_cols; ++i)
    if (on[i]) (*use)[i] = u++;
  return ENT_OK;
}

size_t used_count(const std::vector<int>& use) {
  size_t u = 0;
  for (int x : use) u += x >= 0;
  return u;
}

thread_local std::string g_io_error;

}  // namespace

extern "C" {

const char* ent_io_last_error(void) { return g_io_error.c_str(); }

int ent_coords_file_shape(const char* path, size_t* n_rows, size_t* n_cols) {
  g_io_error.clear();
  if (!path || !n_rows || !n_cols) return ENT_ERR_ARG;
  TextFile tf;
  if (!load_text(path, &tf)) {
    g_io_error = tf.error;
    return ENT_ERR_IO;
  }
  *n_rows = tf.line_start.size();
  *n_cols = tf.n_cols;
  return ENT_OK;
}

int ent_read_coords(const char* path, const size_t* usecols, size_t n_usecols,
                    char primary_index, float* out, size_t n_rows, size_t n_cols_out) {
  g_io_error.clear();
  if (!path || !out || (primary_index != 'C' && primary_index != 'R')) return ENT_ERR_ARG;
  TextFile tf;
  if (!load_text(path, &tf)) {
    g_io_error = tf.error;
    return ENT_ERR_IO;
  }
  std::vector<int> use;
  int s = column_map(tf, usecols, n_usecols, &use, &g_io_error);
  if (s) return s;
  const size_t nu = used_count(use);
  if (n_rows != tf.line_start.size() || n_cols_out != nu) {
    g_io_error = "output shape does not match the file";
    return ENT_ERR_ARG;
  }
  const bool col_major = primary_index == 'C';
  if (!parallel_parse(tf, 0, n_rows, use, out, col_major ? n_rows : 1, col_major ? 1 : nu,
                      &g_io_error))
    return ENT_ERR_IO;
  return ENT_OK;
}

int ent_load_coords_device(ent_ctx* ctx, const char* path, const size_t* usecols,
                           size_t n_usecols, float* d_out, size_t n_rows, size_t n_cols_out) {
  g_io_error.clear();
  if (!ctx || !path || !d_out) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  TextFile tf;
  if (!load_text(path, &tf)) {
    g_io_error = tf.error;
    return c.fail(ENT_ERR_IO, tf.error);
  }
  std::vector<int> use;
  int s = column_map(tf, usecols, n_usecols, &use, &g_io_error);
  if (s) return c.fail(s, g_io_error);
  const size_t nu = used_count(use);
  if (n_rows != tf.line_start.size() || n_cols_out != nu) {
    g_io_error = "output shape does not match the file";
    return c.fail(ENT_ERR_ARG, g_io_error);
  }
  if (n_rows == 0 || nu == 0) return ENT_OK;
  if (cudaSetDevice(c.device) != cudaSuccess) return c.cuda_fail(cudaGetLastError(), "set device");
  // blocks of rows (8 MB, at least one row) through the context's two pinned
  // staging buffers, column-major per block, one parsed while the other is
  // being copied
  const size_t row_bytes = 4 * nu;
  const size_t blk_bytes = std::max(row_bytes, std::min(row_bytes * n_rows, (size_t)8 << 20));
  int rc = c.ensure_staging(blk_bytes);
  if (rc) return rc;
  const size_t R = std::min(n_rows, blk_bytes / row_bytes);
  size_t blk = 0;
  for (size_t r0 = 0; rc == ENT_OK && r0 < n_rows; r0 += R, ++blk) {
    const size_t r1 = std::min(n_rows, r0 + R), nr = r1 - r0;
    const int b = (int)(blk & 1);
    float* stage = reinterpret_cast<float*>(c.h_stage[b]);
    if (blk >= 2 && cudaEventSynchronize(c.ev_stage[b]) != cudaSuccess) {
      rc = c.cuda_fail(cudaGetLastError(), "staging reuse");
      break;
    }
    if (!parallel_parse(tf, r0, r1, use, stage, nr, 1, &g_io_error)) {
      rc = c.fail(ENT_ERR_IO, g_io_error);
      break;
    }
    // nu columns of nr values into the column-major n_rows x nu matrix
    cudaError_t e = cudaMemcpy2DAsync(d_out + r0, 4 * n_rows, stage, 4 * nr, 4 * nr, nu,
                                      cudaMemcpyHostToDevice, c.stream);
    if (e == cudaSuccess) e = cudaEventRecord(c.ev_stage[b], c.stream);
    if (e != cudaSuccess) rc = c.cuda_fail(e, "copy block");
  }
  if (cudaStreamSynchronize(c.stream) != cudaSuccess && rc == ENT_OK)
    rc = c.cuda_fail(cudaGetLastError(), "copy");
  return rc;
}

}  // extern "C"
