// C entry points over the reference's own OpenMP density code, compiled from
// the reference sources in place (see ../Makefile). Test infrastructure only:
// used to pin the oracle restatement and as the timed CPU reference arm.
//
// The reference's boxes() window search lives in an anonymous namespace of
// densities_omp.cpp (densities_omp.cpp:33-65), so this translation unit
// includes that file directly; its combined_densities overloads are renamed
// with a macro so that ref_cuda_sig_adapter.cpp can provide the CUDA-build
// signature (densities_cuda.hpp:9-24) without a symbol clash.
#define combined_densities ref_omp_combined_densities
#include "densities_omp.cpp"
#undef combined_densities

#include "boxedsearch.hpp"
#include "hestimate.hpp"

#include <cstdint>
#include <cstring>
#include <vector>

namespace {
// The reference OMP path is only correct for i_cols == {0..d-1} and tau == 0
// (it indexes the selected buffer with the original column ids,
// densities_omp.cpp:88,117-118,148-150). Repack the selected, lagged columns
// into a fresh column-major n_sel x d buffer first.
std::vector<float> repack(const float* coords, std::size_t n_rows,
                          const unsigned* cols, const unsigned* tau,
                          unsigned d, std::size_t* n_sel_out) {
  unsigned tmax = 0;
  for (unsigned j = 0; j < d; ++j) tmax = tau[j] > tmax ? tau[j] : tmax;
  std::size_t n_sel = n_rows - tmax;
  std::vector<float> buf(n_sel * d);
  for (unsigned j = 0; j < d; ++j)
    std::memcpy(&buf[j * n_sel], coords + (std::size_t)cols[j] * n_rows + tau[j],
                n_sel * sizeof(float));
  *n_sel_out = n_sel;
  return buf;
}
}  // namespace

extern "C" {

// combined_densities (densities_omp.cpp:193-233) on repacked columns.
// out: n_sel floats, already divided by n_sel as the reference does.
int ref_densities(const float* coords, std::size_t n_rows, const unsigned* cols,
                  const float* h, const unsigned* tau, unsigned d, float* out) {
  std::size_t n_sel = 0;
  std::vector<float> buf = repack(coords, n_rows, cols, tau, d, &n_sel);
  std::vector<unsigned> ic(d);
  std::vector<float> hv(h, h + d);
  for (unsigned j = 0; j < d; ++j) ic[j] = j;
  std::vector<float> p = ref_omp_combined_densities(buf.data(), n_sel, ic, hv);
  std::memcpy(out, p.data(), n_sel * sizeof(float));
  return 0;
}

// epa_convolution (densities_omp.cpp:235-277).
float ref_epa_convolution(const float* sorted, std::size_t n, float h) {
  std::vector<float> v(sorted, sorted + n);
  return epa_convolution(v, h);
}

// boxes() window bounds (densities_omp.cpp:33-65) for one column.
void ref_boxes(const float* col, std::size_t n, float h, std::uint64_t* lo,
               std::uint64_t* hi) {
  std::vector<float> s(col, col + n);
  std::sort(s.begin(), s.end());
  Boxes b = boxes(col, 0, s, n, h);
  for (std::size_t i = 0; i < n; ++i) {
    lo[i] = b[i][0];
    hi[i] = b[i][1];
  }
}

// Transs::BoxedSearch::Boxes (boxedsearch.cpp:15-62): number of boxes, the box
// of every state and the size of every state's neighbour list.
std::uint64_t ref_boxedsearch(const float* col, std::size_t n, float box_size,
                              std::uint64_t* box_of_state,
                              std::uint64_t* n_neighbors) {
  Transs::BoxedSearch::Boxes b(col, n, 0, box_size);
  for (std::size_t i = 0; i < n; ++i) {
    std::vector<std::size_t> nb = b.neighbors_of_state_ordered(i);
    n_neighbors[i] = nb.size();
    if (box_of_state) box_of_state[i] = 0;
  }
  return b.n_boxes();
}

// Hestimate::Thumb::Kernel (hestimate.cpp:19-30).
float ref_thumb(float* coords, std::size_t n_rows, std::size_t i_col) {
  return Hestimate::Thumb::Kernel()(coords, n_rows, i_col);
}

// Hestimate::AmiseMin::Kernel (hestimate.cpp:88-104).
float ref_amise_h(float* coords, std::size_t n_rows, std::size_t i_col) {
  return Hestimate::AmiseMin::Kernel()(coords, n_rows, i_col);
}

// Tools::IO::read_coords (tools.hxx:153-235): shape of the file (out == null)
// or its values, column-major ('C') or row-major ('R'), for the used columns.
int ref_read_coords(const char* path, char primary, const std::size_t* usecols,
                    std::size_t n_usecols, float* out, std::size_t* n_rows,
                    std::size_t* n_cols) {
  std::vector<std::size_t> uc(usecols, usecols + n_usecols);
  float* c;
  std::size_t r, k;
  std::tie(c, r, k) = Tools::IO::read_coords<float>(path, primary, uc);
  *n_rows = r;
  *n_cols = k;
  if (out) std::memcpy(out, c, sizeof(float) * r * k);
  Tools::IO::free_coords(c);
  return 0;
}

}  // extern "C"
