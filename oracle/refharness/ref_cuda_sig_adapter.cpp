// The reference's estimators (mi.cpp, transs.cpp, autoent.cpp, kldiv.cpp,
// negs.cpp, dens.cpp) only compile against the CUDA-build density signature
// (densities_cuda.hpp:9-24, returning std::vector<double>); the OpenMP build's
// std::vector<float> return type does not convert. This adapter provides that
// signature on top of the reference's OpenMP numerics so the estimators can
// run on the CPU here, with the CUDA build's normalisation by the original
// n_rows (densities_cuda.cu:98-103). Test infrastructure only.
#include "densities_cuda.hpp"

#include <cstring>
#include <vector>

std::vector<float> ref_omp_combined_densities(const float* coords,
                                              std::size_t n_rows,
                                              std::vector<unsigned int> i_cols,
                                              std::vector<float> h);

std::vector<double> combined_densities(const float* coords, std::size_t n_rows,
                                       std::vector<unsigned int> i_cols,
                                       std::vector<float> h,
                                       std::vector<unsigned int> tau) {
  unsigned d = i_cols.size();
  unsigned tmax = 0;
  for (unsigned t : tau) tmax = t > tmax ? t : tmax;
  std::size_t n_sel = n_rows - tmax;
  std::vector<float> buf(n_sel * d);
  for (unsigned j = 0; j < d; ++j)
    std::memcpy(&buf[j * n_sel], coords + (std::size_t)i_cols[j] * n_rows + tau[j],
                n_sel * sizeof(float));
  std::vector<unsigned> ic(d);
  for (unsigned j = 0; j < d; ++j) ic[j] = j;
  std::vector<float> p = ref_omp_combined_densities(buf.data(), n_sel, ic, h);
  std::vector<double> out(p.size());
  for (std::size_t i = 0; i < p.size(); ++i)
    out[i] = (double)p[i] * (double)n_sel / (double)n_rows;
  return out;
}

std::vector<double> combined_densities(const float* coords, std::size_t n_rows,
                                       std::vector<unsigned int> i_cols,
                                       std::vector<float> h) {
  return combined_densities(coords, n_rows, i_cols, h,
                            std::vector<unsigned int>(i_cols.size(), 0));
}
