// C++ shim: the reference density interface over the entropical GB300 C ABI.
// See densities_gb300.hpp for the behaviour it keeps.
#include "densities_gb300.hpp"

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <mutex>

#include "entropical_gb300.h"

namespace {

std::mutex g_mu;
ent_ctx* g_ctx = nullptr;

[[noreturn]] void die(const char* msg) {
  std::cerr << msg << std::endl;
  std::exit(EXIT_FAILURE);
}

ent_ctx* context() {
  if (!g_ctx) {
    const int s = ent_create(&g_ctx, -1);
    if (s == ENT_ERR_NO_DEVICE) die("error: no CUDA-compatible GPUs found");
    if (s != ENT_OK) die("CUDA error: creating the entropical GB300 context");
  }
  return g_ctx;
}

void fail(ent_ctx* c, int s) {
  switch (s) {
    case ENT_ERR_DIM:
      die("error: can only compute combined probabilities in 1, 2 or 3 dimensions.");
    case ENT_ERR_H_COUNT:
      die("error: number of bandwidth parameters does not match number of selected columns.");
    case ENT_ERR_TAU_COUNT:
      die("error: number of lagtimes (tau) does not match number of selected dimensions.");
    default: {
      std::string m = std::string("CUDA error: ") + ent_last_error(c);
      die(m.c_str());
    }
  }
}

uint32_t shim_flags() {
  const char* v = std::getenv("ENT_SHIM_NORM");
  if (v && std::strcmp(v, "selected") == 0) return 0u;
  return ENT_COMPAT_NORM;
}

}  // namespace

std::vector<double>
combined_densities(const float* coords
                 , std::size_t n_rows
                 , std::vector<unsigned int> i_cols
                 , std::vector<float> h
                 , std::vector<unsigned int> tau) {
  std::lock_guard<std::mutex> lock(g_mu);
  const std::size_t d = i_cols.size();
  // the reference's own checks, in its order (densities_common.hxx:15-33)
  if (d < 1 || 3 < d) fail(nullptr, ENT_ERR_DIM);
  if (h.size() != d) fail(nullptr, ENT_ERR_H_COUNT);
  if (tau.size() != d) fail(nullptr, ENT_ERR_TAU_COUNT);
  ent_ctx* c = context();
  std::vector<uint32_t> cols(i_cols.begin(), i_cols.end());
  std::vector<uint32_t> taus(tau.begin(), tau.end());
  const std::size_t n_cols = *std::max_element(cols.begin(), cols.end()) + 1;
  const unsigned tmax = *std::max_element(taus.begin(), taus.end());
  std::vector<double> out(n_rows > tmax ? n_rows - tmax : 0);
  std::size_t n_out = 0;
  const int s = ent_densities(c, coords, n_rows, n_cols, cols.data(), h.data(), taus.data(),
                              (uint32_t)d, shim_flags(), out.data(), &n_out);
  if (s != ENT_OK) fail(c, s);
  out.resize(n_out);
  return out;
}

std::vector<double>
combined_densities(const float* coords
                 , std::size_t n_rows
                 , std::vector<unsigned int> i_cols
                 , std::vector<float> h) {
  const std::size_t d = i_cols.size();
  if (d < 1 || 3 < d) {
    std::cerr << "error: unsupported number of dimensions. this should never happen!"
              << std::endl;
    std::exit(EXIT_FAILURE);
  }
  return combined_densities(coords, n_rows, i_cols, h, std::vector<unsigned int>(d, 0));
}

float
epa_convolution(const std::vector<float>& sorted_coords
              , float h) {
  std::lock_guard<std::mutex> lock(g_mu);
  ent_ctx* c = context();
  float out = 0.f;
  const int s = ent_epa_convolution(c, sorted_coords.data(), sorted_coords.size(), h, &out);
  if (s != ENT_OK) fail(c, s);
  return out;
}

ent_ctx* densities_gb300_context() {
  std::lock_guard<std::mutex> lock(g_mu);
  return context();
}
