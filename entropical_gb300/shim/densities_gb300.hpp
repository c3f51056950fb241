// Drop-in replacement of the reference's density interface
// (densities_cuda.hpp:9-31): the same three free functions with the same
// signatures, backed by the entropical GB300 C ABI. Code written against the
// reference (mi.cpp, transs.cpp, autoent.cpp, kldiv.cpp, negs.cpp, dens.cpp,
// hestimate.cpp) compiles unchanged against this header and links against
// libentropical_shim.so.
//
// Behaviour kept from the reference CUDA build:
//  * densities are divided by the original n_rows even when lags shorten the
//    sample (densities_cuda.cu:98-103); set ENT_SHIM_NORM=selected in the
//    environment to divide by the selected sample size instead;
//  * invalid selections print the reference's message to stderr and call
//    exit(EXIT_FAILURE) (densities_common.hxx:15-33), CUDA failures print
//    "CUDA error: ..." and exit (tools.cuh:32-42).
#pragma once

#include <vector>

std::vector<double>
combined_densities(const float* coords
                 , std::size_t n_rows
                 , std::vector<unsigned int> i_cols
                 , std::vector<float> h);

std::vector<double>
combined_densities(const float* coords
                 , std::size_t n_rows
                 , std::vector<unsigned int> i_cols
                 , std::vector<float> h
                 , std::vector<unsigned int> tau);

float
epa_convolution(const std::vector<float>& sorted_coords
              , float h);

// Not in the reference interface: the shim's own context (created on first
// use), for callers that want the C ABI's extras on it, e.g. ent_autotune or
// ent_set_tuning before the estimators run. Guarded by the shim's lock only
// inside the three functions above; do not use it concurrently with them.
typedef struct ent_ctx ent_ctx;
ent_ctx* densities_gb300_context();
