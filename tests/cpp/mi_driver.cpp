// Calls the drop-in density interface exactly the way the reference's
// Mi::main does (mi.cpp:37-59): per column i one 1-D density, per pair j > i
// the 1-D density of j again and the 2-D joint density, then
//   mutinf[i][j] += p_ij * log(p_ij / p_i / p_j)
// with the reference's float accumulator and float log (tools.cpp:18-37).
// Input file: int32 n_rows, int32 n_cols, float32 coords (column-major),
// float32 bandwidths[n_cols]. Output file: float32 mutinf[n_cols][n_cols].
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <functional>
#include <vector>

#include "densities_gb300.hpp"

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  std::FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  int32_t n_rows = 0, n_cols = 0;
  if (std::fread(&n_rows, 4, 1, f) != 1 || std::fread(&n_cols, 4, 1, f) != 1) return 4;
  std::vector<float> coords((size_t)n_rows * n_cols), bw(n_cols);
  if (std::fread(coords.data(), 4, coords.size(), f) != coords.size()) return 5;
  if (std::fread(bw.data(), 4, bw.size(), f) != bw.size()) return 6;
  std::fclose(f);
  std::function<float(float)> logfunc = [](float x) -> float {
    return x == 0 ? 0 : std::log(x);
  };
  std::vector<float> mutinf((size_t)n_cols * n_cols);
  for (unsigned i = 0; i < (unsigned)n_cols; ++i) {
    std::vector<double> p_i = combined_densities(coords.data(), n_rows, {i}, {bw[i]});
    for (unsigned j = i + 1; j < (unsigned)n_cols; ++j) {
      std::vector<double> p_j = combined_densities(coords.data(), n_rows, {j}, {bw[j]});
      std::vector<double> p_ij =
          combined_densities(coords.data(), n_rows, {i, j}, {bw[i], bw[j]});
      mutinf[i * n_cols + j] = 0.0f;
      for (int k = 0; k < n_rows; ++k)
        mutinf[i * n_cols + j] += p_ij[k] * logfunc(p_ij[k] / p_i[k] / p_j[k]);
      mutinf[j * n_cols + i] = mutinf[i * n_cols + j];
    }
  }
  f = std::fopen(argv[2], "wb");
  if (!f) return 7;
  std::fwrite(mutinf.data(), 4, mutinf.size(), f);
  std::fclose(f);
  return 0;
}
