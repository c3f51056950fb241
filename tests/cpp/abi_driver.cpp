// Uses the C ABI (include/entropical_gb300.h) from C++ the way a port of the
// reference's mains would: read the coordinate file with the parallel reader
// (in place of Tools::IO::read_coords, tools.hxx:153-235), tune the context on
// the data, then compute the reference's MI formula (mi.cpp:37-59) and the
// resubstitution all-pairs MI, each as one batch. Writes, as float64:
//   n_cols, then mi_ref[n_cols][n_cols], mi_resub[n_cols][n_cols], h_marg[n_cols].
// Usage: abi_driver <coords.txt> <bandwidth> <out.bin>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "entropical_gb300.h"

static int check(int s, const char* what, ent_ctx* ctx) {
  if (s != ENT_OK) {
    std::fprintf(stderr, "%s: %s (%s)\n", what, ent_status_string(s),
                 ctx ? ent_last_error(ctx) : ent_io_last_error());
    std::exit(10 + s);
  }
  return s;
}

int main(int argc, char** argv) {
  if (argc != 4) return 2;
  size_t n_rows = 0, n_cols = 0;
  check(ent_coords_file_shape(argv[1], &n_rows, &n_cols), "shape", nullptr);
  std::vector<float> coords(n_rows * n_cols);
  check(ent_read_coords(argv[1], nullptr, 0, 'C', coords.data(), n_rows, n_cols), "read",
        nullptr);
  std::vector<float> h(n_cols, (float)std::atof(argv[2]));
  ent_ctx* ctx = nullptr;
  check(ent_create(&ctx, -1), "create", nullptr);
  // the context's own autotuner on the data's 2-D densities (first pair)
  ent_instance pair{};
  std::vector<float> xy(coords.begin(), coords.begin() + 2 * n_rows);
  pair.coords = xy.data();
  pair.n = n_rows;
  pair.d = 2;
  pair.h[0] = h[0];
  pair.h[1] = h[1];
  ent_tuning t{};
  check(ent_autotune(ctx, &pair, 1, 2, 0, &t), "autotune", ctx);
  std::vector<double> mi_ref(n_cols * n_cols), mi(n_cols * n_cols), hx(n_cols);
  check(ent_reference_estimator(ctx, coords.data(), n_rows, n_cols, h.data(), ENT_REF_MI, 0, 0,
                                mi_ref.data()),
        "reference MI", ctx);
  check(ent_mi_all_pairs(ctx, coords.data(), n_rows, n_cols, h.data(), 0, mi.data(), hx.data()),
        "MI", ctx);
  ent_destroy(ctx);
  std::FILE* f = std::fopen(argv[3], "wb");
  if (!f) return 3;
  const double nc = (double)n_cols;
  std::fwrite(&nc, 8, 1, f);
  std::fwrite(mi_ref.data(), 8, mi_ref.size(), f);
  std::fwrite(mi.data(), 8, mi.size(), f);
  std::fwrite(hx.data(), 8, hx.size(), f);
  std::fclose(f);
  return 0;
}
