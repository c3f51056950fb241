// Drives a CoordsFile implementation (the reference's coords_file.hpp, or the
// shim's through a coords_file.hpp that includes coords_file_gb300.hpp) the
// way a caller of the reference would.
//
//   coords_driver write <rows.bin> <out>   rows.bin: int32 n_rows, n_cols, then
//                                          n_rows x n_cols float32; each row
//                                          through Handler::write
//   coords_driver read <in> <rows.bin>     every row of Handler::next until
//                                          eof(), written as int32 n_rows, then
//                                          per row int32 length + float32 values
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "coords_file.hpp"

int main(int argc, char** argv) {
  if (argc != 4) return 2;
  if (std::strcmp(argv[1], "write") == 0) {
    FILE* f = std::fopen(argv[2], "rb");
    if (!f) return 3;
    int32_t nr = 0, nc = 0;
    if (std::fread(&nr, 4, 1, f) != 1 || std::fread(&nc, 4, 1, f) != 1) return 3;
    std::vector<float> v((size_t)nr * nc);
    if (std::fread(v.data(), 4, v.size(), f) != v.size()) return 3;
    std::fclose(f);
    CoordsFile::FilePointer h = CoordsFile::open(argv[3], "w");
    for (int32_t r = 0; r < nr; ++r)
      h->write(std::vector<float>(v.begin() + (size_t)r * nc, v.begin() + (size_t)(r + 1) * nc));
    return 0;
  }
  if (std::strcmp(argv[1], "read") == 0) {
    CoordsFile::FilePointer h = CoordsFile::open(argv[2], "r");
    std::vector<std::vector<float>> rows;
    for (;;) {
      std::vector<float> r = h->next();
      if (h->eof()) break;
      rows.push_back(r);
    }
    FILE* f = std::fopen(argv[3], "wb");
    if (!f) return 3;
    const int32_t n = (int32_t)rows.size();
    std::fwrite(&n, 4, 1, f);
    for (const auto& r : rows) {
      const int32_t len = (int32_t)r.size();
      std::fwrite(&len, 4, 1, f);
      if (len) std::fwrite(r.data(), 4, r.size(), f);
    }
    std::fclose(f);
    return 0;
  }
  return 2;
}
