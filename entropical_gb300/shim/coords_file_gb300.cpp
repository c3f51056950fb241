// C++ shim: the reference's coordinate-file interface over the entropical
// GB300 C ABI. See coords_file_gb300.hpp for the behaviour it keeps.
#include "coords_file_gb300.hpp"

#include <cstdlib>
#include <fstream>
#include <iostream>

#include "densities_gb300.hpp"
#include "entropical_gb300.h"

namespace CoordsFile {

namespace {

[[noreturn]] void die(const std::string& msg) {
  std::cerr << msg << std::endl;
  std::exit(EXIT_FAILURE);
}

bool is_xtc_name(const std::string& f) {
  return f.size() > 4 && f.compare(f.size() - 4, 4, ".xtc") == 0;
}

}  // namespace

// ------------------------------------------------------------------ ASCII

struct AsciiHandler::Impl {
  std::ifstream in;
  std::ofstream out;
  bool at_end = false;
};

AsciiHandler::AsciiHandler(std::string fname, std::string mode) : _p(new Impl) {
  if (mode == "r") {
    _p->in.open(fname);
  } else if (mode == "w") {
    _p->out.open(fname);
  } else {
    die("unknown mode: " + mode);
  }
}

AsciiHandler::~AsciiHandler() {}

std::vector<float> AsciiHandler::next() {
  // skip empty lines; a line counts only when the stream is still good
  // after it (a last line without a line break is not returned)
  while (_p->in.is_open() && _p->in.good()) {
    std::string line;
    std::getline(_p->in, line);
    if (!_p->in.good()) break;
    if (!line.empty()) return split<float>(line);
  }
  _p->at_end = true;
  return {};
}

void AsciiHandler::write(std::vector<float> row) {
  if (!_p->out.is_open() || !_p->out.good()) return;
  for (float v : row) _p->out << " " << v;
  _p->out << std::endl;
}

bool AsciiHandler::eof() { return _p->at_end; }

// -------------------------------------------------------------------- XTC

struct XtcHandler::Impl {
  std::string path;
  bool reading = false, writing = false;
  std::vector<float> rows;  // read: every frame; write: the rows written
  size_t n_cols = 0, n_rows = 0, pos = 0;
  bool at_end = false;
};

XtcHandler::XtcHandler(std::string fname, std::string mode) : _p(new Impl) {
  _p->path = fname;
  _p->reading = mode == "r";
  _p->writing = mode == "w";  // other modes read and write nothing, as in the reference
  if (_p->writing) {
    std::ofstream create(fname, std::ios::binary | std::ios::trunc);  // as opening for writing does
    return;
  }
  if (!_p->reading) return;
  size_t nf = 0, nc = 0;
  if (ent_xtc_file_shape(fname.c_str(), &nf, &nc) != ENT_OK) return;  // no frame: at the end
  _p->rows.resize(nf * nc);
  ent_ctx* c = densities_gb300_context();
  const int s = ent_read_xtc(c, fname.c_str(), nullptr, 0, 'R', _p->rows.data(), nf, nc);
  if (s != ENT_OK) die(std::string("error reading ") + fname + ": " + ent_last_error(c));
  _p->n_rows = nf;
  _p->n_cols = nc;
}

XtcHandler::~XtcHandler() {
  if (!_p->writing || _p->n_rows == 0) return;
  const int s = ent_write_xtc(_p->path.c_str(), _p->rows.data(), _p->n_rows, _p->n_cols, 'R',
                              1000.f);
  if (s != ENT_OK) die(std::string("error writing ") + _p->path + ": " + ent_xtc_last_error());
}

std::vector<float> XtcHandler::next() {
  if (_p->reading && _p->pos < _p->n_rows) {
    const float* r = _p->rows.data() + _p->pos++ * _p->n_cols;
    return std::vector<float>(r, r + _p->n_cols);
  }
  _p->at_end = true;
  return {};
}

void XtcHandler::write(std::vector<float> row) {
  if (!_p->writing) return;
  if (_p->n_rows == 0) _p->n_cols = row.size();
  if (row.size() != _p->n_cols || row.size() % 3 != 0 || row.empty())
    die("error: XTC rows must hold the same 3 x natoms values");
  _p->rows.insert(_p->rows.end(), row.begin(), row.end());
  ++_p->n_rows;
}

bool XtcHandler::eof() { return _p->at_end; }

// ------------------------------------------------------------------ open

FilePointer open(std::string fname, std::string mode) {
  if (is_xtc_name(fname)) return FilePointer(new XtcHandler(fname, mode));
  return FilePointer(new AsciiHandler(fname, mode));
}

}  // namespace CoordsFile
