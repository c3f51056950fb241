// Drop-in replacement of the reference's coordinate-file interface
// (coords_file/coords_file.hpp: namespace CoordsFile, Handler, AsciiHandler,
// XtcHandler, open, split), backed by the entropical GB300 C ABI. Code written
// against the reference compiles unchanged against this header (no xdrfile
// headers needed) and links against libentropical_shim.so.
//
// Behaviour kept from the reference (coords_file.cpp):
//  * open() picks XtcHandler for names longer than four characters ending in
//    ".xtc", else AsciiHandler;
//  * AsciiHandler::next() returns the next non-empty line split into floats,
//    {} and eof() == true at the end; as in the reference, a last line not
//    followed by a line break is not returned, and whitespace after the last
//    value repeats that value (split() reads while the stream is good, and a
//    read that finds no number leaves its variable as it was);
//  * AsciiHandler::write() writes " v0 v1 ..." and a line break, default
//    stream formatting; an unknown mode prints "unknown mode: <mode>" and
//    exits with EXIT_FAILURE;
//  * XtcHandler::next() returns frame after frame as rows of 3 natoms floats
//    (x0, y0, z0, x1, ...), then {} and eof() == true; write() appends a row
//    as a frame with step and time = the row's number, a zero box and
//    precision 1000, and the file's bytes equal the reference writer's.
//
// Differences: XtcHandler in "r" mode decodes the whole trajectory on the GPU
// when it is opened (the rows then come from host memory), instead of one
// read_xtc per next(); in "w" mode it collects the rows and writes the file
// when the handler is destroyed. Rows of another length than the first in
// one XTC file are an error here (message, exit), where the reference writes
// frames its own reader stops at.
#pragma once

#include <memory>
#include <sstream>
#include <string>
#include <vector>

namespace CoordsFile {

class Handler {
 public:
  virtual ~Handler() {}
  virtual std::vector<float> next() = 0;
  virtual void write(std::vector<float> row) = 0;
  virtual bool eof() = 0;
};

class AsciiHandler : public Handler {
 public:
  AsciiHandler(std::string fname, std::string mode);
  ~AsciiHandler();
  std::vector<float> next();
  void write(std::vector<float> row);
  bool eof();

 private:
  struct Impl;
  std::unique_ptr<Impl> _p;
};

class XtcHandler : public Handler {
 public:
  XtcHandler(std::string fname, std::string mode);
  ~XtcHandler();
  std::vector<float> next();
  void write(std::vector<float> row);
  bool eof();

 private:
  struct Impl;
  std::unique_ptr<Impl> _p;
};

typedef std::unique_ptr<Handler> FilePointer;

// Values of a whitespace-separated line, read while the stream is good; a
// read that finds no number adds the previous value again (T() for the first),
// which is what the reference's reads into an uninitialised variable give.
template <typename T>
std::vector<T> split(std::string s) {
  std::vector<T> v;
  std::istringstream in(s);
  T last{};
  while (in.good()) {
    T x = last;
    in >> x;
    v.push_back(x);
    last = x;
  }
  return v;
}

FilePointer open(std::string fname, std::string mode);

}  // namespace CoordsFile
