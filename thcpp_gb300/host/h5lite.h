// h5lite: a small self-contained HDF5 reader/writer for thcpp's orbital and QMCPACK files.
//
// Written from the public HDF5 File Format Specification (version 3.0) for the subset
// those files use (libhdf5 is not available on the build or GPU hosts):
//   reading  superblock versions 0/1, version-1 object headers (with continuation
//            blocks), symbol-table groups (v1 B-trees + local heaps), contiguous,
//            compact and chunked (v1 B-tree index, deflate filter) dataset layouts,
//            fixed-point, IEEE floating-point and compound {r, i} datatypes (h5py's
//            complex128).
//   writing  superblock version 0, symbol-table groups, contiguous little-endian
//            f64 / i32 datasets (complex data as a trailing dimension of 2, the
//            QMCPACK convention of src/h5helper.cpp:63-76).
// Datasets are addressed by absolute path ("/Hamiltonian/THC/Luv").
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace h5lite {

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

enum class Kind { Int, Float, Complex, Other };

struct Info {
  std::vector<uint64_t> dims;
  Kind kind = Kind::Other;
  int elem_size = 0;
};

class Reader {
 public:
  explicit Reader(const std::string& path);
  ~Reader();
  bool exists(const std::string& path) const;
  bool is_group(const std::string& path) const;
  Info info(const std::string& path) const;
  // Numeric conversions: ints and floats to double; complex reads (re, im) pairs.
  std::vector<double> read_f64(const std::string& path, std::vector<uint64_t>* dims = nullptr) const;
  std::vector<int> read_i32(const std::string& path, std::vector<uint64_t>* dims = nullptr) const;
  std::vector<double> read_c128(const std::string& path, std::vector<uint64_t>* dims = nullptr) const;
  // Names of the members of a group.
  std::vector<std::string> list(const std::string& group) const;

 private:
  struct Impl;
  std::unique_ptr<Impl> p_;
};

// Accumulates datasets and rewrites the file after every addition: raw data is appended,
// then fresh metadata for the whole tree, then the superblock at offset 0 is updated.
class Writer {
 public:
  // truncate = true starts an empty file; false reloads the existing file's datasets.
  Writer(const std::string& path, bool truncate);
  void write_f64(const std::string& path, const std::vector<uint64_t>& dims, const double* data);
  void write_i32(const std::string& path, const std::vector<uint64_t>& dims, const int* data);
  // complex128 as the compound {r: f64, i: f64} that h5py writes (data: re, im pairs).
  void write_c128(const std::string& path, const std::vector<uint64_t>& dims, const double* data);
  void create_group(const std::string& path);

 private:
  struct Node;
  void add(const std::string& path, const std::vector<uint64_t>& dims, int kind, const void* data,
           size_t bytes);
  void flush();
  std::string path_;
  std::shared_ptr<Node> root_;
  uint64_t eof_ = 0;
};

}  // namespace h5lite
