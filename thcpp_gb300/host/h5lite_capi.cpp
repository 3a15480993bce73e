// C entry points over h5lite, so that Python tools (the synthetic orbital-file writer and
// the tests) can read and write the same HDF5 files as the C++ solver classes.
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "h5lite.h"

namespace {
thread_local std::string g_err;
}

extern "C" {

const char* h5l_last_error() { return g_err.c_str(); }

void* h5l_writer_open(const char* path, int truncate)
{
  try {
    return new h5lite::Writer(path, truncate != 0);
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}

// kind: 0 f64, 1 i32, 2 complex128 ({r, i} compound; data = re, im pairs)
int h5l_writer_write(void* w, const char* dset, int kind, int rank, const unsigned long long* dims,
                     const void* data)
{
  try {
    std::vector<uint64_t> d(dims, dims + rank);
    auto* wr = static_cast<h5lite::Writer*>(w);
    if (kind == 0) wr->write_f64(dset, d, (const double*)data);
    else if (kind == 1) wr->write_i32(dset, d, (const int*)data);
    else wr->write_c128(dset, d, (const double*)data);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

void h5l_writer_close(void* w) { delete static_cast<h5lite::Writer*>(w); }

void* h5l_reader_open(const char* path)
{
  try {
    return new h5lite::Reader(path);
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}

void h5l_reader_close(void* r) { delete static_cast<h5lite::Reader*>(r); }

// kind out: 0 int, 1 float, 2 complex, 3 other, -1 group / missing
int h5l_reader_info(void* r, const char* dset, int* kind, int* rank, unsigned long long* dims)
{
  try {
    auto* rd = static_cast<h5lite::Reader*>(r);
    if (!rd->exists(dset) || rd->is_group(dset)) {
      *kind = -1;
      *rank = 0;
      return 0;
    }
    auto inf = rd->info(dset);
    *kind = (int)inf.kind;
    *rank = (int)inf.dims.size();
    for (size_t i = 0; i < inf.dims.size() && i < 8; i++) dims[i] = inf.dims[i];
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

// Reads as f64 (complex: re, im pairs when as_complex != 0).
int h5l_reader_read(void* r, const char* dset, int as_complex, double* out, unsigned long long n)
{
  try {
    auto* rd = static_cast<h5lite::Reader*>(r);
    std::vector<double> v = as_complex ? rd->read_c128(dset) : rd->read_f64(dset);
    if (v.size() != n) {
      g_err = "size mismatch";
      return 1;
    }
    std::memcpy(out, v.data(), n * sizeof(double));
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

}  // extern "C"
