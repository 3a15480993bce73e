// In-memory stand-ins for the reference's HDF5-backed matrix and reader -- TEST
// INFRASTRUCTURE ONLY.
//
// Force-included (g++ -include) ahead of the reference's src/kmeans.cpp.  It pre-defines the
// include guards of src/distributed_matrix.h and src/h5helper.h (which need the HDF5 C++
// API and ScaLAPACK) and supplies the few members src/kmeans.cpp and the inline functions of
// src/matrix_operations.h use:
//   * DistributedMatrix::Matrix<T>(filename, name, grid): the datasets are served from an
//     in-memory table (thc_ref::dataset) instead of the orbital file, with the reference's
//     read semantics at one rank (distributed_matrix.h:116-197): C-order store,
//     nrows = dims[0], ncols = dims[1];
//   * H5Helper::read_dims(filename, name, dims): the same table's shapes.
// Everything else -- src/kmeans.cpp, src/kmeans.h, src/matrix_operations.h,
// src/context_handler.h, src/utils.h -- is the reference's own source, compiled where it
// lies.
#ifndef THC_REF_PRELUDE_H
#define THC_REF_PRELUDE_H

#include <climits>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <iostream>
#include <map>
#include <string>
#include <vector>

#include "mpi.h"
#include "context_handler.h"
#include "utils.h"

#define DISTRIBUTED_MATRIX_H
#define READ_MATRIX_H

typedef unsigned long long hsize_t;

namespace thc_ref {
struct Dataset {
  hsize_t rows = 0, cols = 0;
  std::vector<double> values;   // C order
};
inline std::map<std::string, Dataset>& table()
{
  static std::map<std::string, Dataset> t;
  return t;
}
inline const Dataset& dataset(const std::string& name)
{
  auto it = table().find(name);
  if (it == table().end()) {
    std::fprintf(stderr, "thc_ref: dataset %s not provided\n", name.c_str());
    std::exit(2);
  }
  return it->second;
}
}  // namespace thc_ref

namespace H5Helper {
inline void read_dims(std::string, std::string data_name, std::vector<hsize_t>& dims)
{
  const thc_ref::Dataset& d = thc_ref::dataset(data_name);
  dims.resize(2);
  dims[0] = d.rows;
  dims[1] = d.cols;
}
}  // namespace H5Helper

namespace DistributedMatrix {
template <class T>
class Matrix {
 public:
  Matrix() : desc(9) {}
  Matrix(int m, int n, ContextHandler::BlacsGrid&) : nrows(m), ncols(n), desc(9)
  {
    local_nrows = m;
    local_ncols = n;
    store.assign((size_t)m * n, T(0));
  }
  Matrix(int m, int n, ContextHandler::BlacsGrid& g, int br, int bc) : Matrix(m, n, g)
  {
    block_nrows = br;
    block_ncols = bc;
  }
  Matrix(std::string, std::string name, ContextHandler::BlacsGrid&, bool row_major = true,
         bool = false)
      : desc(9)
  {
    const thc_ref::Dataset& d = thc_ref::dataset(name);
    store.assign(d.values.begin(), d.values.end());
    nrows = (int)(row_major ? d.rows : d.cols);
    ncols = (int)(row_major ? d.cols : d.rows);
    local_nrows = nrows;
    local_ncols = ncols;
  }
  void initialise_descriptor(std::vector<int>&, ContextHandler::BlacsGrid&, int& nr, int& nc)
  {
    nr = nrows;
    nc = ncols;
  }
  void initialise_descriptor(std::vector<int>&, ContextHandler::BlacsGrid&, int& nr, int& nc,
                             int, int)
  {
    nr = nrows;
    nc = ncols;
  }
  void setup_matrix(int, int, ContextHandler::BlacsGrid&) {}
  void setup_matrix(int, int, ContextHandler::BlacsGrid&, int, int) {}
  void gather_block_cyclic(int) {}
  void scatter_block_cyclic(int) {}
  int nrows = 0, ncols = 0;
  int block_nrows = 64, block_ncols = 64;
  int local_nrows = 0, local_ncols = 0;
  int ccyc_nrows = 0, ccyc_ncols = 0;
  int lld = 1;
  int izero = 0;
  int init_row_idx = 1, init_col_idx = 1;
  int info = 0;
  std::vector<T> store;
  std::vector<int> desc;
};
}  // namespace DistributedMatrix

#endif
