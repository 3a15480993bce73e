// Single-process stand-in for thcpp's BLACS process grids (src/context_handler.h:13-38).
// The GB300 build runs one process on one GPU, so every grid is the 1 x 1 grid of rank 0;
// the classes keep their names and fields so that callers written against the reference
// (main.cpp, the solver constructors) compile unchanged.
#pragma once

namespace ContextHandler {

enum Layouts { root, square, column };

class BlacsGrid {
 public:
  BlacsGrid() {}
  BlacsGrid(int nr, int nc, int rk, Layouts l) : rank(rk), nprocs(nr * nc), nrows(nr), ncols(nc), layout(l) {}
  int rank = 0;
  int nprocs = 1;
  int nrows = 1, ncols = 1;
  int row = 0, col = 0;
  int ctxt = 0;
  Layouts layout = root;
};

class BlacsHandler {
 public:
  BlacsHandler() : Root(1, 1, 0, root), Square(1, 1, 0, square), Column(1, 1, 0, column) {}
  int rank = 0;
  int nprocs = 1, proc_rows = 1, proc_cols = 1;
  BlacsGrid Root;
  BlacsGrid Square;
  BlacsGrid Column;
};

}  // namespace ContextHandler
