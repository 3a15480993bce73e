// Runs the reference's own KMeans::KMeansSolver (src/kmeans.cpp, compiled unmodified from
// the reference tree) on one rank -- TEST INFRASTRUCTURE ONLY.
//
//   kmeans_ref <input.bin> <thc_cfac> <max_it> <threshold> <rng_seed> <out_idx.bin>
//
// input.bin: int64 N_g, int64 N_o, then N_g x 3 doubles (real_space_grid, C order) and
// N_g doubles (the density).  The solver reads them through the in-memory datasets of
// prelude.h as `real_space_grid`, `density` and the shape of `aoR` (N_g x N_o); its own
// stdout (the step table printed every 10 iterations) passes through unchanged.
// out_idx.bin receives the N_mu = thc_cfac * N_o interpolating-point indices as int32.
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "json.hpp"
#include "kmeans.h"

// One-rank BlacsGrid / BlacsHandler (their reference definitions, src/context_handler.cpp,
// set up BLACS process grids; at one rank every grid is the single process).
namespace ContextHandler {
BlacsGrid::~BlacsGrid() {}
BlacsHandler::BlacsHandler()
{
  rank = 0;
  nprocs = 1;
  proc_rows = 1;
  proc_cols = 1;
  comm = MPI_COMM_WORLD;
  for (BlacsGrid* g : {&Root, &Square, &Column}) {
    g->rank = 0;
    g->nprocs = 1;
    g->nrows = 1;
    g->ncols = 1;
    g->row = 0;
    g->col = 0;
    g->ctxt = 0;
    g->comm = MPI_COMM_WORLD;
  }
  Root.layout = root;
  Square.layout = square;
  Column.layout = column;
}
BlacsHandler::~BlacsHandler() {}
}  // namespace ContextHandler

int main(int argc, char** argv)
{
  if (argc != 7) {
    std::fprintf(stderr, "usage: %s input.bin thc_cfac max_it threshold rng_seed out.bin\n",
                 argv[0]);
    return 2;
  }
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int64_t ng = 0, no = 0;
  if (std::fread(&ng, 8, 1, f) != 1 || std::fread(&no, 8, 1, f) != 1) return 2;
  thc_ref::Dataset grid, rho, aor;
  grid.rows = ng;
  grid.cols = 3;
  grid.values.resize((size_t)ng * 3);
  rho.rows = ng;
  rho.cols = 1;
  rho.values.resize((size_t)ng);
  if (std::fread(grid.values.data(), 8, grid.values.size(), f) != grid.values.size()) return 2;
  if (std::fread(rho.values.data(), 8, rho.values.size(), f) != rho.values.size()) return 2;
  std::fclose(f);
  aor.rows = ng;
  aor.cols = no;
  thc_ref::table()["real_space_grid"] = grid;
  thc_ref::table()["density"] = rho;
  thc_ref::table()["aoR"] = aor;

  nlohmann::json input;
  input["orbital_file"] = "in-memory";
  input["interpolating_points"]["kmeans"]["max_it"] = std::stoi(argv[3]);
  input["interpolating_points"]["kmeans"]["threshold"] = std::stod(argv[4]);
  input["interpolating_points"]["kmeans"]["rng_seed"] = std::stoi(argv[5]);
  input["interpolating_points"]["kmeans"]["density"] = "density";
  ContextHandler::BlacsHandler bh;
  std::vector<int> idx;
  KMeans::KMeansSolver solver(input, bh);
  solver.kernel(bh, idx, std::stoi(argv[2]));
  FILE* o = std::fopen(argv[6], "wb");
  if (!o) return 2;
  std::fwrite(idx.data(), sizeof(int), idx.size(), o);
  std::fclose(o);
  return 0;
}
