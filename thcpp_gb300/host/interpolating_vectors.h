// InterpolatingVectors::IVecs with the reference's interface
// (src/interpolating_vectors.h:12-41): ISDF interpolating vectors, the FFT Coulomb matrix
// and its Cholesky factor on the GPU, written in the QMCPACK HDF5 layout.
#pragma once

#include <string>
#include <vector>

#include "context_handler.h"
#include "thc_json.h"

namespace InterpolatingVectors {

class IVecs {
 public:
  IVecs(nlohmann::json& input_file, ContextHandler::BlacsHandler& BH,
        std::vector<int>& interp_indxs, bool half_rotated, bool append);
  void kernel(ContextHandler::BlacsHandler& BH);
  void dump_qmcpack_data(int thc_cfac, int thc_half_cfac, ContextHandler::BlacsHandler& BH);

 private:
  std::string input_file, output_file;
  int nbasis = 0;
  bool half_rotate = false;
  std::vector<int> fft_grid;
  std::vector<int> interp;
  std::vector<double> phi;   // N_g x N_o real orbitals, or N_g x N_o (re, im) pairs
  bool complex_orbitals = false;
  std::vector<double> phi_occ;  // N_g x N_occ (aoR_half), half-rotated runs only
  int nocc = 0;
  std::string prefix;           // "HalfTransformed" for half-rotated runs
  long long ngrid = 0;
};

}  // namespace InterpolatingVectors
