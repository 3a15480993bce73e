// thcpp_gb300.x input.json -- the reference driver's sequence (src/main.cpp:18-77) on one
// GPU: options, interpolating points, interpolating vectors + Luv, QMCPACK metadata.
#include <chrono>
#include <cstdlib>
#include <fstream>
#include <iostream>

#include "context_handler.h"
#include "interpolating_points.h"
#include "interpolating_vectors.h"
#include "thc_json.h"

namespace UTILS {

// src/utils.h:73-113 without the broadcasts.
inline void parse_simple_opts(nlohmann::json& input, int rank, int& thc_cfac, int& thc_half_cfac,
                              bool& half_rotated, bool& find_interp_vec)
{
  (void)rank;
  thc_cfac = input.at("thc_cfac").get<int>();
  try {
    find_interp_vec = input.at("find_interp_vec").get<bool>();
  } catch (nlohmann::json::out_of_range& error) {
    find_interp_vec = true;
  }
  if (find_interp_vec) {
    try {
      half_rotated = input.at("half_rotated").get<bool>();
    } catch (nlohmann::json::out_of_range& error) {
      std::cout << " * Performing THC on full orbital basis." << std::endl;
      half_rotated = false;
    }
    if (half_rotated) {
      try {
        thc_half_cfac = input.at("thc_half_cfac").get<int>();
      } catch (nlohmann::json::out_of_range& error) {
        std::cout << " * thc_half_cfac not specified." << std::endl;
        std::cout << " * Setting to be the same as thc_cfac." << std::endl;
        thc_half_cfac = thc_cfac;
      }
    }
  }
}

}  // namespace UTILS

int main(int argc, char** argv)
{
  ContextHandler::BlacsHandler BH;
  if (argc != 2) {
    std::cout << "Usage: thcpp_gb300.x input.json" << std::endl;
    exit(EXIT_FAILURE);
  }
  auto t0 = std::chrono::steady_clock::now();
  nlohmann::json input_data;
  {
    std::ifstream input_file(argv[1]);
    if (!input_file) {
      std::cerr << "cannot open " << argv[1] << std::endl;
      exit(EXIT_FAILURE);
    }
    input_file >> input_data;
  }
  std::cout << " * Running on 1 process (GB300)." << std::endl;
  std::cout << " * Input file:" << std::endl << input_data.dump(4) << std::endl << std::endl;
  // The reference leaves thc_half_cfac unset when half_rotated is false; here it defaults to
  // thc_cfac so that THC/dims records N_mu in both slots.
  int thc_cfac = 0, thc_half_cfac = 0;
  bool half_rotate = false, find_interp_vec = true;
  UTILS::parse_simple_opts(input_data, BH.rank, thc_cfac, thc_half_cfac, half_rotate, find_interp_vec);
  if (!half_rotate) thc_half_cfac = thc_cfac;
  InterpolatingPoints::IPoints IPSolver(input_data, BH);
  std::vector<int> interp_indxs = IPSolver.kernel(input_data, BH, thc_cfac, false);
  if (find_interp_vec) {
    bool half_rotate_first = false;
    bool open_file = true;
    InterpolatingVectors::IVecs IVSolver(input_data, BH, interp_indxs, half_rotate_first, open_file);
    IVSolver.kernel(BH);
    if (!half_rotate) IVSolver.dump_qmcpack_data(thc_cfac, thc_half_cfac, BH);
  }
  if (find_interp_vec && half_rotate) {
    // Second pass with the half-rotated products, new points when thc_half_cfac differs
    // (src/main.cpp:63-72), appended to the same output file.
    if (thc_half_cfac != thc_cfac) {
      InterpolatingPoints::IPoints IP(input_data, BH);
      interp_indxs = IP.kernel(input_data, BH, thc_half_cfac, half_rotate);
    }
    bool open_file = false;
    InterpolatingVectors::IVecs IVSolver(input_data, BH, interp_indxs, half_rotate, open_file);
    IVSolver.kernel(BH);
    IVSolver.dump_qmcpack_data(thc_cfac, thc_half_cfac, BH);
  }
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::cout << " * Total simulation time : " << secs << " seconds." << std::endl;
  return 0;
}
