// KMeans::KMeansSolver with the reference's interface (src/kmeans.h:13-40), running on
// the GPU through the C ABI (thc_kmeans).
#pragma once

#include <string>
#include <vector>

#include "context_handler.h"
#include "thc_json.h"

namespace KMeans {

class KMeansSolver {
 public:
  KMeansSolver(nlohmann::json& input, ContextHandler::BlacsHandler& BH);
  ~KMeansSolver();
  void kernel(ContextHandler::BlacsHandler& BH, std::vector<int>& interp_indxs, int thc_cfac);

 private:
  std::string filename;
  int max_it = 0;
  double threshold = 0.0;
  unsigned int rng_seed = 0;
  std::string density_label;
};

}  // namespace KMeans
