// InterpolatingPoints::IPoints with the reference's interface
// (src/interpolating_points.h:11-19): k-means interpolating points on the GPU.
#pragma once

#include <string>
#include <vector>

#include "context_handler.h"
#include "thc_json.h"

namespace InterpolatingPoints {

class IPoints {
 public:
  IPoints(nlohmann::json& input_file, ContextHandler::BlacsHandler& BH);
  std::vector<int> kernel(nlohmann::json& input_file, ContextHandler::BlacsHandler& BH, int thc_cfac,
                          bool half_rotate = false);

 private:
  std::string solver = "kmeans";
};

}  // namespace InterpolatingPoints
