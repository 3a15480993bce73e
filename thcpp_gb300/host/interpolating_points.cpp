// InterpolatingPoints::IPoints (reference: src/interpolating_points.cpp:11-63): solver
// selection from the JSON and dispatch to the k-means or QRCP selector.
#include "interpolating_points.h"

#include <cstdlib>
#include <iostream>

#include "kmeans.h"
#include "qrcp.h"

namespace InterpolatingPoints {

IPoints::IPoints(nlohmann::json& input, ContextHandler::BlacsHandler& BH)
{
  (void)BH;
  std::cout << "#################################################" << std::endl;
  std::cout << "##   Setting up interpolating point solver.    ##" << std::endl;
  std::cout << "#################################################" << std::endl;
  std::cout << std::endl;
  // The reference's key precedence: a "kmeans" block wins over a "qrcp" block, and with
  // neither the k-means solver runs after a note.
  const nlohmann::json& base = input.at("interpolating_points");
  if (base.contains("kmeans")) {
    solver = "kmeans";
  } else if (base.contains("qrcp")) {
    solver = "qrcp";
  } else {
    std::cout << "No solver specified." << std::endl;
    solver = "kmeans";
  }
}

std::vector<int> IPoints::kernel(nlohmann::json& input, ContextHandler::BlacsHandler& BH,
                                 int thc_cfac, bool half_rotate)
{
  std::vector<int> interp_indxs;
  if (solver == "qrcp") {
    std::cout << " * Using QRCP solver." << std::endl;
    std::cout << std::endl;
    QRCP::QRCPSolver QR(input, BH);
    QR.kernel(BH, interp_indxs, thc_cfac, half_rotate);
    return interp_indxs;
  }
  std::cout << " * Using K-Means solver." << std::endl;
  std::cout << std::endl;
  KMeans::KMeansSolver KM(input, BH);
  KM.kernel(BH, interp_indxs, thc_cfac);
  return interp_indxs;
}

}  // namespace InterpolatingPoints
