// QRCP::QRCPSolver with the reference's interface (src/qrcp.h:11-28): interpolating points by
// QR with column pivoting of the pair-product matrix, on the GPU through thc_qrcp.
#pragma once

#include <string>
#include <vector>

#include "context_handler.h"
#include "thc_json.h"

namespace QRCP {

class QRCPSolver {
 public:
  QRCPSolver(nlohmann::json& input, ContextHandler::BlacsHandler& BH);
  ~QRCPSolver();
  void kernel(ContextHandler::BlacsHandler& BH, std::vector<int>& interp_indxs, int thc_cfac,
              bool half_rotate = false);

 private:
  std::string input_file;
  bool sub_sample = false;   // read as the reference does; unused there as well
};

}  // namespace QRCP
