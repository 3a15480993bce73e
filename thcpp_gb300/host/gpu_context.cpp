#include "gpu_context.h"

#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>

namespace thc_host {

static thc_ctx* g_ctx = nullptr;

void check(int status, const char* what)
{
  if (status == THC_OK) return;
  std::cerr << " * ERROR: " << what << ": " << thc_status_string(status);
  if (g_ctx) std::cerr << " (" << thc_ctx_last_error(g_ctx) << ")";
  std::cerr << std::endl;
  exit(1);
}

thc_ctx* context(const nlohmann::json* input)
{
  if (g_ctx) return g_ctx;
  int device = 0;
  int precision = THC_PREC_FP64;
  if (input && input->contains("gpu")) {
    const auto& g = input->at("gpu");
    if (g.contains("device")) device = g.at("device").get<int>();
    if (g.contains("precision")) {
      std::string p = g.at("precision").get<std::string>();
      if (p == "mixed") precision = THC_PREC_MIXED;
      else if (p != "fp64") {
        std::cerr << " * ERROR: gpu.precision must be \"fp64\" or \"mixed\"" << std::endl;
        exit(1);
      }
    }
  }
  int st = thc_ctx_create(device, precision, &g_ctx);
  if (st) {
    std::cerr << " * ERROR: cannot create the GPU context on device " << device << ": "
              << thc_status_string(st) << std::endl;
    exit(1);
  }
  std::atexit([] {
    if (g_ctx) thc_ctx_destroy(g_ctx);
    g_ctx = nullptr;
  });
  return g_ctx;
}

}  // namespace thc_host
