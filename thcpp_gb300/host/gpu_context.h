// Process-wide GPU context used by the solver classes (one per process, like the
// reference's one-rank-per-process model), configured from the input JSON's optional
// "gpu" block: {"device": 0, "precision": "fp64" | "mixed"}.
#pragma once

#include "../../include/thc_gb300.h"
#include "thc_json.h"

namespace thc_host {

// Returns the context, creating it on first use (exits with the status on failure).
thc_ctx* context(const nlohmann::json* input = nullptr);
void check(int status, const char* what);

}  // namespace thc_host
