#pragma once

#include "common.cuh"

namespace thc {

int get_plan(Ctx* c, int n0, int n1, int n2, int batch, cufftType type, cufftHandle* out);

int isdf_run(Ctx* c, const double* phi, long long ng, int no, const int* idx, int nmu,
             const int* mesh, const double* coul, double shift_rel, double* out_orb,
             double* out_M, double* out_L, thc_isdf_stats* stats);

// Mixed-precision variant (mesh already validated and copied to the host).
int isdf_run_mixed(Ctx* c, const double* phi, long long ng, int no, const int* idx, int nmu,
                   const int* mesh, const double* coul, double shift_rel, double* out_orb,
                   double* out_M, double* out_L, thc_isdf_stats* stats);

int kmeans_run(Ctx* c, const double* grid, const double* rho, long long ng, int nmu,
               const int* init, int max_it, double threshold, int* out_idx,
               thc_kmeans_stats* stats);

int kmeans_history(Ctx* c, double* diff, double* pct, int n);

}  // namespace thc
