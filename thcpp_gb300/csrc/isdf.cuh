#pragma once

#include "common.cuh"

namespace thc {

int get_plan(Ctx* c, int n0, int n1, int n2, int batch, cufftType type, cufftHandle* out);

// Forward real-to-complex FFTs of `count` real n0 x n1 x n2 fields stored back to back (`in`)
// into their half spectra (`out`, n0 n1 (n2/2+1) complex each); `type` is CUFFT_D2Z or
// CUFFT_R2C.  Runs in chunks of at most kFftChunk fields so that cuFFT's work area stays a
// few GB at the largest meshes.
constexpr int kFftChunk = 1024;
int fft_forward(Ctx* c, int n0, int n1, int n2, int count, cufftType type, void* in, void* out);

// With phi_occ (N_g x nocc) the half-rotated products replace P o P: Z = P_occ o P,
// C = Z[:, idx]; M is returned without a Cholesky factor (out_L unused) and the occupied
// orbitals at the interpolating points go to out_orb_occ.  This path runs in FP64 in both
// precisions.  With complex_orbitals, phi holds N_o (re, im) pairs per point and
// Z = |Phi_mu^H Phi|^2 (real, so the rest of the path is unchanged); FP64 as well.
int isdf_run(Ctx* c, const double* phi, long long ng, int no, const int* idx, int nmu,
             const int* mesh, const double* coul, double shift_rel, double* out_orb,
             double* out_M, double* out_L, thc_isdf_stats* stats,
             const double* phi_occ = nullptr, int nocc = 0, double* out_orb_occ = nullptr,
             bool complex_orbitals = false);

// Mixed-precision variant (mesh already validated and copied to the host).
int isdf_run_mixed(Ctx* c, const double* phi, long long ng, int no, const int* idx, int nmu,
                   const int* mesh, const double* coul, double shift_rel, double* out_orb,
                   double* out_M, double* out_L, thc_isdf_stats* stats);

// Scratch source of one k-means call: the context's grow-only workspace (base == nullptr)
// or a fixed, caller-provided device region that is carved up in order (256-byte aligned);
// a request that does not fit returns nullptr.
struct KmAlloc {
  Ctx* c = nullptr;
  char* base = nullptr;
  size_t cap = 0, used = 0;
  void* get(Slot s, size_t bytes)
  {
    if (!base) return ws_get(c, s, bytes);
    size_t off = (used + 255) & ~(size_t)255;
    if (off > cap || bytes > cap - off) return nullptr;
    used = off + bytes;
    return base + off;
  }
};

// With `fixed` set, every device buffer comes from that region: no device memory is
// allocated, no CUDA graph is built and no profiling events are recorded.
int kmeans_run(Ctx* c, const double* grid, const double* rho, long long ng, int nmu,
               const int* init, int max_it, double threshold, int* out_idx,
               thc_kmeans_stats* stats, KmAlloc* fixed = nullptr);

int kmeans_history(Ctx* c, double* diff, double* pct, int n);

// Half-rotated ISDF with complex orbitals (halfc.cu): phi (N_g x N_o) and phi_occ
// (N_g x N_occ) as (re, im) pairs; FP64 in both precisions.
int isdf_half_complex_run(Ctx* c, const double* phi, long long ng, int no, const double* phi_occ,
                          int nocc, const int* idx, int nmu, const int* mesh, const double* coul,
                          double* out_orb, double* out_orb_occ, double* out_M,
                          thc_isdf_stats* stats);

int qrcp_run(Ctx* c, const double* phi, long long ng, int no, const double* phi_occ, int nocc,
             int npts, int* out_idx, int* out_order, double* out_diag, thc_qrcp_stats* stats,
             bool complex_orbitals = false);

}  // namespace thc
