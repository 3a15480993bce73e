// FP64 dense kernels shared by the ISDF driver.
#pragma once

#include "common.cuh"

namespace thc {

enum GemmMode : int { GEMM_STORE = 0, GEMM_SQUARE = 1 };

// C[m, n] = mode(alpha * sum_k A(m, k) dk[k >> dk_shift] B(k, n)) + beta C[m, n]
// with A(m, k) = A[m*sam + k*sak], B(k, n) = B[n*sbn + k*sbk] and row-major C.
// GEMM_SQUARE stores the squared product.  lower_only restricts C to n <= m.
struct GemmArgs {
  long long M = 0, N = 0;
  int K = 0;
  const double* A = nullptr;
  long long sam = 0, sak = 1;
  const double* B = nullptr;
  long long sbn = 0, sbk = 1;
  double* C = nullptr;
  long long ldc = 0;
  const double* dk = nullptr;
  int dk_shift = 0;
  double alpha = 1.0, beta = 0.0;
  int mode = GEMM_STORE;
  int lower_only = 0;
  const int* skip_flag = nullptr;   // if non-null and set, the kernel does nothing
  int ksplit = 1;                    // > 1: K is split over blockIdx.z into FP64 partials
  double* part = nullptr;            // ksplit x M x N partial buffer (row-major, ld = N)
  int aliased = 0;                   // C overlaps A or B: products go through partials
  // Known zeros: A(m, k) = 0 for k < m (a_zero_below) / B(k, n) = 0 for k < n
  // (b_zero_below), as for a lower-triangular factor read transposed / as it is.  A tile
  // then starts its k loop at its first row / column: the skipped terms are exact zeros,
  // so the result is bit-identical.
  int a_zero_below = 0, b_zero_below = 0;
  int lower_offset = 0;              // lower_only keeps n <= m + lower_offset (C's own indices)
  int no_split = 0;                  // no split of K (no shared partial buffer: a GEMM that
                                     // runs beside others on a second stream)
  int tile = 64;                     // CTA tile edge (64, 32 or 16; chosen by dgemm)
};

struct CholStatus {
  int flag;        // set on breakdown; later kernels of the same solve become no-ops
  int info;        // 1-based index of the failing pivot
  double min_piv;  // smallest / largest accepted pivot (before sqrt)
  double max_piv;
};

// With ksplit <= 1 and no part buffer, dgemm picks the tile edge and a split of K itself so
// that the grid covers the GPU (the FP64 pipe of one SM is narrow, so small GEMMs must spread
// over many SMs); split partials are summed in split order (deterministic).
int dgemm(Ctx* c, const GemmArgs& g);
// Cholesky with GEMM panels; dinv receives the inverted NB x NB diagonal blocks
// (NB = 64: ceil(n/64) x 64 x 64 doubles).
int potrf_inv(Ctx* c, double* A, long long ld, int n, const double* thr, CholStatus* cs,
              double* dinv);
// Cinv = (L L^T)^{-1} via X = L^{-1}; X (n x ld) and T (64 x n) are scratch.
// With Cinv == nullptr only X = L^{-1} is formed.
int chol_inverse(Ctx* c, const double* L, long long ld, int n, const double* dinv, double* X,
                 double* T, double* Cinv, const CholStatus* cs);
// Iterative refinement of a shifted solve, in closed form.  With L L^T = C + sI and
// X = L^{-1} (n x n, ld n), k steps zeta_{j+1} = zeta_j + (C + sI)^{-1} (Z^T - C zeta_j)
// from zeta_0 = (C + sI)^{-1} Z^T give zeta_k = X^T P X Z^T, P = sum_{j<=k} (s X X^T)^j
// (eigenvalue lambda of C: filter 1 - (s / (lambda + s))^{k+1} on 1 / lambda).  Writes
// Xt = P X by Horner's rule in FP64 (k + 1 GEMMs of n^3); G and T are n x n scratch.
int refine_polynomial(Ctx* c, const double* X, int n, double s, int k, double* G, double* T,
                      double* Xt);
int set_identity(Ctx* c, double* A, long long ld, int n);
int add_diag_shift(Ctx* c, double* A, long long ld, int n, double rel, double* shift_out);
int diag_mean(Ctx* c, const double* A, long long ld, int n, double* out);
int zpotrf_small(Ctx* c, double* A, int n, const double* thr, CholStatus* cs);

}  // namespace thc
