// FP64 dense linear algebra on CUDA cores: GEMM, blocked Cholesky and triangular
// solves.  These carry the all-FP64 path, which replaces the reference's ScaLAPACK
// calls one for one:
//   pzgemm 'C','N'  (P = Phi_mu^H Phi, src/interpolating_vectors.cpp:117)  -> dgemm + square
//   pzgels 'N'      (least squares C X = Z, :416)                           -> potrf + trsm
//   pzherk 'L','C'  (M = zeta_hat^H zeta_hat, :278)                         -> dgemm lower
//   pzpotrf 'L'     (Luv, :289)                                             -> potrf
// GB300 runs FP64 at a small fraction of its FP32 rate, so these kernels are bound by
// the FP64 pipe; a 64x64x16 register-blocked tile keeps that pipe fed.
#include <cuda_runtime.h>
#include <math_constants.h>

#include <algorithm>

#include "common.cuh"
#include "dense64.cuh"

namespace thc {

namespace {

constexpr int BM = 64, BN = 64, BK = 16;

// C[m, n] = epilogue(sum_k A(m, k) * dk[k] * B(k, n)); AK / BK select which operand
// index is unit-stride so that the shared-memory loads stay coalesced.
template <bool AK, bool BK_>
__global__ void __launch_bounds__(256) dgemm_kernel(GemmArgs g)
{
  if (g.skip_flag && *g.skip_flag) return;
  long long m0 = (long long)blockIdx.y * BM, n0 = (long long)blockIdx.x * BN;
  if (g.lower_only && n0 > m0 + BM - 1) return;
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];
  int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4] = {};
  int kbeg = 0, kend = g.K;
  if (g.ksplit > 1) {
    int kc = ((g.K + g.ksplit - 1) / g.ksplit + BK - 1) / BK * BK;
    kbeg = blockIdx.z * kc;
    kend = min(g.K, kbeg + kc);
  }
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
    // 1024 elements of each tile, 4 per thread.
#pragma unroll
    for (int r = 0; r < 4; r++) {
      int e = threadIdx.x + 256 * r;
      int mm, kk;
      if (AK) { mm = e / BK; kk = e % BK; } else { kk = e / BM; mm = e % BM; }
      long long m = m0 + mm;
      int k = k0 + kk;
      double av = 0.0;
      if (m < g.M && k < kend) {
        av = g.A[m * g.sam + (long long)k * g.sak];
        if (g.dk) av *= g.dk[k >> g.dk_shift];
      }
      As[kk][mm] = av;
      int nn, kb;
      if (BK_) { nn = e / BK; kb = e % BK; } else { kb = e / BN; nn = e % BN; }
      long long n = n0 + nn;
      int kq = k0 + kb;
      Bs[kb][nn] = (n < g.N && kq < kend) ? g.B[n * g.sbn + (long long)kq * g.sbk] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk++) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = __fma_rn(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    long long m = m0 + ty + 16 * i;
    if (m >= g.M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      long long n = n0 + tx + 16 * j;
      if (n >= g.N) continue;
      if (g.lower_only && n > m) continue;
      double v = acc[i][j];
      if (g.ksplit > 1) {
        g.part[((long long)blockIdx.z * g.M + m) * g.N + n] = v;
        continue;
      }
      double* cp = g.C + m * g.ldc + n;
      if (g.mode == GEMM_SQUARE) v = v * v;
      else v = g.alpha * v;
      if (g.beta != 0.0) v += g.beta * *cp;
      *cp = v;
    }
  }
}

// Sum split-K partials in split order, then apply the epilogue.
__global__ void dgemm_reduce(GemmArgs g)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= g.M * g.N) return;
  long long m = e / g.N, n = e % g.N;
  if (g.lower_only && n > m) return;
  double v = 0.0;
  for (int z = 0; z < g.ksplit; z++) v += g.part[((long long)z * g.M + m) * g.N + n];
  double* cp = g.C + m * g.ldc + n;
  if (g.mode == GEMM_SQUARE) v = v * v;
  else v = g.alpha * v;
  if (g.beta != 0.0) v += g.beta * *cp;
  *cp = v;
}

// ---- Cholesky (lower, in place, row-major) --------------------------------------

constexpr int NB = 64;

// Factor the diagonal block at (k0, k0).  Pivots at or below `thr` stop the
// factorisation: info = global 1-based index, flag set.
__global__ void potrf_diag(double* A, long long ld, int n, int k0, const double* thr_p,
                           CholStatus* cs)
{
  if (cs->flag) return;
  double thr = thr_p ? *thr_p : 0.0;
  __shared__ double a[NB][NB + 1];
  __shared__ int bad;
  int nb = min(NB, n - k0);
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    int r = e / nb, c = e % nb;
    a[r][c] = A[(long long)(k0 + r) * ld + k0 + c];
  }
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < nb; j++) {
    if (threadIdx.x == 0) {
      double d = a[j][j];
      if (!(d > thr)) {
        bad = 1;
        cs->flag = 1;
        cs->info = k0 + j + 1;
      } else {
        double r = sqrt(d);
        a[j][j] = r;
        double p = d;
        if (p < cs->min_piv) cs->min_piv = p;
        if (p > cs->max_piv) cs->max_piv = p;
      }
    }
    __syncthreads();
    if (bad) break;
    double r = a[j][j];
    for (int i = j + 1 + threadIdx.x; i < nb; i += blockDim.x) a[i][j] /= r;
    __syncthreads();
    for (int e = threadIdx.x; e < (nb - j - 1) * (nb - j - 1); e += blockDim.x) {
      int i = j + 1 + e / (nb - j - 1), c = j + 1 + e % (nb - j - 1);
      if (c <= i) a[i][c] = __fma_rn(-a[i][j], a[c][j], a[i][c]);
    }
    __syncthreads();
  }
  if (bad) return;
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    int r = e / nb, c = e % nb;
    A[(long long)(k0 + r) * ld + k0 + c] = c <= r ? a[r][c] : 0.0;
  }
}

// Factor the diagonal block at (k0, k0) and invert its triangle: writes L_kk into A
// (upper part zeroed) and L_kk^{-1} into dinv (nb x nb, row-major, zero above the diagonal).
// Pivots at or below thr stop the factorisation (info = global 1-based index).
__global__ void __launch_bounds__(256) potrf_diag_inv(double* A, long long ld, int n, int k0,
                                                      const double* thr_p, CholStatus* cs,
                                                      double* dinv)
{
  if (cs->flag) return;
  double thr = thr_p ? *thr_p : 0.0;
  extern __shared__ double dsm[];                       // 2 x NB x (NB + 1) doubles
  double (*a)[NB + 1] = reinterpret_cast<double (*)[NB + 1]>(dsm);
  double (*v)[NB + 1] = reinterpret_cast<double (*)[NB + 1]>(dsm + NB * (NB + 1));
  __shared__ double rinv;
  __shared__ int bad;
  const int nb = min(NB, n - k0);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;   // 16 x 16 threads
  for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) {
    int r = e / NB, c = e % NB;
    a[r][c] = (r < nb && c < nb) ? A[(long long)(k0 + r) * ld + k0 + c] : (r == c ? 1.0 : 0.0);
    v[r][c] = 0.0;
  }
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < nb; j++) {
    if (threadIdx.x == 0) {
      double d = a[j][j];
      if (!(d > thr)) {
        bad = 1;
        cs->flag = 1;
        cs->info = k0 + j + 1;
      } else {
        double r = sqrt(d);
        a[j][j] = r;
        rinv = 1.0 / r;
        if (d < cs->min_piv) cs->min_piv = d;
        if (d > cs->max_piv) cs->max_piv = d;
      }
    }
    __syncthreads();
    if (bad) return;
    double ri = rinv;
    for (int i = j + 1 + threadIdx.x; i < nb; i += blockDim.x) a[i][j] *= ri;
    __syncthreads();
    // trailing lower update a[i][c] -= a[i][j] a[c][j], j < c <= i
    for (int i = j + 1 + ty; i < nb; i += 16)
      for (int c = j + 1 + tx; c <= i; c += 16) a[i][c] = __fma_rn(-a[i][j], a[c][j], a[i][c]);
    __syncthreads();
  }
  // Triangular inverse by columns: for column c, v[c][c] = 1/a[c][c] and
  // v[i][c] = -(sum_{k=c}^{i-1} a[i][k] v[k][c]) / a[i][i], i > c (one thread per column).
  for (int c = threadIdx.x; c < nb; c += blockDim.x) {
    v[c][c] = 1.0 / a[c][c];
    for (int i = c + 1; i < nb; i++) {
      double sacc = 0.0;
      for (int k = c; k < i; k++) sacc = __fma_rn(a[i][k], v[k][c], sacc);
      v[i][c] = -sacc / a[i][i];
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    int r = e / nb, c = e % nb;
    A[(long long)(k0 + r) * ld + k0 + c] = c <= r ? a[r][c] : 0.0;
    dinv[(long long)r * nb + c] = c <= r ? v[r][c] : 0.0;
  }
}

// Rows below the diagonal block: x L_kk^T = a, one thread per row.
__global__ void potrf_panel(double* A, long long ld, int n, int k0, CholStatus* cs)
{
  if (cs->flag) return;
  __shared__ double l[NB][NB + 1];
  int nb = min(NB, n - k0);
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    int r = e / nb, c = e % nb;
    l[r][c] = A[(long long)(k0 + r) * ld + k0 + c];
  }
  __syncthreads();
  long long row = (long long)k0 + nb + blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (row >= n) return;
  double x[NB];
  double* ar = A + row * ld + k0;
#pragma unroll 1
  for (int j = 0; j < nb; j++) {
    double s = ar[j];
    for (int t = 0; t < j; t++) s = __fma_rn(-x[t], l[j][t], s);
    x[j] = s / l[j][j];
  }
  for (int j = 0; j < nb; j++) ar[j] = x[j];
}

// Forward substitution on a diagonal block: B[k0..k0+nb, :] = L_kk^{-1} B[...], one thread
// per right-hand-side column.
__global__ void trsm_diag_fwd(const double* L, long long ld, int n, int k0, double* B,
                              long long ldb, long long nrhs, const CholStatus* cs)
{
  if (cs && cs->flag) return;
  __shared__ double l[NB][NB + 1];
  int nb = min(NB, n - k0);
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    int r = e / nb, c = e % nb;
    l[r][c] = L[(long long)(k0 + r) * ld + k0 + c];
  }
  __syncthreads();
  long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (col >= nrhs) return;
  double y[NB];
  for (int j = 0; j < nb; j++) {
    double s = B[(long long)(k0 + j) * ldb + col];
    for (int t = 0; t < j; t++) s = __fma_rn(-l[j][t], y[t], s);
    y[j] = s / l[j][j];
  }
  for (int j = 0; j < nb; j++) B[(long long)(k0 + j) * ldb + col] = y[j];
}

// Backward substitution with L_kk^T on a diagonal block.
__global__ void trsm_diag_bwd(const double* L, long long ld, int n, int k0, double* B,
                              long long ldb, long long nrhs, const CholStatus* cs)
{
  if (cs && cs->flag) return;
  __shared__ double l[NB][NB + 1];
  int nb = min(NB, n - k0);
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    int r = e / nb, c = e % nb;
    l[r][c] = L[(long long)(k0 + r) * ld + k0 + c];
  }
  __syncthreads();
  long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (col >= nrhs) return;
  double x[NB];
  for (int j = nb - 1; j >= 0; j--) {
    double s = B[(long long)(k0 + j) * ldb + col];
    for (int t = j + 1; t < nb; t++) s = __fma_rn(-l[t][j], x[t], s);
    x[j] = s / l[j][j];
  }
  for (int j = 0; j < nb; j++) B[(long long)(k0 + j) * ldb + col] = x[j];
}

__global__ void set_identity_k(double* A, long long ld, int n)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * n) return;
  long long r = e / n, c = e % n;
  A[r * ld + c] = r == c ? 1.0 : 0.0;
}

__global__ void add_diag(double* A, long long ld, int n, const double* trace_src, double rel,
                         double* shift_out)
{
  // shift = rel * trace / n, computed from the diagonal (trace_src = A itself).
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += trace_src[(long long)i * ld + i];
  for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    red[0] = rel * t / n;
    if (shift_out) *shift_out = red[0];
  }
  __syncthreads();
  double sh = red[0];
  for (int i = threadIdx.x; i < n; i += blockDim.x) A[(long long)i * ld + i] += sh;
}

__global__ void diag_mean_k(const double* A, long long ld, int n, double* out)
{
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += A[(long long)i * ld + i];
  for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    *out = t / n;
  }
}

// Complex Hermitian Cholesky (lower) for small matrices, single block, interleaved
// (re, im) row-major.  Pivots at or below thr set info and stop.
__global__ void zpotrf_small_k(double* A, int n, const double* thr_p, CholStatus* cs)
{
  double thr = thr_p ? *thr_p : 0.0;
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < n; j++) {
    if (threadIdx.x == 0) {
      double d = A[2 * ((long long)j * n + j)];
      if (!(d > thr)) {
        bad = 1;
        cs->flag = 1;
        cs->info = j + 1;
      } else {
        A[2 * ((long long)j * n + j)] = sqrt(d);
        A[2 * ((long long)j * n + j) + 1] = 0.0;
      }
    }
    __syncthreads();
    if (bad) return;
    double r = A[2 * ((long long)j * n + j)];
    for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) {
      A[2 * ((long long)i * n + j)] /= r;
      A[2 * ((long long)i * n + j) + 1] /= r;
    }
    __syncthreads();
    long long m = n - j - 1;
    for (long long e = threadIdx.x; e < m * m; e += blockDim.x) {
      int i = j + 1 + (int)(e / m), c = j + 1 + (int)(e % m);
      if (c > i) continue;
      // A[i][c] -= L[i][j] * conj(L[c][j])
      double ar = A[2 * ((long long)i * n + j)], ai = A[2 * ((long long)i * n + j) + 1];
      double br = A[2 * ((long long)c * n + j)], bi = -A[2 * ((long long)c * n + j) + 1];
      double* t = A + 2 * ((long long)i * n + c);
      t[0] -= ar * br - ai * bi;
      t[1] -= ar * bi + ai * br;
    }
    __syncthreads();
  }
}

}  // namespace

int dgemm(Ctx* c, const GemmArgs& g)
{
  if (g.M <= 0 || g.N <= 0) return THC_OK;
  dim3 grid((unsigned)cdiv(g.N, BN), (unsigned)cdiv(g.M, BM), (unsigned)std::max(1, g.ksplit));
  bool ak = g.sak == 1, bk = g.sbk == 1;
  ProfScope prof(c, "dgemm");
  if (ak && bk) dgemm_kernel<true, true><<<grid, 256, 0, c->stream>>>(g);
  else if (ak && !bk) dgemm_kernel<true, false><<<grid, 256, 0, c->stream>>>(g);
  else if (!ak && bk) dgemm_kernel<false, true><<<grid, 256, 0, c->stream>>>(g);
  else dgemm_kernel<false, false><<<grid, 256, 0, c->stream>>>(g);
  THC_LAUNCHED(c, "dgemm");
  if (g.ksplit > 1) {
    dgemm_reduce<<<(unsigned)cdiv(g.M * g.N, 256), 256, 0, c->stream>>>(g);
    THC_LAUNCHED(c, "dgemm_reduce");
  }
  return THC_OK;
}

// Blocked Cholesky whose panel solve is a GEMM with the inverted diagonal block; the
// inverted diagonal blocks are kept in dinv (nblk x 64 x 64) for the triangular inverse.
int potrf_inv(Ctx* c, double* A, long long ld, int n, const double* thr, CholStatus* cs,
              double* dinv)
{
  cudaStream_t s = c->stream;
  for (int k0 = 0; k0 < n; k0 += NB) {
    int nb = std::min(NB, n - k0);
    double* di = dinv + (long long)(k0 / NB) * NB * NB;
    const int smem = 2 * NB * (NB + 1) * (int)sizeof(double);
    THC_CUDA(c, cudaFuncSetAttribute(potrf_diag_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    potrf_diag_inv<<<1, 256, smem, s>>>(A, ld, n, k0, thr, cs, di);
    THC_LAUNCHED(c, "potrf_diag_inv");
    int rest = n - k0 - nb;
    if (rest <= 0) break;
    {
      // L_panel = A_panel L_kk^{-T}, in place (each CTA owns its rows; N = nb <= 64).
      GemmArgs g{};
      g.M = rest; g.N = nb; g.K = nb;
      g.A = A + (long long)(k0 + nb) * ld + k0; g.sam = ld; g.sak = 1;
      g.B = di; g.sbn = nb; g.sbk = 1;
      g.C = A + (long long)(k0 + nb) * ld + k0; g.ldc = ld;
      g.skip_flag = &cs->flag;
      int st = dgemm(c, g);
      if (st) return st;
    }
    GemmArgs g{};
    g.M = rest; g.N = rest; g.K = nb;
    g.A = A + (long long)(k0 + nb) * ld + k0; g.sam = ld; g.sak = 1;
    g.B = A + (long long)(k0 + nb) * ld + k0; g.sbn = ld; g.sbk = 1;
    g.C = A + (long long)(k0 + nb) * ld + k0 + nb; g.ldc = ld;
    g.alpha = -1.0; g.beta = 1.0; g.lower_only = 1; g.mode = GEMM_STORE;
    g.skip_flag = &cs->flag;
    int st = dgemm(c, g);
    if (st) return st;
  }
  return THC_OK;
}

// X = L^{-1} (lower, n x n, ld) from the factor L and its inverted diagonal blocks, block row
// by block row: X_ii = dinv_i, X[i, 0:i] = -dinv_i (L[i, 0:i] X[0:i, 0:i]).  T is an
// NB x n scratch.  Then Cinv = X^T X.
int chol_inverse(Ctx* c, const double* L, long long ld, int n, const double* dinv, double* X,
                 double* T, double* Cinv, const CholStatus* cs)
{
  cudaStream_t s = c->stream;
  THC_CUDA(c, cudaMemsetAsync(X, 0, sizeof(double) * (size_t)n * ld, s));
  int nblk = (n + NB - 1) / NB;
  for (int bi = 0; bi < nblk; bi++) {
    int i0 = bi * NB, nb = std::min(NB, n - i0);
    const double* di = dinv + (long long)bi * NB * NB;
    THC_CUDA(c, cudaMemcpy2DAsync(X + (long long)i0 * ld + i0, sizeof(double) * ld, di,
                                  sizeof(double) * nb, sizeof(double) * nb, nb,
                                  cudaMemcpyDeviceToDevice, s));
    if (bi == 0) continue;
    GemmArgs g{};
    g.M = nb; g.N = i0; g.K = i0;                       // T = L[i, 0:i] X[0:i, 0:i]
    g.A = L + (long long)i0 * ld; g.sam = ld; g.sak = 1;
    g.B = X; g.sbn = 1; g.sbk = ld;
    g.C = T; g.ldc = n;
    g.skip_flag = cs ? &cs->flag : nullptr;
    int st = dgemm(c, g);
    if (st) return st;
    GemmArgs h{};
    h.M = nb; h.N = i0; h.K = nb;                       // X[i, 0:i] = -dinv_i T
    h.A = di; h.sam = nb; h.sak = 1;
    h.B = T; h.sbn = 1; h.sbk = n;
    h.C = X + (long long)i0 * ld; h.ldc = ld;
    h.alpha = -1.0;
    h.skip_flag = cs ? &cs->flag : nullptr;
    st = dgemm(c, h);
    if (st) return st;
  }
  GemmArgs g{};
  g.M = n; g.N = n; g.K = n;                            // Cinv = X^T X
  g.A = X; g.sam = 1; g.sak = ld;
  g.B = X; g.sbn = 1; g.sbk = ld;
  g.C = Cinv; g.ldc = n;
  g.skip_flag = cs ? &cs->flag : nullptr;
  return dgemm(c, g);
}

int potrf(Ctx* c, double* A, long long ld, int n, const double* thr, CholStatus* cs)
{
  cudaStream_t s = c->stream;
  for (int k0 = 0; k0 < n; k0 += NB) {
    potrf_diag<<<1, 256, 0, s>>>(A, ld, n, k0, thr, cs);
    THC_LAUNCHED(c, "potrf_diag");
    int nb = std::min(NB, n - k0);
    int rest = n - k0 - nb;
    if (rest <= 0) break;
    potrf_panel<<<(int)cdiv(rest, 128), 128, 0, s>>>(A, ld, n, k0, cs);
    THC_LAUNCHED(c, "potrf_panel");
    GemmArgs g{};
    g.M = rest; g.N = rest; g.K = nb;
    g.A = A + (long long)(k0 + nb) * ld + k0; g.sam = ld; g.sak = 1;
    g.B = A + (long long)(k0 + nb) * ld + k0; g.sbn = ld; g.sbk = 1;
    g.C = A + (long long)(k0 + nb) * ld + k0 + nb; g.ldc = ld;
    g.alpha = -1.0; g.beta = 1.0; g.lower_only = 1; g.mode = GEMM_STORE;
    g.skip_flag = &cs->flag;
    int st = dgemm(c, g);
    if (st) return st;
  }
  return THC_OK;
}

// B := L^{-T} L^{-1} B (solve (L L^T) X = B), B is n x nrhs row-major.
int potrs(Ctx* c, const double* L, long long ld, int n, double* B, long long ldb,
          long long nrhs, const CholStatus* cs)
{
  cudaStream_t s = c->stream;
  int nthr = 128;
  int nblk = (int)cdiv(nrhs, nthr);
  for (int k0 = 0; k0 < n; k0 += NB) {
    trsm_diag_fwd<<<nblk, nthr, 0, s>>>(L, ld, n, k0, B, ldb, nrhs, cs);
    THC_LAUNCHED(c, "trsm_diag_fwd");
    int nb = std::min(NB, n - k0);
    int rest = n - k0 - nb;
    if (rest <= 0) break;
    GemmArgs g{};
    g.M = rest; g.N = nrhs; g.K = nb;
    g.A = L + (long long)(k0 + nb) * ld + k0; g.sam = ld; g.sak = 1;   // L rows below
    g.B = B + (long long)k0 * ldb; g.sbn = 1; g.sbk = ldb;              // B(k,n) = B[k*ldb+n]
    g.C = B + (long long)(k0 + nb) * ldb; g.ldc = ldb;
    g.alpha = -1.0; g.beta = 1.0; g.mode = GEMM_STORE;
    g.skip_flag = cs ? &cs->flag : nullptr;
    int st = dgemm(c, g);
    if (st) return st;
  }
  int nblocks = (int)cdiv(n, NB);
  for (int kb = nblocks - 1; kb >= 0; kb--) {
    int k0 = kb * NB;
    trsm_diag_bwd<<<nblk, nthr, 0, s>>>(L, ld, n, k0, B, ldb, nrhs, cs);
    THC_LAUNCHED(c, "trsm_diag_bwd");
    if (k0 == 0) break;
    int nb = std::min(NB, n - k0);
    GemmArgs g{};
    g.M = k0; g.N = nrhs; g.K = nb;
    g.A = L + (long long)k0 * ld; g.sam = 1; g.sak = ld;               // A(m,k) = L[k0+k][m]
    g.B = B + (long long)k0 * ldb; g.sbn = 1; g.sbk = ldb;
    g.C = B; g.ldc = ldb;
    g.alpha = -1.0; g.beta = 1.0; g.mode = GEMM_STORE;
    g.skip_flag = cs ? &cs->flag : nullptr;
    int st = dgemm(c, g);
    if (st) return st;
  }
  return THC_OK;
}

int set_identity(Ctx* c, double* A, long long ld, int n)
{
  set_identity_k<<<(int)cdiv((long long)n * n, 256), 256, 0, c->stream>>>(A, ld, n);
  THC_LAUNCHED(c, "set_identity");
  return THC_OK;
}

int add_diag_shift(Ctx* c, double* A, long long ld, int n, double rel, double* shift_out)
{
  add_diag<<<1, 1024, 0, c->stream>>>(A, ld, n, A, rel, shift_out);
  THC_LAUNCHED(c, "add_diag");
  return THC_OK;
}

int diag_mean(Ctx* c, const double* A, long long ld, int n, double* out)
{
  diag_mean_k<<<1, 1024, 0, c->stream>>>(A, ld, n, out);
  THC_LAUNCHED(c, "diag_mean");
  return THC_OK;
}

int zpotrf_small(Ctx* c, double* A, int n, const double* thr, CholStatus* cs)
{
  zpotrf_small_k<<<1, 1024, 0, c->stream>>>(A, n, thr, cs);
  THC_LAUNCHED(c, "zpotrf_small");
  return THC_OK;
}

}  // namespace thc
