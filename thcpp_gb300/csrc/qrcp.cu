// Interpolating points by QR with column pivoting (QRCP::QRCPSolver::kernel,
// src/qrcp.cpp:100-173).
//
// The reference forms Z^T explicitly -- one row per orbital pair, one column per grid point,
// [Z^T]_{(ik)a} = conj(phi_i(r_a)) phi_k(r_a) (setup_Z_matrix, :34-49) -- and runs pzgeqpf on
// it (MatrixOperations::qrcp, src/matrix_operations.h:757-790); the points are the first
// thc_cfac * N_o pivots, sorted (:149-160), and |R_kk| is printed for every step (:161-171).
//
// Here the same pivot sequence comes from a pivoted Cholesky factorisation of Z^T's Gram
// matrix G = Z Z^T, which never needs Z^T (N_o^2 x N_g) in memory: for real orbitals
//   G(a, b) = sum_{ik} phi_i(a) phi_k(a) phi_i(b) phi_k(b) = P(a, b)^2,  P = Phi Phi^T,
// and the squared residual norm of column a after projecting out the first k pivots is
//   d_k(a) = G(a, a) - sum_{j<k} L(a, j)^2,
// the quantity QRCP pivots on (its partial column norms).  Step k picks p = argmax d_k,
// forms L(:, k) = (G(:, p) - L(:, :k) L(p, :k)^T) / sqrt(d_k(p)) and updates d; |R_kk| =
// sqrt(d_k(p)).  Per step: N_g (N_o + k) FP64 FMAs, one pass over L(:, :k).
//
// The half-rotated matrix (setup_Z_half_matrix, :50-67) stores pair (i, k), i < N_occ,
// k < N_o, in row i * N_occ + k, so for N_o > N_occ rows overlap and the last write wins:
// the rows that survive are phi_occ,i phi_k for i < N_occ - 1, k < min(N_occ, N_o), and
// phi_occ,last phi_k for every k.  Its Gram matrix is
//   G(a, b) = P_occ'(a, b) P_min(a, b) + phi_occ,last(a) phi_occ,last(b) P(a, b)
// (P_occ' over the first N_occ - 1 occupied orbitals, P_min over the first min(N_occ, N_o)
// orbitals), which is what runs by default; the context option "qrcp_all_pairs" selects
// every pair instead, G = P_occ o P.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "isdf.cuh"

namespace thc {
namespace {

constexpr int kQrThreads = 256;

struct QrPiv {
  double v;
  int a;
  int pad;
};

struct QrGeom {
  const double* phi;     // N_o x N_g (transposed: a warp reads consecutive points)
  const double* occ;     // N_occ x N_g or null
  long long ng;
  int no, nocc, kmin;    // kmin: orbitals in the P_min factor; 0 = every pair
  int ppb;               // points per block (the grid is a multiple of the SM count)
  int cplx;              // complex orbitals: rows 2k / 2k + 1 of phi hold Re / Im phi_k
};

// dst[i * n + a] = src[a * m + i] for a < n, i < m.
__global__ void transpose_rows(const double* __restrict__ src, long long n, int m,
                               double* __restrict__ dst)
{
  __shared__ double t[32][33];
  const long long a0 = blockIdx.x * 32LL;
  const int i0 = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += 8) {
    const long long a = a0 + r;
    const int i = i0 + threadIdx.x;
    if (a < n && i < m) t[r][threadIdx.x] = src[a * m + i];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int i = i0 + r;
    const long long a = a0 + threadIdx.x;
    if (a < n && i < m) dst[(long long)i * n + a] = t[threadIdx.x][r];
  }
}

__device__ __forceinline__ bool piv_better(double v, int a, double w, int b)
{
  return v > w || (v == w && a < b);
}

// Block argmax (largest value, lowest index) of (v, a); the result is valid in thread 0.
__device__ QrPiv block_argmax(double v, int a)
{
  __shared__ QrPiv red[kQrThreads / 32];
  for (int o = 16; o; o >>= 1) {
    double w = __shfl_down_sync(0xffffffffu, v, o);
    int b = __shfl_down_sync(0xffffffffu, a, o);
    if (piv_better(w, b, v, a)) { v = w; a = b; }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = QrPiv{v, a, 0};
  __syncthreads();
  QrPiv r{-INFINITY, 0x7fffffff, 0};
  if (warp == 0) {
    if (lane < kQrThreads / 32) r = red[lane];
    for (int o = 16; o; o >>= 1) {
      double w = __shfl_down_sync(0xffffffffu, r.v, o);
      int b = __shfl_down_sync(0xffffffffu, r.a, o);
      if (piv_better(w, b, r.v, r.a)) { r.v = w; r.a = b; }
    }
  }
  return r;
}

// Publishes the block's candidate; the last block to finish reduces all of them into
// piv[k] / dpiv[k] and re-arms the ticket for the next launch.
__device__ void finish_argmax(QrPiv mine, QrPiv* blk, unsigned* ticket, int* piv,
                              double* dpiv, int k)
{
  __shared__ bool last;
  if (threadIdx.x == 0) {
    blk[blockIdx.x] = mine;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double v = -INFINITY;
  int a = 0x7fffffff;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
    double w = __ldcg(&blk[b].v);
    int i = __ldcg(&blk[b].a);
    if (piv_better(w, i, v, a)) { v = w; a = i; }
  }
  QrPiv r = block_argmax(v, a);
  if (threadIdx.x == 0) {
    piv[k] = r.a;
    dpiv[k] = r.v;
    *ticket = 0u;
  }
}

// G(a, p): the pivot's values are pp[k * ps] (N_o) and op[i * ps] (N_occ) -- shared memory
// (ps = 1) or the point's own column of the transposed orbitals (ps = N_g, for G(a, a)).
__device__ __forceinline__ double gram(const QrGeom& g, long long a, const double* pp,
                                       const double* op, long long ps)
{
  const double* ra = g.phi + a;
  if (g.cplx) {
    // Complex Z^T rows conj(phi_i) phi_k: G(a, b) = |P(a, b)|^2, P(a, b) = sum_k
    // conj(phi_k(a)) phi_k(b) (real and imaginary parts accumulated separately).
    double re = 0.0, im = 0.0;
    for (int k = 0; k < g.no; k++) {
      const double xr = ra[(2 * k) * g.ng], xi = ra[(2 * k + 1) * g.ng];
      const double yr = pp[(2 * k) * ps], yi = pp[(2 * k + 1) * ps];
      re = fma(xr, yr, fma(xi, yi, re));
      im = fma(xr, yi, fma(-xi, yr, im));
    }
    return fma(re, re, im * im);
  }
  double g3 = 0.0, gmin = 0.0;
  for (int k = 0; k < g.no; k++) {
    if (k == g.kmin) gmin = g3;
    g3 = fma(ra[k * g.ng], pp[k * ps], g3);
  }
  if (!g.occ) return g3 * g3;
  const double* oa = g.occ + a;
  double g1 = 0.0;
  for (int i = 0; i < g.nocc - 1; i++) g1 = fma(oa[i * g.ng], op[i * ps], g1);
  const double ol = oa[(long long)(g.nocc - 1) * g.ng] * op[(g.nocc - 1) * ps];
  if (g.kmin == 0) return (g1 + ol) * g3;           // every pair: P_occ o P
  if (g.kmin >= g.no) gmin = g3;
  return g1 * gmin + ol * g3;
}

// d(a) = G(a, a) and the first pivot.
__global__ void __launch_bounds__(kQrThreads)
qrcp_init_kernel(QrGeom g, double* d, QrPiv* blk, unsigned* ticket, int* piv, double* dpiv)
{
  const long long a = blockIdx.x * (long long)g.ppb + threadIdx.x;
  const bool own = threadIdx.x < g.ppb && a < g.ng;
  double v = -INFINITY;
  if (own) {
    v = gram(g, a, g.phi + a, g.occ ? g.occ + a : nullptr, g.ng);
    d[a] = v;
  }
  QrPiv r = block_argmax(v, own ? (int)a : 0x7fffffff);
  finish_argmax(r, blk, ticket, piv, dpiv, 0);
}

// Step k: column k of L, the residual update and the next pivot.  L is column-major
// (L[j * N_g + a]); a picked point has d = -inf and L(a, k) = 0 after its own step.
__global__ void __launch_bounds__(kQrThreads)
qrcp_step_kernel(QrGeom g, double* __restrict__ L, double* __restrict__ d, int k, int npts,
                 QrPiv* blk, unsigned* ticket, int* piv, double* dpiv)
{
  extern __shared__ double sh[];
  const int kw = g.cplx ? 2 * g.no : g.no;
  double* pp = sh;
  double* op = pp + kw;
  double* lp = op + g.nocc;
  const int p = piv[k];
  const double dp = dpiv[k];
  const long long ng = g.ng;
  if (p < 0 || p >= ng) {
    // No valid pivot (every candidate residual was NaN): pass the marker on without
    // touching memory; the host reports the step.
    if (k + 1 < npts && blockIdx.x == 0 && threadIdx.x == 0) {
      piv[k + 1] = p;
      dpiv[k + 1] = -INFINITY;
    }
    return;
  }
  for (int i = threadIdx.x; i < kw; i += kQrThreads) pp[i] = g.phi[(long long)i * ng + p];
  if (g.occ)
    for (int i = threadIdx.x; i < g.nocc; i += kQrThreads)
      op[i] = g.occ[(long long)i * ng + p];
  for (int j = threadIdx.x; j < k; j += kQrThreads) lp[j] = L[j * ng + p];
  __syncthreads();
  const long long a = blockIdx.x * (long long)g.ppb + threadIdx.x;
  const bool own = threadIdx.x < g.ppb && a < ng;
  double best = -INFINITY;
  if (own) {
    double dv = d[a];
    double l = 0.0;
    if (a == p) {
      l = sqrt(fmax(dp, 0.0));
      dv = -INFINITY;
    } else if (dv != -INFINITY && dp > 0.0) {
      const double gap = gram(g, a, pp, op, 1);
      double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
      const double* la = L + a;
      int j = 0;
      for (; j + 8 <= k; j += 8) {
        // Eight loads in flight before the four FMA chains consume them.
        double x[8];
#pragma unroll
        for (int u = 0; u < 8; u++) x[u] = la[(j + u) * ng];
        s0 = fma(x[0], lp[j + 0], s0);
        s1 = fma(x[1], lp[j + 1], s1);
        s2 = fma(x[2], lp[j + 2], s2);
        s3 = fma(x[3], lp[j + 3], s3);
        s0 = fma(x[4], lp[j + 4], s0);
        s1 = fma(x[5], lp[j + 5], s1);
        s2 = fma(x[6], lp[j + 6], s2);
        s3 = fma(x[7], lp[j + 7], s3);
      }
      for (; j + 4 <= k; j += 4) {
        s0 = fma(la[(j + 0) * ng], lp[j + 0], s0);
        s1 = fma(la[(j + 1) * ng], lp[j + 1], s1);
        s2 = fma(la[(j + 2) * ng], lp[j + 2], s2);
        s3 = fma(la[(j + 3) * ng], lp[j + 3], s3);
      }
      for (; j < k; j++) s0 = fma(la[j * ng], lp[j], s0);
      l = (gap - ((s0 + s1) + (s2 + s3))) / sqrt(dp);
      dv = fma(-l, l, dv);
    }
    L[(long long)k * ng + a] = l;
    d[a] = dv;
    best = dv;
  }
  if (k + 1 >= npts) return;
  QrPiv r = block_argmax(best, own ? (int)a : 0x7fffffff);
  finish_argmax(r, blk, ticket, piv, dpiv, k + 1);
}

}  // namespace

int qrcp_run(Ctx* c, const double* phi_in, long long ng, int no, const double* occ_in, int nocc,
             int npts, int* out_idx, int* out_order, double* out_diag, thc_qrcp_stats* stats,
             bool cplx)
{
  c->zeta_elem = 0;   // L shares the workspace slot of Z and zeta
  if (!phi_in || !out_idx || ng <= 0 || no <= 0 || npts <= 0 || npts > ng ||
      (occ_in && nocc <= 0) || (occ_in && cplx))
    return set_error(c, THC_ERR_ARG, "thc_qrcp: invalid arguments");
  const int kw = cplx ? 2 * no : no;   // doubles per point
  if (ng > 0x7ffffffeLL)
    return set_error(c, THC_ERR_SHAPE, "thc_qrcp: N_g %lld exceeds the 32-bit index range", ng);
  const size_t shmem = sizeof(double) * ((size_t)kw + (occ_in ? nocc : 0) + npts);
  if (shmem > 200 * 1024)
    return set_error(c, THC_ERR_SHAPE, "thc_qrcp: N_o + N_occ + points = %zu values exceed the "
                     "200 KB pivot buffer", shmem / sizeof(double));
  cudaStream_t s = c->stream;
  int st = 0;
  const double* phi = (const double*)to_device(c, phi_in, sizeof(double) * ng * kw, WS_PHI, &st);
  if (st) return st;
  const double* occ = nullptr;
  if (occ_in) {
    occ = (const double*)to_device(c, occ_in, sizeof(double) * ng * nocc, WS_PHIOCC, &st);
    if (st) return st;
  }
  const int nt = occ ? nocc : 0;
  // Balanced grid: a multiple of the SM count, each block a contiguous run of points.
  int sms = 0;
  THC_CUDA(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  sms = std::max(sms, 1);
  const long long nblk = cdiv(cdiv(ng, kQrThreads), sms) * sms;
  const int ppb = (int)cdiv(ng, nblk);
  // L (npts x N_g), the transposed orbitals ((N_o + N_occ) x N_g), d (N_g), block
  // candidates, pivots and their residuals, ticket.
  const size_t l_bytes = sizeof(double) * (size_t)npts * ng;
  const size_t t_bytes = sizeof(double) * (size_t)(kw + nt) * ng;
  const size_t bytes = l_bytes + t_bytes + sizeof(double) * ng + sizeof(QrPiv) * nblk +
                       (sizeof(int) + sizeof(double)) * npts + 1024;
  char* base = (char*)ws_get(c, WS_ZT, bytes);
  if (!base) return set_error(c, THC_ERR_NOMEM, "thc_qrcp: workspace allocation failed");
  double* L = (double*)base;
  double* phit = L + (size_t)npts * ng;
  double* occt = phit + (size_t)kw * ng;
  double* d = occt + (size_t)nt * ng;
  QrPiv* blk = (QrPiv*)(d + ng);
  double* dpiv = (double*)(blk + nblk);
  int* piv = (int*)(dpiv + npts);
  unsigned* ticket = (unsigned*)(((uintptr_t)(piv + npts) + 255) & ~(uintptr_t)255);
  QrGeom g;
  g.phi = phit;
  g.occ = occ ? occt : nullptr;
  g.ng = ng;
  g.no = no;
  g.nocc = nt;
  g.ppb = ppb;
  g.cplx = cplx ? 1 : 0;
  g.kmin = occ ? (c->qrcp_all_pairs ? 0 : std::min(nocc, no)) : no;
  THC_CUDA(c, cudaFuncSetAttribute(qrcp_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)shmem));
  THC_CUDA(c, cudaMemsetAsync(ticket, 0, sizeof(unsigned), s));
  THC_CUDA(c, cudaEventRecord(c->ev0, s));
  {
    ProfScope ps(c, "qrcp_init");
    const dim3 tb(32, 8);
    transpose_rows<<<dim3((unsigned)cdiv(ng, 32), (unsigned)cdiv(kw, 32)), tb, 0, s>>>(phi, ng, kw,
                                                                                     phit);
    if (occ)
      transpose_rows<<<dim3((unsigned)cdiv(ng, 32), (unsigned)cdiv(nt, 32)), tb, 0, s>>>(
          occ, ng, nt, occt);
    qrcp_init_kernel<<<(unsigned)nblk, kQrThreads, 0, s>>>(g, d, blk, ticket, piv, dpiv);
  }
  c->launches += occ ? 2 : 1;  // the transposes
  THC_LAUNCHED(c, "qrcp_init");
  {
    ProfScope ps(c, "qrcp_step");
    for (int k = 0; k < npts; k++) {
      qrcp_step_kernel<<<(unsigned)nblk, kQrThreads, shmem, s>>>(g, L, d, k, npts, blk, ticket,
                                                                 piv, dpiv);
    }
  }
  c->launches += npts - 1;
  THC_LAUNCHED(c, "qrcp_step");
  THC_CUDA(c, cudaEventRecord(c->ev1, s));
  std::vector<int> order(npts);
  std::vector<double> dv(npts);
  THC_CUDA(c, cudaMemcpyAsync(order.data(), piv, sizeof(int) * npts, cudaMemcpyDeviceToHost, s));
  THC_CUDA(c, cudaMemcpyAsync(dv.data(), dpiv, sizeof(double) * npts, cudaMemcpyDeviceToHost, s));
  THC_CUDA(c, cudaStreamSynchronize(s));
  int rank = npts;
  for (int k = 0; k < npts; k++) {
    if (order[k] < 0 || order[k] >= ng)
      return set_error(c, THC_ERR_ARG, "thc_qrcp: no finite residual at step %d (NaN or "
                       "infinite orbital values?)", k);
    dv[k] = std::sqrt(std::max(dv[k], 0.0));
    if (rank == npts && !(dv[k] > 1e-7 * dv[0])) rank = k;
  }
  std::vector<int> idx(order);
  std::sort(idx.begin(), idx.end());
  // Outputs may live on the host or on the device.  Device outputs are written on the
  // context's stream (work the caller queues there afterwards sees them), and the stream
  // is drained before the pageable host vectors go out of scope.
  bool any_dev = false;
  auto put = [&](void* dst, const void* src, size_t bytes) -> int {
    if (!dst) return 0;
    if (is_device_ptr(dst)) {
      THC_CUDA(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
      any_dev = true;
    } else {
      std::memcpy(dst, src, bytes);
    }
    return 0;
  };
  st = put(out_order, order.data(), sizeof(int) * npts);
  if (!st) st = put(out_diag, dv.data(), sizeof(double) * npts);
  if (!st) st = put(out_idx, idx.data(), sizeof(int) * npts);
  if (any_dev) {
    // Also after a failed copy: an earlier one may still read the host vectors.
    const cudaError_t e = cudaStreamSynchronize(s);
    if (!st && e != cudaSuccess)
      st = set_error(c, THC_ERR_CUDA, "thc_qrcp: output copy: %s", cudaGetErrorString(e));
  }
  if (st) return st;
  if (stats) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    stats->numerical_rank = rank;
    stats->device_ms = ms;
  }
  return THC_OK;
}

}  // namespace thc
