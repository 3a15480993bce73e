// Periodised Gaussian s/p basis functions on the real-space grid, on the GPU.
//
// Restates, for the synthetic systems, what the reference's input generator evaluates with
// pyscf (tools/thcpy/thcpy/transform_basis.py:51-148: `gen_uniform_grids`, `eval_ao`):
// phi_f(r) = sum_T g_f(r - R_a - T) with g = exp(-alpha_f |d|^2) (s) or
// d_x,y,z exp(-alpha_f |d|^2) (p_x,y,z), over the lattice images T that come within rcut.
// The host passes the image centres R_a + T (already filtered, sorted by atom); each block
// takes an 8 x 8 x 8 cube of mesh points, keeps the centres within rcut of the cube (in
// centre order), and every thread accumulates its point's functions atom by atom.
// Distances are formed in FP32 relative to the cube's first point (so they keep ~1e-7
// relative accuracy) and the Gaussians use expf: values agree with an FP64 evaluation to
// ~1e-6 relative, which is what synthetic orbitals need, and the C5 grid (1.26e6 points,
// 864 functions) takes a fraction of a second instead of many minutes on the host.
#include <cuda_runtime.h>

#include "common.cuh"

namespace thc {
namespace {

constexpr int kCube = 8;                 // mesh points per block edge
constexpr int kGenThreads = kCube * kCube * kCube;
constexpr int kGenWarps = kGenThreads / 32;
constexpr int kMaxCand = 2048;           // image centres kept per block

__global__ void __launch_bounds__(kGenThreads) gauss_sp_kernel(
    const double* __restrict__ grid, int n0, int n1, int n2, const double* __restrict__ cen,
    const int* __restrict__ catom, int ncen, const double* __restrict__ alphas, int nfunc,
    float rcut, double* __restrict__ out, int* overflow)
{
  __shared__ float ccx[kMaxCand], ccy[kMaxCand], ccz[kMaxCand];
  __shared__ int cat[kMaxCand];
  __shared__ float wred[6][kGenWarps];
  __shared__ float box[6];
  __shared__ int wcnt[kGenWarps];
  __shared__ int ncand;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int tx = threadIdx.x % kCube, ty = (threadIdx.x / kCube) % kCube,
            tz = threadIdx.x / (kCube * kCube);
  const int i = blockIdx.z * kCube + tz, j = blockIdx.y * kCube + ty, k = blockIdx.x * kCube + tx;
  const bool valid = i < n0 && j < n1 && k < n2;
  const long long p = valid ? ((long long)i * n1 + j) * n2 + k : 0;
  // Origin: the cube's first point (always on the mesh).
  const long long p0 = ((long long)(blockIdx.z * kCube) * n1 + blockIdx.y * kCube) * n2 +
                       blockIdx.x * kCube;
  const double o[3] = {grid[3 * p0], grid[3 * p0 + 1], grid[3 * p0 + 2]};
  float g[3] = {0.f, 0.f, 0.f};
  if (valid)
    for (int d = 0; d < 3; d++) g[d] = (float)(grid[3 * p + d] - o[d]);
  // Cube bounds (relative to the origin).
  for (int d = 0; d < 3; d++) {
    float mn = valid ? g[d] : 3e38f, mx = valid ? g[d] : -3e38f;
    for (int off = 16; off; off >>= 1) {
      mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, off));
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    }
    if (lane == 0) { wred[d][wid] = mn; wred[3 + d][wid] = mx; }
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    const int d = threadIdx.x;
    float v = wred[d][0];
    for (int w = 1; w < kGenWarps; w++) v = d < 3 ? fminf(v, wred[d][w]) : fmaxf(v, wred[d][w]);
    box[d] = v;
  }
  if (threadIdx.x == 0) ncand = 0;
  __syncthreads();
  // Centres within rcut of the cube (a little slack for FP32 rounding), compacted in order.
  const float cut2 = (rcut + 1e-3f) * (rcut + 1e-3f);
  for (int c0 = 0; c0 < ncen; c0 += kGenThreads) {
    const int c = c0 + threadIdx.x;
    float rel[3] = {0.f, 0.f, 0.f};
    bool keep = false;
    if (c < ncen) {
      float l2 = 0.f;
      for (int d = 0; d < 3; d++) {
        rel[d] = (float)(cen[3 * c + d] - o[d]);
        const float v = fmaxf(0.f, fmaxf(box[d] - rel[d], rel[d] - box[3 + d]));
        l2 += v * v;
      }
      keep = l2 <= cut2;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) wcnt[wid] = __popc(bal);
    __syncthreads();
    int before = ncand;
    for (int w = 0; w < wid; w++) before += wcnt[w];
    const int slot = before + __popc(bal & ((1u << lane) - 1u));
    if (keep && slot < kMaxCand) {
      ccx[slot] = rel[0]; ccy[slot] = rel[1]; ccz[slot] = rel[2];
      cat[slot] = catom[c];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = ncand;
      for (int w = 0; w < kGenWarps; w++) t += wcnt[w];
      ncand = t;
    }
    __syncthreads();
  }
  const int nc = ncand;
  if (nc > kMaxCand) {
    if (threadIdx.x == 0) atomicExch(overflow, 1);
    return;
  }
  if (!valid) return;
  // Accumulate atom by atom (the centres of one atom are consecutive), one write per atom.
  const float r2cut = rcut * rcut;
  double* row = out + p * nfunc;
  int cur = -1;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  bool any = false;
  auto flush = [&]() {
    if (cur < 0 || !any) return;
    for (int t = 0; t < 4; t++) {
      const int f = 4 * cur + t;
      if (f < nfunc) row[f] = (double)acc[t];
    }
  };
  for (int q = 0; q < nc; q++) {
    const int a = cat[q];
    if (a != cur) {
      flush();
      cur = a;
      any = false;
      acc[0] = acc[1] = acc[2] = acc[3] = 0.f;
    }
    const float dx = g[0] - ccx[q], dy = g[1] - ccy[q], dz = g[2] - ccz[q];
    const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, dx * dx));
    if (!(r2 < r2cut)) continue;
    any = true;
    const float dd[3] = {dx, dy, dz};
#pragma unroll
    for (int t = 0; t < 4; t++) {
      const int f = 4 * a + t;
      if (f >= nfunc) break;
      float e = expf(-(float)alphas[f] * r2);
      if (t) e *= dd[t - 1];
      acc[t] += e;
    }
  }
  flush();
}

}  // namespace
}  // namespace thc

extern "C" int thc_synth_gaussian_basis(thc_ctx* h, const double* grid, const int* mesh,
                                        const double* centres, const int* centre_atom,
                                        int ncentres, const double* alphas, int nfunc,
                                        double rcut, double* out)
{
  if (!h || !grid || !mesh || !centres || !centre_atom || !alphas || !out || ncentres < 0 ||
      nfunc <= 0 || !(rcut > 0.0))
    return THC_ERR_ARG;
  thc::Ctx* c = &h->c;
  if (cudaSetDevice(c->device) != cudaSuccess) return THC_ERR_CUDA;
  const int n0 = mesh[0], n1 = mesh[1], n2 = mesh[2];
  if (n0 <= 0 || n1 <= 0 || n2 <= 0) return thc::set_error(c, THC_ERR_ARG, "mesh");
  const long long ng = (long long)n0 * n1 * n2;
  int st = 0;
  const double* dgrid = (const double*)thc::to_device(c, grid, sizeof(double) * 3 * ng,
                                                      thc::WS_KM_IO, &st);
  if (st) return st;
  const double* dcen = (const double*)thc::to_device(
      c, centres, sizeof(double) * 3 * (size_t)(ncentres > 0 ? ncentres : 1), thc::WS_IDX, &st);
  if (st) return st;
  const int* dcat = (const int*)thc::to_device(
      c, centre_atom, sizeof(int) * (size_t)(ncentres > 0 ? ncentres : 1), thc::WS_COUL, &st);
  if (st) return st;
  const double* dalpha = (const double*)thc::to_device(c, alphas, sizeof(double) * nfunc,
                                                       thc::WS_PHIMU, &st);
  if (st) return st;
  if (!thc::is_device_ptr(out)) return thc::set_error(c, THC_ERR_ARG, "out must be on the device");
  int* flag = (int*)thc::ws_get(c, thc::WS_SCRATCH, 4096);
  if (!flag) return thc::set_error(c, THC_ERR_NOMEM, "scratch");
  cudaStream_t s = c->stream;
  THC_CUDA(c, cudaMemsetAsync(flag, 0, sizeof(int), s));
  THC_CUDA(c, cudaMemsetAsync(out, 0, sizeof(double) * ng * nfunc, s));
  dim3 blocks((unsigned)thc::cdiv(n2, thc::kCube), (unsigned)thc::cdiv(n1, thc::kCube),
              (unsigned)thc::cdiv(n0, thc::kCube));
  thc::gauss_sp_kernel<<<blocks, thc::kGenThreads, 0, s>>>(dgrid, n0, n1, n2, dcen, dcat,
                                                           ncentres, dalpha, nfunc, (float)rcut,
                                                           out, flag);
  THC_LAUNCHED(c, "gauss_sp_basis");
  int hf = 0;
  THC_CUDA(c, cudaMemcpyAsync(&hf, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  THC_CUDA(c, cudaStreamSynchronize(s));
  if (hf) return thc::set_error(c, THC_ERR_SHAPE, "thc_synth_gaussian_basis: more than %d image "
                                "centres near one 8x8x8 cube", thc::kMaxCand);
  return THC_OK;
}
