// Half-rotated ISDF with complex orbitals (IVecs with rotate = true on complex aoR and
// aoR_half), FP64 throughout:
//   P      = Phi_mu^H Phi,  P_occ = Phi_occ,mu^H Phi_occ       setup_pseudo_dm, pzgemm 'C','N'
//                                                            (src/interpolating_vectors.cpp:117)
//   Z      = P_occ o conj(P)                                  setup_CZt_half (:143-161)
//   C      = Z[:, idx]   (complex, not Hermitian)             setup_CCt (:163-190)
//   X      = C^{-1} Z                                         least_squares, pzgels (:416)
//   zeta   = conj(X) (rows: zeta_mu(r))                       fft_vectors' Hermitian transpose
//   IVG    = forward, IVMG = backward unnormalised 3-D FFT    fft_vectors (:384-391)
//   M      = sum_G IVMG_mu(G) v(G) IVG_nu(G)                  construct_muv 'T','N' (:261-273)
// M is HalfTransformedMuv, written without a Cholesky factor (dump_thc_data, :317-328).
//
// C has full rank for a sensible point set but no symmetry, so the reference's QR solve is
// replaced by the inverse from Gauss-Jordan elimination with partial pivoting (one pivot
// kernel and one elimination kernel per column, on [C | I]; N_mu^3 complex FMAs, small next
// to the N_mu^2 N_g of the products), then X = C^{-1} Z as four real FP64 GEMMs.  Complex
// values are (re, im) pairs; P and Z are kept as separate real and imaginary N_mu x N_g
// matrices so that every product is a real GEMM of dense64.cu.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "dense64.cuh"
#include "isdf.cuh"

namespace thc {
namespace {

// Rows of the pair-stored orbitals at the interpolating points: out[mu][*] = phi[idx[mu]][*]
// (kw doubles per row); rot (optional) = the rotated pairs (-im, re), for Im(a^H b) as a
// real dot product; orb (optional) = the (N_o, N_mu, 2) orbital output.
__global__ void gather_pairs(const double* __restrict__ phi, long long ng, int no,
                             const int* __restrict__ idx, int nmu, double* out, double* rot,
                             double* orb, int* bad)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)nmu * no) return;
  const int mu = (int)(e / no), i = (int)(e % no);
  const long long g = idx[mu];
  if (g < 0 || g >= ng) {
    atomicExch(bad, 1);
    return;
  }
  const double re = phi[(g * no + i) * 2], im = phi[(g * no + i) * 2 + 1];
  out[e * 2] = re;
  out[e * 2 + 1] = im;
  rot[e * 2] = -im;
  rot[e * 2 + 1] = re;
  if (orb) {
    orb[2 * ((long long)i * nmu + mu)] = re;
    orb[2 * ((long long)i * nmu + mu) + 1] = im;
  }
}

// Z = Q o conj(P) in place of (PR, PI):  ZR = QR PR + QI PI,  ZI = QI PR - QR PI.
__global__ void half_product(double* pr, double* pi, const double* __restrict__ qr,
                             const double* __restrict__ qi, long long n)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= n) return;
  const double a = pr[e], b = pi[e], c = qr[e], d = qi[e];
  pr[e] = __fma_rn(c, a, d * b);
  pi[e] = __fma_rn(d, a, -c * b);
}

// [C | I] (n x 2n complex, row-major) with C[mu][nu] = Z[mu][idx[nu]].
__global__ void build_augmented(const double* __restrict__ zr, const double* __restrict__ zi,
                                long long ng, const int* __restrict__ idx, int n, double* a)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * 2 * n) return;
  const int r = (int)(e / (2 * n)), c = (int)(e % (2 * n));
  double re = 0.0, im = 0.0;
  if (c < n) {
    const long long g = idx[c];
    re = zr[(long long)r * ng + g];
    im = zi[(long long)r * ng + g];
  } else {
    re = (c - n == r) ? 1.0 : 0.0;
  }
  a[2 * e] = re;
  a[2 * e + 1] = im;
}

struct GjStatus {
  int singular;        // 1-based column without a non-zero pivot
  int pad;
  double min_abs2;     // smallest / largest |pivot|^2
  double max_abs2;
};

// Step k, part 1 (one block): pivot p = argmax_{r >= k} |A[r][k]|^2 (lowest row on ties),
// swap rows k and p, scale row k by 1 / A[k][k], and save column k (after the swap) in f.
__global__ void __launch_bounds__(1024) gj_pivot(double* a, int n, int k, double* f,
                                                 GjStatus* gs)
{
  __shared__ double bv[32];
  __shared__ int bi[32];
  __shared__ double piv[2];
  const long long w = 2LL * n;                        // complex row length
  if (gs->singular) return;
  double best = -1.0;
  int arg = n;
  for (int r = k + threadIdx.x; r < n; r += blockDim.x) {
    const double re = a[2 * (r * w + k)], im = a[2 * (r * w + k) + 1];
    const double v = re * re + im * im;
    if (v > best) { best = v; arg = r; }
  }
  for (int off = 16; off; off >>= 1) {
    const double v2 = __shfl_xor_sync(0xffffffffu, best, off);
    const int i2 = __shfl_xor_sync(0xffffffffu, arg, off);
    if (v2 > best || (v2 == best && i2 < arg)) { best = v2; arg = i2; }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { bv[warp] = best; bi[warp] = arg; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < (int)(blockDim.x >> 5); q++)
      if (bv[q] > bv[0] || (bv[q] == bv[0] && bi[q] < bi[0])) { bv[0] = bv[q]; bi[0] = bi[q]; }
    if (!(bv[0] > 0.0) || bi[0] >= n) {
      gs->singular = k + 1;
    } else {
      gs->min_abs2 = k ? fmin(gs->min_abs2, bv[0]) : bv[0];
      gs->max_abs2 = k ? fmax(gs->max_abs2, bv[0]) : bv[0];
    }
  }
  __syncthreads();
  if (gs->singular) return;
  const int p = bi[0];
  if (p != k)
    for (long long c = threadIdx.x; c < 2 * w; c += blockDim.x) {
      const double t = a[2 * k * w + c];
      a[2 * k * w + c] = a[2 * p * w + c];
      a[2 * p * w + c] = t;
    }
  __syncthreads();
  if (threadIdx.x == 0) {
    // 1 / (x + i y) = (x - i y) / (x^2 + y^2)
    const double x = a[2 * (k * w + k)], y = a[2 * (k * w + k) + 1];
    const double d = x * x + y * y;
    piv[0] = x / d;
    piv[1] = -y / d;
  }
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    f[2 * r] = a[2 * (r * w + k)];
    f[2 * r + 1] = a[2 * (r * w + k) + 1];
  }
  __syncthreads();
  const double ir = piv[0], ii = piv[1];
  // Row k: every column from k on (the left part below k is already zero; the right part,
  // permuted by the row swaps, is dense in general).
  for (long long c = k + threadIdx.x; c < w; c += blockDim.x) {
    const double x = a[2 * (k * w + c)], y = a[2 * (k * w + c) + 1];
    a[2 * (k * w + c)] = x * ir - y * ii;
    a[2 * (k * w + c) + 1] = x * ii + y * ir;
  }
}

// Step k, part 2: A[r][c] -= f[r] A[k][c] for every row r != k and column c >= k (the
// left part before k is zero), and column k becomes e_k.
__global__ void gj_eliminate(double* a, int n, int k, const double* __restrict__ f,
                             const GjStatus* gs)
{
  if (gs->singular) return;
  const long long w = 2LL * n;
  const long long ncols = w - k;
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * ncols) return;
  const int r = (int)(e / ncols);
  const long long c = k + e % ncols;
  if (r == k) return;
  if (c == k) {
    a[2 * (r * w + k)] = 0.0;
    a[2 * (r * w + k) + 1] = 0.0;
    return;
  }
  const double fr = f[2 * r], fi = f[2 * r + 1];
  const double xr = a[2 * (k * w + c)], xi = a[2 * (k * w + c) + 1];
  a[2 * (r * w + c)] = __fma_rn(-fr, xr, __fma_rn(fi, xi, a[2 * (r * w + c)]));
  a[2 * (r * w + c) + 1] = __fma_rn(-fr, xi, __fma_rn(-fi, xr, a[2 * (r * w + c) + 1]));
}

// zeta (interleaved complex, row mu = zeta_mu on the grid) = conj(XR + i XI).
__global__ void conj_interleave(const double* __restrict__ xr, const double* __restrict__ xi,
                                long long n, double* z)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= n) return;
  z[2 * e] = xr[e];
  z[2 * e + 1] = -xi[e];
}

__global__ void interleave(const double* __restrict__ re, const double* __restrict__ im,
                           long long n, double* out)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= n) return;
  out[2 * e] = re[e];
  out[2 * e + 1] = im[e];
}

}  // namespace

int isdf_half_complex_run(Ctx* c, const double* phi_in, long long ng, int no,
                          const double* occ_in, int nocc, const int* idx_in, int nmu,
                          const int* mesh_in, const double* coul_in, double* out_orb,
                          double* out_orb_occ, double* out_M, thc_isdf_stats* stats)
{
  c->zeta_elem = 0;
  if (!phi_in || !occ_in || !idx_in || !mesh_in || !coul_in || ng <= 0 || no <= 0 || nocc <= 0 ||
      nmu <= 0 || nmu > ng)
    return set_error(c, THC_ERR_ARG, "thc_isdf_half_complex: invalid arguments");
  int mesh[3];
  if (is_device_ptr(mesh_in)) {
    THC_CUDA(c, cudaMemcpy(mesh, mesh_in, sizeof(mesh), cudaMemcpyDeviceToHost));
  } else {
    std::copy(mesh_in, mesh_in + 3, mesh);
  }
  if (mesh[0] <= 0 || mesh[1] <= 0 || mesh[2] <= 0 ||
      (long long)mesh[0] * mesh[1] * mesh[2] != ng)
    return set_error(c, THC_ERR_SHAPE, "thc_isdf_half_complex: FFT mesh does not match N_g");
  cudaStream_t s = c->stream;
  int st = 0;
  const double* phi = (const double*)to_device(c, phi_in, sizeof(double) * 2 * ng * no, WS_PHI, &st);
  if (st) return st;
  const double* occ = (const double*)to_device(c, occ_in, sizeof(double) * 2 * ng * nocc,
                                               WS_PHIOCC, &st);
  if (st) return st;
  const int* idx = (const int*)to_device(c, idx_in, sizeof(int) * nmu, WS_IDX, &st);
  if (st) return st;
  const double* coul = (const double*)to_device(c, coul_in, sizeof(double) * ng, WS_COUL, &st);
  if (st) return st;
  const long long nmg = (long long)nmu * ng;
  const long long nn = (long long)nmu * nmu;
  // Gathered rows: Phi_mu, its rotation, Phi_occ,mu, its rotation.
  double* rows = (double*)ws_get(c, WS_PHIMU, sizeof(double) * 4 * nmu * (no + nocc));
  double* prpi = (double*)ws_get(c, WS_ZT, sizeof(double) * 2 * nmg);     // P, then Z, then zeta
  double* qrqi = (double*)ws_get(c, WS_ZETA, sizeof(double) * 2 * nmg);   // P_occ, then X
  double* spec = (double*)ws_get(c, WS_ZHAT, sizeof(double) * 4 * nmg);   // IVG, IVMG
  double* aug = (double*)ws_get(c, WS_C, sizeof(double) * 4 * nn);        // [C | I]
  double* fcol = (double*)ws_get(c, WS_CINV, sizeof(double) * 2 * nmu + 64);
  double* Mw = (double*)ws_get(c, WS_M, sizeof(double) * 4 * nn);
  char* scr = (char*)ws_get(c, WS_SCRATCH, 4096);
  const bool orb_host = out_orb && !is_device_ptr(out_orb);
  const bool occ_host = out_orb_occ && !is_device_ptr(out_orb_occ);
  double* stage = nullptr;
  if (orb_host || occ_host)
    stage = (double*)ws_get(c, WS_ORB, sizeof(double) * 2 * nmu * (no + nocc));
  if (!rows || !prpi || !qrqi || !spec || !aug || !fcol || !Mw || !scr ||
      ((orb_host || occ_host) && !stage))
    return set_error(c, THC_ERR_NOMEM, "thc_isdf_half_complex: workspace allocation failed");
  double* pmu = rows;
  double* pmu_rot = pmu + 2LL * nmu * no;
  double* omu = pmu_rot + 2LL * nmu * no;
  double* omu_rot = omu + 2LL * nmu * nocc;
  double *pr = prpi, *pi = prpi + nmg, *qr = qrqi, *qi = qrqi + nmg;
  GjStatus* gs = (GjStatus*)scr;
  int* bad = (int*)(scr + 512);
  double* orb_dev = out_orb ? (orb_host ? stage : out_orb) : nullptr;
  double* occ_dev = out_orb_occ ? (occ_host ? stage + 2LL * nmu * no : out_orb_occ) : nullptr;
  THC_CUDA(c, cudaMemsetAsync(scr, 0, 1024, s));
  THC_CUDA(c, cudaEventRecord(c->ev0, s));
  gather_pairs<<<(int)cdiv((long long)nmu * no, 256), 256, 0, s>>>(phi, ng, no, idx, nmu, pmu,
                                                                  pmu_rot, orb_dev, bad);
  THC_LAUNCHED(c, "gather_pairs");
  gather_pairs<<<(int)cdiv((long long)nmu * nocc, 256), 256, 0, s>>>(occ, ng, nocc, idx, nmu, omu,
                                                                    omu_rot, occ_dev, bad);
  THC_LAUNCHED(c, "gather_pairs");
  if (orb_host)
    THC_CUDA(c, cudaMemcpyAsync(out_orb, orb_dev, sizeof(double) * 2 * nmu * no,
                                cudaMemcpyDeviceToHost, s));
  if (occ_host)
    THC_CUDA(c, cudaMemcpyAsync(out_orb_occ, occ_dev, sizeof(double) * 2 * nmu * nocc,
                                cudaMemcpyDeviceToHost, s));
  // Re(a^H b) and Im(a^H b) as real dot products over the (re, im) pairs: a . b and
  // rot(a) . b with rot(a) = (-im, re).
  auto pseudo_dm = [&](const double* amu, const double* arot, const double* full, int k,
                       double* re, double* im) -> int {
    GemmArgs g;
    g.M = nmu; g.N = ng; g.K = 2 * k;
    g.A = amu; g.sam = 2 * k; g.sak = 1;
    g.B = full; g.sbn = 2 * k; g.sbk = 1;
    g.C = re; g.ldc = ng;
    int r = dgemm(c, g);
    if (r) return r;
    g.A = arot;
    g.C = im;
    return dgemm(c, g);
  };
  if ((st = pseudo_dm(pmu, pmu_rot, phi, no, pr, pi))) return st;
  if ((st = pseudo_dm(omu, omu_rot, occ, nocc, qr, qi))) return st;
  half_product<<<(int)cdiv(nmg, 256), 256, 0, s>>>(pr, pi, qr, qi, nmg);
  THC_LAUNCHED(c, "half_product");
  // C^{-1} by Gauss-Jordan elimination on [C | I].
  build_augmented<<<(int)cdiv(2 * nn, 256), 256, 0, s>>>(pr, pi, ng, idx, nmu, aug);
  THC_LAUNCHED(c, "build_augmented");
  for (int k = 0; k < nmu; k++) {
    gj_pivot<<<1, 1024, 0, s>>>(aug, nmu, k, fcol, gs);
    const long long items = (long long)nmu * (2LL * nmu - k);
    gj_eliminate<<<(unsigned)cdiv(items, 256), 256, 0, s>>>(aug, nmu, k, fcol, gs);
  }
  c->launches += 2LL * nmu;
  THC_LAUNCHED(c, "gj_eliminate");
  // X = C^{-1} Z:  XR = CiR ZR - CiI ZI,  XI = CiR ZI + CiI ZR  (into the P_occ buffers).
  {
    const double* cir = aug + 2LL * nmu;             // right half, real parts (stride 2)
    const double* cii = cir + 1;
    auto prod = [&](const double* a, const double* b, double* out, double alpha,
                    double beta) -> int {
      GemmArgs g;
      g.M = nmu; g.N = ng; g.K = nmu;
      g.A = a; g.sam = 4LL * nmu; g.sak = 2;
      g.B = b; g.sbn = 1; g.sbk = ng;
      g.C = out; g.ldc = ng; g.alpha = alpha; g.beta = beta;
      return dgemm(c, g);
    };
    if ((st = prod(cir, pr, qr, 1.0, 0.0))) return st;
    if ((st = prod(cii, pi, qr, -1.0, 1.0))) return st;
    if ((st = prod(cir, pi, qi, 1.0, 0.0))) return st;
    if ((st = prod(cii, pr, qi, 1.0, 1.0))) return st;
  }
  // zeta = conj(X), interleaved for cuFFT (in the P buffers), then both transforms.
  double* zc = prpi;
  conj_interleave<<<(int)cdiv(nmg, 256), 256, 0, s>>>(qr, qi, nmg, zc);
  THC_LAUNCHED(c, "conj_interleave");
  double* ivg = spec;
  double* ivmg = spec + 2 * nmg;
  {
    ProfScope prof(c, "fft");
    for (int f0 = 0; f0 < nmu; f0 += kFftChunk) {
      const int nb = std::min(kFftChunk, nmu - f0);
      cufftHandle plan;
      if ((st = get_plan(c, mesh[0], mesh[1], mesh[2], nb, CUFFT_Z2Z, &plan))) return st;
      cufftDoubleComplex* src = (cufftDoubleComplex*)(zc + 2LL * ng * f0);
      if (cufftExecZ2Z(plan, src, (cufftDoubleComplex*)(ivg + 2LL * ng * f0), CUFFT_FORWARD) !=
              CUFFT_SUCCESS ||
          cufftExecZ2Z(plan, src, (cufftDoubleComplex*)(ivmg + 2LL * ng * f0), CUFFT_INVERSE) !=
              CUFFT_SUCCESS)
        return set_error(c, THC_ERR_CUFFT, "thc_isdf_half_complex: cufftExecZ2Z failed");
      c->launches += 2;
    }
  }
  c->zeta_last = nullptr;            // complex vectors: not served by the real accessor
  // M = sum_G v(G) IVMG_mu(G) IVG_nu(G):  MR = sum v (ar br - ai bi), MI = sum v (ar bi + ai br).
  double* mr = Mw;
  double* mi = Mw + nn;
  {
    auto prod = [&](const double* a, const double* b, double* out, double alpha,
                    double beta) -> int {
      GemmArgs g;
      g.M = nmu; g.N = nmu; g.K = (int)ng;
      g.A = a; g.sam = 2 * ng; g.sak = 2;
      g.B = b; g.sbn = 2 * ng; g.sbk = 2;
      g.dk = coul; g.dk_shift = 0;
      g.C = out; g.ldc = nmu; g.alpha = alpha; g.beta = beta;
      return dgemm(c, g);
    };
    if (ng > 0x7fffffffLL) return set_error(c, THC_ERR_SHAPE, "thc_isdf_half_complex: mesh too large");
    if ((st = prod(ivmg, ivg, mr, 1.0, 0.0))) return st;
    if ((st = prod(ivmg + 1, ivg + 1, mr, -1.0, 1.0))) return st;
    if ((st = prod(ivmg, ivg + 1, mi, 1.0, 0.0))) return st;
    if ((st = prod(ivmg + 1, ivg, mi, 1.0, 1.0))) return st;
  }
  double* mcx = Mw + 2 * nn;
  interleave<<<(int)cdiv(nn, 256), 256, 0, s>>>(mr, mi, nn, mcx);
  THC_LAUNCHED(c, "interleave");
  THC_CUDA(c, cudaEventRecord(c->ev1, s));
  if (out_M) THC_CUDA(c, cudaMemcpyAsync(out_M, mcx, sizeof(double) * 2 * nn, cudaMemcpyDefault, s));
  GjStatus hg{};
  int hbad = 0;
  THC_CUDA(c, cudaMemcpyAsync(&hg, gs, sizeof(GjStatus), cudaMemcpyDeviceToHost, s));
  THC_CUDA(c, cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  THC_CUDA(c, cudaStreamSynchronize(s));
  if (hbad) return set_error(c, THC_ERR_ARG, "thc_isdf_half_complex: interpolating index out of range");
  if (stats) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    stats->c_min_pivot = hg.max_abs2 > 0 ? hg.min_abs2 / hg.max_abs2 : 0.0;
    stats->chol_c_info = hg.singular;
    stats->device_ms = ms;
  }
  if (hg.singular)
    return set_error(c, THC_ERR_NOT_PD, "thc_isdf_half_complex: C is singular at column %d",
                     hg.singular);
  return THC_OK;
}

}  // namespace thc
