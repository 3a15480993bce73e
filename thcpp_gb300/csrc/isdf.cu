// ISDF interpolating vectors and the FFT Coulomb matrix on one GPU.
//
// Reference path (src/interpolating_vectors.cpp), single rank, real orbitals:
//   setup_pseudo_dm (:59-125)   Phi_mu = Phi[idx]; P = Phi_mu^H Phi (pzgemm 'C','N')
//   setup_CZt (:127-141)        Z = P o conj(P)                      (N_mu x N_g)
//   setup_CCt (:163-190)        C = Z[:, idx]                        (N_mu x N_mu)
//   kernel -> least_squares     zeta^T = C^{-1} Z  (pzgels, Householder QR)
//   fft_vectors (:331-404)      zeta_hat_mu = forward 3-D DFT of zeta_mu (FFTW C2C)
//   construct_muv (:247-281)    M = zeta_hat^H diag(v) zeta_hat  (pzherk 'L','C')
//   dump_thc_data (:283-329)    L = chol(M) (pzpotrf 'L'), upper zeroed, C order
//
// GPU formulation (all buffers resident in HBM, row-major):
//   Phi (N_g x N_o) -> Phi_mu (N_mu x N_o) gather
//   C  = (Phi_mu Phi_mu^T)^2              FP64 GEMM, square epilogue
//   Z^T = (Phi_mu Phi^T)^2                 FP64 GEMM, square epilogue (N_mu x N_g)
//   L_C = chol(C + shift I); C^{-1} by forward/backward substitution on I
//   zeta^T = C^{-1} Z^T                     (N_mu x N_g; each row is one 3-D field)
//   zeta_hat = batched R2C (cuFFT D2Z)      (N_mu x N_c complex, N_c = n0 n1 (n2/2+1))
//   M = sum_half w [v_sym Re(a) + i v_anti Im(a)],  a = conj(zh_mu) zh_nu,
//       which equals the reference's full C2C sum for any v(G) (v_sym / v_anti are the
//       even / odd parts of v under G -> -G; v_anti != 0 only where the fftfreq mesh
//       of a non-orthogonal cell breaks the G <-> -G symmetry at Nyquist indices).
//   L = chol(M)   real when v_anti == 0, complex Hermitian otherwise.
// Cholesky replaces the reference's QR: for full-rank C both give C^{-1} Z to
// ~cond(C) * 1e-16; a rank-deficient C (N_mu larger than the number of independent
// orbital-pair products) is detected by a pivot threshold and regularised with a
// diagonal shift of 1e-10 tr(C)/N_mu.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "dense64.cuh"
#include "isdf.cuh"

namespace thc {

namespace {

__global__ void gather_rows(const double* __restrict__ phi, long long ng, int no,
                            const int* __restrict__ idx, int nmu, double* phimu,
                            double* orbitals, int* bad)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)nmu * no) return;
  int mu = (int)(e / no), i = (int)(e % no);
  long long g = idx[mu];
  if (g < 0 || g >= ng) {
    atomicExch(bad, 1);
    return;
  }
  double v = phi[g * no + i];
  phimu[e] = v;
  if (orbitals) {
    // /Hamiltonian/THC/Orbitals: (N_o, N_mu, 2), C order.
    orbitals[2 * ((long long)i * nmu + mu)] = v;
    orbitals[2 * ((long long)i * nmu + mu) + 1] = 0.0;
  }
}

// Half-spectrum Coulomb weights: dsym = w (v(G) + v(-G))/2, danti = w (v(G) - v(-G))/2.
__global__ void coulomb_weights(const double* __restrict__ v, int n0, int n1, int n2,
                                double* dsym, double* danti, int* n_anti)
{
  int nc = n2 / 2 + 1;
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  long long tot = (long long)n0 * n1 * nc;
  if (e >= tot) return;
  int k2 = (int)(e % nc);
  long long r = e / nc;
  int k1 = (int)(r % n1), k0 = (int)(r / n1);
  int j0 = (n0 - k0) % n0, j1 = (n1 - k1) % n1, j2 = (n2 - k2) % n2;
  double vp = v[((long long)k0 * n1 + k1) * n2 + k2];
  double vn = v[((long long)j0 * n1 + j1) * n2 + j2];
  double w = (k2 == 0 || (n2 % 2 == 0 && k2 == n2 / 2)) ? 1.0 : 2.0;
  dsym[e] = w * 0.5 * (vp + vn);
  double a = w * 0.5 * (vp - vn);
  danti[e] = a;
  if (a != 0.0) atomicAdd(n_anti, 1);
}

// M (complex interleaved, full Hermitian) from the lower triangle of Re M and the
// antisymmetric imaginary part X - X^T (X may be null).
__global__ void assemble_m(const double* __restrict__ mre, const double* __restrict__ x,
                           int n, double* M)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * n) return;
  int r = (int)(e / n), c = (int)(e % n);
  double re = r >= c ? mre[(long long)r * n + c] : mre[(long long)c * n + r];
  double im = x ? x[(long long)r * n + c] - x[(long long)c * n + r] : 0.0;
  M[2 * e] = re;
  M[2 * e + 1] = im;
}

// Real lower-triangular L -> complex interleaved Luv with the upper triangle zeroed.
__global__ void export_l_real(const double* __restrict__ L, int n, double* out)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * n) return;
  int r = (int)(e / n), c = (int)(e % n);
  out[2 * e] = c <= r ? L[e] : 0.0;
  out[2 * e + 1] = 0.0;
}

__global__ void zero_upper_complex(double* A, int n)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * n) return;
  int r = (int)(e / n), c = (int)(e % n);
  if (c > r) { A[2 * e] = 0.0; A[2 * e + 1] = 0.0; }
}

__global__ void copy_lower_to_full(const double* __restrict__ src, int n, double* dst)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * n) return;
  int r = (int)(e / n), c = (int)(e % n);
  dst[e] = r >= c ? src[e] : src[(long long)c * n + r];
}

__global__ void set_scalar(double* p, double v) { *p = v; }

__global__ void scale_scalar(const double* src, double f, double* dst) { *dst = f * *src; }

// Complex orbitals stored as (re, im) pairs, K = 2 N_o real columns per point:
// out[a, 2i] = Im phi_i(a), out[a, 2i + 1] = -Re phi_i(a), so that a real product of
// the pair layout with this one is Im P = Im(Phi_mu^H Phi).
__global__ void rotate_pairs(const double* __restrict__ in, long long n, double* __restrict__ out)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= n) return;
  const double re = in[2 * e], im = in[2 * e + 1];
  out[2 * e] = im;
  out[2 * e + 1] = -re;
}

// a = a + b * b elementwise (|P|^2 = (Re P)^2 + (Im P)^2, with a = (Re P)^2 on entry).
__global__ void add_square_k(double* a, long long lda, const double* __restrict__ b,
                             long long ldb, long long rows, long long cols)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= rows * cols) return;
  long long r = e / cols, c = e % cols;
  const double v = b[r * ldb + c];
  a[r * lda + c] = __dadd_rn(a[r * lda + c], __dmul_rn(v, v));
}

// /Hamiltonian/THC/Orbitals (N_o, N_mu, 2) from the gathered complex rows (N_mu x 2 N_o).
__global__ void complex_orbitals_out(const double* __restrict__ phimu, int nmu, int no,
                                     double* __restrict__ orbitals)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)nmu * no) return;
  const int mu = (int)(e / no), i = (int)(e % no);
  orbitals[2 * ((long long)i * nmu + mu)] = phimu[2 * e];
  orbitals[2 * ((long long)i * nmu + mu) + 1] = phimu[2 * e + 1];
}

// a[r * lda + c] *= b[r * ldb + c] (the Hadamard products of the half-rotated path).
__global__ void hadamard_k(double* a, long long lda, const double* __restrict__ b,
                           long long ldb, long long rows, long long cols)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= rows * cols) return;
  long long r = e / cols, c = e % cols;
  a[r * lda + c] = __dmul_rn(a[r * lda + c], b[r * ldb + c]);
}

__global__ void init_chol_status(CholStatus* cs)
{
  cs->flag = 0;
  cs->info = 0;
  cs->min_piv = 1.0 / 0.0;
  cs->max_piv = 0.0;
}

}  // namespace

int get_plan(Ctx* c, int n0, int n1, int n2, int batch, cufftType type, cufftHandle* out)
{
  // Plans are cached per context; their work area is the context's own stream-ordered
  // FFT slot (cuFFT's automatic allocation would cudaMalloc, which synchronises the GPU).
  auto key = std::make_tuple(n0, n1, n2, batch, (int)type);
  auto it = c->plans.find(key);
  cufftHandle p;
  if (it != c->plans.end()) {
    p = it->second;
  } else {
    if (cufftCreate(&p) != CUFFT_SUCCESS) return set_error(c, THC_ERR_CUFFT, "cufftCreate failed");
    cufftSetAutoAllocation(p, 0);
    long long n[3] = {n0, n1, n2};
    long long ng = (long long)n0 * n1 * n2;
    long long nc = (long long)n0 * n1 * (n2 / 2 + 1);
    size_t work = 0;
    // Real-to-complex outputs are half spectra; complex-to-complex ones full grids.
    const long long odist = type == CUFFT_Z2Z ? ng : nc;
    cufftResult r = cufftMakePlanMany64(p, 3, n, nullptr, 1, ng, nullptr, 1, odist, type, batch,
                                        &work);
    if (r != CUFFT_SUCCESS) {
      cufftDestroy(p);
      return set_error(c, THC_ERR_CUFFT, "cufftMakePlanMany64 failed (%d)", (int)r);
    }
    c->plans[key] = p;
    c->plan_work[key] = work;
  }
  void* wa = ws_get(c, WS_FFTWORK, c->plan_work[key]);
  if (!wa) return set_error(c, THC_ERR_NOMEM, "cuFFT work area");
  if (cufftSetWorkArea(p, wa) != CUFFT_SUCCESS || cufftSetStream(p, c->stream) != CUFFT_SUCCESS)
    return set_error(c, THC_ERR_CUFFT, "cuFFT work area / stream");
  *out = p;
  return THC_OK;
}

int fft_forward(Ctx* c, int n0, int n1, int n2, int count, cufftType type, void* in, void* out)
{
  const long long ng = (long long)n0 * n1 * n2;
  const long long nc = (long long)n0 * n1 * (n2 / 2 + 1);
  const size_t esz = type == CUFFT_D2Z ? sizeof(double) : sizeof(float);
  ProfScope prof(c, "fft");
  for (int f0 = 0; f0 < count; f0 += kFftChunk) {
    const int nb = std::min(kFftChunk, count - f0);
    cufftHandle plan;
    int st = get_plan(c, n0, n1, n2, nb, type, &plan);
    if (st) return st;
    char* src = (char*)in + esz * ng * f0;
    char* dst = (char*)out + 2 * esz * nc * f0;
    cufftResult r = type == CUFFT_D2Z
        ? cufftExecD2Z(plan, (double*)src, (cufftDoubleComplex*)dst)
        : cufftExecR2C(plan, (float*)src, (cufftComplex*)dst);
    if (r != CUFFT_SUCCESS)
      return set_error(c, THC_ERR_CUFFT, "cufftExec%s failed (%d)",
                       type == CUFFT_D2Z ? "D2Z" : "R2C", (int)r);
    c->launches++;
  }
  return THC_OK;
}

int isdf_run(Ctx* c, const double* phi_in, long long ng, int no, const int* idx_in, int nmu,
             const int* mesh_in, const double* coul_in, double shift_rel, double* out_orb,
             double* out_M, double* out_L, thc_isdf_stats* stats, const double* phiocc_in,
             int nocc, double* out_orb_occ, bool cplx)
{
  c->zeta_elem = 0;   // the workspace is about to be rewritten
  if (!phi_in || !idx_in || !mesh_in || !coul_in || ng <= 0 || no <= 0 || nmu <= 0 ||
      nmu > ng || (phiocc_in && nocc <= 0))
    return set_error(c, THC_ERR_ARG, "thc_isdf: invalid arguments");
  const bool half = phiocc_in != nullptr;
  if (half && cplx)
    return set_error(c, THC_ERR_ARG, "thc_isdf: the half-rotated path takes real orbitals");
  // Row width of phi in doubles: N_o real values, or N_o (re, im) pairs.
  const int kw = cplx ? 2 * no : no;
  int mesh[3];
  if (is_device_ptr(mesh_in)) {
    THC_CUDA(c, cudaMemcpy(mesh, mesh_in, sizeof(mesh), cudaMemcpyDeviceToHost));
  } else {
    std::copy(mesh_in, mesh_in + 3, mesh);
  }
  if (mesh[0] <= 0 || mesh[1] <= 0 || mesh[2] <= 0 ||
      (long long)mesh[0] * mesh[1] * mesh[2] != ng)
    return set_error(c, THC_ERR_SHAPE, "thc_isdf: FFT mesh %dx%dx%d does not match N_g=%lld",
                     mesh[0], mesh[1], mesh[2], ng);
  if (c->precision == THC_PREC_MIXED && !half && !cplx) return isdf_run_mixed(c, phi_in, ng, no, idx_in, nmu, mesh,
                                                            coul_in, shift_rel, out_orb, out_M,
                                                            out_L, stats);
  cudaStream_t s = c->stream;
  int st = 0;
  const double* phi = (const double*)to_device(c, phi_in, sizeof(double) * ng * kw, WS_PHI, &st);
  if (st) return st;
  const int* idx = (const int*)to_device(c, idx_in, sizeof(int) * nmu, WS_IDX, &st);
  if (st) return st;
  const double* coul = (const double*)to_device(c, coul_in, sizeof(double) * ng, WS_COUL, &st);
  if (st) return st;
  const double* phiocc = nullptr;
  double* phimu_occ = nullptr;
  if (half) {
    // One slot: the occupied orbitals (staged when they are on the host), then their rows
    // at the interpolating points.
    const bool dev = is_device_ptr(phiocc_in);
    double* occ = (double*)ws_get(c, WS_PHIOCC, sizeof(double) * ((dev ? 0 : ng) + nmu) * nocc);
    if (!occ) return set_error(c, THC_ERR_NOMEM, "thc_isdf: workspace allocation failed");
    if (dev) {
      phiocc = phiocc_in;
      phimu_occ = occ;
    } else {
      THC_CUDA(c, cudaMemcpyAsync(occ, phiocc_in, sizeof(double) * ng * nocc,
                                  cudaMemcpyHostToDevice, s));
      phiocc = occ;
      phimu_occ = occ + ng * nocc;
    }
  }

  const int n0 = mesh[0], n1 = mesh[1], n2 = mesh[2];
  const long long nc = (long long)n0 * n1 * (n2 / 2 + 1);
  const long long nn = (long long)nmu * nmu;
  // Complex orbitals: phimu holds the gathered pair rows and then their rotated copies.
  double* phimu = (double*)ws_get(c, WS_PHIMU, sizeof(double) * nmu * kw * (cplx ? 2 : 1));
  double* phij = nullptr;
  if (cplx) {
    phij = (double*)ws_get(c, WS_PHIOCC, sizeof(double) * ng * kw);
    if (!phij) return set_error(c, THC_ERR_NOMEM, "thc_isdf: workspace allocation failed");
  }
  double* C = (double*)ws_get(c, WS_C, sizeof(double) * 2 * nn);   // C and its factor
  double* Cinv = (double*)ws_get(c, WS_CINV, sizeof(double) * nn);
  double* zt = (double*)ws_get(c, WS_ZT, sizeof(double) * nmu * ng);
  double* zeta = (double*)ws_get(c, WS_ZETA, sizeof(double) * nmu * ng);
  double* zhat = (double*)ws_get(c, WS_ZHAT, sizeof(double) * 2 * nmu * nc);
  double* dsym = (double*)ws_get(c, WS_DSYM, sizeof(double) * nc);
  double* danti = (double*)ws_get(c, WS_DANTI, sizeof(double) * nc);
  double* Mw = (double*)ws_get(c, WS_M, sizeof(double) * 4 * nn);  // Re M lower, X, complex M
  double* Lw = (double*)ws_get(c, WS_L, sizeof(double) * 2 * nn);
  char* scr = (char*)ws_get(c, WS_SCRATCH, 4096);
  const long long nblk64 = (nmu + 63) / 64;
  double* dinv = (double*)ws_get(c, WS_DINV, sizeof(double) * (nblk64 * 64 * 64 + nn + 64 * (long long)nmu));
  double* Xinv = dinv + nblk64 * 64 * 64;
  double* Tinv = Xinv + nn;
  if (!phimu || !C || !Cinv || !zt || !zeta || !zhat || !dsym || !danti || !Mw || !Lw || !scr || !dinv)
    return set_error(c, THC_ERR_NOMEM, "thc_isdf: workspace allocation failed");
  CholStatus* cs = (CholStatus*)scr;
  CholStatus* csm = cs + 1;
  double* dmean = (double*)(scr + 256);
  double* thr = dmean + 1;
  double* shift_dev = dmean + 2;
  double* zero = dmean + 3;
  int* bad = (int*)(scr + 512);
  int* n_anti = bad + 1;
  // Orbital outputs: written in place on the device, else staged for the host copy.
  double* orb_dev = nullptr;
  double* occ_dev = nullptr;
  const bool orb_host = out_orb && !is_device_ptr(out_orb);
  const bool occ_host = half && out_orb_occ && !is_device_ptr(out_orb_occ);
  double* orb_stage = nullptr;
  if (orb_host || occ_host) {
    orb_stage = (double*)ws_get(c, WS_ORB, sizeof(double) * 2 * nmu * (no + (half ? nocc : 0)));
    if (!orb_stage) return set_error(c, THC_ERR_NOMEM, "thc_isdf: orbital staging buffer");
  }
  if (out_orb) orb_dev = orb_host ? orb_stage : out_orb;
  if (half && out_orb_occ) occ_dev = occ_host ? orb_stage + 2 * (long long)nmu * no : out_orb_occ;
  THC_CUDA(c, cudaMemsetAsync(scr + 512, 0, 64, s));
  THC_CUDA(c, cudaEventRecord(c->ev0, s));

  gather_rows<<<(int)cdiv((long long)nmu * kw, 256), 256, 0, s>>>(phi, ng, kw, idx, nmu, phimu,
                                                                  cplx ? nullptr : orb_dev, bad);
  THC_LAUNCHED(c, "gather_rows");
  double* phimu_j = phimu + (long long)nmu * kw;
  if (cplx) {
    if (orb_dev) {
      complex_orbitals_out<<<(int)cdiv((long long)nmu * no, 256), 256, 0, s>>>(phimu, nmu, no,
                                                                              orb_dev);
      THC_LAUNCHED(c, "complex_orbitals_out");
    }
    rotate_pairs<<<(int)cdiv(ng * no, 256), 256, 0, s>>>(phi, ng * no, phij);
    THC_LAUNCHED(c, "rotate_pairs");
    rotate_pairs<<<(int)cdiv((long long)nmu * no, 256), 256, 0, s>>>(phimu, (long long)nmu * no,
                                                                    phimu_j);
    THC_LAUNCHED(c, "rotate_pairs");
  }
  if (orb_host)
    THC_CUDA(c, cudaMemcpyAsync(out_orb, orb_dev, sizeof(double) * 2 * nmu * no,
                                cudaMemcpyDeviceToHost, s));
  if (half) {
    gather_rows<<<(int)cdiv((long long)nmu * nocc, 256), 256, 0, s>>>(phiocc, ng, nocc, idx, nmu,
                                                                      phimu_occ, occ_dev, bad);
    THC_LAUNCHED(c, "gather_rows");
    if (occ_host)
      THC_CUDA(c, cudaMemcpyAsync(out_orb_occ, occ_dev, sizeof(double) * 2 * nmu * nocc,
                                  cudaMemcpyDeviceToHost, s));
  }
  // C = (Phi_mu Phi_mu^T)^2
  {
    GemmArgs g;
    g.M = nmu; g.N = nmu; g.K = kw;
    g.A = phimu; g.sam = kw; g.sak = 1;
    g.B = phimu; g.sbn = kw; g.sbk = 1;
    g.C = C; g.ldc = nmu; g.mode = half ? GEMM_STORE : GEMM_SQUARE;
    if ((st = dgemm(c, g))) return st;
  }
  // Z^T = (Phi_mu Phi^T)^2
  {
    GemmArgs g;
    g.M = nmu; g.N = ng; g.K = kw;
    g.A = phimu; g.sam = kw; g.sak = 1;
    g.B = phi; g.sbn = kw; g.sbk = 1;
    g.C = zt; g.ldc = ng; g.mode = half ? GEMM_STORE : GEMM_SQUARE;
    if ((st = dgemm(c, g))) return st;
  }
  if (cplx) {
    // Z = P o conj(P) = (Re P)^2 + (Im P)^2 (setup_CZt, src/interpolating_vectors.cpp:127-141):
    // the squared real parts are in C and zt; the imaginary parts go through Cinv and zeta,
    // which are written later.
    GemmArgs g;
    g.M = nmu; g.N = nmu; g.K = kw;
    g.A = phimu; g.sam = kw; g.sak = 1;
    g.B = phimu_j; g.sbn = kw; g.sbk = 1;
    g.C = Cinv; g.ldc = nmu; g.mode = GEMM_STORE;
    if ((st = dgemm(c, g))) return st;
    GemmArgs h;
    h.M = nmu; h.N = ng; h.K = kw;
    h.A = phimu; h.sam = kw; h.sak = 1;
    h.B = phij; h.sbn = kw; h.sbk = 1;
    h.C = zeta; h.ldc = ng; h.mode = GEMM_STORE;
    if ((st = dgemm(c, h))) return st;
    add_square_k<<<(int)cdiv(nn, 256), 256, 0, s>>>(C, nmu, Cinv, nmu, nmu, nmu);
    THC_LAUNCHED(c, "add_square");
    add_square_k<<<(int)cdiv((long long)nmu * ng, 256), 256, 0, s>>>(zt, ng, zeta, ng, nmu, ng);
    THC_LAUNCHED(c, "add_square");
  }
  if (half) {
    // Half-rotated products: C = (Phi_mu Phi_mu^T) o (Phi_occ,mu Phi_occ,mu^T) and
    // Z^T = (Phi_mu Phi^T) o (Phi_occ,mu Phi_occ^T) (setup_CZt_half,
    // src/interpolating_vectors.cpp:143-161).  The occupied products go through Cinv and
    // zeta, which are written later.
    GemmArgs g;
    g.M = nmu; g.N = nmu; g.K = nocc;
    g.A = phimu_occ; g.sam = nocc; g.sak = 1;
    g.B = phimu_occ; g.sbn = nocc; g.sbk = 1;
    g.C = Cinv; g.ldc = nmu; g.mode = GEMM_STORE;
    if ((st = dgemm(c, g))) return st;
    GemmArgs h;
    h.M = nmu; h.N = ng; h.K = nocc;
    h.A = phimu_occ; h.sam = nocc; h.sak = 1;
    h.B = phiocc; h.sbn = nocc; h.sbk = 1;
    h.C = zeta; h.ldc = ng; h.mode = GEMM_STORE;
    if ((st = dgemm(c, h))) return st;
    hadamard_k<<<(int)cdiv(nn, 256), 256, 0, s>>>(C, nmu, Cinv, nmu, nmu, nmu);
    THC_LAUNCHED(c, "hadamard");
    hadamard_k<<<(int)cdiv((long long)nmu * ng, 256), 256, 0, s>>>(zt, ng, zeta, ng, nmu, ng);
    THC_LAUNCHED(c, "hadamard");
  }
  // Cholesky of C with breakdown detection, then the shift policy.
  double* Lc = C + nn;
  if ((st = diag_mean(c, C, nmu, nmu, dmean))) return st;
  scale_scalar<<<1, 1, 0, s>>>(dmean, 1e-13, thr);
  THC_LAUNCHED(c, "scale_scalar");
  set_scalar<<<1, 1, 0, s>>>(shift_dev, 0.0);
  THC_LAUNCHED(c, "set_scalar");
  int chol_c_info = 0;
  bool shifted = false;
  auto factor = [&](double rel) -> int {
    THC_CUDA(c, cudaMemcpyAsync(Lc, C, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s));
    if (rel > 0.0) {
      int r = add_diag_shift(c, Lc, nmu, nmu, rel, shift_dev);
      if (r) return r;
    }
    init_chol_status<<<1, 1, 0, s>>>(cs);
    THC_LAUNCHED(c, "init_chol_status");
    return potrf_inv(c, Lc, nmu, nmu, thr, cs, dinv);
  };
  CholStatus hcs{};
  if ((st = factor(shift_rel > 0.0 ? shift_rel : 0.0))) return st;
  shifted = shift_rel > 0.0;
  THC_CUDA(c, cudaMemcpyAsync(&hcs, cs, sizeof(CholStatus), cudaMemcpyDeviceToHost, s));
  THC_CUDA(c, cudaStreamSynchronize(s));
  if (hcs.flag) {
    chol_c_info = hcs.info;
    if (shift_rel < 0.0 && !shifted) {
      if ((st = factor(1e-10))) return st;
      shifted = true;
      THC_CUDA(c, cudaMemcpyAsync(&hcs, cs, sizeof(CholStatus), cudaMemcpyDeviceToHost, s));
      THC_CUDA(c, cudaStreamSynchronize(s));
    }
    if (hcs.flag)
      return set_error(c, THC_ERR_NOT_PD, "thc_isdf: Cholesky of C failed at pivot %d", hcs.info);
  }
  // C^{-1} and zeta^T = C^{-1} Z^T.  With a shift and refinement steps, C^{-1} becomes
  // X^T P X (X = L^{-1}, P the refinement polynomial; refine_polynomial).
  const bool refining = shifted && c->refine > 0;
  if ((st = chol_inverse(c, Lc, nmu, nmu, dinv, Xinv, Tinv, refining ? nullptr : Cinv, cs)))
    return st;
  if (refining) {
    double hs = 0.0;
    THC_CUDA(c, cudaMemcpyAsync(&hs, shift_dev, sizeof(double), cudaMemcpyDeviceToHost, s));
    THC_CUDA(c, cudaStreamSynchronize(s));
    double* rb = (double*)ws_get(c, WS_REFINE, sizeof(double) * 2 * nn);
    if (!rb) return set_error(c, THC_ERR_NOMEM, "thc_isdf: refinement workspace");
    double* xt = rb + nn;
    if ((st = refine_polynomial(c, Xinv, nmu, hs, c->refine, Cinv, rb, xt))) return st;
    GemmArgs g;                                   // C^{-1}_k = X^T (P X)
    g.M = nmu; g.N = nmu; g.K = nmu;
    g.A = Xinv; g.sam = 1; g.sak = nmu;
    g.a_zero_below = 1;                           // X lower triangular, read transposed
    g.B = xt; g.sbn = 1; g.sbk = nmu;
    g.C = Cinv; g.ldc = nmu;
    if ((st = dgemm(c, g))) return st;
  }
  {
    GemmArgs g;
    g.M = nmu; g.N = ng; g.K = nmu;
    g.A = Cinv; g.sam = nmu; g.sak = 1;
    g.B = zt; g.sbn = 1; g.sbk = ng;
    g.C = zeta; g.ldc = ng;
    if ((st = dgemm(c, g))) return st;
  }
  // FFT of every interpolating vector.
  if ((st = fft_forward(c, n0, n1, n2, nmu, CUFFT_D2Z, zeta, zhat))) return st;
  coulomb_weights<<<(int)cdiv(nc, 256), 256, 0, s>>>(coul, n0, n1, n2, dsym, danti, n_anti);
  THC_LAUNCHED(c, "coulomb_weights");
  int h_anti = 0;
  THC_CUDA(c, cudaMemcpyAsync(&h_anti, n_anti, sizeof(int), cudaMemcpyDeviceToHost, s));
  // Re M (lower) = sum_k zh[mu,k] dsym[k/2] zh[nu,k] over interleaved (re, im) pairs.
  double* mre = Mw;
  double* xim = Mw + nn;
  double* mcx = Mw + 2 * nn;
  {
    GemmArgs g;
    g.M = nmu; g.N = nmu; g.K = (int)(2 * nc);
    g.A = zhat; g.sam = 2 * nc; g.sak = 1;
    g.B = zhat; g.sbn = 2 * nc; g.sbk = 1;
    g.dk = dsym; g.dk_shift = 1;
    g.C = mre; g.ldc = nmu; g.lower_only = 1;
    if (2 * nc > 0x7fffffffLL) return set_error(c, THC_ERR_SHAPE, "thc_isdf: mesh too large");
    // Long K, small output: split K over CTAs (deterministic reduction in split order).
    long long tiles = cdiv(nmu, 64) * (cdiv(nmu, 64) + 1) / 2;
    g.ksplit = (int)std::max<long long>(1, std::min<long long>(cdiv(2 * 152, tiles), cdiv(2 * nc, 4096)));
    if (g.ksplit > 1) {
      g.part = (double*)ws_get(c, WS_PART, sizeof(double) * g.ksplit * nn);
      if (!g.part) return set_error(c, THC_ERR_NOMEM, "thc_isdf: split-K buffer");
    }
    if ((st = dgemm(c, g))) return st;
  }
  THC_CUDA(c, cudaStreamSynchronize(s));
  if (h_anti > 0) {
    // X = sum_c zh_re[mu,c] danti[c] zh_im[nu,c];  Im M = X - X^T.
    GemmArgs g;
    g.M = nmu; g.N = nmu; g.K = (int)nc;
    g.A = zhat; g.sam = 2 * nc; g.sak = 2;
    g.B = zhat + 1; g.sbn = 2 * nc; g.sbk = 2;
    g.dk = danti; g.dk_shift = 0;
    g.C = xim; g.ldc = nmu;
    if ((st = dgemm(c, g))) return st;
  }
  int nb2 = (int)cdiv(nn, 256);
  assemble_m<<<nb2, 256, 0, s>>>(mre, h_anti > 0 ? xim : nullptr, nmu, mcx);
  THC_LAUNCHED(c, "assemble_m");
  // Cholesky of M (the half-rotated M is returned as it is).
  init_chol_status<<<1, 1, 0, s>>>(csm);
  THC_LAUNCHED(c, "init_chol_status");
  set_scalar<<<1, 1, 0, s>>>(zero, 0.0);
  THC_LAUNCHED(c, "set_scalar");
  double* Lout = Lw;
  if (half) {
    // no factor
  } else if (h_anti == 0) {
    copy_lower_to_full<<<nb2, 256, 0, s>>>(mre, nmu, xim);
    THC_LAUNCHED(c, "copy_lower_to_full");
    if ((st = potrf_inv(c, xim, nmu, nmu, zero, csm, dinv))) return st;
    export_l_real<<<nb2, 256, 0, s>>>(xim, nmu, Lout);
    THC_LAUNCHED(c, "export_l_real");
  } else {
    THC_CUDA(c, cudaMemcpyAsync(Lout, mcx, sizeof(double) * 2 * nn, cudaMemcpyDeviceToDevice, s));
    if ((st = zpotrf_small(c, Lout, nmu, zero, csm))) return st;
    zero_upper_complex<<<nb2, 256, 0, s>>>(Lout, nmu);
    THC_LAUNCHED(c, "zero_upper_complex");
  }
  THC_CUDA(c, cudaEventRecord(c->ev1, s));
  if (out_M) THC_CUDA(c, cudaMemcpyAsync(out_M, mcx, sizeof(double) * 2 * nn, cudaMemcpyDefault, s));
  if (out_L && !half)
    THC_CUDA(c, cudaMemcpyAsync(out_L, Lout, sizeof(double) * 2 * nn, cudaMemcpyDefault, s));
  CholStatus hm{};
  int hbad = 0;
  THC_CUDA(c, cudaMemcpyAsync(&hm, csm, sizeof(CholStatus), cudaMemcpyDeviceToHost, s));
  THC_CUDA(c, cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  double hshift = 0.0;
  THC_CUDA(c, cudaMemcpyAsync(&hshift, shift_dev, sizeof(double), cudaMemcpyDeviceToHost, s));
  THC_CUDA(c, cudaStreamSynchronize(s));
  if (hbad) return set_error(c, THC_ERR_ARG, "thc_isdf: interpolating index out of range");
  c->zeta_last = zeta;
  c->zeta_elem = sizeof(double);
  c->zeta_ng = ng;
  c->zeta_nmu = nmu;
  if (stats) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    stats->chol_c_info = chol_c_info;
    stats->chol_m_info = hm.flag ? hm.info : 0;
    stats->rank_deficient = shifted ? 1 : 0;
    stats->n_anti = h_anti;
    stats->shift_used = hshift;
    stats->c_min_pivot = hcs.max_piv > 0 ? hcs.min_piv / hcs.max_piv : 0.0;
    stats->device_ms = ms;
  }
  if (hm.flag)
    return set_error(c, THC_ERR_NOT_PD, "Cholesky decomposition failed: leading minor %d", hm.info);
  return THC_OK;
}

}  // namespace thc
