// Mixed-precision ISDF: the same quantities as isdf.cu with the three large products on
// the BF16 tensor cores through error-free slicing (ozgemm):
//   Z      = (Phi Phi_mu^T)^2      sliced GEMM, FP64 result, squared in the epilogue
//   zeta^T = C^{-1} Z^T            sliced GEMM, FP32 result (input of the FP32 FFT; FP64
//                                  and a D2Z FFT with the fft64 option)
//   Re M   = A A^T, A = zeta_hat * sqrt(w v_sym)  sliced GEMM over the half spectrum
// C, its Cholesky factor and C^{-1} stay FP64 (C is ill-conditioned: cond ~1e6-1e9), and
// so does the Cholesky factorisation of M.  The slice depths fix the accuracy: each
// product is exact to ~(L+2) 2^{-7(L+1)} of sum |A||B| (ozgemm.cuh).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "dense64.cuh"
#include "isdf.cuh"
#include "ozgemm.cuh"

namespace thc {

namespace {

__global__ void gather_rows_m(const double* __restrict__ phi, long long ng, int no,
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
    orbitals[2 * ((long long)i * nmu + mu)] = v;
    orbitals[2 * ((long long)i * nmu + mu) + 1] = 0.0;
  }
}

// With a Coulomb kernel that is negative somewhere, sq / sqd carry sqrt(max(w v_sym, 0))
// and sqn / sqdn sqrt(max(-w v_sym, 0)): M = A+ A+^T - A- A-^T.
__global__ void coulomb_weights_m(const double* __restrict__ v, int n0, int n1, int n2,
                                  double* dsym, double* danti, float* sq, double* sqd,
                                  int* n_anti, float* sqn, double* sqdn, int* n_neg)
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
  double ds = w * 0.5 * (vp + vn);
  dsym[e] = ds;
  const double rt = sqrt(fmax(ds, 0.0));
  sq[e] = (float)rt;
  if (sqd) sqd[e] = rt;
  const double rn = sqrt(fmax(-ds, 0.0));
  sqn[e] = (float)rn;
  if (sqdn) sqdn[e] = rn;
  if (ds < 0.0) atomicAdd(n_neg, 1);
  double a = w * 0.5 * (vp - vn);
  danti[e] = a;
  if (a != 0.0) atomicAdd(n_anti, 1);
}

// X[mu, nu] = sum_c danti[c] Re zh[mu, c] Im zh[nu, c] over the points with danti != 0
// (zh: float2 or double2 half spectra).
template <typename Cplx>
__global__ void imag_part_c64(const Cplx* __restrict__ zh, long long nc, int nmu,
                              const double* __restrict__ danti, double* X)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)nmu * nmu) return;
  int mu = (int)(e / nmu), nu = (int)(e % nmu);
  double s = 0.0;
  for (long long c = 0; c < nc; c++) {
    double d = danti[c];
    if (d != 0.0) s += d * (double)zh[mu * nc + c].x * (double)zh[nu * nc + c].y;
  }
  X[e] = s;
}

__global__ void assemble_m_m(const double* __restrict__ mre, const double* __restrict__ x,
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

__global__ void copy_lower_to_full_m(const double* __restrict__ src, int n, double* dst)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * n) return;
  int r = (int)(e / n), c = (int)(e % n);
  dst[e] = r >= c ? src[e] : src[(long long)c * n + r];
}

__global__ void export_l_real_m(const double* __restrict__ L, int n, double* out)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * n) return;
  int r = (int)(e / n), c = (int)(e % n);
  out[2 * e] = c <= r ? L[e] : 0.0;
  out[2 * e + 1] = 0.0;
}

__global__ void zero_upper_complex_m(double* A, int n)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * n) return;
  int r = (int)(e / n), c = (int)(e % n);
  if (c > r) { A[2 * e] = 0.0; A[2 * e + 1] = 0.0; }
}

// Power-of-two equilibration of a symmetric positive semi-definite C: t_i = 2^{-k_i},
// k_i = round(log2 sqrt(C_ii)) (k_i = 0 for a non-positive diagonal, or when off).
__global__ void equil_scales(const double* __restrict__ C, int n, int on, double* t, int* k)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double d = C[(long long)i * n + i];
  int e = 0;
  if (on && d > 0.0) e = (int)rint(0.5 * log2(d));
  k[i] = e;
  t[i] = ldexp(1.0, -e);
}

// dst = diag(t) src diag(t) (exact: powers of two)
__global__ void scale_sym(const double* __restrict__ src, const double* __restrict__ t, int n,
                          double* dst)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * n) return;
  dst[e] = src[e] * t[e / n] * t[e % n];
}

// A[i][j] *= t[i] (rows) or t[j] (columns), into dst.
__global__ void scale_rows_cols(const double* __restrict__ A, const double* __restrict__ t, int n,
                                int cols, double* dst)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * n) return;
  dst[e] = A[e] * t[cols ? e % n : e / n];
}

// shift = rel * mean diag(C) (of the unscaled C); A_ii += shift t_i^2.
__global__ void add_shift_scaled(double* A, int n, const double* dmean, double rel,
                                 const double* __restrict__ t, double* shift_out)
{
  const double sh = rel * *dmean;
  if (blockIdx.x == 0 && threadIdx.x == 0) *shift_out = sh;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    A[(long long)i * n + i] += sh * t[i] * t[i];
}

__global__ void scaled_threshold(const double* dmean_s, double* thr) { *thr = 1e-13 * *dmean_s; }

// y[i] -= x[i]
__global__ void sub_from(const double* __restrict__ x, long long n, double* y)
{
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) y[i] -= x[i];
}

// y[i] = x[i] + a y[i]
__global__ void axpy_from(const double* __restrict__ x, double a, long long n, double* y)
{
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[i] + a * y[i];
}

__global__ void mixed_scalars(double* dmean, double* thr, double* shift, double* zero)
{
  *thr = 1e-13 * *dmean;
  *shift = 0.0;
  *zero = 0.0;
}

__global__ void init_cs(CholStatus* cs)
{
  cs->flag = 0;
  cs->info = 0;
  cs->min_piv = 1.0 / 0.0;
  cs->max_piv = 0.0;
}

}  // namespace

int isdf_run_mixed(Ctx* c, const double* phi_in, long long ng, int no, const int* idx_in,
                   int nmu, const int* mesh, const double* coul_in, double shift_rel,
                   double* out_orb, double* out_M, double* out_L, thc_isdf_stats* stats)
{
  c->zeta_elem = 0;   // the workspace is about to be rewritten
  cudaStream_t s = c->stream;
  int st = 0;
  const double* phi = (const double*)to_device(c, phi_in, sizeof(double) * ng * no, WS_PHI, &st);
  if (st) return st;
  const int* idx = (const int*)to_device(c, idx_in, sizeof(int) * nmu, WS_IDX, &st);
  if (st) return st;
  const double* coul = (const double*)to_device(c, coul_in, sizeof(double) * ng, WS_COUL, &st);
  if (st) return st;
  const int n0 = mesh[0], n1 = mesh[1], n2 = mesh[2];
  const long long nc = (long long)n0 * n1 * (n2 / 2 + 1);
  const long long nn = (long long)nmu * nmu;
  const int sp = c->slices_p, sz = c->slices_z, sm = c->slices_m;
  const long long mu_pad = oz_pad_mn(nmu), mu_kpad = oz_pad_k(nmu);
  const long long ng_pad = oz_pad_mn(ng), no_kpad = oz_pad_k(no);
  const long long k2_pad = oz_pad_k(2 * nc);

  double* phimu = (double*)ws_get(c, WS_PHIMU, sizeof(double) * nmu * no);
  double* C = (double*)ws_get(c, WS_C, sizeof(double) * 2 * nn);
  double* Cinv = (double*)ws_get(c, WS_CINV, sizeof(double) * nn);
  // One region holds Z (N_g x N_mu double-word) and, once Z has been sliced, zeta followed
  // by zeta_hat: the three never live at the same time, which keeps the largest cells
  // (N_g 1.26e6, N_mu 5184) inside HBM.  zeta and zeta_hat are FP32 (R2C FFT) or, with the
  // context's fft64 option, FP64 (D2Z FFT).
  const bool f64fft = c->fft64 != 0;
  const size_t real_sz = f64fft ? sizeof(double) : sizeof(float);
  const size_t zeta_bytes = ((real_sz * (size_t)nmu * ng + 255) / 256) * 256;
  const size_t zreg_bytes = std::max(sizeof(float2) * (size_t)nmu * ng,
                                     zeta_bytes + 2 * real_sz * (size_t)nmu * nc);
  char* zreg = (char*)ws_get(c, WS_ZT, zreg_bytes);
  float2* zg = (float2*)zreg;                      // Z: N_g x N_mu, double-word
  void* zeta = zreg;                               // zeta^T: N_mu x N_g (after Z is sliced)
  void* zhat = zreg + zeta_bytes;                  // N_mu x N_c complex
  // dsym (FP64), sqrt(dsym) and sqrt(-dsym) in FP64, then both in FP32.
  double* dsym = (double*)ws_get(c, WS_DSYM, (3 * sizeof(double) + 2 * sizeof(float)) * nc + 64);
  double* danti = (double*)ws_get(c, WS_DANTI, sizeof(double) * nc);
  double* Mw = (double*)ws_get(c, WS_M, sizeof(double) * 4 * nn);
  double* Lw = (double*)ws_get(c, WS_L, sizeof(double) * 2 * nn);
  char* scr = (char*)ws_get(c, WS_SCRATCH, 4096);
  const long long nblk64 = (nmu + 63) / 64;
  double* dinv = (double*)ws_get(c, WS_DINV, sizeof(double) * (nblk64 * 64 * 64 + nn + 64 * (long long)nmu));
  double* Xinv = dinv + nblk64 * 64 * 64;
  double* Tinv = Xinv + nn;
  // Slices: A holds Phi's, then C^{-1}'s / X's; B holds Phi_mu's, Z's (or Y's), then,
  // once the solve is done, zeta_hat's for the Coulomb contraction.
  size_t a_elems = std::max((size_t)sp * ng_pad * no_kpad, 2 * (size_t)sz * mu_pad * mu_kpad);
  size_t b_elems = std::max({(size_t)sp * mu_pad * no_kpad, (size_t)sz * ng_pad * mu_kpad,
                             (size_t)sm * mu_pad * k2_pad});
  __nv_bfloat16* sa = (__nv_bfloat16*)ws_get(c, WS_SLICE_A, sizeof(__nv_bfloat16) * a_elems);
  __nv_bfloat16* sb = (__nv_bfloat16*)ws_get(c, WS_SLICE_B, sizeof(__nv_bfloat16) * b_elems);
  int* ex = (int*)ws_get(c, WS_SLICE_E, sizeof(int) * (2 * mu_pad + ng_pad + 64));
  if (!phimu || !C || !Cinv || !zg || !zeta || !zhat || !dsym || !danti || !Mw || !Lw || !scr || !dinv ||
      !sa || !sb || !ex)
    return set_error(c, THC_ERR_NOMEM, "thc_isdf (mixed): workspace allocation failed");
  double* sqd = dsym + nc;
  double* sqdn = dsym + 2 * nc;
  float* sq = (float*)(dsym + 3 * nc);
  float* sqn = sq + nc;
  int* ea = ex;
  int* eb = ex + mu_pad;
  int* et = eb + ng_pad + 64;       // exponents of the refinement's W slices
  CholStatus* cs = (CholStatus*)scr;
  CholStatus* csm = cs + 1;
  double* dmean = (double*)(scr + 256);
  double* thr = dmean + 1;
  double* shift_dev = dmean + 2;
  double* zero = dmean + 3;
  int* bad = (int*)(scr + 512);
  int* n_anti = bad + 1;
  int* gemm_err = bad + 2;
  int* n_neg = bad + 3;
  double* orb_dev = nullptr;
  if (out_orb) {
    orb_dev = is_device_ptr(out_orb) ? out_orb
                                     : (double*)ws_get(c, WS_ORB, sizeof(double) * 2 * nmu * no);
    if (!orb_dev) return set_error(c, THC_ERR_NOMEM, "thc_isdf (mixed): orbital staging buffer");
  }
  THC_CUDA(c, cudaMemsetAsync(scr + 512, 0, 64, s));
  auto gemm = [&](const OzArgs& g) { return c->gemm_tc ? ozgemm_tc(c, g, gemm_err) : ozgemm(c, g); };
  // Slice buffers are k-tiled (both GEMM kernels read either layout).
  auto slices = [&](__nv_bfloat16* buf, int* e, long long rows_pad, long long kpad, int ns) {
    SliceBuf b;
    b.s = buf; b.e = e; b.rows_pad = rows_pad; b.kpad = kpad; b.ns = ns; b.tiled = true;
    return b;
  };
  THC_CUDA(c, cudaEventRecord(c->ev0, s));

  gather_rows_m<<<(int)cdiv((long long)nmu * no, 256), 256, 0, s>>>(phi, ng, no, idx, nmu, phimu,
                                                                    orb_dev, bad);
  THC_LAUNCHED(c, "gather_rows");
  if (out_orb && orb_dev != out_orb)
    THC_CUDA(c, cudaMemcpyAsync(out_orb, orb_dev, sizeof(double) * 2 * nmu * no,
                                cudaMemcpyDeviceToHost, s));
  // C = (Phi_mu Phi_mu^T)^2 in FP64 and its factorisation.
  {
    GemmArgs g;
    g.M = nmu; g.N = nmu; g.K = no;
    g.A = phimu; g.sam = no; g.sak = 1;
    g.B = phimu; g.sbn = no; g.sbk = 1;
    g.C = C; g.ldc = nmu; g.mode = GEMM_SQUARE;
    if ((st = dgemm(c, g))) return st;
  }
  double* Lc = C + nn;
  // The solve runs on T C T (equilibration by powers of two, the context option
  // "equilibrate"): C^{-1} = T (T C T)^{-1} T, and the shift s I becomes s T^2.
  double* teq = (double*)ws_get(c, WS_EQUIL, (sizeof(double) + sizeof(int)) * nmu + 256);
  if (!teq) return set_error(c, THC_ERR_NOMEM, "thc_isdf (mixed): equilibration scales");
  int* keq = (int*)(teq + nmu);
  double* dmean_s = dmean + 4;
  equil_scales<<<(int)cdiv(nmu, 256), 256, 0, s>>>(C, nmu, c->equilibrate, teq, keq);
  THC_LAUNCHED(c, "equil_scales");
  const int nbe = (int)cdiv(nn, 256);
  if ((st = diag_mean(c, C, nmu, nmu, dmean))) return st;
  mixed_scalars<<<1, 1, 0, s>>>(dmean, thr, shift_dev, zero);
  THC_LAUNCHED(c, "mixed_scalars");
  scale_sym<<<nbe, 256, 0, s>>>(C, teq, nmu, Lc);
  THC_LAUNCHED(c, "scale_sym");
  if ((st = diag_mean(c, Lc, nmu, nmu, dmean_s))) return st;
  scaled_threshold<<<1, 1, 0, s>>>(dmean_s, thr);   // pivot threshold on the scaled matrix
  THC_LAUNCHED(c, "scaled_threshold");
  // Factorisation of T C T (+ shift) on the context's current stream.
  auto factor = [&](double rel) -> int {
    cudaStream_t fs = c->stream;
    scale_sym<<<nbe, 256, 0, fs>>>(C, teq, nmu, Lc);
    THC_LAUNCHED(c, "scale_sym");
    if (rel > 0.0) {
      add_shift_scaled<<<(int)cdiv(nmu, 256), 256, 0, fs>>>(Lc, nmu, dmean, rel, teq, shift_dev);
      THC_LAUNCHED(c, "add_shift_scaled");
    }
    init_cs<<<1, 1, 0, fs>>>(cs);
    THC_LAUNCHED(c, "init_cs");
    return potrf_inv(c, Lc, nmu, nmu, thr, cs, dinv);
  };
  // C's factorisation and inverse depend on Phi_mu only: with the context option "overlap"
  // they run on the context's second stream while the P product and Z's slicing run on the
  // main one (the Cholesky's diagonal blocks occupy one SM at a time; by default they run in
  // order on the main stream).  The expected case is taken ahead: the shift as given,
  // X = L^{-1}, and C^{-1} = X^T X in FP64 when N_mu < 512 without a shift; a breakdown of
  // the unshifted factorisation is retried on the main stream after the join.
  bool shifted = shift_rel > 0.0;
  bool cinv_tc = !shifted && nmu >= 512;
  CholStatus* hcs_p = (CholStatus*)c->pinned;      // pinned: the copy stays asynchronous
  const cudaStream_t fs = c->overlap ? c->aux_stream : s;
  {
    if (fs != s) {
      THC_CUDA(c, cudaEventRecord(c->ev_fork, s));
      THC_CUDA(c, cudaStreamWaitEvent(fs, c->ev_fork, 0));
    }
    StreamSwap on_fs(c, fs);
    if ((st = factor(shifted ? shift_rel : 0.0))) return st;
    if ((st = chol_inverse(c, Lc, nmu, nmu, dinv, Xinv, Tinv, (shifted || cinv_tc) ? nullptr : Cinv,
                           cs)))
      return st;
    THC_CUDA(c, cudaMemcpyAsync(hcs_p, cs, sizeof(CholStatus), cudaMemcpyDeviceToHost, fs));
    THC_CUDA(c, cudaEventRecord(c->ev_join, fs));
  }
  // Z = (Phi Phi_mu^T)^2 (N_g x N_mu) via the sliced GEMM: A = Phi sliced by grid point,
  // B = Phi_mu sliced by interpolating point; Z's rows are then K-contiguous for the solve.
  // Z is kept as double-word FP32 (~46 bits; the solve slices it to 42), so the epilogue
  // squares in FP32 arithmetic instead of on the narrow FP64 pipe.
  {
    const SliceBuf pa = slices(sa, eb, ng_pad, no_kpad, sp), pb = slices(sb, ea, mu_pad, no_kpad, sp);
    if ((st = oz_slice_rows_f64(c, phi, ng, no, no, 1, nullptr, 0, pa))) return st;
    if ((st = oz_slice_rows_f64(c, phimu, nmu, no, no, 1, nullptr, 0, pb))) return st;
    OzArgs g;
    g.M = ng; g.N = nmu; g.K = no;
    g.a = pa.operand();
    g.b = pb.operand();
    g.levels = sp; g.epilogue = OZ_SQUARE_DW; g.C = zg; g.ldc = nmu;
    g.tag = "oz_P";
    if ((st = gemm(g))) return st;
  }
  // Z T sliced by rows (grid points) for the solve: the B operand of zeta^T = C^{-1} Z^T, or
  // the A operand of Y^T = Z X^T with a shift (the columns scaled by T, exactly).
  const SliceBuf zs = slices(sb, eb, ng_pad, mu_kpad, sz);
  if ((st = oz_slice_rows_dw(c, zg, ng, nmu, nmu, zs, keq))) return st;
  // Join C's factorisation: the host waits for its status only (the P product and Z's
  // slicing, queued behind it, keep the GPU busy meanwhile).
  THC_CUDA(c, cudaEventSynchronize(c->ev_join));
  if (fs != s) THC_CUDA(c, cudaStreamWaitEvent(s, c->ev_join, 0));
  CholStatus hcs = *hcs_p;
  int chol_c_info = 0;
  if (hcs.flag) {
    chol_c_info = hcs.info;
    if (shift_rel < 0.0 && !shifted) {
      if ((st = factor(1e-10))) return st;
      shifted = true;
      cinv_tc = false;
      THC_CUDA(c, cudaMemcpyAsync(&hcs, cs, sizeof(CholStatus), cudaMemcpyDeviceToHost, s));
      THC_CUDA(c, cudaStreamSynchronize(s));
      if (!hcs.flag && (st = chol_inverse(c, Lc, nmu, nmu, dinv, Xinv, Tinv, nullptr, cs)))
        return st;
    }
    if (hcs.flag)
      return set_error(c, THC_ERR_NOT_PD, "thc_isdf: Cholesky of C failed at pivot %d", hcs.info);
  }
  // X = L^{-1}; C^{-1} = X^T X is needed by the full-rank solve only.  From N_mu = 512 on,
  // that product runs as a sliced tensor GEMM (A = B = the slices of X^T): on C2 its M
  // error is 4e-9, while the FP64 product would cost 2 N_mu^3 on the narrow FP64 pipe.
  if (cinv_tc) {
    const SliceBuf xt = slices(sa, ea, mu_pad, mu_kpad, sz);
    if ((st = oz_slice_rows_f64(c, Xinv, nmu, nmu, 1, nmu, nullptr, 0, xt)))   // rows of X^T
      return st;
    OzArgs g;
    g.M = nmu; g.N = nmu; g.K = nmu;
    g.a = xt.operand();
    g.b = g.a;
    g.levels = sz; g.epilogue = OZ_STORE_F64; g.C = Cinv; g.ldc = nmu;
    g.tag = "oz_cinv";
    g.ksplit = oz_choose_split(nmu, nmu, nmu, false);
    if (g.ksplit > 1) {
      g.part = (double*)ws_get(c, WS_PART, sizeof(double) * g.ksplit * nn);
      if (!g.part) return set_error(c, THC_ERR_NOMEM, "thc_isdf: split-K partials");
    }
    if ((st = gemm(g))) return st;
  }
  if (!shifted) {
    // (T C T)^{-1} -> T (T C T)^{-1}: the left factor T (row scaling; the right one scales Z's
    // columns while they are sliced).
    scale_rows_cols<<<nbe, 256, 0, s>>>(Cinv, teq, nmu, 0, Cinv);
    THC_LAUNCHED(c, "scale_rows_cols");
  }
  // zeta^T = C^{-1} Z^T: A = C^{-1} sliced by rows, B = Z sliced by rows (grid points).
  // A rank-deficient C (shifted) has an inverse whose null-space entries are ~1/shift, so
  // the product cancels by far more than any slice depth resolves: it runs in FP64 then.
  if (shifted) {
    // Regularised (rank-deficient) C: never form C^{-1} = X^T X (X = L^{-1}), whose
    // null-space entries are ~1/shift and would swamp the slices.  Two sliced products with
    // X instead, each amplifying by ~1/sqrt(shift) only: Y^T = Z X^T, then
    // zeta^T = X^T Y.  (Emulated on the C1 cell this is also more accurate than the FP64
    // C^{-1} product: pair-Coulomb invariant 1.7e-8 against 2.2e-6.)
    const SliceBuf xs = slices(sa, ea, mu_pad, mu_kpad, sz);
    // Here X = L^{-1} of the equilibrated T (C + sI) T = L L^T, so (C + sI)^{-1} =
    // T X^T X T and zeta^T = (X T)^T (X (T Z^T)): the first product slices Z's columns scaled
    // by T.  Iterative refinement of the shifted solve (refine_polynomial in dense64.cuh)
    // puts P X in place of X in the first product, P = sum_j (s G)^j with G = X T^2 X^T,
    // formed with the sliced GEMM: G once, then k Horner steps W <- X + s G W.
    double* rb = (double*)ws_get(c, WS_REFINE, sizeof(double) * 3 * nn);
    if (!rb) return set_error(c, THC_ERR_NOMEM, "thc_isdf: refinement workspace");
    double* xsc = rb + 2 * nn;                   // X T
    scale_rows_cols<<<nbe, 256, 0, s>>>(Xinv, teq, nmu, 1, xsc);
    THC_LAUNCHED(c, "scale_rows_cols");
    const double* xfirst = Xinv;
    if (c->refine > 0) {
      double hs = 0.0;
      THC_CUDA(c, cudaMemcpyAsync(&hs, shift_dev, sizeof(double), cudaMemcpyDeviceToHost, s));
      THC_CUDA(c, cudaStreamSynchronize(s));
      double* G = Cinv;                          // unused by the shifted solve
      double* tb[2] = {rb, rb + nn};
      // W's slices behind X's in the A buffer (B holds Z's slices).
      const SliceBuf ts = slices(sa + (size_t)sz * mu_pad * mu_kpad, et, mu_pad, mu_kpad, sz);
      auto product = [&](const SliceBuf& a, const SliceBuf& b, double* out, const char* tag) {
        OzArgs g;
        g.M = nmu; g.N = nmu; g.K = nmu;
        g.a = a.operand();
        g.b = b.operand();
        g.levels = sz; g.epilogue = OZ_STORE_F64; g.C = out; g.ldc = nmu;
        g.tag = tag;
        g.ksplit = oz_choose_split(nmu, nmu, nmu, false);
        if (g.ksplit > 1) {
          g.part = (double*)ws_get(c, WS_PART, sizeof(double) * g.ksplit * nn);
          if (!g.part) return set_error(c, THC_ERR_NOMEM, "thc_isdf: split-K partials");
        }
        return gemm(g);
      };
      if ((st = oz_slice_rows_f64(c, xsc, nmu, nmu, nmu, 1, nullptr, 0, xs))) return st;
      if ((st = product(xs, xs, G, "oz_refine"))) return st;           // G = X T^2 X^T
      if ((st = oz_slice_rows_f64(c, G, nmu, nmu, nmu, 1, nullptr, 0, xs))) return st;
      const double* cur = Xinv;
      for (int j = 1; j <= c->refine; j++) {
        double* dst = tb[j & 1];
        if ((st = oz_slice_rows_f64(c, cur, nmu, nmu, 1, nmu, nullptr, 0, ts))) return st;
        if ((st = product(xs, ts, dst, "oz_refine"))) return st;              // G cur
        axpy_from<<<(int)cdiv(nn, 256), 256, 0, s>>>(Xinv, hs, nn, dst);     // X + s G cur
        THC_LAUNCHED(c, "axpy_from");
        cur = dst;
      }
      xfirst = cur;
    }
    if ((st = oz_slice_rows_f64(c, xfirst, nmu, nmu, nmu, 1, nullptr, 0, xs))) return st; // rows of P X
    {
      OzArgs g;                                  // Y^T (N_g x N_mu) = Z X^T, into zg
      g.M = ng; g.N = nmu; g.K = nmu;
      g.a = zs.operand();
      g.b = xs.operand();
      g.levels = sz; g.epilogue = OZ_STORE_DW; g.C = zg; g.ldc = nmu;
      g.tag = "oz_Y";
      if ((st = gemm(g))) return st;
    }
    if ((st = oz_slice_rows_f64(c, xsc, nmu, nmu, 1, nmu, nullptr, 0, xs))) return st;   // rows of (X T)^T
    if ((st = oz_slice_rows_dw(c, zg, ng, nmu, nmu, zs))) return st;                    // rows of Y^T
    OzArgs g;                                    // zeta^T = X^T Y
    g.M = nmu; g.N = ng; g.K = nmu;
    g.a = xs.operand();
    g.b = zs.operand();
    g.levels = sz; g.epilogue = f64fft ? OZ_STORE_F64 : OZ_STORE_F32; g.C = zeta; g.ldc = ng;
    g.tag = "oz_zeta";
    if ((st = gemm(g))) return st;
  } else {
    const SliceBuf ci = slices(sa, ea, mu_pad, mu_kpad, sz);
    if ((st = oz_slice_rows_f64(c, Cinv, nmu, nmu, nmu, 1, nullptr, 0, ci))) return st;
    OzArgs g;
    g.M = nmu; g.N = ng; g.K = nmu;
    g.a = ci.operand();
    g.b = zs.operand();
    g.levels = sz; g.epilogue = f64fft ? OZ_STORE_F64 : OZ_STORE_F32; g.C = zeta; g.ldc = ng;
    g.tag = "oz_zeta";
    if ((st = gemm(g))) return st;
  }
  // R2C (FP32) or D2Z (FP64) FFT of every interpolating vector.
  if ((st = fft_forward(c, n0, n1, n2, nmu, f64fft ? CUFFT_D2Z : CUFFT_R2C, zeta, zhat)))
    return st;
  coulomb_weights_m<<<(int)cdiv(nc, 256), 256, 0, s>>>(coul, n0, n1, n2, dsym, danti, sq,
                                                       f64fft ? sqd : nullptr, n_anti, sqn,
                                                       f64fft ? sqdn : nullptr, n_neg);
  THC_LAUNCHED(c, "coulomb_weights");
  int* h_flags = (int*)((char*)c->pinned + Ctx::kPinnedCounts);   // [0] n_anti, [1] n_neg
  THC_CUDA(c, cudaMemcpyAsync(h_flags, n_anti, sizeof(int), cudaMemcpyDeviceToHost, s));
  THC_CUDA(c, cudaMemcpyAsync(h_flags + 1, n_neg, sizeof(int), cudaMemcpyDeviceToHost, s));
  THC_CUDA(c, cudaEventRecord(c->ev_fork, s));
  double* mre = Mw;
  double* xim = Mw + nn;
  double* mcx = Mw + 2 * nn;
  // Re M (lower) = A A^T with A = zeta_hat (interleaved re, im) scaled by sqrt(w v_sym)
  // (by sqrt(max(+-w v_sym, 0)) for the two parts of a kernel with negative values).
  auto coulomb_product = [&](const float* scale32, const double* scale64, double* out) -> int {
    const SliceBuf zh = slices(sb, ea, mu_pad, k2_pad, sm);
    int r = f64fft ? oz_slice_rows_f64(c, (const double*)zhat, nmu, 2 * nc, 2 * nc, 1, scale64, 1, zh)
                   : oz_slice_rows_f32(c, (const float*)zhat, nmu, 2 * nc, 2 * nc, scale32, 1, zh);
    if (r) return r;
    OzArgs g;
    g.M = nmu; g.N = nmu; g.K = 2 * nc;
    g.a = zh.operand();
    g.b = g.a;
    g.levels = sm; g.epilogue = OZ_STORE_F64; g.C = out; g.ldc = nmu; g.lower_only = 1;
    g.tag = "oz_M";
    // Long K (2 N_c) and a small N_mu x N_mu output: split K over CTAs.
    g.ksplit = oz_choose_split(nmu, nmu, 2 * nc, true);
    if (g.ksplit > 1) {
      g.part = (double*)ws_get(c, WS_PART, sizeof(double) * g.ksplit * nn);
      if (!g.part) return set_error(c, THC_ERR_NOMEM, "thc_isdf: split-K buffer");
    }
    return gemm(g);
  };
  if ((st = coulomb_product(sq, sqd, mre))) return st;
  // The host waits for the two counts only; the Coulomb product runs meanwhile.
  THC_CUDA(c, cudaEventSynchronize(c->ev_fork));
  const int h_anti = h_flags[0], h_neg = h_flags[1];
  int nb2 = (int)cdiv(nn, 256);
  if (h_neg > 0) {
    double* mneg = Cinv;                          // free once zeta is formed
    if ((st = coulomb_product(sqn, sqdn, mneg))) return st;
    sub_from<<<nb2, 256, 0, s>>>(mneg, nn, mre);
    THC_LAUNCHED(c, "sub_from");
  }
  if (h_anti > 0) {
    if (f64fft)
      imag_part_c64<<<nb2, 256, 0, s>>>((const double2*)zhat, nc, nmu, danti, xim);
    else
      imag_part_c64<<<nb2, 256, 0, s>>>((const float2*)zhat, nc, nmu, danti, xim);
    THC_LAUNCHED(c, "imag_part_c64");
  }
  assemble_m_m<<<nb2, 256, 0, s>>>(mre, h_anti > 0 ? xim : nullptr, nmu, mcx);
  THC_LAUNCHED(c, "assemble_m");
  init_cs<<<1, 1, 0, s>>>(csm);
  THC_LAUNCHED(c, "init_cs");
  double* Lout = Lw;
  if (h_anti == 0) {
    copy_lower_to_full_m<<<nb2, 256, 0, s>>>(mre, nmu, xim);
    THC_LAUNCHED(c, "copy_lower_to_full");
    if ((st = potrf_inv(c, xim, nmu, nmu, zero, csm, dinv))) return st;
    export_l_real_m<<<nb2, 256, 0, s>>>(xim, nmu, Lout);
    THC_LAUNCHED(c, "export_l_real");
  } else {
    THC_CUDA(c, cudaMemcpyAsync(Lout, mcx, sizeof(double) * 2 * nn, cudaMemcpyDeviceToDevice, s));
    if ((st = zpotrf_small(c, Lout, nmu, zero, csm))) return st;
    zero_upper_complex_m<<<nb2, 256, 0, s>>>(Lout, nmu);
    THC_LAUNCHED(c, "zero_upper_complex");
  }
  THC_CUDA(c, cudaEventRecord(c->ev1, s));
  if (out_M) THC_CUDA(c, cudaMemcpyAsync(out_M, mcx, sizeof(double) * 2 * nn, cudaMemcpyDefault, s));
  if (out_L) THC_CUDA(c, cudaMemcpyAsync(out_L, Lout, sizeof(double) * 2 * nn, cudaMemcpyDefault, s));
  CholStatus hm{};
  int hbad = 0, herr = 0;
  double hshift = 0.0;
  THC_CUDA(c, cudaMemcpyAsync(&herr, gemm_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  THC_CUDA(c, cudaMemcpyAsync(&hm, csm, sizeof(CholStatus), cudaMemcpyDeviceToHost, s));
  THC_CUDA(c, cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  THC_CUDA(c, cudaMemcpyAsync(&hshift, shift_dev, sizeof(double), cudaMemcpyDeviceToHost, s));
  THC_CUDA(c, cudaStreamSynchronize(s));
  if (hbad) return set_error(c, THC_ERR_ARG, "thc_isdf: interpolating index out of range");
  if (herr) return set_error(c, THC_ERR_TIMEOUT, "thc_isdf: tensor-core GEMM wait timed out");
  c->zeta_last = zeta;
  c->zeta_elem = (int)real_sz;
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
