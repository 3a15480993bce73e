// FP64 dense linear algebra on CUDA cores: GEMM, blocked Cholesky and triangular
// solves.  These carry the all-FP64 path, which replaces the reference's ScaLAPACK
// calls one for one:
//   pzgemm 'C','N'  (P = Phi_mu^H Phi, src/interpolating_vectors.cpp:117)  -> dgemm + square
//   pzgels 'N'      (least squares C X = Z, :416)             -> potrf_inv + chol_inverse + dgemm
//   pzherk 'L','C'  (M = zeta_hat^H zeta_hat, :278)                         -> dgemm lower
//   pzpotrf 'L'     (Luv, :289)                                             -> potrf_inv
// GB300 runs FP64 at a small fraction of its FP32 rate (about two FMA lanes per clock per
// SM), so these kernels are bound by the FP64 pipe, and a GEMM must spread over all SMs:
// dgemm picks 64, 32 or 16 tiles and a split of K from the problem shape.
#include <cuda_runtime.h>
#include <math_constants.h>

#include <algorithm>

#include "common.cuh"
#include "dense64.cuh"

namespace thc {

namespace {

constexpr int BK = 16;

// C[m, n] = epilogue(sum_k A(m, k) * dk[k] * B(k, n)); AK / BK select which operand
// index is unit-stride so that the shared-memory loads stay coalesced.  T x T tile per
// CTA of 256 threads (16 x 16), (T/16)^2 outputs per thread.
template <bool AK, bool BK_, int T>
__global__ void __launch_bounds__(256) dgemm_kernel(GemmArgs g)
{
  constexpr int R = T / 16;
  constexpr int LOADS = BK * T / 256;
  if (g.skip_flag && *g.skip_flag) return;
  long long m0 = (long long)blockIdx.y * T, n0 = (long long)blockIdx.x * T;
  if (g.lower_only && n0 > m0 + T - 1 + g.lower_offset) return;
  __shared__ double As[BK][T + 1];
  __shared__ double Bs[BK][T + 1];
  int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[R][R] = {};
  int kbeg = 0, kend = g.K;
  if (g.ksplit > 1) {
    int kc = ((g.K + g.ksplit - 1) / g.ksplit + BK - 1) / BK * BK;
    kbeg = blockIdx.z * kc;
    kend = min(g.K, kbeg + kc);
  }
  // Tiles start at multiples of T >= BK, so the first nonzero k is a multiple of BK.
  if (g.a_zero_below) kbeg = max(kbeg, (int)m0);
  if (g.b_zero_below) kbeg = max(kbeg, (int)n0);
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
    for (int r = 0; r < LOADS; r++) {
      int e = threadIdx.x + 256 * r;
      int mm, kk;
      if (AK) { mm = e / BK; kk = e % BK; } else { kk = e / T; mm = e % T; }
      long long m = m0 + mm;
      int k = k0 + kk;
      double av = 0.0;
      if (m < g.M && k < kend) {
        av = g.A[m * g.sam + (long long)k * g.sak];
        if (g.dk) av *= g.dk[k >> g.dk_shift];
      }
      As[kk][mm] = av;
      int nn, kb;
      if (BK_) { nn = e / BK; kb = e % BK; } else { kb = e / T; nn = e % T; }
      long long n = n0 + nn;
      int kq = k0 + kb;
      Bs[kb][nn] = (n < g.N && kq < kend) ? g.B[n * g.sbn + (long long)kq * g.sbk] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk++) {
      double a[R], b[R];
#pragma unroll
      for (int i = 0; i < R; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < R; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < R; i++)
#pragma unroll
        for (int j = 0; j < R; j++) acc[i][j] = __fma_rn(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < R; i++) {
    long long m = m0 + ty + 16 * i;
    if (m >= g.M) continue;
#pragma unroll
    for (int j = 0; j < R; j++) {
      long long n = n0 + tx + 16 * j;
      if (n >= g.N) continue;
      if (g.lower_only && n > m + g.lower_offset) continue;
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
  if (g.lower_only && n > m + g.lower_offset) return;
  double v = 0.0;
  for (int z = 0; z < g.ksplit; z++) v += g.part[((long long)z * g.M + m) * g.N + n];
  double* cp = g.C + m * g.ldc + n;
  if (g.mode == GEMM_SQUARE) v = v * v;
  else v = g.alpha * v;
  if (g.beta != 0.0) v += g.beta * *cp;
  *cp = v;
}

// ---- Cholesky (lower, in place, row-major) --------------------------------------

// Diagonal block edge of the blocked Cholesky.  The serial part (the diagonal blocks, one
// SM each) is a latency chain of NB dependent steps per block; 32 x 32 blocks (a quarter of
// the FP64 work per block) measured no faster at n = 256 (the factorisations of C and M:
// 0.95 ms against 0.99 ms, and the triangular inverse 0.26 ms against 0.16 ms with twice the
// block rows), so both edges stay available and 64 is used.
inline int chol_nb(int) { return 64; }

// 1/sqrt(d) for a positive normal d: an FP32 seed y0 (relative error e0 < 2^-22), then one
// third-order step of the binomial series for (1 - e)^(-1/2), e = 1 - d y0^2:
// y = y0 (1 + e/2 + 3e^2/8), which leaves O(e0^3) -- below FP64 rounding.  Five dependent
// FP64 operations instead of a square root and a division: the pivot is on the critical
// path of every Cholesky step, and FP64 latency is long on this part.
__device__ __forceinline__ double rsqrt_fast(double d)
{
  const long long db = __double_as_longlong(d);
  const int ed = (int)((db >> 52) & 0x7ff);
  if (ed < 1023 - 100 || ed > 1023 + 100) return 1.0 / sqrt(d);   // outside FP32's range
  const double y = (double)rsqrtf((float)d);
  const double e = __fma_rn(-d * y, y, 1.0);
  return __fma_rn(y * e, __fma_rn(0.375, e, 0.5), y);
}

// Factor the diagonal block at (k0, k0) and invert its triangle: writes L_kk into A
// (upper part zeroed) and L_kk^{-1} into dinv (nb x nb, row-major, zero above the diagonal).
// Pivots at or below thr stop the factorisation (info = global 1-based index).
// Right-looking, two barriers per column j: (1) column j of L (a_ij r_j, r_j = 1/sqrt(d_j))
// and row j of V = L^{-1} (v_jc r_j) are scaled in place; (2) the trailing triangle takes
// a_ic -= a_ij a_cj (c > j) and the rows of V below j take v_ic -= a_ij v_jc (c <= j).  The
// FP64 pipe (two lanes per clock per SM on this part, whatever the active mask) bounds the
// block's ~nb^3/3 FMAs, so phase (2) runs as one flat list of work items with every lane
// busy (a triangle ordered by decreasing column makes the items of step j a prefix).  The
// thread that updates the next pivot a_{j+1,j+1} forms its reciprocal root at once.
template <int NB>
__global__ void __launch_bounds__(256) potrf_diag_inv(double* A, long long ld, int n, int k0,
                                                      const double* thr_p, CholStatus* cs,
                                                      double* dinv)
{
  if (cs->flag) return;
  const double thr = thr_p ? *thr_p : 0.0;
  extern __shared__ double dsm[];                       // 2 x NB x (NB + 1) doubles
  double (*a)[NB + 1] = reinterpret_cast<double (*)[NB + 1]>(dsm);
  double (*v)[NB + 1] = reinterpret_cast<double (*)[NB + 1]>(dsm + NB * (NB + 1));
  __shared__ double rr[NB], piv[NB];
  __shared__ unsigned short tri[NB * (NB - 1) / 2];     // (i << 8) | c, c descending
  const int nb = min(NB, n - k0);
  for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) {
    int r = e / NB, c = e % NB;
    a[r][c] = (r < nb && c < nb) ? A[(long long)(k0 + r) * ld + k0 + c] : (r == c ? 1.0 : 0.0);
    v[r][c] = r == c ? 1.0 : 0.0;
  }
  // Column c (1 <= c < nb) holds items (c..nb-1, c); columns nb-1, nb-2, ... come first, so
  // column c starts at T(c) = sum_{c' > c} (nb - c') = (nb - 1 - c)(nb - c) / 2.
  for (int c = 1 + (int)threadIdx.x; c < nb; c += blockDim.x) {
    const int base = (nb - 1 - c) * (nb - c) / 2;
    for (int i = c; i < nb; i++) tri[base + (i - c)] = (unsigned short)((i << 8) | c);
  }
  double pmin = cs->min_piv, pmax = cs->max_piv;
  __syncthreads();
  auto pivot = [&](int j, double d) {
    piv[j] = d;
    rr[j] = d > 0.0 ? rsqrt_fast(d) : 1.0;
  };
  if (threadIdx.x == 0) pivot(0, a[0][0]);
  __syncthreads();
  bool bad = false;
  // d > thr (thr >= 0) as an integer comparison of the bit patterns, which order like the
  // values for non-negative doubles (a negative d compares below): the FP64 pipe is the
  // scarce resource here, and every thread takes this test every step.
  const long long thr_bits = __double_as_longlong(thr > 0.0 ? thr : 0.0);
  for (int j = 0; j < nb; j++) {
    const double d = piv[j];                             // the same value in every thread
    const long long db = __double_as_longlong(d);
    if (!(db > thr_bits && ((db >> 52) & 0x7ff) != 0x7ff)) {
      if (threadIdx.x == 0) {
        cs->flag = 1;
        cs->info = k0 + j + 1;
      }
      bad = true;
      break;
    }
    if (threadIdx.x == 0) {
      pmin = fmin(pmin, d);
      pmax = fmax(pmax, d);
    }
    const double r = rr[j];
    // (1) scale column j of L (rows j..nb-1) and row j of V (columns 0..j)
    {
      const int t = threadIdx.x, na = nb - j;
      if (t < na) a[j + t][j] *= r;
      else if (t - na <= j) v[j][t - na] *= r;
    }
    __syncthreads();
    // (2) the trailing triangle (T(j) items) and the rows of V below j ((nb-1-j)(j+1) items)
    const int ntri = (nb - 1 - j) * (nb - j) / 2;
    const int nrect = (nb - 1 - j) * (j + 1);
    const int pe = ntri - (nb - 1 - j);                  // item (j+1, j+1): the next pivot
    const int w = j + 1;                                 // rectangle row length
    const float rw = 1.0f / (float)w;
    for (int e = threadIdx.x; e < ntri + nrect; e += blockDim.x) {
      if (e < ntri) {
        const unsigned code = tri[e];
        const int i = code >> 8, c = code & 255;
        const double nv = __fma_rn(-a[i][j], a[c][j], a[i][c]);
        a[i][c] = nv;
        if (e == pe) pivot(j + 1, nv);
      } else {
        // q = r w + c without an integer division: the FP32 quotient of q < 2^12 is off by
        // at most one, which the two corrections fix.
        const int q = e - ntri;
        int r = (int)((float)q * rw);
        int c = q - r * w;
        if (c < 0) { r--; c += w; }
        if (c >= w) { r++; c -= w; }
        const int i = j + 1 + r;
        v[i][c] = __fma_rn(-a[i][j], v[j][c], v[i][c]);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    cs->min_piv = pmin;
    cs->max_piv = pmax;
  }
  if (bad) return;
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    int r = e / nb, c = e % nb;
    A[(long long)(k0 + r) * ld + k0 + c] = c <= r ? a[r][c] : 0.0;
    dinv[(long long)r * nb + c] = c <= r ? v[r][c] : 0.0;
  }
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

template <int T>
static void launch_dgemm(const GemmArgs& g, cudaStream_t s)
{
  dim3 grid((unsigned)cdiv(g.N, T), (unsigned)cdiv(g.M, T), (unsigned)std::max(1, g.ksplit));
  bool ak = g.sak == 1, bk = g.sbk == 1;
  if (ak && bk) dgemm_kernel<true, true, T><<<grid, 256, 0, s>>>(g);
  else if (ak && !bk) dgemm_kernel<true, false, T><<<grid, 256, 0, s>>>(g);
  else if (!ak && bk) dgemm_kernel<false, true, T><<<grid, 256, 0, s>>>(g);
  else dgemm_kernel<false, false, T><<<grid, 256, 0, s>>>(g);
}

int dgemm(Ctx* c, const GemmArgs& g_in)
{
  if (g_in.M <= 0 || g_in.N <= 0) return THC_OK;
  GemmArgs g = g_in;
  if (g.ksplit <= 1 && !g.part) {
    // Tile and split-K so that the grid covers the SMs about twice.
    const long long want = 2LL * 152;
    auto tiles = [&](int t) {
      long long mt = cdiv(g.M, t), nt = cdiv(g.N, t);
      return g.lower_only ? (mt * nt + mt) / 2 : mt * nt;
    };
    g.tile = tiles(64) >= want / 2 ? 64 : (tiles(32) >= want / 2 ? 32 : 16);
    long long split = std::min<long long>(cdiv(want, tiles(g.tile)), std::max(1, g.K / 32));
    if (g.aliased) split = std::max<long long>(split, 2);
    if (g.no_split) {
      if (g.aliased) return set_error(c, THC_ERR_ARG, "dgemm: aliased operands need a split");
      split = 1;
    }
    g.ksplit = (int)std::max<long long>(1, std::min<long long>(split, cdiv(g.K, BK)));
    if (g.ksplit > 1) {
      g.part = (double*)ws_get(c, WS_DPART, sizeof(double) * g.ksplit * g.M * g.N);
      if (!g.part) return set_error(c, THC_ERR_NOMEM, "dgemm: split-K partials");
    }
  } else if (g.aliased && g.ksplit <= 1) {
    return set_error(c, THC_ERR_ARG, "dgemm: aliased operands need split-K partials");
  }
  ProfScope prof(c, "dgemm");
  if (g.tile == 16) launch_dgemm<16>(g, c->stream);
  else if (g.tile == 32) launch_dgemm<32>(g, c->stream);
  else launch_dgemm<64>(g, c->stream);
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
  ProfScope prof(c, "potrf_inv");
  cudaStream_t s = c->stream;
  const int NB = chol_nb(n);
  // Look-ahead (n >= 512, with the context's second stream): after block k's panel, the
  // next diagonal block is updated first, on the main stream, and factored there while the
  // rest of block k's trailing update runs on the second stream; the next panel waits for
  // that update.  The diagonal blocks' one-SM chain then runs beside the FP64 GEMMs on the
  // other SMs instead of between them.
  const bool la = n >= 512 && c->aux_stream && c->aux_stream != s;
  cudaStream_t s2 = la ? c->aux_stream : s;
  bool trail_pending = false;
  for (int k0 = 0; k0 < n; k0 += NB) {
    int nb = std::min(NB, n - k0);
    double* di = dinv + (long long)(k0 / NB) * NB * NB;
    const int smem = 2 * NB * (NB + 1) * (int)sizeof(double);
    if (NB == 32) {
      THC_CUDA(c, cudaFuncSetAttribute(potrf_diag_inv<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
      potrf_diag_inv<32><<<1, 256, smem, s>>>(A, ld, n, k0, thr, cs, di);
    } else {
      THC_CUDA(c, cudaFuncSetAttribute(potrf_diag_inv<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
      potrf_diag_inv<64><<<1, 256, smem, s>>>(A, ld, n, k0, thr, cs, di);
    }
    THC_LAUNCHED(c, "potrf_diag_inv");
    int rest = n - k0 - nb;
    if (rest <= 0) break;
    if (trail_pending) {     // the panel rows below were updated on the second stream
      THC_CUDA(c, cudaStreamWaitEvent(s, c->ev_trail, 0));
      trail_pending = false;
    }
    {
      // L_panel = A_panel L_kk^{-T}, in place (each CTA owns its rows; N = nb <= 64).
      GemmArgs g{};
      g.M = rest; g.N = nb; g.K = nb;
      g.A = A + (long long)(k0 + nb) * ld + k0; g.sam = ld; g.sak = 1;
      g.B = di; g.sbn = nb; g.sbk = 1;
      g.C = A + (long long)(k0 + nb) * ld + k0; g.ldc = ld;
      g.skip_flag = &cs->flag;
      g.aliased = 1;
      int st = dgemm(c, g);
      if (st) return st;
    }
    const double* l21 = A + (long long)(k0 + nb) * ld + k0;
    if (!la) {
      GemmArgs g{};
      g.M = rest; g.N = rest; g.K = nb;
      g.A = l21; g.sam = ld; g.sak = 1;
      g.B = l21; g.sbn = ld; g.sbk = 1;
      g.C = A + (long long)(k0 + nb) * ld + k0 + nb; g.ldc = ld;
      g.alpha = -1.0; g.beta = 1.0; g.lower_only = 1; g.mode = GEMM_STORE;
      g.skip_flag = &cs->flag;
      int st = dgemm(c, g);
      if (st) return st;
      continue;
    }
    const int nb1 = std::min(NB, rest);
    {
      // The next diagonal block first (rows and columns k0 + nb .. k0 + nb + nb1).
      GemmArgs g{};
      g.M = nb1; g.N = nb1; g.K = nb;
      g.A = l21; g.sam = ld; g.sak = 1;
      g.B = l21; g.sbn = ld; g.sbk = 1;
      g.C = A + (long long)(k0 + nb) * ld + k0 + nb; g.ldc = ld;
      g.alpha = -1.0; g.beta = 1.0; g.lower_only = 1; g.mode = GEMM_STORE;
      g.skip_flag = &cs->flag;
      int st = dgemm(c, g);
      if (st) return st;
    }
    if (rest > nb1) {
      // The rest of the trailing triangle (rows below the next diagonal block, columns from
      // it on) on the second stream, after the panel.
      THC_CUDA(c, cudaEventRecord(c->ev_panel, s));
      THC_CUDA(c, cudaStreamWaitEvent(s2, c->ev_panel, 0));
      GemmArgs g{};
      g.M = rest - nb1; g.N = rest; g.K = nb;
      g.A = l21 + (long long)nb1 * ld; g.sam = ld; g.sak = 1;
      g.B = l21; g.sbn = ld; g.sbk = 1;
      g.C = A + (long long)(k0 + nb + nb1) * ld + k0 + nb; g.ldc = ld;
      g.alpha = -1.0; g.beta = 1.0; g.lower_only = 1; g.lower_offset = nb1;
      g.mode = GEMM_STORE; g.no_split = 1;
      g.skip_flag = &cs->flag;
      int st;
      {
        StreamSwap on_s2(c, s2);
        st = dgemm(c, g);
      }
      if (st) return st;
      THC_CUDA(c, cudaEventRecord(c->ev_trail, s2));
      trail_pending = true;
    }
  }
  if (trail_pending) THC_CUDA(c, cudaStreamWaitEvent(s, c->ev_trail, 0));
  return THC_OK;
}

// X = L^{-1} (lower, n x n, ld) from the factor L and its inverted diagonal blocks, block row
// by block row: X_ii = dinv_i, X[i, 0:i] = -dinv_i (L[i, 0:i] X[0:i, 0:i]), with the block
// edge NB = chol_nb(n) that potrf_inv used.  T is an NB x n scratch.  Then Cinv = X^T X.
int chol_inverse(Ctx* c, const double* L, long long ld, int n, const double* dinv, double* X,
                 double* T, double* Cinv, const CholStatus* cs)
{
  ProfScope prof(c, "chol_inverse");
  cudaStream_t s = c->stream;
  THC_CUDA(c, cudaMemsetAsync(X, 0, sizeof(double) * (size_t)n * ld, s));
  const int NB = chol_nb(n);
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
    g.b_zero_below = 1;                                 // X[0:i, 0:i] is lower triangular
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
  if (!Cinv) return THC_OK;
  GemmArgs g{};
  g.M = n; g.N = n; g.K = n;                            // Cinv = X^T X
  g.A = X; g.sam = 1; g.sak = ld;
  g.B = X; g.sbn = 1; g.sbk = ld;
  g.a_zero_below = g.b_zero_below = 1;                  // X lower triangular
  g.C = Cinv; g.ldc = n;
  g.skip_flag = cs ? &cs->flag : nullptr;
  return dgemm(c, g);
}

int refine_polynomial(Ctx* c, const double* X, int n, double s, int k, double* G, double* T,
                      double* Xt)
{
  cudaStream_t st = c->stream;
  const size_t bytes = sizeof(double) * (size_t)n * n;
  int r;
  {
    GemmArgs g;                                   // G = s X X^T
    g.M = n; g.N = n; g.K = n;
    g.A = X; g.sam = n; g.sak = 1;
    g.B = X; g.sbn = n; g.sbk = 1;
    g.alpha = s;
    g.C = G; g.ldc = n;
    if ((r = dgemm(c, g))) return r;
  }
  // Horner: Xt = X + G (X + G (... X)); the last step lands in Xt.
  const double* cur = X;
  double* buf[2] = {Xt, T};
  if (k <= 0) THC_CUDA(c, cudaMemcpyAsync(Xt, X, bytes, cudaMemcpyDeviceToDevice, st));
  for (int j = 1; j <= k; j++) {
    double* dst = buf[(k - j) % 2];
    THC_CUDA(c, cudaMemcpyAsync(dst, X, bytes, cudaMemcpyDeviceToDevice, st));
    GemmArgs g;                                   // dst = X + G cur
    g.M = n; g.N = n; g.K = n;
    g.A = G; g.sam = n; g.sak = 1;
    g.B = cur; g.sbn = 1; g.sbk = n;
    g.beta = 1.0;
    g.C = dst; g.ldc = n;
    if ((r = dgemm(c, g))) return r;
    cur = dst;
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
