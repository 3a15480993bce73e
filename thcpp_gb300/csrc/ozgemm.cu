// Sliced-BF16 GEMM with exact chunk accumulation (see ozgemm.cuh for the scheme).
//
// Warp-level BF16 MMA (m16n8k16, FP32 accumulate), 4 warps per CTA, CTA tile 64 x 32,
// warp tile 16 x 32; every level's FP32 accumulator is live for one 256-long k chunk and
// is then folded into FP64 registers.  Operands are staged through shared memory with
// cp.async (two stages) and read with ldmatrix.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "ozgemm.cuh"

namespace thc {

namespace {

// Final store of one FP64 product value under the epilogue (FP64 arithmetic: used by the
// mma.sync kernel and the split-K reduction, not on the tcgen05 fast path).
__device__ __forceinline__ void store_epilogue(const OzArgs& g, long long m, long long n, double v)
{
  if (g.epilogue == OZ_SQUARE_F64 || g.epilogue == OZ_SQUARE_DW) v = v * v;
  if (g.epilogue == OZ_STORE_F32) {
    ((float*)g.C)[m * g.ldc + n] = (float)v;
  } else if (g.epilogue == OZ_SQUARE_DW || g.epilogue == OZ_STORE_DW) {
    float hi = (float)v;
    ((float2*)g.C)[m * g.ldc + n] = make_float2(hi, (float)(v - (double)hi));
  } else {
    ((double*)g.C)[m * g.ldc + n] = v;
  }
}

constexpr int OBM = 64, OBN = 32, OBK = 32, OCHUNK = 256, OPAD = 8;
constexpr int OLDA = OBK + OPAD;      // shared row length (bf16) of A and k-contiguous B
constexpr int OLDBN = OBN + OPAD;     // shared row length of n-contiguous B

__device__ __forceinline__ unsigned smem_u32(const void* p)
{
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(smem)), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }

__device__ __forceinline__ void ldsm_x4(unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3,
                                        const void* p)
{
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3,
                                          const void* p)
{
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16(float* d, const unsigned* a, unsigned b0, unsigned b1)
{
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ double pow2(int e)
{
  // 2^e for the normal range; outside it fall back to ldexp.
  if (e > -1022 && e < 1023) return __longlong_as_double((long long)(e + 1023) << 52);
  return ldexp(1.0, e);
}

template <int LV, bool BK>
__global__ void __launch_bounds__(128, 2) ozgemm_kernel(OzArgs g)
{
  const long long m0 = (long long)blockIdx.x * OBM;
  const long long n0 = (long long)blockIdx.y * OBN;
  if (g.lower_only && n0 > m0 + OBM - 1) return;
  extern __shared__ __align__(16) unsigned char smem[];
  const int a_stage = LV * OBM * OLDA;                       // bf16 elements per stage
  const int b_stage = BK ? LV * OBN * OLDA : LV * OBK * OLDBN;
  __nv_bfloat16* sA = (__nv_bfloat16*)smem;
  __nv_bfloat16* sB = sA + 2 * a_stage;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  auto load_stage = [&](int buf, long long k0) {
    __nv_bfloat16* dA = sA + buf * a_stage;
    __nv_bfloat16* dB = sB + buf * b_stage;
#pragma unroll
    for (int s = 0; s < LV; s++) {
      // Row stride and first element of this slice's k tile (plain or tiled storage).
      const long long lda = g.a.kt_stride ? 32 : g.a.ld;
      const __nv_bfloat16* ga = g.a.s + (g.a.kt_stride ? (k0 >> 5) * g.a.kt_stride + s * g.a.slice_stride + m0 * 32
                                                       : s * g.a.slice_stride + m0 * g.a.ld + k0);
#pragma unroll
      for (int r = 0; r < 2; r++) {
        int ch = tid + 128 * r;        // 256 chunks of 16 B: 64 rows x 4
        int row = ch >> 2, col = (ch & 3) * 8;
        cp_async16(dA + (s * OBM + row) * OLDA + col, ga + row * lda + col);
      }
      if (BK) {
        const long long ldb = g.b.kt_stride ? 32 : g.b.ld;
        const __nv_bfloat16* gb = g.b.s + (g.b.kt_stride ? (k0 >> 5) * g.b.kt_stride + s * g.b.slice_stride + n0 * 32
                                                         : s * g.b.slice_stride + n0 * g.b.ld + k0);
        int row = tid >> 2, col = (tid & 3) * 8;   // 32 rows (n) x 4 chunks
        cp_async16(dB + (s * OBN + row) * OLDA + col, gb + row * ldb + col);
      } else {
        const __nv_bfloat16* gb = g.b.s + s * g.b.slice_stride + k0 * g.b.ld + n0;
        int row = tid >> 2, col = (tid & 3) * 8;   // 32 rows (k) x 4 chunks
        cp_async16(dB + (s * OBK + row) * OLDBN + col, gb + row * g.b.ld + col);
      }
    }
    cp_async_commit();
  };

  double acc64[4][4];
#pragma unroll
  for (int t = 0; t < 4; t++)
#pragma unroll
    for (int q = 0; q < 4; q++) acc64[t][q] = 0.0;
  float acc[LV][4][4];

  long long kbeg = 0, kend = g.K;
  if (g.ksplit > 1) {
    long long kc = ((g.K + g.ksplit - 1) / g.ksplit + 511) / 512 * 512;
    kbeg = blockIdx.z * kc;
    kend = kbeg + kc < g.K ? kbeg + kc : g.K;
  }
  const long long K = kend - kbeg;
  long long nsteps = K > 0 ? (K + OBK - 1) / OBK : 0;
  if (nsteps > 0) load_stage(0, kbeg);
  int buf = 0;
  for (long long st = 0; st < nsteps; st++) {
    if ((st * OBK) % OCHUNK == 0) {
#pragma unroll
      for (int l = 0; l < LV; l++)
#pragma unroll
        for (int t = 0; t < 4; t++)
#pragma unroll
          for (int q = 0; q < 4; q++) acc[l][t][q] = 0.f;
    }
    cp_async_wait_all();
    __syncthreads();
    if (st + 1 < nsteps) load_stage(buf ^ 1, kbeg + (st + 1) * OBK);
    const __nv_bfloat16* cA = sA + buf * a_stage;
    const __nv_bfloat16* cB = sB + buf * b_stage;
#pragma unroll
    for (int kk = 0; kk < OBK; kk += 16) {
      unsigned af[LV][4];
#pragma unroll
      for (int s = 0; s < LV; s++) {
        const __nv_bfloat16* p = cA + (s * OBM + warp * 16 + (lane & 15)) * OLDA + kk + (lane >> 4) * 8;
        ldsm_x4(af[s][0], af[s][1], af[s][2], af[s][3], p);
      }
#pragma unroll
      for (int j = 0; j < LV; j++) {
        unsigned bf[4][2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
          unsigned r0, r1, r2, r3;
          if (BK) {
            int nrow = h * 16 + (lane >> 4) * 8 + (lane & 7);
            int kof = kk + ((lane >> 3) & 1) * 8;
            ldsm_x4(r0, r1, r2, r3, cB + (j * OBN + nrow) * OLDA + kof);
          } else {
            int krow = kk + ((lane >> 3) & 1) * 8 + (lane & 7);
            int nof = h * 16 + (lane >> 4) * 8;
            ldsm_x4_t(r0, r1, r2, r3, cB + (j * OBK + krow) * OLDBN + nof);
          }
          bf[2 * h][0] = r0; bf[2 * h][1] = r1;
          bf[2 * h + 1][0] = r2; bf[2 * h + 1][1] = r3;
        }
#pragma unroll
        for (int i = 0; i + j < LV; i++)
#pragma unroll
          for (int t = 0; t < 4; t++) mma_bf16(acc[i + j][t], af[i], bf[t][0], bf[t][1]);
      }
    }
    if (((st + 1) * OBK) % OCHUNK == 0 || st + 1 == nsteps) {
#pragma unroll
      for (int l = 0; l < LV; l++) {
        // Slices are stored pre-scaled, so every level is already in the final units.
#pragma unroll
        for (int t = 0; t < 4; t++)
#pragma unroll
          for (int q = 0; q < 4; q++) acc64[t][q] = __dadd_rn((double)acc[l][t][q], acc64[t][q]);
      }
    }
    buf ^= 1;
  }
  // Epilogue: thread holds rows (g, g+8) x cols (2t, 2t+1) of each n8 tile.
  const int gr = lane >> 2, tc = (lane & 3) * 2;
#pragma unroll
  for (int t = 0; t < 4; t++) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      long long m = m0 + warp * 16 + gr + (q >= 2 ? 8 : 0);
      long long n = n0 + t * 8 + tc + (q & 1);
      if (m >= g.M || n >= g.N) continue;
      if (g.lower_only && n > m) continue;
      double v = acc64[t][q] * pow2(g.a.e[m] + g.b.e[n] - 14);
      if (g.ksplit > 1) {
        g.part[((long long)blockIdx.z * g.M + m) * g.N + n] = v;
        continue;
      }
      store_epilogue(g, m, n, v);
    }
  }
}

template <int LV>
int launch_lv(Ctx* c, const OzArgs& g)
{
  size_t a_stage = (size_t)LV * OBM * OLDA;
  size_t b_stage = g.b.k_contig ? (size_t)LV * OBN * OLDA : (size_t)LV * OBK * OLDBN;
  size_t smem = 2 * (a_stage + b_stage) * sizeof(__nv_bfloat16);
  dim3 grid((unsigned)cdiv(g.M, OBM), (unsigned)cdiv(g.N, OBN), (unsigned)std::max(1, g.ksplit));
  if (grid.y > 65535) return set_error(c, THC_ERR_SHAPE, "ozgemm: N too large");
  ProfScope prof(c, "ozgemm");
  ProfScope prof_tag(g.tag ? c : nullptr, g.tag ? g.tag : "");
  if (g.b.k_contig) {
    THC_CUDA(c, cudaFuncSetAttribute(ozgemm_kernel<LV, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    ozgemm_kernel<LV, true><<<grid, 128, smem, c->stream>>>(g);
  } else {
    THC_CUDA(c, cudaFuncSetAttribute(ozgemm_kernel<LV, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    ozgemm_kernel<LV, false><<<grid, 128, smem, c->stream>>>(g);
  }
  THC_LAUNCHED(c, "ozgemm");
  if (g.ksplit > 1) return oz_split_reduce(c, g);
  return THC_OK;
}

__global__ void oz_reduce_kernel(OzArgs g)
{
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= g.M * g.N) return;
  long long m = e / g.N, n = e % g.N;
  if (g.lower_only && n > m) return;
  double v = 0.0;
  for (int z = 0; z < g.ksplit; z++) v += g.part[((long long)z * g.M + m) * g.N + n];
  store_epilogue(g, m, n, v);
}

// Slicing.  A row's entries are cut relative to the row exponent e (|x| < 2^e for every
// entry, from the row maximum) into ns signed base-128 digits,
//     x = 2^{e-7} sum_{i<ns} S_i 2^{-7i},
// computed in 32-bit arithmetic: with nh = min(ns, 3) and nl = ns - nh, the scaled value
// a = x 2^{7 nh - e} (|a| < 2^{7 nh}) gives A = rint(a) and, from the exact remainder
// a - A (plus the low word of a double-word input), B = rint((a - A + a_lo) 2^{7 nl}); A
// and B are integers below 2^21 held exactly in FP32 and are split into nh and nl
// balanced digits by exact power-of-two divisions and rint.  |S_0| <= 128, |S_1|, |S_2| <=
// 64, |S_3| <= 72, |S_4|, |S_5| <= 64, all exact in BF16, and the expansion is within
// 0.57 units of the last digit of x.  Each lane cuts eight consecutive columns, so every
// slice is written as one 16-byte store per lane (the eight columns lie in one 32-wide k
// tile of the tiled layout).

// Slices are stored pre-scaled: digit S_s as S_s 2^{-7s} (exact in BF16), so that a product
// of slices i and j carries its level's weight 2^{-7(i+j)} and the GEMM kernels need no
// per-level scaling.
__device__ __forceinline__ float slice_scale(int s) { return __int_as_float((127 - 7 * s) << 23); }

// 2^e as an FP32 value, for -126 <= e <= 127.
__device__ __forceinline__ float pow2_f32(int e) { return __int_as_float((e + 127) << 23); }

// x * 2^e, exact whenever the result is a normal number (one multiply in range, else ldexpf).
__device__ __forceinline__ float scale2(float x, int e)
{
  return (e >= -126 && e <= 127) ? __fmul_rn(x, pow2_f32(e)) : ldexpf(x, e);
}

// N balanced base-128 digits of an integer |x| <= 2^{7N} + 2^{7N-4} held in FP32.
template <int N>
__device__ __forceinline__ void int_digits(float x, float* d)
{
#pragma unroll
  for (int i = 0; i < N; i++) {
    const int sh = 7 * (N - 1 - i);
    if (sh) {
      const float q = rintf(__fmul_rn(x, pow2_f32(-sh)));
      x = __fmaf_rn(-q, pow2_f32(sh), x);   // exact: an integer below 2^24
      d[i] = q;
    } else {
      d[i] = x;
    }
  }
}

// The NS digits of a (scaled by 2^{7 nh - e}) with low word al.
template <int NS>
__device__ __forceinline__ void value_digits(float a, float al, float* d)
{
  constexpr int NH = NS < 3 ? NS : 3, NL = NS - NH;
  const float A = rintf(a);
  int_digits<NH>(A, d);
  if (NL) {
    const float B = rintf(__fmul_rn(__fadd_rn(__fsub_rn(a, A), al), pow2_f32(7 * NL)));
    int_digits<NL>(B, d + NH);
  }
}

// Offset of element (slice s2, row r, column cc) in a plain (kts == 0) or tiled slice
// buffer (OzOperand).
__device__ __forceinline__ long long slice_at(int s2, long long r, long long cc, long long ldo,
                                              long long sstride, long long kts)
{
  return kts ? (cc >> 5) * kts + s2 * sstride + r * 32 + (cc & 31)
             : s2 * sstride + r * ldo + cc;
}

// Columns c..c+7 (c a multiple of 8) of row r, every slice: one 16-byte store per slice.
template <int NS>
__device__ __forceinline__ void store_digits8(__nv_bfloat16* out, long long r, long long c,
                                              long long ldo, long long sstride, long long kts,
                                              const float (&d)[8][NS])
{
#pragma unroll
  for (int s2 = 0; s2 < NS; s2++) {
    const float sc = slice_scale(s2);
    __nv_bfloat162 p[4];
#pragma unroll
    for (int q = 0; q < 4; q++)
      p[q] = __floats2bfloat162_rn(__fmul_rn(d[2 * q][s2], sc), __fmul_rn(d[2 * q + 1][s2], sc));
    *(uint4*)(out + slice_at(s2, r, c, ldo, sstride, kts)) = *(const uint4*)p;
  }
}

// round(|x| * 2^shift_total) of an FP64 value with the sign of x, from the IEEE bits (round
// half to even); |x| * 2^shift_total < 2^62 assumed.
__device__ __forceinline__ long long fixed_point(double x, int shift_total)
{
  unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  int E = (int)((bits >> 52) & 0x7ff);
  if (E == 0) return 0;                              // zero or subnormal: below every slice
  unsigned long long m = (bits & 0xfffffffffffffULL) | (1ULL << 52);
  int s = E - 1075 + shift_total;
  unsigned long long X;
  if (s >= 0) {
    X = m << s;
  } else if (s <= -64) {
    X = 0;
  } else {
    int r = -s;
    unsigned long long q = m >> r;
    unsigned long long rem = m & ((1ULL << r) - 1);
    unsigned long long half = 1ULL << (r - 1);
    if (rem > half || (rem == half && (q & 1))) q++;
    X = q;
  }
  return (bits >> 63) ? -(long long)X : (long long)X;
}

// Lanes per row of the row-per-warp slicers: a power of two with 8 columns per lane, so
// that short rows (N_o = 32 orbitals: four lanes) share a warp with other rows.
inline int slice_lanes_per_row(long long ldo)
{
  int l = 32;
  while (l > 4 && 8LL * l > ldo) l >>= 1;
  return l;
}

// FP64 input, LPR lanes per row (32 / LPR rows per warp).  The FP64 value is taken to the
// fixed-point integer R = round(x 2^{7 ns - e}) (|R| <= 2^{7 ns}) in integer arithmetic on
// its bits (no FP64 arithmetic on this part's slow FP64 pipe), then R = A 2^{7 nl} + B with
// FP32-exact A, B and the same digit split as above.  Rows scaled by `scale` (optional,
// indexed c >> shift) are multiplied in FP64 first.  Element (r, c) is X[r * ldx + c * sc].
template <int NS>
__global__ void __launch_bounds__(256) slice_rows_kernel(
    const double* __restrict__ X, long long rows, long long cols, long long ldx, long long sc,
    const double* __restrict__ scale, int shift, __nv_bfloat16* out, long long ldo,
    long long sstride, long long kts, int* exps, long long rows_pad, int lpr)
{
  constexpr int NH = NS < 3 ? NS : 3, NL = NS - NH;
  const int lane = threadIdx.x & 31, sub = lane & (lpr - 1);
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long r0 = warp * (32 / lpr);
  if (r0 >= rows_pad) return;                        // whole warp
  const long long r = r0 + lane / lpr;
  const bool live_row = r < rows;
  auto val = [&](long long cidx) -> double {
    double v = X[r * ldx + cidx * sc];
    if (scale) v *= scale[cidx >> shift];
    return v;
  };
  // Row maximum of |x| through the bit patterns (monotone for non-negative doubles).
  unsigned long long mx = 0;
  if (live_row)
    for (long long cc = sub; cc < cols; cc += lpr) {
      unsigned long long a = (unsigned long long)__double_as_longlong(val(cc)) & 0x7fffffffffffffffULL;
      mx = a > mx ? a : mx;
    }
  for (int off = lpr >> 1; off; off >>= 1) {
    unsigned long long o = __shfl_xor_sync(0xffffffffu, mx, off);
    mx = o > mx ? o : mx;
  }
  if (r >= rows_pad) return;                         // after the warp's shuffles
  // frexp exponent of the maximum: |x| < 2^e for every entry of the row.
  int e = 0;
  const int Em = (int)(mx >> 52);
  if (Em > 0) e = Em - 1022;
  if (sub == 0) exps[r] = e;
  const int total = 7 * NS - e;
  for (long long c0 = 8 * sub; c0 < ldo; c0 += 8 * lpr) {
    float d[8][NS];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const long long cc = c0 + j;
      const long long R = (live_row && cc < cols && Em > 0) ? fixed_point(val(cc), total) : 0;
      // A = round(R / 2^{7 nl}), B = R - A 2^{7 nl}: |A| <= 2^{7 nh}, |B| <= 2^{7 nl - 1}.
      const long long A = NL ? (R + (1LL << (7 * NL - 1))) >> (7 * NL) : R;
      int_digits<NH>((float)(int)A, d[j]);
      if (NL) int_digits<NL>((float)(int)(R - (A << (7 * NL))), d[j] + NH);
    }
    store_digits8<NS>(out, r, c0, ldo, sstride, kts, d);
  }
}

// Eight consecutive double-word entries (columns c..c+7) of a row; entries at or past
// `cols` read as zero.  vec: the row is 16-byte aligned and c + 8 <= cols.
__device__ __forceinline__ void load_dw8(const float2* __restrict__ row, long long c,
                                         long long cols, bool vec, float2 (&v)[8])
{
  if (vec && c + 8 <= cols) {
    const float4* p = (const float4*)(row + c);
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const float4 t = __ldg(p + q);
      v[2 * q] = make_float2(t.x, t.y);
      v[2 * q + 1] = make_float2(t.z, t.w);
    }
  } else {
#pragma unroll
    for (int j = 0; j < 8; j++) v[j] = c + j < cols ? __ldg(row + c + j) : make_float2(0.f, 0.f);
  }
}

// Slices of a double-word (hi, lo) matrix, LPR lanes per row: the row exponent comes from
// max |hi| (|hi + lo| < 2^e whenever |hi| < 2^e), and a = hi 2^{7 nh - e}, a_lo = lo
// 2^{7 nh - e} feed the digit split above.  With kexp, column k is scaled by 2^{-kexp[k]}
// (an exact shift of the cut).  Rows of at most 8 LPR entries are read once and kept in
// registers between the two passes.
template <int NS>
__global__ void __launch_bounds__(256, 3) slice_rows_dw_kernel(
    const float2* __restrict__ X, long long rows, long long cols, long long ldx,
    __nv_bfloat16* out, long long ldo, long long sstride, long long kts, int* exps,
    long long rows_pad, const int* __restrict__ kexp, bool vec, int lpr)
{
  constexpr int NH = NS < 3 ? NS : 3;
  const int lane = threadIdx.x & 31, sub = lane & (lpr - 1);
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long r0 = warp * (32 / lpr);
  if (r0 >= rows_pad) return;                        // whole warp
  const long long r = r0 + lane / lpr;
  const float2* row = X + (r < rows ? r : 0) * ldx;
  const long long ncols = r < rows ? cols : 0;
  const bool one = ldo <= 8 * lpr;   // a single chunk of eight columns per lane
  float2 keep[8];
  unsigned mx = 0;
  for (long long c0 = 8 * sub; c0 < ncols; c0 += 8 * lpr) {
    float2 v[8];
    load_dw8(row, c0, ncols, vec, v);
#pragma unroll
    for (int j = 0; j < 8; j++) {
      float h = v[j].x;
      if (kexp && c0 + j < ncols) h = scale2(h, -__ldg(kexp + c0 + j));
      mx = max(mx, __float_as_uint(h) & 0x7fffffffu);
      if (one) keep[j] = v[j];
    }
  }
  for (int off = lpr >> 1; off; off >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if (r >= rows_pad) return;                         // after the warp's shuffles
  int e = 0;
  const int Em = (int)(mx >> 23);
  if (Em > 0) e = Em - 126;
  if (sub == 0) exps[r] = e;
  const int sh0 = 7 * NH - e;
  for (long long c0 = 8 * sub; c0 < ldo; c0 += 8 * lpr) {
    float2 v[8];
    if (one && c0 < ncols) {
#pragma unroll
      for (int j = 0; j < 8; j++) v[j] = keep[j];
    } else {
      load_dw8(row, c0, ncols, vec, v);
    }
    float d[8][NS];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const bool live = Em > 0 && c0 + j < ncols;
      const int sh = kexp && live ? sh0 - __ldg(kexp + c0 + j) : sh0;
      const float a = live ? scale2(v[j].x, sh) : 0.f;
      const float al = live ? scale2(v[j].y, sh) : 0.f;
      value_digits<NS>(a, al, d[j]);
    }
    store_digits8<NS>(out, r, c0, ldo, sstride, kts, d);
  }
}

// Eight consecutive FP32 entries (columns c..c+7) of a row times their scales; entries at
// or past `cols` read as zero.  vec: 16-byte aligned row and ldx a multiple of 4.
__device__ __forceinline__ void load_f32x8(const float* __restrict__ row, long long c,
                                           long long cols, bool vec,
                                           const float* __restrict__ scale, int shift,
                                           float (&v)[8])
{
  if (vec && c + 8 <= cols) {
    const float4 t0 = __ldg((const float4*)(row + c)), t1 = __ldg((const float4*)(row + c) + 1);
    v[0] = t0.x; v[1] = t0.y; v[2] = t0.z; v[3] = t0.w;
    v[4] = t1.x; v[5] = t1.y; v[6] = t1.z; v[7] = t1.w;
  } else {
#pragma unroll
    for (int j = 0; j < 8; j++) v[j] = c + j < cols ? __ldg(row + c + j) : 0.f;
  }
  if (scale) {
#pragma unroll
    for (int j = 0; j < 8; j++)
      if (c + j < cols) v[j] = __fmul_rn(v[j], __ldg(scale + ((c + j) >> shift)));
  }
}

// FP32 input scaled by an FP32 copy of `scale` (rounded once to FP32, then sliced exactly
// in FP32 arithmetic).  Two passes so that long rows use the whole GPU: per-row maxima by
// column chunks of 4096 (atomicMax on the bit pattern, valid for non-negative floats), then
// the slices, eight columns per thread.
__global__ void __launch_bounds__(256) rowmax_f32_kernel(
    const float* __restrict__ X, long long rows, long long cols, long long ldx,
    const float* __restrict__ scale, int shift, unsigned* rowmax, bool vec)
{
  const long long r = blockIdx.y;
  if (r >= rows) return;
  const float* row = X + r * ldx;
  float mx = 0.f;
  const long long c1 = min(cols, (long long)(blockIdx.x + 1) * 4096);
  for (long long c = (long long)blockIdx.x * 4096 + 8 * threadIdx.x; c < c1; c += 2048) {
    float v[8];
    load_f32x8(row, c, c1, vec, scale, shift, v);
#pragma unroll
    for (int j = 0; j < 8; j++) mx = fmaxf(mx, fabsf(v[j]));
  }
  for (int off = 16; off; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if ((threadIdx.x & 31) == 0 && mx > 0.f) atomicMax(&rowmax[r], __float_as_uint(mx));
}

template <int NS>
__global__ void __launch_bounds__(256) slice_rows_f32_kernel(
    const float* __restrict__ X, long long rows, long long cols, long long ldx,
    const float* __restrict__ scale, int shift, __nv_bfloat16* out, long long ldo,
    long long sstride, long long kts, const unsigned* __restrict__ rowmax, int* exps, bool vec)
{
  constexpr int NH = NS < 3 ? NS : 3;
  const long long r = blockIdx.y;
  const long long c0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 8;
  const float mx = __uint_as_float(rowmax[r]);
  int e = 0;
  if (mx > 0.f) frexpf(mx, &e);
  if (c0 == 0) exps[r] = e;
  if (c0 >= ldo) return;
  const long long ncols = r < rows ? cols : 0;
  float v[8];
  load_f32x8(X + (r < rows ? r : 0) * ldx, c0, ncols, vec, scale, shift, v);
  const int sh = 7 * NH - e;
  float d[8][NS];
#pragma unroll
  for (int j = 0; j < 8; j++) value_digits<NS>(mx > 0.f ? scale2(v[j], sh) : 0.f, 0.f, d[j]);
  store_digits8<NS>(out, r, c0, ldo, sstride, kts, d);
}

}  // namespace

int oz_choose_split(long long M, long long N, long long K, bool lower)
{
  // Tiles of the tensor-core kernel (128 x 128); with `lower`, those on or below the
  // diagonal.  Modelled time of a split k: waves x (k range per CTA, in whole 512-k chunks,
  // + ~256 k worth of prologue and epilogue); the FP64 partials (k M N doubles) stay below
  // 4 GB.
  const long long mt = cdiv(M, 128), nt = cdiv(N, 128);
  const long long tiles = lower ? mt * (mt + 1) / 2 : mt * nt;
  const long long chunks = (long long)cdiv(K, 512);
  const long long kmem = std::max(1LL, (4LL << 30) / std::max(1LL, 8 * M * N));
  const long long maxk = std::max(1LL, std::min(std::min(chunks, kmem), 1024LL));
  long long best_k = 1;
  double best_t = 0.0;
  for (long long k = 1; k <= maxk; k++) {
    const long long per = (long long)cdiv(chunks, k) * 512;
    const double t = (double)cdiv(tiles * k, 152) * (double)(per + 256);
    if (k == 1 || t < best_t) { best_t = t; best_k = k; }
  }
  return (int)best_k;
}

int oz_split_reduce(Ctx* c, const OzArgs& g)
{
  ProfScope prof(c, "oz_split_reduce");
  oz_reduce_kernel<<<(unsigned)cdiv(g.M * g.N, 256), 256, 0, c->stream>>>(g);
  THC_LAUNCHED(c, "oz_split_reduce");
  return THC_OK;
}

// Dispatch of a slicing kernel on the slice count (2..6); ARGS is the parenthesised
// argument list.
#define OZ_SLICE_DISPATCH(ns, KERNEL, GRID, ARGS)                                    \
  switch (ns) {                                                                     \
    case 2: KERNEL<2><<<GRID, 256, 0, c->stream>>> ARGS; break;                     \
    case 3: KERNEL<3><<<GRID, 256, 0, c->stream>>> ARGS; break;                     \
    case 4: KERNEL<4><<<GRID, 256, 0, c->stream>>> ARGS; break;                     \
    case 5: KERNEL<5><<<GRID, 256, 0, c->stream>>> ARGS; break;                     \
    case 6: KERNEL<6><<<GRID, 256, 0, c->stream>>> ARGS; break;                     \
    default: return set_error(c, THC_ERR_ARG, "slicing: slice count must be 2..6");  \
  }

int oz_slice_rows_f64(Ctx* c, const double* X, long long rows, long long cols, long long ldx,
                      long long sc, const double* scale, int scale_shift, const SliceBuf& out)
{
  ProfScope prof(c, "slice");
  if (out.kpad % 32) return set_error(c, THC_ERR_ARG, "slicing: padded K must be a multiple of 32");
  const int lpr = slice_lanes_per_row(out.kpad);
  const unsigned blocks = (unsigned)cdiv(cdiv(out.rows_pad, 32 / lpr) * 32, 256);
  OZ_SLICE_DISPATCH(out.ns, slice_rows_kernel, blocks,
                    (X, rows, cols, ldx, sc, scale, scale_shift, out.s, out.kpad,
                     out.slice_stride(), out.kt_stride(), out.e, out.rows_pad, lpr))
  THC_LAUNCHED(c, "slice_rows_f64");
  return THC_OK;
}

int oz_slice_rows_dw(Ctx* c, const float2* X, long long rows, long long cols, long long ldx,
                     const SliceBuf& out, const int* kexp)
{
  ProfScope prof(c, "slice");
  if (out.kpad % 32) return set_error(c, THC_ERR_ARG, "slicing: padded K must be a multiple of 32");
  const int lpr = slice_lanes_per_row(out.kpad);
  const unsigned blocks = (unsigned)cdiv(cdiv(out.rows_pad, 32 / lpr) * 32, 256);
  const bool vec = (ldx % 2 == 0) && ((uintptr_t)X % 16 == 0);
  OZ_SLICE_DISPATCH(out.ns, slice_rows_dw_kernel, blocks,
                    (X, rows, cols, ldx, out.s, out.kpad, out.slice_stride(), out.kt_stride(),
                     out.e, out.rows_pad, kexp, vec, lpr))
  THC_LAUNCHED(c, "slice_rows_dw");
  return THC_OK;
}

int oz_slice_rows_f32(Ctx* c, const float* X, long long rows, long long cols, long long ldx,
                      const float* scale, int scale_shift, const SliceBuf& out)
{
  ProfScope prof(c, "slice");
  if (out.kpad % 32) return set_error(c, THC_ERR_ARG, "slicing: padded K must be a multiple of 32");
  const long long rows_pad = out.rows_pad;
  unsigned* rowmax = (unsigned*)ws_get(c, WS_ROWMAX, sizeof(unsigned) * rows_pad);
  if (!rowmax) return set_error(c, THC_ERR_NOMEM, "slice_rows_f32: row maxima");
  THC_CUDA(c, cudaMemsetAsync(rowmax, 0, sizeof(unsigned) * rows_pad, c->stream));
  if (rows_pad > 65535) return set_error(c, THC_ERR_SHAPE, "slice_rows_f32: too many rows");
  const bool vec = (ldx % 4 == 0) && ((uintptr_t)X % 16 == 0);
  dim3 g1((unsigned)cdiv(cols, 4096), (unsigned)rows_pad);
  rowmax_f32_kernel<<<g1, 256, 0, c->stream>>>(X, rows, cols, ldx, scale, scale_shift, rowmax, vec);
  THC_LAUNCHED(c, "rowmax_f32");
  dim3 g2((unsigned)cdiv(out.kpad, 8 * 256), (unsigned)rows_pad);
  OZ_SLICE_DISPATCH(out.ns, slice_rows_f32_kernel, g2,
                    (X, rows, cols, ldx, scale, scale_shift, out.s, out.kpad, out.slice_stride(),
                     out.kt_stride(), rowmax, out.e, vec))
  THC_LAUNCHED(c, "slice_rows_f32");
  return THC_OK;
}

int ozgemm(Ctx* c, const OzArgs& g)
{
  if (g.M <= 0 || g.N <= 0) return THC_OK;
  if (!g.b.k_contig && g.b.kt_stride)
    return set_error(c, THC_ERR_ARG, "ozgemm: tiled B must be K-contiguous");
  switch (g.levels) {
    case 2: return launch_lv<2>(c, g);
    case 3: return launch_lv<3>(c, g);
    case 4: return launch_lv<4>(c, g);
    case 5: return launch_lv<5>(c, g);
    case 6: return launch_lv<6>(c, g);
    case 7: return launch_lv<7>(c, g);
    default: return set_error(c, THC_ERR_ARG, "ozgemm: levels must be 2..7");
  }
}

}  // namespace thc
