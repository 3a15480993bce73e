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

// One warp per row: exponent from the row maximum, then the slices of an FP64 input in
// integer arithmetic.  With e the row exponent (|x| < 2^e), X = round(x 2^{7 ns - e}) is an
// integer below 2^{7 ns} built from the IEEE bits (round half to even at the cut), and the
// slices are its signed base-128 digits S_i = round(R_i / 2^{7(ns-1-i)}), R_{i+1} = R_i -
// S_i 2^{7(ns-1-i)}, so |S_0| <= 128 and |S_i| <= 64.  Rows scaled by `scale` (optional,
// indexed c >> shift) are multiplied in FP64 first.
__device__ __forceinline__ long long fixed_point(double x, int shift_total)
{
  // round(|x| * 2^shift_total) with the sign of x; |x| * 2^shift_total < 2^62 assumed.
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

// Slices are stored pre-scaled: digit S_s as S_s 2^{-7s} (exact in BF16), so that a product
// of slices i and j carries its level's weight 2^{-7(i+j)} and the GEMM kernels need no
// per-level scaling.
__device__ __forceinline__ float slice_scale(int s) { return __int_as_float((127 - 7 * s) << 23); }

// Offset of element (slice s2, row r, column cc) in a plain (kts == 0) or tiled slice
// buffer (OzOperand).
__device__ __forceinline__ long long slice_at(int s2, long long r, long long cc, long long ldo,
                                              long long sstride, long long kts)
{
  return kts ? (cc >> 5) * kts + s2 * sstride + r * 32 + (cc & 31)
             : s2 * sstride + r * ldo + cc;
}

__global__ void slice_rows_kernel(const double* __restrict__ X, long long rows, long long cols,
                                  long long ldx, long long sc, const double* __restrict__ scale,
                                  int shift, int ns, __nv_bfloat16* out, long long ldo,
                                  long long sstride, long long kts, int* exps, long long rows_pad)
{
  long long r = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (r >= rows_pad) return;
  auto val = [&](long long cidx) -> double {
    double v = X[r * ldx + cidx * sc];
    if (scale) v *= scale[cidx >> shift];
    return v;
  };
  // Row maximum of |x| through the bit patterns (monotone for non-negative doubles).
  unsigned long long mx = 0;
  if (r < rows)
    for (long long cc = lane; cc < cols; cc += 32) {
      unsigned long long a = (unsigned long long)__double_as_longlong(val(cc)) & 0x7fffffffffffffffULL;
      mx = a > mx ? a : mx;
    }
  for (int off = 16; off; off >>= 1) {
    unsigned long long o = __shfl_xor_sync(0xffffffffu, mx, off);
    mx = o > mx ? o : mx;
  }
  // frexp exponent of the maximum: |x| < 2^e for every entry of the row.
  int e = 0;
  int Em = (int)(mx >> 52);
  if (Em > 0) e = Em - 1022;
  if (lane == 0) exps[r] = e;
  const int total = 7 * ns - e;
  for (long long cc = lane; cc < ldo; cc += 32) {
    long long R = (r < rows && cc < cols && Em > 0) ? fixed_point(val(cc), total) : 0;
    for (int s2 = 0; s2 < ns; s2++) {
      int sh = 7 * (ns - 1 - s2);
      long long S = sh ? ((R + (1LL << (sh - 1))) >> sh) : R;
      R -= S << sh;
      // |S| <= 128: convert through int32 (a 64-bit integer conversion runs on the slow
      // FP64-class path on this part).
      out[slice_at(s2, r, cc, ldo, sstride, kts)] = __float2bfloat16_rn((float)(int)S * slice_scale(s2));
    }
  }
}

// round(|x| 2^shift_total) of an FP32 value as a signed 64-bit integer (round half even).
__device__ __forceinline__ long long fixed_point_f32(float x, int shift_total)
{
  unsigned bits = __float_as_uint(x);
  int E = (int)((bits >> 23) & 0xff);
  if (E == 0) return 0;
  unsigned long long m = (bits & 0x7fffffu) | 0x800000u;
  int s = E - 150 + shift_total;
  unsigned long long X;
  if (s >= 0) {
    X = s < 40 ? m << s : 0;   // beyond 2^63: cannot occur for |x| < 2^e rows
  } else if (s <= -32) {
    X = 0;
  } else {
    int r = -s;
    unsigned long long q = m >> r;
    unsigned long long rem = m & ((1ULL << r) - 1);
    unsigned long long half = 1ULL << (r - 1);
    if (rem > half || (rem == half && (q & 1))) q++;
    X = q;
  }
  return (bits >> 31) ? -(long long)X : (long long)X;
}

// Slices of a double-word (hi, lo) matrix, one warp per row, as slice_rows_kernel: the row
// exponent comes from max |hi| (|hi + lo| < 2^e whenever |hi| < 2^e), and the fixed-point
// integer is the sum of the two parts' roundings (within one unit of the exact value).
// With kexp, column k is scaled by 2^{-kexp[k]}: a shift of the fixed-point cut, exact.
__global__ void slice_rows_dw_kernel(const float2* __restrict__ X, long long rows, long long cols,
                                     long long ldx, int ns, __nv_bfloat16* out, long long ldo,
                                     long long sstride, long long kts, int* exps,
                                     long long rows_pad, const int* __restrict__ kexp)
{
  long long r = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (r >= rows_pad) return;
  unsigned mx = 0;
  if (r < rows)
    for (long long cc = lane; cc < cols; cc += 32) {
      float h = X[r * ldx + cc].x;
      if (kexp) h = ldexpf(h, -kexp[cc]);
      unsigned a = __float_as_uint(h) & 0x7fffffffu;
      mx = a > mx ? a : mx;
    }
  for (int off = 16; off; off >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  int e = 0;
  int Em = (int)(mx >> 23);
  if (Em > 0) e = Em - 126;
  if (lane == 0) exps[r] = e;
  const int total = 7 * ns - e;
  for (long long cc = lane; cc < ldo; cc += 32) {
    long long R = 0;
    if (r < rows && cc < cols && Em > 0) {
      float2 v = X[r * ldx + cc];
      const int t = kexp ? total - kexp[cc] : total;
      R = fixed_point_f32(v.x, t) + fixed_point_f32(v.y, t);
    }
    for (int s2 = 0; s2 < ns; s2++) {
      int sh = 7 * (ns - 1 - s2);
      long long S = sh ? ((R + (1LL << (sh - 1))) >> sh) : R;
      R -= S << sh;
      out[slice_at(s2, r, cc, ldo, sstride, kts)] = __float2bfloat16_rn((float)(int)S * slice_scale(s2));
    }
  }
}

// FP32 input scaled by an FP32 copy of `scale` (rounded once to FP32, then sliced exactly
// in FP32 arithmetic).  Two passes so that long rows use the whole GPU: per-row maxima by
// column chunks (atomicMax on the bit pattern, valid for non-negative floats), then the
// slices with one thread per element.
__global__ void rowmax_f32_kernel(const float* __restrict__ X, long long rows, long long cols,
                                  long long ldx, const float* __restrict__ scale, int shift,
                                  unsigned* rowmax)
{
  long long r = blockIdx.y;
  long long c0 = (long long)blockIdx.x * 4096;
  float mx = 0.f;
  if (r < rows)
    for (long long cc = c0 + threadIdx.x; cc < cols && cc < c0 + 4096; cc += blockDim.x) {
      float v = X[r * ldx + cc];
      if (scale) v *= scale[cc >> shift];
      mx = fmaxf(mx, fabsf(v));
    }
  for (int off = 16; off; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if ((threadIdx.x & 31) == 0 && mx > 0.f) atomicMax(&rowmax[r], __float_as_uint(mx));
}

__global__ void slice_rows_f32_kernel(const float* __restrict__ X, long long rows,
                                      long long cols, long long ldx,
                                      const float* __restrict__ scale, int shift, int ns,
                                      __nv_bfloat16* out, long long ldo, long long sstride,
                                      long long kts, const unsigned* __restrict__ rowmax,
                                      int* exps)
{
  long long r = blockIdx.y;
  long long cc = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float mx = __uint_as_float(rowmax[r]);
  int e = 0;
  if (mx > 0.f) frexpf(mx, &e);
  if (cc == 0) exps[r] = e;
  if (cc >= ldo) return;
  float x = 0.f;
  if (r < rows && cc < cols) {
    float v = X[r * ldx + cc];
    if (scale) v *= scale[cc >> shift];
    x = ldexpf(v, 7 - e);
  }
  for (int s = 0; s < ns; s++) {
    float q = rintf(x);
    out[slice_at(s, r, cc, ldo, sstride, kts)] = __float2bfloat16_rn(q * slice_scale(s));
    x = (x - q) * 128.f;
  }
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

int oz_slice_rows_f64(Ctx* c, const double* X, long long rows, long long cols, long long ldx,
                      long long sc, const double* scale, int scale_shift, const SliceBuf& out)
{
  ProfScope prof(c, "slice");
  long long threads = out.rows_pad * 32;
  slice_rows_kernel<<<(unsigned)cdiv(threads, 256), 256, 0, c->stream>>>(
      X, rows, cols, ldx, sc, scale, scale_shift, out.ns, out.s, out.kpad, out.slice_stride(),
      out.kt_stride(), out.e, out.rows_pad);
  THC_LAUNCHED(c, "slice_rows_f64");
  return THC_OK;
}

int oz_slice_rows_dw(Ctx* c, const float2* X, long long rows, long long cols, long long ldx,
                     const SliceBuf& out, const int* kexp)
{
  ProfScope prof(c, "slice");
  long long threads = out.rows_pad * 32;
  slice_rows_dw_kernel<<<(unsigned)cdiv(threads, 256), 256, 0, c->stream>>>(
      X, rows, cols, ldx, out.ns, out.s, out.kpad, out.slice_stride(), out.kt_stride(), out.e,
      out.rows_pad, kexp);
  THC_LAUNCHED(c, "slice_rows_dw");
  return THC_OK;
}

int oz_slice_rows_f32(Ctx* c, const float* X, long long rows, long long cols, long long ldx,
                      const float* scale, int scale_shift, const SliceBuf& out)
{
  ProfScope prof(c, "slice");
  const long long rows_pad = out.rows_pad;
  unsigned* rowmax = (unsigned*)ws_get(c, WS_ROWMAX, sizeof(unsigned) * rows_pad);
  if (!rowmax) return set_error(c, THC_ERR_NOMEM, "slice_rows_f32: row maxima");
  THC_CUDA(c, cudaMemsetAsync(rowmax, 0, sizeof(unsigned) * rows_pad, c->stream));
  if (rows_pad > 65535) return set_error(c, THC_ERR_SHAPE, "slice_rows_f32: too many rows");
  dim3 g1((unsigned)cdiv(cols, 4096), (unsigned)rows_pad);
  rowmax_f32_kernel<<<g1, 256, 0, c->stream>>>(X, rows, cols, ldx, scale, scale_shift, rowmax);
  THC_LAUNCHED(c, "rowmax_f32");
  dim3 g2((unsigned)cdiv(out.kpad, 256), (unsigned)rows_pad);
  slice_rows_f32_kernel<<<g2, 256, 0, c->stream>>>(X, rows, cols, ldx, scale, scale_shift,
                                                   out.ns, out.s, out.kpad, out.slice_stride(),
                                                   out.kt_stride(), rowmax, out.e);
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
