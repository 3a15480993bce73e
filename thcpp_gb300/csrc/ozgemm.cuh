// Error-free sliced-BF16 GEMM ("Ozaki"-style splitting onto BF16 tensor cores).
//
// Each row of A (each column of B) is scaled by a power of two 2^e so that its entries lie
// in (-1, 1), then split into s integer slices of 7 bits:
//     x = 2^e * sum_{i<s} S_i 2^{-7(i+1)},  |S_0| <= 128, |S_3| <= 72, |S_i| <= 64 otherwise,
// every slice exactly representable in BF16 and stored pre-scaled as S_i 2^{-7i}.  The
// product keeps the slice pairs with i + j <= L (L = s - 1):
//     C[m,n] = 2^{eA[m] + eB[n] - 14} sum_{l<=L} sum_{i+j=l} sum_k (S_i 2^{-7i})[m,k] (T_j 2^{-7j})[k,n].
// Every slice product of level l is an integer multiple of 2^{-7l} below 2^{14-7l} in
// magnitude (levels 0-2 use digits 0-2 only) and every level sum over a chunk of 256 k (512
// on the tensor-core kernel, for levels 0-2) such a multiple below 2^{24-7l}, so the tensor
// cores' FP32 accumulation of a chunk is exact; chunks are combined in FP64.  The only error is the truncation of the
// slice expansion, about (L+2) 2^{-7(L+1)} relative to sum_k |A||B|.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace thc {

// OZ_SQUARE_DW stores the squared product as a double-word FP32 pair (float2 {hi, lo},
// hi + lo carrying ~46 bits), which needs no FP64 arithmetic in the epilogue.
// OZ_STORE_DW stores the product itself as such a pair.
enum OzEpilogue : int {
  OZ_STORE_F64 = 0, OZ_SQUARE_F64 = 1, OZ_STORE_F32 = 2, OZ_SQUARE_DW = 3, OZ_STORE_DW = 4
};

// Slice storage.  Plain: element (slice s, row r, k) at s*slice_stride + r*ld + k.
// Tiled (kt_stride > 0): at (k/32)*kt_stride + s*slice_stride + r*32 + k%32, i.e.
// [k/32][slice][row][32]: the 32-wide k tile of a block of rows is one contiguous run of
// memory, so a tile load reads whole DRAM pages instead of 64-byte pieces of rows that lie
// kilobytes (for the Coulomb product's 1.28e6-long rows, megabytes) apart.
struct OzOperand {
  const __nv_bfloat16* s = nullptr;  // slices
  const int* e = nullptr;            // exponent per row (A) / per column (B)
  long long ld = 0;                  // plain: elements between rows; both: padded K
  long long slice_stride = 0;        // elements between slices (tiled: within one k tile)
  long long kt_stride = 0;           // tiled: elements between k tiles; 0 = plain
  bool k_contig = true;              // B only: true for [n][k] storage, false for [k][n]
};

struct OzArgs {
  long long M = 0, N = 0, K = 0;     // logical sizes; slice buffers are zero padded to
                                     // multiples of the tile sizes (64 in M/N, 32 in K)
  OzOperand a, b;
  int levels = 5;                    // L + 1 = number of slices used
  int epilogue = OZ_STORE_F64;
  void* C = nullptr;
  long long ldc = 0;
  int lower_only = 0;
  int ksplit = 1;                    // > 1: K split over blockIdx.z (multiples of 512)
  double* part = nullptr;            // ksplit x M x N FP64 partials (scaled, pre-epilogue)
  const char* tag = nullptr;         // profile name of this product (besides "ozgemm")
};

// Number of k-splits that fills the GPU for an M x N output with long K (chunk = 512).
int oz_choose_split(long long M, long long N, long long K, bool lower);
// part[z] summed in split order, then the epilogue, into C.
int oz_split_reduce(Ctx* c, const OzArgs& g);

// Padded sizes expected by both sliced-GEMM kernels for the slice buffers.
inline long long oz_pad_mn(long long x) { return (x + 127) / 128 * 128; }
inline long long oz_pad_k(long long x) { return (x + 31) / 32 * 32; }

// Destination of a slicing call: ns slices of a rows_pad x kpad matrix (kpad a multiple
// of 32) and one exponent per row, plain or tiled (see OzOperand); ns * rows_pad * kpad
// elements either way.
struct SliceBuf {
  __nv_bfloat16* s = nullptr;
  int* e = nullptr;
  long long rows_pad = 0, kpad = 0;
  int ns = 0;
  bool tiled = false;
  long long slice_stride() const { return tiled ? rows_pad * 32 : rows_pad * kpad; }
  long long kt_stride() const { return tiled ? (long long)ns * rows_pad * 32 : 0; }
  OzOperand operand() const
  {
    OzOperand o;
    o.s = s; o.e = e; o.ld = kpad; o.slice_stride = slice_stride(); o.kt_stride = kt_stride();
    o.k_contig = true;
    return o;
  }
};

// Slice rows of a matrix X (rows x cols, element (r, c) at X[r*ldx + c*sc]) into
// out[slice][r][c] (row length ldo, padded entries zero) with one exponent per row.
// `scale` (optional, length cols, indexed c >> scale_shift) multiplies entries first.
int oz_slice_rows_f64(Ctx* c, const double* X, long long rows, long long cols, long long ldx,
                      long long sc, const double* scale, int scale_shift, const SliceBuf& out);
// Slices of a double-word matrix (float2 {hi, lo} entries, row-major, ld = ldx).
// kexp (optional, one per column): column k is scaled by 2^{-kexp[k]} first (exact).
int oz_slice_rows_dw(Ctx* c, const float2* X, long long rows, long long cols, long long ldx,
                     const SliceBuf& out, const int* kexp = nullptr);
int oz_slice_rows_f32(Ctx* c, const float* X, long long rows, long long cols, long long ldx,
                      const float* scale, int scale_shift, const SliceBuf& out);
// Warp-level mma.sync implementation (reference for the tensor-core kernel below).
int ozgemm(Ctx* c, const OzArgs& g);
// tcgen05 / TMEM / TMA implementation; both operands K-contiguous.  err_flag (device int)
// is set when a bounded wait inside the kernel gave up.
int ozgemm_tc(Ctx* c, const OzArgs& g, int* err_flag);
// One line per shape class the tensor-core kernel's autotuner has decided on this device.
std::string ozgemm_tune_log(int device);

}  // namespace thc
