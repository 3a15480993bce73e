// Sliced-BF16 GEMM on the 5th-generation tensor cores (tcgen05 + TMEM + TMA).
//
// Same arithmetic as ozgemm.cu (see ozgemm.cuh): C = sum over slice pairs (i, j), i + j < LV,
// of S_i T_j (slices stored pre-scaled by 2^{-7i}), with exact FP32 chunk sums folded into a
// double-word FP32 total.
//
// CTA tile 128 x BN (BN = 128, or 64 for two CTAs per SM), k-step BK (16 or 32) per
// pipeline stage, all LV slices of A and B per stage, as many stages as fit in ~200 KB of
// shared memory (BN = 128) or ~80 KB (BN = 64).
// Warp roles (320 threads):
//   warp 0      TMA producer: 2*LV tiled loads per stage (K-major, 32- or 64-byte swizzle)
//   warp 1      TMEM allocator + single-thread MMA issuer
//   warps 2-9   epilogue: two warps per TMEM lane quadrant, 64 columns each
// TMEM (4 BN columns) holds four 128 x BN FP32 accumulators: one each for the pair levels
// 0, 1 and 2, which carry the bulk of the value and are drained every 512 k while each of
// their sums is still exact (an integer multiple of 2^{-7l} below 2^{24-7l}), and one for
// all levels >= 3 together, which weigh <= 2^-21 of the total and are inexact FP32 sums
// (drained every 128 k, so that no running sum grows over the whole K).  Around a drain the
// MMA thread issues the pairs of the other accumulators first, which covers it.
// BN = 64 halves the epilogue of a tile and its TMEM (256 columns) and shared memory, so two
// CTAs share an SM and one's epilogue overlaps the other's loads and MMAs: the short-K
// products (K = N_o) are epilogue-bound with one CTA per SM.
// Every mbarrier wait is bounded; on timeout the kernel records an error, stops issuing,
// and every role falls through to the teardown, which frees TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "ozgemm.cuh"

namespace thc {

namespace {

constexpr int TBM = 128;
constexpr int kChunkK = 512;            // exact levels are drained every 512 k
constexpr int kStageBudget = 200 * 1024;  // shared memory for the stage buffers (BN = 128)
constexpr int kStageBudget64 = 80 * 1024;  // the same for BN = 64 (two CTAs per SM)
constexpr int kSmemGuard = 16 * 1024;   // slack after the buffers (descriptor reads stay inside)
constexpr int TEPI_WARPS = 8;
constexpr int TTHREADS = 32 * (2 + TEPI_WARPS);
constexpr long long kDrainLimit = 1LL << 22;   // teardown waits after an abort

__device__ __forceinline__ uint32_t su32(const void* p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(su32(b)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(su32(b)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* b)
{
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(su32(b)) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t* b, uint32_t parity)
{
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(su32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: false (and *abort set) when the barrier phase does not complete within
// `limit` polls (the context option "spin_limit"; 0 gives up at once).
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, volatile int* abort,
                                          long long limit)
{
  for (long long i = 0; i < limit; i++) {
    if (mbar_try(b, parity)) return true;
    if (*abort) return false;
  }
  *abort = 1;
  return false;
}

// Teardown wait after an abort: polls a phase a bounded number of times, whatever *abort.
__device__ __forceinline__ void mbar_drain(uint64_t* b, uint32_t parity)
{
  for (long long i = 0; i < kDrainLimit; i++)
    if (mbar_try(b, parity)) return;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar)
{
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
          su32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(su32(bar))
      : "memory");
}

// UMMA shared-memory descriptor, K-major with the rows of one tile BK bf16 (2 BK bytes)
// long: BK = 32 uses the 64-byte swizzle (8-row groups 512 B apart), BK = 16 the 32-byte
// swizzle (groups 256 B apart).
template <int BK>
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr)
{
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;                       // leading byte offset (unused when swizzled)
  d |= (uint64_t)((8 * 2 * BK) >> 4) << 32;     // stride byte offset: one 8-row group
  d |= (uint64_t)1 << 46;                       // descriptor version
  d |= (uint64_t)(BK == 32 ? 4 : 6) << 61;      // layout: 64- or 32-byte swizzle
  return d;
}

// kind::f16 instruction descriptor: D f32, A/B bf16, both K-major, M = 128, N = BN.
template <int BN>
__host__ __device__ constexpr uint32_t idesc()
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
         ((uint32_t)(TBM >> 4) << 24);
}

template <int BN>
__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t acc)
{
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc<BN>()), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                   su32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v)
{
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

// Error-free transformations in FP32 (Knuth's TwoSum; Dekker's FastTwoSum for |a| >= |b|).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e)
{
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
// (h, l) += x for a double-word accumulator (error ~2^-48 relative).
__device__ __forceinline__ void dw_add(float& h, float& l, float x)
{
  float s, e;
  two_sum(h, x, s, e);
  e = __fadd_rn(e, l);
  fast_two_sum(s, e, h, l);
}
__device__ __forceinline__ float pow2f(int e)
{
  if (e > -127 && e < 128) return __int_as_float((e + 127) << 23);
  return ldexpf(1.f, e);
}

__device__ __forceinline__ double pow2d(int e)
{
  if (e > -1022 && e < 1023) return __longlong_as_double((long long)(e + 1023) << 52);
  return ldexp(1.0, e);
}

struct TcArgs {
  long long M, N, K;
  long long a_rows_pad, b_rows_pad;   // rows of one slice in the 2-D tensor maps
  long long a_tile_rows, b_tile_rows; // tiled operands: map rows per 32-wide k tile; 0 = plain
  int hi_stages;                      // stages between drains of the level >= 3 accumulator
  const int* ea;
  const int* eb;
  void* C;
  long long ldc;
  int epilogue;
  int lower_only;
  int* error;                         // set to 1 when a bounded wait gave up
  long long spin_limit;               // polls before a wait gives up
  int group_m;                        // m-tiles per group of the tile order
  int ksplit;
  double* part;
};

// Stage geometry of one (LV, BK, BN) instantiation.
template <int LV, int BK, int BN>
struct TcCfg {
  static constexpr int A_BYTES = TBM * BK * 2;            // one slice tile of A
  static constexpr int B_BYTES = BN * BK * 2;             // one slice tile of B
  static constexpr int STAGE_BYTES = LV * (A_BYTES + B_BYTES);
  static constexpr int BUDGET = BN == 128 ? kStageBudget : kStageBudget64;
  static constexpr int STAGES = BUDGET / STAGE_BYTES < 4 ? BUDGET / STAGE_BYTES : 4;
  static constexpr int CHUNK_STAGES = kChunkK / BK;
  static constexpr int NEXACT = LV < 3 ? LV : 3;          // exact level accumulators
  static constexpr int ECOLS = BN / 2;                    // columns per epilogue warp
  static constexpr int TMEM_COLS = 4 * BN;                // four accumulators
  // The stage buffers, reused after the main loop to stage the epilogue's 8 warps x 32 x
  // ECOLS 8-byte results; the barriers follow.
  static constexpr int EPI_BYTES = TEPI_WARPS * 32 * ECOLS * 8;
  static constexpr int BUF_BYTES = STAGES * STAGE_BYTES > EPI_BYTES ? STAGES * STAGE_BYTES : EPI_BYTES;
  // + barriers (256 B) + the tile's 128 column exponents (512 B) + guard.
  static constexpr size_t SMEM = (size_t)BUF_BYTES + 1024 + 256 + 512 + kSmemGuard;
  static_assert(STAGES >= 2, "stage buffers");
  static_assert(BN == 128 || BN == 64, "tile width");
};

// Epilogue results whose power-of-two scale leaves the FP32 range (rare): formed in FP64.
// mode: OZ_SQUARE_DW / OZ_STORE_DW give a double-word pair's bits, others the FP64 value.
__device__ __noinline__ double wide_result(float h, float l, int ex, int mode)
{
  double val = ((double)h + (double)l) * pow2d(ex);
  if (mode == OZ_SQUARE_F64 || mode == OZ_SQUARE_DW) val = val * val;
  if (mode == OZ_SQUARE_DW || mode == OZ_STORE_DW) {
    const float hi = (float)val, lo = (float)(val - (double)hi);
    return __hiloint2double(__float_as_int(lo), __float_as_int(hi));
  }
  return val;
}

__device__ __noinline__ float wide_f32(float h, float l, int ex)
{
  return (float)(((double)h + (double)l) * pow2d(ex));
}

template <int LV, int BK, int BN>
__global__ void __launch_bounds__(TTHREADS, (BN == 128 ? 1 : 2))   // CTAs per SM
    ozgemm_tc_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
                     TcArgs g)
{
  using Cfg = TcCfg<LV, BK, BN>;
  constexpr int EC = Cfg::ECOLS;
  constexpr int A_BYTES = Cfg::A_BYTES, B_BYTES = Cfg::B_BYTES, STAGE_BYTES = Cfg::STAGE_BYTES;
  constexpr int NST = Cfg::STAGES;
  // Grouped tile order: consecutive blocks sweep g.group_m m-tiles for each n-tile, so the
  // CTAs resident at one time share a few A and B row blocks through L2.
  long long mt, nt;
  {
    const long long mtn = gridDim.x, ntn = gridDim.y;
    const long long b = (long long)blockIdx.y * mtn + blockIdx.x;
    const long long grpm = g.group_m;
    const long long per_group = grpm * ntn;
    const long long grp = b / per_group, first_m = grp * grpm;
    const long long gm = mtn - first_m < grpm ? mtn - first_m : grpm;
    const long long r = b - grp * per_group;
    mt = first_m + r % gm;
    nt = r / gm;
  }
  const long long m0 = mt * TBM;
  const long long n0 = nt * BN;
  if (g.lower_only && n0 > m0 + TBM - 1) return;

  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + Cfg::BUF_BYTES);
  uint64_t* empty = full + NST;
  uint64_t* acc_full = empty + NST;
  uint64_t* acc_empty = acc_full + 1;      // exact levels drained
  uint64_t* acc_empty_hi = acc_empty + 1;  // the level >= 3 accumulator drained
  uint64_t* acc_full_hi = acc_empty_hi + 1;  // the level >= 3 accumulator ready
  uint64_t* mma_done = acc_full_hi + 1;      // every issued MMA has completed (teardown)
  uint32_t* tmem_slot = (uint32_t*)(mma_done + 1);
  volatile int* abort = (volatile int*)(tmem_slot + 1);
  volatile int* issued = abort + 1;          // stages whose loads the producer issued
  volatile int* consumed = issued + 1;       // stages the MMA issuer saw land

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  long long kbeg = 0, kend = g.K;
  if (g.ksplit > 1) {
    long long kc = ((g.K + g.ksplit - 1) / g.ksplit + kChunkK - 1) / kChunkK * kChunkK;
    kbeg = blockIdx.z * kc;
    kend = kbeg + kc < g.K ? kbeg + kc : g.K;
  }
  const int nstages = kend > kbeg ? (int)((kend - kbeg + BK - 1) / BK) : 0;
  const int nchunks = (nstages + Cfg::CHUNK_STAGES - 1) / Cfg::CHUNK_STAGES;
  const int HS = g.hi_stages;                       // divides CHUNK_STAGES
  // The level >= 3 periods are offset by half a period from the exact chunks, so the two
  // accumulators never need draining at the same stage (each drain is covered by the other
  // accumulator's MMAs).
  const int HOFF = HS / 2;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(acc_full, 1);
    mbar_init(acc_empty, TEPI_WARPS);
    mbar_init(acc_empty_hi, TEPI_WARPS);
    mbar_init(acc_full_hi, 1);
    mbar_init(mma_done, 1);
    *abort = 0;
    *issued = 0;
    *consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     su32(tmem_slot)), "n"(Cfg::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------------------------ TMA producer
    if (lane == 0) {
      for (int it = 0; it < nstages; it++) {
        int s = it % NST;
        uint32_t ph = (uint32_t)((it / NST) & 1);
        if (!mbar_wait(&empty[s], ph ^ 1, abort, g.spin_limit)) break;
        unsigned char* st = smem + s * STAGE_BYTES;
        *issued = it + 1;
        mbar_expect_tx(&full[s], STAGE_BYTES);
        const long long k = kbeg + (long long)it * BK;
        // Plain maps: x = k, y = slice row.  Tiled maps (64-byte rows): x = k % 32 and y
        // walks the 32-wide k tiles first.
        const int ax = g.a_tile_rows ? (int)(k & 31) : (int)k;
        const int bx = g.b_tile_rows ? (int)(k & 31) : (int)k;
        const long long ay0 = g.a_tile_rows ? (k >> 5) * g.a_tile_rows : 0;
        const long long by0 = g.b_tile_rows ? (k >> 5) * g.b_tile_rows : 0;
#pragma unroll
        for (int sl = 0; sl < LV; sl++) {
          tma_load_2d(st + sl * A_BYTES, &ta, ax, (int)(ay0 + sl * g.a_rows_pad + m0), &full[s]);
          tma_load_2d(st + LV * A_BYTES + sl * B_BYTES, &tb, bx,
                      (int)(by0 + sl * g.b_rows_pad + n0), &full[s]);
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      for (int it = 0; it < nstages && !*abort; it++) {
        int s = it % NST;
        uint32_t ph = (uint32_t)((it / NST) & 1);
        int chunk = it / Cfg::CHUNK_STAGES;
        bool chunk_first = (it % Cfg::CHUNK_STAGES) == 0;
        bool chunk_last = ((it + 1) % Cfg::CHUNK_STAGES) == 0 || it + 1 == nstages;
        if (!mbar_wait(&full[s], ph, abort, g.spin_limit)) break;
        *consumed = it + 1;
        asm volatile("tcgen05.fence::after_thread_sync;\n");
        unsigned char* st = smem + s * STAGE_BYTES;
        uint32_t a0 = su32(st), b0 = su32(st + LV * A_BYTES);
        const int hp = (it + HOFF) / HS;
        const bool hp_first = it == 0 || ((it + HOFF) % HS) == 0;
        const bool hp_last = ((it + HOFF + 1) % HS) == 0 || it + 1 == nstages;
        // Levels >= 3 into the fourth accumulator, which the epilogue drains every HS
        // stages: the tensor cores' FP32 accumulation loses low bits of each addend relative
        // to the running sum, and a sum over the whole K (~2000 instructions at N_mu 2048)
        // cost 8x in the final error; a drain every 128 k brings it to within 15 % of an
        // FP64 fold per 256 k.
        auto issue_hi = [&]() {
          bool first = hp_first;
#pragma unroll
          for (int l = 3; l < LV; l++) {
#pragma unroll
            for (int i = 0; i <= l; i++) {
              int j = l - i;
#pragma unroll
              for (int kk = 0; kk < BK / 16; kk++) {
                uint64_t ad = sdesc<BK>(a0 + i * A_BYTES + kk * 32);
                uint64_t bd = sdesc<BK>(b0 + j * B_BYTES + kk * 32);
                umma<BN>(tmem + 3 * BN, ad, bd, first ? 0u : 1u);
                first = false;
              }
            }
          }
        };
        // Levels 0-2: exact per chunk.
        auto issue_ex = [&]() {
#pragma unroll
          for (int l = 0; l < Cfg::NEXACT; l++) {
            bool first = chunk_first;
#pragma unroll
            for (int i = 0; i <= l; i++) {
              int j = l - i;
#pragma unroll
              for (int kk = 0; kk < BK / 16; kk++) {
                uint64_t ad = sdesc<BK>(a0 + i * A_BYTES + kk * 32);
                uint64_t bd = sdesc<BK>(b0 + j * B_BYTES + kk * 32);
                umma<BN>(tmem + l * BN, ad, bd, first ? 0u : 1u);
                first = false;
              }
            }
          }
        };
        const bool wait_hi = LV > 3 && hp_first && hp > 0;
        const bool wait_ex = chunk_first && chunk > 0;
        if (wait_ex) {
          // Both drains pending: the epilogue empties the level >= 3 accumulator first, so
          // those pairs go first and cover the drain of the exact levels.
          if (wait_hi) {
            if (!mbar_wait(acc_empty_hi, (uint32_t)((hp - 1) & 1), abort, g.spin_limit)) break;
            asm volatile("tcgen05.fence::after_thread_sync;\n");
          }
          issue_hi();
          if (!mbar_wait(acc_empty, (uint32_t)((chunk - 1) & 1), abort, g.spin_limit)) break;
          asm volatile("tcgen05.fence::after_thread_sync;\n");
          issue_ex();
        } else {
          // At most the level >= 3 drain pending: the exact pairs cover it.
          issue_ex();
          if (wait_hi) {
            if (!mbar_wait(acc_empty_hi, (uint32_t)((hp - 1) & 1), abort, g.spin_limit)) break;
            asm volatile("tcgen05.fence::after_thread_sync;\n");
          }
          issue_hi();
        }
        umma_commit(&empty[s]);
        if (LV > 3 && hp_last) umma_commit(acc_full_hi);
        if (chunk_last) umma_commit(acc_full);
      }
      // Completion of every MMA this thread issued, for the teardown.
      umma_commit(mma_done);
    }
  } else {
    // ------------------------------------------------------------------ epilogue
    const int ew = warp - 2;                 // 0..7
    const int quad = warp & 3;               // TMEM lane quadrant this warp may access
    const int half = ew >> 2;                // which EC-column half of the tile
    const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
    const int col0 = half * EC;
    // Exponents of this row and of the half's EC columns, loaded while the MMAs run (both
    // warps of a half store the same values).
    int* seb = (int*)((unsigned char*)full + 256) + col0;
#pragma unroll
    for (int q = lane; q < EC; q += 32) {
      const long long na = n0 + col0 + q;
      seb[q] = na < g.N ? g.eb[na] : 0;
    }
    const long long m = m0 + quad * 32 + lane;
    const int ea = (m < g.M ? g.ea[m] : 0) - 14;
    __syncwarp();
    // Double-word FP32 totals of this thread's row, EC columns.
    float ah[EC], al[EC];
#pragma unroll
    for (int q = 0; q < EC; q++) { ah[q] = 0.f; al[q] = 0.f; }
    bool ok = true;
    const int nhp = nstages > 0 ? (nstages - 1 + HOFF) / HS + 1 : 0;
    int hpd = 0;                                     // level >= 3 periods drained
    for (int ch = 0; ch < nchunks; ch++) {
      // The level >= 3 periods of this chunk first (the MMA waits for each).
      const int hp_end = min(nhp, (ch + 1) * (Cfg::CHUNK_STAGES / HS));
      for (; LV > 3 && hpd < hp_end; hpd++) {
        if (!mbar_wait(acc_full_hi, (uint32_t)(hpd & 1), abort, g.spin_limit)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;\n");
#pragma unroll
        for (int b = 0; b < EC / 8; b++) {
          float v[8];
          tmem_ld8(tmem + lane_base + 3 * BN + (uint32_t)(col0 + 8 * b), v);
          // |v| <= 2^-21 |ah|: the low word takes it with an FP32 rounding of ~2^-45 |ah|.
#pragma unroll
          for (int q = 0; q < 8; q++) al[8 * b + q] = __fadd_rn(al[8 * b + q], v[q]);
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n");
        __syncwarp();
        if (lane == 0) mbar_arrive(acc_empty_hi);
      }
      if (!ok) break;
      if (!mbar_wait(acc_full, (uint32_t)(ch & 1), abort, g.spin_limit)) { ok = false; break; }
      asm volatile("tcgen05.fence::after_thread_sync;\n");
#pragma unroll
      for (int b = 0; b < EC / 8; b++) {   // 8 columns at a time (register pressure)
        float l0[8], l1[8], l2[8];
        const uint32_t cb = (uint32_t)(col0 + 8 * b);
        tmem_ld8(tmem + lane_base + 0 * BN + cb, l0);
        if (LV > 1) tmem_ld8(tmem + lane_base + 1 * BN + cb, l1);
        if (LV > 2) tmem_ld8(tmem + lane_base + 2 * BN + cb, l2);
        // l0, l1, l2 are exact (multiples of 1, 2^-7, 2^-14 below 2^24, 2^17, 2^10); their
        // sum needs <= 38 bits and is carried exactly in (s, e).
#pragma unroll
        for (int q = 0; q < 8; q++) {
          float s1 = l0[q], e1 = 0.f;
          if (LV > 1) two_sum(l0[q], l1[q], s1, e1);
          if (LV > 2) {
            float s2, e2;
            two_sum(s1, l2[q], s2, e2);
            s1 = s2;
            e1 = __fadd_rn(e1, e2);
          }
          dw_add(ah[8 * b + q], al[8 * b + q], s1);
          dw_add(ah[8 * b + q], al[8 * b + q], e1);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;\n");
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty);
    }
    // The level >= 3 period that ends with the last stage.
    for (; ok && LV > 3 && hpd < nhp; hpd++) {
      if (!mbar_wait(acc_full_hi, (uint32_t)(hpd & 1), abort, g.spin_limit)) { ok = false; break; }
      asm volatile("tcgen05.fence::after_thread_sync;\n");
#pragma unroll
      for (int b = 0; b < EC / 8; b++) {
        float v[8];
        tmem_ld8(tmem + lane_base + 3 * BN + (uint32_t)(col0 + 8 * b), v);
#pragma unroll
        for (int q = 0; q < 8; q++) al[8 * b + q] = __fadd_rn(al[8 * b + q], v[q]);
      }
      asm volatile("tcgen05.fence::before_thread_sync;\n");
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty_hi);
    }
    if (ok && !*abort) {
      // The warp's 32 x 64 results go through shared memory (the stage buffers are free:
      // every MMA has completed, so every TMA load has landed and been consumed) and are
      // written row by row, so each store instruction covers 256-512 contiguous bytes
      // instead of 32 rows kilobytes apart.
      const bool split = g.ksplit > 1;
      const bool f32 = !split && g.epilogue == OZ_STORE_F32;
      unsigned char* stg = smem + (size_t)ew * (32 * EC * 8);
      float* stg32 = (float*)stg;
      double* stg64 = (double*)stg;
      // One unrolled loop per epilogue, so that the instructions a CTA executes are one
      // contiguous stretch (instruction fetch was the first stall of the short-K products);
      // results whose scale leaves the FP32 range take a call.
      const int mode = split ? -1 : g.epilogue;
      if (mode == OZ_STORE_F32) {
#pragma unroll
        for (int q = 0; q < EC; q++) {
          const int ex = ea + seb[q];
          const float v = (ex > -126 && ex < 127) ? __fadd_rn(ah[q], al[q]) * pow2f(ex)
                                                  : wide_f32(ah[q], al[q], ex);
          stg32[lane * EC + (q ^ lane)] = v;
        }
      } else if (mode == OZ_SQUARE_DW) {
#pragma unroll
        for (int q = 0; q < EC; q++) {
          const int ex = ea + seb[q];
          double w;
          if (ex > -60 && ex < 60) {
            // (h + l)^2 in double-word FP32: p + e = h^2 exactly (FMA), plus 2 h l.
            const float sc = pow2f(ex);
            const float h = ah[q] * sc, l = al[q] * sc;
            const float pp = __fmul_rn(h, h);
            float e = __fmaf_rn(h, h, -pp);
            e = __fmaf_rn(2.f * h, l, e);
            float zh, zl;
            fast_two_sum(pp, e, zh, zl);
            w = __hiloint2double(__float_as_int(zl), __float_as_int(zh));
          } else {
            w = wide_result(ah[q], al[q], ex, mode);
          }
          stg64[lane * EC + (q ^ (lane & 15))] = w;
        }
      } else if (mode == OZ_STORE_DW) {
#pragma unroll
        for (int q = 0; q < EC; q++) {
          const int ex = ea + seb[q];
          double w;
          if (ex > -100 && ex < 100) {
            const float sc = pow2f(ex);
            float zh, zl;
            fast_two_sum(ah[q] * sc, al[q] * sc, zh, zl);
            w = __hiloint2double(__float_as_int(zl), __float_as_int(zh));
          } else {
            w = wide_result(ah[q], al[q], ex, mode);
          }
          stg64[lane * EC + (q ^ (lane & 15))] = w;
        }
      } else {
        // FP64 results (stored, squared, or split-K partials).
        const bool sq = mode == OZ_SQUARE_F64;
#pragma unroll
        for (int q = 0; q < EC; q++) {
          double val = ((double)ah[q] + (double)al[q]) * pow2d(ea + seb[q]);
          if (sq) val = val * val;
          stg64[lane * EC + (q ^ (lane & 15))] = val;
        }
      }
      __syncwarp();
      // Row r of the staging: EC / 2 lanes per row, each writing two adjacent columns (one
      // row per pass for EC = 64, two for EC = 32).
      const long long ld = split ? g.N : g.ldc;
      constexpr int LPR = EC / 2, RPP = 32 / LPR;
      const int c0 = 2 * (lane % LPR);
      const long long n = n0 + col0 + c0;
      for (int r0 = 0; r0 < 32; r0 += RPP) {
        const int r = r0 + lane / LPR;
        const long long mr = m0 + quad * 32 + r;
        if (mr >= g.M) break;
        const bool v0 = n < g.N && !(g.lower_only && n > mr);
        const bool v1 = n + 1 < g.N && !(g.lower_only && n + 1 > mr);
        const long long off = mr * ld + n;
        if (f32) {
          const float a = stg32[r * EC + (c0 ^ r)], bb = stg32[r * EC + ((c0 + 1) ^ r)];
          float* dst = (float*)g.C + off;
          if (v0 && v1 && !((uintptr_t)dst & 7)) *(float2*)dst = make_float2(a, bb);
          else {
            if (v0) dst[0] = a;
            if (v1) dst[1] = bb;
          }
        } else {
          const double a = stg64[r * EC + (c0 ^ (r & 15))];
          const double bb = stg64[r * EC + ((c0 + 1) ^ (r & 15))];
          double* dst = split ? g.part + (long long)blockIdx.z * g.M * g.N + off
                              : (double*)g.C + off;
          // Paired stores only at 16-byte aligned addresses (the partials of split z start at
          // z M N, odd for odd M N).
          if (v0 && v1 && !((uintptr_t)dst & 15)) *(double2*)dst = make_double2(a, bb);
          else {
            if (v0) dst[0] = a;
            if (v1) dst[1] = bb;
          }
        }
      }
    }
  }
  // ---------------------------------------------------------------------- teardown
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  if (threadIdx.x == 0) {
    // Before shared memory and TMEM are released, bounded: after an abort the loads issued
    // but never consumed land (each stage's phase completes); in every case the MMAs issued
    // so far have completed (mma_done; at once on the normal path).
    if (*abort) {
      atomicExch(g.error, 1);
      for (int it = *consumed; it < *issued; it++)
        mbar_drain(&full[it % NST], (uint32_t)((it / NST) & 1));
    }
    mbar_drain(mma_done, 0);
  }
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "n"(Cfg::TMEM_COLS));
  }
}

// ---------------------------------------------------------------------------------------
// Persistent variant for short K (K <= 512, no split): one CTA per SM walks the tiles
// blockIdx.x, blockIdx.x + gridDim.x, ... in the grouped order, with 128 x 64 tiles and two
// TMEM buffers of four 64-column accumulators, so the epilogue of one tile (TMEM drain,
// double-word fold, staging and stores) runs while the MMAs of the next tile fill the other
// buffer, and the TMA ring of stages runs on across tiles.  With K <= 512 every exact level
// is exact over the whole K and the level >= 3 accumulator is drained once, at the end of
// the tile.  The epilogue stages its results in a buffer of its own (the stage ring stays
// in use).
constexpr int kPersistBudget = 176 * 1024;   // stage ring + epilogue staging

template <int LV, int BK>
struct TpCfg {
  static constexpr int BN = 64;
  static constexpr int A_BYTES = TBM * BK * 2;
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int STAGE_BYTES = LV * (A_BYTES + B_BYTES);
  static constexpr int EC = BN / 2;                          // columns per epilogue warp
  static constexpr int STG_BYTES = TEPI_WARPS * 32 * EC * 8;  // epilogue staging
  static constexpr int STAGES_FIT = (kPersistBudget - STG_BYTES) / STAGE_BYTES;
  static constexpr int STAGES = STAGES_FIT < 4 ? STAGES_FIT : 4;
  static constexpr int BUF_COLS = 4 * BN;                    // one buffer of accumulators
  // stage ring | staging | barriers (256 B) | exponents (8 warps x 32 ints) | guard
  static constexpr size_t SMEM =
      (size_t)STAGES * STAGE_BYTES + STG_BYTES + 1024 + 256 + 1024 + kSmemGuard;
  static_assert(STAGES >= 2, "stage ring");
};

// Tile t of the grouped order (group_m m-tiles per n-tile, as ozgemm_tc_kernel's grid).
__device__ __forceinline__ void tile_coords(long long t, long long mtn, long long ntn,
                                            long long grpm, long long& mt, long long& nt)
{
  const long long per_group = grpm * ntn;
  const long long grp = t / per_group, first_m = grp * grpm;
  const long long gm = mtn - first_m < grpm ? mtn - first_m : grpm;
  const long long r = t - grp * per_group;
  mt = first_m + r % gm;
  nt = r / gm;
}

template <int LV, int BK>
__global__ void __launch_bounds__(TTHREADS, 1)
    ozgemm_tc_persistent(const __grid_constant__ CUtensorMap ta,
                         const __grid_constant__ CUtensorMap tb, TcArgs g)
{
  using Cfg = TpCfg<LV, BK>;
  constexpr int BN = Cfg::BN, EC = Cfg::EC;
  constexpr int A_BYTES = Cfg::A_BYTES, B_BYTES = Cfg::B_BYTES, STAGE_BYTES = Cfg::STAGE_BYTES;
  constexpr int NST = Cfg::STAGES;
  const long long mtn = (g.M + TBM - 1) / TBM, ntn = (g.N + BN - 1) / BN;
  const long long ntiles = mtn * ntn;

  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* stg_base = smem + (size_t)NST * STAGE_BYTES;
  uint64_t* full = (uint64_t*)(stg_base + Cfg::STG_BYTES);
  uint64_t* empty = full + NST;
  uint64_t* acc_full = empty + NST;          // [2] a buffer's accumulators are final
  uint64_t* acc_empty = acc_full + 2;        // [2] the epilogue has drained a buffer
  uint64_t* mma_done = acc_empty + 2;
  uint32_t* tmem_slot = (uint32_t*)(mma_done + 1);
  volatile int* abort = (volatile int*)(tmem_slot + 1);
  volatile int* issued = abort + 1;
  volatile int* consumed = issued + 1;
  int* sexp = (int*)((unsigned char*)full + 256);   // 8 warps x 32 column exponents

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nstages = (int)((g.K + BK - 1) / BK);

  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], TEPI_WARPS);
    }
    mbar_init(mma_done, 1);
    *abort = 0;
    *issued = 0;
    *consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(
                     su32(tmem_slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------------------------ TMA producer
    if (lane == 0) {
      int git = 0;
      bool ok = true;
      for (long long t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        long long mt, nt;
        tile_coords(t, mtn, ntn, g.group_m, mt, nt);
        const long long m0 = mt * TBM, n0 = nt * BN;
        for (int it = 0; it < nstages; it++, git++) {
          const int s = git % NST;
          const uint32_t ph = (uint32_t)((git / NST) & 1);
          if (!mbar_wait(&empty[s], ph ^ 1, abort, g.spin_limit)) { ok = false; break; }
          unsigned char* st = smem + s * STAGE_BYTES;
          *issued = git + 1;
          mbar_expect_tx(&full[s], STAGE_BYTES);
          const long long k = (long long)it * BK;
          const int ax = g.a_tile_rows ? (int)(k & 31) : (int)k;
          const int bx = g.b_tile_rows ? (int)(k & 31) : (int)k;
          const long long ay0 = g.a_tile_rows ? (k >> 5) * g.a_tile_rows : 0;
          const long long by0 = g.b_tile_rows ? (k >> 5) * g.b_tile_rows : 0;
#pragma unroll
          for (int sl = 0; sl < LV; sl++) {
            tma_load_2d(st + sl * A_BYTES, &ta, ax, (int)(ay0 + sl * g.a_rows_pad + m0), &full[s]);
            tma_load_2d(st + LV * A_BYTES + sl * B_BYTES, &tb, bx,
                        (int)(by0 + sl * g.b_rows_pad + n0), &full[s]);
          }
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      int git = 0, tc = 0;
      bool ok = true;
      for (long long t = blockIdx.x; t < ntiles && ok; t += gridDim.x, tc++) {
        const int b = tc & 1, use = tc >> 1;
        const uint32_t acc0 = tmem + (uint32_t)(b * Cfg::BUF_COLS);
        if (use > 0) {
          if (!mbar_wait(&acc_empty[b], (uint32_t)((use - 1) & 1), abort, g.spin_limit)) break;
          asm volatile("tcgen05.fence::after_thread_sync;\n");
        }
        for (int it = 0; it < nstages; it++, git++) {
          const int s = git % NST;
          const uint32_t ph = (uint32_t)((git / NST) & 1);
          if (!mbar_wait(&full[s], ph, abort, g.spin_limit)) { ok = false; break; }
          *consumed = git + 1;
          asm volatile("tcgen05.fence::after_thread_sync;\n");
          unsigned char* st = smem + s * STAGE_BYTES;
          const uint32_t a0 = su32(st), b0 = su32(st + LV * A_BYTES);
          bool first_hi = it == 0;
#pragma unroll
          for (int l = 0; l < LV; l++) {
            bool first = it == 0;
#pragma unroll
            for (int i = 0; i <= l; i++) {
              const int j = l - i;
#pragma unroll
              for (int kk = 0; kk < BK / 16; kk++) {
                const uint64_t ad = sdesc<BK>(a0 + i * A_BYTES + kk * 32);
                const uint64_t bd = sdesc<BK>(b0 + j * B_BYTES + kk * 32);
                if (l < 3) {
                  umma<BN>(acc0 + l * BN, ad, bd, first ? 0u : 1u);
                  first = false;
                } else {
                  umma<BN>(acc0 + 3 * BN, ad, bd, first_hi ? 0u : 1u);
                  first_hi = false;
                }
              }
            }
          }
          umma_commit(&empty[s]);
        }
        if (!ok) break;
        umma_commit(&acc_full[b]);
      }
      umma_commit(mma_done);
    }
  } else {
    // ------------------------------------------------------------------ epilogue
    const int ew = warp - 2;
    const int quad = warp & 3;
    const int half = ew >> 2;
    const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
    const int col0 = half * EC;
    int* seb = sexp + ew * 32;
    unsigned char* stg = stg_base + (size_t)ew * (32 * EC * 8);
    float* stg32 = (float*)stg;
    double* stg64 = (double*)stg;
    const int mode = g.epilogue;
    int tc = 0;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x, tc++) {
      const int b = tc & 1, use = tc >> 1;
      long long mt, nt;
      tile_coords(t, mtn, ntn, g.group_m, mt, nt);
      const long long m0 = mt * TBM, n0 = nt * BN;
      {
        const long long na = n0 + col0 + lane;
        seb[lane] = na < g.N ? g.eb[na] : 0;
      }
      const long long m = m0 + quad * 32 + lane;
      const int ea = (m < g.M ? g.ea[m] : 0) - 14;
      __syncwarp();
      if (!mbar_wait(&acc_full[b], (uint32_t)(use & 1), abort, g.spin_limit)) break;
      asm volatile("tcgen05.fence::after_thread_sync;\n");
      const uint32_t acc0 = tmem + (uint32_t)(b * Cfg::BUF_COLS) + lane_base;
      float ah[EC], al[EC];
#pragma unroll
      for (int bb = 0; bb < EC / 8; bb++) {
        float l0[8], l1[8], l2[8], hi[8];
        const uint32_t cb = (uint32_t)(col0 + 8 * bb);
        tmem_ld8(acc0 + 0 * BN + cb, l0);
        if (LV > 1) tmem_ld8(acc0 + 1 * BN + cb, l1);
        if (LV > 2) tmem_ld8(acc0 + 2 * BN + cb, l2);
        if (LV > 3) tmem_ld8(acc0 + 3 * BN + cb, hi);
#pragma unroll
        for (int q = 0; q < 8; q++) {
          // The exact levels' sum needs <= 38 bits and is carried exactly in (s1, e1); the
          // levels >= 3 (<= 2^-21 of the value) go to the low word.
          float s1 = l0[q], e1 = 0.f;
          if (LV > 1) two_sum(l0[q], l1[q], s1, e1);
          if (LV > 2) {
            float s2, e2;
            two_sum(s1, l2[q], s2, e2);
            s1 = s2;
            e1 = __fadd_rn(e1, e2);
          }
          float h = 0.f, lo = LV > 3 ? hi[q] : 0.f;
          dw_add(h, lo, s1);
          dw_add(h, lo, e1);
          ah[8 * bb + q] = h;
          al[8 * bb + q] = lo;
        }
      }
      // The buffer is free for the MMAs of the tile after next.
      asm volatile("tcgen05.fence::before_thread_sync;\n");
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_empty[b]);
      if (mode == OZ_STORE_F32) {
#pragma unroll
        for (int q = 0; q < EC; q++) {
          const int ex = ea + seb[q];
          const float v = (ex > -126 && ex < 127) ? __fadd_rn(ah[q], al[q]) * pow2f(ex)
                                                  : wide_f32(ah[q], al[q], ex);
          stg32[lane * EC + (q ^ lane)] = v;
        }
      } else if (mode == OZ_SQUARE_DW) {
#pragma unroll
        for (int q = 0; q < EC; q++) {
          const int ex = ea + seb[q];
          double w;
          if (ex > -60 && ex < 60) {
            const float sc = pow2f(ex);
            const float h = ah[q] * sc, l = al[q] * sc;
            const float pp = __fmul_rn(h, h);
            float e = __fmaf_rn(h, h, -pp);
            e = __fmaf_rn(2.f * h, l, e);
            float zh, zl;
            fast_two_sum(pp, e, zh, zl);
            w = __hiloint2double(__float_as_int(zl), __float_as_int(zh));
          } else {
            w = wide_result(ah[q], al[q], ex, mode);
          }
          stg64[lane * EC + (q ^ (lane & 15))] = w;
        }
      } else if (mode == OZ_STORE_DW) {
#pragma unroll
        for (int q = 0; q < EC; q++) {
          const int ex = ea + seb[q];
          double w;
          if (ex > -100 && ex < 100) {
            const float sc = pow2f(ex);
            float zh, zl;
            fast_two_sum(ah[q] * sc, al[q] * sc, zh, zl);
            w = __hiloint2double(__float_as_int(zl), __float_as_int(zh));
          } else {
            w = wide_result(ah[q], al[q], ex, mode);
          }
          stg64[lane * EC + (q ^ (lane & 15))] = w;
        }
      } else {
        const bool sq = mode == OZ_SQUARE_F64;
#pragma unroll
        for (int q = 0; q < EC; q++) {
          double val = ((double)ah[q] + (double)al[q]) * pow2d(ea + seb[q]);
          if (sq) val = val * val;
          stg64[lane * EC + (q ^ (lane & 15))] = val;
        }
      }
      __syncwarp();
      // Two rows per pass: 16 lanes per row, two adjacent columns per lane.
      const bool f32 = mode == OZ_STORE_F32;
      const int c0 = 2 * (lane & 15);
      const long long n = n0 + col0 + c0;
      for (int r0 = 0; r0 < 32; r0 += 2) {
        const int r = r0 + (lane >> 4);
        const long long mr = m0 + quad * 32 + r;
        if (mr >= g.M) break;
        const bool v0 = n < g.N, v1 = n + 1 < g.N;
        const long long off = mr * g.ldc + n;
        if (f32) {
          const float a = stg32[r * EC + (c0 ^ r)], bv = stg32[r * EC + ((c0 + 1) ^ r)];
          float* dst = (float*)g.C + off;
          if (v0 && v1 && !((uintptr_t)dst & 7)) *(float2*)dst = make_float2(a, bv);
          else {
            if (v0) dst[0] = a;
            if (v1) dst[1] = bv;
          }
        } else {
          const double a = stg64[r * EC + (c0 ^ (r & 15))];
          const double bv = stg64[r * EC + ((c0 + 1) ^ (r & 15))];
          double* dst = (double*)g.C + off;
          if (v0 && v1 && !((uintptr_t)dst & 15)) *(double2*)dst = make_double2(a, bv);
          else {
            if (v0) dst[0] = a;
            if (v1) dst[1] = bv;
          }
        }
      }
      __syncwarp();   // the staging and the exponents are rewritten for the next tile
    }
  }
  // ---------------------------------------------------------------------- teardown
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  if (threadIdx.x == 0) {
    if (*abort) {
      atomicExch(g.error, 1);
      for (int it = *consumed; it < *issued; it++)
        mbar_drain(&full[it % NST], (uint32_t)((it / NST) & 1));
    }
    mbar_drain(mma_done, 0);
  }
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;\n" ::"r"(tmem));
  }
}

PFN_cuTensorMapEncodeTiled_v12000 get_encoder()
{
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    // The entry point with the ABI of CUDA 12.0, which the PFN type above describes.
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

// 2-D map of a slice buffer: rows of `width` bf16 (kpad for plain storage, 32 for tiled),
// box bk x box_rows with the swizzle that matches the UMMA descriptor (sdesc<bk>).
int make_map(Ctx* c, CUtensorMap* map, const void* base, long long width, long long rows,
             int box_rows, int bk)
{
  auto enc = get_encoder();
  if (!enc) return set_error(c, THC_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  // Row coordinates are 32-bit in the copy instruction.
  if (rows > 0x7fffffffLL) return set_error(c, THC_ERR_SHAPE, "ozgemm_tc: slice buffer too tall");
  cuuint64_t dims[2] = {(cuuint64_t)width, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)width * 2};
  cuuint32_t box[2] = {(cuuint32_t)bk, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides,
                   box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   bk == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(c, THC_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return THC_OK;
}

// Launch choices of one product: k-step per stage, m-tiles per group of the tile order, and
// the split of K (at most the caller's, whose partial buffer is sized for it).
struct TcChoice {
  int bk = 32;
  int group_m = 8;
  int ksplit = 1;
  int bn = 128;          // tile width: 128, or 64 (with bk = 16) for two CTAs per SM
  int persistent = 0;    // ozgemm_tc_persistent (bn 64, bk 16; K <= 512, no split)
};

// Products the persistent kernel takes: the whole K in one exact chunk, no split of K, no
// triangle.
bool persistent_ok(const OzArgs& g)
{
  return g.K <= kChunkK && g.ksplit <= 1 && !g.lower_only;
}

template <int LV, int BK, int BN>
int launch_tc(Ctx* c, const OzArgs& g, int* err_flag, int group_m)
{
  using Cfg = TcCfg<LV, BK, BN>;
  CUtensorMap ta, tb;
  const bool at = g.a.kt_stride > 0, bt = g.b.kt_stride > 0;
  long long a_rows = at ? g.a.slice_stride / 32 : g.a.slice_stride / g.a.ld;
  long long b_rows = bt ? g.b.slice_stride / 32 : g.b.slice_stride / g.b.ld;
  // Tiled: one map row per 64 bytes; k tiles of LV slices x rows each, g.*.ld / 32 of them.
  if ((at && g.a.kt_stride != LV * g.a.slice_stride) ||
      (bt && g.b.kt_stride != LV * g.b.slice_stride))
    return set_error(c, THC_ERR_ARG, "ozgemm_tc: tiled operand with another slice count");
  int st = at ? make_map(c, &ta, g.a.s, 32, (g.a.ld / 32) * (g.a.kt_stride / 32), TBM, BK)
              : make_map(c, &ta, g.a.s, g.a.ld, a_rows * LV, TBM, BK);
  if (st) return st;
  st = bt ? make_map(c, &tb, g.b.s, 32, (g.b.ld / 32) * (g.b.kt_stride / 32), BN, BK)
          : make_map(c, &tb, g.b.s, g.b.ld, b_rows * LV, BN, BK);
  if (st) return st;
  TcArgs t;
  t.M = g.M; t.N = g.N; t.K = g.K;
  t.a_rows_pad = a_rows; t.b_rows_pad = b_rows;
  t.a_tile_rows = at ? g.a.kt_stride / 32 : 0;
  t.b_tile_rows = bt ? g.b.kt_stride / 32 : 0;
  t.hi_stages = std::max(1, std::min(Cfg::CHUNK_STAGES, c->tc_hi_stages / (BK / 16)));
  t.ea = g.a.e; t.eb = g.b.e; t.C = g.C; t.ldc = g.ldc;
  t.epilogue = g.epilogue; t.lower_only = g.lower_only; t.error = err_flag;
  t.spin_limit = c->spin_limit;
  t.group_m = group_m;
  t.ksplit = std::max(1, g.ksplit); t.part = g.part;
  const size_t smem = Cfg::SMEM;
  THC_CUDA(c, cudaFuncSetAttribute(ozgemm_tc_kernel<LV, BK, BN>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((unsigned)cdiv(g.M, TBM), (unsigned)cdiv(g.N, BN), (unsigned)t.ksplit);
  if (grid.y > 65535) return set_error(c, THC_ERR_SHAPE, "ozgemm_tc: N too large");
  {
    ProfScope prof(c, "ozgemm");
    ProfScope prof_tag(g.tag ? c : nullptr, g.tag ? g.tag : "");
    ozgemm_tc_kernel<LV, BK, BN><<<grid, TTHREADS, smem, c->stream>>>(ta, tb, t);
    THC_LAUNCHED(c, "ozgemm_tc");
  }
  if (t.ksplit > 1) return oz_split_reduce(c, g);
  return THC_OK;
}

template <int BK, int BN>
int launch_bk(Ctx* c, const OzArgs& g, int* err_flag, int group_m)
{
  switch (g.levels) {
    case 2: return launch_tc<2, BK, BN>(c, g, err_flag, group_m);
    case 3: return launch_tc<3, BK, BN>(c, g, err_flag, group_m);
    case 4: return launch_tc<4, BK, BN>(c, g, err_flag, group_m);
    case 5: return launch_tc<5, BK, BN>(c, g, err_flag, group_m);
    case 6: return launch_tc<6, BK, BN>(c, g, err_flag, group_m);
    default: return set_error(c, THC_ERR_ARG, "ozgemm_tc: levels must be 2..6");
  }
}

template <int LV>
int launch_persistent(Ctx* c, const OzArgs& g, int* err_flag, int group_m)
{
  using Cfg = TpCfg<LV, 16>;
  if (!persistent_ok(g)) return set_error(c, THC_ERR_ARG, "ozgemm_tc: persistent kernel takes K <= 512");
  CUtensorMap ta, tb;
  const bool at = g.a.kt_stride > 0, bt = g.b.kt_stride > 0;
  long long a_rows = at ? g.a.slice_stride / 32 : g.a.slice_stride / g.a.ld;
  long long b_rows = bt ? g.b.slice_stride / 32 : g.b.slice_stride / g.b.ld;
  if ((at && g.a.kt_stride != LV * g.a.slice_stride) ||
      (bt && g.b.kt_stride != LV * g.b.slice_stride))
    return set_error(c, THC_ERR_ARG, "ozgemm_tc: tiled operand with another slice count");
  int st = at ? make_map(c, &ta, g.a.s, 32, (g.a.ld / 32) * (g.a.kt_stride / 32), TBM, 16)
              : make_map(c, &ta, g.a.s, g.a.ld, a_rows * LV, TBM, 16);
  if (st) return st;
  st = bt ? make_map(c, &tb, g.b.s, 32, (g.b.ld / 32) * (g.b.kt_stride / 32), Cfg::BN, 16)
          : make_map(c, &tb, g.b.s, g.b.ld, b_rows * LV, Cfg::BN, 16);
  if (st) return st;
  TcArgs t;
  t.M = g.M; t.N = g.N; t.K = g.K;
  t.a_rows_pad = a_rows; t.b_rows_pad = b_rows;
  t.a_tile_rows = at ? g.a.kt_stride / 32 : 0;
  t.b_tile_rows = bt ? g.b.kt_stride / 32 : 0;
  t.hi_stages = 0;
  t.ea = g.a.e; t.eb = g.b.e; t.C = g.C; t.ldc = g.ldc;
  t.epilogue = g.epilogue; t.lower_only = 0; t.error = err_flag;
  t.spin_limit = c->spin_limit;
  t.group_m = group_m;
  t.ksplit = 1; t.part = nullptr;
  int sms = 0;
  THC_CUDA(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  const long long tiles = cdiv(g.M, TBM) * cdiv(g.N, Cfg::BN);
  const unsigned grid = (unsigned)std::min<long long>(tiles, sms);
  THC_CUDA(c, cudaFuncSetAttribute(ozgemm_tc_persistent<LV, 16>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::SMEM));
  {
    ProfScope prof(c, "ozgemm");
    ProfScope prof_tag(g.tag ? c : nullptr, g.tag ? g.tag : "");
    ozgemm_tc_persistent<LV, 16><<<grid, TTHREADS, Cfg::SMEM, c->stream>>>(ta, tb, t);
    THC_LAUNCHED(c, "ozgemm_tc_persistent");
  }
  return THC_OK;
}

int launch_persistent_lv(Ctx* c, const OzArgs& g, int* err_flag, int group_m)
{
  switch (g.levels) {
    case 2: return launch_persistent<2>(c, g, err_flag, group_m);
    case 3: return launch_persistent<3>(c, g, err_flag, group_m);
    case 4: return launch_persistent<4>(c, g, err_flag, group_m);
    case 5: return launch_persistent<5>(c, g, err_flag, group_m);
    case 6: return launch_persistent<6>(c, g, err_flag, group_m);
    default: return set_error(c, THC_ERR_ARG, "ozgemm_tc: levels must be 2..6");
  }
}

int launch_choice(Ctx* c, const OzArgs& g_in, int* err_flag, const TcChoice& ch)
{
  OzArgs g = g_in;
  g.ksplit = ch.ksplit;
  if (g.ksplit <= 1) { g.ksplit = 1; g.part = nullptr; }
  if (ch.persistent) return launch_persistent_lv(c, g, err_flag, ch.group_m);
  if (ch.bn == 64) return launch_bk<16, 64>(c, g, err_flag, ch.group_m);
  return ch.bk == 32 ? launch_bk<32, 128>(c, g, err_flag, ch.group_m)
                     : launch_bk<16, 128>(c, g, err_flag, ch.group_m);
}

// The autotuner's decisions, one table per process and device, keyed by the shape class of a
// product (log2 buckets of M, N and K, slice count, epilogue, lower-triangle flag, the
// caller's split): every context uses the same decision for the same class, so two contexts
// that factorise the same system produce the same bits.  A class is timed once, when first
// met, on the stream of the context that meets it.
struct TuneEntry {
  TcChoice choice;
  float us = 0.f;       // time of the chosen launch when it was tuned (0: model default)
  int candidates = 0;
};
std::mutex g_tune_mu;
std::map<std::vector<long long>, TuneEntry> g_tune;

int ilog2c(long long x)
{
  int r = 0;
  while ((1LL << r) < x) r++;
  return r;
}

}  // namespace

std::string ozgemm_tune_log(int device)
{
  std::lock_guard<std::mutex> lk(g_tune_mu);
  std::string out;
  char buf[256];
  for (const auto& kv : g_tune) {
    const auto& k = kv.first;
    if (k[0] != device) continue;
    const TuneEntry& e = kv.second;
    snprintf(buf, sizeof(buf),
             "M<=2^%lld N<=2^%lld K<=2^%lld slices=%lld epi=%lld lower=%lld split<=%lld: bk=%d "
             "bn=%d%s group_m=%d split=%d %.1fus (%d tried)\n",
             k[1], k[2], k[3], k[4], k[5], k[6], k[7], e.choice.bk, e.choice.bn,
             e.choice.persistent ? " persistent" : "", e.choice.group_m, e.choice.ksplit, e.us,
             e.candidates);
    out += buf;
  }
  return out;
}

int ozgemm_tc(Ctx* c, const OzArgs& g, int* err_flag)
{
  if (g.M <= 0 || g.N <= 0) return THC_OK;
  if (!g.b.k_contig) return set_error(c, THC_ERR_ARG, "ozgemm_tc: B must be K-contiguous");
  const long long ar = g.a.kt_stride ? g.a.slice_stride / 32 : g.a.slice_stride / g.a.ld;
  const long long br = g.b.kt_stride ? g.b.slice_stride / 32 : g.b.slice_stride / g.b.ld;
  if (g.a.ld % 32 || g.b.ld % 32 || ar % TBM || br % 128)
    return set_error(c, THC_ERR_ARG, "ozgemm_tc: operand padding");
  TcChoice dflt;
  dflt.bk = c->tc_bn == 64 ? 16 : c->tc_bk;
  dflt.bn = c->tc_bn;
  if (c->tc_persistent && persistent_ok(g)) {
    dflt.bk = 16;
    dflt.bn = 64;
    dflt.persistent = 1;
  }
  dflt.ksplit = g.ksplit;
  if (!c->autotune) return launch_choice(c, g, err_flag, dflt);
  const std::vector<long long> key = {c->device, ilog2c(g.M), ilog2c(g.N), ilog2c(g.K),
                                      g.levels, g.epilogue, g.lower_only, g.ksplit};
  std::lock_guard<std::mutex> lk(g_tune_mu);   // one tuning at a time; look-ups are brief
  auto it = g_tune.find(key);
  if (it != g_tune.end()) return launch_choice(c, g, err_flag, it->second.choice);
  // Candidates: 128-wide tiles with k-step 32 / 16, 64-wide tiles (k-step 16, two CTAs per
  // SM), each with 8 / 16 m-tiles per group and the caller's split or half of it, and the
  // persistent kernel (8 / 16 m-tiles per group) where K <= 512 without a split.  Products
  // above ~10 ms of tensor work keep the default (their tiles fill the GPU many times over
  // and a trial run would cost more than any choice gains).
  const double work = (double)g.levels * (g.levels + 1) / 2 * 2.0 * g.M * g.N * g.K;
  TuneEntry e;
  e.choice = dflt;
  if (work > 2e13) {
    g_tune[key] = e;
    return launch_choice(c, g, err_flag, dflt);
  }
  std::vector<TcChoice> cands;
  // (bk, bn) = (32, 128), (16, 128), (16, 64), and the persistent kernel where K fits.
  for (int v : {0, 1, 2, 3}) {
    if (v == 3 && !persistent_ok(g)) continue;
    for (int gm : {8, 16})
      for (int sp : {g.ksplit, std::max(1, g.ksplit / 2)}) {
        TcChoice ch;
        ch.bk = v == 0 ? 32 : 16; ch.bn = v >= 2 ? 64 : 128; ch.persistent = v == 3;
        ch.group_m = gm; ch.ksplit = v == 3 ? 1 : sp;
        bool dup = false;
        for (const auto& x : cands)
          dup |= x.bk == ch.bk && x.bn == ch.bn && x.persistent == ch.persistent &&
                 x.group_m == gm && x.ksplit == ch.ksplit;
        if (!dup) cands.push_back(ch);
      }
  }
  cudaEvent_t ea = nullptr, eb = nullptr;
  THC_CUDA(c, cudaEventCreate(&ea));
  THC_CUDA(c, cudaEventCreate(&eb));
  float best = 0.f;
  int best_i = -1, last = -1;
  int st = THC_OK;
  for (size_t i = 0; i < cands.size() && st == THC_OK; i++) {
    cudaEventRecord(ea, c->stream);
    st = launch_choice(c, g, err_flag, cands[i]);
    cudaEventRecord(eb, c->stream);
    if (st) break;
    if (cudaEventSynchronize(eb) != cudaSuccess) { st = THC_ERR_CUDA; break; }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ea, eb);
    last = (int)i;
    if (best_i < 0 || ms < best) { best = ms; best_i = (int)i; }
  }
  cudaEventDestroy(ea);
  cudaEventDestroy(eb);
  if (st) return st;
  e.choice = cands[best_i];
  e.us = 1e3f * best;
  e.candidates = (int)cands.size();
  g_tune[key] = e;
  // The result in C must be the chosen launch's.
  if (last != best_i) return launch_choice(c, g, err_flag, e.choice);
  return THC_OK;
}

}  // namespace thc
