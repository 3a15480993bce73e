// Warp-parallel evaluation of a sequential FP64 sum of non-negative terms, bit-identical to
// the left-to-right loop `acc = acc + t[i]` (the reference's centroid sums,
// src/kmeans.cpp:121-126).
//
// warp_seqsum (seqsum.cuh) walks the terms window by window; its loop-carried chain
// (exponent -> units -> prefix -> validity -> new sum) costs ~40 cycles per term on GB300,
// whose FP64 adds have 55-cycle latency.  This version removes the chain from all but a
// handful of steps of each 256-term window:
//
//   1. an integer prefix sum of the terms (each truncated to a common fixed-point unit)
//      predicts the binade (biased exponent E_i) of every running sum s_i; a segment starts
//      at the window's first term and wherever the prediction changes;
//   2. inside a segment every partial sum is on the grid g = 2^(E-1075), and one step is
//      the integer map r -> r + k_i (k_i = t_i / g rounded to nearest) or, when t_i / g is an
//      exact half, r -> r + kf_i + ((r + kf_i) & 1) (ties to even).  Both are maps
//      r -> r + c[r & 1]; such maps compose into maps of the same form, so a segmented
//      warp scan gives each segment's composite (c0, c1);
//   3. the warp then walks the segments: the first step of a segment is a real FP64 add,
//      the rest of the segment is S -> S + c[S & 1] on the integer significand, valid when
//      the sum after the first step lies in the predicted binade and the segment's last
//      partial sum stays below 2^(E+1) (terms are non-negative, so the sums rise
//      monotonically).  A failed check, a negative or non-finite term, or too many
//      segments hands the rest of the window to warp_seqsum.  Every accepted step provably
//      rounds as the FP64 add would, so the result never depends on the prediction.
// One warp per quantity, synchronised only with __syncwarp: no block barrier waits on the
// serial walk of another quantity.
#pragma once
#include "seqsum.cuh"

namespace thc {

constexpr int kSegPer = 8;                   // terms per lane
constexpr int kSegWin = 32 * kSegPer;        // terms per window
constexpr int kSegMax = 64;                  // segments per window before falling back

// Per-warp shared scratch: the segment table of the current window.
struct SegScratch {
  int nseg;                    // segments of the window, -1: walk it term by term
  int seg_pos[kSegMax];
  int seg_e[kSegMax];
  long long seg_c0[kSegMax];   // -1: the segment holds an invalid step
  long long seg_c1[kSegMax];
  double seg_t[kSegMax];       // the segment's first term
};

// Composite of the parity maps x then y: c_p = x_p + y_[(p + x_p) & 1].
__device__ __forceinline__ void seg_compose(long long x0, long long x1, long long& y0,
                                            long long& y1)
{
  long long n0 = x0 + ((x0 & 1) ? y1 : y0);
  long long n1 = x1 + (((1 + x1) & 1) ? y1 : y0);
  y0 = n0;
  y1 = n1;
}

// The parity map of one non-start term t (finite, non-negative) on the grid of biased
// exponent e, without branches so that the eight terms of a lane overlap.  A term of at
// least 2^52 grid units (shift <= 0) cannot stay inside the binade: flagged invalid.  In a
// segment predicted to stay at +0 (e == 0: leading zero terms of a quantity, e.g. rho x at
// x = 0) a step is valid only for t == +0, and it leaves the sum at +0 (c = 0).
__device__ __forceinline__ void seg_term(double t, int e, long long& c0, long long& c1, bool& bad)
{
  if (e == 0) {
    c0 = c1 = 0;
    bad = __double_as_longlong(t) != 0;
    return;
  }
  const unsigned long long tb = (unsigned long long)__double_as_longlong(t);
  const int et = (int)((tb >> 52) & 0x7ff);
  unsigned long long m = tb & ((1ULL << 52) - 1);
  if (et) m |= 1ULL << 52;
  const int sh = e - max(et, 1);                 // t = m 2^(-sh) grid units
  bad = sh <= 0;
  const int shc = min(max(sh, 1), 63);
  const unsigned long long kf = m >> shc;
  const unsigned long long rem = m & ((1ULL << shc) - 1);
  const unsigned long long half = 1ULL << (shc - 1);
  const bool tie = rem == half;
  const long long k = (long long)(kf + (rem > half ? 1 : 0));
  const long long f = (long long)kf;
  c0 = tie ? f + (f & 1) : k;
  c1 = tie ? f + ((f + 1) & 1) : k;
}

// Phases 1-3 for one window of cnt <= kSegWin terms: the segment table in sc (sc.nseg = -1
// when the window must be walked term by term).  acc_pred only steers the binade
// prediction; it need not be the exact running sum.  One full warp.
__device__ __noinline__ void seg_build(double acc_pred, const double* tw, int cnt, SegScratch& sc)
{
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int i0 = lane * kSegPer;
  auto term = [&](int u) -> double { return i0 + u < cnt ? tw[i0 + u] : 0.0; };
  // ---- 1. sanity and the binade prediction from an integer prefix sum: every term
  //         truncated to units of 2^U, U chosen from the largest exponent so that the
  //         window's sum stays below 2^62 units (no FP64 instruction).
  bool odd = false;
  int emax = (int)((__double_as_longlong(acc_pred) >> 52) & 0x7ff);
#pragma unroll
  for (int u = 0; u < kSegPer; u++) {
    const long long bb = __double_as_longlong(term(u));
    const int et = (int)((bb >> 52) & 0x7ff);
    odd |= bb < 0 || et == 0x7ff;
    emax = max(emax, et);
  }
  if (__any_sync(full, odd) || __double_as_longlong(acc_pred) < 0) {
    if (lane == 0) sc.nseg = -1;
    __syncwarp();
    return;
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) emax = max(emax, __shfl_xor_sync(full, emax, off));
  if (emax == 0) {             // zero or subnormal terms only: rare, plain walk
    if (lane == 0) sc.nseg = -1;
    __syncwarp();
    return;
  }
  // Sum < 257 * 2^(emax - 1022) < 2^(emax - 1013); a unit is 2^(emax - 1075), so the sum has
  // at most 62 integer bits and the truncation error of a prefix is below 2^8 units.
  const int U = emax - 1075;
  auto units = [&](double x) -> long long {
    const long long xb = __double_as_longlong(x);
    const int ex = (int)((xb >> 52) & 0x7ff);
    long long m = xb & ((1LL << 52) - 1);
    if (ex) m |= 1LL << 52;
    const int sh = (ex ? ex : 1) - 1075 - U;   // x = m 2^sh units, sh <= 0
    return sh <= -63 ? 0 : (m >> (-sh));
  };
  long long loc[kSegPer];
  long long run = 0;
#pragma unroll
  for (int u = 0; u < kSegPer; u++) {
    run += units(term(u));
    loc[u] = run;
  }
  long long incl = run;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    long long y = __shfl_up_sync(full, incl, off);
    if (lane >= off) incl += y;
  }
  const long long base = units(acc_pred) + incl - run;
  int E[kSegPer];
#pragma unroll
  for (int u = 0; u < kSegPer; u++) {
    const long long P = base + loc[u];
    E[u] = P > 0 ? (63 - __clzll(P)) + U + 1023 : 0;
  }
  int prev_e = __shfl_up_sync(full, E[kSegPer - 1], 1);
  if (lane == 0) prev_e = -1;
  // ---- 2. segment starts, the lane's segmented composite, the warp's segmented scan
  unsigned stm = 0;
#pragma unroll
  for (int u = 0; u < kSegPer; u++) {
    const int pe = u ? E[u - 1] : prev_e;
    if (i0 + u < cnt && (i0 + u == 0 || E[u] != pe)) stm |= 1u << u;
  }
  long long a0 = 0, a1 = 0;
  int af = 0;                  // bit 0: a segment starts in the lane, bit 1: invalid step
#pragma unroll
  for (int u = 0; u < kSegPer; u++) {
    if (i0 + u >= cnt) continue;
    if (stm >> u & 1) {
      a0 = a1 = 0;
      af = 1;
    } else {
      long long c0, c1;
      bool bad;
      seg_term(term(u), E[u], c0, c1, bad);
      seg_compose(a0, a1, c0, c1);
      a0 = c0;
      a1 = c1;
      if (bad) af |= 2;
    }
  }
  // (x then y) = y if y starts a segment, else their composite.
  long long s0 = a0, s1 = a1;
  int sf = af, sn = __popc(stm);
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    long long x0 = __shfl_up_sync(full, s0, off), x1 = __shfl_up_sync(full, s1, off);
    int xf = __shfl_up_sync(full, sf, off), xn = __shfl_up_sync(full, sn, off);
    if (lane >= off) {
      if (!(sf & 1)) {
        seg_compose(x0, x1, s0, s1);
        sf = (xf & 1) | ((xf | sf) & 2);
      }
      sn += xn;
    }
  }
  long long e0 = __shfl_up_sync(full, s0, 1), e1 = __shfl_up_sync(full, s1, 1);
  int ef = __shfl_up_sync(full, sf, 1), en = __shfl_up_sync(full, sn, 1);
  if (lane == 0) { e0 = e1 = 0; ef = 0; en = 0; }
  const int total = __shfl_sync(full, sn, 31);
  if (total > kSegMax) {
    if (lane == 0) sc.nseg = -1;
    __syncwarp();
    return;
  }
  // ---- 3. segment table: start position and exponent, end composite
  {
    unsigned next_start = __shfl_down_sync(full, stm & 1, 1);
    if (lane == 31) next_start = 0;
    int sidx = en - 1;
    long long c0 = e0, c1 = e1;
    bool cbad = (ef & 2) != 0;
#pragma unroll
    for (int u = 0; u < kSegPer; u++) {
      const int i = i0 + u;
      if (i >= cnt) continue;
      if (stm >> u & 1) {
        sidx++;
        sc.seg_pos[sidx] = i;
        sc.seg_e[sidx] = E[u];
        sc.seg_t[sidx] = term(u);
        c0 = c1 = 0;
        cbad = false;
      } else {
        long long d0, d1;
        bool bad;
        seg_term(term(u), E[u], d0, d1, bad);
        seg_compose(c0, c1, d0, d1);
        c0 = d0;
        c1 = d1;
        cbad |= bad;
      }
      const bool end = i == cnt - 1 || (u + 1 < kSegPer ? (stm >> (u + 1) & 1) : next_start);
      if (end) {
        sc.seg_c0[sidx] = cbad ? -1 : c0;
        sc.seg_c1[sidx] = c1;
      }
    }
  }
  if (lane == 0) sc.nseg = total;
  __syncwarp();
}

// Phase 4 for one window: the exact running sum acc advanced over the window's terms with
// the segment table built by seg_build.  One full warp; all lanes get the result.
__device__ __noinline__ double seg_walk(double acc, const double* tw, int cnt, const SegScratch& sc)
{
  const long long kLo = 1LL << 52, kHi = 1LL << 53;
  const int total = sc.nseg;
  if (total < 0) return warp_seqsum(acc, tw, cnt);
  // ---- 4. walk the segments (all lanes alike)
  for (int j = 0; j < total; j++) {
    const int a = sc.seg_pos[j];
    const int bnd = (j + 1 < total ? sc.seg_pos[j + 1] : cnt) - 1;
    acc = __dadd_rn(acc, tw[a]);
    if (bnd == a) continue;
    const long long ab = __double_as_longlong(acc);
    const int ea = (int)((ab >> 52) & 0x7ff);
    const long long S = (ab & (kLo - 1)) + kLo;
    const long long c0 = sc.seg_c0[j];
    if (ab == 0 && sc.seg_e[j] == 0 && c0 >= 0) continue;   // +0 through +0 terms
    const long long R = S + ((S & 1) ? sc.seg_c1[j] : c0);
    if (ab > 0 && ea >= 1 && ea < 0x7fe && ea == sc.seg_e[j] && c0 >= 0 && R < kHi) {
      acc = __longlong_as_double(((long long)ea << 52) | (R - kLo));
    } else {
      acc = warp_seqsum(acc, tw + a + 1, cnt - a - 1);
      break;
    }
  }
  return acc;
}

// A segment table held in registers: lane l holds entries l and l + 32.
struct SegRegs {
  int total;
  int pA, pB, eA, eB;
  long long aA, aB, bA, bB;
  double tA, tB;
};

// Loads a table from global memory into registers (one round trip; the loads are issued
// together and can be in flight while the warp walks the previous window).
__device__ __forceinline__ SegRegs seg_load(const SegScratch& sc, int cnt)
{
  const int lane = threadIdx.x & 31;
  SegRegs r;
  r.total = sc.nseg;
  const bool ha = lane < r.total, hb = lane + 32 < r.total;
  r.pA = ha ? sc.seg_pos[lane] : cnt;
  r.pB = hb ? sc.seg_pos[lane + 32] : cnt;
  r.eA = ha ? sc.seg_e[lane] : 0;
  r.eB = hb ? sc.seg_e[lane + 32] : 0;
  r.aA = ha ? sc.seg_c0[lane] : 0;
  r.aB = hb ? sc.seg_c0[lane + 32] : 0;
  r.bA = ha ? sc.seg_c1[lane] : 0;
  r.bB = hb ? sc.seg_c1[lane + 32] : 0;
  r.tA = ha ? sc.seg_t[lane] : 0.0;
  r.tB = hb ? sc.seg_t[lane + 32] : 0.0;
  return r;
}

// seg_walk with the table in registers, so the serial walk waits on no memory.
__device__ __forceinline__ double seg_walk_regs(double acc, const double* tw, int cnt,
                                                const SegRegs& r)
{
  const unsigned full = 0xffffffffu;
  const long long kLo = 1LL << 52, kHi = 1LL << 53;
  const int total = r.total;
  if (total < 0) return warp_seqsum(acc, tw, cnt);
  for (int j = 0; j < total; j++) {
    const int src = j & 31;
    const bool hi = j >= 32;
    const int a = __shfl_sync(full, hi ? r.pB : r.pA, src);
    const int jn = j + 1;
    const int nx = __shfl_sync(full, jn >= 32 ? r.pB : r.pA, jn & 31);
    const int bnd = (jn < total ? nx : cnt) - 1;
    const int e = __shfl_sync(full, hi ? r.eB : r.eA, src);
    const long long c0 = __shfl_sync(full, hi ? r.aB : r.aA, src);
    const long long c1 = __shfl_sync(full, hi ? r.bB : r.bA, src);
    const double t0 = __shfl_sync(full, hi ? r.tB : r.tA, src);
    acc = __dadd_rn(acc, t0);
    if (bnd == a) continue;
    const long long ab = __double_as_longlong(acc);
    if (ab == 0 && e == 0 && c0 >= 0) continue;   // +0 through +0 terms
    const int ea = (int)((ab >> 52) & 0x7ff);
    const long long S = (ab & (kLo - 1)) + kLo;
    const long long R = S + ((S & 1) ? c1 : c0);
    if (ab > 0 && ea >= 1 && ea < 0x7fe && ea == e && c0 >= 0 && R < kHi) {
      acc = __longlong_as_double(((long long)ea << 52) | (R - kLo));
    } else {
      acc = warp_seqsum(acc, tw + a + 1, cnt - a - 1);
      break;
    }
  }
  return acc;
}

// acc + t[0] + ... + t[n-1] evaluated left to right in FP64 round-to-nearest by one full
// warp (all lanes get the result); t in shared or global memory, sc private to the warp.
__device__ __noinline__ double warp_segsum(double acc, const double* t, int n, SegScratch& sc)
{
  for (int w0 = 0; w0 < n; w0 += kSegWin) {
    const int cnt = min(kSegWin, n - w0);
    seg_build(acc, t + w0, cnt, sc);
    acc = seg_walk(acc, t + w0, cnt, sc);
    __syncwarp();
  }
  return acc;
}

}  // namespace thc
