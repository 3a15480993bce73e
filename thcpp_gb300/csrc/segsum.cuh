// Group-parallel evaluation of a sequential FP64 sum of non-negative terms, bit-identical to
// the left-to-right loop `acc = acc + t[i]` (the reference's centroid sums,
// src/kmeans.cpp:121-126).
//
// warp_seqsum (seqsum.cuh) still walks the terms window by window; its loop-carried chain
// (exponent -> units -> prefix -> validity -> new sum) costs ~40 cycles per term on GB300,
// whose FP64 adds have 55-cycle latency.  This version removes the chain from all but a
// handful of steps:
//
//   1. an integer prefix sum of the terms (each truncated to a common fixed-point unit)
//      predicts the binade (biased exponent E_i) of every running sum s_i; a segment starts
//      wherever the prediction changes;
//   2. inside a segment every partial sum is on the grid g = 2^(E-1075), and one step is
//      the integer map r -> r + k_i (k_i = t_i / g rounded to nearest) or, when t_i / g is an
//      exact half, r -> r + kf_i + ((r + kf_i) & 1) (ties to even).  Both are maps
//      r -> r + c[r & 1]; such maps compose into maps of the same form, so a segmented
//      parallel scan gives each segment's composite (c0, c1);
//   3. one warp then walks the segments: the first step of a segment is a real FP64 add,
//      the rest of the segment is S -> S + c[S & 1] on the integer significand, valid when
//      the sum after the first step lies in the predicted binade and the segment's last
//      partial sum stays below 2^(E+1) (terms are non-negative, so the sums rise
//      monotonically).  A failed check, a negative or non-finite term, or too many
//      segments hands the rest of the chunk to warp_seqsum.  Every accepted step provably
//      rounds as the FP64 add would, so the result never depends on the prediction.
#pragma once
#include "seqsum.cuh"

namespace thc {

constexpr int kSegGroup = 128;               // threads per quantity
constexpr int kSegPer = 8;                   // terms per thread
constexpr int kSegChunk = kSegGroup * kSegPer;
constexpr int kSegMax = 96;                  // segments per chunk before falling back
constexpr int kSegWarps = kSegGroup / 32;

// Per-group shared scratch (one per quantity of the block).
struct SegScratch {
  double acc;
  int fall;
  int nseg;
  long long wtot[kSegWarps];
  int wemax[kSegWarps];
  int wlast_e[kSegWarps];
  int wfirst_start[kSegWarps];
  long long wc0[kSegWarps], wc1[kSegWarps];
  int wflags[kSegWarps];       // bit 0: a segment starts in the warp, bit 1: invalid step
  int wstarts[kSegWarps];
  int seg_pos[kSegMax];
  int seg_e[kSegMax];
  long long seg_c0[kSegMax];   // -1: the segment holds an invalid step
  long long seg_c1[kSegMax];
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

// The parity map of one non-start term t on the grid of biased exponent e.
__device__ __forceinline__ void seg_term(double t, int e, long long& c0, long long& c1, bool& bad)
{
  bool tie;
  long long k = seqsum_units(t, e - 1075, tie);
  bad = k >= (1LL << 53);
  if (bad) k = 0;
  c0 = tie ? k + (k & 1) : k;
  c1 = tie ? k + ((k + 1) & 1) : k;
}

// acc + t[0] + ... + t[cnt-1] (cnt <= kSegChunk, t in shared memory) by the group of
// kSegGroup threads `gt` = 0..kSegGroup-1 of this block, with the running sum in sc.acc.
// Every thread of the block must call it (it holds block-wide barriers); groups differ
// only in their data.  On return sc.acc holds the new sum.
__device__ __forceinline__ void group_seqsum(const double* t, int cnt, int gt, SegScratch& sc)
{
  const unsigned full = 0xffffffffu;
  const int lane = gt & 31, wg = gt >> 5;
  const int i0 = gt * kSegPer;
  const long long kLo = 1LL << 52, kHi = 1LL << 53;
  // ---- 1. terms, sanity, and the binade prediction from an integer prefix sum: every
  //         term truncated to units of 2^U, U chosen from the largest exponent so that the
  //         chunk's sum stays below 2^62 units (no FP64 instruction: GB300 issues those at
  //         two lanes per clock).
  // Terms are re-read from shared memory in every phase (registers stay below 64).
  auto term = [&](int u) -> double { return i0 + u < cnt ? t[i0 + u] : 0.0; };
  bool odd = false;
  int emax = 0;
#pragma unroll
  for (int u = 0; u < kSegPer; u++) {
    long long bb = __double_as_longlong(term(u));
    const int et = (int)((bb >> 52) & 0x7ff);
    odd |= bb < 0 || et == 0x7ff;
    emax = max(emax, et);
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) emax = max(emax, __shfl_xor_sync(full, emax, off));
  if (lane == 0) sc.wemax[wg] = emax;
  if (odd) sc.fall = 1;
  __syncthreads();
  const double acc0 = sc.acc;
  {
    const long long ab = __double_as_longlong(acc0);
    emax = (int)((ab >> 52) & 0x7ff);
    for (int w = 0; w < kSegWarps; w++) emax = max(emax, sc.wemax[w]);
  }
  // Sum < (cnt + 1) 2^(emax - 1022) <= 2^(emax - 1011); a unit is 2^(emax - 1073), so every
  // term and the sum have at most 62 integer bits and the truncation error of the prefix
  // is below 2^10 units.
  const int U = emax - 1073;
  auto units = [&](double x) -> long long {
    const long long xb = __double_as_longlong(x);
    const int ex = (int)((xb >> 52) & 0x7ff);
    long long m = xb & ((1LL << 52) - 1);
    if (ex) m |= 1LL << 52;
    const int sh = (ex ? ex : 1) - 1075 - U;     // x = m 2^sh units, sh <= -2
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
  long long excl = incl - run;
  if (lane == 31) sc.wtot[wg] = incl;
  __syncthreads();
  long long base = units(acc0) + excl;
  for (int w = 0; w < wg; w++) base += sc.wtot[w];
  // Predicted biased exponent of each running sum (0 when it is below one unit).
  int E[kSegPer];
#pragma unroll
  for (int u = 0; u < kSegPer; u++) {
    const long long P = base + loc[u];
    E[u] = P > 0 ? (63 - __clzll(P)) + U + 1023 : 0;
  }
  int prev_e = __shfl_up_sync(full, E[kSegPer - 1], 1);
  if (lane == 31) sc.wlast_e[wg] = E[kSegPer - 1];
  __syncthreads();
  if (lane == 0) prev_e = wg > 0 ? sc.wlast_e[wg - 1] : -1;
  // ---- 2. segment starts and the thread's segmented composite
  unsigned stm = 0;   // bit u: element i0 + u starts a segment
#pragma unroll
  for (int u = 0; u < kSegPer; u++) {
    const int pe = u ? E[u - 1] : prev_e;
    if (i0 + u < cnt && (i0 + u == 0 || E[u] != pe)) stm |= 1u << u;
  }
  long long a0 = 0, a1 = 0;
  int af = 0;                  // bit 0 reset inside, bit 1 invalid
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
  int nst = __popc(stm);
  // Warp-level segmented inclusive scan: (x then y) = y if y resets, else composite.
  long long s0 = a0, s1 = a1;
  int sf = af, sn = nst;
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
  if (lane == 31) {
    sc.wc0[wg] = s0; sc.wc1[wg] = s1; sc.wflags[wg] = sf; sc.wstarts[wg] = sn;
  }
  if (lane == 0) sc.wfirst_start[wg] = stm & 1;
  __syncthreads();
  // Prefix of everything before this thread: the earlier warps, then the earlier lanes.
  long long p0 = 0, p1 = 0;
  int pf = 0, pn = 0, total = 0;
  for (int w = 0; w < kSegWarps; w++) {
    if (w < wg) {
      long long y0 = sc.wc0[w], y1 = sc.wc1[w];
      int yf = sc.wflags[w];
      if (yf & 1) { p0 = y0; p1 = y1; pf = yf; }
      else { seg_compose(p0, p1, y0, y1); p0 = y0; p1 = y1; pf |= yf & 2; }
      pn += sc.wstarts[w];
    }
    total += sc.wstarts[w];
  }
  if (ef & 1) { p0 = e0; p1 = e1; pf = ef; }
  else { seg_compose(p0, p1, e0, e1); p0 = e0; p1 = e1; pf |= ef & 2; }
  pn += en;
  const bool overflow = total > kSegMax;
  // ---- 3. segment table: start position and exponent, end composite
  if (!overflow) {
    unsigned next_start = __shfl_down_sync(full, stm & 1, 1);
    if (lane == 31) next_start = wg + 1 < kSegWarps ? sc.wfirst_start[wg + 1] : 0;
    int sidx = pn - 1;
    long long c0 = p0, c1 = p1;
    bool cbad = (pf & 2) != 0;
#pragma unroll
    for (int u = 0; u < kSegPer; u++) {
      const int i = i0 + u;
      if (i >= cnt) continue;
      if (stm >> u & 1) {
        sidx++;
        sc.seg_pos[sidx] = i;
        sc.seg_e[sidx] = E[u];
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
  if (gt == 0) sc.nseg = overflow ? -1 : total;
  __syncthreads();
  // ---- 4. one warp walks the segments (all lanes alike); fallback on any failed check
  if (wg == 0) {
    double acc = sc.acc;
    const int nseg = sc.nseg;
    if (sc.fall || nseg < 0) {
      acc = warp_seqsum(acc, t, cnt);
    } else {
      for (int j = 0; j < nseg; j++) {
        const int a = sc.seg_pos[j];
        const int bnd = (j + 1 < nseg ? sc.seg_pos[j + 1] : cnt) - 1;
        acc = __dadd_rn(acc, t[a]);
        if (bnd == a) continue;
        const long long ab = __double_as_longlong(acc);
        const int ea = (int)((ab >> 52) & 0x7ff);
        const long long S = (ab & (kLo - 1)) + kLo;
        const long long c0 = sc.seg_c0[j];
        const long long R = S + ((S & 1) ? sc.seg_c1[j] : c0);
        if (ab > 0 && ea >= 1 && ea < 0x7fe && ea == sc.seg_e[j] && c0 >= 0 && R < kHi) {
          acc = __longlong_as_double(((long long)ea << 52) | (R - kLo));
        } else {
          acc = warp_seqsum(acc, t + a + 1, cnt - a - 1);
          break;
        }
      }
    }
    if (lane == 0) {
      sc.acc = acc;
      sc.fall = 0;
    }
  }
}

}  // namespace thc
