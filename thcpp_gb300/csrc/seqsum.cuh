// Warp-parallel evaluation of a sequential FP64 sum with the sequential rounding.
//
// The reference accumulates several quantities with plain loops `acc = acc + t[i]` in
// ascending order (centroid sums, src/kmeans.cpp:121-126; the normed difference,
// src/kmeans.cpp:22-38).  Bit-identical results need the same rounding at every step, so
// the chain cannot be reassociated; on GB300 a dependent FP64 add is long-latency, which
// makes a 1000-term chain cost tens of microseconds.
//
// Observation: while the running sum stays inside one binade [2^e, 2^(e+1)), every partial
// sum lies on the grid of spacing g = 2^(e-52), and for an addend t with exact result inside
// the same binade, fl(acc + t) = acc + round_g(t): the rounding of t to a multiple of g
// (round-to-nearest; exact halves -- ties -- are left to the FP64 unit because their
// direction depends on the parity of the running sum).  Integers add exactly, so 32 steps
// become one warp prefix sum of int64 multiples of g.  The first step whose result would
// leave the binade (or that holds a tie, a NaN or an infinity) is executed as a real FP64
// add, after which the binade is re-read.  The result equals the sequential loop bit for
// bit: every step is either the FP64 add itself or provably rounds to the same value.
#pragma once
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define THC_HD __host__ __device__ __forceinline__
#else
#define THC_HD inline
#endif

namespace thc {

THC_HD long long seqsum_bits(double x)
{
  long long b;
  memcpy(&b, &x, sizeof b);
  return b;
}

// Multiple of g = 2^ga (ga = unbiased exponent of the grid, i.e. acc's biased exponent
// - 1075) nearest to t, signed as t.  `flag` is set for ties, NaN/Inf and magnitudes
// too large to stay in the binade (those steps must be executed in FP64).
THC_HD long long seqsum_units(double t, int ga, bool& flag)
{
  unsigned long long tb = (unsigned long long)seqsum_bits(t);
  int et = (int)((tb >> 52) & 0x7ff);
  long long m = (long long)(tb & ((1ULL << 52) - 1));
  if (et) m |= 1LL << 52;
  int sh = ga - ((et ? et : 1) - 1075);   // t = m 2^(-sh) g
  long long k;
  flag = et == 0x7ff;
  if (sh <= 0) {
    k = (-sh >= 2) ? (1LL << 54) : (m << -sh);   // >= 2^53 g: always leaves the binade
  } else if (sh >= 55) {
    k = 0;                                        // |t| < g/4
  } else {
    k = m >> sh;
    long long rem = m & ((1LL << sh) - 1), half = 1LL << (sh - 1);
    if (rem > half) k++;
    else if (rem == half) flag = true;
  }
  return (tb >> 63) ? -k : k;
}

#if defined(__CUDACC__)
// acc + t[0] + ... + t[n-1] evaluated left to right in FP64 round-to-nearest, by one full
// warp (all lanes get the result).  t may live in shared or global memory.  A window covers
// 128 consecutive terms, four per lane (lane l holds terms 4l .. 4l+3 of the window).
__device__ __noinline__ double warp_seqsum(double acc, const double* t, int n)
{
  constexpr int TPL = 4, WIN = 32 * TPL;
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const long long kLo = 1LL << 52, kHi = 1LL << 53;
  int pos = 0;
  while (pos < n) {
    const long long ab = __double_as_longlong(acc);
    const int ea = (int)((ab >> 52) & 0x7ff);
    if (ab == 0 || ea == 0 || ea >= 0x7fe) {
      // Rare states, 32 terms at a time.  +0 stays +0 through zero terms and the first
      // nonzero term is then the sum exactly; a subnormal, near-overflow, infinite or NaN
      // running sum takes one FP64 add.
      const int j = pos + lane;
      const double tj = j < n ? t[j] : 0.0;
      if (ab == 0) {
        unsigned nz = __ballot_sync(full, tj != 0.0);
        if (!nz) { pos += 32; continue; }
        int z = __ffs(nz) - 1;
        acc = __shfl_sync(full, tj, z);
        pos += z + 1;
      } else {
        acc = __dadd_rn(acc, __shfl_sync(full, tj, 0));
        pos++;
      }
      continue;
    }
    const bool acc_neg = ab < 0;
    double tv[TPL];
    long long c[TPL];
    bool ok[TPL];
    long long run = 0;
#pragma unroll
    for (int u = 0; u < TPL; u++) {
      const int j = pos + TPL * lane + u;
      tv[u] = j < n ? t[j] : 0.0;
      bool flag;
      long long k = seqsum_units(tv[u], ea - 1075, flag);
      if (acc_neg) k = -k;
      if (j >= n) { k = 0; flag = false; }
      run += k;
      c[u] = run;
      ok[u] = !flag;
    }
    // Exclusive prefix of the lane totals (|run| <= 4 * 2^54: no overflow).
    long long incl = run;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      long long o = __shfl_up_sync(full, incl, off);
      if (lane >= off) incl += o;
    }
    const long long base = (ab & (kLo - 1)) + kLo + (incl - run);
    int ubad = TPL;
#pragma unroll
    for (int u = TPL - 1; u >= 0; u--) {
      const int j = pos + TPL * lane + u;
      const long long r = base + c[u];
      // Valid while the exact partial sums stay inside [2^e, 2^(e+1)): r == 2^52 only when
      // the step did not decrease the magnitude (else the exact value may lie below 2^e).
      const bool along = tv[u] == 0.0 || ((__double_as_longlong(tv[u]) < 0) == acc_neg);
      const bool good = j >= n || (ok[u] && r < kHi && (r > kLo || (r == kLo && along)));
      if (!good) ubad = u;
    }
    const unsigned badl = __ballot_sync(full, ubad < TPL);
    int m;
    if (badl) {
      const int L = __ffs(badl) - 1;
      m = TPL * L + __shfl_sync(full, ubad, L);
    } else {
      m = min(WIN, n - pos);
    }
    if (m > 0) {
      const int q = m - 1, ql = q / TPL, qu = q % TPL;
      long long rsel = base + c[0];
#pragma unroll
      for (int u = 1; u < TPL; u++)
        if (qu == u) rsel = base + c[u];
      const long long rm = __shfl_sync(full, rsel, ql);
      acc = __longlong_as_double((ab & (1LL << 63)) | ((long long)ea << 52) | (rm - kLo));
    }
    pos += m;
    if (badl) {   // the step that leaves the binade, or holds a tie: one FP64 add
      const int ql = m / TPL, qu = m % TPL;
      double tsel = tv[0];
#pragma unroll
      for (int u = 1; u < TPL; u++)
        if (qu == u) tsel = tv[u];
      acc = __dadd_rn(acc, __shfl_sync(full, tsel, ql));
      pos++;
    }
  }
  return acc;
}
#endif

}  // namespace thc
