// k-means interpolating points on the GPU, bit-identical to one rank of the reference.
//
// Reference semantics (src/kmeans.cpp):
//   classify_grid_points (:88-106)  label[i] = first argmin_k sqrt(dx*dx + dy*dy + dz*dz),
//                                   dx = c_k - g_i, evaluated left to right without FMA.
//   update_centroids (:108-144)     w_k = sum rho_i, s_k = sum rho_i * g_i over the members
//                                   of cluster k in ascending i; c_k = s_k / w_k; any
//                                   w_k < 1e-8 is fatal.
//   normed_difference               scale * sqrt(sum_i ((a_i - b_i)/scale)^2) summed in
//   (src/matrix_operations.h:42-57) index order, scale = max|a| + max|b|.
//   kernel (:187-264)               iterate until diff < threshold or max_it, then
//                                   map_to_grid (:146-157): for each centroid the first
//                                   nearest grid point, sorted ascending.
//
// GPU layout (HBM): grid as SoA x[], y[], z[] in FP64 and FP32; two centroid buffers
// (current / new) in FP64 and FP32 SoA; two label buffers (this / previous iteration).
//
// Exactness:
//   * every FP64 operation on the reference's path uses the _rn intrinsics, so no FMA
//     contraction changes a rounding;
//   * the argmin compares squared distances first (sqrt is monotone, so d2 >= best_d2
//     can never win) and takes the correctly rounded sqrt only for candidates that can;
//     a candidate replaces the best only if its sqrt is strictly smaller, which keeps the
//     first index among equal sqrt values exactly as std::min_element does;
//   * per-cluster sums run in ascending grid order through a stable counting sort of
//     the labels (block histograms -> per-cluster scans -> stable warp scatter), then
//     each cluster's members are accumulated in that order by warp_seqsum, which
//     reproduces the sequential loop's rounding exactly (seqsum.cuh);
//   * the normed difference that is reported is the sequential sum in index order (again
//     warp_seqsum); the per-iteration convergence test uses a fixed-order approximation
//     and falls back to the exact sum whenever the two could decide differently.
// Mixed precision: an FP32 pass keeps the best and second-best squared distance and
// accepts its argmin only when the gap exceeds a proven bound on the FP32 error;
// every other point is queued and resolved by a warp-parallel FP64 scan with the exact
// semantics above.  The labels, and hence every later result, equal the FP64 path's.
#include <cuda_runtime.h>
#include <math_constants.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "isdf.cuh"
#include "seqsum.cuh"
#include "segsum.cuh"

namespace thc {

namespace {

constexpr int kAssignThreads = 256;
constexpr int kTile = 1024;       // centroids staged per shared-memory tile
constexpr int kBP = 512;          // points per histogram / scatter block
constexpr int kMapChunk = 1024;   // grid points per map_to_grid block

struct KmState {
  int iter;
  int done;
  int converged;
  int empty;
  int zero_fill;
  int final_buf;
  int recheck_n;
  int max_it;
  unsigned long long changed;
  long long rechecked_total;
  double diff;
  double pct;
  double threshold;
  double abound;        // |a| bound of the FP32 error estimate
  unsigned long long absmax[3];
  int bad_label;
  int pad2;
  unsigned long long bmin[3], bmax[3];   // grid bounding box (order-preserving bit patterns)
  int nbin[3];
  int nbins;
  double blo[3], binv[3];                // bin origin and inverse bin width
  double slack32;                        // absolute slack of the FP32 candidate bound
  int diff_exact;                        // st->diff came from the sequential sum
  int ticket;                            // blocks of km_sums finished this iteration
  int scan_ticket;                       // blocks of km_colscan finished this iteration
  int nwin;                              // windows of the exact sums this iteration
};

// One window of <= kSegWin consecutive terms of one cluster in the sorted term arrays.
struct KmWin {
  int pos;     // sorted position of the window's first term
  int cnt;     // terms in the window
  int first;   // sorted position of the cluster's first term
  int k;       // cluster
};

struct KmBufs {
  const double* gx; const double* gy; const double* gz;
  const float* fx; const float* fy; const float* fz;
  const double* rho;
  double* cen;     // [2][3][nmu]
  float* cen32;    // [2][3][nmu]
  int* labels;     // [2][ng]
  int* hist;       // [nmu][nb]
  int* total;      // [nmu]
  int* start;      // [nmu]
  int* member;     // [ng]
  double* terms;   // [3 nmu]
  int* recheck;    // [ng]
  double* log;     // [2][max_it]
  KmState* st;
  long long ng;
  int nmu;
  int nb;
  int* perm;       // [ng] point indices grouped by spatial bin
  int* pbin;       // [ng] bin of each point
  int* bcount;     // [nbins_max] counts, then offsets, then cursors
  int nbins_max;
  float* pf;       // [3][ng] FP32 coordinates in the binned order (pf[d][t] of point perm[t])
  // Window-parallel exact sums (nwin_max == 0: the one-kernel km_sums path).
  const double* tq;   // [4][ng] rho_i, rho_i x_i, rho_i y_i, rho_i z_i in point order
  double* sv;         // [4][ng] the same terms in sorted (cluster, ascending point) order
  KmWin* win;         // [nwin_max]
  int* wbase;         // [nmu + 1] first window of each cluster
  SegScratch* seg;    // [nwin_max][4] segment tables
  int nwin_max;
  int pad5;
};

__device__ __forceinline__ double d2_exact(double cx, double cy, double cz, double gx,
                                           double gy, double gz)
{
  double dx = __dsub_rn(cx, gx);
  double dy = __dsub_rn(cy, gy);
  double dz = __dsub_rn(cz, gz);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// Running first-argmin over sqrt distances fed in ascending index order.
struct ArgMin {
  double s, m;
  int k;
  // Index 0 until something compares smaller, as std::min_element does.
  __device__ void init() { s = CUDART_INF; m = CUDART_INF; k = 0; }
  __device__ __forceinline__ void push(double d2, int idx)
  {
    if (d2 < m) {
      double r = __dsqrt_rn(d2);
      if (r < s) { s = r; m = d2; k = idx; }
    }
  }
  // Combine with a partial result over a disjoint index set.
  __device__ __forceinline__ void merge(double s2, double m2, int k2)
  {
    if (s2 < s || (s2 == s && k2 < k)) { s = s2; m = m2; k = k2; }
  }
};

// Order-preserving map of a double to an unsigned key (for atomic min / max).
__device__ __forceinline__ unsigned long long dkey(double x)
{
  unsigned long long u = (unsigned long long)__double_as_longlong(x);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ULL);
}
__device__ __forceinline__ double dunkey(unsigned long long k)
{
  unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
  return __longlong_as_double((long long)u);
}

__global__ void km_prep(const double* __restrict__ grid, const double* __restrict__ rho_in,
                        const int* __restrict__ init_idx, KmBufs b)
{
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double* gx = const_cast<double*>(b.gx);
  double* gy = const_cast<double*>(b.gy);
  double* gz = const_cast<double*>(b.gz);
  float* fx = const_cast<float*>(b.fx);
  float* fy = const_cast<float*>(b.fy);
  float* fz = const_cast<float*>(b.fz);
  double* rho = const_cast<double*>(b.rho);
  double ax = 0.0, ay = 0.0, az = 0.0;
  if (i < b.ng) {
    double x = grid[3 * i], y = grid[3 * i + 1], z = grid[3 * i + 2];
    gx[i] = x; gy[i] = y; gz[i] = z;
    fx[i] = (float)x; fy[i] = (float)y; fz[i] = (float)z;
    const double r = rho_in[i];
    rho[i] = r;
    if (b.tq) {
      // The products of the reference's centroid loop (src/kmeans.cpp:121-126), rounded
      // once each; they do not change between iterations.
      double* tq = const_cast<double*>(b.tq);
      tq[i] = r;
      tq[b.ng + i] = __dmul_rn(r, x);
      tq[2 * b.ng + i] = __dmul_rn(r, y);
      tq[3 * b.ng + i] = __dmul_rn(r, z);
    }
    ax = fabs(x); ay = fabs(y); az = fabs(z);
  }
  for (int off = 16; off; off >>= 1) {
    ax = fmax(ax, __shfl_xor_sync(0xffffffffu, ax, off));
    ay = fmax(ay, __shfl_xor_sync(0xffffffffu, ay, off));
    az = fmax(az, __shfl_xor_sync(0xffffffffu, az, off));
  }
  if ((threadIdx.x & 31) == 0) {
    // Non-negative doubles order like their bit patterns.
    atomicMax(&b.st->absmax[0], (unsigned long long)__double_as_longlong(ax));
    atomicMax(&b.st->absmax[1], (unsigned long long)__double_as_longlong(ay));
    atomicMax(&b.st->absmax[2], (unsigned long long)__double_as_longlong(az));
  }
  for (int d = 0; d < 3; d++) {
    unsigned long long mn = ~0ULL, mx = 0ULL;
    if (i < b.ng) mn = mx = dkey(grid[3 * i + d]);
    for (int off = 16; off; off >>= 1) {
      unsigned long long o1 = __shfl_xor_sync(0xffffffffu, mn, off);
      unsigned long long o2 = __shfl_xor_sync(0xffffffffu, mx, off);
      mn = o1 < mn ? o1 : mn;
      mx = o2 > mx ? o2 : mx;
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&b.st->bmin[d], mn);
      atomicMax(&b.st->bmax[d], mx);
    }
  }
  if (i < b.nmu) {
    long long g = init_idx[i];
    for (int d = 0; d < 3; d++) {
      double v = grid[3 * g + d];
      b.cen[d * b.nmu + i] = v;
      b.cen32[d * b.nmu + i] = (float)v;
    }
  }
}

__global__ void km_finish_prep(KmState* st, long long ng, int nbins_max)
{
  // |a| <= |c| + |g| per component; centroids stay inside the grid's bounding box.
  double a2 = 0.0;
  for (int d = 0; d < 3; d++) {
    double m = __longlong_as_double((long long)st->absmax[d]);
    a2 += 4.0 * m * m;
  }
  st->abound = sqrt(a2);
  st->slack32 = 1e-4 * a2;
  // Spatial bins of ~128 points: cubic cells over the bounding box.
  double ext[3], vol = 1.0;
  for (int d = 0; d < 3; d++) {
    ext[d] = dunkey(st->bmax[d]) - dunkey(st->bmin[d]);
    if (!(ext[d] > 0.0)) ext[d] = 1.0;
    vol *= ext[d];
  }
  double h = cbrt(vol * 128.0 / (double)ng);
  int nb = 1;
  for (int d = 0; d < 3; d++) {
    int n = (int)ceil(ext[d] / h);
    n = n < 1 ? 1 : (n > 1024 ? 1024 : n);
    st->nbin[d] = n;
    nb *= n;
  }
  while (nb > nbins_max) {   // coarsen if the bin table would overflow
    nb = 1;
    for (int d = 0; d < 3; d++) {
      st->nbin[d] = (st->nbin[d] + 1) / 2;
      nb *= st->nbin[d];
    }
  }
  st->nbins = nb;
  for (int d = 0; d < 3; d++) {
    st->blo[d] = dunkey(st->bmin[d]);
    st->binv[d] = st->nbin[d] / ext[d];
  }
}

__global__ void km_bin_count(const double* __restrict__ grid, KmBufs b)
{
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= b.ng) return;
  const KmState* st = b.st;
  int bin = 0;
  for (int d = 0; d < 3; d++) {
    int q = (int)((grid[3 * i + d] - st->blo[d]) * st->binv[d]);
    q = q < 0 ? 0 : (q >= st->nbin[d] ? st->nbin[d] - 1 : q);
    bin = bin * st->nbin[d] + q;
  }
  b.pbin[i] = bin;
  atomicAdd(&b.bcount[bin], 1);
}

// Single block: counts -> exclusive offsets (bcount[0..nbins)), cursors zeroed after.
__global__ void km_bin_scan(KmBufs b)
{
  __shared__ int warp_sums[32];
  int n = b.st->nbins;
  int per = (n + blockDim.x - 1) / blockDim.x;
  int lo = threadIdx.x * per, hi = min(n, lo + per);
  int s = 0;
  for (int k = lo; k < hi; k++) s += b.bcount[k];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = s;
  for (int off = 1; off < 32; off <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
    int xw = w;
    for (int off = 1; off < 32; off <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, xw, off);
      if (lane >= off) xw += y;
    }
    warp_sums[lane] = xw - w;
  }
  __syncthreads();
  int run = warp_sums[wid] + x - s;
  for (int k = lo; k < hi; k++) {
    int c = b.bcount[k];
    b.bcount[k] = run;
    b.bcount[b.nbins_max + k] = 0;
    run += c;
  }
}

__global__ void km_bin_scatter(KmBufs b)
{
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= b.ng) return;
  int bin = b.pbin[i];
  int pos = b.bcount[bin] + atomicAdd(&b.bcount[b.nbins_max + bin], 1);
  b.perm[pos] = (int)i;
  // The binned order's own copy of the FP32 coordinates: the pruned kernels read them
  // coalesced instead of through perm (a dependent gather).
  b.pf[pos] = b.fx[i];
  b.pf[b.ng + pos] = b.fy[i];
  b.pf[2 * b.ng + pos] = b.fz[i];
}

// Ordered block-wide compaction of `flag` over the block's threads: returns this thread's
// slot (or -1) and adds the block's count to *total (all threads see the new total).
__device__ __forceinline__ int block_compact(bool flag, int* wsum, int* total)
{
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned bal = __ballot_sync(0xffffffffu, flag);
  if (lane == 0) wsum[wid] = __popc(bal);
  __syncthreads();
  int before = *total;
  for (int w = 0; w < wid; w++) before += wsum[w];
  int slot = flag ? before + __popc(bal & ((1u << lane) - 1u)) : -1;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = *total;
    for (int w = 0; w < nw; w++) t += wsum[w];
    *total = t;
  }
  __syncthreads();
  return slot;
}

// A final label of the pruned assign kernels, with the counting sort's histogram entry
// (cluster k, block of kBP consecutive point indices) and the changed-label count: the
// separate histogram pass is not needed on this path.
__device__ __forceinline__ void put_label(const KmBufs& b, int it, long long i, int k,
                                          unsigned& changed)
{
  b.labels[(size_t)(it & 1) * b.ng + i] = k;
  atomicAdd(&b.hist[(size_t)k * b.nb + i / kBP], 1);
  if (it > 0 && b.labels[(size_t)((it + 1) & 1) * b.ng + i] != k) changed++;
}

// Warp sums of the changed-label counts into the state (whole warp).
__device__ __forceinline__ void flush_changed(KmState* st, unsigned changed)
{
  for (int off = 16; off; off >>= 1) changed += __shfl_xor_sync(0xffffffffu, changed, off);
  if ((threadIdx.x & 31) == 0 && changed) atomicAdd(&st->changed, (unsigned long long)changed);
}

constexpr int kPruneMax = 2048;   // candidate centroids kept in shared memory per tile

// FP64 assign with exact spatial pruning.  A tile is 256 consecutive points of the
// binned order.  With lb(c) / ub(c) the smallest / largest squared distance from centroid
// c to the tile's bounding box and U = min_c ub(c), every point's nearest centroid has
// squared distance <= U; a centroid with lb(c) > U (1 + 1e-9) is farther from every point
// of the tile than its nearest centroid by a relative margin far above the rounding of
// either bound or of the distance itself, so it can neither win nor tie after sqrt.  The
// kept centroids are scanned in ascending index order with the exact semantics.
__global__ void __launch_bounds__(kAssignThreads) km_assign64p(KmBufs b)
{
  const KmState* st = b.st;
  if (st->done) return;
  int it = st->iter;
  const double* cx = b.cen + (size_t)(it & 1) * 3 * b.nmu;
  const double* cy = cx + b.nmu;
  const double* cz = cy + b.nmu;
  extern __shared__ unsigned char sm[];
  int* cand = (int*)sm;
  double* ccx = (double*)(sm + sizeof(int) * kPruneMax);
  double* ccy = ccx + kPruneMax;
  double* ccz = ccy + kPruneMax;
  __shared__ double red[3][2][kAssignThreads / 32];
  __shared__ double uw[kAssignThreads / 32];
  __shared__ int wsum[kAssignThreads / 32];
  __shared__ int ncand;
  long long t = blockIdx.x * (long long)kAssignThreads + threadIdx.x;
  bool valid = t < b.ng;
  long long i = valid ? b.perm[t] : 0;
  double g[3] = {0, 0, 0};
  if (valid) { g[0] = b.gx[i]; g[1] = b.gy[i]; g[2] = b.gz[i]; }
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double lo[3], hi[3];
  for (int d = 0; d < 3; d++) {
    double mn = valid ? g[d] : CUDART_INF, mx = valid ? g[d] : -CUDART_INF;
    for (int off = 16; off; off >>= 1) {
      mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, off));
      mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    }
    if (lane == 0) { red[d][0][wid] = mn; red[d][1][wid] = mx; }
  }
  if (threadIdx.x == 0) ncand = 0;
  __syncthreads();
  for (int d = 0; d < 3; d++) {
    lo[d] = red[d][0][0];
    hi[d] = red[d][1][0];
    for (int w = 1; w < kAssignThreads / 32; w++) {
      lo[d] = fmin(lo[d], red[d][0][w]);
      hi[d] = fmax(hi[d], red[d][1][w]);
    }
  }
  // U = min over centroids of the largest squared distance to the box.
  double u = CUDART_INF;
  for (int k = threadIdx.x; k < b.nmu; k += kAssignThreads) {
    double c3[3] = {cx[k], cy[k], cz[k]}, ub = 0.0;
    for (int d = 0; d < 3; d++) {
      double a = c3[d] - lo[d], e = c3[d] - hi[d];
      ub += fmax(a * a, e * e);
    }
    u = fmin(u, ub);
  }
  for (int off = 16; off; off >>= 1) u = fmin(u, __shfl_xor_sync(0xffffffffu, u, off));
  if (lane == 0) uw[wid] = u;
  __syncthreads();
  double U = uw[0];
  for (int w = 1; w < kAssignThreads / 32; w++) U = fmin(U, uw[w]);
  double cut = U * (1.0 + 1e-9);
  for (int kb = 0; kb < b.nmu; kb += kAssignThreads) {
    int k = kb + threadIdx.x;
    bool keep = false;
    double c3[3] = {0, 0, 0};
    if (k < b.nmu) {
      c3[0] = cx[k]; c3[1] = cy[k]; c3[2] = cz[k];
      double lb = 0.0;
      for (int d = 0; d < 3; d++) {
        double v = fmax(0.0, fmax(lo[d] - c3[d], c3[d] - hi[d]));
        lb += v * v;
      }
      keep = lb <= cut;
    }
    int slot = block_compact(keep, wsum, &ncand);
    if (slot >= 0 && slot < kPruneMax) {
      cand[slot] = k; ccx[slot] = c3[0]; ccy[slot] = c3[1]; ccz[slot] = c3[2];
    }
  }
  __syncthreads();   // every thread reads every candidate written above
  int nc = ncand;
  ArgMin am;
  am.init();
  if (nc <= kPruneMax) {
    if (valid)
      for (int j = 0; j < nc; j++) am.push(d2_exact(ccx[j], ccy[j], ccz[j], g[0], g[1], g[2]), cand[j]);
  } else if (valid) {
    for (int k = 0; k < b.nmu; k++) am.push(d2_exact(cx[k], cy[k], cz[k], g[0], g[1], g[2]), k);
  }
  unsigned changed = 0;
  if (valid) put_label(b, it, i, am.k, changed);
  flush_changed(const_cast<KmState*>(st), changed);
}

// FP32 filter with pruning.  Bounds are computed in FP32 with a relative margin 1e-4 and
// an absolute slack 1e-4 |a|^2, far above their FP32 rounding, so the FP64 nearest
// centroid is always kept; the margin test and the FP64 recheck then work as in km_assign32.
__global__ void __launch_bounds__(kAssignThreads) km_assign32p(KmBufs b)
{
  KmState* st = b.st;
  if (st->done) return;
  int it = st->iter;
  const float* cx = b.cen32 + (size_t)(it & 1) * 3 * b.nmu;
  const float* cy = cx + b.nmu;
  const float* cz = cy + b.nmu;
  extern __shared__ unsigned char sm[];
  int* cand = (int*)sm;
  float* ccx = (float*)(sm + sizeof(int) * kPruneMax);
  float* ccy = ccx + kPruneMax;
  float* ccz = ccy + kPruneMax;
  __shared__ float red[3][2][kAssignThreads / 32];
  __shared__ float uw[kAssignThreads / 32];
  __shared__ int wsum[kAssignThreads / 32];
  __shared__ int ncand;
  long long t = blockIdx.x * (long long)kAssignThreads + threadIdx.x;
  bool valid = t < b.ng;
  long long i = valid ? b.perm[t] : 0;
  float g[3] = {0, 0, 0};
  if (valid) { g[0] = b.pf[t]; g[1] = b.pf[b.ng + t]; g[2] = b.pf[2 * b.ng + t]; }
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float lo[3], hi[3];
  for (int d = 0; d < 3; d++) {
    float mn = valid ? g[d] : INFINITY, mx = valid ? g[d] : -INFINITY;
    for (int off = 16; off; off >>= 1) {
      mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, off));
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    }
    if (lane == 0) { red[d][0][wid] = mn; red[d][1][wid] = mx; }
  }
  if (threadIdx.x == 0) ncand = 0;
  __syncthreads();
  for (int d = 0; d < 3; d++) {
    lo[d] = red[d][0][0];
    hi[d] = red[d][1][0];
    for (int w = 1; w < kAssignThreads / 32; w++) {
      lo[d] = fminf(lo[d], red[d][0][w]);
      hi[d] = fmaxf(hi[d], red[d][1][w]);
    }
  }
  float u = INFINITY;
  for (int k = threadIdx.x; k < b.nmu; k += kAssignThreads) {
    float c3[3] = {cx[k], cy[k], cz[k]}, ub = 0.f;
    for (int d = 0; d < 3; d++) {
      float a = c3[d] - lo[d], e = c3[d] - hi[d];
      ub += fmaxf(a * a, e * e);
    }
    u = fminf(u, ub);
  }
  for (int off = 16; off; off >>= 1) u = fminf(u, __shfl_xor_sync(0xffffffffu, u, off));
  if (lane == 0) uw[wid] = u;
  __syncthreads();
  float U = uw[0];
  for (int w = 1; w < kAssignThreads / 32; w++) U = fminf(U, uw[w]);
  float cut = U * (1.0f + 1e-4f) + (float)st->slack32;
  for (int kb = 0; kb < b.nmu; kb += kAssignThreads) {
    int k = kb + threadIdx.x;
    bool keep = false;
    float c3[3] = {0, 0, 0};
    if (k < b.nmu) {
      c3[0] = cx[k]; c3[1] = cy[k]; c3[2] = cz[k];
      float lb = 0.f;
      for (int d = 0; d < 3; d++) {
        float v = fmaxf(0.f, fmaxf(lo[d] - c3[d], c3[d] - hi[d]));
        lb += v * v;
      }
      keep = lb <= cut;
    }
    int slot = block_compact(keep, wsum, &ncand);
    if (slot >= 0 && slot < kPruneMax) {
      cand[slot] = k; ccx[slot] = c3[0]; ccy[slot] = c3[1]; ccz[slot] = c3[2];
    }
  }
  __syncthreads();   // every thread reads every candidate written above
  int nc = ncand;
  bool amb = false;
  unsigned changed = 0;
  if (valid) {
    float m1 = INFINITY, m2 = INFINITY;
    int k1 = 0;
    if (nc <= kPruneMax) {
      for (int j = 0; j < nc; j++) {
        float dx = ccx[j] - g[0], dy = ccy[j] - g[1], dz = ccz[j] - g[2];
        float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, dx * dx));
        if (d2 < m1) { m2 = m1; m1 = d2; k1 = cand[j]; }
        else if (d2 < m2) { m2 = d2; }
      }
    } else {
      for (int k = 0; k < b.nmu; k++) {
        float dx = cx[k] - g[0], dy = cy[k] - g[1], dz = cz[k] - g[2];
        float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, dx * dx));
        if (d2 < m1) { m2 = m1; m1 = d2; k1 = k; }
        else if (d2 < m2) { m2 = d2; }
      }
    }
    const double uu = 5.9604644775390625e-08;
    double a = st->abound;
    double e1 = 2.0 * uu * (2.0 * sqrt((double)m1) * a + 5.0 * (double)m1);
    double e2 = 2.0 * uu * (2.0 * sqrt((double)m2) * a + 5.0 * (double)m2);
    if ((double)m2 - (double)m1 > e1 + e2 + 1e-300) put_label(b, it, i, k1, changed);
    else amb = true;
  }
  // FP64 rescue of the near ties, at once and by the whole warp, one point at a time: the
  // exact first argmin of the sqrt distances (as km_recheck) over the tile's candidates in
  // ascending index order, which hold the FP64 nearest centroid.
  unsigned todo = __ballot_sync(0xffffffffu, amb);
  if (todo && lane == 0) atomicAdd(&st->recheck_n, __popc(todo));
  const double* px = b.cen + (size_t)(it & 1) * 3 * b.nmu;
  const double* py = px + b.nmu;
  const double* pz = py + b.nmu;
  while (todo) {
    const int p = __ffs(todo) - 1;
    todo &= todo - 1;
    const long long ip = __shfl_sync(0xffffffffu, i, p);
    const double gx = b.gx[ip], gy = b.gy[ip], gz = b.gz[ip];
    ArgMin am;
    am.init();
    if (nc <= kPruneMax) {
      for (int j = lane; j < nc; j += 32) {
        const int k = cand[j];
        am.push(d2_exact(px[k], py[k], pz[k], gx, gy, gz), k);
      }
    } else {
      for (int k = lane; k < b.nmu; k += 32) am.push(d2_exact(px[k], py[k], pz[k], gx, gy, gz), k);
    }
    for (int off = 16; off; off >>= 1) {
      double s2 = __shfl_xor_sync(0xffffffffu, am.s, off);
      double m2 = __shfl_xor_sync(0xffffffffu, am.m, off);
      int k2 = __shfl_xor_sync(0xffffffffu, am.k, off);
      am.merge(s2, m2, k2);
    }
    if (lane == 0) put_label(b, it, ip, am.k, changed);
  }
  flush_changed(st, changed);
}

// FP64 assign: one thread per grid point, centroids staged through shared memory.
__global__ void __launch_bounds__(kAssignThreads) km_assign64(KmBufs b)
{
  const KmState* st = b.st;
  if (st->done) return;
  int it = st->iter;
  const double* cx = b.cen + (size_t)(it & 1) * 3 * b.nmu;
  const double* cy = cx + b.nmu;
  const double* cz = cy + b.nmu;
  __shared__ double sx[kTile], sy[kTile], sz[kTile];
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  bool valid = i < b.ng;
  double gx = 0, gy = 0, gz = 0;
  if (valid) { gx = b.gx[i]; gy = b.gy[i]; gz = b.gz[i]; }
  ArgMin am;
  am.init();
  for (int t = 0; t < b.nmu; t += kTile) {
    int n = min(kTile, b.nmu - t);
    __syncthreads();
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      sx[j] = cx[t + j]; sy[j] = cy[t + j]; sz[j] = cz[t + j];
    }
    __syncthreads();
    if (valid) {
#pragma unroll 4
      for (int j = 0; j < n; j++) am.push(d2_exact(sx[j], sy[j], sz[j], gx, gy, gz), t + j);
    }
  }
  if (valid) b.labels[(size_t)(it & 1) * b.ng + i] = am.k;
}

// FP32 filter.  With u = 2^-24, inputs rounded to FP32 and the FP32 evaluation
//   |d2_32 - d2_64| <= u (2 |d| |a| + 5 d2) + O(u^2),   a_i = |c_i| + |g_i|,
// so a gap m2 - m1 > E(m1) + E(m2) with E(m) = 2u (2 sqrt(m) |a| + 5 m) (a factor-2
// margin for the O(u^2) terms and the evaluation of E itself) proves that every other
// centroid is strictly farther in FP64 than the FP32 winner, hence also after sqrt.
__global__ void __launch_bounds__(kAssignThreads) km_assign32(KmBufs b)
{
  KmState* st = b.st;
  if (st->done) return;
  int it = st->iter;
  const float* cx = b.cen32 + (size_t)(it & 1) * 3 * b.nmu;
  const float* cy = cx + b.nmu;
  const float* cz = cy + b.nmu;
  __shared__ float sx[kTile], sy[kTile], sz[kTile];
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  bool valid = i < b.ng;
  float gx = 0, gy = 0, gz = 0;
  if (valid) { gx = b.fx[i]; gy = b.fy[i]; gz = b.fz[i]; }
  float m1 = INFINITY, m2 = INFINITY;
  int k1 = 0;
  for (int t = 0; t < b.nmu; t += kTile) {
    int n = min(kTile, b.nmu - t);
    __syncthreads();
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      sx[j] = cx[t + j]; sy[j] = cy[t + j]; sz[j] = cz[t + j];
    }
    __syncthreads();
    if (valid) {
#pragma unroll 8
      for (int j = 0; j < n; j++) {
        float dx = sx[j] - gx, dy = sy[j] - gy, dz = sz[j] - gz;
        float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, dx * dx));
        if (d2 < m1) { m2 = m1; m1 = d2; k1 = t + j; }
        else if (d2 < m2) { m2 = d2; }
      }
    }
  }
  if (!valid) return;
  const double u = 5.9604644775390625e-08;  // 2^-24
  double a = st->abound;
  double e1 = 2.0 * u * (2.0 * sqrt((double)m1) * a + 5.0 * (double)m1);
  double e2 = 2.0 * u * (2.0 * sqrt((double)m2) * a + 5.0 * (double)m2);
  if ((double)m2 - (double)m1 > e1 + e2 + 1e-300) {
    b.labels[(size_t)(it & 1) * b.ng + i] = k1;
  } else {
    int slot = atomicAdd(&st->recheck_n, 1);
    b.recheck[slot] = (int)i;
  }
}

// FP64 recheck of queued points: one warp per point, lanes split the centroids.
__global__ void km_recheck(KmBufs b)
{
  const KmState* st = b.st;
  if (st->done) return;
  int it = st->iter;
  int n = st->recheck_n;
  const double* cx = b.cen + (size_t)(it & 1) * 3 * b.nmu;
  const double* cy = cx + b.nmu;
  const double* cz = cy + b.nmu;
  int lane = threadIdx.x & 31;
  long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long w = warp; w < n; w += nwarps) {
    long long i = b.recheck[w];
    double gx = b.gx[i], gy = b.gy[i], gz = b.gz[i];
    ArgMin am;
    am.init();
    for (int j = lane; j < b.nmu; j += 32) am.push(d2_exact(cx[j], cy[j], cz[j], gx, gy, gz), j);
    for (int off = 16; off; off >>= 1) {
      double s2 = __shfl_xor_sync(0xffffffffu, am.s, off);
      double m2 = __shfl_xor_sync(0xffffffffu, am.m, off);
      int k2 = __shfl_xor_sync(0xffffffffu, am.k, off);
      am.merge(s2, m2, k2);
    }
    if (lane == 0) b.labels[(size_t)(it & 1) * b.ng + i] = am.k;
  }
}

// Per-block label histogram (sparse write into the zeroed hist[k][block]) and the
// count of labels that changed since the previous iteration.
__global__ void km_hist(KmBufs b)
{
  KmState* st = b.st;
  if (st->done) return;
  int it = st->iter;
  extern __shared__ int sh[];
  for (int k = threadIdx.x; k < b.nmu; k += blockDim.x) sh[k] = 0;
  __syncthreads();
  const int* lab = b.labels + (size_t)(it & 1) * b.ng;
  const int* old = b.labels + (size_t)((it + 1) & 1) * b.ng;
  long long base = (long long)blockIdx.x * kBP;
  unsigned changed = 0;
  for (int t = threadIdx.x; t < kBP; t += blockDim.x) {
    long long i = base + t;
    if (i < b.ng) {
      int l = lab[i];
      if ((unsigned)l >= (unsigned)b.nmu) {   // never produced by the assign kernels
        atomicExch(&st->bad_label, 1);
        continue;
      }
      atomicAdd(&sh[l], 1);
      if (it > 0 && old[i] != l) changed++;
    }
  }
  for (int off = 16; off; off >>= 1) changed += __shfl_xor_sync(0xffffffffu, changed, off);
  if ((threadIdx.x & 31) == 0 && changed) atomicAdd(&st->changed, (unsigned long long)changed);
  __syncthreads();
  for (int k = threadIdx.x; k < b.nmu; k += blockDim.x)
    if (sh[k]) b.hist[(size_t)k * b.nb + blockIdx.x] = sh[k];
}

// Exclusive block-wide scan of one int per thread (all threads of the block).
__device__ int block_exscan(int v, int* warp_sums)
{
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
  for (int off = 1; off < 32; off <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  __syncthreads();
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
    int xw = w;
    for (int off = 1; off < 32; off <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, xw, off);
      if (lane >= off) xw += y;
    }
    warp_sums[lane] = xw - w;
  }
  __syncthreads();
  return warp_sums[wid] + x - v;
}

// Exclusive scan of the cluster totals into cluster start offsets (one block); with the
// window-parallel sums also the window table: cluster k's terms are cut into windows of
// kSegWin, numbered consecutively from wbase[k].
__device__ void kscan_block(KmBufs& b)
{
  __shared__ int warp_sums[32];
  int n = b.nmu;
  int per = (n + blockDim.x - 1) / blockDim.x;
  int lo = threadIdx.x * per, hi = min(n, lo + per);
  int s = 0, nw = 0;
  for (int k = lo; k < hi; k++) {
    int t = __ldcg(b.total + k);
    s += t;
    nw += (t + kSegWin - 1) / kSegWin;
  }
  int run = block_exscan(s, warp_sums);
  int wrun = b.nwin_max ? block_exscan(nw, warp_sums) : 0;
  for (int k = lo; k < hi; k++) {
    const int t = __ldcg(b.total + k);
    b.start[k] = run;
    if (b.nwin_max) {
      b.wbase[k] = wrun;
      for (int j = 0; j * kSegWin < t; j++) {
        KmWin w;
        w.pos = run + j * kSegWin;
        w.cnt = min(kSegWin, t - j * kSegWin);
        w.first = run;
        w.k = k;
        b.win[wrun++] = w;
      }
    }
    run += t;
  }
  if (b.nwin_max && hi == n && lo < hi) {
    b.wbase[n] = wrun;
    b.st->nwin = wrun;
  }
  if (b.nwin_max && n == 0 && threadIdx.x == 0) b.st->nwin = 0;
}

// One warp per cluster: exclusive scan of its block counts (in place) and its total.  The
// last block to finish (a ticket in the state) turns the totals into start offsets.
__global__ void __launch_bounds__(256) km_colscan(KmBufs b)
{
  KmState* st = b.st;
  if (st->done) return;
  __shared__ int last;
  int lane = threadIdx.x & 31;
  long long k = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  if (k < b.nmu) {
    int* h = b.hist + (size_t)k * b.nb;
    int carry = 0;
    for (int c = 0; c < b.nb; c += 32) {
      int j = c + lane;
      int v = j < b.nb ? h[j] : 0;
      int x = v;
      for (int off = 1; off < 32; off <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
      }
      if (j < b.nb) h[j] = carry + x - v;
      carry += __shfl_sync(0xffffffffu, x, 31);
    }
    if (lane == 0) b.total[k] = carry;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&st->scan_ticket, 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  kscan_block(b);
  if (threadIdx.x == 0) st->scan_ticket = 0;
}

// Stable scatter of point indices into per-cluster member lists.  The block's labels and
// every cluster's output offset are staged in shared memory by all threads; then warp 0
// ranks the points in ascending order, 32 at a time (lanes with equal labels take ranks
// from __match_any_sync, so each cluster keeps ascending grid order), and all threads
// write the members -- and, for the window-parallel sums, their four terms -- in place.
__global__ void __launch_bounds__(256) km_scatter(KmBufs b)
{
  if (b.st->done) return;
  const int it = b.st->iter;
  extern __shared__ int base[];          // nmu offsets
  __shared__ int slab[kBP];
  __shared__ int spos[kBP];
  const int* lab = b.labels + (size_t)(it & 1) * b.ng;
  const long long blk = (long long)blockIdx.x * kBP;
  for (int k = threadIdx.x; k < b.nmu; k += blockDim.x)
    base[k] = b.start[k] + b.hist[(size_t)k * b.nb + blockIdx.x];
  for (int t = threadIdx.x; t < kBP; t += blockDim.x) {
    long long i = blk + t;
    int l = i < b.ng ? lab[i] : -1;
    if (i < b.ng && (unsigned)l >= (unsigned)b.nmu) l = 0;  // flagged by km_hist
    slab[t] = l;
    spos[t] = -1;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const unsigned lt = (1u << lane) - 1u;
    for (int c = 0; c < kBP; c += 32) {
      const int l = slab[c + lane];
      const bool valid = l >= 0;
      const unsigned active = __ballot_sync(0xffffffffu, valid);
      if (!active) break;
      if (valid) {
        unsigned peers = __match_any_sync(active, l);
        int leader = __ffs(peers) - 1;
        spos[c + lane] = base[l] + __popc(peers & lt);
        __syncwarp(active);
        if (lane == leader) base[l] += __popc(peers);
      }
      __syncwarp();
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < kBP; t += blockDim.x) {
    const int pos = spos[t];
    if (pos < 0) continue;
    const long long i = blk + t;
    b.member[pos] = (int)i;
    if (b.sv) {
#pragma unroll
      for (int q = 0; q < 4; q++) b.sv[(size_t)q * b.ng + pos] = __ldg(b.tq + (size_t)q * b.ng + i);
    }
  }
}

__device__ __forceinline__ double block_max(double v, double* red)
{
  for (int off = 16; off; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
    for (int off = 16; off; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
    if (lane == 0) red[0] = v;
  }
  __syncthreads();
  return red[0];
}

// Fixed-order block sum (deterministic; not the reference's rounding).
__device__ __forceinline__ double block_sum(double v, double* red)
{
  for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    red[0] = t;
  }
  __syncthreads();
  return red[0];
}

// The terms ((a_i - c_i) / scale)^2 of the reference's normed difference in its index order
// i = 3k + d (centroid k, coordinate d), written to `terms`; returns scale.  Whole block.
__device__ double normdiff_terms(const KmBufs& b, const double* a, const double* c,
                                 double* terms, double* red)
{
  const int n3 = 3 * b.nmu;
  double ma = 0.0, mc = 0.0;
  for (int i = threadIdx.x; i < n3; i += blockDim.x) {
    ma = fmax(ma, fabs(__ldcg(a + i)));
    mc = fmax(mc, fabs(__ldcg(c + i)));
  }
  ma = block_max(ma, red);
  mc = block_max(mc, red);
  const double scale = __dadd_rn(ma, mc);
  for (int i = threadIdx.x; i < n3; i += blockDim.x) {
    int k = i / 3, d = i - 3 * k;
    double q = __ddiv_rn(__dsub_rn(__ldcg(a + d * b.nmu + k), __ldcg(c + d * b.nmu + k)), scale);
    terms[i] = __dmul_rn(q, q);
  }
  __syncthreads();
  return scale;
}

// End of an iteration's sums for cluster k (whole block; res[0..3] = w, x, y, z sums): the
// new centroid, its squared move, and -- in the last block to finish, found by a ticket in
// the state -- the convergence decision: the normed difference approximated by a
// fixed-order sum of squared centroid moves (relative deviation from the reference's value
// below (3 N_mu + 8) u), evaluated exactly when within 1e-10 of the threshold.
__device__ void sums_finish(const KmBufs& b, int k, int it, double* res, double* red, int& last)
{
  KmState* st = b.st;
  const int nmu = b.nmu;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* part = b.terms + 3 * (size_t)nmu;   // per-cluster squared move
  if (threadIdx.x < 3) {   // one coordinate each: c_d = sum_d / w (the reference's division)
    const int d = threadIdx.x;
    double* nc = b.cen + (size_t)((it + 1) & 1) * 3 * nmu;
    float* nc32 = b.cen32 + (size_t)((it + 1) & 1) * 3 * nmu;
    const double* oc = b.cen + (size_t)(it & 1) * 3 * nmu;
    const double v = __ddiv_rn(res[1 + d], res[0]);
    nc[d * nmu + k] = v;
    nc32[d * nmu + k] = (float)v;
    red[d] = __dsub_rn(v, oc[d * nmu + k]);
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (res[0] < 1e-8) atomicExch(&st->empty, 1);
    double sq = 0.0;
    for (int d = 0; d < 3; d++) sq = __fma_rn(red[d], red[d], sq);
    part[k] = sq;
    __threadfence();
    last = atomicAdd(&st->ticket, 1) == nmu - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // ---- last block: the convergence decision and the state update of this iteration ----
  if (*(volatile int*)&st->empty || *(volatile int*)&st->bad_label) {
    if (threadIdx.x == 0) { st->done = 1; st->iter = it + 1; st->ticket = 0; }
    return;
  }
  double v = 0.0;
  for (int i = threadIdx.x; i < nmu; i += blockDim.x) v += __ldcg(part + i);
  const double approx = sqrt(block_sum(v, red));
  const double thr = st->threshold;
  const bool exact = fabs(approx - thr) <= 1e-10 * thr;
  double diff = approx;
  if (exact) {
    const double* a = b.cen + (size_t)((it + 1) & 1) * 3 * nmu;
    const double* c = b.cen + (size_t)(it & 1) * 3 * nmu;
    double scale = normdiff_terms(b, a, c, b.terms, red);
    if (warp == 0) {
      double ssum = warp_seqsum(0.0, b.terms, 3 * nmu);
      if (lane == 0) res[0] = __dmul_rn(scale, __dsqrt_rn(ssum));
    }
    __syncthreads();
    diff = res[0];
  }
  if (threadIdx.x == 0) {
    st->diff_exact = exact;
    st->diff = diff;
    st->pct = 100.0 * (double)st->changed / (double)b.ng;
    b.log[it] = diff;
    b.log[st->max_it + it] = st->pct;
    st->changed = 0;
    st->rechecked_total += st->recheck_n;
    st->recheck_n = 0;
    st->final_buf = (it + 1) & 1;
    if (diff < thr) {
      st->converged = 1;
      st->done = 1;
    } else if (it + 1 >= st->max_it) {
      st->done = 1;
      st->zero_fill = !(diff > thr);
    }
    st->ticket = 0;
    st->iter = it + 1;
  }
}

// One block of sixteen warps per cluster.  All threads gather up to kSumCap members and
// form the products rho_i * g_i (each rounded on its own, as the reference's
// `rho[i] * grid[i*ndim]`).  Quantity q (0 = w, 1 = x, 2 = y, 3 = z) is summed strictly in
// ascending member order, rounding exactly as the reference's sequential loop
// (src/kmeans.cpp:121-126): every 256-term window of every quantity gets its own warp for
// the parallel part (seg_build, steered by an FP32 estimate of the running sum at the
// window's start), then one warp per quantity walks its windows in order (seg_walk) with
// the exact running sum.  The last block to finish (a ticket in the state) also takes the
// convergence decision of the iteration: the normed difference approximated by a
// fixed-order sum of squared centroid moves (relative deviation from the reference's value
// below (3 N_mu + 8) u), evaluated exactly when within 1e-10 of the threshold.
constexpr int kSumWin = kSegWin;                  // terms per window
constexpr int kSumWins = 4;                       // windows per quantity and chunk
constexpr int kSumCap = kSumWin * kSumWins;       // members per chunk
constexpr int kSumThreads = 32 * 4 * kSumWins;    // one warp per (quantity, window)
struct SumSmem {
  double sv[4][kSumCap];
  SegScratch tab[4][kSumWins];
  float wsum[4][kSumWins];
  double acc[4];
  double res[4];
  double red[32];
  int last;
};
__global__ void __launch_bounds__(kSumThreads) km_sums(KmBufs b)
{
  KmState* st = b.st;
  if (st->done) return;
  extern __shared__ __align__(16) unsigned char sum_smem[];
  SumSmem& sm = *reinterpret_cast<SumSmem*>(sum_smem);
  double* res = sm.res;
  double* red = sm.red;
  int& last = sm.last;
  const int it = st->iter;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tq = warp / kSumWins, tw = warp % kSumWins;   // this warp's window task
  const int k = blockIdx.x;
  const int s = b.start[k], n = b.total[k];
  if (threadIdx.x < 4) sm.acc[threadIdx.x] = 0.0;
  for (int base = 0; base < n; base += kSumCap) {
    const int cnt = min(kSumCap, n - base);
    __syncthreads();
    // Gather two members per thread: indices first, then the dependent loads.
    {
      int id[2];
#pragma unroll
      for (int r = 0; r < 2; r++) {
        const int m = r * kSumThreads + threadIdx.x;
        id[r] = m < cnt ? b.member[s + base + m] : -1;
      }
      double rv[2], xv[2], yv[2], zv[2];
#pragma unroll
      for (int r = 0; r < 2; r++) {
        if (id[r] < 0) continue;
        rv[r] = b.rho[id[r]];
        xv[r] = b.gx[id[r]];
        yv[r] = b.gy[id[r]];
        zv[r] = b.gz[id[r]];
      }
#pragma unroll
      for (int r = 0; r < 2; r++) {
        if (id[r] < 0) continue;
        const int m = r * kSumThreads + threadIdx.x;
        sm.sv[0][m] = rv[r];
        sm.sv[1][m] = __dmul_rn(rv[r], xv[r]);
        sm.sv[2][m] = __dmul_rn(rv[r], yv[r]);
        sm.sv[3][m] = __dmul_rn(rv[r], zv[r]);
      }
    }
    __syncthreads();
    const int w0 = tw * kSumWin;
    const int wcnt = max(0, min(kSumWin, cnt - w0));
    {   // FP32 estimate of the window's sum (it only steers the binade prediction)
      float f = 0.f;
      for (int i = lane; i < wcnt; i += 32) f += (float)sm.sv[tq][w0 + i];
      for (int off = 16; off; off >>= 1) f += __shfl_xor_sync(0xffffffffu, f, off);
      if (lane == 0) sm.wsum[tq][tw] = f;
    }
    __syncthreads();
    if (wcnt > 0) {
      double pred = sm.acc[tq];
      for (int v = 0; v < tw; v++) pred += (double)sm.wsum[tq][v];
      seg_build(pred, &sm.sv[tq][w0], wcnt, sm.tab[tq][tw]);
    }
    __syncthreads();
    if (warp < 4) {
      double acc = sm.acc[warp];
      for (int v = 0; v < kSumWins && v * kSumWin < cnt; v++)
        acc = seg_walk(acc, &sm.sv[warp][v * kSumWin], min(kSumWin, cnt - v * kSumWin),
                       sm.tab[warp][v]);
      if (lane == 0) sm.acc[warp] = acc;
    }
  }
  __syncthreads();
  if (threadIdx.x < 4) res[threadIdx.x] = sm.acc[threadIdx.x];
  __syncthreads();
  sums_finish(b, k, it, res, red, last);
}

// Window-parallel exact sums, phase 1: one warp per (window, quantity) builds the window's
// segment table (seg_build), steered by an FP32 estimate of the cluster's running sum at
// the window's start (the sum of the cluster's earlier terms; it only has to predict
// binades).  Windows are independent, so every SM takes part however uneven the clusters.
constexpr int kBuildThreads = 256;
__global__ void __launch_bounds__(kBuildThreads) km_sbuild(KmBufs b)
{
  const KmState* st = b.st;
  if (st->done) return;
  const int gw = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const int w = gw >> 2, q = gw & 3;
  if (w >= st->nwin) return;
  const int lane = threadIdx.x & 31;
  const KmWin wi = b.win[w];
  const double* t = b.sv + (size_t)q * b.ng;
  float f = 0.f;
  for (int i = wi.first + lane; i < wi.pos; i += 32) f += (float)t[i];
  for (int off = 16; off; off >>= 1) f += __shfl_xor_sync(0xffffffffu, f, off);
  seg_build((double)f, t + wi.pos, wi.cnt, b.seg[(size_t)w * 4 + q]);
}

// Phase 2: one block of four warps per cluster; warp q walks quantity q (0 = w, 1 = x,
// 2 = y, 3 = z) over the cluster's windows in order with the exact running sum, strictly in
// ascending member order as the reference's loop (src/kmeans.cpp:121-126).  Then the new
// centroid and, in the last block, the convergence decision (sums_finish).
__global__ void __launch_bounds__(128) km_swalk(KmBufs b)
{
  KmState* st = b.st;
  if (st->done) return;
  __shared__ double res[4];
  __shared__ double red[32];
  __shared__ int last;
  const int it = st->iter;
  const int k = blockIdx.x, q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w0 = b.wbase[k], w1 = b.wbase[k + 1];
  const double* t = b.sv + (size_t)q * b.ng;
  double acc = 0.0;
  if (w0 < w1) {
    // The next window's position and table are loaded while the current one is walked.
    KmWin wi = b.win[w0];
    SegRegs cur = seg_load(b.seg[(size_t)w0 * 4 + q], wi.cnt);
    for (int w = w0; w < w1; w++) {
      KmWin wn = wi;
      SegRegs nxt = cur;
      if (w + 1 < w1) {
        wn = b.win[w + 1];
        nxt = seg_load(b.seg[(size_t)(w + 1) * 4 + q], wn.cnt);
      }
      acc = seg_walk_regs(acc, t + wi.pos, wi.cnt, cur);
      wi = wn;
      cur = nxt;
    }
  }
  if (lane == 0) res[q] = acc;
  __syncthreads();
  sums_finish(b, k, it, res, red, last);
}

// The reference's normed difference of the last iteration, exactly (one block).
__global__ void __launch_bounds__(1024) km_normdiff_exact(KmBufs b)
{
  KmState* st = b.st;
  if (st->diff_exact || st->empty || st->iter < 1) return;
  __shared__ double red[32];
  __shared__ double out;
  const int it = st->iter - 1;
  const double* a = b.cen + (size_t)((it + 1) & 1) * 3 * b.nmu;
  const double* c = b.cen + (size_t)(it & 1) * 3 * b.nmu;
  const double scale = normdiff_terms(b, a, c, b.terms, red);
  __shared__ SegScratch scx;
  if (threadIdx.x < 32) {
    double ssum = warp_segsum(0.0, b.terms, 3 * b.nmu, scx);
    if (threadIdx.x == 0) out = __dmul_rn(scale, __dsqrt_rn(ssum));
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    st->diff = out;
    b.log[it] = out;
    st->diff_exact = 1;
  }
}

// Bounding box of each 256-point tile of the binned order, from the FP32 coordinates (for
// the pruned map_to_grid).
__global__ void km_tile_boxes(KmBufs b, float* box)
{
  __shared__ float red[6][8];
  long long t = blockIdx.x * 256LL + threadIdx.x;
  bool valid = t < b.ng;
  float g[3] = {valid ? b.pf[t] : 0.f, valid ? b.pf[b.ng + t] : 0.f,
                valid ? b.pf[2 * b.ng + t] : 0.f};
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int d = 0; d < 3; d++) {
    float mn = valid ? g[d] : INFINITY, mx = valid ? g[d] : -INFINITY;
    for (int off = 16; off; off >>= 1) {
      mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, off));
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    }
    if (lane == 0) { red[d][wid] = mn; red[3 + d][wid] = mx; }
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    int d = threadIdx.x;
    float v = red[d][0];
    for (int w = 1; w < 8; w++) v = d < 3 ? fminf(v, red[d][w]) : fmaxf(v, red[d][w]);
    box[(long long)blockIdx.x * 6 + d] = v;
  }
}

// map_to_grid with exact pruning: one block of kMapWarps warps per centroid, the warps
// taking every kMapWarps-th 32-tile stretch.  U = min over tiles of the largest squared
// distance from the centroid to the tile box bounds the nearest squared distance; only
// tiles whose smallest squared distance is <= U (1 + 1e-4) + slack32 are scanned.  The
// bounds are FP32 (the FP64 pipe runs two lanes per clock here); the margins are those of
// the pruned FP32 assign, far above the FP32 rounding of the boxes and distances, so the
// FP64 nearest point and every sqrt tie survive.  Tiles are not in grid-index order, so
// candidates merge on (sqrt distance, grid index), which keeps the reference's first-index
// rule (classify with the roles swapped, src/kmeans.cpp:146-150).
constexpr int kMapWarps = 8;
constexpr int kMapThreads = 32 * kMapWarps;
__global__ void __launch_bounds__(kMapThreads) km_map_pruned(KmBufs b, const float* __restrict__ box,
                                                             int ntiles, int* idx)
{
  const double* cen = b.cen + (size_t)b.st->final_buf * 3 * b.nmu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long k = blockIdx.x;
  if (k >= b.nmu) return;
  __shared__ float redf[kMapWarps];
  __shared__ double reds[kMapWarps];
  __shared__ int redk[kMapWarps];
  double c3[3] = {cen[k], cen[b.nmu + k], cen[2 * b.nmu + k]};
  const float* cf = b.cen32 + (size_t)b.st->final_buf * 3 * b.nmu;
  const float f3[3] = {cf[k], cf[b.nmu + k], cf[2 * b.nmu + k]};
  // Block minimum of one float per thread (every thread gets it).
  auto block_min = [&](float v) {
    for (int off = 16; off; off >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, off));
    __syncthreads();
    if (lane == 0) redf[warp] = v;
    __syncthreads();
    float m = redf[0];
    for (int w = 1; w < kMapWarps; w++) m = fminf(m, redf[w]);
    return m;
  };
  float u = INFINITY;
  for (int t = threadIdx.x; t < ntiles; t += kMapThreads) {
    float ub = 0.f;
    for (int d = 0; d < 3; d++) {
      float a = f3[d] - box[t * 6 + d], e = f3[d] - box[t * 6 + 3 + d];
      ub += fmaxf(a * a, e * e);
    }
    u = fminf(u, ub);
  }
  u = block_min(u);
  const float cut = u * (1.0f + 1e-4f) + (float)b.st->slack32;
  // The candidate tiles' points are scanned twice: first in FP32 for the smallest squared
  // distance m, then in FP64 only for points whose FP32 squared distance is within
  // m (1 + 1e-4) + slack32 -- a margin far above the FP32 rounding of the distances (the
  // same one the pruned assign uses) -- so the FP64 pipe, which GB300 runs at two lanes
  // per clock, sees a handful of points per centroid.
  float m32 = INFINITY;
  for (int pass = 0; pass < 2; pass++) {
    const float thr32 = pass ? m32 * (1.0f + 1e-4f) + (float)b.st->slack32 : 0.f;
    double bs = CUDART_INF, bm = CUDART_INF;
    int bk = 0x7fffffff;
    for (int t0 = warp * 32; t0 < ntiles; t0 += 32 * kMapWarps) {
      int t = t0 + lane;
      bool cand = false;
      if (t < ntiles) {
        float lb = 0.f;
        for (int d = 0; d < 3; d++) {
          float v = fmaxf(0.f, fmaxf(box[t * 6 + d] - f3[d], f3[d] - box[t * 6 + 3 + d]));
          lb += v * v;
        }
        cand = lb <= cut;
      }
      unsigned m = __ballot_sync(0xffffffffu, cand);
      while (m) {
        int tt = t0 + __ffs(m) - 1;
        m &= m - 1;
        long long p0 = (long long)tt * 256, p1 = min((long long)b.ng, p0 + 256);
        for (long long q = p0 + lane; q < p1; q += 32) {
          float dx = b.pf[q] - f3[0], dy = b.pf[b.ng + q] - f3[1], dz = b.pf[2 * b.ng + q] - f3[2];
          float d32 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, dx * dx));
          if (!pass) {
            m32 = fminf(m32, d32);
            continue;
          }
          if (d32 > thr32) continue;
          const int i = b.perm[q];
          if ((unsigned)i >= (unsigned)b.ng) {   // a binning permutation entry out of range
            atomicExch(&b.st->bad_label, 1);
            continue;
          }
          double d2 = d2_exact(b.gx[i], b.gy[i], b.gz[i], c3[0], c3[1], c3[2]);
          // Any order: a candidate can win on a smaller sqrt or on an equal sqrt and a
          // smaller index; equal sqrt values come from squared distances within a few ulps.
          if (d2 <= bm * (1.0 + 0x1p-50)) {
            double r = __dsqrt_rn(d2);
            if (r < bs || (r == bs && i < bk)) { bs = r; bk = i; bm = fmin(bm, d2); }
          }
        }
      }
    }
    if (!pass) {
      m32 = block_min(m32);
      continue;
    }
    for (int off = 16; off; off >>= 1) {
      double s2 = __shfl_xor_sync(0xffffffffu, bs, off);
      int k2 = __shfl_xor_sync(0xffffffffu, bk, off);
      if (s2 < bs || (s2 == bs && k2 < bk)) { bs = s2; bk = k2; }
    }
    if (lane == 0) { reds[warp] = bs; redk[warp] = bk; }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int w = 1; w < kMapWarps; w++)
        if (reds[w] < bs || (reds[w] == bs && redk[w] < bk)) { bs = reds[w]; bk = redk[w]; }
      idx[k] = bk;
    }
  }
}

// map_to_grid, part 1: each thread owns one centroid and scans one chunk of grid points.
__global__ void km_map_part(KmBufs b, double* part_s, int* part_i, int nch)
{
  const double* cen = b.cen + (size_t)b.st->final_buf * 3 * b.nmu;
  __shared__ double sx[kMapChunk], sy[kMapChunk], sz[kMapChunk];
  long long p0 = (long long)blockIdx.x * kMapChunk;
  int n = (int)min((long long)kMapChunk, b.ng - p0);
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    sx[j] = b.gx[p0 + j]; sy[j] = b.gy[p0 + j]; sz[j] = b.gz[p0 + j];
  }
  __syncthreads();
  int k = blockIdx.y * blockDim.x + threadIdx.x;
  if (k >= b.nmu) return;
  double cx = cen[k], cy = cen[b.nmu + k], cz = cen[2 * b.nmu + k];
  ArgMin am;
  am.init();
  // map_to_grid calls classify with the roles swapped: dx = g_j - c_k.
#pragma unroll 4
  for (int j = 0; j < n; j++) am.push(d2_exact(sx[j], sy[j], sz[j], cx, cy, cz), (int)(p0 + j));
  part_s[(size_t)k * nch + blockIdx.x] = am.s;
  part_i[(size_t)k * nch + blockIdx.x] = am.k;
}

__global__ void km_map_reduce(int nmu, int nch, const double* part_s, const int* part_i,
                              int* idx)
{
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nmu) return;
  double s = CUDART_INF;
  int best = 0;
  for (int c = 0; c < nch; c++) {
    double v = part_s[(size_t)k * nch + c];
    int i = part_i[(size_t)k * nch + c];
    if (v < s || (v == s && i < best)) { s = v; best = i; }
  }
  idx[k] = best;
}

// Single-block bitonic sort of the nmu indices (padded to a power of two) and the
// count of adjacent duplicates.
__global__ void km_sort(int* idx, int n, int npow2, int* dups)
{
  extern __shared__ int a[];
  for (int i = threadIdx.x; i < npow2; i += blockDim.x) a[i] = i < n ? idx[i] : 0x7fffffff;
  __syncthreads();
  for (int size = 2; size <= npow2; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < npow2; i += blockDim.x) {
        int j = i ^ stride;
        if (j > i) {
          bool up = (i & size) == 0;
          int x = a[i], y = a[j];
          if ((x > y) == up) { a[i] = y; a[j] = x; }
        }
      }
      __syncthreads();
    }
  }
  int d = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    idx[i] = a[i];
    if (i + 1 < n && a[i] == a[i + 1]) d++;
  }
  if (d) atomicAdd(dups, d);
}

}  // namespace

int kmeans_run(Ctx* c, const double* grid_in, const double* rho_in, long long ng, int nmu,
               const int* init_in, int max_it, double threshold, int* out_idx,
               thc_kmeans_stats* stats, KmAlloc* fixed)
{
  KmAlloc ws_alloc;
  ws_alloc.c = c;
  KmAlloc& al = fixed ? *fixed : ws_alloc;
  ProfScope prof_all(fixed ? nullptr : c, "kmeans");
  if (!grid_in || !rho_in || !init_in || !out_idx || ng <= 0 || nmu <= 0 || nmu > ng ||
      max_it < 1 || ng > 0x7fffffffLL)
    return set_error(c, THC_ERR_ARG, "thc_kmeans: invalid arguments");
  if (nmu > 16384) return set_error(c, THC_ERR_SHAPE, "thc_kmeans: nmu > 16384 unsupported");
  cudaStream_t s = c->stream;
  int st_status = 0;
  const double* grid = nullptr;
  if (!fixed) {
    grid = (const double*)to_device(c, grid_in, sizeof(double) * 3 * ng, WS_KM_IO, &st_status);
    if (st_status) return st_status;
  } else if (is_device_ptr(grid_in)) {
    grid = grid_in;
  } else {
    double* gs = (double*)al.get(WS_KM_IO, sizeof(double) * 3 * ng);
    if (!gs) return set_error(c, THC_ERR_NOMEM, "thc_kmeans: grid staging exceeds the scratch");
    THC_CUDA(c, cudaMemcpyAsync(gs, grid_in, sizeof(double) * 3 * ng, cudaMemcpyHostToDevice, s));
    grid = gs;
  }
  // rho and the initial indices share a second staging area after the grid copy.
  const double* rho = nullptr;
  const int* init = nullptr;
  {
    size_t rb = sizeof(double) * ng, ib = sizeof(int) * nmu;
    bool rd = is_device_ptr(rho_in), id = is_device_ptr(init_in);
    char* stage = nullptr;
    if (!rd || !id) {
      stage = (char*)al.get(WS_KM_IDX, rb + ib + 256);
      if (!stage) return set_error(c, THC_ERR_NOMEM, "thc_kmeans: staging");
    }
    if (rd) rho = rho_in;
    else {
      THC_CUDA(c, cudaMemcpyAsync(stage, rho_in, rb, cudaMemcpyHostToDevice, s));
      rho = (const double*)stage;
    }
    if (id) init = init_in;
    else {
      char* p = stage + ((rb + 255) / 256) * 256;
      THC_CUDA(c, cudaMemcpyAsync(p, init_in, ib, cudaMemcpyHostToDevice, s));
      init = (const int*)p;
    }
  }
  KmBufs b;
  memset(&b, 0, sizeof b);   // padding included: the bytes key the cached graph
  b.ng = ng;
  b.nmu = nmu;
  b.nb = (int)cdiv(ng, kBP);
  double* g64 = (double*)al.get(WS_KM_GRID, sizeof(double) * 4 * ng);
  float* g32 = (float*)al.get(WS_KM_GRID32, sizeof(float) * 6 * ng);
  double* cen = (double*)al.get(WS_KM_CENT, sizeof(double) * 6 * nmu);
  float* cen32 = (float*)al.get(WS_KM_CENT32, sizeof(float) * 6 * nmu);
  int* labels = (int*)al.get(WS_KM_LABELS, sizeof(int) * 2 * ng);
  int* hist = (int*)al.get(WS_KM_HIST, sizeof(int) * (size_t)nmu * b.nb);
  int* tot = (int*)al.get(WS_KM_TOTAL, sizeof(int) * 2 * nmu);
  int* member = (int*)al.get(WS_KM_MEMBER, sizeof(int) * ng);
  double* terms = (double*)al.get(WS_KM_TERMS, sizeof(double) * 4 * nmu);
  int* recheck = (int*)al.get(WS_KM_RECHECK, sizeof(int) * ng);
  KmState* st = (KmState*)al.get(WS_KM_STATE, sizeof(KmState) + 64);
  double* logb = (double*)al.get(WS_KM_LOG, sizeof(double) * 2 * max_it);
  int nch = (int)cdiv(ng, kMapChunk);
  double* part_s = (double*)al.get(WS_KM_PART, (sizeof(double) + sizeof(int)) * (size_t)nmu * nch + 64);
  const int nbins_max = (int)std::max<long long>(1024, ng / 32);
  int* permw = (int*)al.get(WS_KM_PERM, sizeof(int) * (2 * (size_t)ng + 2 * (size_t)nbins_max));
  if (!g64 || !g32 || !cen || !cen32 || !labels || !hist || !tot || !member || !terms ||
      !recheck || !st || !logb || !part_s || !permw)
    return set_error(c, THC_ERR_NOMEM, "thc_kmeans: workspace allocation failed");
  b.perm = permw;
  b.pbin = permw + ng;
  b.bcount = permw + 2 * ng;
  b.nbins_max = nbins_max;
  int* part_i = (int*)(part_s + (size_t)nmu * nch);
  b.gx = g64; b.gy = g64 + ng; b.gz = g64 + 2 * ng; b.rho = g64 + 3 * ng;
  b.fx = g32; b.fy = g32 + ng; b.fz = g32 + 2 * ng;
  b.pf = g32 + 3 * ng;
  b.cen = cen; b.cen32 = cen32; b.labels = labels; b.hist = hist; b.total = tot;
  b.start = tot + nmu; b.member = member; b.terms = terms; b.recheck = recheck;
  b.log = logb; b.st = st;
  if (!fixed) {
    // Window-parallel exact sums (the caller-provided fixed scratch keeps the one-kernel
    // sums, whose footprint is smaller).
    const long long nwin_max = ng / kSegWin + nmu + 1;
    double* svb = (double*)al.get(WS_KM_SV, sizeof(double) * 8 * ng);
    const size_t win_bytes = ((sizeof(KmWin) * nwin_max + sizeof(int) * (nmu + 1) + 255) / 256) * 256;
    char* wb = (char*)al.get(WS_KM_WIN, win_bytes + sizeof(SegScratch) * 4 * nwin_max);
    if (!svb || !wb) return set_error(c, THC_ERR_NOMEM, "thc_kmeans: workspace allocation failed");
    b.tq = svb;
    b.sv = svb + 4 * ng;
    b.win = (KmWin*)wb;
    b.wbase = (int*)(wb + sizeof(KmWin) * nwin_max);
    b.seg = (SegScratch*)(wb + win_bytes);
    b.nwin_max = (int)nwin_max;
  }

  KmState h{};
  h.max_it = max_it;
  h.threshold = threshold;
  for (int d = 0; d < 3; d++) h.bmin[d] = ~0ULL;
  THC_CUDA(c, cudaMemcpyAsync(st, &h, sizeof(KmState), cudaMemcpyHostToDevice, s));
  THC_CUDA(c, cudaEventRecord(c->ev0, s));
  int nprep = (int)cdiv(std::max<long long>(ng, nmu), 256);
  km_prep<<<nprep, 256, 0, s>>>(grid, rho, init, b);
  THC_LAUNCHED(c, "km_prep");
  km_finish_prep<<<1, 1, 0, s>>>(st, ng, nbins_max);
  THC_LAUNCHED(c, "km_finish_prep");
  // Spatial binning of the grid (once per call): perm lists the points bin by bin.
  const bool prune = c->km_prune && nmu >= 64;
  if (prune) {
    THC_CUDA(c, cudaMemsetAsync(b.bcount, 0, sizeof(int) * 2 * (size_t)nbins_max, s));
    km_bin_count<<<(int)cdiv(ng, 256), 256, 0, s>>>(grid, b);
    THC_LAUNCHED(c, "km_bin_count");
    km_bin_scan<<<1, 1024, 0, s>>>(b);
    THC_LAUNCHED(c, "km_bin_scan");
    km_bin_scatter<<<(int)cdiv(ng, 256), 256, 0, s>>>(b);
    THC_LAUNCHED(c, "km_bin_scatter");
  }
  const size_t prune64_smem = (size_t)kPruneMax * (sizeof(int) + 3 * sizeof(double));
  const size_t prune32_smem = (size_t)kPruneMax * (sizeof(int) + 3 * sizeof(float));
  if (prune) {
    THC_CUDA(c, cudaFuncSetAttribute(km_assign64p, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)prune64_smem));
    THC_CUDA(c, cudaFuncSetAttribute(km_assign32p, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)prune32_smem));
  }

  const bool mixed = c->precision == THC_PREC_MIXED;
  int nassign = (int)cdiv(ng, kAssignThreads);
  size_t hist_smem = sizeof(int) * nmu;
  if (hist_smem > 16 * 1024) {  // dynamic + static above the 48 KB default needs the opt-in
    THC_CUDA(c, cudaFuncSetAttribute(km_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hist_smem));
    THC_CUDA(c, cudaFuncSetAttribute(km_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hist_smem));
  }
  THC_CUDA(c, cudaFuncSetAttribute(km_sums, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)sizeof(SumSmem)));
  int* hflag = (int*)c->pinned;   // [2]: the done flag after a block of iterations
  const int kCheckEvery = 8;
  // One k-means iteration; every kernel reads the iteration index from device state and
  // returns at once after convergence, so the same launch sequence serves any iteration.
  auto iteration = [&](bool prof) -> int {
    // The pruned assign kernels count the histogram themselves (put_label).
    THC_CUDA(c, cudaMemsetAsync(hist, 0, sizeof(int) * (size_t)nmu * b.nb, s));
    if (mixed) {
      {
        ProfScope p(prof ? c : nullptr, "km_assign");
        if (prune) km_assign32p<<<nassign, kAssignThreads, prune32_smem, s>>>(b);
        else km_assign32<<<nassign, kAssignThreads, 0, s>>>(b);
      }
      THC_LAUNCHED(c, "km_assign32");
      if (!prune) {   // the pruned kernel rescues its near ties itself
        km_recheck<<<152 * 4, 256, 0, s>>>(b);
        THC_LAUNCHED(c, "km_recheck");
      }
    } else {
      {
        ProfScope p(prof ? c : nullptr, "km_assign");
        if (prune) km_assign64p<<<nassign, kAssignThreads, prune64_smem, s>>>(b);
        else km_assign64<<<nassign, kAssignThreads, 0, s>>>(b);
      }
      THC_LAUNCHED(c, "km_assign64");
    }
    if (!prune) {
      km_hist<<<b.nb, 256, hist_smem, s>>>(b);
      THC_LAUNCHED(c, "km_hist");
    }
    km_colscan<<<(int)cdiv((long long)nmu * 32, 256), 256, 0, s>>>(b);
    THC_LAUNCHED(c, "km_colscan");
    km_scatter<<<b.nb, 256, hist_smem, s>>>(b);
    THC_LAUNCHED(c, "km_scatter");
    if (b.nwin_max) {
      km_sbuild<<<(int)cdiv((long long)b.nwin_max * 4 * 32, kBuildThreads), kBuildThreads, 0, s>>>(b);
      THC_LAUNCHED(c, "km_sbuild");
      km_swalk<<<nmu, 128, 0, s>>>(b);
      THC_LAUNCHED(c, "km_swalk");
    } else {
      km_sums<<<nmu, kSumThreads, sizeof(SumSmem), s>>>(b);
      THC_LAUNCHED(c, "km_sums");
    }
    return THC_OK;
  };
  // A CUDA graph of kCheckEvery iterations, cached on the context for these buffers.
  // Profiling keeps the graph: only iterations launched outside it (the tail when max_it is
  // not a multiple of the graph length) get per-kernel events.
  const bool graphs = c->use_graphs && !fixed;
  cudaGraphExec_t gexec = nullptr;
  if (graphs) {
    // The graph bakes in every kernel argument: key it on all of them (the whole KmBufs,
    // whose pointers can move when a workspace slot grows) and on the launch shapes.
    std::vector<long long> key = {ng, nmu, mixed, prune, (long long)(uintptr_t)s,
                                  (long long)hist_smem, (long long)nassign};
    {
      const size_t words = (sizeof(KmBufs) + sizeof(long long) - 1) / sizeof(long long);
      std::vector<long long> raw(words, 0);
      memcpy(raw.data(), &b, sizeof(KmBufs));
      key.insert(key.end(), raw.begin(), raw.end());
    }
    auto hit = std::find_if(c->km_graphs.begin(), c->km_graphs.end(),
                            [&](const auto& e) { return e.first == key; });
    if (hit != c->km_graphs.end()) {
      gexec = hit->second;
      std::rotate(hit, hit + 1, c->km_graphs.end());      // most recently used last
    } else {
      constexpr size_t kGraphCache = 32;
      if (c->km_graphs.size() >= kGraphCache) {             // previous runs have finished
        cudaGraphExecDestroy(c->km_graphs.front().second);
        c->km_graphs.erase(c->km_graphs.begin());
      }
      cudaGraph_t graph;
      THC_CUDA(c, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      int rc = THC_OK;
      for (int k = 0; k < kCheckEvery && rc == THC_OK; k++) rc = iteration(false);
      cudaError_t ce = cudaStreamEndCapture(s, &graph);
      if (rc) return rc;
      if (ce != cudaSuccess) return set_error(c, THC_ERR_CUDA, "k-means graph capture: %s", cudaGetErrorString(ce));
      ce = cudaGraphInstantiate(&gexec, graph, 0);
      cudaGraphDestroy(graph);
      if (ce != cudaSuccess) return set_error(c, THC_ERR_CUDA, "k-means graph instantiate: %s", cudaGetErrorString(ce));
      c->km_graphs.emplace_back(key, gexec);
    }
  }
  // Blocks of kCheckEvery iterations, the host's convergence check one block behind the GPU:
  // the done flag after block k is copied (with an event) while block k + 1 runs, so the GPU
  // never waits for the host between blocks.  Iterations after convergence return at once,
  // so at most one block of empty launches is spent after the last real iteration.
  int launched = 0, blocks = 0, checked = 0;
  auto launch_block = [&]() -> int {
    const int nblock = std::min(kCheckEvery, max_it - launched);
    if (gexec && nblock == kCheckEvery) {
      THC_CUDA(c, cudaGraphLaunch(gexec, s));
      c->launches += (mixed ? 6LL : 5LL) * kCheckEvery;  // kernels per captured iteration
    } else {
      for (int k = 0; k < nblock; k++) {
        int rc = iteration(!fixed);
        if (rc) return rc;
      }
    }
    launched += nblock;
    const int slot = blocks++ & 1;
    THC_CUDA(c, cudaMemcpyAsync(hflag + slot, &st->done, sizeof(int), cudaMemcpyDeviceToHost, s));
    THC_CUDA(c, cudaEventRecord(c->ev_check[slot], s));
    return THC_OK;
  };
  while (launched < max_it && blocks < 2) {
    int rc = launch_block();
    if (rc) return rc;
  }
  while (checked < blocks) {
    const int slot = checked & 1;
    THC_CUDA(c, cudaEventSynchronize(c->ev_check[slot]));
    checked++;
    if (hflag[slot]) break;                  // converged (or stopped): later blocks are no-ops
    if (launched < max_it) {
      int rc = launch_block();
      if (rc) return rc;
    }
  }
  km_normdiff_exact<<<1, 1024, 0, s>>>(b);
  THC_LAUNCHED(c, "km_normdiff_exact");
  // Map the final centroids to the grid, sort, count duplicates.
  int* didx = is_device_ptr(out_idx) ? out_idx : (int*)((char*)hist);  // hist is free now
  int* dups = (int*)(part_i + (size_t)nmu * nch);
  THC_CUDA(c, cudaMemsetAsync(dups, 0, sizeof(int), s));
  if (prune) {
    int ntiles = (int)cdiv(ng, 256);
    float* box = (float*)part_s;   // 6 floats per tile fit in the partials buffer
    km_tile_boxes<<<ntiles, 256, 0, s>>>(b, box);
    THC_LAUNCHED(c, "km_tile_boxes");
    km_map_pruned<<<nmu, kMapThreads, 0, s>>>(b, box, ntiles, didx);
    THC_LAUNCHED(c, "km_map_pruned");
  } else {
    dim3 mg((unsigned)nch, (unsigned)cdiv(nmu, 256));
    km_map_part<<<mg, 256, 0, s>>>(b, part_s, part_i, nch);
    THC_LAUNCHED(c, "km_map_part");
    km_map_reduce<<<(int)cdiv(nmu, 256), 256, 0, s>>>(nmu, nch, part_s, part_i, didx);
    THC_LAUNCHED(c, "km_map_reduce");
  }
  int np2 = 1;
  while (np2 < nmu) np2 <<= 1;
  size_t sort_smem = sizeof(int) * np2;
  if (sort_smem > 16 * 1024)  // dynamic + static above the 48 KB default needs the opt-in
    THC_CUDA(c, cudaFuncSetAttribute(km_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sort_smem));
  km_sort<<<1, 1024, sort_smem, s>>>(didx, nmu, np2, dups);
  THC_LAUNCHED(c, "km_sort");
  THC_CUDA(c, cudaEventRecord(c->ev1, s));
  KmState hs{};
  THC_CUDA(c, cudaMemcpyAsync(&hs, st, sizeof(KmState), cudaMemcpyDeviceToHost, s));
  int hd = 0;
  THC_CUDA(c, cudaMemcpyAsync(&hd, dups, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (didx != out_idx)
    THC_CUDA(c, cudaMemcpyAsync(out_idx, didx, sizeof(int) * nmu, cudaMemcpyDeviceToHost, s));
  THC_CUDA(c, cudaStreamSynchronize(s));
  // The history of a fixed-scratch call lives in the shared region, which later calls
  // overwrite: thc_kmeans_history reports none for it.
  c->km_last_iters = fixed ? 0 : hs.iter;
  c->km_last_max_it = max_it;
  if (hs.bad_label) return set_error(c, THC_ERR_CUDA, "thc_kmeans: internal label out of range");
  if (hs.empty) {
    if (stats) stats->iterations = hs.iter;
    return set_error(c, THC_ERR_EMPTY_CLUSTER, "CRITICAL ERROR: Found centroid with weight ~ 0");
  }
  if (hs.zero_fill) {
    // The reference leaves interp_indxs zero-filled when the last diff equals the threshold.
    THC_CUDA(c, cudaMemsetAsync(didx, 0, sizeof(int) * nmu, s));
    if (didx != out_idx) std::fill(out_idx, out_idx + nmu, 0);
    THC_CUDA(c, cudaStreamSynchronize(s));
  }
  if (stats) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    stats->iterations = hs.iter;
    stats->converged = hs.converged;
    stats->zero_filled = hs.zero_fill;
    stats->duplicates = hd;
    stats->final_diff = hs.diff;
    stats->pct_changed = hs.pct;
    stats->rechecked = hs.rechecked_total;
    stats->device_ms = ms;
  }
  return THC_OK;
}

int kmeans_history(Ctx* c, double* diff, double* pct, int n)
{
  if (n < 0 || n > c->km_last_iters || !c->ws[WS_KM_LOG]) return THC_ERR_ARG;
  if (n == 0) return THC_OK;
  const double* logb = (const double*)c->ws[WS_KM_LOG];
  THC_CUDA(c, cudaMemcpyAsync(diff, logb, sizeof(double) * n, cudaMemcpyDefault, c->stream));
  THC_CUDA(c, cudaMemcpyAsync(pct, logb + c->km_last_max_it, sizeof(double) * n, cudaMemcpyDefault,
                              c->stream));
  THC_CUDA(c, cudaStreamSynchronize(c->stream));
  return THC_OK;
}

}  // namespace thc
