// Shared internals of libthc_gb300: the context, its workspace arena and error helpers.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "../../include/thc_gb300.h"

namespace thc {

// Workspace slots: each grows on demand and is reused across calls.
enum Slot : int {
  // k-means
  WS_KM_GRID = 0,   // 3 x ng doubles (SoA)
  WS_KM_GRID32,     // 3 x ng floats (SoA) in point order, 3 x ng in the binned order
  WS_KM_RHO,
  WS_KM_CENT,       // 2 buffers x 3 x nmu doubles
  WS_KM_CENT32,     // 2 buffers x 3 x nmu floats
  WS_KM_LABELS,     // 2 x ng ints
  WS_KM_HIST,       // nmu x nblocks ints
  WS_KM_TOTAL,      // nmu ints (counts) + nmu ints (starts)
  WS_KM_MEMBER,     // ng ints
  WS_KM_TERMS,      // 4 x nmu doubles
  WS_KM_RECHECK,    // ng ints
  WS_KM_STATE,
  WS_KM_PART,       // map_to_grid partials
  WS_KM_LOG,        // per-iteration diff / pct
  WS_KM_IO,         // staging of caller arrays
  WS_KM_IDX,
  WS_KM_PERM,       // spatial binning: perm[ng], bin of each point, bin counts / offsets
  // ISDF
  WS_PHI,           // ng x norb doubles
  WS_PHIMU,         // nmu x norb doubles
  WS_IDX,
  WS_COUL,          // ng doubles
  WS_C,             // nmu x nmu doubles
  WS_CINV,          // nmu x nmu doubles
  WS_ZT,            // nmu x ng doubles (Z^T)
  WS_ZETA,          // nmu x ng doubles (zeta^T)
  WS_ZHAT,          // nmu x nc x 2 doubles
  WS_DSYM,          // nc doubles
  WS_DANTI,         // nc doubles + index list
  WS_M,             // nmu x nmu x 2 doubles
  WS_L,             // nmu x nmu x 2 doubles
  WS_SCRATCH,       // small reductions / status
  WS_SLICE_A,       // sliced-GEMM operands
  WS_SLICE_B,
  WS_SLICE_E,
  WS_OUT,           // staging of caller outputs
  WS_PART,          // split-K partial sums
  WS_DINV,          // inverted diagonal blocks + L^{-1} + scratch of the inverse
  WS_ROWMAX,        // per-row maxima for slicing
  WS_DPART,         // split-K partials chosen inside dgemm
  WS_FFTWORK,       // cuFFT work area of the context's plans
  WS_KM_SV,         // k-means terms: 4 x ng doubles in point order + 4 x ng sorted
  WS_KM_WIN,        // k-means windows, cluster window offsets, segment tables
  WS_PHIOCC,        // half-rotated path: ng x nocc occupied orbitals, then nmu x nocc rows
  WS_ORB,           // (N_o + N_occ) x N_mu x 2 orbital outputs staged for a host copy
  WS_REFINE,        // 3 x nmu x nmu doubles: refinement polynomial, L^{-1} T (mixed)
  WS_EQUIL,         // nmu doubles + nmu ints: power-of-two equilibration of C (mixed)
  WS_NSLOTS
};

struct Ctx {
  int device = 0;
  int precision = THC_PREC_FP64;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  // Second stream for work that may overlap the main one (C's factorisation beside the P
  // product), forked and joined with these events.  Off by default ("overlap" option): the
  // P product's CTAs fill every SM, so the overlap measured no gain at N_g 1.1e5.
  cudaStream_t aux_stream = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaEvent_t ev_panel = nullptr, ev_trail = nullptr;   // Cholesky look-ahead (dense64.cu)
  int overlap = 0;
  void* ws[WS_NSLOTS] = {};
  size_t ws_bytes[WS_NSLOTS] = {};
  std::map<std::tuple<int, int, int, int, int>, cufftHandle> plans;  // (n0,n1,n2,batch,type)
  std::map<std::tuple<int, int, int, int, int>, size_t> plan_work;   // their work-area bytes
  // 4 KB pinned host scratch for asynchronous device-to-host flags.  Users (never live at
  // the same time within one call): bytes [0, 32) the k-means done flags of two blocks in
  // flight (kmeans.cu) or the CholStatus of C (mixed.cu); bytes [kPinnedCounts, +8) the
  // Coulomb kernel's two counts (mixed.cu).
  void* pinned = nullptr;
  static constexpr size_t kPinnedCounts = 64;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t ev_check[2] = {nullptr, nullptr};   // k-means convergence checks in flight
  long long launches = 0;
  int slices_p = 6;
  int slices_z = 6;
  // The Coulomb product's rows span many binades (sqrt(v) ~ 1/|G| on top of the decay of
  // zeta_hat): 4 slices leave 1.3e-6 on M at N_g 1.26e6 (a bias from the dropped level-4
  // pairs on the diagonal), 5 slices 2.7e-7.
  int slices_m = 5;
  int gemm_tc = 1;      // 1: tcgen05 sliced GEMM, 0: mma.sync sliced GEMM
  int km_prune = 1;     // 1: spatially pruned k-means assign, 0: exhaustive
  int use_graphs = 1;   // capture the k-means iteration block in a CUDA graph
  // k-step per pipeline stage of the tensor-core GEMM: 32 (2-3 stages of all slices, the
  // faster: 0.90 s against 1.00 s for the zeta product at N_g 1.26e6, N_mu 5184) or 16
  // (4 stages of half the size).
  int tc_bk = 32;
  // Tile width of the tensor-core GEMM without the autotuner: 128, or 64 (k-step 16, two
  // CTAs per SM).  Setting "tc_bn" turns the autotuner off for the context.
  int tc_bn = 128;
  // Without the autotuner: the persistent short-K kernel (64-wide tiles, two TMEM buffers)
  // for every product it takes (K <= 512, no split of K, no triangle).
  int tc_persistent = 0;
  // Pick the tensor-core kernel's k-step, tile order and split of K per shape class by
  // timing the candidates the first time a class is met (process-wide table; ozgemm_tc.cu).
  // Setting "tc_bk" turns it off for the context.
  int autotune = 1;
  std::string tune_log;   // last thc_ctx_autotune_log text
  int tc_hi_stages = 8; // drain period of the level >= 3 accumulator, in 16-k MMA steps
  int fft64 = 0;        // mixed path: zeta in FP64 and a D2Z FFT (else FP32 and R2C)
  int qrcp_all_pairs = 0;  // half-rotated QRCP: every (occupied, orbital) pair as a row
  // Iterative-refinement steps of zeta when C is solved with a diagonal shift s: step j
  // adds (C + sI)^{-1} (Z^T - C zeta_j) (see isdf.cu, refine_polynomial).
  int refine = 0;
  // Mixed path: solve with C scaled to a unit-range diagonal by powers of two, T C T
  // (T = 2^{-round(log2 sqrt(C_ii))}), so that the rows sliced for the solve products are
  // balanced (an ill-conditioned C with a wide diagonal otherwise loses most of the 42 bits
  // of its small entries).
  int equilibrate = 1;
  // Polls of an mbarrier before a bounded device wait gives up (THC_ERR_TIMEOUT).
  long long spin_limit = 1LL << 24;
  // Instantiated k-means iteration graphs, most recently used last, keyed by every kernel
  // argument they bake in.
  std::vector<std::pair<std::vector<long long>, cudaGraphExec_t>> km_graphs;
  // Interpolating vectors zeta^T (N_mu x N_g, row mu = zeta_mu on the grid) of the last
  // ISDF call, where they stay in the workspace until the next call: element size 8 (FP64)
  // or 4 (FP32, the mixed path's R2C input); zeta_elem = 0 when there are none.
  const void* zeta_last = nullptr;
  int zeta_elem = 0;
  long long zeta_ng = 0;
  int zeta_nmu = 0;
  std::string last_error;
  // History of the last k-means run (device buffer WS_KM_LOG: diff[max_it], pct[max_it]).
  int km_last_iters = 0;
  int km_last_max_it = 0;
  // Opt-in per-kernel event timing.
  bool profile = false;
  struct Rec { std::string name; cudaEvent_t a, b; };
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> event_pool;
};

// Runs the enclosing scope's launches on another stream (the context's current stream is
// what every helper launches on), restoring the previous one on exit.
struct StreamSwap {
  Ctx* c;
  cudaStream_t prev;
  StreamSwap(Ctx* ctx, cudaStream_t s) : c(ctx), prev(ctx->stream) { c->stream = s; }
  ~StreamSwap() { c->stream = prev; }
};

// RAII event pair around one launch when profiling is on.
struct ProfScope {
  Ctx* c;
  size_t i = (size_t)-1;
  ProfScope(Ctx* ctx, const char* name);
  ~ProfScope();
};

// Grow-only workspace slot; returns nullptr on allocation failure.
void* ws_get(Ctx* c, Slot s, size_t bytes);

int set_error(Ctx* c, int status, const char* fmt, ...);

// Record a CUDA error after launches (cudaGetLastError).
int check_launch(Ctx* c, const char* what);

inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Residency of a caller pointer.
bool is_device_ptr(const void* p);

// Bring a caller array onto the device: returns the device pointer (the caller's own if
// already resident, else the staging slot after an async copy).
const void* to_device(Ctx* c, const void* p, size_t bytes, Slot staging, int* status);

}  // namespace thc

// The opaque handle of the C ABI.
struct thc_ctx {
  thc::Ctx c;
};

#define THC_CUDA(c, call)                                                          \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return thc::set_error((c), THC_ERR_CUDA, "%s: %s (%s:%d)", #call,            \
                            cudaGetErrorString(e_), __FILE__, __LINE__);           \
  } while (0)

#define THC_LAUNCHED(c, what)                                                      \
  do {                                                                             \
    (c)->launches++;                                                               \
    int s_ = thc::check_launch((c), (what));                                       \
    if (s_) return s_;                                                             \
  } while (0)
