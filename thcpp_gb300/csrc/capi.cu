// The C ABI (include/thc_gb300.h): contexts, workspace, residency and dispatch.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <memory>
#include <mutex>
#include <thread>
#include <cstdio>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "common.cuh"
#include "ozgemm.cuh"
#include "isdf.cuh"

namespace thc {

void* ws_get(Ctx* c, Slot s, size_t bytes)
{
  // Stream-ordered allocation: growing a slot neither synchronises the device nor stalls
  // other contexts' streams (a plain cudaFree would wait for the whole GPU).
  if (bytes == 0) bytes = 16;
  if (c->ws_bytes[s] >= bytes) return c->ws[s];
  if (c->ws[s]) {
    cudaFreeAsync(c->ws[s], c->stream);
    c->ws[s] = nullptr;
    c->ws_bytes[s] = 0;
  }
  // Headroom so that slightly larger calls reuse the slot (at most 256 MiB of it).
  size_t want = bytes + std::min(bytes / 8, (size_t)256 << 20);
  void* p = nullptr;
  if (cudaMallocAsync(&p, want, c->stream) != cudaSuccess) {
    cudaGetLastError();
    if (cudaMallocAsync(&p, bytes, c->stream) != cudaSuccess) {
      cudaGetLastError();
      // The pool keeps freed memory reserved (release threshold = max), possibly in pieces
      // too small for this request: return what no allocation uses and try once more.
      // The whole device first: trimming may then release nothing that a kernel of another
      // stream or context still uses.
      cudaMemPool_t pool;
      if (cudaDeviceSynchronize() != cudaSuccess ||
          cudaDeviceGetDefaultMemPool(&pool, c->device) != cudaSuccess ||
          cudaMemPoolTrimTo(pool, 0) != cudaSuccess ||
          cudaMallocAsync(&p, bytes, c->stream) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
      }
    }
    want = bytes;
  }
  c->ws[s] = p;
  c->ws_bytes[s] = want;
  return p;
}

int set_error(Ctx* c, int status, const char* fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (c) c->last_error = buf;
  return status;
}

int check_launch(Ctx* c, const char* what)
{
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return set_error(c, THC_ERR_CUDA, "launch of %s failed: %s", what, cudaGetErrorString(e));
  return THC_OK;
}

bool is_device_ptr(const void* p)
{
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

const void* to_device(Ctx* c, const void* p, size_t bytes, Slot staging, int* status)
{
  *status = THC_OK;
  if (is_device_ptr(p)) return p;
  void* d = ws_get(c, staging, bytes);
  if (!d) {
    *status = set_error(c, THC_ERR_NOMEM, "staging allocation of %zu bytes failed", bytes);
    return nullptr;
  }
  cudaError_t e = cudaMemcpyAsync(d, p, bytes, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) {
    *status = set_error(c, THC_ERR_CUDA, "host-to-device copy failed: %s", cudaGetErrorString(e));
    return nullptr;
  }
  return d;
}

static cudaEvent_t take_event(Ctx* c)
{
  if (!c->event_pool.empty()) {
    cudaEvent_t e = c->event_pool.back();
    c->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

ProfScope::ProfScope(Ctx* ctx, const char* name) : c(ctx)
{
  if (!c || !c->profile) return;
  Ctx::Rec r{name, take_event(c), take_event(c)};
  cudaEventRecord(r.a, c->stream);
  c->recs.push_back(r);
  i = c->recs.size() - 1;
}

ProfScope::~ProfScope()
{
  if (i != (size_t)-1) cudaEventRecord(c->recs[i].b, c->stream);
}

static void clear_profile(Ctx* c)
{
  cudaStreamSynchronize(c->stream);
  for (auto& r : c->recs) {
    c->event_pool.push_back(r.a);
    c->event_pool.push_back(r.b);
  }
  c->recs.clear();
}

}  // namespace thc

namespace {
// out[i] = in[i] for FP32 interpolating vectors (grid-stride).
__global__ void widen_f32(const float* __restrict__ in, long long n, double* __restrict__ out)
{
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = (double)in[i];
}
}  // namespace

extern "C" {

const char* thc_status_string(int status)
{
  switch (status) {
    case THC_OK: return "ok";
    case THC_ERR_ARG: return "invalid argument";
    case THC_ERR_CUDA: return "CUDA error";
    case THC_ERR_EMPTY_CLUSTER: return "empty k-means cluster";
    case THC_ERR_NOT_PD: return "matrix not positive definite";
    case THC_ERR_SHAPE: return "shape mismatch";
    case THC_ERR_IO: return "I/O error";
    case THC_ERR_TIMEOUT: return "device wait timed out";
    case THC_ERR_NOMEM: return "device allocation failed";
    case THC_ERR_CUFFT: return "cuFFT error";
    default: return "unknown status";
  }
}

int thc_ctx_create(int device, int precision, thc_ctx** out)
{
  if (!out || (precision != THC_PREC_FP64 && precision != THC_PREC_MIXED)) return THC_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return THC_ERR_CUDA;
  }
  if (cudaSetDevice(device) != cudaSuccess) return THC_ERR_CUDA;
  thc_ctx* h = new (std::nothrow) thc_ctx;
  if (!h) return THC_ERR_NOMEM;
  thc::Ctx* c = &h->c;
  c->device = device;
  c->precision = precision;
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->aux_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_panel, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_trail, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_check[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_check[1], cudaEventDisableTiming) != cudaSuccess ||
      cudaMallocHost(&c->pinned, 4096) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return THC_ERR_CUDA;
  }
  c->stream = c->own_stream;
  {
    // Keep freed workspace in the device's default pool instead of returning it to the
    // driver at every synchronisation (process-local setting of this process's pool).
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      unsigned long long keep = ~0ULL;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
  }
  *out = h;
  return THC_OK;
}

int thc_ctx_destroy(thc_ctx* h)
{
  if (!h) return THC_ERR_ARG;
  thc::Ctx* c = &h->c;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto& kv : c->plans) cufftDestroy(kv.second);
  for (int s = 0; s < thc::WS_NSLOTS; s++)
    if (c->ws[s]) cudaFreeAsync(c->ws[s], c->stream);
  cudaStreamSynchronize(c->stream);
  thc::clear_profile(c);
  for (auto e : c->event_pool) cudaEventDestroy(e);
  for (auto& g : c->km_graphs) cudaGraphExecDestroy(g.second);
  if (c->pinned) cudaFreeHost(c->pinned);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  for (cudaEvent_t e : c->ev_check)
    if (e) cudaEventDestroy(e);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  if (c->ev_panel) cudaEventDestroy(c->ev_panel);
  if (c->ev_trail) cudaEventDestroy(c->ev_trail);
  if (c->aux_stream) {
    cudaStreamSynchronize(c->aux_stream);
    cudaStreamDestroy(c->aux_stream);
  }
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete h;
  return THC_OK;
}

int thc_ctx_set_stream(thc_ctx* h, void* stream)
{
  if (!h) return THC_ERR_ARG;
  // Workspace is allocated in the order of the current stream: finish it before switching.
  cudaStreamSynchronize(h->c.stream);
  h->c.stream = stream ? (cudaStream_t)stream : h->c.own_stream;
  for (auto& kv : h->c.plans) cufftSetStream(kv.second, h->c.stream);
  return THC_OK;
}

int thc_ctx_set_option(thc_ctx* h, const char* key, double value)
{
  if (!h || !key) return THC_ERR_ARG;
  if (!strcmp(key, "slices_p")) {
    if (value < 2 || value > 6) return THC_ERR_ARG;
    h->c.slices_p = (int)value;
    return THC_OK;
  }
  if (!strcmp(key, "slices_m")) {
    if (value < 2 || value > 6) return THC_ERR_ARG;
    h->c.slices_m = (int)value;
    return THC_OK;
  }
  if (!strcmp(key, "graphs")) {
    h->c.use_graphs = value != 0.0;
    return THC_OK;
  }
  if (!strcmp(key, "km_prune")) {
    h->c.km_prune = value != 0.0;
    return THC_OK;
  }
  if (!strcmp(key, "gemm_tc")) {
    h->c.gemm_tc = value != 0.0;
    return THC_OK;
  }
  if (!strcmp(key, "profile")) {
    thc::clear_profile(&h->c);
    h->c.profile = value != 0.0;
    return THC_OK;
  }
  if (!strcmp(key, "tc_hi")) {   // 1, 2, 4, ... 32 sixteen-k steps per drain
    const int v = (int)value;
    if (v < 1 || v > 32 || (v & (v - 1))) return THC_ERR_ARG;
    h->c.tc_hi_stages = v;
    return THC_OK;
  }
  if (!strcmp(key, "tc_bk")) {
    if (value != 16.0 && value != 32.0) return THC_ERR_ARG;
    h->c.tc_bk = (int)value;
    h->c.autotune = 0;
    return THC_OK;
  }
  if (!strcmp(key, "tc_bn")) {
    if (value != 64.0 && value != 128.0) return THC_ERR_ARG;
    h->c.tc_bn = (int)value;
    h->c.autotune = 0;
    return THC_OK;
  }
  if (!strcmp(key, "tc_persistent")) {
    h->c.tc_persistent = value != 0.0;
    h->c.autotune = 0;
    return THC_OK;
  }
  if (!strcmp(key, "autotune")) {
    h->c.autotune = value != 0.0;
    return THC_OK;
  }
  if (!strcmp(key, "qrcp_all_pairs")) {
    h->c.qrcp_all_pairs = value != 0.0;
    return THC_OK;
  }
  if (!strcmp(key, "overlap")) {
    h->c.overlap = value != 0.0;
    return THC_OK;
  }
  if (!strcmp(key, "spin_limit")) {
    if (value < 0 || value > 1e12) return THC_ERR_ARG;
    h->c.spin_limit = (long long)value;
    return THC_OK;
  }
  if (!strcmp(key, "equilibrate")) {
    h->c.equilibrate = value != 0.0;
    return THC_OK;
  }
  if (!strcmp(key, "refine")) {
    if (value < 0 || value > 8) return THC_ERR_ARG;
    h->c.refine = (int)value;
    return THC_OK;
  }
  if (!strcmp(key, "fft64")) {
    h->c.fft64 = value != 0.0;
    return THC_OK;
  }
  if (!strcmp(key, "slices_z")) {
    if (value < 2 || value > 6) return THC_ERR_ARG;
    h->c.slices_z = (int)value;
    return THC_OK;
  }
  return THC_ERR_ARG;
}

const char* thc_ctx_autotune_log(thc_ctx* h)
{
  if (!h) return "";
  h->c.tune_log = thc::ozgemm_tune_log(h->c.device);
  return h->c.tune_log.c_str();
}

const char* thc_ctx_last_error(const thc_ctx* h)
{
  return h ? h->c.last_error.c_str() : "null context";
}

long long thc_ctx_kernel_launches(const thc_ctx* h) { return h ? h->c.launches : 0; }

int thc_ctx_kernel_time(thc_ctx* h, const char* kernel, double* ms, long long* launches)
{
  if (!h || !kernel || !ms || !launches) return THC_ERR_ARG;
  thc::Ctx* c = &h->c;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return THC_ERR_CUDA;
  double t = 0.0;
  long long n = 0;
  for (auto& r : c->recs) {
    if (r.name != kernel) continue;
    float x = 0.f;
    if (cudaEventElapsedTime(&x, r.a, r.b) == cudaSuccess) {
      t += x;
      n++;
    }
  }
  *ms = t;
  *launches = n;
  return THC_OK;
}

int thc_kmeans_initial_indices(long long ng, int nmu, unsigned int seed, int* out_idx)
{
  // KMeansSolver::guess_initial_centroids (src/kmeans.cpp:159-168): the same standard
  // library calls on the same types, so the sequence matches the reference's libstdc++.
  if (ng <= 0 || nmu <= 0 || nmu > ng || !out_idx || ng > 0x7fffffffLL) return THC_ERR_ARG;
  std::vector<int> tmp((size_t)ng);
  for (long long i = 0; i < ng; i++) tmp[i] = (int)i;
  std::mt19937 mt(seed);
  std::shuffle(tmp.begin(), tmp.end(), mt);
  std::vector<int> ind(tmp.begin(), tmp.begin() + nmu);
  std::sort(ind.begin(), ind.end());
  std::copy(ind.begin(), ind.end(), out_idx);
  return THC_OK;
}

int thc_kmeans(thc_ctx* h, const double* grid, const double* rho, long long ng, int nmu,
               const int* init_idx, int max_it, double threshold, int* out_idx,
               thc_kmeans_stats* stats)
{
  if (!h) return THC_ERR_ARG;
  if (cudaSetDevice(h->c.device) != cudaSuccess) return THC_ERR_CUDA;
  if (stats) memset(stats, 0, sizeof(*stats));
  return thc::kmeans_run(&h->c, grid, rho, ng, nmu, init_idx, max_it, threshold, out_idx, stats);
}

int thc_kmeans_history(thc_ctx* h, double* diff, double* pct_changed, int n)
{
  if (!h || (n > 0 && (!diff || !pct_changed))) return THC_ERR_ARG;
  return thc::kmeans_history(&h->c, diff, pct_changed, n);
}

int thc_isdf(thc_ctx* h, const double* phi, long long ng, int norb, const int* idx, int nmu,
             const int* mesh, const double* coulG, double shift_rel, double* out_orbitals,
             double* out_M, double* out_L, thc_isdf_stats* stats)
{
  if (!h) return THC_ERR_ARG;
  if (cudaSetDevice(h->c.device) != cudaSuccess) return THC_ERR_CUDA;
  if (stats) memset(stats, 0, sizeof(*stats));
  return thc::isdf_run(&h->c, phi, ng, norb, idx, nmu, mesh, coulG, shift_rel, out_orbitals,
                       out_M, out_L, stats);
}

int thc_isdf_complex(thc_ctx* h, const double* phi, long long ng, int norb, const int* idx,
                     int nmu, const int* mesh, const double* coulG, double shift_rel,
                     double* out_orbitals, double* out_M, double* out_L, thc_isdf_stats* stats)
{
  if (!h) return THC_ERR_ARG;
  if (cudaSetDevice(h->c.device) != cudaSuccess) return THC_ERR_CUDA;
  if (stats) memset(stats, 0, sizeof(*stats));
  return thc::isdf_run(&h->c, phi, ng, norb, idx, nmu, mesh, coulG, shift_rel, out_orbitals,
                       out_M, out_L, stats, nullptr, 0, nullptr, true);
}

int thc_isdf_half(thc_ctx* h, const double* phi, long long ng, int norb, const double* phi_occ,
                  int nocc, const int* idx, int nmu, const int* mesh, const double* coulG,
                  double shift_rel, double* out_orbitals, double* out_occ_orbitals,
                  double* out_M, thc_isdf_stats* stats)
{
  if (!h || !phi_occ || nocc <= 0) return THC_ERR_ARG;
  if (cudaSetDevice(h->c.device) != cudaSuccess) return THC_ERR_CUDA;
  if (stats) memset(stats, 0, sizeof(*stats));
  return thc::isdf_run(&h->c, phi, ng, norb, idx, nmu, mesh, coulG, shift_rel, out_orbitals,
                       out_M, nullptr, stats, phi_occ, nocc, out_occ_orbitals);
}

int thc_isdf_half_complex(thc_ctx* h, const double* phi, long long ng, int norb,
                          const double* phi_occ, int nocc, const int* idx, int nmu,
                          const int* mesh, const double* coulG, double* out_orbitals,
                          double* out_occ_orbitals, double* out_M, thc_isdf_stats* stats)
{
  if (!h) return THC_ERR_ARG;
  if (cudaSetDevice(h->c.device) != cudaSuccess) return THC_ERR_CUDA;
  if (stats) memset(stats, 0, sizeof(*stats));
  return thc::isdf_half_complex_run(&h->c, phi, ng, norb, phi_occ, nocc, idx, nmu, mesh, coulG,
                                    out_orbitals, out_occ_orbitals, out_M, stats);
}

int thc_isdf_interpolating_vectors(thc_ctx* h, long long ng, int nmu, double* out_zeta)
{
  if (!h || !out_zeta) return THC_ERR_ARG;
  thc::Ctx* c = &h->c;
  if (cudaSetDevice(c->device) != cudaSuccess) return THC_ERR_CUDA;
  if (!c->zeta_elem || !c->zeta_last)
    return thc::set_error(c, THC_ERR_ARG, "thc_isdf_interpolating_vectors: no ISDF result on "
                          "this context (none yet, or a later call reused its workspace)");
  if (ng != c->zeta_ng || nmu != c->zeta_nmu)
    return thc::set_error(c, THC_ERR_SHAPE, "thc_isdf_interpolating_vectors: the last ISDF "
                          "call had N_g %lld, N_mu %d", c->zeta_ng, c->zeta_nmu);
  const long long n = (long long)nmu * ng;
  cudaStream_t s = c->stream;
  if (c->zeta_elem == (int)sizeof(double)) {
    THC_CUDA(c, cudaMemcpyAsync(out_zeta, c->zeta_last, sizeof(double) * n, cudaMemcpyDefault, s));
  } else if (thc::is_device_ptr(out_zeta)) {
    widen_f32<<<(unsigned)std::min<long long>(thc::cdiv(n, 256), 1 << 20), 256, 0, s>>>(
        (const float*)c->zeta_last, n, out_zeta);
    THC_LAUNCHED(c, "widen_f32");
  } else {
    // Host output: widen 32 Mi values at a time in a staging slot, then copy each chunk.
    const long long chunk = 1LL << 25;
    double* stage = (double*)thc::ws_get(c, thc::WS_OUT, sizeof(double) * std::min(n, chunk));
    if (!stage) return thc::set_error(c, THC_ERR_NOMEM, "thc_isdf_interpolating_vectors: staging");
    for (long long o = 0; o < n; o += chunk) {
      const long long m = std::min(chunk, n - o);
      widen_f32<<<(unsigned)std::min<long long>(thc::cdiv(m, 256), 1 << 20), 256, 0, s>>>(
          (const float*)c->zeta_last + o, m, stage);
      THC_LAUNCHED(c, "widen_f32");
      THC_CUDA(c, cudaMemcpyAsync(out_zeta + o, stage, sizeof(double) * m,
                                  cudaMemcpyDeviceToHost, s));
      // The next chunk reuses the staging slot: wait for this copy.
      THC_CUDA(c, cudaStreamSynchronize(s));
    }
  }
  THC_CUDA(c, cudaStreamSynchronize(s));
  return THC_OK;
}

int thc_qrcp(thc_ctx* h, const double* phi, long long ng, int norb, const double* phi_occ,
             int nocc, int npts, int* out_idx, int* out_order, double* out_diag,
             thc_qrcp_stats* stats)
{
  if (!h) return THC_ERR_ARG;
  if (cudaSetDevice(h->c.device) != cudaSuccess) return THC_ERR_CUDA;
  if (stats) memset(stats, 0, sizeof(*stats));
  return thc::qrcp_run(&h->c, phi, ng, norb, phi_occ, nocc, npts, out_idx, out_order, out_diag,
                       stats);
}

int thc_qrcp_complex(thc_ctx* h, const double* phi, long long ng, int norb, int npts,
                     int* out_idx, int* out_order, double* out_diag, thc_qrcp_stats* stats)
{
  if (!h) return THC_ERR_ARG;
  if (cudaSetDevice(h->c.device) != cudaSuccess) return THC_ERR_CUDA;
  if (stats) memset(stats, 0, sizeof(*stats));
  return thc::qrcp_run(&h->c, phi, ng, norb, nullptr, 0, npts, out_idx, out_order, out_diag,
                       stats, true);
}

namespace {
std::mutex g_pool_mu;
std::map<std::pair<int, int>, std::vector<thc_ctx*>> g_pool;
}  // namespace

int thc_factorize_batched(int device, int precision, thc_system* sys, int nsys, int nstreams)
{
  if (!sys || nsys < 0 || nstreams < 1 || nstreams > 64) return THC_ERR_ARG;
  if (nsys == 0) return THC_OK;
  nstreams = std::min(nstreams, nsys);
  std::vector<thc_ctx*> workers;
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    auto& pool = g_pool[{device, precision}];
    while ((int)pool.size() < nstreams) {
      thc_ctx* h = nullptr;
      int st = thc_ctx_create(device, precision, &h);
      if (st) return st;
      // The systems already overlap across the workers' streams: each worker keeps its
      // whole factorisation on its own stream (whatever the default of "overlap").
      h->c.overlap = 0;
      pool.push_back(h);
    }
    workers.assign(pool.begin(), pool.begin() + nstreams);
  }
  // Largest systems first (N_g N_mu estimates the work), taken dynamically by the workers.
  std::vector<int> order(nsys);
  for (int i = 0; i < nsys; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return (double)sys[x].ng * sys[x].nmu > (double)sys[y].ng * sys[y].nmu;
  });
  std::atomic<int> next(0);
  auto work = [&](thc_ctx* h) {
    cudaSetDevice(device);
    for (int n_ = next++; n_ < nsys; n_ = next++) {
      thc_system& s = sys[order[n_]];
      memset(&s.kmeans_stats, 0, sizeof(s.kmeans_stats));
      memset(&s.isdf_stats, 0, sizeof(s.isdf_stats));
      s.error[0] = 0;
      h->c.last_error.clear();
      s.status = thc::kmeans_run(&h->c, s.grid, s.rho, s.ng, s.nmu, s.init_idx, s.max_it,
                                 s.threshold, s.out_idx, &s.kmeans_stats);
      if (s.status == THC_OK)
        s.status = thc::isdf_run(&h->c, s.phi, s.ng, s.norb, s.out_idx, s.nmu, s.mesh,
                                 s.coulG, s.shift_rel, s.out_orbitals, s.out_M, s.out_L,
                                 &s.isdf_stats);
      if (s.status != THC_OK) {
        snprintf(s.error, sizeof(s.error), "%s", h->c.last_error.c_str());
        cudaGetLastError();
      }
    }
    cudaStreamSynchronize(h->c.stream);
  };
  if (nstreams == 1) {
    work(workers[0]);
  } else {
    std::vector<std::thread> th;
    for (int w = 0; w < nstreams; w++) th.emplace_back(work, workers[w]);
    for (auto& t : th) t.join();
  }
  for (int i = 0; i < nsys; i++)
    if (sys[i].status != THC_OK && sys[i].status != THC_ERR_NOT_PD) return sys[i].status;
  return THC_OK;
}

}  // extern "C"
