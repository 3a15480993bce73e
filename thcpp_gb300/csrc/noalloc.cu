// thc_kmeans_noalloc: the k-means entry point for callers that cannot allocate device
// memory.  It has no counterpart in the reference.
//
// Who needs it: a host program whose device memory is owned by its own pool allocator
// (a QMC driver that reserves the GPU's memory up front, a framework's caching allocator)
// cannot let a library call cudaMalloc/cudaFree behind its back -- the call would fail once
// the pool holds the memory, or would synchronise the device and disturb the pool's
// streams.  thc_kmeans grows a per-context workspace on first use; this variant takes every
// buffer from one file-scope device array instead.
//
// Limits: N_g <= 65,536 grid points, N_mu <= 1,024 centroids, max_it <= 1,000 (about 8 MB
// of the 12 MiB array at the maximum; larger problems return THC_ERR_SHAPE).  The array is
// shared by every call in the process and keeps the last call's contents; everything the
// k-means needs zeroed is cleared by the call itself.  Calls that overlap on the GPU (two
// streams, two host threads) race on it: serialise them.  The first call on a device looks
// up the array's device address (cudaGetSymbolAddress, with that device current), which
// may load the module; make that first call before any stream capture.
#include <cuda_runtime.h>

#include <mutex>

#include "common.cuh"
#include "isdf.cuh"

namespace thc {
namespace {

constexpr long long kNoAllocMaxNg = 65536;
constexpr int kNoAllocMaxNmu = 1024;
constexpr int kNoAllocMaxIt = 1000;
constexpr size_t kNoAllocBytes = 12u << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_km_scratch[kNoAllocBytes];

std::mutex g_setup_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on `device` (the current device), looked up once.
int scratch_for(Ctx* c, int device, void** out)
{
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_km_scratch);
    if (e != cudaSuccess || !p)
      return set_error(c, THC_ERR_CUDA, "thc_kmeans_noalloc: cudaGetSymbolAddress: %s",
                       cudaGetErrorString(e));
    g_scratch_ptr[device] = p;
  }
  *out = g_scratch_ptr[device];
  return THC_OK;
}

}  // namespace
}  // namespace thc

extern "C" int thc_kmeans_noalloc(thc_ctx* h, const double* grid, const double* rho,
                                  long long ng, int nmu, const int* init_idx, int max_it,
                                  double threshold, int* out_idx, thc_kmeans_stats* stats)
{
  if (!h) return THC_ERR_ARG;
  thc::Ctx* c = &h->c;
  if (stats) memset(stats, 0, sizeof(*stats));
  if (ng > thc::kNoAllocMaxNg || nmu > thc::kNoAllocMaxNmu || max_it > thc::kNoAllocMaxIt)
    return thc::set_error(c, THC_ERR_SHAPE,
                          "thc_kmeans_noalloc: N_g %lld, N_mu %d, max_it %d exceed the fixed "
                          "scratch limits (N_g <= %lld, N_mu <= %d, max_it <= %d)",
                          ng, nmu, max_it, thc::kNoAllocMaxNg, thc::kNoAllocMaxNmu,
                          thc::kNoAllocMaxIt);
  if (c->device < 0 || c->device >= thc::kMaxDevices) return THC_ERR_ARG;
  if (cudaSetDevice(c->device) != cudaSuccess) return THC_ERR_CUDA;
  void* base = nullptr;
  int st = thc::scratch_for(c, c->device, &base);
  if (st) return st;
  thc::KmAlloc al;
  al.c = c;
  al.base = (char*)base;
  al.cap = thc::kNoAllocBytes;
  return thc::kmeans_run(c, grid, rho, ng, nmu, init_idx, max_it, threshold, out_idx, stats, &al);
}
