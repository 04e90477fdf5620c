// sort_noalloc.cu - the radix sort with scratch memory that lives inside the library.
//
// rtp_radix_sort needs a scratch buffer from its caller.  Some callers cannot allocate
// device memory at the point where they sort: a plugin inside a host application whose
// engine owns the GPU heap and forbids other allocations, a frame loop that must not stall
// on cudaMalloc's implicit device synchronisation, or code that must not be able to fail
// with out-of-memory after start-up.  rtp_radix_sort_noalloc serves them from a fixed
// array declared here, so it never calls cudaMalloc, cudaFree or any allocating routine.
//
// Costs and limits: the array (RTP_NOALLOC_SORT_SCRATCH_BYTES, about 5 MiB) is held by
// every GPU that loads the library until the process exits; one call sorts at most
// RTP_NOALLOC_SORT_MAX_KEYS keys; all calls share the array, so calls that overlap on the
// GPU (different streams, or host threads without ordering) race and must be serialised
// by the caller.  The array keeps the last call's contents; each call clears the
// histogram area it accumulates into before using it.
#include <cuda.h>

#include <mutex>

#include "rtp_internal.hpp"

namespace rtp {
namespace {

constexpr size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr uint32_t kMaxKeys = RTP_NOALLOC_SORT_MAX_KEYS;
constexpr uint32_t kMaxTiles = (kMaxKeys + kSortTile - 1) / kSortTile;
constexpr int kMaxPasses = (32 + kMaxRadixBits - 1) / kMaxRadixBits;
// Same layout as sort_scratch_bytes(): 4 key/index arrays, per-pass tile histograms, totals,
// digit-scan group sums (one group: kMaxTiles <= kScanTilesPerGroup).
static_assert(kMaxTiles <= kScanTilesPerGroup, "one digit-scan group");
constexpr size_t kScratchBytes = 4 * al256(sizeof(uint32_t) * (size_t)kMaxKeys) +
                                 al256(sizeof(uint32_t) * (size_t)kMaxPasses * kMaxTiles * kMaxBins) +
                                 al256(sizeof(uint32_t) * (size_t)kMaxPasses * kMaxBins) +
                                 al256(sizeof(uint32_t) * (size_t)kMaxBins);
static_assert(kScratchBytes == RTP_NOALLOC_SORT_SCRATCH_BYTES, "keep rtp.h in step with the scratch layout");

// The scratch itself: file scope, one copy per device that loads the library.
static __device__ __align__(256) unsigned char g_sort_scratch[kScratchBytes];

// Host code cannot use g_sort_scratch's name as a device address: the address is looked up
// with the device current and cached per device together with the identity of the context it
// was looked up in (cuCtxGetId: unique for the life of the process).  A call from another
// context on that device, or after cudaDeviceReset re-created the primary context, finds a
// different identity and looks the address up again (that call must not be under stream
// capture).  The driver entry points are resolved through the runtime, so the library does
// not link libcuda.
constexpr int kMaxDevices = 128;
struct ScratchAddress {
  unsigned long long ctxId;
  void* ptr;
};
std::mutex g_mutex;
ScratchAddress g_scratch_address[kMaxDevices] = {};
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

int resolve_driver_entry_points() {  // caller holds g_mutex
  if (g_ctx_get_current && g_ctx_get_id) return RTP_OK;
  void* f0 = nullptr;
  void* f1 = nullptr;
  cudaDriverEntryPointQueryResult q0 = cudaDriverEntryPointSymbolNotFound, q1 = cudaDriverEntryPointSymbolNotFound;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDriverEntryPointByVersion(cuCtxGetCurrent)");
  e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDriverEntryPointByVersion(cuCtxGetId)");
  if (q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1)
    return fail(RTP_ERR_NOT_SUPPORTED, "rtp_radix_sort_noalloc: driver lacks cuCtxGetCurrent / cuCtxGetId");
  g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f0);
  g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f1);
  return RTP_OK;
}

// Identity of the context current on the calling thread; with none current yet, the device's
// primary context is made current first (cudaSetDevice initialises it).
int current_context_id(int dev, unsigned long long* id) {  // caller holds g_mutex
  CUcontext ctx = nullptr;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return fail(RTP_ERR_CUDA, "rtp_radix_sort_noalloc: cuCtxGetCurrent failed");
  if (!ctx) {
    RTP_CUDA(cudaSetDevice(dev));
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx)
      return fail(RTP_ERR_CUDA, "rtp_radix_sort_noalloc: no CUDA context is current");
  }
  if (g_ctx_get_id(ctx, id) != CUDA_SUCCESS) return fail(RTP_ERR_CUDA, "rtp_radix_sort_noalloc: cuCtxGetId failed");
  return RTP_OK;
}

int scratch_on_current_device(void** out) {
  int dev = -1;
  RTP_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(RTP_ERR_NOT_SUPPORTED, "rtp_radix_sort_noalloc: device ordinal too large");
  std::lock_guard<std::mutex> lock(g_mutex);
  int rc = resolve_driver_entry_points();
  if (rc) return rc;
  unsigned long long id = 0;
  rc = current_context_id(dev, &id);
  if (rc) return rc;
  ScratchAddress& a = g_scratch_address[dev];
  if (!a.ptr || a.ctxId != id) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_sort_scratch)");
    if (!p) return fail(RTP_ERR_CUDA, "rtp_radix_sort_noalloc: null scratch address");
    a.ptr = p;
    a.ctxId = id;
  }
  *out = a.ptr;
  return RTP_OK;
}

}  // namespace
}  // namespace rtp

using namespace rtp;

extern "C" int rtp_radix_sort_noalloc(const uint32_t* d_keys_in, uint32_t n, uint32_t keyBits, uint32_t* d_keys_out,
                                      uint32_t* d_perm_out, void* stream) {
  if (keyBits > 32) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_radix_sort_noalloc: keyBits > 32");
  if (n > kMaxKeys)
    return fail(RTP_ERR_CAPACITY,
                "rtp_radix_sort_noalloc: " + std::to_string(n) + " keys exceed the fixed scratch limit of " +
                    std::to_string(kMaxKeys) + " keys; use rtp_radix_sort with caller-provided scratch");
  if (n == 0) return RTP_OK;
  if (!d_keys_in || !d_keys_out) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_radix_sort_noalloc: null pointer");
  const SortPlan p = make_sort_plan(n, keyBits);
  if (sort_scratch_bytes(p) > kScratchBytes)
    return fail(RTP_ERR_CAPACITY, "rtp_radix_sort_noalloc: plan does not fit the fixed scratch");
  void* scratch = nullptr;
  int rc = scratch_on_current_device(&scratch);
  if (rc) return rc;
  SortScratch s;
  sort_scratch_carve(p, scratch, s);
  Launcher L;
  L.stream = (cudaStream_t)stream;
  rc = launch_sort_clear(p, s, L);  // histograms of passes >= 1 start at zero
  if (rc) return rc;
  rc = launch_sort_histogram(p, d_keys_in, s, L);
  if (rc) return rc;
  GatherList g;
  g.perm = d_perm_out;
  return launch_sort_passes(p, d_keys_in, d_keys_out, s, g, L);
}
