// wah_noalloc.cu -- wah_build_noalloc: the index build for callers that may
// not allocate device memory.
//
// Some callers own every byte of device memory and cannot call cudaMalloc:
// an ingest plugin inside a database or stream engine whose host process
// hands out device memory from its own pool and forbids plugins from calling
// the CUDA allocator, and serving loops where a cudaMalloc/cudaFree pair would
// add a device-wide synchronisation to every request.  They still provide the
// column and the output buffers; this entry point takes the rest of what the
// build needs (the sort ping-pong buffers, digit histograms, range counters
// and key-start bits) from one fixed array in this library's device image.
//
// The array is a file-scope __device__ variable of kNoAllocBytes, so every
// GPU that loads the library holds it until the process exits.  Columns of up
// to WAH_NOALLOC_MAX_ROWS rows fit; longer ones are refused with WAH_ERANGE
// before anything is enqueued (d_counts is then left untouched).  All calls
// share the array and it keeps the last call's contents: the build clears
// everything it needs zeroed itself, but two calls whose work overlaps on the
// GPU (different streams, or different host threads, without ordering
// between them) race on it.
//
// The array has its own device address in every CUDA context that loads the
// library (the primary context of each device, a context the caller created
// with the driver API, a context re-created after cudaDeviceReset).  So every
// call looks the address up again in the context current on the calling
// thread (cudaGetSymbolAddress: a host-side table lookup once the module is
// loaded, no allocation and no device work); nothing is cached across calls.
// The first call in a context loads the library's device code into it when
// loading is lazy: make that first call before any stream capture.
#include "wah_common.cuh"

namespace {

// Workspace of wah_build for WAH_NOALLOC_MAX_ROWS rows (22.4 MiB), rounded up.
constexpr size_t kNoAllocBytes = (size_t)24 << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of g_noalloc_scratch in the current context.  Host code
// cannot pass the symbol itself: on the host it is only a stand-in, not a
// device address.
int noalloc_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return WAH_ENODEV;
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return WAH_ECUDA;
  *out = p;
  return WAH_OK;
}

}  // namespace

extern "C" int wah_build_noalloc(const uint32_t* d_values, uint64_t n, uint32_t bound,
                                 uint32_t* d_keys, uint32_t* d_offsets, uint32_t* d_index,
                                 wah_counts* d_counts, void* stream) {
  if (n > WAH_NOALLOC_MAX_ROWS) return WAH_ERANGE;
  const size_t need = wah_workspace_bytes(n, bound);
  if (need > kNoAllocBytes) return WAH_ERANGE;
  void* scratch = nullptr;
  const int rc = noalloc_scratch(&scratch);
  if (rc != WAH_OK) return rc;
  return wah_build(d_values, n, bound, d_keys, d_offsets, d_index, d_counts, scratch,
                   kNoAllocBytes, stream);
}
