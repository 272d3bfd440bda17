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
// before anything is enqueued.  All calls share the array and it keeps the
// last call's contents: the build clears everything it needs zeroed itself,
// but two calls whose work overlaps on the GPU (different streams, or
// different host threads, without ordering between them) race on it.
//
// The device address of the array is looked up once per device, with that
// device current, by the first call on it (cudaGetSymbolAddress); make that
// first call before any stream capture on the device.
#include <mutex>

#include "wah_common.cuh"

namespace {

// Workspace of wah_build for WAH_NOALLOC_MAX_ROWS rows (21.4 MiB), rounded up.
constexpr size_t kNoAllocBytes = (size_t)22 << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (set-up on first
// use per device).  Host code cannot pass the symbol itself: on the host it is
// only a stand-in, not a device address.
int noalloc_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return WAH_ENODEV;
  if (dev < 0 || dev >= kMaxDevices) return WAH_ENODEV;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return WAH_ECUDA;
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
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
