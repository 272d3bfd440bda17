// wah_api.cu -- the C ABI (include/wah/wah.h): argument checks, workspace
// layout, stream-ordered launch sequence, host-buffer context.
//
// The reference path this replaces is the CAF OpenCL facade chain of
// src/phases.cpp:713-1088 (spawned kernel actors + mem_ref buffers) and the
// per-batch worker of src/gpu.cpp:356-367.
#include <algorithm>
#include <cstring>
#include <new>

#include "wah_common.cuh"

namespace wah {
namespace {

thread_local uint32_t g_last_launches = 0;
int g_sort_items = 16;      // onesweep rows per thread (wah_set_tuning)
int g_sort_peers = 0;       // peer-mask mode (wah_set_tuning)

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

struct WsLayout {
  size_t ctrl, range_hist, range_start, lb_build, keys_a, rids_a, keys_b, rids_b, total;
};

WsLayout ws_layout(uint64_t n) {
  WsLayout l;
  size_t off = 0;
  l.ctrl = off;
  off += align_up(sizeof(WahCtrl));
  l.range_hist = off;
  off += align_up((size_t)kDigits * kMaxRanges * kRadix * sizeof(uint32_t));
  l.range_start = off;
  off += align_up((size_t)kMaxRanges * kRadix * sizeof(uint32_t));
  l.lb_build = off;
  off += align_up((size_t)kMaxRanges * 6 * sizeof(uint32_t));
  const size_t col = align_up(std::max<uint64_t>(n, 1) * sizeof(uint32_t));
  l.keys_a = off;
  off += col;
  l.rids_a = off;
  off += col;
  l.keys_b = off;
  off += col;
  l.rids_b = off;
  off += col;
  l.total = off;
  return l;
}

int passes_for_bound(uint32_t bound) {
  if (bound == 0) return kDigits;  // unknown: plan on the device, skip trivial digits
  int bits = 32 - __builtin_clz(bound);
  return (bits + kRadixBits - 1) / kRadixBits;
}

int sm_count_current() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (dev < 64 && cached[dev]) return cached[dev];
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (dev < 64) cached[dev] = sms;
  return sms;
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return WAH_OK;
  if (e == cudaErrorMemoryAllocation) return WAH_ENOMEM;
  if (e == cudaErrorNoKernelImageForDevice || e == cudaErrorNoDevice ||
      e == cudaErrorInsufficientDriver)
    return WAH_ENODEV;
  return WAH_ECUDA;
}

// Sort into the workspace ping-pong buffers; the final home is chosen on the
// device (WahCtrl::final_sel).
int enqueue_sort(const uint32_t* d_values, uint64_t n, uint32_t bound, const WsLayout& l,
                 unsigned char* ws, uint32_t* status, cudaStream_t s, uint32_t* launches,
                 SortBufs* bufs_out, cudaEvent_t* events = nullptr) {
  WahCtrl* ctrl = reinterpret_cast<WahCtrl*>(ws + l.ctrl);
  cudaError_t e = cudaMemsetAsync(ctrl, 0, sizeof(WahCtrl), s);
  if (e != cudaSuccess) return cuda_status(e);
  SortLaunch a;
  a.values = d_values;
  a.n = n;
  a.passes = passes_for_bound(bound);
  a.ctrl = ctrl;
  a.range_hist = reinterpret_cast<uint32_t*>(ws + l.range_hist);
  a.range_start = reinterpret_cast<uint32_t*>(ws + l.range_start);
  a.buf_keys[0] = reinterpret_cast<uint32_t*>(ws + l.keys_a);
  a.buf_rids[0] = reinterpret_cast<uint32_t*>(ws + l.rids_a);
  a.buf_keys[1] = reinterpret_cast<uint32_t*>(ws + l.keys_b);
  a.buf_rids[1] = reinterpret_cast<uint32_t*>(ws + l.rids_b);
  a.status = status;
  a.events = events;
  a.sort_items = g_sort_items;
  a.sort_peers = g_sort_peers;
  a.sm_count = sm_count_current();
  if (a.sm_count <= 0) return WAH_ENODEV;
  e = launch_sort(a, s, launches);
  if (e != cudaSuccess) return cuda_status(e);
  bufs_out->keys[kSelInput] = d_values;
  bufs_out->rids[kSelInput] = nullptr;
  bufs_out->keys[kSelA] = a.buf_keys[0];
  bufs_out->rids[kSelA] = a.buf_rids[0];
  bufs_out->keys[kSelB] = a.buf_keys[1];
  bufs_out->rids[kSelB] = a.buf_rids[1];
  return WAH_OK;
}

}  // namespace
}  // namespace wah

using namespace wah;

extern "C" {

const char* wah_strerror(int status) {
  switch (status) {
    case WAH_OK: return "ok";
    case WAH_EINVAL: return "invalid argument";
    case WAH_ENOMEM: return "out of memory / workspace too small";
    case WAH_ECUDA: return "CUDA runtime error";
    case WAH_ETIMEOUT: return "device-side wait timed out";
    case WAH_ERANGE: return "value or size out of range";
    case WAH_EOVERFLOW: return "output capacity exceeded";
    case WAH_ENODEV: return "no usable sm_103 device";
    default: return "unknown status";
  }
}

void wah_output_caps(uint64_t n, uint32_t bound, uint64_t* keys_cap, uint64_t* index_cap) {
  uint64_t kc = n;
  if (bound != 0) kc = std::min<uint64_t>(n, (uint64_t)bound + 1);
  if (keys_cap) *keys_cap = kc;
  if (index_cap) *index_cap = 2 * n;
}

size_t wah_workspace_bytes(uint64_t n, uint32_t /*bound*/) { return ws_layout(n).total; }

uint32_t wah_last_launch_count(void) { return g_last_launches; }

int wah_set_tuning(int sort_items) {
  const int items = sort_items & 0xff;
  if (items != 8 && items != 12 && items != 16) return WAH_EINVAL;
  if ((sort_items & WAH_TUNE_MATCH) && (sort_items & WAH_TUNE_HYBRID)) return WAH_EINVAL;
  g_sort_items = items;
  g_sort_peers = (sort_items & WAH_TUNE_MATCH) ? 1 : (sort_items & WAH_TUNE_HYBRID) ? 2 : 0;
  return WAH_OK;
}

int wah_get_tuning(void) {
  return g_sort_items | (g_sort_peers == 1 ? WAH_TUNE_MATCH : 0) |
         (g_sort_peers == 2 ? WAH_TUNE_HYBRID : 0);
}

static int build_impl(const uint32_t* d_values, uint64_t n, uint32_t bound, uint32_t* d_keys,
                      uint32_t* d_offsets, uint32_t* d_index, wah_counts* d_counts,
                      void* d_workspace, size_t workspace_bytes, void* stream,
                      cudaEvent_t* events) {
  g_last_launches = 0;
  if (!d_counts || !aligned16(d_counts)) return WAH_EINVAL;
  if (n >= WAH_MAX_ROWS) return WAH_ERANGE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(d_counts, 0, sizeof(wah_counts), s);
  if (e != cudaSuccess) return cuda_status(e);
  if (n == 0) return WAH_OK;
  if (!d_values || !d_keys || !d_offsets || !d_index || !d_workspace) return WAH_EINVAL;
  if (!aligned16(d_values) || !aligned16(d_workspace)) return WAH_EINVAL;
  const WsLayout l = ws_layout(n);
  if (workspace_bytes < l.total) return WAH_ENOMEM;
  unsigned char* ws = static_cast<unsigned char*>(d_workspace);

  SortBufs bufs;
  int rc = enqueue_sort(d_values, n, bound, l, ws, &d_counts->status, s, &g_last_launches, &bufs,
                        events);
  if (rc != WAH_OK) return rc;

  BuildLaunch b;
  b.events = events;
  b.src = bufs;
  b.sel = -1;
  b.n = n;
  b.ctrl = reinterpret_cast<WahCtrl*>(ws + l.ctrl);
  b.range_counts = reinterpret_cast<uint32_t*>(ws + l.lb_build);
  b.range_first = b.range_counts + kMaxRanges * 4;
  b.sm_count = sm_count_current();
  b.keys = d_keys;
  b.offsets = d_offsets;
  b.index = d_index;
  wah_output_caps(n, bound, &b.keys_cap, &b.index_cap);
  b.counts = d_counts;
  return cuda_status(launch_build(b, s, &g_last_launches));
}

int wah_build(const uint32_t* d_values, uint64_t n, uint32_t bound, uint32_t* d_keys,
              uint32_t* d_offsets, uint32_t* d_index, wah_counts* d_counts, void* d_workspace,
              size_t workspace_bytes, void* stream) {
  return build_impl(d_values, n, bound, d_keys, d_offsets, d_index, d_counts, d_workspace,
                    workspace_bytes, stream, nullptr);
}

int wah_events_create(uint32_t count, void** events) {
  if (!events) return WAH_EINVAL;
  for (uint32_t i = 0; i < count; ++i) {
    cudaEvent_t e;
    cudaError_t err = cudaEventCreate(&e);
    if (err != cudaSuccess) return cuda_status(err);
    events[i] = e;
  }
  return WAH_OK;
}

void wah_events_destroy(uint32_t count, void** events) {
  if (!events) return;
  for (uint32_t i = 0; i < count; ++i)
    if (events[i]) cudaEventDestroy(static_cast<cudaEvent_t>(events[i]));
}

int wah_events_elapsed(void* start, void* end, float* ms) {
  if (!start || !end || !ms) return WAH_EINVAL;
  return cuda_status(cudaEventElapsedTime(ms, static_cast<cudaEvent_t>(start),
                                          static_cast<cudaEvent_t>(end)));
}

int wah_build_timed(const uint32_t* d_values, uint64_t n, uint32_t bound, uint32_t* d_keys,
                    uint32_t* d_offsets, uint32_t* d_index, wah_counts* d_counts,
                    void* d_workspace, size_t workspace_bytes, void* stream, void** events) {
  if (!events) return WAH_EINVAL;
  return build_impl(d_values, n, bound, d_keys, d_offsets, d_index, d_counts, d_workspace,
                    workspace_bytes, stream, reinterpret_cast<cudaEvent_t*>(events));
}

int wah_sort_rids_by_value(const uint32_t* d_values, uint64_t n, uint32_t bound,
                           uint32_t* d_sorted_values, uint32_t* d_rids, uint32_t* d_status,
                           void* d_workspace, size_t workspace_bytes, void* stream) {
  g_last_launches = 0;
  if (n >= WAH_MAX_ROWS) return WAH_ERANGE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (d_status) {
    cudaError_t e = cudaMemsetAsync(d_status, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return cuda_status(e);
  }
  if (n == 0) return WAH_OK;
  if (!d_values || !d_sorted_values || !d_rids || !d_workspace) return WAH_EINVAL;
  if (!aligned16(d_values) || !aligned16(d_workspace)) return WAH_EINVAL;
  const WsLayout l = ws_layout(n);
  if (workspace_bytes < l.total) return WAH_ENOMEM;
  unsigned char* ws = static_cast<unsigned char*>(d_workspace);
  SortBufs bufs;
  int rc = enqueue_sort(d_values, n, bound, l, ws, d_status, s, &g_last_launches, &bufs);
  if (rc != WAH_OK) return rc;
  // Deliver the device-chosen final home into the caller's buffers.
  rc = cuda_status(
      launch_sort_deliver(bufs, reinterpret_cast<WahCtrl*>(ws + l.ctrl), n, d_sorted_values,
                          d_rids, s, &g_last_launches));
  return rc;
}

int wah_build_sorted(const uint32_t* d_sorted_values, const uint32_t* d_rids, uint64_t n,
                     uint32_t* d_keys, uint32_t* d_offsets, uint32_t* d_index,
                     wah_counts* d_counts, void* d_workspace, size_t workspace_bytes,
                     void* stream) {
  g_last_launches = 0;
  if (!d_counts || !aligned16(d_counts)) return WAH_EINVAL;
  if (n >= WAH_MAX_ROWS) return WAH_ERANGE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(d_counts, 0, sizeof(wah_counts), s);
  if (e != cudaSuccess) return cuda_status(e);
  if (n == 0) return WAH_OK;
  if (!d_sorted_values || !d_rids || !d_keys || !d_offsets || !d_index || !d_workspace)
    return WAH_EINVAL;
  if (!aligned16(d_sorted_values) || !aligned16(d_rids)) return WAH_EINVAL;
  const WsLayout l = ws_layout(n);
  if (workspace_bytes < l.total) return WAH_ENOMEM;
  unsigned char* ws = static_cast<unsigned char*>(d_workspace);
  WahCtrl* ctrl = reinterpret_cast<WahCtrl*>(ws + l.ctrl);
  e = cudaMemsetAsync(ctrl, 0, sizeof(WahCtrl), s);
  if (e != cudaSuccess) return cuda_status(e);
  BuildLaunch b;
  b.events = nullptr;
  b.src.keys[0] = d_sorted_values;
  b.src.rids[0] = d_rids;
  b.src.keys[1] = b.src.keys[2] = nullptr;
  b.src.rids[1] = b.src.rids[2] = nullptr;
  b.sel = 0;
  b.n = n;
  b.ctrl = ctrl;
  b.range_counts = reinterpret_cast<uint32_t*>(ws + l.lb_build);
  b.range_first = b.range_counts + kMaxRanges * 4;
  b.sm_count = sm_count_current();
  b.keys = d_keys;
  b.offsets = d_offsets;
  b.index = d_index;
  wah_output_caps(n, 0, &b.keys_cap, &b.index_cap);
  b.counts = d_counts;
  return cuda_status(launch_build(b, s, &g_last_launches));
}

// ---------------------------------------------------------------------------
// Host-buffer context.
// ---------------------------------------------------------------------------
struct wah_ctx {
  uint64_t max_n = 0;
  uint32_t bound = 0;
  cudaStream_t stream = nullptr;
  uint32_t* d_values = nullptr;
  uint32_t* d_keys = nullptr;
  uint32_t* d_offsets = nullptr;
  uint32_t* d_index = nullptr;
  wah_counts* d_counts = nullptr;
  wah_counts* h_counts = nullptr;  // pinned
  void* d_ws = nullptr;
  size_t ws_bytes = 0;
};

void wah_ctx_destroy(wah_ctx* c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  cudaFree(c->d_values);
  cudaFree(c->d_keys);
  cudaFree(c->d_offsets);
  cudaFree(c->d_index);
  cudaFree(c->d_counts);
  cudaFree(c->d_ws);
  if (c->h_counts) cudaFreeHost(c->h_counts);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int wah_ctx_create(uint64_t max_n, uint32_t bound, wah_ctx** out) {
  if (!out) return WAH_EINVAL;
  *out = nullptr;
  if (max_n >= WAH_MAX_ROWS) return WAH_ERANGE;
  wah_ctx* c = new (std::nothrow) wah_ctx;
  if (!c) return WAH_ENOMEM;
  c->max_n = max_n;
  c->bound = bound;
  uint64_t keys_cap, index_cap;
  wah_output_caps(std::max<uint64_t>(max_n, 1), bound, &keys_cap, &index_cap);
  c->ws_bytes = wah_workspace_bytes(std::max<uint64_t>(max_n, 1), bound);
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_values, std::max<uint64_t>(max_n, 1) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_keys, keys_cap * 4);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_offsets, keys_cap * 4);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_index, index_cap * 4);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_counts, sizeof(wah_counts));
  if (e == cudaSuccess) e = cudaMalloc(&c->d_ws, c->ws_bytes);
  if (e == cudaSuccess) e = cudaMallocHost(&c->h_counts, sizeof(wah_counts));
  if (e != cudaSuccess) {
    wah_ctx_destroy(c);
    return cuda_status(e);
  }
  *out = c;
  return WAH_OK;
}

int wah_ctx_build_host(wah_ctx* c, const uint32_t* h_values, uint64_t n, uint32_t* h_keys,
                       uint32_t* h_offsets, uint32_t* h_index, wah_counts* h_counts) {
  if (!c || !h_counts) return WAH_EINVAL;
  if (n > c->max_n) return WAH_ERANGE;
  if (n > 0 && (!h_values || !h_keys || !h_offsets || !h_index)) return WAH_EINVAL;
  cudaError_t e = cudaSuccess;
  if (n > 0) e = cudaMemcpyAsync(c->d_values, h_values, n * 4, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_status(e);
  int rc = wah_build(c->d_values, n, c->bound, c->d_keys, c->d_offsets, c->d_index, c->d_counts,
                     c->d_ws, c->ws_bytes, c->stream);
  const uint32_t launches = g_last_launches;
  if (rc != WAH_OK) return rc;
  e = cudaMemcpyAsync(c->h_counts, c->d_counts, sizeof(wah_counts), cudaMemcpyDeviceToHost,
                      c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_status(e);
  *h_counts = *c->h_counts;
  g_last_launches = launches;
  if (h_counts->status != WAH_OK) return (int)h_counts->status;
  const uint64_t K = h_counts->keycnt, L = h_counts->index_len;
  if (K) e = cudaMemcpyAsync(h_keys, c->d_keys, K * 4, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess && K)
    e = cudaMemcpyAsync(h_offsets, c->d_offsets, K * 4, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess && L)
    e = cudaMemcpyAsync(h_index, c->d_index, L * 4, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return cuda_status(e);
}

}  // extern "C"
