// wah_api.cu -- the C ABI (include/wah/wah.h): argument checks, workspace
// layout, stream-ordered launch sequence, host-buffer context.
//
// The reference path this replaces is the CAF OpenCL facade chain of
// src/phases.cpp:713-1088 (spawned kernel actors + mem_ref buffers) and the
// per-batch worker of src/gpu.cpp:356-367.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <new>

#include "wah_common.cuh"

namespace wah {

thread_local uint32_t g_last_launches = 0;
// Tile shape of the digit passes (wah_set_tuning): rows per thread | peer
// mode flags, for digit pass 0 and (upper 16 bits) the later passes, one
// atomic word so concurrent builds read a consistent set.  The default is
// the autotuner's choice on GB300 for a 268M-row 16-bit column: 16 rows per
// thread for pass 0, 12 for the later passes, 3/8 of the peer masks by
// match.any in both.
std::atomic<int> g_tuning{(16 | WAH_TUNE_HYBRID) | WAH_TUNE_LATER(12 | WAH_TUNE_HYBRID)};

uint32_t* last_launches_slot() { return &g_last_launches; }

int passes_for_bound(uint32_t bound) {
  if (bound == 0) return kDigits;  // unknown: plan on the device, skip trivial digits
  int bits = 32 - __builtin_clz(bound);
  return (bits + kRadixBits - 1) / kRadixBits;
}

int sm_count_current() {
  static std::atomic<int> cached[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (dev >= 0 && dev < 64) {
    const int c = cached[dev].load(std::memory_order_relaxed);
    if (c) return c;
  }
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (dev >= 0 && dev < 64) cached[dev].store(sms, std::memory_order_relaxed);
  return sms;
}

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return WAH_OK;
  if (e == cudaErrorMemoryAllocation) return WAH_ENOMEM;
  if (e == cudaErrorNoKernelImageForDevice || e == cudaErrorNoDevice ||
      e == cudaErrorInsufficientDriver)
    return WAH_ENODEV;
  return WAH_ECUDA;
}

// One tile shape: rows per thread | peer mode flag (| WAH_TUNE_PACK in the
// shape of digit pass 0).
static bool valid_shape(int t, bool first) {
  const int items = t & 0xff;
  if (items != 8 && items != 12 && items != 16) return false;
  if ((t & WAH_TUNE_MATCH) && (t & WAH_TUNE_HYBRID)) return false;
  const int flags = WAH_TUNE_MATCH | WAH_TUNE_HYBRID | (first ? WAH_TUNE_PACK : 0);
  return (t & ~(0xff | flags)) == 0;
}

bool valid_tuning(int t) {
  if (t <= 0) return false;
  const int later = (t >> 16) & 0xffff;
  return valid_shape(t & 0xffff, true) && (later == 0 || valid_shape(later, false));
}

LaunchOpts launch_opts(int max_passes, cudaEvent_t* events, int tuning) {
  LaunchOpts o;
  const int t = tuning ? tuning : g_tuning.load(std::memory_order_relaxed);
  const int first = t & 0xffff;
  const int later = (t >> 16) & 0xffff ? (t >> 16) & 0xffff : first;
  o.sort_items = first & 0xff;
  o.sort_peers = (first & WAH_TUNE_MATCH) ? 1 : (first & WAH_TUNE_HYBRID) ? 2 : 0;
  o.later_items = later & 0xff;
  o.later_peers = (later & WAH_TUNE_MATCH) ? 1 : (later & WAH_TUNE_HYBRID) ? 2 : 0;
  o.pack_force = (first & WAH_TUNE_PACK) != 0;
  o.max_passes = max_passes;
  o.sm_count = sm_count_current();
  o.events = events;
  return o;
}

namespace {

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

struct WsLayout {
  size_t ctrl, range_hist, range_counts, zero_end, range_start, seg0, range_first, keyhist,
      keystart, keys_a, rids_a, keys_b, rids_b, total;
};

WsLayout ws_layout(uint64_t n) {
  WsLayout l;
  size_t off = 0;
  // the control block, the histograms and the range counts are contiguous:
  // one memset clears them before each build
  l.ctrl = off;
  off += align_up(sizeof(WahCtrl));
  l.range_hist = off;  // per-range histograms, then the bin totals of each pass
  off += align_up((size_t)kDigits * (kMaxRanges + kBinTotCopies) * kRadix * sizeof(uint32_t));
  l.range_counts = off;
  off += align_up((size_t)kMaxRanges * 4 * sizeof(uint32_t));
  l.zero_end = off;
  l.range_start = off;
  off += align_up((size_t)kMaxRanges * kRadix * sizeof(uint32_t));
  l.seg0 = off;
  off += align_up((size_t)kMaxRanges * kRadix * sizeof(uint32_t));
  l.range_first = off;
  off += align_up((size_t)kMaxRanges * 2 * sizeof(uint32_t));
  l.keyhist = off;
  off += align_up((size_t)65536 * sizeof(uint32_t));
  l.keystart = off;
  off += align_up((ceil_div(std::max<uint64_t>(n, 1), 32) + 16) * sizeof(uint32_t));
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

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// The column view and range arrays of one build inside a workspace.
void workspace_views(const WsLayout& l, unsigned char* ws, uint64_t n, ColumnView* c,
                     RangeArrays* ra) {
  std::memset(c, 0, sizeof(*c));
  c->n = n;
  c->ctrl = reinterpret_cast<WahCtrl*>(ws + l.ctrl);
  c->keys_a = reinterpret_cast<uint32_t*>(ws + l.keys_a);
  c->rids_a = reinterpret_cast<uint32_t*>(ws + l.rids_a);
  c->keys_b = reinterpret_cast<uint32_t*>(ws + l.keys_b);
  c->rids_b = reinterpret_cast<uint32_t*>(ws + l.rids_b);
  c->fixed_sel = -1;
  c->keyhist = reinterpret_cast<uint32_t*>(ws + l.keyhist);
  c->keystart = reinterpret_cast<uint32_t*>(ws + l.keystart);
  c->derive_ok = 0;
  ra->hist = reinterpret_cast<uint32_t*>(ws + l.range_hist);
  ra->bintot = ra->hist + (size_t)kDigits * kMaxRanges * kRadix;
  ra->start = reinterpret_cast<uint32_t*>(ws + l.range_start);
  ra->seg0 = reinterpret_cast<uint32_t*>(ws + l.seg0);
  ra->counts = reinterpret_cast<uint32_t*>(ws + l.range_counts);
  ra->first = reinterpret_cast<uint32_t*>(ws + l.range_first);
  ra->max_ranges = kMaxRanges;
  ra->zero = ws + l.ctrl;
  ra->zero_bytes = l.zero_end - l.ctrl;
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
    case WAH_ECORRUPT: return "index words do not describe the stated rows";
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
  if (!valid_tuning(sort_items)) return WAH_EINVAL;
  g_tuning.store(sort_items, std::memory_order_relaxed);
  return WAH_OK;
}

int wah_get_tuning(void) { return g_tuning.load(std::memory_order_relaxed); }

static int build_impl(const uint32_t* d_values, uint64_t n, uint32_t bound, uint32_t* d_keys,
                      uint32_t* d_offsets, uint32_t* d_index, wah_counts* d_counts,
                      void* d_workspace, size_t workspace_bytes, void* stream,
                      cudaEvent_t* events, int tuning = 0) {
  g_last_launches = 0;
  if (tuning != 0 && !valid_tuning(tuning)) return WAH_EINVAL;
  if (!d_counts || !aligned16(d_counts)) return WAH_EINVAL;
  if (n >= WAH_MAX_ROWS) return WAH_ERANGE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (n == 0) return cuda_status(cudaMemsetAsync(d_counts, 0, sizeof(wah_counts), s));
  if (!d_values || !d_keys || !d_offsets || !d_index || !d_workspace) return WAH_EINVAL;
  if (!aligned16(d_values) || !aligned16(d_workspace)) return WAH_EINVAL;
  const WsLayout l = ws_layout(n);
  if (workspace_bytes < l.total) return WAH_ENOMEM;
  ColumnView c;
  RangeArrays ra;
  workspace_views(l, static_cast<unsigned char*>(d_workspace), n, &c, &ra);
  c.input = d_values;
  c.keys = d_keys;
  c.offsets = d_offsets;
  c.index = d_index;
  wah_output_caps(n, bound, &c.keys_cap, &c.index_cap);
  c.counts = d_counts;  // zeroed by the histogram kernel, the build's first
  c.status = &d_counts->status;
  c.passes = passes_for_bound(bound);
  c.derive_ok = 1;  // an index build: the sorted keys themselves are never read back
  const LaunchOpts o = launch_opts(c.passes, events, tuning);
  if (o.sm_count <= 0) return WAH_ENODEV;
  // the control block is cleared with the histograms (launch_sort_one)
  cudaError_t e = launch_sort_one(c, ra, o, s, &g_last_launches);
  if (e != cudaSuccess) return cuda_status(e);
  return cuda_status(launch_build_one(c, ra, o, s, &g_last_launches));
}

int wah_build(const uint32_t* d_values, uint64_t n, uint32_t bound, uint32_t* d_keys,
              uint32_t* d_offsets, uint32_t* d_index, wah_counts* d_counts, void* d_workspace,
              size_t workspace_bytes, void* stream) {
  return build_impl(d_values, n, bound, d_keys, d_offsets, d_index, d_counts, d_workspace,
                    workspace_bytes, stream, nullptr);
}

int wah_build_tuned(const uint32_t* d_values, uint64_t n, uint32_t bound, uint32_t* d_keys,
                    uint32_t* d_offsets, uint32_t* d_index, wah_counts* d_counts,
                    void* d_workspace, size_t workspace_bytes, int tuning, void* stream) {
  return build_impl(d_values, n, bound, d_keys, d_offsets, d_index, d_counts, d_workspace,
                    workspace_bytes, stream, nullptr, tuning);
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
  ColumnView c;
  RangeArrays ra;
  workspace_views(l, static_cast<unsigned char*>(d_workspace), n, &c, &ra);
  c.input = d_values;
  c.status = d_status;
  c.passes = passes_for_bound(bound);
  const LaunchOpts o = launch_opts(c.passes, nullptr);
  if (o.sm_count <= 0) return WAH_ENODEV;
  // the control block is cleared with the histograms (launch_sort_one)
  cudaError_t e = launch_sort_one(c, ra, o, s, &g_last_launches);
  if (e != cudaSuccess) return cuda_status(e);
  // Deliver the device-chosen final home into the caller's buffers.
  return cuda_status(launch_sort_deliver(c, d_sorted_values, d_rids, s, &g_last_launches));
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
  ColumnView c;
  RangeArrays ra;
  workspace_views(l, static_cast<unsigned char*>(d_workspace), n, &c, &ra);
  c.input = d_sorted_values;
  c.input_rids = d_rids;
  c.fixed_sel = kSelInput;
  c.keys = d_keys;
  c.offsets = d_offsets;
  c.index = d_index;
  wah_output_caps(n, 0, &c.keys_cap, &c.index_cap);
  c.counts = d_counts;
  c.status = &d_counts->status;
  c.passes = kDigits;
  const LaunchOpts o = launch_opts(kDigits, nullptr);
  if (o.sm_count <= 0) return WAH_ENODEV;
  // no sort: the control block and the range counts are cleared here
  e = cudaMemsetAsync(ra.zero, 0, ra.zero_bytes, s);
  if (e != cudaSuccess) return cuda_status(e);
  return cuda_status(launch_build_one(c, ra, o, s, &g_last_launches));
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

// ---------------------------------------------------------------------------
// Thin device helpers for host programs that use only this header (the
// reference's CAF OpenCL manager: find_device_if, global_argument,
// mem_ref::data, dev->synchronize; src/phases.cpp:376-388, :720, :1087).
// ---------------------------------------------------------------------------
extern "C" {

int wah_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n;
}

int wah_device_name(int device, char* out, size_t cap) {
  cudaDeviceProp p;
  if (!out || cap == 0) return WAH_EINVAL;
  cudaError_t e = cudaGetDeviceProperties(&p, device);
  if (e != cudaSuccess) return cuda_status(e);
  std::strncpy(out, p.name, cap - 1);
  out[cap - 1] = '\0';
  return WAH_OK;
}

int wah_device_select(int device) { return cuda_status(cudaSetDevice(device)); }

int wah_dev_alloc(size_t bytes, void** out) {
  if (!out) return WAH_EINVAL;
  *out = nullptr;
  return cuda_status(cudaMalloc(out, bytes ? bytes : 1));
}

void wah_dev_free(void* p) { cudaFree(p); }

int wah_host_alloc(size_t bytes, void** out) {
  if (!out) return WAH_EINVAL;
  *out = nullptr;
  return cuda_status(cudaMallocHost(out, bytes ? bytes : 1));
}

void wah_host_free(void* p) { cudaFreeHost(p); }

int wah_copy(void* dst, const void* src, size_t bytes, void* stream) {
  return cuda_status(
      cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, static_cast<cudaStream_t>(stream)));
}

int wah_stream_create(void** out) {
  if (!out) return WAH_EINVAL;
  cudaStream_t s = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  *out = s;
  return cuda_status(e);
}

int wah_stream_sync(void* stream) {
  return cuda_status(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
}

void wah_stream_destroy(void* stream) {
  if (stream) cudaStreamDestroy(static_cast<cudaStream_t>(stream));
}

}  // extern "C"

namespace wah {
// The empty kernel of the launch-overhead measurements.
__global__ void k_noop() {}
}  // namespace wah

struct wah_noop_graph {
  cudaGraphExec_t exec = nullptr;
  cudaStream_t capture = nullptr;
};

extern "C" {

int wah_noop(void* stream) {
  k_noop<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>();
  *last_launches_slot() = 1;
  return cuda_status(cudaGetLastError());
}

void wah_noop_graph_destroy(wah_noop_graph* g) {
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->capture) cudaStreamDestroy(g->capture);
  delete g;
}

int wah_noop_graph_create(uint32_t count, wah_noop_graph** out) {
  if (!out || count == 0) return WAH_EINVAL;
  *out = nullptr;
  wah_noop_graph* g = new (std::nothrow) wah_noop_graph;
  if (!g) return WAH_ENOMEM;
  cudaError_t e = cudaStreamCreateWithFlags(&g->capture, cudaStreamNonBlocking);
  cudaGraph_t graph = nullptr;
  if (e == cudaSuccess) e = cudaStreamBeginCapture(g->capture, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    for (uint32_t i = 0; i < count; ++i) k_noop<<<1, 32, 0, g->capture>>>();
    const cudaError_t le = cudaGetLastError();
    e = cudaStreamEndCapture(g->capture, &graph);
    if (e == cudaSuccess) e = le;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    wah_noop_graph_destroy(g);
    return cuda_status(e);
  }
  *out = g;
  return WAH_OK;
}

int wah_noop_graph_launch(wah_noop_graph* g, void* stream) {
  if (!g) return WAH_EINVAL;
  return cuda_status(cudaGraphLaunch(g->exec, static_cast<cudaStream_t>(stream)));
}

}  // extern "C"
