// wah_batch.cu -- many columns in one launch sequence (wah_batch_*).
//
// The reference indexes independent row batches one work-group each inside a
// single kernel (kernel_wah_index, include/kernel_wah_bitindex.cl:43-91,
// driven per batch by src/gpu.cpp:194-259), and each batch's index is
// relative to that batch.  Here each column of a batch is indexed exactly as
// wah_build would index it alone, but every kernel of the pipeline runs once
// for the whole batch: columns are cut into row ranges (a range never crosses
// a column), and the per-range tables tell each CTA which column it works on.
// Columns of different widths run their own number of digit passes; trivial
// digits are skipped per column.
//
// The plan (range layout, buffer offsets) depends only on the row counts and
// bounds given at creation; the columns' buffers are set by
// wah_batch_set_columns, which refreshes the device descriptor table, so a
// captured CUDA graph of wah_batch_build can be replayed on new columns of
// the same sizes.
#include <algorithm>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "wah_common.cuh"

using namespace wah;

namespace {

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// Zeroes every column's result counters (they are scattered caller buffers).
__global__ void k_batch_reset(const ColumnView* __restrict__ cols, uint32_t ncols) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncols) {
    wah_counts* k = cols[c].counts;
    k->keycnt = 0;
    k->index_len = 0;
    k->merged = 0;
    k->status = 0;
  }
}

}  // namespace

struct wah_batch {
  uint32_t ncols = 0;
  uint32_t ranges = 0;
  int max_passes = 1;
  std::vector<uint64_t> n;
  std::vector<uint32_t> bound;
  std::vector<uint32_t> order;       // columns by decreasing n (range order)
  std::vector<uint64_t> buf_off;     // row offset of each column in the ping-pong arrays
  std::vector<uint32_t> col_first;   // by column id: first range (+ end in [ncols])
  std::vector<RangeView> host_ranges;
  // device memory (one allocation)
  unsigned char* dev = nullptr;
  size_t dev_bytes = 0;
  ColumnView* d_cols = nullptr;
  RangeView* d_ranges = nullptr;
  uint32_t* d_col_first = nullptr;
  WahCtrl* d_ctrl = nullptr;
  uint32_t* d_keys_a = nullptr;
  uint32_t* d_rids_a = nullptr;
  uint32_t* d_keys_b = nullptr;
  uint32_t* d_rids_b = nullptr;
  RangeArrays ra{};
  // pinned staging of the column table (source of its async upload)
  ColumnView* h_cols = nullptr;
  bool columns_set = false;
  // captured graph of wah_batch_build
  cudaGraphExec_t graph = nullptr;
  cudaStream_t graph_stream = nullptr;
};

extern "C" {

void wah_batch_destroy(wah_batch* b) {
  if (!b) return;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->dev);
  if (b->h_cols) cudaFreeHost(b->h_cols);
  delete b;
}

size_t wah_batch_device_bytes(const wah_batch* b) { return b ? b->dev_bytes : 0; }

uint32_t wah_batch_ranges(const wah_batch* b) { return b ? b->ranges : 0; }

int wah_batch_create(const uint64_t* ns, const uint32_t* bounds, uint32_t ncols,
                     wah_batch** out) {
  if (!out || !ns || ncols == 0) return WAH_EINVAL;
  *out = nullptr;
  for (uint32_t c = 0; c < ncols; ++c)
    if (ns[c] >= WAH_MAX_ROWS) return WAH_ERANGE;
  wah_batch* b = new (std::nothrow) wah_batch;
  if (!b) return WAH_ENOMEM;
  b->ncols = ncols;
  b->n.assign(ns, ns + ncols);
  b->bound.assign(ncols, 0);
  if (bounds) b->bound.assign(bounds, bounds + ncols);
  for (uint32_t c = 0; c < ncols; ++c)
    b->max_passes = std::max(b->max_passes, passes_for_bound(b->bound[c]));

  // Range size: about 8 ranges per resident scatter CTA over the whole batch,
  // whole radix tiles, and at most kMaxRanges ranges per column.
  const int sms = std::max(sm_count_current(), 1);
  const uint64_t total = std::accumulate(b->n.begin(), b->n.end(), (uint64_t)0);
  const uint64_t nmax = *std::max_element(b->n.begin(), b->n.end());
  uint64_t rr = ceil_div(std::max<uint64_t>(total, 1), (uint64_t)sms * 2 * 8);
  rr = std::max<uint64_t>(rr, ceil_div(nmax, kMaxRanges));
  rr = std::max<uint64_t>(ceil_div(rr, kRangeQuantum) * kRangeQuantum, kRangeQuantum);

  // Largest columns first: their long ranges start early, small ones fill
  // the tail.  A column's ranges are contiguous.
  b->order.resize(ncols);
  std::iota(b->order.begin(), b->order.end(), 0u);
  std::stable_sort(b->order.begin(), b->order.end(),
                   [&](uint32_t x, uint32_t y) { return b->n[x] > b->n[y]; });
  b->col_first.assign(ncols + 1, 0);
  std::vector<uint32_t> col_end(ncols, 0);
  for (uint32_t oc : b->order) {
    b->col_first[oc] = (uint32_t)b->host_ranges.size();
    for (uint64_t lo = 0; lo < b->n[oc]; lo += rr) {
      RangeView v;
      v.col = oc;
      v.pad = 0;
      v.lo = lo;
      v.hi = std::min(lo + rr, b->n[oc]);
      b->host_ranges.push_back(v);
    }
    col_end[oc] = (uint32_t)b->host_ranges.size();
  }
  b->ranges = (uint32_t)b->host_ranges.size();
  b->buf_off.resize(ncols);
  uint64_t rows = 0;
  for (uint32_t c = 0; c < ncols; ++c) {
    b->buf_off[c] = rows;
    rows += ceil_div(std::max<uint64_t>(b->n[c], 1), 64) * 64;  // 256-byte aligned columns
  }

  // Device layout.
  const uint32_t R = std::max<uint32_t>(b->ranges, 1);
  size_t off = 0;
  const size_t o_cols = off;
  off += align_up(sizeof(ColumnView) * ncols);
  const size_t o_ranges = off;
  off += align_up(sizeof(RangeView) * R);
  const size_t o_first = off;
  off += align_up(sizeof(uint32_t) * 2 * (ncols + 1));
  const size_t o_ctrl = off;
  off += align_up(sizeof(WahCtrl) * ncols);
  const size_t o_hist = off;
  off += align_up((size_t)kDigits * R * kRadix * 4);
  const size_t o_start = off;
  off += align_up((size_t)R * kRadix * 4);
  const size_t o_counts = off;
  off += align_up((size_t)R * 4 * 4);
  const size_t o_rfirst = off;
  off += align_up((size_t)R * 2 * 4);
  const size_t col_bytes = align_up(rows * 4);
  const size_t o_buf = off;
  off += 4 * col_bytes;
  b->dev_bytes = off;
  cudaError_t e = cudaMalloc(&b->dev, off);
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_cols, sizeof(ColumnView) * ncols);
  if (e != cudaSuccess) {
    wah_batch_destroy(b);
    return cuda_status(e);
  }
  b->d_cols = reinterpret_cast<ColumnView*>(b->dev + o_cols);
  b->d_ranges = reinterpret_cast<RangeView*>(b->dev + o_ranges);
  b->d_col_first = reinterpret_cast<uint32_t*>(b->dev + o_first);
  b->d_ctrl = reinterpret_cast<WahCtrl*>(b->dev + o_ctrl);
  b->ra.hist = reinterpret_cast<uint32_t*>(b->dev + o_hist);
  b->ra.start = reinterpret_cast<uint32_t*>(b->dev + o_start);
  b->ra.counts = reinterpret_cast<uint32_t*>(b->dev + o_counts);
  b->ra.first = reinterpret_cast<uint32_t*>(b->dev + o_rfirst);
  b->ra.max_ranges = R;
  b->d_keys_a = reinterpret_cast<uint32_t*>(b->dev + o_buf);
  b->d_rids_a = reinterpret_cast<uint32_t*>(b->dev + o_buf + col_bytes);
  b->d_keys_b = reinterpret_cast<uint32_t*>(b->dev + o_buf + 2 * col_bytes);
  b->d_rids_b = reinterpret_cast<uint32_t*>(b->dev + o_buf + 3 * col_bytes);

  // Static tables: ranges and per-column range spans ([c] first, [ncols+1+c] end).
  std::vector<uint32_t> spans(2 * (ncols + 1), 0);
  for (uint32_t c = 0; c < ncols; ++c) {
    spans[c] = b->col_first[c];
    spans[ncols + 1 + c] = col_end[c];
  }
  e = cudaMemcpy(b->d_ranges, b->host_ranges.data(), sizeof(RangeView) * b->ranges,
                 cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_col_first, spans.data(), spans.size() * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    wah_batch_destroy(b);
    return cuda_status(e);
  }
  *out = b;
  return WAH_OK;
}

int wah_batch_set_columns(wah_batch* b, const wah_column* cols, void* stream) {
  if (!b || !cols) return WAH_EINVAL;
  for (uint32_t c = 0; c < b->ncols; ++c) {
    const wah_column& x = cols[c];
    if (x.n != b->n[c] || x.bound != b->bound[c]) return WAH_EINVAL;
    if (!x.counts || (reinterpret_cast<uintptr_t>(x.counts) & 15)) return WAH_EINVAL;
    if (x.n > 0 && (!x.values || !x.keys || !x.offsets || !x.index)) return WAH_EINVAL;
    if (reinterpret_cast<uintptr_t>(x.values) & 15) return WAH_EINVAL;
  }
  // wait for the previous upload's source to be consumed before rewriting it
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e);
  for (uint32_t c = 0; c < b->ncols; ++c) {
    const wah_column& x = cols[c];
    ColumnView& v = b->h_cols[c];
    std::memset(&v, 0, sizeof(v));
    v.input = x.values;
    v.input_rids = nullptr;
    v.keys_a = b->d_keys_a + b->buf_off[c];
    v.rids_a = b->d_rids_a + b->buf_off[c];
    v.keys_b = b->d_keys_b + b->buf_off[c];
    v.rids_b = b->d_rids_b + b->buf_off[c];
    v.n = x.n;
    v.ctrl = b->d_ctrl + c;
    v.keys = x.keys;
    v.offsets = x.offsets;
    v.index = x.index;
    wah_output_caps(x.n, x.bound, &v.keys_cap, &v.index_cap);
    v.counts = x.counts;
    v.status = &x.counts->status;
    v.passes = passes_for_bound(x.bound);
    v.fixed_sel = -1;
  }
  e = cudaMemcpyAsync(b->d_cols, b->h_cols, sizeof(ColumnView) * b->ncols,
                      cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_status(e);
  b->columns_set = true;
  return WAH_OK;
}

int wah_batch_build(wah_batch* b, void* stream) {
  if (!b) return WAH_EINVAL;
  if (!b->columns_set) return WAH_EINVAL;
  uint32_t* launches = last_launches_slot();
  *launches = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const LaunchOpts o = launch_opts(b->max_passes, nullptr);
  if (o.sm_count <= 0) return WAH_ENODEV;
  cudaError_t e = cudaMemsetAsync(b->d_ctrl, 0, sizeof(WahCtrl) * b->ncols, s);
  if (e != cudaSuccess) return cuda_status(e);
  k_batch_reset<<<ceil_div(b->ncols, 256), 256, 0, s>>>(b->d_cols, b->ncols);
  ++*launches;
  if (b->ranges == 0) return cuda_status(cudaGetLastError());
  ManyColumns g;
  g.cols = b->d_cols;
  g.rngs = b->d_ranges;
  g.col_first = b->d_col_first;
  g.col_end = b->d_col_first + b->ncols + 1;
  e = launch_sort_many(g, b->ncols, b->ranges, b->ra, o, s, launches);
  if (e != cudaSuccess) return cuda_status(e);
  return cuda_status(launch_build_many(g, b->ncols, b->ranges, b->ra, o, s, launches));
}

int wah_batch_launch_graph(wah_batch* b, void* stream) {
  if (!b || !b->columns_set) return WAH_EINVAL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!b->graph) {
    // capture on a private stream so the caller's stream state is untouched
    cudaStream_t cs;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_status(e);
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int rc = e == cudaSuccess ? wah_batch_build(b, cs) : cuda_status(e);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(cs, &graph);
    if (rc == WAH_OK && e != cudaSuccess) rc = cuda_status(e);
    if (rc == WAH_OK) rc = cuda_status(cudaGraphInstantiate(&b->graph, graph, 0));
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (rc != WAH_OK) return rc;
  }
  return cuda_status(cudaGraphLaunch(b->graph, s));
}

}  // extern "C"
