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

namespace wah {

void plan_batch_layout(const uint64_t* ns, const uint32_t* bounds, uint32_t ncols, int sms,
                       BatchLayout* L) {
  L->ncols = ncols;
  L->max_passes = 1;
  for (uint32_t c = 0; c < ncols; ++c)
    L->max_passes = std::max(L->max_passes, passes_for_bound(bounds ? bounds[c] : 0));
  // Range size: about 8 ranges per resident scatter CTA over the whole batch,
  // whole radix tiles, and at most kMaxRanges ranges per column.
  uint64_t total = 0, nmax = 0;
  for (uint32_t c = 0; c < ncols; ++c) {
    total += ns[c];
    nmax = std::max<uint64_t>(nmax, ns[c]);
  }
  uint64_t rr = ceil_div(std::max<uint64_t>(total, 1), (uint64_t)std::max(sms, 1) * 2 * 8);
  rr = std::max<uint64_t>(rr, ceil_div(nmax, kMaxRanges));
  rr = std::max<uint64_t>(ceil_div(rr, kRangeQuantum) * kRangeQuantum, kRangeQuantum);
  // Largest columns first: their long ranges start early, small ones fill
  // the tail.  A column's ranges are contiguous.
  std::vector<uint32_t> order(ncols);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(),
                   [&](uint32_t x, uint32_t y) { return ns[x] > ns[y]; });
  L->ranges.clear();
  L->spans.assign(2 * (ncols + 1), 0);
  for (uint32_t oc : order) {
    L->spans[oc] = (uint32_t)L->ranges.size();
    for (uint64_t lo = 0; lo < ns[oc]; lo += rr) {
      RangeView v;
      v.col = oc;
      v.pad = 0;
      v.lo = lo;
      v.hi = std::min(lo + rr, ns[oc]);
      L->ranges.push_back(v);
    }
    L->spans[ncols + 1 + oc] = (uint32_t)L->ranges.size();
  }
  L->nranges = (uint32_t)L->ranges.size();
  L->buf_off.resize(ncols);
  uint64_t rows = 0;
  for (uint32_t c = 0; c < ncols; ++c) {
    L->buf_off[c] = rows;
    rows += ceil_div(std::max<uint64_t>(ns[c], 1), 64) * 64;  // 256-byte aligned columns
  }
  const uint32_t R = std::max<uint32_t>(L->nranges, 1);
  size_t off = 0;
  L->o_cols = off;
  off += align_up(sizeof(ColumnView) * ncols);
  L->o_ranges = off;
  off += align_up(sizeof(RangeView) * R);
  L->o_spans = off;
  off += align_up(sizeof(uint32_t) * 2 * (ncols + 1));
  L->o_ctrl = off;
  off += align_up(sizeof(WahCtrl) * ncols);
  L->o_hist = off;
  off += align_up((size_t)kDigits * R * kRadix * 4);
  L->o_start = off;
  off += align_up((size_t)R * kRadix * 4);
  L->o_counts = off;
  off += align_up((size_t)R * 4 * 4);
  L->o_rfirst = off;
  off += align_up((size_t)R * 2 * 4);
  L->col_bytes = align_up(rows * 4);
  L->o_buf = off;
  off += 4 * L->col_bytes;
  L->bytes = off;
}

void fill_batch_columns(const BatchLayout& L, unsigned char* dev, const wah_column* cols,
                        ColumnView* out) {
  uint32_t* ka = reinterpret_cast<uint32_t*>(dev + L.o_buf);
  uint32_t* ra = reinterpret_cast<uint32_t*>(dev + L.o_buf + L.col_bytes);
  uint32_t* kb = reinterpret_cast<uint32_t*>(dev + L.o_buf + 2 * L.col_bytes);
  uint32_t* rb = reinterpret_cast<uint32_t*>(dev + L.o_buf + 3 * L.col_bytes);
  WahCtrl* ctrl = reinterpret_cast<WahCtrl*>(dev + L.o_ctrl);
  for (uint32_t c = 0; c < L.ncols; ++c) {
    const wah_column& x = cols[c];
    ColumnView& v = out[c];
    std::memset(&v, 0, sizeof(v));
    v.input = x.values;
    v.input_rids = nullptr;
    v.keys_a = ka + L.buf_off[c];
    v.rids_a = ra + L.buf_off[c];
    v.keys_b = kb + L.buf_off[c];
    v.rids_b = rb + L.buf_off[c];
    v.n = x.n;
    v.ctrl = ctrl + c;
    v.keys = x.keys;
    v.offsets = x.offsets;
    v.index = x.index;
    wah_output_caps(x.n, x.bound, &v.keys_cap, &v.index_cap);
    v.counts = x.counts;
    v.status = &x.counts->status;
    v.passes = passes_for_bound(x.bound);
    v.fixed_sel = -1;
  }
}

cudaError_t enqueue_batch(const BatchLayout& L, unsigned char* dev, cudaStream_t s,
                          uint32_t* launches, int tuning) {
  const LaunchOpts o = launch_opts(L.max_passes, nullptr, tuning);
  if (o.sm_count <= 0) return cudaErrorNoDevice;
  ColumnView* d_cols = reinterpret_cast<ColumnView*>(dev + L.o_cols);
  cudaError_t e = cudaMemsetAsync(dev + L.o_ctrl, 0, sizeof(WahCtrl) * L.ncols, s);
  if (e != cudaSuccess) return e;
  k_batch_reset<<<(unsigned)ceil_div(L.ncols, 256), 256, 0, s>>>(d_cols, L.ncols);
  ++*launches;
  if (L.nranges == 0) return cudaGetLastError();
  ManyColumns g;
  g.cols = d_cols;
  g.rngs = reinterpret_cast<const RangeView*>(dev + L.o_ranges);
  g.col_first = reinterpret_cast<const uint32_t*>(dev + L.o_spans);
  g.col_end = g.col_first + L.ncols + 1;
  RangeArrays ra;
  ra.hist = reinterpret_cast<uint32_t*>(dev + L.o_hist);
  ra.start = reinterpret_cast<uint32_t*>(dev + L.o_start);
  ra.seg0 = nullptr;  // no key-start mode in batches
  ra.bintot = nullptr;
  ra.counts = reinterpret_cast<uint32_t*>(dev + L.o_counts);
  ra.first = reinterpret_cast<uint32_t*>(dev + L.o_rfirst);
  ra.max_ranges = std::max<uint32_t>(L.nranges, 1);
  ra.zero = ra.hist;
  ra.zero_bytes = (size_t)kDigits * ra.max_ranges * kRadix * sizeof(uint32_t);
  e = launch_sort_many(g, L.ncols, L.nranges, ra, o, s, launches);
  if (e != cudaSuccess) return e;
  return launch_build_many(g, L.ncols, L.nranges, ra, o, s, launches);
}

}  // namespace wah

struct wah_batch {
  BatchLayout L;
  std::vector<uint64_t> n;
  std::vector<uint32_t> bound;
  unsigned char* dev = nullptr;
  ColumnView* h_cols = nullptr;  // pinned staging of the column table
  bool columns_set = false;
  cudaGraphExec_t graph = nullptr;
  int tuning = 0;  // 0: the process default
};

extern "C" {

void wah_batch_destroy(wah_batch* b) {
  if (!b) return;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->dev);
  if (b->h_cols) cudaFreeHost(b->h_cols);
  delete b;
}

size_t wah_batch_device_bytes(const wah_batch* b) { return b ? b->L.bytes : 0; }

uint32_t wah_batch_ranges(const wah_batch* b) { return b ? b->L.nranges : 0; }

int wah_batch_create(const uint64_t* ns, const uint32_t* bounds, uint32_t ncols,
                     wah_batch** out) {
  return wah_batch_create_tuned(ns, bounds, ncols, 0, out);
}

int wah_batch_create_tuned(const uint64_t* ns, const uint32_t* bounds, uint32_t ncols,
                           int tuning, wah_batch** out) {
  if (!out || !ns || ncols == 0) return WAH_EINVAL;
  *out = nullptr;
  if (tuning != 0 && !valid_tuning(tuning)) return WAH_EINVAL;
  for (uint32_t c = 0; c < ncols; ++c)
    if (ns[c] >= WAH_MAX_ROWS) return WAH_ERANGE;
  wah_batch* b = new (std::nothrow) wah_batch;
  if (!b) return WAH_ENOMEM;
  b->tuning = tuning;
  b->n.assign(ns, ns + ncols);
  b->bound.assign(ncols, 0);
  if (bounds) b->bound.assign(bounds, bounds + ncols);
  plan_batch_layout(ns, b->bound.data(), ncols, sm_count_current(), &b->L);
  cudaError_t e = cudaMalloc(&b->dev, b->L.bytes);
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_cols, sizeof(ColumnView) * ncols);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->dev + b->L.o_ranges, b->L.ranges.data(),
                   sizeof(RangeView) * b->L.nranges, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->dev + b->L.o_spans, b->L.spans.data(), b->L.spans.size() * 4,
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    wah_batch_destroy(b);
    return cuda_status(e);
  }
  *out = b;
  return WAH_OK;
}

int wah_batch_set_columns(wah_batch* b, const wah_column* cols, void* stream) {
  if (!b || !cols) return WAH_EINVAL;
  for (uint32_t c = 0; c < b->L.ncols; ++c) {
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
  fill_batch_columns(b->L, b->dev, cols, b->h_cols);
  e = cudaMemcpyAsync(b->dev + b->L.o_cols, b->h_cols, sizeof(ColumnView) * b->L.ncols,
                      cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_status(e);
  b->columns_set = true;
  return WAH_OK;
}

int wah_batch_build(wah_batch* b, void* stream) {
  if (!b || !b->columns_set) return WAH_EINVAL;
  uint32_t* launches = last_launches_slot();
  *launches = 0;
  return cuda_status(
      enqueue_batch(b->L, b->dev, static_cast<cudaStream_t>(stream), launches, b->tuning));
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
