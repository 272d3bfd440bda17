// wah_common.cuh -- shared device helpers for the GB300 WAH index kernels.
//
// Layout of one build's device state (all in the caller's workspace):
//   WahCtrl            pass plan (trivial digits skipped, ping-pong homes),
//                      OR of the keys and of their complements
//   range arrays       per-(range, bin) digit counts and starts; per-range
//                      word/key/segment counts and first positions of the
//                      index build
//   ping-pong buffers  sorted keys and row ids, 4 x n u32
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "wah/wah.h"

namespace wah {

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;  // 256 bins per digit
constexpr int kDigits = 4;               // 32-bit keys -> up to 4 passes

// Packed pass-0 words carry a row's offset in its range in 24 bits; they are
// used where pass-0 ranges hold at least kPackMinRangeRows rows (runs of
// about 256 rows per bin and range, or more), or when a tuning word asks.
constexpr uint64_t kPackRangeRows = 1ull << 24;
constexpr uint64_t kPackMinRangeRows = 1ull << 16;

// Radix scatter: 256 threads (one per bin), rows per thread a tuning choice
// (8/12/16).  The column is cut into at most kMaxRanges equal row ranges, one
// persistent scatter CTA each; histogram/count kernels use
// kCountCtasPerRange CTAs per range.
constexpr int kSortThreads = 256;
constexpr int kMaxRanges = 1024;
constexpr int kCountCtasPerRange = 2;
// Bin totals of a one-column build are summed in this many copies (each
// counting CTA adds to copy blockIdx % kBinTotCopies), which spreads the
// atomics of hundreds of CTAs over as many words per bin.
constexpr int kBinTotCopies = 16;


// Fused index build: 128 threads x 16 rows, blocked.
constexpr int kBuildThreads = 128;
constexpr int kBuildItems = 16;
constexpr int kBuildTile = kBuildThreads * kBuildItems;  // 2048 rows

constexpr int kHistThreads = 256;
constexpr int kHistUnroll = 4;  // uint4 loads in flight per thread
constexpr int kHistWarps = kHistThreads / 32;

// Source/destination selectors of a sort pass.
constexpr int kSelInput = 0;  // the caller's values, rid = row index
constexpr int kSelA = 1;
constexpr int kSelB = 2;

struct WahCtrl {
  int32_t pass_src[kDigits];          // -1: pass skipped (trivial digit)
  int32_t pass_dst[kDigits];
  int32_t final_sel;                  // where the sorted stream ends up
  int32_t derive;                     // key starts replace the sorted keys (ColumnView)
  uint32_t key_or;                    // OR of all keys (range check vs bound)
  uint32_t key_nor;                   // OR of the complements: bits some key has clear
  int32_t narrow;                     // every key below 2^16: 16-bit keys between passes
};


__host__ __device__ constexpr inline uint64_t ceil_div(uint64_t a, uint64_t b) {
  return (a + b - 1) / b;
}

#if defined(__CUDACC__)

__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_relaxed_u64(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(uint64_t* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Streaming 128-bit load (read once: do not keep in L1).
__device__ __forceinline__ uint4 ld_stream_v4(const uint4* p) {
  uint4 v;
  asm volatile("ld.global.cs.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}
__device__ __forceinline__ uint32_t lanemask_gt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_gt;" : "=r"(m));
  return m;
}
// Bit-field extract of `len` bits starting at `pos`.
__device__ __forceinline__ uint32_t bfe(uint32_t x, uint32_t pos, uint32_t len) {
  uint32_t r;
  asm("bfe.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(x), "r"(pos), "r"(len));
  return r;
}

static_assert(kRadixBits == 8, "digits are bytes");
// Byte `byte` (0..3) of x: an 8-bit radix digit in one byte permute.
__device__ __forceinline__ uint32_t digit8(uint32_t x, uint32_t byte) {
  return __byte_perm(x, 0u, 0x4440u | byte);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// mbarrier + bulk-copy (TMA, non-tensor) helpers.
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Orders this thread's (and, after a barrier, the block's) generic-proxy
// shared-memory accesses before later async-proxy (bulk copy) writes.
__device__ __forceinline__ void fence_proxy_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// Global -> shared bulk copy; both addresses 16-byte aligned, bytes % 16 == 0.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for a phase of an mbarrier: false after about kWaitCycles SM
// clocks (~1 s).  try_wait may itself suspend for a while, so the bound is on
// elapsed clocks, not on polls.
constexpr long long kWaitCycles = 2000000000ll;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  long long limit = kWaitCycles) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > limit) return false;
  }
  return true;
}

// First error wins.
__device__ __forceinline__ void set_status(uint32_t* status, uint32_t code) {
  if (status) atomicCAS(status, 0u, code);
}

// Programmatic dependent launch: a one-column build's kernels are launched
// with launch_kernel(programmatic = true), so each is launched as the one
// before it on the stream finishes rather than after it has drained, and
// every kernel of a build calls this first: it waits until that kernel has
// finished and its writes are visible (a no-op for a normal launch).  No
// kernel triggers its dependents early: CTAs parked in this wait would hold
// SM slots, which cost the many-stream serving mix its tail latency.
__device__ __forceinline__ void griddep_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Exclusive scan of one u32 per thread across a block of up to 256 threads
// with one barrier: warp scans, then every thread adds up the totals of the
// warps before its own.  The caller keeps a barrier between its reads of
// s_warp here and the next call's writes.
template <int THREADS>
__device__ __forceinline__ uint32_t block_exclusive_scan_1b(uint32_t x, uint32_t* total,
                                                            uint32_t* s_warp /* THREADS/32 */) {
  static_assert(THREADS <= 256, "one pass over the warp totals");
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= (uint32_t)d) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  uint32_t before = 0, all = 0;
#pragma unroll
  for (int w = 0; w < THREADS / 32; ++w) {
    const uint32_t t = s_warp[w];
    before += (uint32_t)w < warp ? t : 0u;
    all += t;
  }
  *total = all;
  return before + incl - x;
}

// Exclusive scan of one u32 per thread across a block of THREADS threads.
// Returns the thread's exclusive prefix; *total gets the block sum.
template <int THREADS>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t x, uint32_t* total,
                                                         uint32_t* s_warp /* >= THREADS/32 */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < THREADS / 32 ? s_warp[lane] : 0;
    uint32_t wi = w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, wi, d);
      if (lane >= d) wi += y;
    }
    if (lane < THREADS / 32) s_warp[lane] = wi - w;  // exclusive warp prefix
    if (lane == THREADS / 32 - 1) s_warp[THREADS / 32] = wi;
  }
  __syncthreads();
  uint32_t r = s_warp[warp] + incl - x;
  *total = s_warp[THREADS / 32];
  __syncthreads();  // s_warp reusable after return
  return r;
}

// Same for 64-bit packed counters (no carries between fields by construction).
template <int THREADS>
__device__ __forceinline__ uint64_t block_exclusive_scan64(uint64_t x, uint64_t* total,
                                                           uint64_t* s_warp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t incl = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint64_t y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint64_t w = lane < THREADS / 32 ? s_warp[lane] : 0;
    uint64_t wi = w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      uint64_t y = __shfl_up_sync(0xffffffffu, wi, d);
      if (lane >= d) wi += y;
    }
    if (lane < THREADS / 32) s_warp[lane] = wi - w;
    if (lane == THREADS / 32 - 1) s_warp[THREADS / 32] = wi;
  }
  __syncthreads();
  uint64_t r = s_warp[warp] + incl - x;
  *total = s_warp[THREADS / 32];
  __syncthreads();
  return r;
}

#endif  // __CUDACC__

// Timed phases (wah_build_timed): histogram, plan, four digit passes, build;
// then spans of single kernels inside them: each pass's scatter kernel and
// the build's emit kernel.
constexpr int kPhaseHist = 0;
constexpr int kPhasePlan = 1;
constexpr int kPhasePass0 = 2;
constexpr int kPhaseBuild = 6;
constexpr int kPhaseScatter0 = 7;
constexpr int kPhaseEmit = 11;
constexpr int kPhases = 12;

inline void record_phase(cudaEvent_t* ev, int phase, bool end, cudaStream_t s) {
  if (ev) cudaEventRecord(ev[2 * phase + (end ? 1 : 0)], s);
}

#if defined(__CUDACC__)
// Launches a kernel of a build; programmatic: with programmatic stream
// serialization, so it is launched while the kernel before it on the stream
// finishes (in a captured graph, through a programmatic edge) and waits for
// it in griddep_wait before touching memory.  That saves a launch gap per
// kernel boundary, which is what small columns are made of; one-column
// builds use it, batches (the serving mix, several streams) do not.
template <typename... KArgs, typename... Args>
cudaError_t launch_kernel(bool programmatic, void (*kernel)(KArgs...), dim3 grid, dim3 block,
                          size_t smem, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = programmatic ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}
#endif

// ---------------------------------------------------------------------------
// Columns and ranges as the kernels see them.
//
// Every kernel works on row ranges; a range lies inside one column.  A
// geometry maps a range id to (column, rows [lo, hi)) and a column id to its
// buffers.  OneColumn carries the single column of wah_build in the kernel
// parameters; ManyColumns reads per-column and per-range tables from device
// memory (wah_build_batched), so one launch of each kernel covers every
// column of a batch.
// ---------------------------------------------------------------------------
struct ColumnView {
  const uint32_t* input;       // the caller's values (selector kSelInput)
  const uint32_t* input_rids;  // nullptr: rid = row index; else the caller's rids
  uint32_t* keys_a;            // ping-pong homes of the sort (n rows each)
  uint32_t* rids_a;
  uint32_t* keys_b;
  uint32_t* rids_b;
  uint64_t n;
  WahCtrl* ctrl;
  uint32_t* keys;  // outputs
  uint32_t* offsets;
  uint32_t* index;
  uint64_t keys_cap;
  uint64_t index_cap;
  wah_counts* counts;  // build results (nullptr when only sorting)
  uint32_t* status;    // device-side errors of this column
  int32_t passes;      // digit passes its bound allows (1..4)
  int32_t fixed_sel;   // >= 0: the build reads this home instead of final_sel
  // Key starts instead of sorted keys (two active digit passes, index builds
  // of one column): the pass-1 count also counts every 16-bit key
  // (keyhist[65536]), k_key_starts marks where each key starts in the sorted
  // order (keystart, one bit per row) and writes the keys; the last pass then
  // writes row ids only and the index build reads the bits instead of keys.
  uint32_t* keyhist;
  uint32_t* keystart;
  int32_t derive_ok;
  int32_t pad2;
};

struct RangeView {
  uint32_t col;
  uint32_t pad;
  uint64_t lo, hi;  // rows of the column
};

__host__ __device__ __forceinline__ const uint32_t* sel_keys(const ColumnView& c, int s) {
  return s == kSelInput ? c.input : (s == kSelA ? c.keys_a : c.keys_b);
}
// A sort buffer between two digit passes holds 16-bit keys when every key
// fits 16 bits (the OR of the keys, whatever the bound); the caller's input
// and the last pass's output (read by the index build) keep 32-bit keys.  A
// narrow buffer uses the first half of its u32 array.  Valid once the sort
// plan has run.
__device__ __forceinline__ bool narrow_keys(const ColumnView& c, int s) {
  return c.ctrl->narrow && s != kSelInput && s != c.ctrl->final_sel;
}
__host__ __device__ __forceinline__ const uint32_t* sel_rids(const ColumnView& c, int s) {
  return s == kSelInput ? c.input_rids : (s == kSelA ? c.rids_a : c.rids_b);
}

struct OneColumn {
  ColumnView c;
  uint64_t range_rows;  // multiple of every tile size
  uint32_t ranges;
  // Key-start mode packs digit pass 0's output (one word per row: the row's
  // offset in its pass-0 range << 8 | its high digit); the later pass reads
  // the starts of pass 0's (bin, range) runs, bin-major, to recover row ids.
  uint32_t ranges0;        // ranges of digit pass 0
  uint64_t range_rows0;    // rows per pass-0 range (< kPackRangeRows)
  uint32_t* seg0;          // [256 * ranges0] run starts of pass 0, bin-major
  uint32_t* bintot;        // [kBinTotCopies][kDigits][256] rows per bin of each pass
  uint32_t packed;         // key-start mode exchanges packed words (host-decided)
  uint32_t count_parts;    // counting CTAs per range (0: kCountCtasPerRange)
  __device__ __forceinline__ const ColumnView& col(uint32_t) const { return c; }
  __device__ __forceinline__ RangeView range(uint32_t r) const {
    RangeView v;
    v.col = 0;
    v.pad = 0;
    const uint64_t lo = (uint64_t)r * range_rows;
    v.lo = lo < c.n ? lo : c.n;
    v.hi = lo + range_rows < c.n ? lo + range_rows : c.n;
    return v;
  }
  __device__ __forceinline__ uint32_t first_range(uint32_t) const { return 0; }
  __device__ __forceinline__ uint32_t end_range(uint32_t) const { return ranges; }
};

struct ManyColumns {
  const ColumnView* cols;     // [ncols]
  const RangeView* rngs;      // [ranges]; each column's ranges are contiguous
  const uint32_t* col_first;  // [ncols]: first range of each column
  const uint32_t* col_end;    // [ncols]: one past its last range
  __device__ __forceinline__ ColumnView col(uint32_t c) const { return cols[c]; }
  __device__ __forceinline__ RangeView range(uint32_t r) const { return rngs[r]; }
  __device__ __forceinline__ uint32_t first_range(uint32_t c) const { return col_first[c]; }
  __device__ __forceinline__ uint32_t end_range(uint32_t c) const { return col_end[c]; }
};

// Range bookkeeping arrays of one build (device memory).
struct RangeArrays {
  uint32_t* hist;    // [kDigits][max_ranges][256] digit counts per range, zeroed per build
  uint32_t* start;   // [max_ranges][256] first output position per (range, bin)
  uint32_t* seg0;    // [256][max_ranges] pass-0 run starts, bin-major (key-start mode;
                     // nullptr where that mode is not used)
  uint32_t* bintot;  // [kBinTotCopies][kDigits][256] rows per bin, right after hist
                     // (zeroed with it; one-column builds only, else nullptr)
  uint32_t* counts;  // [max_ranges][4] words, keys, segments per range
  uint32_t* first;   // [max_ranges][2] first word and key per range
  uint32_t max_ranges;
  // cleared by one memset before the histogram: for one column the control
  // block, the histograms, the bin totals and the range counts (contiguous
  // in the workspace); for batches the histograms (their range counts are
  // cleared before the build count)
  void* zero;
  size_t zero_bytes;
};

// Tuning and instrumentation of one launch sequence.
struct LaunchOpts {
  int sort_items;       // radix tile rows per thread (8, 12, 16) of digit pass 0
  int sort_peers;       // peer masks: 0 ballots, 1 match.any, 2 half and half
  int later_items;      // the same for the later digit passes (one-column index builds)
  int later_peers;
  int max_passes;       // digit passes launched (max over the columns)
  int sm_count;
  int pack_force;       // key-start mode exchanges packed words whatever the run length
  cudaEvent_t* events;  // optional: [2*phase] before, [2*phase+1] after
};

// Host-side launchers (defined in the .cu files).  The one-column forms
// choose the range geometry themselves; the batched forms take it from the
// plan (ranges, per-column tables).
cudaError_t launch_sort_one(const ColumnView& c, const RangeArrays& ra, const LaunchOpts& o,
                            cudaStream_t s, uint32_t* launches);
cudaError_t launch_build_one(const ColumnView& c, const RangeArrays& ra, const LaunchOpts& o,
                             cudaStream_t s, uint32_t* launches);
cudaError_t launch_sort_many(const ManyColumns& g, uint32_t ncols, uint32_t ranges,
                             const RangeArrays& ra, const LaunchOpts& o, cudaStream_t s,
                             uint32_t* launches);
cudaError_t launch_build_many(const ManyColumns& g, uint32_t ncols, uint32_t ranges,
                              const RangeArrays& ra, const LaunchOpts& o, cudaStream_t s,
                              uint32_t* launches);
// Tile sizes the batched planner must respect (ranges are whole tiles except
// a column's last).
constexpr uint64_t kRangeQuantum = 4096;
cudaError_t launch_sort_deliver(const ColumnView& c, uint32_t* out_keys, uint32_t* out_rids,
                                cudaStream_t s, uint32_t* launches);

// Batched builds (wah_batch.cu): layout of one batch in one device block --
// column table, ranges, per-column range spans, control blocks, range arrays
// and the concatenated ping-pong buffers.
struct BatchLayout {
  uint32_t ncols = 0, nranges = 0;
  int max_passes = 1;
  std::vector<RangeView> ranges;
  std::vector<uint32_t> spans;    // [c] first range, [ncols + 1 + c] end
  std::vector<uint64_t> buf_off;  // row offset of each column in the buffers
  size_t o_cols = 0, o_ranges = 0, o_spans = 0, o_ctrl = 0, o_hist = 0, o_start = 0,
         o_counts = 0, o_rfirst = 0, o_buf = 0, col_bytes = 0, bytes = 0;
};
void plan_batch_layout(const uint64_t* ns, const uint32_t* bounds, uint32_t ncols, int sms,
                       BatchLayout* L);
// Column table for columns placed in `dev` (laid out by L); host memory.
void fill_batch_columns(const BatchLayout& L, unsigned char* dev, const wah_column* cols,
                        ColumnView* out);
// Enqueue the whole build; the column, range and span tables must be in
// `dev` already (stream-ordered before this).
cudaError_t enqueue_batch(const BatchLayout& L, unsigned char* dev, cudaStream_t s,
                          uint32_t* launches, int tuning = 0);

// Shared host helpers (wah_api.cu).
int passes_for_bound(uint32_t bound);
int sm_count_current();
int cuda_status(cudaError_t e);
// tuning: a tuning word as wah_set_tuning takes, 0 = the process default
LaunchOpts launch_opts(int max_passes, cudaEvent_t* events, int tuning = 0);
bool valid_tuning(int tuning);
uint32_t* last_launches_slot();

}  // namespace wah
