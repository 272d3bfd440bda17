// wah_index.cu -- phases a2..a6 fused over the sorted (value, rid) stream.
//
// Reference steps (sequential semantics, src/cpu.cpp):
//   produce_chunk_id_literals  chid = rid / 31, lit = 1<<31 | 1<<(rid % 31)
//                              (:201-211)
//   merged_lit_by_val_chids    OR-reduce runs of equal (value, chid) (:78-116)
//   produce_fills              head of a value: fill = chid; else
//                              fill = chid - prev_chid - 1 (:223-241)
//   fuse_fill_literals         [fill, lit] per entry, zero words dropped
//                              (:245-257, :170-174)
//   compute_colum_length       keys, per-key word counts, exclusive-scanned
//                              offsets (:261-272)
// The reference GPU path runs these as ~20 kernels with three stream
// compactions and host read-backs of k (src/phases.cpp:817-1077).
//
// Every row is classified from itself and the row before it: head of a
// (value, chunk) segment when either changes, head of a value when the value
// changes; a head emits 1 + (fill != 0) words.  The sorted stream is cut into
// equal row ranges, one per resident emit CTA:
//   k_build_count  streams the range's rows (128-bit loads) and counts its
//                  words, keys and segments
//   k_build_scan   exclusive scan over ranges: each range's first word and key
//   k_build_emit   one persistent CTA per range (128 threads x 16 rows) walks
//                  its tiles of 2048 rows; the next tile's window (4 rows
//                  behind, 32 ahead: a segment has at most 31 rows, so the
//                  tile owning a segment's head can finish its literal) is
//                  fetched by cp.async.bulk while this one is processed;
//                  literals come from a reverse segmented OR over each
//                  thread's rows; a block scan gives tile-local positions;
//                  words are staged in the tile's own window buffer, keys and
//                  offsets beside it, and written once, coalesced, at the
//                  range's running offsets.  No zero word is ever written and
//                  no compaction pass is needed.
// In key-start mode (the sort's plan: every key below 2^16, both low digits
// vary) the sorted keys are never written; the count and the emit read the
// row ids and one key-start bit per row instead, and the keys come from the
// sort's key counts.
#include <algorithm>
#include <type_traits>

#include "wah_common.cuh"

namespace wah {

constexpr int kLookAhead = 30;  // rows after a tile that can continue its last segment
constexpr int kWinBehind = 4;   // window starts 4 rows before the tile (16-byte aligned)
constexpr int kWinRows = kWinBehind + kBuildTile + 32;  // rows fetched per tile

// Staging index skew: position i lives at i + i/32, so threads writing runs
// that start ~2 x kBuildItems = 32 words apart hit different banks.
__device__ __forceinline__ uint32_t skew(uint32_t i) { return i + (i >> 5); }
constexpr int kSkewed(int n) { return n + n / 32 + 1; }
constexpr int kStagedWords = kSkewed(2 * kBuildTile);  // a tile's words, skewed

// A tile's words (<= 2 per row) and keys (<= 1 per row) pack into one
// 32-bit scan value: words in the low 16 bits, keys in the high 16.
constexpr int kPackShift = 16;
constexpr uint32_t kPackMask = (1u << kPackShift) - 1;
static_assert(2 * kBuildTile <= (int)kPackMask, "tile words fit 16 bits");

// ---------------------------------------------------------------------------
// Count: words, keys, segments per range.
// ---------------------------------------------------------------------------
// Words and segments of one sorted row.  vh: the row starts a key; c, pc:
// the chunk ids of the row and of the row before (pc <= c within a key).
// x = 0: the row's chunk continues the segment (no word); x = 1: a new chunk
// right after the last one (literal only); x >= 2: a zero fill, then the
// literal.  A key's first row has a fill unless its chunk is 0 (x = c + 1).
__device__ __forceinline__ void count_words(bool vh, uint32_t c, uint32_t pc, uint32_t& words,
                                            uint32_t& segs) {
  const uint32_t x = vh ? c + 1 : c - pc;
  words += min(x, 2u);
  segs += min(x, 1u);
}

__device__ __forceinline__ void count_row(uint32_t v, uint32_t c, uint32_t pv, uint32_t pc,
                                          uint32_t& words, uint32_t& keys, uint32_t& segs) {
  const bool vh = v != pv;
  count_words(vh, c, pc, words, segs);
  keys += vh;
}

template <class G>
__global__ void __launch_bounds__(kHistThreads)
    k_build_count(G g, uint32_t* __restrict__ range_counts /* [ranges][4] */) {
  griddep_wait();
  const uint32_t c = blockIdx.x / kCountCtasPerRange, q = blockIdx.x % kCountCtasPerRange;
  const RangeView rv = g.range(c);
  const ColumnView col = g.col(rv.col);
  const int s = col.fixed_sel >= 0 ? col.fixed_sel : col.ctrl->final_sel;
  const uint32_t* __restrict__ sv = sel_keys(col, s);
  const uint32_t* __restrict__ sr = sel_rids(col, s);
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // part q of the range (parts start on multiples of 8 rows: aligned loads,
  // and a lane's 8 rows in one key-start bit word)
  const uint64_t part = ((rv.hi - rv.lo) / kCountCtasPerRange) & ~(uint64_t)7;
  const uint64_t lo = rv.lo + q * part;
  const uint64_t hi = q + 1 == kCountCtasPerRange ? rv.hi : lo + part;

  uint32_t words = 0, keys = 0, segs = 0;
  const uint64_t chunks = (hi - lo) / 128;  // 32 lanes x 4 rows
  if (col.fixed_sel < 0 && col.ctrl->derive) {
    // key heads from the key-start bits (a lane's 8 rows share one bit
    // word), chunks from the row ids; no keys read.  Loads of kHistUnroll
    // chunks of 256 rows are issued together, then counted.
    const uint32_t* __restrict__ ks = col.keystart;
    auto count8 = [&](const uint4& a, const uint4& b, uint32_t bits, uint32_t pr) {
      const uint32_t up = __shfl_up_sync(0xffffffffu, b.w, 1);
      uint32_t pc = (lane == 0 ? pr : up) / 31;
      const uint32_t r[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const uint32_t cj = r[j] / 31;
        count_words((bits >> j) & 1u, cj, pc, words, segs);
        pc = cj;
      }
      keys += __popc(bits & 0xFFu);
    };
    const uint64_t chunks8 = (hi - lo) / 256;  // 32 lanes x 8 rows
    uint64_t k = warp;
    for (; k + (kHistUnroll - 1) * kHistWarps < chunks8; k += kHistUnroll * kHistWarps) {
      uint4 ra[kHistUnroll], rb[kHistUnroll];
      uint32_t bits[kHistUnroll], pr[kHistUnroll];
#pragma unroll
      for (int u = 0; u < kHistUnroll; ++u) {
        const uint64_t p = lo + (k + u * kHistWarps) * 256 + lane * 8;
        ra[u] = ld_stream_v4(reinterpret_cast<const uint4*>(sr + p));
        rb[u] = ld_stream_v4(reinterpret_cast<const uint4*>(sr + p + 4));
        bits[u] = ks[p >> 5] >> (p & 31);
        pr[u] = (lane == 0 && p > 0) ? sr[p - 1] : 0u;
      }
#pragma unroll
      for (int u = 0; u < kHistUnroll; ++u) count8(ra[u], rb[u], bits[u], pr[u]);
    }
    for (; k < chunks8; k += kHistWarps) {
      const uint64_t p = lo + k * 256 + lane * 8;
      count8(ld_stream_v4(reinterpret_cast<const uint4*>(sr + p)),
             ld_stream_v4(reinterpret_cast<const uint4*>(sr + p + 4)), ks[p >> 5] >> (p & 31),
             (lane == 0 && p > 0) ? sr[p - 1] : 0u);
    }
    if (warp == 0) {
      for (uint64_t p = lo + chunks8 * 256 + lane; p < hi; p += 32) {
        const uint32_t cc = sr[p] / 31;
        const uint32_t pc = p > 0 ? sr[p - 1] / 31 : 0u;
        const uint32_t vh = (ks[p >> 5] >> (p & 31)) & 1u;
        count_words(vh, cc, pc, words, segs);
        keys += vh;
      }
    }
  } else {
  for (uint64_t k = warp; k < chunks; k += kHistWarps) {
    const uint64_t p = lo + k * 128 + lane * 4;
    const uint4 v4 = ld_stream_v4(reinterpret_cast<const uint4*>(sv + p));
    uint4 r4;
    if (sr) {
      r4 = ld_stream_v4(reinterpret_cast<const uint4*>(sr + p));
    } else {
      r4 = make_uint4((uint32_t)p, (uint32_t)p + 1, (uint32_t)p + 2, (uint32_t)p + 3);
    }
    // row p - 1: the previous lane's last row, or a load for lane 0
    uint32_t pv = __shfl_up_sync(0xffffffffu, v4.w, 1);
    uint32_t pr = __shfl_up_sync(0xffffffffu, r4.w, 1);
    if (lane == 0) {
      if (p > 0) {
        pv = sv[p - 1];
        pr = sr ? sr[p - 1] : (uint32_t)(p - 1);
      } else {
        pv = ~v4.x;  // row 0 heads a key
        pr = 0;
      }
    }
    const uint32_t pc = pr / 31;
    const uint32_t c0 = r4.x / 31, c1 = r4.y / 31, c2 = r4.z / 31, c3 = r4.w / 31;
    count_row(v4.x, c0, pv, pc, words, keys, segs);
    count_row(v4.y, c1, v4.x, c0, words, keys, segs);
    count_row(v4.z, c2, v4.y, c1, words, keys, segs);
    count_row(v4.w, c3, v4.z, c2, words, keys, segs);
  }
  if (warp == 0) {  // ragged end of the sub-range, one row per lane
    for (uint64_t p = lo + chunks * 128 + lane; p < hi; p += 32) {
      const uint32_t v = sv[p];
      const uint32_t cc = (sr ? sr[p] : (uint32_t)p) / 31;
      uint32_t pv, pc;
      if (p > 0) {
        pv = sv[p - 1];
        pc = (sr ? sr[p - 1] : (uint32_t)(p - 1)) / 31;
      } else {
        pv = ~v;
        pc = 0;
      }
      count_row(v, cc, pv, pc, words, keys, segs);
    }
  }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    words += __shfl_xor_sync(0xffffffffu, words, d);
    keys += __shfl_xor_sync(0xffffffffu, keys, d);
    segs += __shfl_xor_sync(0xffffffffu, segs, d);
  }
  if (lane == 0) {
    if (words) atomicAdd(&range_counts[c * 4 + 0], words);
    if (keys) atomicAdd(&range_counts[c * 4 + 1], keys);
    if (segs) atomicAdd(&range_counts[c * 4 + 2], segs);
  }
}

// Exclusive scan of (words, keys) over ranges; totals into the counts.
constexpr int kBuildScanThreads = 1024;
static_assert(kBuildScanThreads >= kMaxRanges, "one thread per range");

// One CTA per column, one thread per range of the column (<= kMaxRanges).
template <class G>
__global__ void __launch_bounds__(kBuildScanThreads)
    k_build_scan(G g, const uint32_t* __restrict__ range_counts,
                 uint32_t* __restrict__ range_first /* [ranges][2] */) {
  griddep_wait();
  __shared__ uint64_t s_warp[kBuildScanThreads / 32 + 1];
  const ColumnView col = g.col(blockIdx.x);
  const uint32_t r0 = g.first_range(blockIdx.x), r1 = g.end_range(blockIdx.x);
  const uint32_t c = r0 + threadIdx.x;
  uint64_t x = 0;
  uint32_t segs = 0;
  if (c < r1) {
    x = ((uint64_t)range_counts[c * 4 + 1] << 32) | range_counts[c * 4 + 0];
    segs = range_counts[c * 4 + 2];
  }
  uint64_t total;
  const uint64_t excl = block_exclusive_scan64<kBuildScanThreads>(x, &total, s_warp);
  if (c < r1) {
    range_first[c * 2 + 0] = (uint32_t)(excl & 0xffffffffu);
    range_first[c * 2 + 1] = (uint32_t)(excl >> 32);
  }
  if (segs) atomicAdd(&col.counts->merged, segs);
  if (threadIdx.x == 0) {
    col.counts->index_len = (uint32_t)(total & 0xffffffffu);
    col.counts->keycnt = (uint32_t)(total >> 32);
  }
}

// ---------------------------------------------------------------------------
// Emit.
// ---------------------------------------------------------------------------
struct EmitSmem {
  // Per buffer: the window's keys (or key-start bits) and row ids, rows
  // base-4 .. base+TILE+31.  Once every thread has its rows (the tile scan's
  // barrier), the current buffer stages the tile's words in skewed order.
  struct Win {
    uint32_t v[kWinRows];
    uint32_t r[kWinRows];
    uint32_t pad[(kStagedWords - 2 * kWinRows + 3) / 4 * 4];
  } win[2];
  uint32_t keys[kSkewed(kBuildTile)];
  uint32_t offs[kSkewed(kBuildTile)];
  uint32_t warp_tot[kBuildThreads / 32];  // the warps' packed (words, keys) totals
  uint64_t red[3 * (kBuildThreads / 32)];  // one column: the range-start sums
  uint64_t bar[2];
  int abort;
};
static_assert(sizeof(EmitSmem::Win) >= kStagedWords * sizeof(uint32_t), "staging fits a buffer");
static_assert(sizeof(EmitSmem::Win) % 16 == 0, "16-byte aligned bulk-copy targets");

// A tile's window can come by bulk copy when all its rows exist and it does
// not start before row 0.
__device__ __forceinline__ bool window_bulk(uint64_t base, uint64_t n) {
  return base >= (uint64_t)kWinBehind && base + kBuildTile + 32 <= n;
}

// Derive mode: the key-start bits of rows base .. base+TILE+95 take the
// place of the keys in wv (base is a multiple of the tile, so the bit words
// start 16-byte aligned; the bit array has 16 words of slack at its end).
constexpr uint32_t kWinBitWords = 68;

__device__ __forceinline__ void fetch_window(uint32_t* wv, uint32_t* wr, uint64_t* bar,
                                             const uint32_t* sv, const uint32_t* sr,
                                             const uint32_t* ks, uint64_t base, bool derive) {
  const uint32_t bytes = kWinRows * 4u;
  const uint32_t vbytes = derive ? kWinBitWords * 4u : bytes;
  fence_proxy_async_shared();
  mbar_arrive_expect_tx(bar, vbytes + (sr ? bytes : 0u));
  if (derive) bulk_copy_g2s(wv, ks + (base >> 5), vbytes, bar);
  else bulk_copy_g2s(wv, sv + base - kWinBehind, bytes, bar);
  if (sr) bulk_copy_g2s(wr, sr + base - kWinBehind, bytes, bar);
}

// One column: range r's first word and key are the sums of the word and key
// counts of ranges 0 .. r-1, summed by the emit CTA itself instead of a
// separate scan launch; CTA 0 also sums every range and writes the column's
// totals (the index length, the key count, the merged entries).
__device__ __forceinline__ void own_range_start(const OneColumn& g,
                                                const uint32_t* __restrict__ counts,
                                                uint32_t* run_w, uint32_t* run_k,
                                                uint64_t* s_red) {
  const uint32_t r = blockIdx.x, nr = g.ranges;
  const uint32_t lim = r == 0 ? nr : r;
  uint64_t mine = 0, all = 0, segs = 0;
  for (uint32_t i = threadIdx.x; i < lim; i += kBuildThreads) {
    const uint4 c = reinterpret_cast<const uint4*>(counts)[i];
    const uint64_t x = ((uint64_t)c.y << 32) | c.x;  // keys, words
    all += x;
    segs += c.z;
    if (i < r) mine += x;
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    mine += __shfl_xor_sync(0xffffffffu, mine, d);
    all += __shfl_xor_sync(0xffffffffu, all, d);
    segs += __shfl_xor_sync(0xffffffffu, segs, d);
  }
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int NW = kBuildThreads / 32;
  if (lane == 0) {
    s_red[warp] = mine;
    s_red[NW + warp] = all;
    s_red[2 * NW + warp] = segs;
  }
  __syncthreads();
  uint64_t m = 0, a = 0, sg = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    m += s_red[w];
    a += s_red[NW + w];
    sg += s_red[2 * NW + w];
  }
  *run_w = (uint32_t)(m & 0xffffffffu);
  *run_k = (uint32_t)(m >> 32);
  if (r == 0 && threadIdx.x == 0) {
    const ColumnView& col = g.col(0);
    col.counts->index_len = (uint32_t)(a & 0xffffffffu);
    col.counts->keycnt = (uint32_t)(a >> 32);
    col.counts->merged = (uint32_t)sg;
  }
  __syncthreads();
}

// kDerive: key heads from the key-start bits, keys written already (derive
// mode, one column only)
template <class G, bool kDerive>
__device__ __forceinline__ void build_emit(const G& g, const uint32_t* __restrict__ range_first,
                                           EmitSmem& sm) {
  const RangeView rv = g.range(blockIdx.x);
  const ColumnView col = g.col(rv.col);
  const int s = col.fixed_sel >= 0 ? col.fixed_sel : col.ctrl->final_sel;
  const uint32_t* __restrict__ sv = sel_keys(col, s);
  const uint32_t* __restrict__ sr = sel_rids(col, s);
  uint32_t* __restrict__ out_index = col.index;
  uint32_t* __restrict__ out_keys = col.keys;
  uint32_t* __restrict__ out_offsets = col.offsets;
  const uint64_t keys_cap = col.keys_cap, index_cap = col.index_cap;
  uint32_t* status = col.status;
  constexpr bool derive = kDerive;
  const uint32_t* __restrict__ ks = col.keystart;

  const uint32_t tid = threadIdx.x;
  const uint64_t n = col.n;
  const uint64_t lo = rv.lo, hi = rv.hi;
  if (lo >= hi) return;
  const uint32_t ntiles = (uint32_t)ceil_div(hi - lo, kBuildTile);
  uint32_t run_w, run_k;  // words and keys before this tile
  if constexpr (std::is_same<G, OneColumn>::value) {
    // range_first holds the per-range counts here
    own_range_start(g, range_first, &run_w, &run_k, sm.red);
  } else {
    run_w = range_first[blockIdx.x * 2 + 0];
    run_k = range_first[blockIdx.x * 2 + 1];
  }

  if (tid == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    sm.abort = 0;
    fence_mbar_init();
    if (window_bulk(lo, n))
      fetch_window(sm.win[0].v, sm.win[0].r, &sm.bar[0], sv, sr, ks, lo, derive);
  }
  __syncthreads();

  const uint32_t first = tid * kBuildItems;  // this thread's first tile row
  uint32_t phase_bits = 0;  // parity of the next phase of bar[0], bar[1]
  for (uint32_t i = 0; i < ntiles; ++i) {
    const uint32_t cur = i & 1;
    const uint64_t base = lo + (uint64_t)i * kBuildTile;
    const uint32_t valid = hi - base < kBuildTile ? (uint32_t)(hi - base) : kBuildTile;
    if (tid == 0 && i + 1 < ntiles && window_bulk(base + kBuildTile, n))
      fetch_window(sm.win[cur ^ 1].v, sm.win[cur ^ 1].r, &sm.bar[cur ^ 1], sv, sr, ks,
                   base + kBuildTile, derive);
    uint32_t* wv = sm.win[cur].v;
    uint32_t* wr = sm.win[cur].r;
    // the tile's staged words, in the same buffer once its rows are read
    uint32_t* words = sm.win[cur].v;
    // rows of the window that exist, counted from the tile start
    const uint64_t left = n - base;
    const uint32_t wend = left < (uint64_t)(kBuildTile + kLookAhead)
                              ? (uint32_t)left
                              : (uint32_t)(kBuildTile + kLookAhead);
    if (window_bulk(base, n)) {
      // phases of each buffer's barrier complete in turn; the parity of the
      // next one is tracked per buffer (a tile read with plain loads uses none)
      const bool ok = mbar_wait_bounded(&sm.bar[cur], (phase_bits >> cur) & 1u);
      phase_bits ^= 1u << cur;
      if (!ok) {
        set_status(status, WAH_ETIMEOUT);
        sm.abort = 1;
      }
      if (!sr) {  // identity row ids: the bulk copy brought values only
        for (uint32_t w = tid; w < kWinRows; w += kBuildThreads)
          wr[w] = (uint32_t)(base - kWinBehind + w);
        __syncthreads();
      }
    } else {
      // First or last tiles of the column: plain loads of the rows that exist.
      for (uint32_t w = tid; w < kWinRows; w += kBuildThreads) {
        const uint64_t row = base - kWinBehind + w;  // wraps below row 0: excluded
        if (row < n) {
          if (!derive) wv[w] = sv[row];
          wr[w] = sr ? sr[row] : (uint32_t)row;
        }
      }
      if (derive && tid < kWinBitWords && base + 32ull * tid < n) wv[tid] = ks[(base >> 5) + tid];
      __syncthreads();
    }

    // This thread's rows from the window (16-byte loads).
    static_assert(kBuildItems % 4 == 0, "whole 16-byte loads");
    uint32_t v[kBuildItems], ch[kBuildItems], bt[kBuildItems];  // key, chunk, bit in chunk
    {
      const uint4* r4 = reinterpret_cast<const uint4*>(wr + kWinBehind + first);
      const uint4* v4 = reinterpret_cast<const uint4*>(wv + kWinBehind + first);
#pragma unroll
      for (int q = 0; q < kBuildItems / 4; ++q) {
        const uint4 b = r4[q];
        const uint32_t r[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          ch[4 * q + i] = r[i] / 31;
          bt[4 * q + i] = r[i] - ch[4 * q + i] * 31;
        }
        if (!derive) {
          const uint4 a = v4[q];
          v[4 * q + 0] = a.x; v[4 * q + 1] = a.y; v[4 * q + 2] = a.z; v[4 * q + 3] = a.w;
        } else {
          v[4 * q + 0] = v[4 * q + 1] = v[4 * q + 2] = v[4 * q + 3] = 0;
        }
      }
    }
    const bool full = valid == kBuildTile;
    // rows that exist from the tile start: rows past the range end but before
    // n still belong to segments that started in the range
    const uint32_t exist = left < (uint64_t)kBuildTile ? (uint32_t)left : (uint32_t)kBuildTile;
    // the row before the thread's first row (row 0 of the column heads a key)
    uint32_t pv, pc;
    if (base + first > 0) {
      pv = derive ? 0u : wv[kWinBehind + first - 1];
      pc = wr[kWinBehind + first - 1] / 31;
    } else {
      pv = ~v[0];
      pc = 0;
    }
    // derive mode: which of this thread's rows start a key (one bit word;
    // the row offset is a multiple of the rows per thread, which divides 32)
    static_assert(32 % kBuildItems == 0, "a thread's key-start bits in one word");
    constexpr uint32_t kItemMask = (1u << kBuildItems) - 1;
    const uint32_t kbits = derive ? (wv[first >> 5] >> (first & 31)) & kItemMask : 0u;

    uint32_t headm = 0, vheadm = 0, fills[kBuildItems];
    uint32_t nw = 0;
#pragma unroll
    for (int j = 0; j < kBuildItems; ++j) {
      const uint32_t c = ch[j];
      const bool ok = full || first + j < valid;
      const bool vh = derive ? ((kbits >> j) & 1u) != 0 : v[j] != pv;
      // x as in count_words: 0 continues the segment, else the fill is x - 1
      const uint32_t x = vh ? c + 1 : c - pc;
      fills[j] = x - 1;
      if (ok && x != 0) {
        headm |= 1u << j;
        if (vh) vheadm |= 1u << j;
        nw += min(x, 2u);
      }
      pv = v[j];
      pc = c;
    }
    const uint32_t nk = __popc(vheadm);
    // A warp whose every thread has 16 heads, each with a fill, and no key
    // start (most warps of a column whose keys are spread over its chunks)
    // writes its words in a fixed pattern: fill, literal, row by row.
    const bool fast = __all_sync(0xffffffffu, full && nw == 2u * kBuildItems && vheadm == 0);

    // Literals: the rows after this thread's last row that continue its last
    // segment (from the window), then a reverse segmented OR over its rows.
    uint32_t acc = 0x80000000u;  // the literal flag, set from the start
    {
      const uint32_t v7 = v[kBuildItems - 1], c7 = ch[kBuildItems - 1];
      for (uint32_t m = first + kBuildItems; m < wend; ++m) {
        const uint32_t rm = wr[kWinBehind + m];
        if (rm / 31 != c7) break;
        if (derive) {
          if ((wv[m >> 5] >> (m & 31)) & 1u) break;  // m < wend <= TILE + 30
        } else if (wv[kWinBehind + m] != v7) {
          break;
        }
        acc |= 1u << (rm % 31);
      }
    }
    uint32_t lits[kBuildItems];
    if (fast) {  // every row is its own segment; the last one takes the continuation
#pragma unroll
      for (int j = 0; j < kBuildItems; ++j) lits[j] = 0x80000000u | (1u << bt[j]);
      lits[kBuildItems - 1] |= acc;
    } else {
#pragma unroll
      for (int j = kBuildItems - 1; j >= 0; --j) {
        if (first + j < exist) acc |= 1u << bt[j];  // rows past n add nothing
        lits[j] = acc;
        if (headm & (1u << j)) acc = 0x80000000u;
      }
    }

    // Tile scan of (words, keys); the warp totals are read before the
    // staging barrier below and written again after the tile's last one.
    uint32_t tile_agg;
    const uint32_t my_prefix = block_exclusive_scan_1b<kBuildThreads>(
        nw | (nk << kPackShift), &tile_agg, sm.warp_tot);
    const uint32_t tw = tile_agg & kPackMask;
    const uint32_t tk = tile_agg >> kPackShift;

    uint32_t pw = my_prefix & kPackMask;
    uint32_t pk = my_prefix >> kPackShift;
    if (fast) {
#pragma unroll
      for (int j = 0; j < kBuildItems; ++j) {
        words[skew(pw + 2 * j)] = fills[j];
        words[skew(pw + 2 * j + 1)] = lits[j];
      }
    } else {
#pragma unroll
      for (int j = 0; j < kBuildItems; ++j) {
        if (headm & (1u << j)) {
          if (vheadm & (1u << j)) {
            if (!derive) sm.keys[skew(pk)] = v[j];
            sm.offs[skew(pk)] = run_w + pw;
            ++pk;
          }
          if (fills[j]) words[skew(pw++)] = fills[j];
          words[skew(pw++)] = lits[j];
        }
      }
    }
    __syncthreads();

    if (!sm.abort) {
      bool overflow = false;
      if ((uint64_t)run_w + tw <= index_cap &&
          (reinterpret_cast<uintptr_t>(out_index) & 15) == 0) {
        // words up to the next 16-byte boundary of the index, then groups of
        // four with one 16-byte store each, then the rest
        const uint32_t head = ((4u - (run_w & 3u)) & 3u) < tw ? ((4u - (run_w & 3u)) & 3u) : tw;
        if (tid < head) out_index[run_w + tid] = words[skew(tid)];
        const uint32_t groups = (tw - head) >> 2;
        for (uint32_t g = tid; g < groups; g += kBuildThreads) {
          const uint32_t k = head + 4 * g;
          uint4 q;
          q.x = words[skew(k)];
          q.y = words[skew(k + 1)];
          q.z = words[skew(k + 2)];
          q.w = words[skew(k + 3)];
          *reinterpret_cast<uint4*>(out_index + run_w + k) = q;
        }
        const uint32_t tail = head + 4 * groups;
        if (tid < tw - tail) out_index[run_w + tail + tid] = words[skew(tail + tid)];
      } else {
        for (uint32_t k = tid; k < tw; k += kBuildThreads) {
          const uint64_t pos = (uint64_t)run_w + k;
          if (pos < index_cap)
            out_index[pos] = words[skew(k)];
          else
            overflow = true;
        }
      }
      for (uint32_t k = tid; k < tk; k += kBuildThreads) {
        const uint64_t pos = (uint64_t)run_k + k;
        if (pos < keys_cap) {
          if (!derive) out_keys[pos] = sm.keys[skew(k)];
          out_offsets[pos] = sm.offs[skew(k)];
        } else {
          overflow = true;
        }
      }
      if (overflow) set_status(status, WAH_EOVERFLOW);
    }
    run_w += tw;
    run_k += tk;
    __syncthreads();  // staging and window buffer reusable
  }
}

template <class G>
__global__ void __launch_bounds__(kBuildThreads, 4)
    k_build_emit(G g, const uint32_t* __restrict__ range_first) {
  griddep_wait();
  extern __shared__ __align__(128) unsigned char smem_raw[];
  EmitSmem& sm = *reinterpret_cast<EmitSmem*>(smem_raw);
  if constexpr (std::is_same<G, OneColumn>::value) {
    const ColumnView& col = g.col(0);
    if (col.fixed_sel < 0 && col.ctrl->derive) {
      build_emit<G, true>(g, range_first, sm);
      return;
    }
  }
  build_emit<G, false>(g, range_first, sm);
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
template <class G>
cudaError_t launch_build_t(const G& g, uint32_t ncols, uint32_t ranges, const RangeArrays& ra,
                           const LaunchOpts& o, cudaStream_t s, uint32_t* launches) {
  constexpr bool kPdl = std::is_same<G, OneColumn>::value;  // programmatic launches
  const size_t smem = sizeof(EmitSmem);
  cudaError_t err = cudaFuncSetAttribute(k_build_emit<G>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  if constexpr (!std::is_same<G, OneColumn>::value) {  // one column: cleared before the sort
    err = cudaMemsetAsync(ra.counts, 0, (size_t)ra.max_ranges * 4 * sizeof(uint32_t), s);
    if (err != cudaSuccess) return err;
  }
  record_phase(o.events, kPhaseBuild, false, s);
  err = launch_kernel(kPdl,k_build_count<G>, ranges * kCountCtasPerRange, kHistThreads, 0, s, g,
                   ra.counts);
  if (err != cudaSuccess) return err;
  if constexpr (!std::is_same<G, OneColumn>::value) {  // one column: inside the emit
    err = launch_kernel(kPdl,k_build_scan<G>, ncols, kBuildScanThreads, 0, s, g,
                     (const uint32_t*)ra.counts, ra.first);
    if (err != cudaSuccess) return err;
    ++*launches;
  }
  record_phase(o.events, kPhaseEmit, false, s);
  err = launch_kernel(kPdl,k_build_emit<G>, ranges, kBuildThreads, smem, s, g,
                   (const uint32_t*)(std::is_same<G, OneColumn>::value ? ra.counts : ra.first));
  if (err != cudaSuccess) return err;
  record_phase(o.events, kPhaseEmit, true, s);
  record_phase(o.events, kPhaseBuild, true, s);
  *launches += 2;
  return cudaSuccess;
}

cudaError_t launch_build_one(const ColumnView& c, const RangeArrays& ra, const LaunchOpts& o,
                             cudaStream_t s, uint32_t* launches) {
  int per_sm = 0;
  cudaError_t err = cudaFuncSetAttribute(k_build_emit<OneColumn>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(EmitSmem));
  if (err != cudaSuccess) return err;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_build_emit<OneColumn>,
                                                      kBuildThreads, sizeof(EmitSmem));
  if (err != cudaSuccess) return err;
  uint64_t want = (uint64_t)std::max(o.sm_count, 1) * std::max(per_sm, 1);
  if (want > ra.max_ranges) want = ra.max_ranges;
  OneColumn g{};
  g.c = c;
  g.range_rows =
      std::max<uint64_t>(ceil_div(ceil_div(c.n, want), kBuildTile) * kBuildTile, kBuildTile);
  g.ranges = (uint32_t)std::max<uint64_t>(ceil_div(c.n, g.range_rows), 1);
  return launch_build_t<OneColumn>(g, 1, g.ranges, ra, o, s, launches);
}

cudaError_t launch_build_many(const ManyColumns& g, uint32_t ncols, uint32_t ranges,
                              const RangeArrays& ra, const LaunchOpts& o, cudaStream_t s,
                              uint32_t* launches) {
  return launch_build_t<ManyColumns>(g, ncols, ranges, ra, o, s, launches);
}

}  // namespace wah
