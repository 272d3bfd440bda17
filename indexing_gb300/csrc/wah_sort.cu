// wah_sort.cu -- phase a1, sort_rids_by_value: a stable LSD radix sort of the
// column by value, carrying row ids, with 8-bit digits.
//
// Reference semantics: src/cpu.cpp:180-197 (stable bubble sort by value,
// rids = iota) and src/phases.cpp:143-160 (the same as std::stable_sort).
// The reference GPU path (src/phases.cpp:745-773 over include/radix.cl:65-233)
// runs 4 passes x (count, scan, reorder_kv) of 4-bit digits over the low 16
// bits only.  Here the column is cut into R equal row ranges (R = resident
// scatter CTAs); each range is owned by one persistent CTA, so no CTA ever
// waits for another:
//
//   k_digit_histogram  one read of the keys (128-bit loads): the digit-0
//                      histogram per range, the OR of all keys and the OR of
//                      their complements (one column: also its bin totals,
//                      and CTA 0 zeroes the result counters)
//   k_sort_plan        batches: trivial digits (every key shares them)
//                      skipped, homes of each pass
//   k_range_count      for digit passes after the first: per-range histogram
//                      of the digit over the current order (one read of keys);
//                      in key-start mode also the rows of every 16-bit key
//   k_range_scan       batches: start of every (range, bin) = bin offset (a
//                      scan of the bins' totals over all ranges) + counts of
//                      the same bin in earlier ranges
//   k_range_scan_one   one column: the same starts, one CTA per bin from the
//                      bin totals; digit pass 0 also writes the plan and
//                      zeroes the key counts and key-start bits, and for digit
//                      pass 1 more CTAs of the same launch run the key starts
//                      (the first row of every key in the sorted order marked
//                      in a bit per row, the keys written)
//   k_radix_scatter    per range, tile after tile: the next tile's keys and
//                      row ids are fetched by cp.async.bulk into shared memory
//                      while this one is ranked (warp peer masks, stable per
//                      warp counters), staged in tile-sorted order and written
//                      out run by run at the range's running bin offsets.  The
//                      first active pass takes rid = row index.  Digit pass 0
//                      and the later passes may use different tile shapes,
//                      each over its own ranges; keys between two passes are
//                      16-bit when every key is below 2^16, and in key-start
//                      mode the last pass writes row ids only; where pass-0
//                      ranges are long, the two passes exchange one packed
//                      word per row instead (scatter_pack0 / scatter_pack1).
// Every kernel of a one-column build is launched as a programmatic dependent
// of the one before it (launch_kernel) and waits for it on entry.
#include <algorithm>
#include <numeric>
#include <type_traits>

#include "wah_common.cuh"

namespace wah {

// ---------------------------------------------------------------------------
// Digit histograms: one shared atomic per key and digit into the warp's
// private counters.  (Counting a digit the whole warp shares once per warp,
// found from the warp's OR and AND of the keys, measured slower on every
// distribution, run-clustered ones included: the two warp reductions per key
// cost more than the same-address atomics they save.)
// ---------------------------------------------------------------------------
template <int DIGITS>
struct WarpHist {
  uint32_t (*h)[kRadix];  // this warp's private [DIGITS][256] counters
  int first;              // digit of h[0]
  __device__ __forceinline__ void add(uint32_t x, uint32_t& acc_or, uint32_t& acc_nor) {
    acc_or |= x;
    acc_nor |= ~x;
#pragma unroll
    for (int p = 0; p < DIGITS; ++p) atomicAdd(&h[p][digit8(x, first + p)], 1u);
  }
};

// Histogram of keys[lo, hi) for digits first..first+DIGITS-1 into the
// block-shared s_h[warp][DIGITS][256]; returns the warp's OR of the keys and
// OR of their complements (the bits some key has clear).
template <int DIGITS>
__device__ __forceinline__ uint2 histogram_range(const uint32_t* __restrict__ keys, uint64_t lo,
                                                    uint64_t hi, int first,
                                                    uint32_t (*s_h)[DIGITS][kRadix]) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nwarps = blockDim.x >> 5;
  WarpHist<DIGITS> wh{s_h[warp], first};
  uint32_t acc_or = 0, acc_nor = 0;
  // lo is a multiple of 4 (ranges are whole tiles), so keys + lo is 16-byte
  // aligned.  Work unit: 32 consecutive uint4 (128 keys), one per lane.
  const uint4* kv = reinterpret_cast<const uint4*>(keys + lo);
  const uint64_t rows = hi - lo;
  const uint64_t chunks = rows / 128;
  uint64_t c = warp;
  for (; c + (kHistUnroll - 1) * nwarps < chunks; c += kHistUnroll * nwarps) {
    uint4 q[kHistUnroll];
#pragma unroll
    for (int u = 0; u < kHistUnroll; ++u) q[u] = ld_stream_v4(kv + (c + u * nwarps) * 32 + lane);
#pragma unroll
    for (int u = 0; u < kHistUnroll; ++u) {
      wh.add(q[u].x, acc_or, acc_nor);
      wh.add(q[u].y, acc_or, acc_nor);
      wh.add(q[u].z, acc_or, acc_nor);
      wh.add(q[u].w, acc_or, acc_nor);
    }
  }
  for (; c < chunks; c += nwarps) {
    const uint4 q = ld_stream_v4(kv + c * 32 + lane);
    wh.add(q.x, acc_or, acc_nor);
    wh.add(q.y, acc_or, acc_nor);
    wh.add(q.z, acc_or, acc_nor);
    wh.add(q.w, acc_or, acc_nor);
  }
  // Ragged end (< 128 keys): warp 0, one key per lane.
  if (warp == 0)
    for (uint64_t i = lo + chunks * 128 + lane; i < hi; i += 32)
      wh.add(keys[i], acc_or, acc_nor);
  return make_uint2(__reduce_or_sync(0xffffffffu, acc_or), __reduce_or_sync(0xffffffffu, acc_nor));
}

// 16-bit keys: the same over uint4 loads of 8 keys (lo a multiple of 8).
template <int DIGITS>
__device__ __forceinline__ void histogram_range16(const uint16_t* __restrict__ keys, uint64_t lo,
                                                  uint64_t hi, int first,
                                                  uint32_t (*s_h)[DIGITS][kRadix]) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nwarps = blockDim.x >> 5;
  WarpHist<DIGITS> wh{s_h[warp], first};
  uint32_t acc_or = 0, acc_nor = 0;
  const uint4* kv = reinterpret_cast<const uint4*>(keys + lo);
  const uint64_t chunks = (hi - lo) / 256;  // 32 lanes x 8 keys
  auto add8 = [&](const uint4& q) {
    wh.add(q.x & 0xFFFFu, acc_or, acc_nor);
    wh.add(q.x >> 16, acc_or, acc_nor);
    wh.add(q.y & 0xFFFFu, acc_or, acc_nor);
    wh.add(q.y >> 16, acc_or, acc_nor);
    wh.add(q.z & 0xFFFFu, acc_or, acc_nor);
    wh.add(q.z >> 16, acc_or, acc_nor);
    wh.add(q.w & 0xFFFFu, acc_or, acc_nor);
    wh.add(q.w >> 16, acc_or, acc_nor);
  };
  uint64_t c = warp;
  for (; c + (kHistUnroll - 1) * nwarps < chunks; c += kHistUnroll * nwarps) {
    uint4 q[kHistUnroll];
#pragma unroll
    for (int u = 0; u < kHistUnroll; ++u) q[u] = ld_stream_v4(kv + (c + u * nwarps) * 32 + lane);
#pragma unroll
    for (int u = 0; u < kHistUnroll; ++u) add8(q[u]);
  }
  for (; c < chunks; c += nwarps) add8(ld_stream_v4(kv + c * 32 + lane));
  if (warp == 0)
    for (uint64_t i = lo + chunks * 256 + lane; i < hi; i += 32) wh.add(keys[i], acc_or, acc_nor);
}

// Key-start mode, the count before digit pass 1.  Pass 0 wrote one packed
// word per row, (row offset in its pass-0 range) << 8 | high digit, in order
// of the low digit; a row's low digit is the pass-0 bin its position lies in
// (binoff[d] = first position of bin d, binoff[256] = n).  Counts the high
// digits of the rows into the range's digit-1 counts h1 and every full key
// into keyhist.  A 128-row chunk inside one low-digit bin (all but at most
// 255 chunks of the column) counts its high digits into the warp's counters
// for that low digit, hw, which go to h1 and keyhist when the warp's low
// digit changes (one shared atomic per row); a chunk that spans low digits
// adds its rows to h1 and keyhist one by one.
__device__ __forceinline__ void flush_keyhist(uint32_t* hw, uint32_t* h1, uint32_t d0,
                                              uint32_t lane, uint32_t* __restrict__ keyhist) {
  __syncwarp();
  for (uint32_t d1 = lane; d1 < kRadix; d1 += 32) {
    const uint32_t x = hw[d1];
    if (x) {
      h1[d1] += x;  // the warp's own counters, one lane per bin
      atomicAdd(&keyhist[(d1 << 8) | d0], x);
      hw[d1] = 0;
    }
  }
  __syncwarp();
}

// Low digit of position p: the last bin whose first position is <= p
// (empty bins share their start with the next bin; the last of them is the
// bin p is in).
__device__ __forceinline__ uint32_t bin_of(const uint32_t* binoff, uint32_t p) {
  uint32_t a = 0;
#pragma unroll
  for (uint32_t step = 128; step > 0; step >>= 1)
    if (binoff[a + step] <= p) a += step;
  return a;
}

__device__ __forceinline__ void count_packed_keys(const uint32_t* __restrict__ words, uint64_t lo,
                                                  uint64_t hi, const uint32_t* binoff,
                                                  uint32_t (*s_h)[1][kRadix],
                                                  uint32_t (*s_full)[kRadix],
                                                  uint32_t* __restrict__ keyhist) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nwarps = blockDim.x >> 5;
  uint32_t* h1 = s_h[warp][0];  // digit-1 counts of the range
  uint32_t* hw = s_full[warp];  // digit-1 counts for the warp's current low digit
  uint32_t cur = kRadix;        // the low digit hw counts (none yet)
  uint32_t cur_lo = 0, cur_hi = 0;  // its positions [cur_lo, cur_hi)
  const uint4* wv = reinterpret_cast<const uint4*>(words + lo);
  const uint64_t chunks = (hi - lo) / 128;  // 32 lanes x 4 words
  auto add_chunk = [&](const uint4& q, uint64_t c) {
    const uint32_t c0 = (uint32_t)(lo + c * 128);
    // a warp's chunks ascend, so most lie in the bin of the chunk before:
    // the bin is looked up only when a chunk leaves it
    if (!(c0 >= cur_lo && c0 + 127 < cur_hi)) {
      const uint32_t d0 = bin_of(binoff, c0);
      const uint32_t d_hi = binoff[d0 + 1];
      if (c0 + 127 >= d_hi) {  // the chunk spans low digits: row by row
        const uint32_t w4[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const uint32_t d1 = w4[i] & 0xFFu;
          atomicAdd(&h1[d1], 1u);
          atomicAdd(&keyhist[(d1 << 8) | bin_of(binoff, c0 + lane * 4 + i)], 1u);
        }
        return;
      }
      if (d0 != cur) {
        if (cur < kRadix) flush_keyhist(hw, h1, cur, lane, keyhist);
        cur = d0;
      }
      cur_lo = binoff[d0];
      cur_hi = d_hi;
    }
    atomicAdd(&hw[q.x & 0xFFu], 1u);
    atomicAdd(&hw[q.y & 0xFFu], 1u);
    atomicAdd(&hw[q.z & 0xFFu], 1u);
    atomicAdd(&hw[q.w & 0xFFu], 1u);
  };
  uint64_t c = warp;
  for (; c + (kHistUnroll - 1) * nwarps < chunks; c += kHistUnroll * nwarps) {
    uint4 q[kHistUnroll];
#pragma unroll
    for (int u = 0; u < kHistUnroll; ++u) q[u] = ld_stream_v4(wv + (c + u * nwarps) * 32 + lane);
#pragma unroll
    for (int u = 0; u < kHistUnroll; ++u) add_chunk(q[u], c + u * nwarps);
  }
  for (; c < chunks; c += nwarps) add_chunk(ld_stream_v4(wv + c * 32 + lane), c);
  if (cur < kRadix) flush_keyhist(hw, h1, cur, lane, keyhist);
  __syncwarp();
  if (warp == 0)
    for (uint64_t i = lo + chunks * 128 + lane; i < hi; i += 32) {
      const uint32_t d1 = words[i] & 0xFFu;
      atomicAdd(&h1[d1], 1u);
      atomicAdd(&keyhist[(d1 << 8) | bin_of(binoff, (uint32_t)i)], 1u);
    }
}

// Key-start mode without packed words (columns whose pass-0 runs are short):
// pass 0 wrote 16-bit keys in order of their low digit.  The same counts as
// count_packed_keys, the low digit read from the key itself; 256-row chunks.
__device__ __forceinline__ void histogram_range16_full(const uint16_t* __restrict__ keys,
                                                       uint64_t lo, uint64_t hi,
                                                       uint32_t (*s_h)[1][kRadix],
                                                       uint32_t (*s_full)[kRadix],
                                                       uint32_t* __restrict__ keyhist) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nwarps = blockDim.x >> 5;
  uint32_t* h1 = s_h[warp][0];    // digit-1 counts of the range
  uint32_t* hw = s_full[warp];    // digit-1 counts for the warp's current low digit
  uint32_t cur = kRadix;          // the low digit hw counts (none yet)
  const uint4* kv = reinterpret_cast<const uint4*>(keys + lo);
  const uint64_t chunks = (hi - lo) / 256;  // 32 lanes x 8 keys
  auto add_chunk = [&](const uint4& q) {
    const uint32_t k8[8] = {q.x & 0xFFFFu, q.x >> 16, q.y & 0xFFFFu, q.y >> 16,
                            q.z & 0xFFFFu, q.z >> 16, q.w & 0xFFFFu, q.w >> 16};
    const uint32_t first = __shfl_sync(0xffffffffu, k8[0], 0) & 0xFFu;
    const uint32_t last = __shfl_sync(0xffffffffu, k8[7], 31) & 0xFFu;
    if (first == last) {
      if (first != cur) {
        if (cur < kRadix) flush_keyhist(hw, h1, cur, lane, keyhist);
        cur = first;
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) atomicAdd(&hw[k8[i] >> 8], 1u);
    } else {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        atomicAdd(&h1[k8[i] >> 8], 1u);
        atomicAdd(&keyhist[k8[i]], 1u);
      }
    }
  };
  uint64_t c = warp;
  for (; c + (kHistUnroll - 1) * nwarps < chunks; c += kHistUnroll * nwarps) {
    uint4 q[kHistUnroll];
#pragma unroll
    for (int u = 0; u < kHistUnroll; ++u) q[u] = ld_stream_v4(kv + (c + u * nwarps) * 32 + lane);
#pragma unroll
    for (int u = 0; u < kHistUnroll; ++u) add_chunk(q[u]);
  }
  for (; c < chunks; c += nwarps) add_chunk(ld_stream_v4(kv + c * 32 + lane));
  if (cur < kRadix) flush_keyhist(hw, h1, cur, lane, keyhist);
  __syncwarp();
  if (warp == 0)
    for (uint64_t i = lo + chunks * 256 + lane; i < hi; i += 32) {
      const uint32_t k = keys[i];
      atomicAdd(&h1[k >> 8], 1u);
      atomicAdd(&keyhist[k], 1u);
    }
}

// Counting CTAs per range: two, or one where a one-column build's ranges
// are short.
template <class G>
__device__ __forceinline__ uint32_t count_parts(const G& g) {
  if constexpr (std::is_same<G, OneColumn>::value)
    return g.count_parts ? g.count_parts : kCountCtasPerRange;
  return kCountCtasPerRange;
}

// Part q of `parts` of a range: the rows one counting CTA covers (parts
// start on multiples of 8 rows, so 16-byte loads of 32- and 16-bit keys stay
// aligned).
__device__ __forceinline__ void sub_range(const RangeView& rv, uint32_t q, uint32_t parts,
                                          uint64_t* lo, uint64_t* hi) {
  const uint64_t part = ((rv.hi - rv.lo) / parts) & ~(uint64_t)7;
  *lo = rv.lo + q * part;
  *hi = q + 1 == parts ? rv.hi : *lo + part;
}

// Adds one counting CTA's bin total to its copy of the bin totals.
template <class G>
__device__ __forceinline__ void add_bin_total(const G& g, int pass, uint32_t bin, uint32_t x) {
  if constexpr (std::is_same<G, OneColumn>::value)
    atomicAdd(&g.bintot[((blockIdx.x % kBinTotCopies) * kDigits + pass) * kRadix + bin], x);
}

// One read of the keys: per-range counts of digit 0, and the OR of the keys
// and of their complements (which digits vary at all).  Later digits are
// counted per range by k_range_count over the order they are sorted from.
template <class G>
__global__ void __launch_bounds__(kHistThreads)
    k_digit_histogram(G g, uint32_t* __restrict__ range_hist0) {
  griddep_wait();
  __shared__ uint32_t s_h[kHistWarps][1][kRadix];
  for (int i = threadIdx.x; i < kHistWarps * kRadix; i += kHistThreads) (&s_h[0][0][0])[i] = 0;
  __syncthreads();
  const uint32_t parts = count_parts(g);
  const uint32_t r = blockIdx.x / parts;
  const RangeView rv = g.range(r);
  const ColumnView c = g.col(rv.col);
  if constexpr (std::is_same<G, OneColumn>::value) {
    // an index build's result counters start at zero here: no kernel of the
    // build before this one, and none in it sets a status
    if (blockIdx.x == 0 && threadIdx.x == 0 && c.counts)
      *reinterpret_cast<uint4*>(c.counts) = make_uint4(0, 0, 0, 0);
  }
  uint64_t lo, hi;
  sub_range(rv, blockIdx.x % parts, parts, &lo, &hi);
  const uint2 acc = histogram_range<1>(c.input, lo, hi, 0, s_h);
  if ((threadIdx.x & 31) == 0) {
    if (acc.x) atomicOr(&c.ctrl->key_or, acc.x);
    if (acc.y) atomicOr(&c.ctrl->key_nor, acc.y);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < kRadix; j += kHistThreads) {
    uint32_t s = 0;
#pragma unroll
    for (int w = 0; w < kHistWarps; ++w) s += s_h[w][0][j];
    if (s) {
      atomicAdd(&range_hist0[(uint64_t)r * kRadix + j], s);
      add_bin_total(g, 0, j, s);
    }
  }
}

// Per-range histogram of digit `pass` over the current order of the keys.
template <class G>
__global__ void __launch_bounds__(kHistThreads)
    k_range_count(G g, int pass, uint32_t* __restrict__ range_hist) {
  griddep_wait();
  const uint32_t parts = count_parts(g);
  const uint32_t r = blockIdx.x / parts;
  const RangeView rv = g.range(r);
  const ColumnView c = g.col(rv.col);
  const int src = c.ctrl->pass_src[pass];
  if (src < 0) return;
  const uint32_t* keys = sel_keys(c, src);
  __shared__ uint32_t s_h[kHistWarps][1][kRadix];
  __shared__ uint32_t s_full[kHistWarps][kRadix];
  __shared__ uint32_t s_binoff[kRadix + 1];
  bool packed = false;  // key-start mode with packed pass-0 words
  if constexpr (std::is_same<G, OneColumn>::value) packed = g.packed && c.ctrl->derive && pass == 1;
  for (int i = threadIdx.x; i < kHistWarps * kRadix; i += kHistThreads) {
    (&s_h[0][0][0])[i] = 0;
    (&s_full[0][0])[i] = 0;
  }
  if constexpr (std::is_same<G, OneColumn>::value) {
    // pass-0 bin starts: the run of (bin d, range 0) starts bin d
    if (packed)
      for (int d = threadIdx.x; d <= kRadix; d += kHistThreads)
        s_binoff[d] = d < kRadix ? g.seg0[(uint64_t)d * g.ranges0] : (uint32_t)c.n;
  }
  __syncthreads();
  uint64_t lo, hi;
  sub_range(rv, blockIdx.x % parts, parts, &lo, &hi);
  if (packed) {
    if constexpr (std::is_same<G, OneColumn>::value)
      count_packed_keys(keys, lo, hi, s_binoff, s_h, s_full, c.keyhist);
  } else if (c.ctrl->derive && pass == 1) {  // 16-bit keys in low-digit order
    histogram_range16_full(reinterpret_cast<const uint16_t*>(keys), lo, hi, s_h, s_full,
                           c.keyhist);
  } else if (narrow_keys(c, src))
    histogram_range16<1>(reinterpret_cast<const uint16_t*>(keys), lo, hi, pass, s_h);
  else
    histogram_range<1>(keys, lo, hi, pass, s_h);
  __syncthreads();
  for (int j = threadIdx.x; j < kRadix; j += kHistThreads) {
    uint32_t s = 0;
#pragma unroll
    for (int w = 0; w < kHistWarps; ++w) s += s_h[w][0][j];
    if (s) {
      atomicAdd(&range_hist[(uint64_t)r * kRadix + j], s);
      add_bin_total(g, pass, j, s);
    }
  }
}

// ---------------------------------------------------------------------------
// Pass plan: bin offsets per digit, trivial digits skipped, ping-pong homes.
// ---------------------------------------------------------------------------
// The plan of one column from the OR of its keys and of their complements;
// written to ctrl when `write`, and returns the source of digit pass 0
// (-1: trivial).
__device__ __forceinline__ int plan_column(const ColumnView& c, bool write) {
  WahCtrl* ctrl = c.ctrl;
  const int passes = c.passes;
  const uint32_t key_or = ctrl->key_or;
  // a digit every key shares is trivial: one bin, order unchanged
  const uint32_t varying = key_or & ctrl->key_nor;
  int s_active[kDigits];
  for (int p = 0; p < kDigits; ++p) s_active[p] = digit8(varying, p) != 0;
  int src0 = -1;
  if (write) {
    // every key below 2^16 (digits 2 and 3 then inactive): 16-bit keys
    // between the passes, and key starts when both low digits vary
    ctrl->narrow = (key_or >> 16) == 0;
    ctrl->derive = c.derive_ok && ctrl->narrow && s_active[0] && s_active[1];
    // A set bit above the digits the bound allows: the sort would be wrong.
    if (passes < kDigits && (key_or >> (passes * kRadixBits)) != 0)
      set_status(c.status, WAH_ERANGE);
  }
  int cur = kSelInput;
  for (int p = 0; p < kDigits; ++p) {
    if (p < passes && s_active[p]) {
      const int dst = (cur == kSelA) ? kSelB : kSelA;
      if (p == 0) src0 = cur;
      if (write) {
        ctrl->pass_src[p] = cur;
        ctrl->pass_dst[p] = dst;
      }
      cur = dst;
    } else if (write) {
      ctrl->pass_src[p] = -1;
      ctrl->pass_dst[p] = -1;
    }
  }
  if (write) ctrl->final_sel = cur;
  return src0;
}

template <class G>
__global__ void __launch_bounds__(kRadix) k_sort_plan(G g) {
  griddep_wait();
  if (threadIdx.x == 0) plan_column(g.col(blockIdx.x), true);
}

// Key starts (derive mode): keyhist scanned in key order; the first row of
// every present key in the sorted order gets its bit in keystart, and the
// keys go to the output in order (the index build writes their offsets).
// One thread per key; each CTA first sums the rows and present keys below
// its own 1024 keys.  Rows (< 2^32) and present keys pack into one 64-bit sum.
constexpr int kKeyStartThreads = 1024;
constexpr int kKeyStartCtas = 65536 / kKeyStartThreads;

template <class G>
__device__ __forceinline__ void key_starts(const G& g, uint32_t block, uint64_t* s_warp) {
  const ColumnView c = g.col(0);
  if (!c.ctrl->derive) return;
  const uint32_t k0 = block * kKeyStartThreads;
  const uint4* kh4 = reinterpret_cast<const uint4*>(c.keyhist);
  uint64_t below = 0;
#pragma unroll 4
  for (uint32_t k = threadIdx.x; k < k0 / 4; k += kKeyStartThreads) {
    const uint4 h = kh4[k];
    const uint32_t present = (h.x != 0) + (h.y != 0) + (h.z != 0) + (h.w != 0);
    below += (uint64_t)(h.x + h.y + h.z + h.w) | ((uint64_t)present << 32);
  }
  uint64_t base;
  block_exclusive_scan64<kKeyStartThreads>(below, &base, s_warp);
  const uint32_t key = k0 + threadIdx.x;
  const uint32_t h = c.keyhist[key];
  uint64_t total;
  const uint64_t pre =
      base + block_exclusive_scan64<kKeyStartThreads>(
                 (uint64_t)h | ((uint64_t)(h != 0) << 32), &total, s_warp);
  if (!h) return;
  const uint32_t row = (uint32_t)pre, rank = (uint32_t)(pre >> 32);
  if (row < c.n) atomicOr(&c.keystart[row >> 5], 1u << (row & 31));
  else set_status(c.status, WAH_ECORRUPT);
  if (rank < c.keys_cap) c.keys[rank] = key;
  else set_status(c.status, WAH_EOVERFLOW);
}

// Start of every (range, bin) of one column for one pass: the bin's offset
// (rows of smaller digits in all ranges) plus the bin's rows in earlier
// ranges.  Four threads per bin, each over a quarter of the ranges.
constexpr int kRangeScanParts = 4;
constexpr int kRangeScanThreads = kRadix * kRangeScanParts;

template <class G>
__global__ void __launch_bounds__(kRangeScanThreads)
    k_range_scan(G g, int pass, const uint32_t* __restrict__ range_hist,
                 uint32_t* __restrict__ range_start) {
  griddep_wait();
  __shared__ uint32_t s_warp[kRangeScanThreads / 32 + 1];
  __shared__ uint32_t s_part[kRangeScanParts][kRadix];
  const ColumnView col = g.col(blockIdx.x);
  if (col.ctrl->pass_src[pass] < 0) return;
  const uint32_t b = threadIdx.x % kRadix, q = threadIdx.x / kRadix;
  const uint32_t c0 = g.first_range(blockIdx.x);
  const uint32_t end = g.end_range(blockIdx.x);
  const uint32_t per = (end - c0 + kRangeScanParts - 1) / kRangeScanParts;
  const uint32_t lo = c0 + q * per < end ? c0 + q * per : end;
  const uint32_t hi = lo + per < end ? lo + per : end;
  uint32_t part = 0;
#pragma unroll 8
  for (uint32_t c = lo; c < hi; ++c) part += range_hist[(uint64_t)c * kRadix + b];
  s_part[q][b] = part;
  __syncthreads();
  uint32_t total = 0, before = 0;
#pragma unroll
  for (int k = 0; k < kRangeScanParts; ++k) {
    const uint32_t x = s_part[k][b];
    if (k < (int)q) before += x;
    total += x;
  }
  // threads of part 0 carry the bins' totals through the scan, the others 0
  uint32_t all;
  const uint32_t off = block_exclusive_scan<kRangeScanThreads>(q == 0 ? total : 0u, &all, s_warp);
  __syncthreads();
  if (q == 0) s_part[0][b] = off;
  __syncthreads();
  uint32_t run = s_part[0][b] + before;
  uint32_t c = lo;
  for (; c + 8 <= hi; c += 8) {
    uint32_t h[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) h[u] = range_hist[(uint64_t)(c + u) * kRadix + b];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      range_start[(uint64_t)(c + u) * kRadix + b] = run;
      run += h[u];
    }
  }
  for (; c < hi; ++c) {
    range_start[(uint64_t)c * kRadix + b] = run;
    run += range_hist[(uint64_t)c * kRadix + b];
  }
}

// One column: the same starts with one CTA per bin.  The bin's offset is
// the sum of the totals of the smaller bins (kept by the count kernels), its
// runs follow range by range (a scan of the bin's column of counts).
// The same launch also does the column's plan (digit pass 0: every CTA
// derives it from the key OR and NOR, CTA 0 writes it) and, for digit pass
// 1, the key starts (kKeyStartCtas more CTAs after the 256 bin CTAs): two
// launches fewer per build, which counts for small columns.
constexpr int kRangeScanOneThreads = kMaxRanges;
static_assert(kKeyStartThreads == kRangeScanOneThreads, "key-start CTAs share the launch");
__global__ void __launch_bounds__(kRangeScanOneThreads)
    k_range_scan_one(OneColumn g, int pass, const uint32_t* __restrict__ range_hist,
                     uint32_t* __restrict__ range_start) {
  griddep_wait();
  __shared__ uint32_t s_warp[kRangeScanOneThreads / 32 + 1];
  __shared__ uint64_t s_warp64[kRangeScanOneThreads / 32 + 1];
  if (blockIdx.x >= kRadix) {  // digit pass 1: the key starts
    key_starts(g, blockIdx.x - kRadix, s_warp64);
    return;
  }
  if (pass == 0) {
    // key-start mode's key counts and bits start at zero (first used by the
    // count before digit pass 1); the 256 CTAs clear them with 16-byte stores
    if (g.c.derive_ok && g.c.passes >= 2) {
      const uint64_t stride = (uint64_t)gridDim.x * kRangeScanOneThreads;
      const uint64_t t = (uint64_t)blockIdx.x * kRangeScanOneThreads + threadIdx.x;
      uint4* kh = reinterpret_cast<uint4*>(g.c.keyhist);
      for (uint64_t i = t; i < 65536 / 4; i += stride) kh[i] = make_uint4(0, 0, 0, 0);
      uint4* ks = reinterpret_cast<uint4*>(g.c.keystart);  // n/32 words + 16 of slack
      const uint64_t q = ceil_div(ceil_div(g.c.n, 32), 4);
      for (uint64_t i = t; i < q; i += stride) ks[i] = make_uint4(0, 0, 0, 0);
    }
    if (plan_column(g.c, blockIdx.x == 0 && threadIdx.x == 0) < 0) return;
  } else if (g.c.ctrl->pass_src[pass] < 0) {
    return;
  }
  const uint32_t b = blockIdx.x, t = threadIdx.x;
  uint32_t tot = 0;  // bin t's total: the sum of its copies
  if (t < b)
#pragma unroll
    for (int k = 0; k < kBinTotCopies; ++k) tot += g.bintot[(k * kDigits + pass) * kRadix + t];
  uint32_t below;
  block_exclusive_scan<kRangeScanOneThreads>(tot, &below, s_warp);
  const uint32_t x = t < g.ranges ? range_hist[(uint64_t)t * kRadix + b] : 0u;
  uint32_t all;
  const uint32_t pre = block_exclusive_scan<kRangeScanOneThreads>(x, &all, s_warp);
  if (t < g.ranges) range_start[(uint64_t)t * kRadix + b] = below + pre;
}

// ---------------------------------------------------------------------------
// Range scatter: one persistent CTA per range, 256 threads x ITEMS rows per
// tile.
//
//  fetch    cp.async.bulk of the next tile's keys (and row ids) into the other
//           half of a double buffer, completion on an mbarrier
//  rank     warp-striped rows (item j of lane l in warp w is tile row
//           w*32*ITEMS + j*32 + l, so (j, l) order is row order); peer masks
//           (lanes holding the same digit) from eight ballots or
//           __match_any_sync; two independent per-warp counter chains (first
//           and second half of the warp's rows) give stable warp ranks
//  stage    rows in tile-sorted order in shared memory
//  write    consecutive threads to consecutive positions of each bin run, at
//           the range's running bin offsets, which then advance by the
//           tile's counts
// ---------------------------------------------------------------------------
constexpr int kSortWarps = kSortThreads / 32;
static_assert(kSortThreads == kRadix, "one thread per bin");

// The tile-sorted keys are staged in the input key buffer the tile came from
// (its keys are in registers by then); row ids need their own staging.
template <int ITEMS>
struct ScatterSmem {
  uint32_t in_keys[2][kSortThreads * ITEMS];
  uint32_t in_rids[2][kSortThreads * ITEMS];
  uint32_t out_rids[kSortThreads * ITEMS];
  // per-warp, per-half counters (16-bit: at most a tile's rows, < 2^16)
  uint16_t whist[kSortWarps][2][kRadix];
  uint32_t run_off[kRadix];               // range's next free position per bin
  uint32_t bin_base[kRadix];              // run_off - tile-local bin start
  uint32_t warp_tmp[kSortWarps + 1];
  uint64_t bar[2];
  int abort;
};

// Lanes of the warp holding the same 8-bit digit as this lane: eight ballots
// (ALU pipe) or __match_any_sync (MIO pipe).
template <bool BALLOT>
__device__ __forceinline__ uint32_t digit_peers(uint32_t d) {
  if (BALLOT) {
    uint32_t m = 0xffffffffu;
#pragma unroll
    for (int bit = 0; bit < kRadixBits; ++bit) {
      const bool set = (d >> bit) & 1u;
      const uint32_t bb = __ballot_sync(0xffffffffu, set);
      m &= set ? bb : ~bb;
    }
    return m;
  } else {
    return __match_any_sync(0xffffffffu, d);
  }
}

// PEERS: 0 all items by ballots, 1 all by match.any, 2 the first
// kHybridMatchItems by match.any and the rest by ballots (the two pipes work
// in parallel).
#ifndef WAH_HYBRID_MATCH_NUM
#define WAH_HYBRID_MATCH_NUM 3  // match.any share of the items: NUM / 8 (measured best)
#endif
__host__ __device__ constexpr int kHybridMatchItems(int items) {
  return items * WAH_HYBRID_MATCH_NUM / 8;
}

// Stable ranks of a tile's rows within their warp, by digit: dig[j] is item
// j's digit (item j of lane l in warp w is tile row w*32*ITEMS + j*32 + l);
// rank[j] receives its rank among the warp's rows of the same digit (not yet
// offset by the warp's start in the tile).  Peer masks first (independent),
// then two interleaved counter chains (whA: the first half of the items,
// whB: the second half; this warp's zeroed 16-bit counters); on return whA
// holds the warp's count per digit of the first half, whB of the second.
template <int ITEMS, int PEERS>
__device__ __forceinline__ void warp_rank(const uint32_t (&dig)[ITEMS], uint32_t (&rank)[ITEMS],
                                          uint16_t* whA, uint16_t* whB) {
  constexpr int HALF = ITEMS / 2;
  const uint32_t lt = lanemask_lt(), gt = lanemask_gt();
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    const bool ballot = PEERS == 0 || (PEERS == 2 && j >= kHybridMatchItems(ITEMS));
    rank[j] = ballot ? digit_peers<true>(dig[j]) : digit_peers<false>(dig[j]);
  }
#pragma unroll
  for (int j = 0; j < HALF; ++j) {
    const uint32_t pa = rank[j], pb = rank[j + HALF];
    const uint32_t da = dig[j], db = dig[j + HALF];
    const uint32_t ca = whA[da];
    const uint32_t cb = whB[db];
    __syncwarp();
    if ((pa & gt) == 0) whA[da] = (uint16_t)(ca + __popc(pa));
    if ((pb & gt) == 0) whB[db] = (uint16_t)(cb + __popc(pb));
    __syncwarp();
    rank[j] = ca + __popc(pa & lt);
    rank[j + HALF] = cb + __popc(pb & lt);
  }
#pragma unroll
  for (int j = HALF; j < ITEMS; ++j) rank[j] += whA[dig[j]];
}

// Thread b (one per bin), after every warp ranked its rows: the tile's count
// of bin b, its tile-local start (scan over the bins), each warp's start of
// bin b in the tile (into whist[w][0][b]), bin_base[b] = the range's next
// free position of bin b minus the tile-local start, and the running offset
// advanced by the count.  One barrier inside (the scan); the caller
// synchronises before anyone reads whist or bin_base.
__device__ __forceinline__ void tile_bin_starts(uint16_t (*whist)[2][kRadix], uint32_t* run_off,
                                                uint32_t* bin_base, uint32_t* warp_tmp) {
  const uint32_t b = threadIdx.x;
  uint32_t cnt[kSortWarps];
  uint32_t count = 0;
#pragma unroll
  for (int w = 0; w < kSortWarps; ++w) {
    cnt[w] = whist[w][0][b] + whist[w][1][b];
    count += cnt[w];
  }
  uint32_t tile_total;
  // (warp totals read here, written again after this tile's later barriers)
  const uint32_t lstart = block_exclusive_scan_1b<kSortThreads>(count, &tile_total, warp_tmp);
  uint32_t run = lstart;
#pragma unroll
  for (int w = 0; w < kSortWarps; ++w) {
    whist[w][0][b] = (uint16_t)run;
    run += cnt[w];
  }
  bin_base[b] = run_off[b] - lstart;
  run_off[b] += count;
}

// Each warp zeroes its own two counter chains.
__device__ __forceinline__ void zero_warp_counters(uint16_t* whA, uint32_t lane) {
  uint4* w4 = reinterpret_cast<uint4*>(whA);
#pragma unroll
  for (uint32_t k = lane; k < 2 * kRadix * 2 / 16; k += 32) w4[k] = make_uint4(0, 0, 0, 0);
  __syncwarp();
}

// Issue the bulk copies of one whole tile (thread 0 only); k16: the keys are
// 16-bit (tiles start on multiples of 8 rows, so the copy stays 16-byte aligned).
__device__ __forceinline__ void fetch_tile(uint32_t* dst_k, uint32_t* dst_r, uint64_t* bar,
                                           const uint32_t* kin, const uint32_t* rin,
                                           uint64_t base, uint32_t rows, bool k16) {
  const uint32_t kbytes = rows * (k16 ? 2u : 4u), rbytes = rows * 4u;
  fence_proxy_async_shared();
  mbar_arrive_expect_tx(bar, rin ? kbytes + rbytes : kbytes);
  if (k16)
    bulk_copy_g2s(dst_k, reinterpret_cast<const uint16_t*>(kin) + base, kbytes, bar);
  else
    bulk_copy_g2s(dst_k, kin + base, kbytes, bar);
  if (rin) bulk_copy_g2s(dst_r, rin + base, rbytes, bar);
}

// ---------------------------------------------------------------------------
// Key-start mode (one-column index builds whose keys all fit 16 bits and
// whose two low digits both vary): the two digit passes exchange one packed
// word per row instead of a 16-bit key stream beside a row-id stream.
//
//  pass 0  ranks rows by the low digit and writes, for each row, its offset
//          in its pass-0 range << 8 | its high digit (the low digit is
//          implied by the bin the row lands in, the range start by the run)
//  pass 1  ranks those words by the high digit and writes row ids; a row's
//          pass-0 run -- the last run of the bin-major table seg0 starting
//          at or before the row's position -- gives its range, so
//          row id = range * range_rows0 + offset.  Every warp follows the
//          runs itself: the run holding the tile's first row (i0) and the
//          next 32 run starts in registers; a warp slice of a tile (32 x
//          ITEMS consecutive rows) mostly holds no run start, and all its
//          rows then share one base.  A slice with 32 or more run starts
//          after i0 searches seg0 in global memory row by row.
//
// Both kernels keep three tile buffers and issue the bulk copy of tile i + 2
// after the first barrier of tile i (every thread has finished tile i - 1 by
// then, whose buffer the copy reuses), so there is no barrier at the end of
// a tile and warps that finish writing start ranking the next tile.
// ---------------------------------------------------------------------------
constexpr int kPackBufs = 3;  // input tiles in flight: the copy of tile i + 2 runs during tile i

template <int ITEMS>
struct PackSmem {
  uint32_t in[kPackBufs][kSortThreads * ITEMS];  // input tiles; the current one then holds
                                                  // the staged rows
  uint8_t bins[kSortThreads * ITEMS];             // pass 1: digit of each staged row
  uint16_t whist[kSortWarps][2][kRadix];
  uint32_t run_off[kRadix];
  uint32_t bin_base[kRadix];
  uint32_t warp_tmp[kSortWarps + 1];
  uint64_t bar[kPackBufs];
  int abort;
};
static_assert(sizeof(PackSmem<8>) <= sizeof(ScatterSmem<8>), "packed passes fit the allocation");
static_assert(sizeof(PackSmem<12>) <= sizeof(ScatterSmem<12>), "packed passes fit the allocation");
static_assert(sizeof(PackSmem<16>) <= sizeof(ScatterSmem<16>), "packed passes fit the allocation");

// Number of entries of the sorted seg[0, count) that are <= p (warp-wide
// 32-ary search; every lane returns it).
__device__ __forceinline__ uint32_t warp_count_le(const uint32_t* __restrict__ seg,
                                                 uint32_t count, uint32_t p) {
  const uint32_t lane = threadIdx.x & 31;
  uint32_t a = 0, b = count;  // the answer lies in [a, b]
  while (a < b) {
    const uint32_t step = (b - a + 31) / 32;
    const uint32_t idx = a + lane * step;
    const bool le = idx < b && seg[idx] <= p;
    const uint32_t k = __popc(__ballot_sync(0xffffffffu, le));
    if (k == 0) {
      b = a;
    } else {
      const uint32_t last = a + (k - 1) * step;
      const uint32_t nb = a + k * step;
      a = last + 1;
      b = nb < b ? nb : b;
    }
  }
  return a;
}

// Last index of the sorted seg[0, count) whose value is <= p (seg[0] <= p).
__device__ __forceinline__ uint32_t last_le(const uint32_t* __restrict__ seg, uint32_t count,
                                            uint32_t p) {
  uint32_t a = 0, b = count;  // seg[a] <= p; answer in [a, b)
  while (b - a > 1) {
    const uint32_t m = a + (b - a) / 2;
    if (seg[m] <= p) a = m;
    else b = m;
  }
  return a;
}

template <int ITEMS, int PEERS>
__device__ __forceinline__ void scatter_pack0(const OneColumn& g,
                                              const uint32_t* __restrict__ range_start,
                                              unsigned char* smem_raw) {
  constexpr uint32_t TILE = kSortThreads * ITEMS;
  PackSmem<ITEMS>& sm = *reinterpret_cast<PackSmem<ITEMS>*>(smem_raw);
  const ColumnView& col = g.c;
  const RangeView rv = g.range(blockIdx.x);
  const uint32_t* __restrict__ kin = sel_keys(col, col.ctrl->pass_src[0]);
  uint32_t* __restrict__ out = const_cast<uint32_t*>(sel_keys(col, col.ctrl->pass_dst[0]));
  uint32_t* status = col.status;
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t lo = rv.lo, hi = rv.hi;
  {
    // this range's run start of every bin, also into the bin-major table of
    // pass-0 runs that the packed later pass reads
    const uint32_t st = range_start[(uint64_t)blockIdx.x * kRadix + tid];
    sm.run_off[tid] = st;
    g.seg0[(uint64_t)tid * g.ranges + blockIdx.x] = st;
  }
  if (lo >= hi) return;
  const uint32_t ntiles = (uint32_t)ceil_div(hi - lo, TILE);

  if (tid == 0) {
    for (int b = 0; b < kPackBufs; ++b) mbar_init(&sm.bar[b], 1);
    sm.abort = 0;
    fence_mbar_init();
    for (uint32_t t = 0; t < 2; ++t)  // the first two tiles (whole tiles only)
      if (hi - lo >= (uint64_t)(t + 1) * TILE)
        fetch_tile(sm.in[t], nullptr, &sm.bar[t], kin, nullptr, lo + (uint64_t)t * TILE, TILE,
                   false);
  }
  __syncthreads();

  const uint32_t row0 = warp * 32 * ITEMS + lane;
  uint16_t* whA = sm.whist[warp][0];
  uint16_t* whB = sm.whist[warp][1];
  uint32_t phase_bits = 0;
  const uint32_t n32 = (uint32_t)col.n;

  for (uint32_t i = 0, cur = 0; i < ntiles; ++i, cur = cur + 1 == kPackBufs ? 0 : cur + 1) {
    const uint64_t base = lo + (uint64_t)i * TILE;
    const uint32_t valid = hi - base < TILE ? (uint32_t)(hi - base) : TILE;
    zero_warp_counters(whA, lane);
    uint32_t key[ITEMS];
    if (valid == TILE) {
      if (!mbar_wait_bounded(&sm.bar[cur], (phase_bits >> cur) & 1u)) {
        set_status(status, WAH_ETIMEOUT);
        sm.abort = 1;
      }
      phase_bits ^= 1u << cur;
      const uint32_t* kp = sm.in[cur] + row0;
#pragma unroll
      for (int j = 0; j < ITEMS; ++j) key[j] = kp[j * 32];
    } else {
      // ragged last tile: rows past n take digit 255 and rank after every
      // real row of the tile (never written out)
#pragma unroll
      for (int j = 0; j < ITEMS; ++j) {
        const uint32_t r = row0 + j * 32;
        key[j] = r < valid ? kin[base + r] : 0xffffffffu;
      }
    }
    uint32_t dig[ITEMS], rank[ITEMS];
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) dig[j] = key[j] & 0xFFu;
    warp_rank<ITEMS, PEERS>(dig, rank, whA, whB);
    __syncthreads();
    // every thread is past tile i - 1: its buffer takes tile i + 2
    if (tid == 0 && i + 2 < ntiles && hi - (base + 2 * TILE) >= TILE) {
      const uint32_t nb = cur == 0 ? kPackBufs - 1 : cur - 1;
      fetch_tile(sm.in[nb], nullptr, &sm.bar[nb], kin, nullptr, base + 2 * TILE, TILE, false);
    }
    tile_bin_starts(sm.whist, sm.run_off, sm.bin_base, sm.warp_tmp);
    __syncthreads();
    // staged word: tile row << 16 | 16-bit key
    uint32_t* staged = sm.in[cur];
#pragma unroll
    for (int j = 0; j < ITEMS; ++j)
      staged[whA[dig[j]] + rank[j]] = ((row0 + j * 32) << 16) | (key[j] & 0xFFFFu);
    __syncthreads();
    if (!sm.abort) {
      const uint32_t toff = (uint32_t)(base - lo);  // tile's first row in the range
#pragma unroll 4
      for (int it = 0; it < ITEMS; ++it) {
        const uint32_t k = it * kSortThreads + tid;
        if (k < valid) {
          const uint32_t w = staged[k];
          const uint32_t gpos = sm.bin_base[w & 0xFFu] + k;
          if (gpos < n32) out[gpos] = ((toff + (w >> 16)) << 8) | ((w >> 8) & 0xFFu);
          else set_status(status, WAH_ECORRUPT);
        }
      }
    }
  }
}

template <int ITEMS, int PEERS>
__device__ __forceinline__ void scatter_pack1(const OneColumn& g,
                                              const uint32_t* __restrict__ range_start,
                                              unsigned char* smem_raw) {
  constexpr uint32_t TILE = kSortThreads * ITEMS;
  constexpr uint32_t SLICE = 32 * ITEMS;
  PackSmem<ITEMS>& sm = *reinterpret_cast<PackSmem<ITEMS>*>(smem_raw);
  const ColumnView& col = g.c;
  const RangeView rv = g.range(blockIdx.x);
  const uint32_t* __restrict__ win_in = sel_keys(col, col.ctrl->pass_src[1]);
  uint32_t* __restrict__ rout = const_cast<uint32_t*>(sel_rids(col, col.ctrl->pass_dst[1]));
  const uint32_t* __restrict__ seg0 = g.seg0;
  const uint32_t nseg = g.ranges0 * kRadix;
  const uint32_t r0 = g.ranges0;
  const uint32_t rows0 = (uint32_t)g.range_rows0;
  uint32_t* status = col.status;
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t lo = rv.lo, hi = rv.hi;
  if (lo >= hi) return;
  const uint32_t ntiles = (uint32_t)ceil_div(hi - lo, TILE);

  sm.run_off[tid] = range_start[(uint64_t)blockIdx.x * kRadix + tid];
  if (tid == 0) {
    for (int b = 0; b < kPackBufs; ++b) mbar_init(&sm.bar[b], 1);
    sm.abort = 0;
    fence_mbar_init();
    for (uint32_t t = 0; t < 2; ++t)  // the first two tiles (whole tiles only)
      if (hi - lo >= (uint64_t)(t + 1) * TILE)
        fetch_tile(sm.in[t], nullptr, &sm.bar[t], win_in, nullptr, lo + (uint64_t)t * TILE, TILE,
                   false);
  }
  // every warp: the run holding the range's first row (seg0[0] = 0 <= lo)
  uint32_t i0 = warp_count_le(seg0, nseg, (uint32_t)lo) - 1;
  uint32_t ent = i0 + 1 + lane < nseg ? seg0[i0 + 1 + lane] : 0xffffffffu;  // run starts i0+1..
  uint32_t rmod = (i0 + lane) % r0;  // range of run i0 + lane, followed as i0 advances
  __syncthreads();

  const uint32_t row0 = warp * SLICE + lane;
  uint16_t* whA = sm.whist[warp][0];
  uint16_t* whB = sm.whist[warp][1];
  uint32_t phase_bits = 0;
  const uint32_t n32 = (uint32_t)col.n;

  for (uint32_t i = 0, cur = 0; i < ntiles; ++i, cur = cur + 1 == kPackBufs ? 0 : cur + 1) {
    const uint64_t base = lo + (uint64_t)i * TILE;
    const uint32_t valid = hi - base < TILE ? (uint32_t)(hi - base) : TILE;
    zero_warp_counters(whA, lane);
    uint32_t word[ITEMS], rid[ITEMS];
    if (valid == TILE) {
      if (!mbar_wait_bounded(&sm.bar[cur], (phase_bits >> cur) & 1u)) {
        set_status(status, WAH_ETIMEOUT);
        sm.abort = 1;
      }
      phase_bits ^= 1u << cur;
      const uint32_t* wp = sm.in[cur] + row0;
#pragma unroll
      for (int j = 0; j < ITEMS; ++j) word[j] = wp[j * 32];
    } else {
#pragma unroll
      for (int j = 0; j < ITEMS; ++j) {
        const uint32_t r = row0 + j * 32;
        word[j] = r < valid ? win_in[base + r] : 0xFFu;  // rows past n: digit 255
      }
    }
    // Row ids.  Slot t (1..32) = run i0 + t, its start in lane t-1's ent;
    // the slice's rows [s0, s1) lie in runs i0 + k0 .. i0 + k1.
    {
      const uint32_t s0 = (uint32_t)base + warp * SLICE, s1 = s0 + SLICE;
      const uint32_t k0 = __popc(__ballot_sync(0xffffffffu, ent <= s0));
      const uint32_t k1 = __popc(__ballot_sync(0xffffffffu, ent < s1));
      if (k1 < 32) {
        const uint32_t mybase = rmod * rows0;  // first row id of run i0 + lane
        const uint32_t b0 = __shfl_sync(0xffffffffu, mybase, k0);
        if (k1 == k0) {
#pragma unroll
          for (int j = 0; j < ITEMS; ++j) rid[j] = b0 + (word[j] >> 8);
        } else if (k1 == k0 + 1) {  // one run starts inside the slice
          const uint32_t bnd = __shfl_sync(0xffffffffu, ent, k0);
          const uint32_t b1 = __shfl_sync(0xffffffffu, mybase, k0 + 1);
#pragma unroll
          for (int j = 0; j < ITEMS; ++j)
            rid[j] = (s0 + lane + j * 32 >= bnd ? b1 : b0) + (word[j] >> 8);
        } else {
#pragma unroll
          for (int j = 0; j < ITEMS; ++j) {
            const uint32_t p = s0 + lane + j * 32;
            uint32_t k = k0;
            for (uint32_t t = k0; t < k1; ++t) k += __shfl_sync(0xffffffffu, ent, t) <= p;
            rid[j] = __shfl_sync(0xffffffffu, mybase, k) + (word[j] >> 8);
          }
        }
      } else {
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
          const uint32_t p = s0 + lane + j * 32;
          const uint32_t sidx = last_le(seg0, nseg, p < n32 ? p : n32 - 1);
          rid[j] = (sidx % r0) * rows0 + (word[j] >> 8);
        }
      }
      // the runs of the next tile
      if (i + 1 < ntiles) {
        const uint32_t p_next = (uint32_t)(base + TILE);
        const uint32_t adv = __popc(__ballot_sync(0xffffffffu, ent <= p_next));
        if (adv < 32) {
          i0 += adv;
          rmod += adv;
          while (rmod >= r0) rmod -= r0;
        } else {
          i0 = warp_count_le(seg0, nseg, p_next) - 1;
          rmod = (i0 + lane) % r0;
        }
        ent = i0 + 1 + lane < nseg ? seg0[i0 + 1 + lane] : 0xffffffffu;
      }
    }
    uint32_t dig[ITEMS], rank[ITEMS];
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) dig[j] = word[j] & 0xFFu;
    warp_rank<ITEMS, PEERS>(dig, rank, whA, whB);
    __syncthreads();
    // every thread is past tile i - 1: its buffer takes tile i + 2
    if (tid == 0 && i + 2 < ntiles && hi - (base + 2 * TILE) >= TILE) {
      const uint32_t nb = cur == 0 ? kPackBufs - 1 : cur - 1;
      fetch_tile(sm.in[nb], nullptr, &sm.bar[nb], win_in, nullptr, base + 2 * TILE, TILE, false);
    }
    tile_bin_starts(sm.whist, sm.run_off, sm.bin_base, sm.warp_tmp);
    __syncthreads();
    uint32_t* staged = sm.in[cur];
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
      const uint32_t r = whA[dig[j]] + rank[j];
      staged[r] = rid[j];
      sm.bins[r] = (uint8_t)dig[j];
    }
    __syncthreads();
    if (!sm.abort) {
#pragma unroll 4
      for (int it = 0; it < ITEMS; ++it) {
        const uint32_t k = it * kSortThreads + tid;
        if (k < valid) {
          const uint32_t gpos = sm.bin_base[sm.bins[k]] + k;
          if (gpos < n32) rout[gpos] = staged[k];
          else set_status(status, WAH_ECORRUPT);
        }
      }
    }
  }
}

template <int ITEMS, int PEERS, class G>
__global__ void __launch_bounds__(kSortThreads, ITEMS <= 12 ? 3 : 2)
    k_radix_scatter(G g, int pass, const uint32_t* __restrict__ range_start) {
  griddep_wait();
  constexpr uint32_t TILE = kSortThreads * ITEMS;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  ScatterSmem<ITEMS>& sm = *reinterpret_cast<ScatterSmem<ITEMS>*>(smem_raw);

  const RangeView rv = g.range(blockIdx.x);
  const ColumnView col = g.col(rv.col);
  const int src = col.ctrl->pass_src[pass];
  if (src < 0) return;  // trivial digit: every row in one bin, order unchanged
  if constexpr (std::is_same<G, OneColumn>::value) {
    if (g.packed && col.ctrl->derive) {  // key-start mode: passes 0 and 1 exchange packed words
      if (pass == 0) scatter_pack0<ITEMS, PEERS>(g, range_start, smem_raw);
      else scatter_pack1<ITEMS, PEERS>(g, range_start, smem_raw);
      return;
    }
  }
  const int dst = col.ctrl->pass_dst[pass];
  const uint32_t* kin = sel_keys(col, src);
  const uint32_t* rin = sel_rids(col, src);
  uint32_t* __restrict__ kout = const_cast<uint32_t*>(sel_keys(col, dst));
  uint32_t* __restrict__ rout = const_cast<uint32_t*>(sel_rids(col, dst));
  uint32_t* status = col.status;
  // 16-bit keys in the sort buffers (every key below 2^16)
  const bool k16_in = narrow_keys(col, src), k16_out = narrow_keys(col, dst);
  // derive mode: the last pass writes row ids only
  const bool keys_out = !(col.ctrl->derive && dst == col.ctrl->final_sel);
  const uint16_t* kin16 = reinterpret_cast<const uint16_t*>(kin);
  uint16_t* kout16 = reinterpret_cast<uint16_t*>(kout);

  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t lo = rv.lo, hi = rv.hi;
  if (lo >= hi) return;
  const uint32_t ntiles = (uint32_t)ceil_div(hi - lo, TILE);

  sm.run_off[tid] = range_start[(uint64_t)blockIdx.x * kRadix + tid];
  if (tid == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    sm.abort = 0;
    fence_mbar_init();
    if (hi - lo >= TILE)
      fetch_tile(sm.in_keys[0], sm.in_rids[0], &sm.bar[0], kin, rin, lo, TILE, k16_in);
  }
  __syncthreads();

  const uint32_t row0 = warp * 32 * ITEMS + lane;  // tile row of item 0
  uint16_t* whA = sm.whist[warp][0];
  uint16_t* whB = sm.whist[warp][1];
  static_assert(kSortThreads * ITEMS < 65536, "tile rows fit the 16-bit counters");
  uint32_t phase_bits = 0;  // parity of the next phase of bar[0], bar[1]

  for (uint32_t i = 0; i < ntiles; ++i) {
    const uint32_t cur = i & 1;
    const uint64_t base = lo + (uint64_t)i * TILE;
    const uint32_t valid = hi - base < TILE ? (uint32_t)(hi - base) : TILE;
    // Prefetch tile i + 1 into the other buffer (read during tile i - 1,
    // whose reads ended at the barrier that closed that iteration).  Only the
    // column's last tile can be ragged; it is read with plain loads instead.
    if (tid == 0 && i + 1 < ntiles && hi - (base + TILE) >= TILE)
      fetch_tile(sm.in_keys[cur ^ 1], sm.in_rids[cur ^ 1], &sm.bar[cur ^ 1], kin, rin,
                 base + TILE, TILE, k16_in);
    // Each warp zeroes its own counters (every read of them in the previous
    // tile came before the barrier that closed it).
    zero_warp_counters(whA, lane);
    uint32_t key[ITEMS];
    if (valid == TILE) {
      // phases of each buffer's barrier complete in turn; the parity of the
      // next one is tracked per buffer (a tile read with plain loads uses
      // none).  Every thread waits for the copy itself.
      if (!mbar_wait_bounded(&sm.bar[cur], (phase_bits >> cur) & 1u)) {
        set_status(status, WAH_ETIMEOUT);
        sm.abort = 1;
      }
      phase_bits ^= 1u << cur;
    }
    if (valid == TILE) {
      if (k16_in) {
        const uint16_t* kp = reinterpret_cast<const uint16_t*>(sm.in_keys[cur]) + row0;
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) key[j] = kp[j * 32];
      } else {
        const uint32_t* kp = sm.in_keys[cur] + row0;
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) key[j] = kp[j * 32];
      }
    } else {
      // The column's ragged last tile: plain loads; rows past n get key
      // 0xFFFFFFFF (digit 255 in every pass: stable ranking puts them after
      // every real row of the last bin, at tile positions >= valid, which are
      // never written out).
#pragma unroll
      for (int j = 0; j < ITEMS; ++j) {
        const uint32_t r = row0 + j * 32;
        key[j] = r < valid ? (k16_in ? kin16[base + r] : kin[base + r]) : 0xffffffffu;
        if (rin) sm.in_rids[cur][r] = r < valid ? rin[base + r] : 0u;
      }
    }

    uint32_t dig[ITEMS], rank[ITEMS];
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) dig[j] = digit8(key[j], pass);
    warp_rank<ITEMS, PEERS>(dig, rank, whA, whB);
    __syncthreads();
    tile_bin_starts(sm.whist, sm.run_off, sm.bin_base, sm.warp_tmp);
    __syncthreads();

    // Stage in tile-sorted order.
    uint32_t* out_keys = sm.in_keys[cur];
    const uint32_t* rsrc = sm.in_rids[cur] + row0;
    const uint32_t rid0 = (uint32_t)base + row0;
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
      const uint32_t r = whA[dig[j]] + rank[j];
      out_keys[r] = key[j];
      sm.out_rids[r] = rin ? rsrc[j * 32] : rid0 + j * 32;
    }
    __syncthreads();

    if (!sm.abort) {
      const uint32_t n32 = (uint32_t)col.n;
#pragma unroll 4
      for (int it = 0; it < ITEMS; ++it) {
        const uint32_t k = it * kSortThreads + tid;
        if (k < valid) {
          const uint32_t kk = out_keys[k];
          const uint32_t g = sm.bin_base[digit8(kk, pass)] + k;
          if (g < n32) {
            if (keys_out) {
              if (k16_out) kout16[g] = (uint16_t)kk;
              else kout[g] = kk;
            }
            rout[g] = sm.out_rids[k];
          } else {
            set_status(status, WAH_ECORRUPT);
          }
        }
      }
    }
    __syncthreads();  // staging and input buffer reusable
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
// Compiled tile shapes of the scatter pass; sort_items selects one, the
// autotuner measures them.
template <class G>
struct SortVariant {
  int items;
  void (*fn)(G, int, const uint32_t*);
  size_t smem;
};

template <int PEERS, class G>
SortVariant<G> sort_variant_peers(int items) {
  switch (items) {
    case 8: return {8, k_radix_scatter<8, PEERS, G>, sizeof(ScatterSmem<8>)};
    case 12: return {12, k_radix_scatter<12, PEERS, G>, sizeof(ScatterSmem<12>)};
    default: return {16, k_radix_scatter<16, PEERS, G>, sizeof(ScatterSmem<16>)};
  }
}

template <class G>
SortVariant<G> sort_variant(int items, int peers) {
  if (peers == 1) return sort_variant_peers<1, G>(items);
  if (peers == 2) return sort_variant_peers<2, G>(items);
  return sort_variant_peers<0, G>(items);
}

template <class G>
cudaError_t scatter_variant(int items, int peers, SortVariant<G>* v, int* per_sm) {
  *v = sort_variant<G>(items, peers);
  cudaError_t err =
      cudaFuncSetAttribute(v->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)v->smem);
  if (err != cudaSuccess) return err;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, v->fn, kSortThreads, v->smem);
}

// The launch sequence over any geometry: histogram, plan, then per digit
// pass (count,) scan and scatter.  Digit pass 0 (and the histogram that
// counts for it) runs over geometry g0 with scatter variant v0, the later
// passes over g1 with v1: each pass counts and scatters over its own ranges.
template <class G>
cudaError_t launch_sort_t(const G& g0, uint32_t ranges0, const SortVariant<G>& v0, const G& g1,
                          uint32_t ranges1, const SortVariant<G>& v1, uint32_t ncols,
                          const RangeArrays& ra, const LaunchOpts& o, cudaStream_t s,
                          uint32_t* launches) {
  constexpr bool kPdl = std::is_same<G, OneColumn>::value;  // programmatic launches
  uint32_t parts0 = kCountCtasPerRange, parts1 = kCountCtasPerRange;
  if constexpr (std::is_same<G, OneColumn>::value) {
    if (g0.count_parts) parts0 = g0.count_parts;
    if (g1.count_parts) parts1 = g1.count_parts;
  }
  const unsigned count_grid = ranges0 * parts0;
  // the per-range histograms (for one column with the control block before
  // them and the bin totals and range counts after them)
  cudaError_t err = cudaMemsetAsync(ra.zero, 0, ra.zero_bytes, s);
  if (err != cudaSuccess) return err;
  record_phase(o.events, kPhaseHist, false, s);
  err = launch_kernel(kPdl,k_digit_histogram<G>, count_grid, kHistThreads, 0, s, g0, ra.hist);
  if (err != cudaSuccess) return err;
  record_phase(o.events, kPhaseHist, true, s);
  ++*launches;
  record_phase(o.events, kPhasePlan, false, s);
  if constexpr (!std::is_same<G, OneColumn>::value) {  // one column: in the pass-0 range scan
    err = launch_kernel(kPdl,k_sort_plan<G>, ncols, kRadix, 0, s, g0);
    if (err != cudaSuccess) return err;
    ++*launches;
  }
  record_phase(o.events, kPhasePlan, true, s);
  for (int p = 0; p < kDigits; ++p) {
    if (p >= o.max_passes) {  // not launched: empty spans keep every event valid
      record_phase(o.events, kPhasePass0 + p, false, s);
      record_phase(o.events, kPhasePass0 + p, true, s);
      record_phase(o.events, kPhaseScatter0 + p, false, s);
      record_phase(o.events, kPhaseScatter0 + p, true, s);
      continue;
    }
    uint32_t* rh = ra.hist + (size_t)p * ra.max_ranges * kRadix;
    const G& gp = p == 0 ? g0 : g1;
    const uint32_t ranges = p == 0 ? ranges0 : ranges1;
    const SortVariant<G>& v = p == 0 ? v0 : v1;
    record_phase(o.events, kPhasePass0 + p, false, s);
    if (p > 0) {
      err = launch_kernel(kPdl,k_range_count<G>, ranges * (p == 0 ? parts0 : parts1), kHistThreads, 0, s,
                       gp, p, rh);
      if (err != cudaSuccess) return err;
      ++*launches;
    }
    if constexpr (std::is_same<G, OneColumn>::value)  // + the key starts for digit pass 1
      err = launch_kernel(kPdl,k_range_scan_one, kRadix + (p == 1 && gp.c.derive_ok ? kKeyStartCtas : 0),
                       kRangeScanOneThreads, 0, s, gp, p, (const uint32_t*)rh, ra.start);
    else
      err = launch_kernel(kPdl,k_range_scan<G>, ncols, kRangeScanThreads, 0, s, gp, p,
                       (const uint32_t*)rh, ra.start);
    if (err != cudaSuccess) return err;
    ++*launches;
    record_phase(o.events, kPhaseScatter0 + p, false, s);
    err = launch_kernel(kPdl,v.fn, ranges, kSortThreads, v.smem, s, gp, p, (const uint32_t*)ra.start);
    if (err != cudaSuccess) return err;
    ++*launches;
    record_phase(o.events, kPhaseScatter0 + p, true, s);
    record_phase(o.events, kPhasePass0 + p, true, s);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

// Equal ranges of whole tiles of one scatter variant (multiples of its tile
// and of kRangeQuantum), one per resident scatter CTA.
static OneColumn one_column_ranges(const ColumnView& c, const SortVariant<OneColumn>& v,
                                   int per_sm, const RangeArrays& ra, const LaunchOpts& o) {
  uint64_t want = (uint64_t)std::max(o.sm_count, 1) * std::max(per_sm, 1);
  if (want > ra.max_ranges) want = ra.max_ranges;
  // ranges of whole tiles (a column's last range may end inside a tile)
  const uint64_t quantum = (uint64_t)kSortThreads * v.items;
  OneColumn g{};
  g.c = c;
  g.range_rows = std::max<uint64_t>(ceil_div(ceil_div(c.n, want), quantum) * quantum, quantum);
  g.ranges = (uint32_t)std::max<uint64_t>(ceil_div(c.n, g.range_rows), 1);
  g.count_parts = g.range_rows < 32768 ? 1 : kCountCtasPerRange;  // short ranges: one CTA
  return g;
}

cudaError_t launch_sort_one(const ColumnView& c, const RangeArrays& ra, const LaunchOpts& o,
                            cudaStream_t s, uint32_t* launches) {
  SortVariant<OneColumn> v0, v1;
  int per_sm0 = 0, per_sm1 = 0;
  // The later passes' own shape is for index builds, whose last pass writes
  // row ids only (key-start mode); a sort returns its keys and keeps one shape.
  cudaError_t err = scatter_variant<OneColumn>(o.sort_items, o.sort_peers, &v0, &per_sm0);
  if (err == cudaSuccess)
    err = c.derive_ok
              ? scatter_variant<OneColumn>(o.later_items, o.later_peers, &v1, &per_sm1)
              : scatter_variant<OneColumn>(o.sort_items, o.sort_peers, &v1, &per_sm1);
  if (err != cudaSuccess) return err;
  OneColumn g0 = one_column_ranges(c, v0, per_sm0, ra, o);
  OneColumn g1 = one_column_ranges(c, v1, per_sm1, ra, o);
  // Key-start mode packs a row's offset in its pass-0 range into 24 bits and
  // needs the table of pass-0 runs; it pays where those runs are long (each
  // pass-1 warp slice then mostly lies inside one run), else the 16-bit keys
  // go between the passes.
  g0.packed = g1.packed = ra.seg0 && g0.range_rows < kPackRangeRows &&
                          (o.pack_force || g0.range_rows >= kPackMinRangeRows);
  g0.bintot = g1.bintot = ra.bintot;
  g0.ranges0 = g1.ranges0 = g0.ranges;
  g0.range_rows0 = g1.range_rows0 = g0.range_rows;
  g0.seg0 = g1.seg0 = ra.seg0;
  return launch_sort_t<OneColumn>(g0, g0.ranges, v0, g1, g1.ranges, v1, 1, ra, o, s, launches);
}

cudaError_t launch_sort_many(const ManyColumns& g, uint32_t ncols, uint32_t ranges,
                             const RangeArrays& ra, const LaunchOpts& o, cudaStream_t s,
                             uint32_t* launches) {
  SortVariant<ManyColumns> v;  // one shape for every pass (the plan's ranges)
  int per_sm = 0;
  cudaError_t err = scatter_variant<ManyColumns>(o.sort_items, o.sort_peers, &v, &per_sm);
  if (err != cudaSuccess) return err;
  return launch_sort_t<ManyColumns>(g, ranges, v, g, ranges, v, ncols, ra, o, s, launches);
}

// Copies the sorted stream from its device-chosen home into caller buffers
// (rid = row index when no pass ran: all values equal, or n == 1).
__global__ void k_sort_deliver(ColumnView c, uint32_t* __restrict__ out_keys,
                               uint32_t* __restrict__ out_rids) {
  const int sel = c.ctrl->final_sel;
  const uint32_t* __restrict__ k = sel_keys(c, sel);
  const uint16_t* __restrict__ k16 = reinterpret_cast<const uint16_t*>(k);
  const bool narrow = narrow_keys(c, sel);
  const uint32_t* __restrict__ r = sel_rids(c, sel);
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < c.n; i += stride) {
    out_keys[i] = narrow ? k16[i] : k[i];
    out_rids[i] = r ? r[i] : (uint32_t)i;
  }
}

cudaError_t launch_sort_deliver(const ColumnView& c, uint32_t* out_keys, uint32_t* out_rids,
                                cudaStream_t s, uint32_t* launches) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint64_t want = ceil_div(c.n, 256), cap = (uint64_t)(sms > 0 ? sms : 1) * 8;
  const int grid = (int)(want < cap ? want : cap);
  k_sort_deliver<<<grid, 256, 0, s>>>(c, out_keys, out_rids);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace wah
