// wah_query.cu -- decoding and querying a built index on the GPU.
//
// The reference only decodes on the host, one key at a time, into a '0'/'1'
// string (decoded_bitmap, src/cpu.cpp:47-74; src/gpu.cpp:65-94): a literal
// (bit 31 set) gives 31 rows, a fill (bit 31 clear) skips (word & ~(3<<30))
// all-zero chunks.  Here the same reading of the words runs as a
// device-wide walk over a contiguous run of keys' words:
//
//   chunk(word)  = sum over the key's earlier words of (literal ? 1 : fill)
//   rows(word)   = chunk * 31 + b for every set bit b < 31 of a literal
//   position     = number of rows in all earlier words (keys ascending,
//                  rows ascending within a key)
//
// i.e. a segmented exclusive scan (segments = keys, starting at offsets[k])
// of the chunk advances and a plain exclusive scan of the literals'
// popcounts.  Like the builds, the walk is look-back free: the words are cut
// into equal ranges, one persistent CTA per range; k_walk_count reduces each
// range (rows, chunk advance after its last key head), k_walk_scan scans the
// range aggregates, and k_walk_emit re-reads the range tile by tile with the
// carries and hands every literal to an action:
//
//   decode  writes row ids (the stable sort's rid order), optionally each
//           row's value and the reconstructed column, and each key's first
//           row position;
//   expand  ORs the literals of a key range into a dense chunk array.
//
// A query combines one or two dense chunk arrays (OR / AND / AND NOT) and
// compacts the result in one more range pass into row ids and into a WAH
// bitmap in the reference's format (literal per non-empty chunk, a fill word
// for each gap, no trailing fill) -- for a single key that is exactly the
// key's own words.
#include "wah_walk.cuh"

namespace wah {
namespace {

// Per-range aggregate of a dense compaction.
struct DenseAgg {
  uint32_t rows;      // set bits of the combined chunks
  uint32_t words;     // output words, not counting the first non-empty chunk's fill
  uint32_t first_nz;  // first / last non-empty chunk, kNone if none
  uint32_t last_nz;
  uint32_t rows_base;  // written by the scan
  uint32_t words_base;
  uint32_t prev_nz;    // last non-empty chunk before the range, kNone if none
  uint32_t pad;
};

// Decode action: row ids in key order, optional per-row values, the
// reconstructed column and each key's first row position.
struct DecodeAct {
  const uint32_t* keys;
  uint32_t* rows;        // [n] or nullptr
  uint32_t* row_values;  // [n] or nullptr
  uint32_t* column;      // [n] or nullptr
  uint32_t* key_rows;    // [K] or nullptr
  uint64_t n;
  uint32_t* status;
  static constexpr bool kNeedsValue = true;
  __device__ __forceinline__ void head(uint32_t key, uint32_t pos) const {
    if (key_rows) key_rows[key] = pos;
  }
  __device__ __forceinline__ void literal(uint32_t value, uint32_t chunk, uint32_t bits,
                                          uint32_t pos) const {
    while (bits) {
      const uint32_t b = __ffs(bits) - 1;
      bits &= bits - 1;
      const uint64_t row = (uint64_t)chunk * 31u + b;
      if (row >= n || pos >= n) {
        set_status(status, WAH_ECORRUPT);
        return;
      }
      if (rows) rows[pos] = (uint32_t)row;
      if (row_values) row_values[pos] = value;
      if (column) column[row] = value;
      ++pos;
    }
  }
};

// Decode to row ids only (with optional per-key first positions): no key
// values are read, and the bounds are checked once per literal word.
struct DecodeRowsAct {
  uint32_t* rows;
  uint32_t* key_rows;  // [K] or nullptr
  uint64_t n;
  uint32_t* status;
  static constexpr bool kNeedsValue = false;
  __device__ __forceinline__ void head(uint32_t key, uint32_t pos) const {
    if (key_rows) key_rows[key] = pos;
  }
  __device__ __forceinline__ void literal(uint32_t, uint32_t chunk, uint32_t bits,
                                          uint32_t pos) const {
    const uint64_t base = (uint64_t)chunk * 31u;
    const uint32_t top = 31u - __clz(bits);  // highest row of the chunk (bits != 0)
    if (bits == 0 || base + top >= n || (uint64_t)pos + __popc(bits) > n) {
      if (bits) set_status(status, WAH_ECORRUPT);
      return;
    }
    uint32_t* out = rows + pos;
    while (bits) {
      const uint32_t b = __ffs(bits) - 1;
      bits &= bits - 1;
      *out++ = (uint32_t)(base + b);
    }
  }
};

// Expand action: OR every literal into a dense chunk array.
struct ExpandAct {
  uint32_t* dense;
  uint64_t nchunks;
  uint32_t* status;
  static constexpr bool kNeedsValue = false;
  __device__ __forceinline__ void head(uint32_t, uint32_t) const {}
  __device__ __forceinline__ void literal(uint32_t, uint32_t chunk, uint32_t bits, uint32_t) const {
    if (chunk >= nchunks) {
      set_status(status, WAH_ECORRUPT);
      return;
    }
    atomicOr(dense + chunk, bits);
  }
};

// ---------------------------------------------------------------------------
// Dense chunk arrays -> row ids and a WAH bitmap.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t combine_op(const uint32_t* a, const uint32_t* b, int op,
                                               uint32_t c) {
  const uint32_t x = a[c];
  if (op == WAH_QUERY_KEYS) return x;
  const uint32_t y = b[c];
  if (op == WAH_QUERY_OR) return x | y;
  if (op == WAH_QUERY_AND) return x & y;
  return x & ~y;  // WAH_QUERY_ANDNOT
}

struct DenseIn {
  const uint32_t* a;
  const uint32_t* b;
  int op;
  uint32_t nchunks;
  uint32_t range_chunks;  // multiple of kQTile
};

__global__ void __launch_bounds__(kQThreads) k_dense_count(DenseIn in, DenseAgg* agg) {
  __shared__ uint32_t s_red[3][kQThreads / 32];
  __shared__ uint32_t s_first, s_last;
  const uint32_t r = blockIdx.x;
  const uint64_t s64 = (uint64_t)r * in.range_chunks;
  const uint32_t s = s64 < in.nchunks ? (uint32_t)s64 : in.nchunks;
  const uint32_t e = s64 + in.range_chunks < in.nchunks ? (uint32_t)(s64 + in.range_chunks)
                                                         : in.nchunks;
  if (threadIdx.x == 0) {
    s_first = kNone;
    s_last = 0;
  }
  __syncthreads();
  // rows, non-empty chunks, and fills inside the range: a non-empty chunk
  // whose predecessor (c - 1) is empty and which is not the range's first
  // non-empty chunk gets a fill word
  uint32_t rows = 0, nz = 0, gaps = 0;
  uint32_t first = kNone, last = 0;
  for (uint32_t c = s + threadIdx.x; c < e; c += kQThreads) {
    const uint32_t v = combine_op(in.a, in.b, in.op, c);
    if (!v) continue;
    rows += __popc(v);
    ++nz;
    first = c < first ? c : first;
    last = c > last ? c : last;
    if (c > s && combine_op(in.a, in.b, in.op, c - 1) == 0) ++gaps;
  }
  if (first != kNone) {
    atomicMin(&s_first, first);
    atomicMax(&s_last, last);
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    rows += __shfl_xor_sync(0xffffffffu, rows, d);
    nz += __shfl_xor_sync(0xffffffffu, nz, d);
    gaps += __shfl_xor_sync(0xffffffffu, gaps, d);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    s_red[0][warp] = rows;
    s_red[1][warp] = nz;
    s_red[2][warp] = gaps;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t R = 0, N = 0, G = 0;
    for (int w = 0; w < kQThreads / 32; ++w) {
      R += s_red[0][w];
      N += s_red[1][w];
      G += s_red[2][w];
    }
    DenseAgg g = {};
    g.rows = R;
    g.first_nz = N ? s_first : kNone;
    g.last_nz = N ? s_last : kNone;
    // a gap before the first non-empty chunk is decided by the scan
    if (N && s_first > s && combine_op(in.a, in.b, in.op, s_first - 1) == 0) --G;
    g.words = N + G;
    agg[r] = g;
  }
}

__global__ void __launch_bounds__(kScanThreads) k_dense_scan(DenseAgg* agg, uint32_t ranges,
                                                             wah_query_result* res) {
  __shared__ uint32_t s_w[kScanThreads / 32 + 1];
  __shared__ int s_m[kScanThreads / 32 + 1];
  constexpr uint32_t PER = kMaxQueryRanges / kScanThreads;
  const uint32_t base = threadIdx.x * PER;
  // 1. last non-empty chunk before each range
  int last = -1;
  for (uint32_t i = 0; i < PER; ++i)
    if (base + i < ranges && agg[base + i].last_nz != kNone) last = (int)agg[base + i].last_nz;
  int mtot;
  int prev = block_exclusive_max<kScanThreads>(last, &mtot, s_m);
  // 2. words (with the first chunk's fill) and rows
  uint32_t words = 0, rows = 0;
  uint32_t wl[PER];
  for (uint32_t i = 0; i < PER; ++i) {
    wl[i] = 0;
    if (base + i >= ranges) continue;
    const DenseAgg a = agg[base + i];
    if (a.first_nz != kNone) {
      const uint32_t gap = prev < 0 ? a.first_nz : a.first_nz - (uint32_t)prev - 1;
      wl[i] = a.words + (gap ? 1u : 0u);
      prev = (int)a.last_nz;
    }
    words += wl[i];
    rows += a.rows;
  }
  uint32_t wtot, rtot;
  uint32_t wex = block_exclusive_scan<kScanThreads>(words, &wtot, s_w);
  uint32_t rex = block_exclusive_scan<kScanThreads>(rows, &rtot, s_w);
  int prev2 = block_exclusive_max<kScanThreads>(last, &mtot, s_m);
  for (uint32_t i = 0; i < PER; ++i) {
    if (base + i >= ranges) continue;
    DenseAgg& a = agg[base + i];
    a.words_base = wex;
    a.rows_base = rex;
    a.prev_nz = prev2 < 0 ? kNone : (uint32_t)prev2;
    wex += wl[i];
    rex += a.rows;
    if (a.last_nz != kNone) prev2 = (int)a.last_nz;
  }
  if (threadIdx.x == 0) {
    res->words = wtot;
    res->rows = rtot;
  }
}

__global__ void __launch_bounds__(kQThreads) k_dense_emit(DenseIn in, const DenseAgg* agg,
                                                          uint32_t* words_out, uint64_t words_cap,
                                                          uint32_t* rows_out, uint64_t rows_cap,
                                                          wah_query_result* res) {
  __shared__ uint32_t s_w[kQThreads / 32 + 1];
  __shared__ int s_m[kQThreads / 32 + 1];
  const uint32_t r = blockIdx.x;
  const uint64_t s64 = (uint64_t)r * in.range_chunks;
  const uint32_t s = s64 < in.nchunks ? (uint32_t)s64 : in.nchunks;
  const uint32_t e = s64 + in.range_chunks < in.nchunks ? (uint32_t)(s64 + in.range_chunks)
                                                         : in.nchunks;
  if (s >= e || agg[r].first_nz == kNone) return;
  int prev_carry = agg[r].prev_nz == kNone ? -1 : (int)agg[r].prev_nz;
  uint32_t wpos_carry = agg[r].words_base;
  uint32_t rpos_carry = agg[r].rows_base;
  for (uint32_t t0 = s; t0 < e; t0 += kQTile) {
    const uint32_t t1 = t0 + kQTile < e ? t0 + kQTile : e;
    const uint32_t p = t0 + threadIdx.x * kQItems;
    uint32_t v[kQItems];
    int last = -1;
    uint32_t rows = 0;
#pragma unroll
    for (int q = 0; q < kQItems; ++q) {
      v[q] = p + q < t1 ? combine_op(in.a, in.b, in.op, p + q) : 0u;
      if (v[q]) {
        last = (int)(p + q);
        rows += __popc(v[q]);
      }
    }
    int mtot;
    int prev = block_exclusive_max<kQThreads>(last, &mtot, s_m);
    if (prev < prev_carry) prev = prev_carry;
    uint32_t words = 0;
    {
      int pv = prev;
#pragma unroll
      for (int q = 0; q < kQItems; ++q)
        if (v[q]) {
          const uint32_t c = p + q;
          const uint32_t gap = pv < 0 ? c : c - (uint32_t)pv - 1;
          words += 1 + (gap ? 1u : 0u);
          pv = (int)c;
        }
    }
    uint32_t wtot, rtot;
    const uint32_t wex = block_exclusive_scan<kQThreads>(words, &wtot, s_w);
    const uint32_t rex = block_exclusive_scan<kQThreads>(rows, &rtot, s_w);
    uint32_t wpos = wpos_carry + wex, rpos = rpos_carry + rex;
    int pv = prev;
#pragma unroll
    for (int q = 0; q < kQItems; ++q) {
      if (!v[q]) continue;
      const uint32_t c = p + q;
      const uint32_t gap = pv < 0 ? c : c - (uint32_t)pv - 1;
      pv = (int)c;
      if (words_out) {
        if ((uint64_t)wpos + (gap ? 2u : 1u) > words_cap) {
          set_status(&res->status, WAH_EOVERFLOW);
        } else {
          if (gap) words_out[wpos] = gap;
          words_out[wpos + (gap ? 1 : 0)] = kLitBit | v[q];
        }
      }
      wpos += gap ? 2u : 1u;
      if (rows_out) {
        uint32_t bits = v[q];
        while (bits) {
          const uint32_t b = __ffs(bits) - 1;
          bits &= bits - 1;
          if (rpos < rows_cap) rows_out[rpos] = c * 31u + b;
          else set_status(&res->status, WAH_EOVERFLOW);
          ++rpos;
        }
      } else {
        rpos += __popc(v[q]);
      }
    }
    if (mtot > prev_carry) prev_carry = mtot;
    wpos_carry += wtot;
    rpos_carry += rtot;
  }
}

__global__ void k_status_to_result(const uint32_t* status, wah_query_result* res) {
  if (threadIdx.x == 0 && *status != WAH_OK && res->status == WAH_OK) res->status = *status;
}

__global__ void k_decode_check(const Span* sp, uint64_t n, uint32_t* status) {
  if (threadIdx.x == 0 && sp->rows != n) set_status(status, WAH_ECORRUPT);
}

}  // namespace
}  // namespace wah

using namespace wah;

extern "C" {

size_t wah_decode_workspace_bytes(void) { return walk_bytes(); }

int wah_decode(const uint32_t* d_keys, const uint32_t* d_offsets, const uint32_t* d_index,
               uint32_t keycnt, uint32_t index_len, uint64_t n, uint32_t* d_rows,
               uint32_t* d_row_values, uint32_t* d_column, uint32_t* d_key_rows,
               uint32_t* d_status, void* d_workspace, size_t workspace_bytes, void* stream) {
  if (!d_status || !aligned16(d_status)) return WAH_EINVAL;
  if (n >= WAH_MAX_ROWS) return WAH_ERANGE;
  if (keycnt > 0 && (!d_keys || !d_offsets || !d_index)) return WAH_EINVAL;
  if (!d_workspace || workspace_bytes < walk_bytes() || !aligned16(d_workspace))
    return WAH_ENOMEM;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  uint32_t launches = 0;
  cudaError_t e = cudaMemsetAsync(d_status, 0, sizeof(uint32_t), s);
  WalkIn in{d_keys, d_offsets, d_index, keycnt, index_len};
  WalkWs ws = walk_ws(static_cast<unsigned char*>(d_workspace));
  if (e == cudaSuccess) {
    if (d_rows && !d_row_values && !d_column) {
      DecodeRowsAct act{d_rows, d_key_rows, n, d_status};
      e = enqueue_walk(in, 0u, 0xFFFFFFFFu, ws, act, s, &launches);
    } else {
      DecodeAct act{d_keys, d_rows, d_row_values, d_column, d_key_rows, n, d_status};
      e = enqueue_walk(in, 0u, 0xFFFFFFFFu, ws, act, s, &launches);
    }
  }
  if (e == cudaSuccess) {
    k_decode_check<<<1, 32, 0, s>>>(ws.span, n, d_status);
    ++launches;
    e = cudaGetLastError();
  }
  *last_launches_slot() = launches;
  return cuda_status(e);
}

size_t wah_query_workspace_bytes(uint64_t n) {
  const uint64_t nchunks = ceil_div(n, 31);
  return 2 * walk_bytes() + 2 * align_up(nchunks * 4 + 4) + align_up(sizeof(uint32_t) * 4) +
         align_up(sizeof(DenseAgg) * kMaxQueryRanges);
}

int wah_query(const uint32_t* d_keys, const uint32_t* d_offsets, const uint32_t* d_index,
              uint32_t keycnt, uint32_t index_len, uint64_t n, uint32_t a_lo, uint32_t a_hi,
              int op, uint32_t b_lo, uint32_t b_hi, uint32_t* d_words, uint64_t words_cap,
              uint32_t* d_rows, uint64_t rows_cap, wah_query_result* d_result, void* d_workspace,
              size_t workspace_bytes, void* stream) {
  if (!d_result || !aligned16(d_result)) return WAH_EINVAL;
  if (op < WAH_QUERY_KEYS || op > WAH_QUERY_ANDNOT) return WAH_EINVAL;
  if (n >= WAH_MAX_ROWS) return WAH_ERANGE;
  if (keycnt > 0 && (!d_keys || !d_offsets || !d_index)) return WAH_EINVAL;
  if (!d_workspace || workspace_bytes < wah_query_workspace_bytes(n) || !aligned16(d_workspace))
    return WAH_ENOMEM;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const uint64_t nchunks = ceil_div(n, 31);
  unsigned char* base = static_cast<unsigned char*>(d_workspace);
  WalkWs wa = walk_ws(base);
  WalkWs wb = walk_ws(base + walk_bytes());
  size_t off = 2 * walk_bytes();
  uint32_t* dense_a = reinterpret_cast<uint32_t*>(base + off);
  off += align_up(nchunks * 4 + 4);
  uint32_t* dense_b = reinterpret_cast<uint32_t*>(base + off);
  off += align_up(nchunks * 4 + 4);
  uint32_t* status = reinterpret_cast<uint32_t*>(base + off);
  off += align_up(sizeof(uint32_t) * 4);
  DenseAgg* dagg = reinterpret_cast<DenseAgg*>(base + off);

  uint32_t launches = 0;
  cudaError_t e = cudaMemsetAsync(d_result, 0, sizeof(wah_query_result), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, sizeof(uint32_t), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(dense_a, 0, nchunks * 4 + 4, s);
  const bool two = op != WAH_QUERY_KEYS;
  if (e == cudaSuccess && two) e = cudaMemsetAsync(dense_b, 0, nchunks * 4 + 4, s);
  WalkIn in{d_keys, d_offsets, d_index, keycnt, index_len};
  if (e == cudaSuccess)
    e = enqueue_walk(in, a_lo, a_hi, wa, ExpandAct{dense_a, nchunks, status}, s, &launches);
  if (e == cudaSuccess && two)
    e = enqueue_walk(in, b_lo, b_hi, wb, ExpandAct{dense_b, nchunks, status}, s, &launches);
  const uint32_t R = query_ranges();
  DenseIn di;
  di.a = dense_a;
  di.b = dense_b;
  di.op = op;
  di.nchunks = (uint32_t)nchunks;
  di.range_chunks = (uint32_t)(ceil_div(ceil_div(nchunks ? nchunks : 1, R), kQTile) * kQTile);
  if (e == cudaSuccess) {
    k_dense_count<<<R, kQThreads, 0, s>>>(di, dagg);
    k_dense_scan<<<1, kScanThreads, 0, s>>>(dagg, R, d_result);
    k_dense_emit<<<R, kQThreads, 0, s>>>(di, dagg, d_words, d_words ? words_cap : 0, d_rows,
                                         d_rows ? rows_cap : 0, d_result);
    k_status_to_result<<<1, 32, 0, s>>>(status, d_result);
    launches += 4;
    e = cudaGetLastError();
  }
  *last_launches_slot() = launches;
  return cuda_status(e);
}

}  // extern "C"
