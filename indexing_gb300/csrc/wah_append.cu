// wah_append.cu -- appending a row slice's index to an existing index on the
// device (incremental builds).
//
// The reference's `gpu` program indexes its column in slices and its merger
// appends each slice's words to its key's bitmap (src/gpu.cpp:103-165,
// :228-259).  A slice's bitmap starts at the slice's first row and has no
// trailing fill, so the plain append loses the zero chunks between a key's
// last row in earlier slices and its first row in the new one.  Here A (the
// index of rows [0, R)) and B (the index of rows [R, R + n), R a multiple of
// 31) become the index of all R + n rows, exactly as one build of the whole
// column gives it:
//
//   keys     the union of A's and B's keys, ascending (a merge of two sorted
//            lists: each B key's place in A by binary search, a scan of the
//            keys new to A)
//   words    per key: A's words, then B's words with B's leading fill (the
//            zero chunks before the key's first row in the slice) replaced by
//            the zero chunks between A's last literal of the key and that
//            row: fill = R/31 + lead - end_A, dropped when 0
//   end_A    the chunk after a key's last literal in A: the sum of the
//            chunk advances of the key's words (k_key_ends)
//
// Offsets are an exclusive scan of the per-key word counts; the words move
// in load-balanced pieces of 4,096 (a scan over per-key piece counts tells
// each warp which key and part its pieces belong to).
#include "wah_walk.cuh"

namespace wah {
namespace {

// End chunk of every A key: the chunks its words cover (a literal one, a
// fill its count), summed over the key's words.  Grid-stride tiles of
// 256 x 16 words; thread t sums words t*16 .. t*16+15 of the tile, finding
// the key of its first word by binary search over the keys the tile touches.
// A thread adds each finished key's share with an atomic; a warp whose lanes
// all end in one key adds their shares with one atomic.  Sums are 64-bit so a
// corrupt A (fills past row R) cannot wrap back into range.
constexpr uint32_t kEndItems = 16;
constexpr uint32_t kEndTile = 256 * kEndItems;

// Last key whose first word is <= i, searched in [lo, hi] (offsets[lo] <= i).
__device__ __forceinline__ uint32_t key_of_word(const uint32_t* offsets, uint32_t lo, uint32_t hi,
                                                uint32_t i) {
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (offsets[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// First key of every tile of A's words: key k writes the tiles that start
// inside its words (tile_key was zeroed; offsets are clamped so a corrupt
// index cannot write out of range).
__global__ void k_tile_keys(const uint32_t* __restrict__ offsets, uint32_t ka, uint32_t la,
                            uint32_t* __restrict__ tile_key) {
  const uint32_t ntiles = (uint32_t)ceil_div(la, kEndTile);
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < ka; k += gridDim.x * blockDim.x) {
    uint32_t w1 = k + 1 < ka ? offsets[k + 1] : la;
    w1 = w1 < la ? w1 : la;
    uint32_t w0 = offsets[k];
    w0 = w0 < w1 ? w0 : w1;
    const uint32_t t_end = (uint32_t)ceil_div(w1, kEndTile);
    for (uint32_t t = (uint32_t)ceil_div(w0, kEndTile); t < t_end && t < ntiles; ++t)
      tile_key[t] = k;
  }
}

// Tile word i lives at i + i/32 in shared memory: the coalesced loads
// (consecutive i per warp) and the per-thread reads (i = 16 t + j) both
// spread over all 32 banks.
__device__ __forceinline__ uint32_t end_skew(uint32_t i) { return i + (i >> 5); }

__global__ void __launch_bounds__(256) k_key_ends(const uint32_t* __restrict__ offsets,
                                                  const uint32_t* __restrict__ index,
                                                  uint32_t ka, uint32_t la,
                                                  const uint32_t* __restrict__ tile_key,
                                                  unsigned long long* __restrict__ ends) {
  __shared__ uint32_t s_w[kEndTile + kEndTile / 32];
  const uint32_t ntiles = (uint32_t)ceil_div(la, kEndTile);
  const uint32_t lane = threadIdx.x & 31;
  for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const uint32_t t0 = t * kEndTile;
    const uint32_t t1 = la - t0 < kEndTile ? la : t0 + kEndTile;
    // the keys this tile touches: from its first word's key up to the next
    // tile's first key (a bound on its last word's key)
    const uint32_t k_lo = tile_key[t] < ka ? tile_key[t] : ka - 1;
    const uint32_t k_nx = t + 1 < ntiles ? tile_key[t + 1] : ka - 1;
    const uint32_t k_hi = k_nx < ka ? k_nx : ka - 1;
#pragma unroll
    for (uint32_t j = 0; j < kEndItems; ++j) {
      const uint32_t i = j * 256 + threadIdx.x;
      s_w[end_skew(i)] = t0 + i < t1 ? index[t0 + i] : 0u;
    }
    __syncthreads();
    const uint32_t l0 = threadIdx.x * kEndItems;  // this thread's first tile word
    uint32_t key = kNone;
    unsigned long long acc = 0;
    if (t0 + l0 < t1) {
      key = key_of_word(offsets, k_lo, k_hi, t0 + l0);
      uint32_t next = key + 1 < ka ? offsets[key + 1] : la;
      const uint32_t l1 = t1 - t0 - l0 < kEndItems ? t1 - t0 : l0 + kEndItems;
      for (uint32_t l = l0; l < l1; ++l) {
        while (t0 + l >= next) {  // the key ended before this word (every key has a word)
          atomicAdd(&ends[key], acc);
          acc = 0;
          ++key;
          next = key + 1 < ka ? offsets[key + 1] : la;
        }
        acc += chunk_advance(s_w[end_skew(l)]);
      }
    }
    const uint32_t key0 = __shfl_sync(0xffffffffu, key, 0);
    if (__all_sync(0xffffffffu, key == key0 || key == kNone)) {
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, d);
      if (lane == 0 && key0 != kNone) atomicAdd(&ends[key0], acc);
    } else if (key != kNone) {
      atomicAdd(&ends[key], acc);
    }
    __syncthreads();  // s_w is rewritten by the next tile
  }
}

// ---------------------------------------------------------------------------
// Exclusive scan of n u32 values (look-back free: per-range sums, one CTA
// scanning the range sums, per-range rescans with the carries).
// ---------------------------------------------------------------------------
constexpr uint32_t kAScanRanges = 1024;
constexpr int kAThreads = 256;
constexpr uint32_t kATile = kAThreads * 4;

__global__ void __launch_bounds__(kAThreads) k_range_sums(const uint32_t* in, uint64_t n,
                                                          uint64_t per, uint32_t* sums) {
  __shared__ uint32_t s_red[kAThreads / 32];
  const uint64_t lo = (uint64_t)blockIdx.x * per;
  const uint64_t hi = lo + per < n ? lo + per : n;
  uint32_t acc = 0;
  for (uint64_t i = lo + threadIdx.x; i < hi; i += kAThreads) acc += in[i];
  acc = __reduce_add_sync(0xffffffffu, acc);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < kAThreads / 32; ++w) t += s_red[w];
    sums[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(1024) k_scan_sums(uint32_t* sums, uint32_t ranges,
                                                    uint32_t* total) {
  __shared__ uint32_t s_w[1024 / 32 + 1];
  const uint32_t x = threadIdx.x < ranges ? sums[threadIdx.x] : 0u;
  uint32_t t;
  const uint32_t ex = block_exclusive_scan<1024>(x, &t, s_w);
  if (threadIdx.x < ranges) sums[threadIdx.x] = ex;
  if (threadIdx.x == 0 && total) *total = t;
}

__global__ void __launch_bounds__(kAThreads) k_range_rescan(const uint32_t* in, uint32_t* out,
                                                            uint64_t n, uint64_t per,
                                                            const uint32_t* sums) {
  __shared__ uint32_t s_w[kAThreads / 32 + 1];
  const uint64_t lo = (uint64_t)blockIdx.x * per;
  const uint64_t hi = lo + per < n ? lo + per : n;
  uint32_t carry = sums[blockIdx.x];
  for (uint64_t t0 = lo; t0 < hi; t0 += kATile) {
    uint32_t v[4], sum = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint64_t i = t0 + threadIdx.x * 4 + q;
      v[q] = i < hi ? in[i] : 0u;
      sum += v[q];
    }
    uint32_t tot;
    uint32_t ex = carry + block_exclusive_scan<kAThreads>(sum, &tot, s_w);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint64_t i = t0 + threadIdx.x * 4 + q;
      if (i < hi) out[i] = ex;
      ex += v[q];
    }
    carry += tot;
  }
}

// out[i] = sum of in[0..i), *total = sum of all (device); in may equal out.
cudaError_t scan_u32(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* total,
                     uint32_t* sums, cudaStream_t s) {
  if (n == 0) return total ? cudaMemsetAsync(total, 0, 4, s) : cudaSuccess;
  const uint64_t per = ceil_div(ceil_div(n, kAScanRanges), kATile) * kATile;
  const uint32_t ranges = (uint32_t)ceil_div(n, per);
  k_range_sums<<<ranges, kAThreads, 0, s>>>(in, n, per, sums);
  k_scan_sums<<<1, 1024, 0, s>>>(sums, ranges, total);
  k_range_rescan<<<ranges, kAThreads, 0, s>>>(in, out, n, per, sums);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Merging the key sets.
// ---------------------------------------------------------------------------
struct AppendIn {
  const uint32_t *a_keys, *a_offsets, *a_index;
  uint32_t ka, la;
  const uint32_t *b_keys, *b_offsets, *b_index;
  uint32_t kb, lb;
  uint32_t first_chunk;  // rows_a / 31
};

__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t* a, uint32_t n, uint32_t x) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Per B key: its place in A and whether A lacks it.
__global__ void k_match_b(AppendIn in, uint32_t* b_pos, uint32_t* b_new) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < in.kb; j += gridDim.x * blockDim.x) {
    const uint32_t x = in.b_keys[j];
    const uint32_t pos = lower_bound_u32(in.a_keys, in.ka, x);
    b_pos[j] = pos;
    b_new[j] = (pos < in.ka && in.a_keys[pos] == x) ? 0u : 1u;
  }
}

// Output slots: A key i goes to i + (new B keys below it), B key j to its
// place in A + (new B keys before it).  b_rank[kb] = new B keys in all.
__global__ void k_place(AppendIn in, const uint32_t* b_pos, const uint32_t* b_rank,
                        uint32_t* src_a, uint32_t* src_b, uint32_t* out_keys) {
  const uint32_t total = in.ka + in.kb;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += gridDim.x * blockDim.x) {
    if (t < in.ka) {
      const uint32_t x = in.a_keys[t];
      const uint32_t o = t + b_rank[lower_bound_u32(in.b_keys, in.kb, x)];
      src_a[o] = t;
      out_keys[o] = x;
    } else {
      const uint32_t j = t - in.ka;
      const uint32_t o = b_pos[j] + b_rank[j];
      src_b[o] = j;
      out_keys[o] = in.b_keys[j];
    }
  }
}

struct KeyParts {
  uint32_t a_begin, a_len;  // A's words of the key
  uint32_t b_begin, b_len;  // B's words after its leading fill
  uint32_t gap;             // fill word between them (0: none)
  bool has_b;
};

__device__ __forceinline__ KeyParts key_parts(const AppendIn& in, const unsigned long long* ends,
                                              uint32_t ia, uint32_t jb, uint32_t* status) {
  KeyParts k = {0, 0, 0, 0, 0, false};
  uint64_t end_a = 0;
  if (ia != kNone) {
    k.a_begin = in.a_offsets[ia];
    k.a_len = (ia + 1 < in.ka ? in.a_offsets[ia + 1] : in.la) - k.a_begin;
    end_a = ends[ia];
  }
  if (jb != kNone) {
    k.has_b = true;
    const uint32_t b0 = in.b_offsets[jb];
    const uint32_t b1 = jb + 1 < in.kb ? in.b_offsets[jb + 1] : in.lb;
    const uint32_t w = in.b_index[b0];
    uint32_t lead = 0, skip = 0;
    if (!(w & kLitBit)) {
      lead = w & kFillMask;
      skip = 1;
    }
    k.b_begin = b0 + skip;
    k.b_len = b1 - b0 - skip;
    const uint64_t start = (uint64_t)in.first_chunk + lead;  // chunk of the key's first row in B
    if (start < end_a) {
      set_status(status, WAH_ECORRUPT);  // A has rows at or past row R
    } else {
      k.gap = (uint32_t)(start - end_a);
    }
  }
  return k;
}

// Words per output key; pieces of the copy per key.
constexpr uint32_t kPiece = 4096;

__global__ void k_key_words(AppendIn in, const unsigned long long* ends, const uint32_t* src_a,
                            const uint32_t* src_b, const uint32_t* out_count, uint32_t* words,
                            uint32_t* pieces, uint32_t* status) {
  const uint32_t K = *out_count;
  for (uint32_t o = blockIdx.x * blockDim.x + threadIdx.x; o < K; o += gridDim.x * blockDim.x) {
    const KeyParts k = key_parts(in, ends, src_a[o], src_b[o], status);
    words[o] = k.a_len + (k.gap ? 1u : 0u) + k.b_len;
    pieces[o] = (uint32_t)(ceil_div(k.a_len, kPiece) + ceil_div(k.b_len, kPiece));
  }
}

// Every piece: copy up to kPiece words of one key's A or B part.  Each warp
// takes a contiguous share of the pieces: one binary search finds the key
// of its first piece (the last key whose first piece is <= it), later pieces
// step forward.  Warps work independently, so one warp's key lookups overlap
// the others' copies; each lane keeps 8 loads in flight.
constexpr uint32_t kCopyUnroll = 8;

__global__ void __launch_bounds__(kAThreads) k_copy_pieces(
    AppendIn in, const unsigned long long* ends, const uint32_t* src_a, const uint32_t* src_b,
    const uint32_t* out_count, const uint32_t* piece_base, const uint32_t* total_pieces,
    const uint32_t* out_offsets, uint32_t* out_index, uint32_t* status) {
  const uint32_t K = *out_count;
  const uint32_t T = *total_pieces;
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t)gridDim.x * (kAThreads / 32);
  const uint64_t wid = (uint64_t)blockIdx.x * (kAThreads / 32) + threadIdx.x / 32;
  const uint64_t per = ceil_div(T, warps);
  const uint64_t first = wid * per;
  if (first >= T) return;  // no pieces left for this warp
  const uint32_t c0 = (uint32_t)first;
  const uint32_t c1 = T - c0 < per ? T : c0 + (uint32_t)per;
  uint32_t lo = 0, hi = K;  // every lane runs the same search (same loads)
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (piece_base[mid] <= c0) lo = mid + 1;
    else hi = mid;
  }
  uint32_t o = lo - 1;
  for (uint32_t c = c0; c < c1; ++c) {
    while (o + 1 < K && piece_base[o + 1] <= c) ++o;
    const KeyParts k = key_parts(in, ends, src_a[o], src_b[o], status);
    const uint32_t na = (uint32_t)ceil_div(k.a_len, kPiece);
    const uint32_t local = c - piece_base[o];
    const uint32_t dst0 = out_offsets[o];
    const uint32_t* src;
    uint32_t* dst;
    uint32_t len;
    if (local < na) {
      const uint32_t off = local * kPiece;
      src = in.a_index + k.a_begin + off;
      dst = out_index + dst0 + off;
      len = k.a_len - off < kPiece ? k.a_len - off : kPiece;
    } else {
      const uint32_t off = (local - na) * kPiece;
      src = in.b_index + k.b_begin + off;
      dst = out_index + dst0 + k.a_len + (k.gap ? 1u : 0u) + off;
      len = k.b_len - off < kPiece ? k.b_len - off : kPiece;
    }
    for (uint32_t base = 0; base < len; base += 32 * kCopyUnroll) {
      uint32_t v[kCopyUnroll];
#pragma unroll
      for (uint32_t j = 0; j < kCopyUnroll; ++j) {
        const uint32_t i = base + j * 32 + lane;
        if (i < len) v[j] = src[i];
      }
#pragma unroll
      for (uint32_t j = 0; j < kCopyUnroll; ++j) {
        const uint32_t i = base + j * 32 + lane;
        if (i < len) dst[i] = v[j];
      }
    }
  }
}

// Gap words (keys with a B part and a non-zero gap), and keys with no piece.
__global__ void k_gap_words(AppendIn in, const unsigned long long* ends, const uint32_t* src_a,
                            const uint32_t* src_b, const uint32_t* out_count,
                            const uint32_t* out_offsets, uint32_t* out_index, uint32_t* status) {
  const uint32_t K = *out_count;
  for (uint32_t o = blockIdx.x * blockDim.x + threadIdx.x; o < K; o += gridDim.x * blockDim.x) {
    const KeyParts k = key_parts(in, ends, src_a[o], src_b[o], status);
    if (k.has_b && k.gap) out_index[out_offsets[o] + k.a_len] = k.gap;
  }
}

__global__ void k_keycount(uint32_t ka, const uint32_t* new_keys, uint32_t* out_k) {
  if (threadIdx.x == 0) *out_k = ka + *new_keys;
}

__global__ void k_append_counts(const uint32_t* out_k, const uint32_t* words,
                                const uint32_t* status, wah_counts* counts) {
  if (threadIdx.x != 0) return;
  wah_counts c;
  c.keycnt = *out_k;
  c.index_len = *words;
  c.merged = 0;
  c.status = *status;
  *counts = c;
}

__global__ void k_set_u32(uint32_t* p, uint32_t v) {
  if (threadIdx.x == 0) *p = v;
}

// Workspace layout of one append.
struct AppendWs {
  unsigned long long* ends;
  uint32_t *b_pos, *b_rank, *src_a, *src_b, *words, *pieces, *sums, *scalars;
  size_t bytes;
};

AppendWs append_layout(unsigned char* base, uint64_t ka, uint64_t kb) {
  AppendWs w;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char* p = base ? base + off : nullptr;
    off += align_up(bytes);
    return p;
  };
  const uint64_t kc = ka + kb;
  w.ends = reinterpret_cast<unsigned long long*>(take((ka + 1) * 8));
  w.b_pos = reinterpret_cast<uint32_t*>(take((kb + 1) * 4));
  w.b_rank = reinterpret_cast<uint32_t*>(take((kb + 1) * 4));
  w.src_a = reinterpret_cast<uint32_t*>(take((kc + 1) * 4));
  w.src_b = reinterpret_cast<uint32_t*>(take((kc + 1) * 4));
  w.words = reinterpret_cast<uint32_t*>(take((kc + 1) * 4));
  w.pieces = reinterpret_cast<uint32_t*>(take((kc + 1) * 4));
  w.sums = reinterpret_cast<uint32_t*>(take(kAScanRanges * 4));
  w.scalars = reinterpret_cast<uint32_t*>(take(16 * 4));
  w.bytes = off;
  return w;
}

}  // namespace
}  // namespace wah

using namespace wah;

extern "C" {

size_t wah_append_workspace_bytes(uint32_t keycnt_a, uint32_t keycnt_b) {
  return append_layout(nullptr, keycnt_a, keycnt_b).bytes;
}

int wah_append(const uint32_t* a_keys, const uint32_t* a_offsets, const uint32_t* a_index,
               uint32_t keycnt_a, uint32_t index_len_a, uint64_t rows_a, const uint32_t* b_keys,
               const uint32_t* b_offsets, const uint32_t* b_index, uint32_t keycnt_b,
               uint32_t index_len_b, uint32_t* out_keys, uint32_t* out_offsets,
               uint32_t* out_index, uint64_t keys_cap, uint64_t index_cap, wah_counts* d_counts,
               void* d_workspace, size_t workspace_bytes, void* stream) {
  if (!d_counts || !aligned16(d_counts)) return WAH_EINVAL;
  if (rows_a % 31 || rows_a >= WAH_MAX_ROWS) return WAH_ERANGE;
  if ((keycnt_a && (!a_keys || !a_offsets || !a_index)) ||
      (keycnt_b && (!b_keys || !b_offsets || !b_index)))
    return WAH_EINVAL;
  const uint64_t kc = (uint64_t)keycnt_a + keycnt_b;
  if (kc && (!out_keys || !out_offsets || !out_index)) return WAH_EINVAL;
  // every B key can gain one gap word
  if (kc > keys_cap || (uint64_t)index_len_a + index_len_b + keycnt_b > index_cap)
    return WAH_EOVERFLOW;
  if ((uint64_t)index_len_a + index_len_b + keycnt_b >= (1ull << 32)) return WAH_ERANGE;
  if (!d_workspace || !aligned16(d_workspace) ||
      workspace_bytes < wah_append_workspace_bytes(keycnt_a, keycnt_b))
    return WAH_ENOMEM;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  AppendWs w = append_layout(static_cast<unsigned char*>(d_workspace), keycnt_a, keycnt_b);
  uint32_t* status = w.scalars + 0;
  uint32_t* out_k = w.scalars + 1;
  uint32_t* total_words = w.scalars + 2;
  uint32_t* total_pieces = w.scalars + 3;
  AppendIn in{a_keys, a_offsets, a_index, keycnt_a, index_len_a,
              b_keys, b_offsets, b_index, keycnt_b, index_len_b, (uint32_t)(rows_a / 31)};
  const unsigned grid = (unsigned)sm_count_current() * 4;
  uint32_t launches = 0;
  cudaError_t e = cudaMemsetAsync(w.scalars, 0, 16 * 4, s);
  // 1. end chunk of every A key
  if (e == cudaSuccess && keycnt_a) e = cudaMemsetAsync(w.ends, 0, (size_t)keycnt_a * 8, s);
  if (e == cudaSuccess && keycnt_a && index_len_a) {
    // each tile's first key, kept in the tail of out_index (its words are
    // written only by the copy below, later on the same stream)
    const uint64_t tiles = ceil_div(index_len_a, kEndTile);
    uint32_t* tile_key = out_index + (index_cap - tiles);
    e = cudaMemsetAsync(tile_key, 0, tiles * 4, s);
    if (e == cudaSuccess) {
      k_tile_keys<<<(unsigned)std::min<uint64_t>(ceil_div(keycnt_a, 256), (uint64_t)grid), 256, 0,
                    s>>>(a_offsets, keycnt_a, index_len_a, tile_key);
      k_key_ends<<<(unsigned)std::min<uint64_t>(tiles, (uint64_t)grid * 2), 256, 0, s>>>(
          a_offsets, a_index, keycnt_a, index_len_a, tile_key, w.ends);
      launches += 2;
    }
  }
  // 2. the merged key set: K = ka + B keys new to A
  if (e == cudaSuccess && kc) e = cudaMemsetAsync(w.src_a, 0xFF, kc * 4, s);
  if (e == cudaSuccess && kc) e = cudaMemsetAsync(w.src_b, 0xFF, kc * 4, s);
  if (e == cudaSuccess && keycnt_b) {
    k_match_b<<<grid, 256, 0, s>>>(in, w.b_pos, w.b_rank);
    ++launches;
    e = scan_u32(w.b_rank, w.b_rank, keycnt_b, w.b_rank + keycnt_b, w.sums, s);
    launches += 3;
  } else if (e == cudaSuccess) {
    k_set_u32<<<1, 32, 0, s>>>(w.b_rank, 0u);
    ++launches;
  }
  if (e == cudaSuccess && kc) {
    k_place<<<grid, 256, 0, s>>>(in, w.b_pos, w.b_rank, w.src_a, w.src_b, out_keys);
    ++launches;
  }
  if (e == cudaSuccess) {
    k_keycount<<<1, 32, 0, s>>>(keycnt_a, w.b_rank + keycnt_b, out_k);
    ++launches;
    e = cudaGetLastError();
  }
  // 3. words per key -> offsets; copy pieces per key -> piece starts (slots
  // past K stay zero, so the scans may run over all ka + kb slots)
  if (e == cudaSuccess && kc) e = cudaMemsetAsync(w.words, 0, kc * 4, s);
  if (e == cudaSuccess && kc) e = cudaMemsetAsync(w.pieces, 0, kc * 4, s);
  if (e == cudaSuccess && kc) {
    k_key_words<<<grid, 256, 0, s>>>(in, w.ends, w.src_a, w.src_b, out_k, w.words, w.pieces,
                                     status);
    ++launches;
    e = scan_u32(w.words, out_offsets, kc, total_words, w.sums, s);
    launches += 3;
  }
  if (e == cudaSuccess && kc) {
    e = scan_u32(w.pieces, w.pieces, kc, total_pieces, w.sums, s);
    launches += 3;
  }
  // 4. the words
  if (e == cudaSuccess && kc) {
    k_copy_pieces<<<grid * 2, kAThreads, 0, s>>>(in, w.ends, w.src_a, w.src_b, out_k, w.pieces,
                                                 total_pieces, out_offsets, out_index, status);
    k_gap_words<<<grid, 256, 0, s>>>(in, w.ends, w.src_a, w.src_b, out_k, out_offsets,
                                     out_index, status);
    launches += 2;
  }
  if (e == cudaSuccess) {
    k_append_counts<<<1, 32, 0, s>>>(out_k, total_words, status, d_counts);
    ++launches;
    e = cudaGetLastError();
  }
  *last_launches_slot() = launches;
  return cuda_status(e);
}

}  // extern "C"
