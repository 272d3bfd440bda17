// wah_walk.cuh -- the device-wide walk over a run of keys' WAH words.
//
// Used by the decoder and queries (wah_query.cu); incremental appends
// (wah_append.cu) take only its word constants and chunk_advance.  For every
// word of keys [ka, kb) it knows the word's key, the chunk position of the
// word within its key (a segmented exclusive scan of chunk advances: 1 per
// literal, the count of a fill) and the number of rows in all earlier words
// (a plain exclusive scan of the literals' popcounts), and hands every
// literal to an action.  Look-back free: the words are cut
// into equal ranges, one persistent CTA per range; k_walk_count reduces each
// range, k_walk_scan scans the range aggregates, k_walk_emit re-reads the
// range tile by tile with the carries.
#pragma once

#include "wah_common.cuh"

namespace wah {
namespace {

constexpr int kQThreads = 256;
constexpr int kQItems = 8;
constexpr uint32_t kQTile = kQThreads * kQItems;  // 2048 words or chunks per tile
constexpr uint32_t kLitBit = 0x80000000u;
constexpr uint32_t kFillMask = 0x3FFFFFFFu;
constexpr uint32_t kNone = 0xFFFFFFFFu;

// Control block of one walk (device memory, written by k_span_setup).
struct Span {
  uint32_t ka, kb;       // keys [ka, kb)
  uint32_t w0, w1;       // their words [w0, w1)
  uint32_t range_words;  // words per range, a multiple of kQTile
  uint32_t rows;         // rows decoded (written by k_walk_scan)
  uint32_t pad[2];
};

// Per-range aggregate of a walk; the scan fills the second half.
struct WalkAgg {
  uint32_t pop;       // rows in the range
  uint32_t adv;       // chunk advance after the range's last key head (whole range if none)
  uint32_t has_head;  // a key starts inside the range
  uint32_t pad;
  uint32_t pop_base;  // rows before the range
  uint32_t carry;     // chunk position of the key running into the range
  uint32_t pad2[2];
};

struct Seg {
  uint32_t f;  // a key head lies in the span
  uint32_t s;  // chunk advance since the last head (or over the whole span)
};

__device__ __forceinline__ Seg seg_combine(Seg a, Seg b) {
  Seg r;
  r.f = a.f | b.f;
  r.s = b.f ? b.s : a.s + b.s;
  return r;
}

__device__ __forceinline__ Seg shfl_up_seg(Seg x, int d) {
  Seg y;
  y.f = __shfl_up_sync(0xffffffffu, x.f, d);
  y.s = __shfl_up_sync(0xffffffffu, x.s, d);
  return y;
}

// Exclusive segmented scan of one Seg per thread; *total = block aggregate.
template <int THREADS>
__device__ __forceinline__ Seg block_seg_exclusive(Seg x, Seg* total, Seg* s_warp) {
  constexpr int NW = THREADS / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  Seg incl = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const Seg y = shfl_up_seg(incl, d);
    if (lane >= d) incl = seg_combine(y, incl);
  }
  Seg ex_lane = shfl_up_seg(incl, 1);
  if (lane == 0) ex_lane = Seg{0, 0};
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const Seg w = lane < NW ? s_warp[lane] : Seg{0, 0};
    Seg wi = w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const Seg y = shfl_up_seg(wi, d);
      if (lane >= d) wi = seg_combine(y, wi);
    }
    Seg ex = shfl_up_seg(wi, 1);
    if (lane == 0) ex = Seg{0, 0};
    __syncwarp();
    if (lane < NW) s_warp[lane] = ex;
    if (lane == NW - 1) s_warp[NW] = wi;
  }
  __syncthreads();
  const Seg r = seg_combine(s_warp[warp], ex_lane);
  *total = s_warp[NW];
  __syncthreads();
  return r;
}

// Exclusive max-scan of one signed value per thread (-1 = none).
template <int THREADS>
__device__ __forceinline__ int block_exclusive_max(int x, int* total, int* s_warp) {
  constexpr int NW = THREADS / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl = y > incl ? y : incl;
  }
  int ex_lane = __shfl_up_sync(0xffffffffu, incl, 1);
  if (lane == 0) ex_lane = -1;
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const int w = lane < NW ? s_warp[lane] : -1;
    int wi = w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, wi, d);
      if (lane >= d) wi = y > wi ? y : wi;
    }
    int ex = __shfl_up_sync(0xffffffffu, wi, 1);
    if (lane == 0) ex = -1;
    __syncwarp();
    if (lane < NW) s_warp[lane] = ex;
    if (lane == NW - 1) s_warp[NW] = wi;
  }
  __syncthreads();
  const int wp = s_warp[warp];
  const int r = wp > ex_lane ? wp : ex_lane;
  *total = s_warp[NW];
  __syncthreads();
  return r;
}

// First index i in [0, n) with a[i] > x (upper) or a[i] >= x (lower), n if
// none; a ascending.  One warp searches 32 ways per step.
__device__ uint32_t warp_search(const uint32_t* a, uint32_t n, uint32_t x, bool upper) {
  const int lane = threadIdx.x & 31;
  uint32_t lo = 0, hi = n;  // the answer lies in [lo, hi]
  while (lo < hi) {
    const uint32_t span = hi - lo;
    const uint32_t step = span <= 32 ? 1 : (span + 31) / 32;
    const uint32_t idx = lo + lane * step;
    bool pred = true;
    if (idx < hi) {
      const uint32_t v = a[idx];
      pred = upper ? (v > x) : (v >= x);
    }
    const uint32_t b = __ballot_sync(0xffffffffu, pred);
    if (b == 0) {
      lo = lo + 31 * step + 1;
      continue;
    }
    const int f = __ffs(b) - 1;
    const uint32_t at = lo + f * step;
    if (f == 0) {
      hi = lo;
    } else {
      const uint32_t prev = lo + (f - 1) * step;
      lo = prev + 1;
      hi = at < hi ? at : hi;
    }
  }
  return lo;
}

struct WalkIn {
  const uint32_t* keys;
  const uint32_t* offsets;
  const uint32_t* index;
  uint32_t K, L;
};

// Keys with value in [lo, hi] and their words; range geometry for `ranges`.
__global__ void k_span_setup(WalkIn in, uint32_t lo, uint32_t hi, uint32_t ranges, Span* sp) {
  uint32_t ka = 0, kb = 0;
  if (lo <= hi) {
    ka = warp_search(in.keys, in.K, lo, false);
    kb = warp_search(in.keys, in.K, hi, true);
  }
  if (threadIdx.x != 0) return;
  if (kb < ka) kb = ka;
  Span s;
  s.ka = ka;
  s.kb = kb;
  s.w0 = ka < in.K ? in.offsets[ka] : in.L;
  s.w1 = kb < in.K ? in.offsets[kb] : in.L;
  if (s.w1 < s.w0) s.w1 = s.w0;
  const uint32_t per = (uint32_t)ceil_div(s.w1 - s.w0, ranges);
  s.range_words = (uint32_t)(ceil_div(per ? per : 1, kQTile) * kQTile);
  s.rows = 0;
  s.pad[0] = s.pad[1] = 0;
  *sp = s;
}

__device__ __forceinline__ uint32_t lit_rows(uint32_t w) {
  return (w & kLitBit) ? __popc(w & 0x7FFFFFFFu) : 0u;
}
__device__ __forceinline__ uint32_t chunk_advance(uint32_t w) {
  return (w & kLitBit) ? 1u : (w & kFillMask);
}

__global__ void __launch_bounds__(kQThreads) k_walk_count(WalkIn in, const Span* sp, WalkAgg* agg) {
  __shared__ uint32_t s_red[2][kQThreads / 32];
  __shared__ uint32_t s_from;
  const Span S = *sp;
  const uint32_t r = blockIdx.x;
  const uint64_t s64 = (uint64_t)S.w0 + (uint64_t)r * S.range_words;
  const uint32_t s = s64 < S.w1 ? (uint32_t)s64 : S.w1;
  const uint32_t e = s64 + S.range_words < S.w1 ? (uint32_t)(s64 + S.range_words) : S.w1;
  if (s >= e) {
    if (threadIdx.x == 0) {
      WalkAgg a = {};
      agg[r] = a;
    }
    return;
  }
  // the last key head inside [s, e)
  if (threadIdx.x < 32) {
    const uint32_t u = warp_search(in.offsets + S.ka, S.kb - S.ka, e - 1, true);  // > e-1
    if (threadIdx.x == 0) {
      const uint32_t head = in.offsets[S.ka + u - 1];  // u >= 1: offsets[ka] = w0 <= s
      s_from = head >= s ? head : kNone;
    }
  }
  __syncthreads();
  const uint32_t from = s_from;
  const uint32_t start = from == kNone ? s : from;
  uint32_t pop = 0, adv = 0;
  for (uint32_t i = s + threadIdx.x; i < e; i += kQThreads) {
    const uint32_t w = in.index[i];
    pop += lit_rows(w);
    if (i >= start) adv += chunk_advance(w);
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    pop += __shfl_xor_sync(0xffffffffu, pop, d);
    adv += __shfl_xor_sync(0xffffffffu, adv, d);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    s_red[0][warp] = pop;
    s_red[1][warp] = adv;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t p = 0, a = 0;
    for (int w = 0; w < kQThreads / 32; ++w) {
      p += s_red[0][w];
      a += s_red[1][w];
    }
    WalkAgg g = {};
    g.pop = p;
    g.adv = a;
    g.has_head = from != kNone;
    agg[r] = g;
  }
}

// One CTA of 1024 threads scans up to 4096 range aggregates.
constexpr int kScanThreads = 1024;
constexpr uint32_t kMaxQueryRanges = 4096;

__global__ void __launch_bounds__(kScanThreads) k_walk_scan(WalkAgg* agg, uint32_t ranges, Span* sp) {
  __shared__ uint32_t s_w[kScanThreads / 32 + 1];
  __shared__ Seg s_seg[kScanThreads / 32 + 1];
  constexpr uint32_t PER = kMaxQueryRanges / kScanThreads;
  const uint32_t base = threadIdx.x * PER;
  uint32_t pop = 0;
  Seg loc = {0, 0};
  for (uint32_t i = 0; i < PER; ++i)
    if (base + i < ranges) {
      const WalkAgg a = agg[base + i];
      pop += a.pop;
      loc = seg_combine(loc, Seg{a.has_head, a.adv});
    }
  uint32_t pop_total;
  uint32_t pop_ex = block_exclusive_scan<kScanThreads>(pop, &pop_total, s_w);
  Seg tot;
  Seg ex = block_seg_exclusive<kScanThreads>(loc, &tot, s_seg);
  for (uint32_t i = 0; i < PER; ++i)
    if (base + i < ranges) {
      WalkAgg& a = agg[base + i];
      a.pop_base = pop_ex;
      a.carry = ex.s;
      pop_ex += a.pop;
      ex = seg_combine(ex, Seg{a.has_head, a.adv});
    }
  if (threadIdx.x == 0) sp->rows = pop_total;
}

// One tile [t0, t1) of the emit walk, each thread's kQItems words.  kFull:
// the tile holds kQTile words (16-byte loads where the words are aligned);
// kHeads: key heads (s_heads[0, nh)) may lie in it.  Both are the same for
// the whole block, so every thread takes the same instance and the block
// scans inside line up.  Most tiles are full and hold no key head.
template <bool kFull, bool kHeads, class Act>
__device__ __forceinline__ void walk_tile(const WalkIn& in, const Act& act,
                                          const uint32_t* s_heads, uint32_t nh, uint32_t t0,
                                          uint32_t t1, uint32_t kcur, uint32_t& chunk_carry,
                                          uint32_t& pop_carry, Seg* s_seg, uint32_t* s_pop) {
  const uint32_t p = t0 + threadIdx.x * kQItems;  // this thread's words [p, p + kQItems)
  uint32_t h0 = 0;  // heads before p
  if constexpr (kHeads) {
    uint32_t lo = 0, hi = nh;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (s_heads[mid] < p) lo = mid + 1;
      else hi = mid;
    }
    h0 = lo;
  }
  uint32_t w[kQItems];
  if (kFull && (reinterpret_cast<uintptr_t>(in.index + t0) & 15) == 0) {
    const uint4* w4 = reinterpret_cast<const uint4*>(in.index + p);
#pragma unroll
    for (int q = 0; q < kQItems / 4; ++q) {
      const uint4 v = w4[q];
      w[4 * q + 0] = v.x;
      w[4 * q + 1] = v.y;
      w[4 * q + 2] = v.z;
      w[4 * q + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int q = 0; q < kQItems; ++q) w[q] = (kFull || p + q < t1) ? in.index[p + q] : 0u;
  }
  Seg loc = {0, 0};
  uint32_t pop = 0;
  {
    uint32_t h = h0;
#pragma unroll
    for (int q = 0; q < kQItems; ++q) {
      if (!kFull && p + q >= t1) break;
      if (kHeads && h < nh && s_heads[h] == p + q) {
        loc = Seg{1, 0};
        ++h;
      }
      loc.s += chunk_advance(w[q]);
      pop += lit_rows(w[q]);
    }
  }
  Seg tot;
  const Seg ex = block_seg_exclusive<kQThreads>(loc, &tot, s_seg);
  uint32_t pop_tot;
  const uint32_t pop_ex = block_exclusive_scan<kQThreads>(pop, &pop_tot, s_pop);
  uint32_t chunk = ex.f ? ex.s : chunk_carry + ex.s;
  uint32_t pos = pop_carry + pop_ex;
  // key of word p - 1; a head at p (or later) moves it on before any
  // literal of the new key, so keys[] is read only for valid keys
  uint32_t key = kcur + h0;
  uint32_t value = 0, value_key = kNone;
  {
    uint32_t h = h0;
#pragma unroll
    for (int q = 0; q < kQItems; ++q) {
      if (!kFull && p + q >= t1) break;
      if (kHeads && h < nh && s_heads[h] == p + q) {
        ++h;
        ++key;
        chunk = 0;
        act.head(key, pos);
      }
      const uint32_t x = w[q];
      if (x & kLitBit) {
        if (Act::kNeedsValue && key != value_key) {
          value = in.keys[key];
          value_key = key;
        }
        act.literal(value, chunk, x & 0x7FFFFFFFu, pos);
        pos += __popc(x & 0x7FFFFFFFu);
        chunk += 1;
      } else {
        chunk += x & kFillMask;
      }
    }
  }
  chunk_carry = tot.f ? tot.s : chunk_carry + tot.s;
  pop_carry += pop_tot;
}

template <class Act>
__global__ void __launch_bounds__(kQThreads) k_walk_emit(WalkIn in, const Span* sp,
                                                          const WalkAgg* agg, Act act) {
  __shared__ uint32_t s_heads[kQTile];
  __shared__ Seg s_seg[kQThreads / 32 + 1];
  __shared__ uint32_t s_pop[kQThreads / 32 + 1];
  __shared__ uint32_t s_kcur;
  const Span S = *sp;
  const uint32_t r = blockIdx.x;
  const uint64_t s64 = (uint64_t)S.w0 + (uint64_t)r * S.range_words;
  const uint32_t s = s64 < S.w1 ? (uint32_t)s64 : S.w1;
  const uint32_t e = s64 + S.range_words < S.w1 ? (uint32_t)(s64 + S.range_words) : S.w1;
  if (s >= e) return;
  if (threadIdx.x < 32) {
    // kcur = the key of word s - 1 (the last head below s; ka - 1, wrapping,
    // when s is ka's head), so every head in a tile [t0, t1) is among
    // offsets[kcur + 1 ...] and resets the chunk position where it lies
    const uint32_t u = warp_search(in.offsets + S.ka, S.kb - S.ka, s, false);
    if (threadIdx.x == 0) s_kcur = S.ka + u - 1u;
  }
  __syncthreads();
  uint32_t kcur = s_kcur;
  uint32_t chunk_carry = agg[r].carry;
  uint32_t pop_carry = agg[r].pop_base;
  for (uint32_t t0 = s; t0 < e; t0 += kQTile) {
    const uint32_t t1 = t0 + kQTile < e ? t0 + kQTile : e;
    // key heads inside [t0, t1): offsets[kcur + 1 ...] below t1, read 256 at
    // a time until one reaches t1 (at most kQTile of them)
    uint32_t nh = 0;
    for (uint32_t step = 0; step < kQTile / kQThreads; ++step) {
      const uint32_t j = step * kQThreads + threadIdx.x;
      const uint32_t idx = kcur + 1u + j;  // kcur may be ka - 1 wrapped
      const uint32_t pos = idx < S.kb ? in.offsets[idx] : kNone;
      s_heads[j] = pos;
      const uint32_t inside = __syncthreads_count(pos < t1);
      nh += inside;
      if (inside < (uint32_t)kQThreads) break;
    }
    if (t1 - t0 == kQTile) {
      if (nh == 0)
        walk_tile<true, false>(in, act, s_heads, nh, t0, t1, kcur, chunk_carry, pop_carry,
                               s_seg, s_pop);
      else
        walk_tile<true, true>(in, act, s_heads, nh, t0, t1, kcur, chunk_carry, pop_carry, s_seg,
                              s_pop);
    } else {
      walk_tile<false, true>(in, act, s_heads, nh, t0, t1, kcur, chunk_carry, pop_carry, s_seg,
                             s_pop);
    }
    kcur += nh;
    __syncthreads();  // s_heads is rewritten by the next tile
  }
}

// ---------------------------------------------------------------------------
// Host side of a walk.
// ---------------------------------------------------------------------------
constexpr size_t kAlign = 256;
size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

uint32_t query_ranges() {
  const uint32_t r = (uint32_t)sm_count_current() * 8;
  return r < kMaxQueryRanges ? r : kMaxQueryRanges;
}

// Workspace of one walk: span + range aggregates.
size_t walk_bytes() { return align_up(sizeof(Span)) + align_up(sizeof(WalkAgg) * kMaxQueryRanges); }

struct WalkWs {
  Span* span;
  WalkAgg* agg;
};
WalkWs walk_ws(unsigned char* base) {
  WalkWs w;
  w.span = reinterpret_cast<Span*>(base);
  w.agg = reinterpret_cast<WalkAgg*>(base + align_up(sizeof(Span)));
  return w;
}

template <class Act>
cudaError_t enqueue_walk(const WalkIn& in, uint32_t lo, uint32_t hi, const WalkWs& ws,
                         const Act& act, cudaStream_t s, uint32_t* launches) {
  const uint32_t R = query_ranges();
  k_span_setup<<<1, 32, 0, s>>>(in, lo, hi, R, ws.span);
  k_walk_count<<<R, kQThreads, 0, s>>>(in, ws.span, ws.agg);
  k_walk_scan<<<1, kScanThreads, 0, s>>>(ws.agg, R, ws.span);
  k_walk_emit<Act><<<R, kQThreads, 0, s>>>(in, ws.span, ws.agg, act);
  *launches += 4;
  return cudaGetLastError();
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }


}  // namespace
}  // namespace wah
