// wah_index.cu -- phases a2..a6 fused into one pass over the sorted
// (value, rid) stream.
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
// Here one kernel does all of it, over tiles of 2048 sorted rows (256
// threads x 8 consecutive rows, loaded with 128-bit loads into registers and
// mirrored in shared memory with one row of look-behind and 30 rows of
// look-ahead: a (value, chunk) segment has at most 31 rows, so the tile that
// owns a segment's head can finish its literal).  Each row is classified
// locally: segment head when (value, chunk) changes, value head when the
// value changes; a head emits 1 + (fill != 0) words.  Literals come from a
// reverse segmented OR over the thread's rows.  One packed block scan plus a
// decoupled look-back across tiles (64-bit entries carrying the word and key
// prefixes together) gives every head its final position; words, keys and
// offsets are staged in shared memory and written once, coalesced, with no
// zero words and no compaction pass.
#include "wah_common.cuh"

namespace wah {

constexpr int kLookAhead = 30;  // a segment has at most 31 rows
constexpr int kWinRows = kBuildTile + kLookAhead + 2;

// Staging index skew: position i lives at i + i/16, so threads writing runs
// that start ~16 words apart hit different banks.
__device__ __forceinline__ uint32_t skew(uint32_t i) { return i + (i >> 4); }
constexpr int kSkewed(int n) { return n + n / 16 + 1; }

struct BuildSmem {
  uint32_t v[kWinRows];   // sorted values of rows base .. base+TILE+29
  uint32_t cb[kWinRows];  // (chunk << 5) | (rid % 31) of the same rows
  uint32_t words[kSkewed(2 * kBuildTile)];
  uint32_t keys[kSkewed(kBuildTile)];
  uint32_t offs[kSkewed(kBuildTile)];
  uint64_t warp_tmp[kBuildThreads / 32 + 1];
  uint64_t tile_prefix;  // exclusive (keys << 32 | words) before this tile
  uint32_t prev_v, prev_cb;
  uint32_t tile;
  int abort;
};

__device__ __forceinline__ uint32_t chunk_bit(uint32_t rid) {
  const uint32_t c = rid / 31;
  return (c << 5) | (rid - c * 31);
}

// Look-back over earlier tiles by warp 0; returns the exclusive prefix.
__device__ __forceinline__ uint64_t build_lookback(uint64_t* __restrict__ lb, uint32_t tile,
                                                   uint32_t* status, int* abort) {
  const int lane = threadIdx.x & 31;
  uint64_t excl = 0;
  int64_t k = (int64_t)tile - 1 - lane;
  uint32_t spins = 0;
  while (true) {
    const uint64_t e = k >= 0 ? ld_relaxed_u64(lb + k) : kLbPrefix64;
    const uint32_t fl = (uint32_t)(e >> 62);
    if (__any_sync(0xffffffffu, fl == 0)) {
      if (++spins > kSpinLimit) {
        if (lane == 0) {
          set_status(status, WAH_ETIMEOUT);
          *abort = 1;
        }
        break;
      }
      __nanosleep(spins > kSpinFast ? 256 : 32);
      continue;
    }
    const uint32_t pmask = __ballot_sync(0xffffffffu, fl == 2);
    const int stop = pmask ? __ffs(pmask) - 1 : 31;
    uint64_t val = lane <= stop ? (e & kLbMask64) : 0;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) val += __shfl_xor_sync(0xffffffffu, val, d);
    excl += val;
    if (pmask) break;
    k -= 32;
  }
  return excl;
}

// Per-thread counters packed for one block scan: words | keys << 21 | segs << 42.
constexpr int kPackShift = 21;
constexpr uint64_t kPackMask = (1ull << kPackShift) - 1;

__global__ void __launch_bounds__(kBuildThreads, 4)
    k_wah_build(SortBufs bufs, int sel, uint64_t n, WahCtrl* ctrl, uint64_t* __restrict__ lb,
                uint32_t* __restrict__ keys, uint32_t* __restrict__ offsets,
                uint32_t* __restrict__ index, uint64_t keys_cap, uint64_t index_cap,
                wah_counts* counts) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  BuildSmem& sm = *reinterpret_cast<BuildSmem*>(smem_raw);
  uint32_t* status = &counts->status;

  const int s = sel >= 0 ? sel : ctrl->final_sel;
  const uint32_t* __restrict__ sv = s == 0 ? bufs.keys[0] : (s == 1 ? bufs.keys[1] : bufs.keys[2]);
  const uint32_t* __restrict__ sr = s == 0 ? bufs.rids[0] : (s == 1 ? bufs.rids[1] : bufs.rids[2]);

  const uint32_t tid = threadIdx.x;
  if (tid == 0) {
    sm.tile = atomicAdd(&ctrl->tile_ctr[4], 1u);
    sm.abort = 0;
  }
  __syncthreads();
  const uint32_t tile = sm.tile;
  const uint64_t base = (uint64_t)tile * kBuildTile;
  const bool full = base + kBuildTile <= n;
  const uint32_t valid = full ? kBuildTile : (uint32_t)(n - base);
  // rows of the window that exist (tile + look-ahead, clipped at n)
  const uint64_t left = n - base;
  const uint32_t wend = left < (uint64_t)(kBuildTile + kLookAhead) ? (uint32_t)left
                                                                    : (uint32_t)(kBuildTile + kLookAhead);

  // This thread's rows: first .. first+7 of the tile, in registers.
  const uint32_t first = tid * kBuildItems;
  uint32_t v[kBuildItems], cb[kBuildItems];
  if (full) {
    const uint4* v4 = reinterpret_cast<const uint4*>(sv + base + first);
    const uint4 a0 = v4[0], a1 = v4[1];
    v[0] = a0.x; v[1] = a0.y; v[2] = a0.z; v[3] = a0.w;
    v[4] = a1.x; v[5] = a1.y; v[6] = a1.z; v[7] = a1.w;
    if (sr) {
      const uint4* r4 = reinterpret_cast<const uint4*>(sr + base + first);
      const uint4 b0 = r4[0], b1 = r4[1];
      cb[0] = chunk_bit(b0.x); cb[1] = chunk_bit(b0.y); cb[2] = chunk_bit(b0.z);
      cb[3] = chunk_bit(b0.w); cb[4] = chunk_bit(b1.x); cb[5] = chunk_bit(b1.y);
      cb[6] = chunk_bit(b1.z); cb[7] = chunk_bit(b1.w);
    } else {
#pragma unroll
      for (int j = 0; j < kBuildItems; ++j) cb[j] = chunk_bit((uint32_t)base + first + j);
    }
  } else {
#pragma unroll
    for (int j = 0; j < kBuildItems; ++j) {
      const bool ok = first + j < valid;
      v[j] = ok ? sv[base + first + j] : 0u;
      const uint32_t r = ok ? (sr ? sr[base + first + j] : (uint32_t)base + first + j) : 0u;
      cb[j] = chunk_bit(r);
    }
  }
  {
    uint4* wv = reinterpret_cast<uint4*>(&sm.v[first]);
    uint4* wc = reinterpret_cast<uint4*>(&sm.cb[first]);
    wv[0] = make_uint4(v[0], v[1], v[2], v[3]);
    wv[1] = make_uint4(v[4], v[5], v[6], v[7]);
    wc[0] = make_uint4(cb[0], cb[1], cb[2], cb[3]);
    wc[1] = make_uint4(cb[4], cb[5], cb[6], cb[7]);
  }
  // Look-ahead rows (segments that start in this tile end inside them).
  if (tid < kLookAhead) {
    const uint32_t i = kBuildTile + tid;
    if (i < wend) {
      sm.v[i] = sv[base + i];
      sm.cb[i] = chunk_bit(sr ? sr[base + i] : (uint32_t)(base + i));
    }
  }
  // Look-behind row: the last row of the previous tile, or, for the first
  // tile, a value that differs from row 0 (so row 0 heads a new key).
  if (tid == kBuildThreads - 1) {
    if (base > 0) {
      sm.prev_v = sv[base - 1];
      sm.prev_cb = chunk_bit(sr ? sr[base - 1] : (uint32_t)(base - 1));
    } else {
      sm.prev_v = ~sv[0];
      sm.prev_cb = 0;
    }
  }
  __syncthreads();

  // Classify rows: head of a (value, chunk) segment / head of a value.
  uint32_t pv = tid ? sm.v[first - 1] : sm.prev_v;
  uint32_t pc = (tid ? sm.cb[first - 1] : sm.prev_cb) >> 5;
  uint32_t headm = 0, vheadm = 0, fills[kBuildItems];
  uint32_t nw = 0;
#pragma unroll
  for (int j = 0; j < kBuildItems; ++j) {
    const uint32_t c = cb[j] >> 5;
    const bool ok = full || first + j < valid;
    const bool vh = v[j] != pv;
    const bool h = ok && (vh || c != pc);
    fills[j] = vh ? c : c - pc - 1;
    if (h) {
      headm |= 1u << j;
      if (vh) vheadm |= 1u << j;
      nw += 1 + (fills[j] != 0);
    }
    pv = v[j];
    pc = c;
  }
  const uint32_t nk = __popc(vheadm), ns = __popc(headm);

  // Literals: reverse segmented OR.  First the rows after this thread's last
  // row that continue its last segment (from shared memory), then backwards.
  uint32_t acc = 0;
  {
    const uint32_t c7 = cb[kBuildItems - 1] >> 5;
    for (uint32_t m = first + kBuildItems; m < wend; ++m) {
      if (sm.v[m] != v[kBuildItems - 1] || (sm.cb[m] >> 5) != c7) break;
      acc |= 1u << (sm.cb[m] & 31);
    }
  }
  uint32_t lits[kBuildItems];
#pragma unroll
  for (int j = kBuildItems - 1; j >= 0; --j) {
    if (full || first + j < valid) acc |= 1u << (cb[j] & 31);  // rows past n add nothing
    lits[j] = acc | 0x80000000u;
    if (headm & (1u << j)) acc = 0;
  }

  uint64_t tile_agg;
  const uint64_t my_prefix = block_exclusive_scan64<kBuildThreads>(
      (uint64_t)nw | ((uint64_t)nk << kPackShift) | ((uint64_t)ns << (2 * kPackShift)), &tile_agg,
      sm.warp_tmp);
  const uint32_t tw = (uint32_t)(tile_agg & kPackMask);
  const uint32_t tk = (uint32_t)((tile_agg >> kPackShift) & kPackMask);
  const uint32_t ts = (uint32_t)(tile_agg >> (2 * kPackShift));

  if (tid == 0 && ts) atomicAdd(&counts->merged, ts);
  const uint64_t agg = ((uint64_t)tk << 32) | tw;
  if (tid == 0) st_relaxed_u64(lb + tile, (tile == 0 ? kLbPrefix64 : kLbAggregate64) | agg);

  // Stage this thread's words, keys and offsets at tile-local positions
  // (before the look-back, which then finds its predecessors published).
  uint32_t pw = (uint32_t)(my_prefix & kPackMask);
  uint32_t pk = (uint32_t)((my_prefix >> kPackShift) & kPackMask);
#pragma unroll
  for (int j = 0; j < kBuildItems; ++j) {
    if (headm & (1u << j)) {
      if (vheadm & (1u << j)) {
        sm.keys[skew(pk)] = v[j];
        sm.offs[skew(pk)] = pw;  // tile-local; the tile's word prefix is added below
        ++pk;
      }
      if (fills[j]) sm.words[skew(pw++)] = fills[j];
      sm.words[skew(pw++)] = lits[j];
    }
  }
  if (tid < 32) {
    uint64_t excl = 0;
    if (tile > 0) {
      excl = build_lookback(lb, tile, status, &sm.abort);
      if (tid == 0) st_relaxed_u64(lb + tile, kLbPrefix64 | (excl + agg));
    }
    if (tid == 0) sm.tile_prefix = excl;
  }
  __syncthreads();
  if (sm.abort) return;
  const uint64_t tile_prefix = sm.tile_prefix;
  const uint32_t xw = (uint32_t)(tile_prefix & 0xffffffffu);
  const uint32_t xk = (uint32_t)(tile_prefix >> 32);

  bool overflow = false;
  for (uint32_t i = tid; i < tw; i += kBuildThreads) {
    const uint64_t pos = (uint64_t)xw + i;
    if (pos < index_cap)
      index[pos] = sm.words[skew(i)];
    else
      overflow = true;
  }
  for (uint32_t i = tid; i < tk; i += kBuildThreads) {
    const uint64_t pos = (uint64_t)xk + i;
    if (pos < keys_cap) {
      keys[pos] = sm.keys[skew(i)];
      offsets[pos] = xw + sm.offs[skew(i)];
    } else {
      overflow = true;
    }
  }
  if (overflow) set_status(status, WAH_EOVERFLOW);

  // The last tile knows the totals.
  if (tid == 0 && base + kBuildTile >= n) {
    const uint64_t tot = tile_prefix + (((uint64_t)tk << 32) | tw);
    counts->index_len = (uint32_t)(tot & 0xffffffffu);
    counts->keycnt = (uint32_t)(tot >> 32);
  }
}

cudaError_t launch_build(const BuildLaunch& a, cudaStream_t s, uint32_t* launches) {
  const uint64_t tiles = ceil_div(a.n, kBuildTile);
  const size_t smem = sizeof(BuildSmem);
  cudaError_t err =
      cudaFuncSetAttribute(k_wah_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  err = cudaMemsetAsync(a.lb_build, 0, tiles * sizeof(uint64_t), s);
  if (err != cudaSuccess) return err;
  record_phase(a.events, kPhaseBuild, false, s);
  k_wah_build<<<(unsigned)tiles, kBuildThreads, smem, s>>>(
      a.src, a.sel, a.n, a.ctrl, a.lb_build, a.keys, a.offsets, a.index, a.keys_cap,
      a.index_cap, a.counts);
  record_phase(a.events, kPhaseBuild, true, s);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace wah
