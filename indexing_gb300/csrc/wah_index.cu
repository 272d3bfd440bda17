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
// Here one kernel does all of it.  A tile of 2048 sorted rows sits in shared
// memory with one row of look-behind (to classify the first row) and 30 rows
// of look-ahead (a (value, chunk) segment has at most 31 rows, so the tile
// that owns a segment's head can finish its literal).  Each row is classified
// locally: segment head when (value, chunk) changes, value head when the
// value changes; a head emits 1 + (fill != 0) words.  A block scan plus a
// decoupled look-back across tiles (64-bit entries carrying the word and key
// prefixes together) gives every head its final position, so the words are
// written once, in place, with no zero words and no compaction pass.  Keys
// and offsets fall out of the same scan at value heads.
#include "wah_common.cuh"

namespace wah {

__device__ __forceinline__ uint32_t pad_idx(uint32_t i) { return i + (i >> 5); }

constexpr int kWindow = kBuildTile + 31;  // 1 behind + tile + 30 ahead
constexpr int kWindowPadded = kWindow + kWindow / 32 + 1;

struct BuildSmem {
  uint32_t v[kWindowPadded];
  uint32_t r[kWindowPadded];
  uint32_t words[2 * kBuildTile];  // staged index words of this tile
  uint64_t warp_tmp[kBuildThreads / 32 + 1];
  uint64_t tile_prefix;            // exclusive (keys << 32 | words) prefix
  uint32_t tile;
  int abort;
};

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
      if (spins > kSpinFast) __nanosleep(128);
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

__global__ void __launch_bounds__(kBuildThreads, 4)
    k_wah_build(SortBufs bufs, int sel, uint64_t n, WahCtrl* ctrl, uint64_t* __restrict__ lb,
                uint32_t* __restrict__ keys, uint32_t* __restrict__ offsets,
                uint32_t* __restrict__ index, uint64_t keys_cap, uint64_t index_cap,
                wah_counts* counts) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  BuildSmem& sm = *reinterpret_cast<BuildSmem*>(smem_raw);
  uint32_t* status = &counts->status;

  const int s = sel >= 0 ? sel : ctrl->final_sel;
  const uint32_t* __restrict__ sv = bufs.keys[s];
  const uint32_t* __restrict__ sr = bufs.rids[s];  // null: rid = row index

  const int tid = threadIdx.x;
  if (tid == 0) {
    sm.tile = atomicAdd(&ctrl->tile_ctr[4], 1u);
    sm.abort = 0;
  }
  __syncthreads();
  const uint32_t tile = sm.tile;
  const uint64_t base = (uint64_t)tile * kBuildTile;

  // Window element i is row base - 1 + i.
  for (int i = tid; i < kWindow; i += kBuildThreads) {
    const uint64_t g = base + i - 1;  // wraps to 2^64-1 for row -1: excluded
    if (g < n) {
      sm.v[pad_idx(i)] = sv[g];
      sm.r[pad_idx(i)] = sr ? sr[g] : (uint32_t)g;
    }
  }
  __syncthreads();

  // Classify this thread's rows: rows tid*ITEMS .. +ITEMS-1 of the tile.
  const uint32_t first = tid * kBuildItems;
  uint32_t my_words = 0, my_keys = 0, my_segs = 0;
#pragma unroll
  for (int j = 0; j < kBuildItems; ++j) {
    const uint32_t li = first + j;
    const uint64_t g = base + li;
    if (g < n) {
      const uint32_t v = sm.v[pad_idx(li + 1)];
      const uint32_t c = sm.r[pad_idx(li + 1)] / 31;
      bool vhead = true, head = true;
      uint32_t fill = c;
      if (g > 0) {
        const uint32_t vp = sm.v[pad_idx(li)];
        const uint32_t cp = sm.r[pad_idx(li)] / 31;
        vhead = v != vp;
        head = vhead || c != cp;
        if (!vhead) fill = c - cp - 1;
      }
      if (head) {
        my_words += 1 + (fill != 0);
        my_keys += vhead;
        my_segs += 1;
      }
    }
  }

  // Block scan of the packed (keys << 32 | words) counters.
  uint64_t tile_agg;
  const uint64_t my_prefix = block_exclusive_scan64<kBuildThreads>(
      ((uint64_t)my_keys << 32) | my_words, &tile_agg, sm.warp_tmp);

  // Merged-entry count k for the caller (one atomic per tile).
  {
    uint32_t segs_total;
    __shared__ uint32_t s_segs_warp[kBuildThreads / 32 + 1];
    block_exclusive_scan<kBuildThreads>(my_segs, &segs_total, s_segs_warp);
    if (tid == 0 && segs_total) atomicAdd(&counts->merged, segs_total);
  }

  // Look-back: warp 0 publishes the aggregate, waits for the prefix.
  if (tid < 32) {
    uint64_t* lbt = lb + tile;
    uint64_t excl = 0;
    if (tile == 0) {
      if (tid == 0) st_relaxed_u64(lbt, kLbPrefix64 | tile_agg);
    } else {
      if (tid == 0) st_relaxed_u64(lbt, kLbAggregate64 | tile_agg);
      excl = build_lookback(lb, tile, status, &sm.abort);
      if (tid == 0) st_relaxed_u64(lbt, kLbPrefix64 | (excl + tile_agg));
    }
    if (tid == 0) sm.tile_prefix = excl;
  }
  __syncthreads();
  if (sm.abort) return;
  const uint64_t tile_prefix = sm.tile_prefix;
  const uint32_t xw = (uint32_t)(tile_prefix & 0xffffffffu);  // words before tile
  const uint32_t xk = (uint32_t)(tile_prefix >> 32);          // keys before tile

  // Emit: words into shared staging, keys/offsets straight to global.
  uint32_t pw = (uint32_t)(my_prefix & 0xffffffffu);
  uint32_t pk = (uint32_t)(my_prefix >> 32);
  bool overflow = false;
#pragma unroll
  for (int j = 0; j < kBuildItems; ++j) {
    const uint32_t li = first + j;
    const uint64_t g = base + li;
    if (g < n) {
      const uint32_t v = sm.v[pad_idx(li + 1)];
      const uint32_t r = sm.r[pad_idx(li + 1)];
      const uint32_t c = r / 31;
      bool vhead = true, head = true;
      uint32_t fill = c;
      if (g > 0) {
        const uint32_t vp = sm.v[pad_idx(li)];
        const uint32_t cp = sm.r[pad_idx(li)] / 31;
        vhead = v != vp;
        head = vhead || c != cp;
        if (!vhead) fill = c - cp - 1;
      }
      if (head) {
        // OR the segment's rows (at most 31, all inside the window).
        uint32_t lit = 0x80000000u | (1u << (r % 31));
        for (uint32_t m = li + 1; m < li + 31 && base + m < n; ++m) {
          const uint32_t rm = sm.r[pad_idx(m + 1)];
          if (sm.v[pad_idx(m + 1)] != v || rm / 31 != c) break;
          lit |= 1u << (rm % 31);
        }
        if (vhead) {
          const uint64_t kpos = (uint64_t)xk + pk;
          if (kpos < keys_cap) {
            keys[kpos] = v;
            offsets[kpos] = xw + pw;
          } else {
            overflow = true;
          }
          ++pk;
        }
        if (fill) sm.words[pw++] = fill;
        sm.words[pw++] = lit;
      }
    }
  }
  __syncthreads();

  // Coalesced write of the tile's words.
  const uint32_t tw = (uint32_t)(tile_agg & 0xffffffffu);
  for (uint32_t i = tid; i < tw; i += kBuildThreads) {
    const uint64_t pos = (uint64_t)xw + i;
    if (pos < index_cap)
      index[pos] = sm.words[i];
    else
      overflow = true;
  }
  if (overflow) set_status(status, WAH_EOVERFLOW);

  // The last tile knows the totals.
  if (tid == 0 && base + kBuildTile >= n) {
    const uint64_t tot = tile_prefix + tile_agg;
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
