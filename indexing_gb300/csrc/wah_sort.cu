// wah_sort.cu -- phase a1, sort_rids_by_value, as a stable onesweep LSD radix
// sort carrying row ids.
//
// Reference semantics: src/cpu.cpp:180-197 (stable bubble sort by value,
// rids = iota) and src/phases.cpp:143-160 (the same as std::stable_sort).
// The reference GPU path (src/phases.cpp:745-773 over include/radix.cl:65-233)
// runs 4 passes x (count, scan, reorder_kv) of 4-bit digits over the low 16
// bits only.  Here:
//   k_digit_histogram  one read of the keys builds the histograms of all four
//                      8-bit digits (128-bit loads; per-thread run-length
//                      counting so constant digits cost no shared atomics)
//   k_sort_plan        scans the histograms into global bin offsets and plans
//                      the passes: a digit whose values all fall in one bin is
//                      skipped (the stable sort by it is the identity)
//   k_onesweep_pass    one launch per digit: tile load, warp match-based
//                      stable ranking, decoupled look-back across tiles for
//                      each bin's global offset, staged scatter.  The first
//                      active pass takes rid = row index (no iota kernel).
#include <algorithm>

#include "wah_common.cuh"

namespace wah {

// ---------------------------------------------------------------------------
// Digit histograms.  Keys are read once with 128-bit loads.  Per warp and key
// slot, a digit whose 8 bits agree across all 32 lanes (found from the warp's
// OR and AND of the keys) is counted with one shared atomic for the warp
// instead of 32: constant high digits of small keys and runs of equal values
// cost almost nothing.  DIGITS is the number of digit passes the bound allows;
// the OR of all keys is kept so the plan can flag values above the bound.
// ---------------------------------------------------------------------------
template <int DIGITS>
struct WarpHist {
  uint32_t (*h)[kRadix];  // this warp's private [DIGITS][256] counters
  __device__ __forceinline__ void add_full_warp(uint32_t x, uint32_t lane, uint32_t& acc_or) {
    const uint32_t o = __reduce_or_sync(0xffffffffu, x);
    const uint32_t a = __reduce_and_sync(0xffffffffu, x);
    acc_or |= o;
    const uint32_t varying = o ^ a;
#pragma unroll
    for (int p = 0; p < DIGITS; ++p) {
      const uint32_t d = bfe(x, p * kRadixBits, kRadixBits);
      if (bfe(varying, p * kRadixBits, kRadixBits) == 0) {
        if (lane == 0) atomicAdd(&h[p][d], 32u);
      } else {
        atomicAdd(&h[p][d], 1u);
      }
    }
  }
  __device__ __forceinline__ void add_one(uint32_t x, uint32_t& acc_or) {
    acc_or |= x;
#pragma unroll
    for (int p = 0; p < DIGITS; ++p) atomicAdd(&h[p][bfe(x, p * kRadixBits, kRadixBits)], 1u);
  }
};

template <int DIGITS>
__global__ void __launch_bounds__(kHistThreads)
    k_digit_histogram(const uint32_t* __restrict__ keys, uint64_t n, WahCtrl* ctrl) {
  __shared__ uint32_t s_h[kHistWarps][DIGITS][kRadix];
  for (int i = threadIdx.x; i < kHistWarps * DIGITS * kRadix; i += kHistThreads)
    (&s_h[0][0][0])[i] = 0;
  __syncthreads();

  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  WarpHist<DIGITS> wh{s_h[warp]};
  uint32_t acc_or = 0;
  // Work unit: a chunk of 32 consecutive uint4 (512 keys), one per lane.
  const uint64_t n4 = n / 4;
  const uint64_t chunks = n4 / 32;  // full chunks
  const uint4* kv = reinterpret_cast<const uint4*>(keys);
  const uint64_t gwarp = (uint64_t)blockIdx.x * kHistWarps + warp;
  const uint64_t nwarps = (uint64_t)gridDim.x * kHistWarps;
  uint64_t c = gwarp;
  for (; c + (kHistUnroll - 1) * nwarps < chunks; c += kHistUnroll * nwarps) {
    uint4 q[kHistUnroll];
#pragma unroll
    for (int u = 0; u < kHistUnroll; ++u) q[u] = ld_stream_v4(kv + (c + u * nwarps) * 32 + lane);
#pragma unroll
    for (int u = 0; u < kHistUnroll; ++u) {
      wh.add_full_warp(q[u].x, lane, acc_or);
      wh.add_full_warp(q[u].y, lane, acc_or);
      wh.add_full_warp(q[u].z, lane, acc_or);
      wh.add_full_warp(q[u].w, lane, acc_or);
    }
  }
  for (; c < chunks; c += nwarps) {
    const uint4 q = ld_stream_v4(kv + c * 32 + lane);
    wh.add_full_warp(q.x, lane, acc_or);
    wh.add_full_warp(q.y, lane, acc_or);
    wh.add_full_warp(q.z, lane, acc_or);
    wh.add_full_warp(q.w, lane, acc_or);
  }
  // Ragged end (< 512 keys): the first warp of the grid, one key per lane.
  if (gwarp == 0) {
    for (uint64_t i = chunks * 128 + lane; i < n; i += 32) wh.add_one(keys[i], acc_or);
  }
  acc_or = __reduce_or_sync(0xffffffffu, acc_or);
  if (lane == 0 && acc_or) atomicOr(&ctrl->key_or, acc_or);
  __syncthreads();
  for (int j = threadIdx.x; j < DIGITS * kRadix; j += kHistThreads) {
    uint32_t c2 = 0;
#pragma unroll
    for (int w = 0; w < kHistWarps; ++w) c2 += (&s_h[w][0][0])[j];
    if (c2) atomicAdd(&(&ctrl->hist[0][0])[j], c2);
  }
}

// ---------------------------------------------------------------------------
// Pass plan: bin offsets per digit, trivial digits skipped, ping-pong homes.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kRadix)
    k_sort_plan(WahCtrl* ctrl, uint64_t n, int passes, uint32_t* status) {
  __shared__ uint32_t s_warp[kRadix / 32 + 1];
  __shared__ int s_active[kDigits];
  const int b = threadIdx.x;
  for (int p = 0; p < passes; ++p) {
    const uint32_t h = ctrl->hist[p][b];
    const int trivial = __syncthreads_or(h == (uint32_t)n);
    uint32_t total;
    const uint32_t excl = block_exclusive_scan<kRadix>(h, &total, s_warp);
    ctrl->bin_off[p][b] = excl;
    if (b == 0) s_active[p] = !trivial;
  }
  __syncthreads();
  if (b == 0) {
    // A set bit above the digits the bound allows: the sort would be wrong.
    if (passes < kDigits && (ctrl->key_or >> (passes * kRadixBits)) != 0)
      set_status(status, WAH_ERANGE);
    int cur = kSelInput;
    for (int p = 0; p < kDigits; ++p) {
      if (p < passes && s_active[p]) {
        ctrl->pass_src[p] = cur;
        const int dst = (cur == kSelA) ? kSelB : kSelA;
        ctrl->pass_dst[p] = dst;
        cur = dst;
      } else {
        ctrl->pass_src[p] = -1;
        ctrl->pass_dst[p] = -1;
      }
    }
    ctrl->final_sel = cur;
  }
}

// ---------------------------------------------------------------------------
// One onesweep digit pass over tiles of 4096 rows (256 threads x 16).
//
//  load     warp-striped: item j of lane l in warp w is tile row
//           w*512 + j*32 + l, so a warp's item-j load is one 128-byte line;
//           (j, l) order is row order, which makes the ranking stable
//  rank     all 16 peer masks first (__match_any_sync, independent, so their
//           latency overlaps), then per item one shared read of the warp's
//           bin counter, a leader update and a popcount
//  publish  per-bin tile counts as look-back aggregates, then a per-bin
//           decoupled look-back (thread b walks bin b) for the global offset
//  scatter  rows to shared memory in tile-sorted order, then written out by
//           consecutive threads to consecutive positions of each bin run
// ---------------------------------------------------------------------------
constexpr int kSortWarps = kSortThreads / 32;
static_assert(kSortThreads == kRadix, "one thread per bin in the look-back");

template <int ITEMS>
struct SortPassSmem {
  uint32_t whist[kSortWarps][kRadix];  // per-warp counts -> tile-local starts
  uint32_t bin_base[kRadix];           // global position - tile-local start
  uint32_t warp_tmp[kSortWarps + 1];
  uint32_t tile;
  int abort;
  uint32_t keys[kSortThreads * ITEMS];
  uint32_t rids[kSortThreads * ITEMS];
};

struct SortPassArgs {
  const uint32_t* input;  // selector kSelInput (rid = row index)
  uint32_t* keys_a;
  uint32_t* rids_a;
  uint32_t* keys_b;
  uint32_t* rids_b;
  uint64_t n;
  int pass;
  WahCtrl* ctrl;
  uint32_t* lookback;
  uint32_t* status;
};

// Rows past n in the last tile are padded with key 0xFFFFFFFF: digit 255 in
// every pass, and since the ranking is stable they land after every real row
// of bin 255, which is the last bin -- i.e. at tile-local positions >= the
// number of real rows, which are never written out.  Only the last tile's
// look-back counts include them, and no tile reads those.
template <int ITEMS>
__device__ __forceinline__ void onesweep_tile(const SortPassArgs& a, SortPassSmem<ITEMS>& sm,
                                              const uint32_t* __restrict__ kin,
                                              const uint32_t* __restrict__ rin,
                                              uint32_t* __restrict__ kout,
                                              uint32_t* __restrict__ rout, uint32_t tile,
                                              uint64_t base) {
  constexpr uint32_t TILE = kSortThreads * ITEMS;
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t shift = a.pass * kRadixBits;
  const bool full = base + TILE <= a.n;
  const uint32_t valid = full ? TILE : (uint32_t)(a.n - base);
  const uint32_t row0 = warp * 32 * ITEMS + lane;  // tile row of item 0

  uint32_t key[ITEMS], rid[ITEMS];
  {
    const uint32_t* kp = kin + base + row0;
    if (full) {
#pragma unroll
      for (int j = 0; j < ITEMS; ++j) key[j] = kp[j * 32];
    } else {
#pragma unroll
      for (int j = 0; j < ITEMS; ++j)
        key[j] = row0 + j * 32 < valid ? kp[j * 32] : 0xffffffffu;
    }
  }

  // Peer masks first (independent), then the sequential counter updates.
  uint32_t rank[ITEMS];
#pragma unroll
  for (int j = 0; j < ITEMS; ++j)
    rank[j] = __match_any_sync(0xffffffffu, bfe(key[j], shift, kRadixBits));
  const uint32_t lt = lanemask_lt(), gt = lanemask_gt();
  uint32_t* wh = sm.whist[warp];
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    const uint32_t peers = rank[j];
    const uint32_t d = bfe(key[j], shift, kRadixBits);
    const uint32_t cnt = wh[d];
    __syncwarp();
    if ((peers & gt) == 0) wh[d] = cnt + __popc(peers);
    __syncwarp();
    rank[j] = cnt + __popc(peers & lt);
  }
  // Row ids are loaded only now (registers are free of the peer masks); the
  // loads overlap the look-back below.
  if (rin) {
    const uint32_t* rp = rin + base + row0;
    if (full) {
#pragma unroll
      for (int j = 0; j < ITEMS; ++j) rid[j] = rp[j * 32];
    } else {
#pragma unroll
      for (int j = 0; j < ITEMS; ++j) rid[j] = row0 + j * 32 < valid ? rp[j * 32] : 0u;
    }
  } else {
    const uint32_t r0 = (uint32_t)base + row0;
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) rid[j] = r0 + j * 32;
  }
  __syncthreads();

  // Thread b: the tile's count for bin b, then warp starts within the tile.
  const uint32_t b = tid;
  uint32_t count = 0;
#pragma unroll
  for (int w = 0; w < kSortWarps; ++w) count += sm.whist[w][b];
  uint32_t* lb = a.lookback + (uint64_t)tile * kRadix + b;
  st_relaxed_u32(lb, (tile == 0 ? kLbPrefix32 : kLbAggregate32) | count);

  uint32_t tile_total;
  const uint32_t lstart = block_exclusive_scan<kSortThreads>(count, &tile_total, sm.warp_tmp);
  {
    uint32_t run = lstart;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
      const uint32_t c = sm.whist[w][b];
      sm.whist[w][b] = run;
      run += c;
    }
  }

  uint32_t excl = 0;
  if (tile > 0) {
    uint32_t k = tile - 1;
    uint32_t spins = 0;
    while (true) {
      const uint32_t e = ld_relaxed_u32(a.lookback + (uint64_t)k * kRadix + b);
      const uint32_t fl = e >> kLbFlagShift32;
      if (fl == 0) {
        if (++spins > kSpinLimit) {
          set_status(a.status, WAH_ETIMEOUT);
          sm.abort = 1;
          break;
        }
        if (spins > kSpinFast) __nanosleep(128);
        continue;
      }
      excl += e & kLbMask32;
      if (fl == 2 || k == 0) break;
      --k;
    }
    st_relaxed_u32(lb, kLbPrefix32 | (excl + count));
  }
  sm.bin_base[b] = a.ctrl->bin_off[a.pass][b] + excl - lstart;
  __syncthreads();

#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    const uint32_t r = wh[bfe(key[j], shift, kRadixBits)] + rank[j];
    sm.keys[r] = key[j];
    sm.rids[r] = rid[j];
  }
  __syncthreads();
  if (sm.abort) return;  // positions unknown: write nothing

  const uint32_t n32 = (uint32_t)a.n;
#pragma unroll 4
  for (int it = 0; it < ITEMS; ++it) {
    const uint32_t i = it * kSortThreads + tid;
    if (i < valid) {
      const uint32_t k = sm.keys[i];
      const uint32_t g = sm.bin_base[bfe(k, shift, kRadixBits)] + i;
      if (g < n32) {
        kout[g] = k;
        rout[g] = sm.rids[i];
      } else {
        set_status(a.status, WAH_ETIMEOUT);
      }
    }
  }
}

template <int ITEMS, int MIN_BLOCKS>
__global__ void __launch_bounds__(kSortThreads, MIN_BLOCKS) k_onesweep_pass(SortPassArgs a) {
  constexpr uint32_t TILE = kSortThreads * ITEMS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SortPassSmem<ITEMS>& sm = *reinterpret_cast<SortPassSmem<ITEMS>*>(smem_raw);
  const int src = a.ctrl->pass_src[a.pass];
  if (src < 0) return;  // trivial digit: every row in one bin, order unchanged
  const int dst = a.ctrl->pass_dst[a.pass];
  const uint32_t* kin = src == kSelInput ? a.input : (src == kSelA ? a.keys_a : a.keys_b);
  const uint32_t* rin = src == kSelInput ? nullptr : (src == kSelA ? a.rids_a : a.rids_b);
  uint32_t* kout = dst == kSelA ? a.keys_a : a.keys_b;
  uint32_t* rout = dst == kSelA ? a.rids_a : a.rids_b;

  const uint32_t tid = threadIdx.x;
  if (tid == 0) {
    sm.tile = atomicAdd(&a.ctrl->tile_ctr[a.pass], 1u);
    sm.abort = 0;
  }
  {
    uint4* w4 = reinterpret_cast<uint4*>(&sm.whist[0][0]);
    for (uint32_t i = tid; i < kSortWarps * kRadix / 4; i += kSortThreads)
      w4[i] = make_uint4(0, 0, 0, 0);
  }
  __syncthreads();
  const uint32_t tile = sm.tile;
  onesweep_tile<ITEMS>(a, sm, kin, rin, kout, rout, tile, (uint64_t)tile * TILE);
}

// Compiled tile shapes of the onesweep pass (rows per thread, CTAs per SM the
// register budget is fitted to).  sort_items selects one; the autotuner
// measures them.
struct SortVariant {
  int items;
  void (*fn)(SortPassArgs);
  size_t smem;
};

SortVariant sort_variant(int items) {
  switch (items) {
    case 8: return {8, k_onesweep_pass<8, 4>, sizeof(SortPassSmem<8>)};
    case 12: return {12, k_onesweep_pass<12, 3>, sizeof(SortPassSmem<12>)};
    case 20: return {20, k_onesweep_pass<20, 2>, sizeof(SortPassSmem<20>)};
    default: return {16, k_onesweep_pass<16, 2>, sizeof(SortPassSmem<16>)};
  }
}

uint64_t sort_tiles(uint64_t n, int items) {
  return ceil_div(n, (uint64_t)kSortThreads * sort_variant(items).items);
}

cudaError_t launch_sort(const SortLaunch& a, cudaStream_t s, uint32_t* launches) {
  const uint64_t n = a.n;
  // Histogram: enough CTAs to keep every SM busy with 16-byte loads in flight.
  {
    const uint64_t work = ceil_div(n / 128 + 1, (uint64_t)kHistWarps * kHistUnroll);
    const uint64_t cap = (uint64_t)a.sm_count * 8;
    const int grid = (int)(work < cap ? work : cap);
    record_phase(a.events, kPhaseHist, false, s);
    switch (a.passes) {
      case 1: k_digit_histogram<1><<<grid, kHistThreads, 0, s>>>(a.values, n, a.ctrl); break;
      case 2: k_digit_histogram<2><<<grid, kHistThreads, 0, s>>>(a.values, n, a.ctrl); break;
      case 3: k_digit_histogram<3><<<grid, kHistThreads, 0, s>>>(a.values, n, a.ctrl); break;
      default: k_digit_histogram<4><<<grid, kHistThreads, 0, s>>>(a.values, n, a.ctrl); break;
    }
    record_phase(a.events, kPhaseHist, true, s);
    ++*launches;
  }
  record_phase(a.events, kPhasePlan, false, s);
  k_sort_plan<<<1, kRadix, 0, s>>>(a.ctrl, n, a.passes, a.status);
  record_phase(a.events, kPhasePlan, true, s);
  ++*launches;
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;

  SortPassArgs pa;
  pa.input = a.values;
  pa.keys_a = a.buf_keys[0];
  pa.rids_a = a.buf_rids[0];
  pa.keys_b = a.buf_keys[1];
  pa.rids_b = a.buf_rids[1];
  pa.n = n;
  pa.ctrl = a.ctrl;
  pa.lookback = a.lb_sort;
  pa.status = a.status;
  const SortVariant v = sort_variant(a.sort_items);
  const uint64_t tiles = ceil_div(n, (uint64_t)kSortThreads * v.items);
  err = cudaFuncSetAttribute(v.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)v.smem);
  if (err != cudaSuccess) return err;
  for (int p = 0; p < kDigits; ++p) {
    if (p >= a.passes) {  // not launched: empty span keeps every event valid
      record_phase(a.events, kPhasePass0 + p, false, s);
      record_phase(a.events, kPhasePass0 + p, true, s);
      continue;
    }
    err = cudaMemsetAsync(a.lb_sort, 0, tiles * kRadix * sizeof(uint32_t), s);
    if (err != cudaSuccess) return err;
    pa.pass = p;
    record_phase(a.events, kPhasePass0 + p, false, s);
    v.fn<<<(unsigned)tiles, kSortThreads, v.smem, s>>>(pa);
    record_phase(a.events, kPhasePass0 + p, true, s);
    ++*launches;
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

// Copies the sorted stream from its device-chosen home into caller buffers
// (rid = row index when no pass ran: all values equal, or n == 1).
__global__ void k_sort_deliver(SortBufs bufs, const WahCtrl* ctrl, uint64_t n,
                               uint32_t* __restrict__ out_keys, uint32_t* __restrict__ out_rids) {
  const int sel = ctrl->final_sel;
  const uint32_t* __restrict__ k = sel == 0 ? bufs.keys[0] : (sel == 1 ? bufs.keys[1] : bufs.keys[2]);
  const uint32_t* __restrict__ r = sel == 0 ? bufs.rids[0] : (sel == 1 ? bufs.rids[1] : bufs.rids[2]);
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    out_keys[i] = k[i];
    out_rids[i] = r ? r[i] : (uint32_t)i;
  }
}

cudaError_t launch_sort_deliver(const SortBufs& bufs, const WahCtrl* ctrl, uint64_t n,
                                uint32_t* out_keys, uint32_t* out_rids, cudaStream_t s,
                                uint32_t* launches) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint64_t want = ceil_div(n, 256), cap = (uint64_t)(sms > 0 ? sms : 1) * 8;
  const int grid = (int)(want < cap ? want : cap);
  k_sort_deliver<<<grid, 256, 0, s>>>(bufs, ctrl, n, out_keys, out_rids);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace wah
