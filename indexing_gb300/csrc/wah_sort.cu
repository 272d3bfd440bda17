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
// Histogram of all four 8-bit digits.
// ---------------------------------------------------------------------------
struct DigitCounter {
  uint32_t last[kDigits];
  uint32_t cnt[kDigits];
  __device__ __forceinline__ void init() {
#pragma unroll
    for (int p = 0; p < kDigits; ++p) {
      last[p] = 0;
      cnt[p] = 0;
    }
  }
  __device__ __forceinline__ void add(uint32_t key, uint32_t (*s_h)[kRadix]) {
#pragma unroll
    for (int p = 0; p < kDigits; ++p) {
      const uint32_t d = (key >> (p * kRadixBits)) & (kRadix - 1);
      if (d == last[p]) {
        ++cnt[p];
      } else {
        if (cnt[p]) atomicAdd(&s_h[p][last[p]], cnt[p]);
        last[p] = d;
        cnt[p] = 1;
      }
    }
  }
  __device__ __forceinline__ void flush(uint32_t (*s_h)[kRadix]) {
#pragma unroll
    for (int p = 0; p < kDigits; ++p)
      if (cnt[p]) atomicAdd(&s_h[p][last[p]], cnt[p]);
  }
};

__global__ void __launch_bounds__(kHistThreads)
    k_digit_histogram(const uint32_t* __restrict__ keys, uint64_t n, WahCtrl* ctrl) {
  __shared__ uint32_t s_h[kDigits][kRadix];
  for (int i = threadIdx.x; i < kDigits * kRadix; i += kHistThreads) (&s_h[0][0])[i] = 0;
  __syncthreads();

  DigitCounter dc;
  dc.init();
  const uint64_t n4 = n / 4;
  const uint4* kv = reinterpret_cast<const uint4*>(keys);
  const uint64_t stride = (uint64_t)gridDim.x * kHistThreads;
  uint64_t i = (uint64_t)blockIdx.x * kHistThreads + threadIdx.x;
  // kHistUnroll independent 16-byte loads in flight per thread.
  for (; i + (kHistUnroll - 1) * stride < n4; i += kHistUnroll * stride) {
    uint4 q[kHistUnroll];
#pragma unroll
    for (int u = 0; u < kHistUnroll; ++u) q[u] = ld_stream_v4(kv + i + u * stride);
#pragma unroll
    for (int u = 0; u < kHistUnroll; ++u) {
      dc.add(q[u].x, s_h);
      dc.add(q[u].y, s_h);
      dc.add(q[u].z, s_h);
      dc.add(q[u].w, s_h);
    }
  }
  for (; i < n4; i += stride) {
    uint4 q = ld_stream_v4(kv + i);
    dc.add(q.x, s_h);
    dc.add(q.y, s_h);
    dc.add(q.z, s_h);
    dc.add(q.w, s_h);
  }
  // ragged tail (n % 4 keys)
  const uint64_t t = n4 * 4 + (uint64_t)blockIdx.x * kHistThreads + threadIdx.x;
  if (t < n) dc.add(keys[t], s_h);
  dc.flush(s_h);
  __syncthreads();
  for (int j = threadIdx.x; j < kDigits * kRadix; j += kHistThreads) {
    const uint32_t c = (&s_h[0][0])[j];
    if (c) atomicAdd(&(&ctrl->hist[0][0])[j], c);
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
  for (int p = 0; p < kDigits; ++p) {
    const uint32_t h = ctrl->hist[p][b];
    const int trivial = __syncthreads_or(h == (uint32_t)n);
    uint32_t total;
    const uint32_t excl = block_exclusive_scan<kRadix>(h, &total, s_warp);
    ctrl->bin_off[p][b] = excl;
    if (b == 0) s_active[p] = !trivial;
  }
  __syncthreads();
  if (b == 0) {
    int cur = kSelInput;
    for (int p = 0; p < kDigits; ++p) {
      if (s_active[p] && p < passes) {
        ctrl->pass_src[p] = cur;
        const int dst = (cur == kSelA) ? kSelB : kSelA;
        ctrl->pass_dst[p] = dst;
        cur = dst;
      } else {
        ctrl->pass_src[p] = -1;
        ctrl->pass_dst[p] = -1;
        // A varying digit above the stated bound: the sort would be wrong.
        if (s_active[p]) set_status(status, WAH_ERANGE);
      }
    }
    ctrl->final_sel = cur;
  }
}

// ---------------------------------------------------------------------------
// One onesweep digit pass.
// ---------------------------------------------------------------------------
struct SortPassSmem {
  uint32_t whist[kSortThreads / 32][kRadix];  // per-warp counts -> prefixes
  uint32_t local_start[kRadix];               // tile-local bin start
  uint32_t bin_base[kRadix];                  // global position - local rank
  uint32_t warp_tmp[kSortThreads / 32 + 1];
  uint32_t tile;
  int abort;
  uint32_t keys[kSortTile];
  uint32_t rids[kSortTile];
};

__global__ void __launch_bounds__(kSortThreads, 3)
    k_onesweep_pass(SortBufs bufs, uint32_t* __restrict__ out_keys_a,
                    uint32_t* __restrict__ out_rids_a, uint32_t* __restrict__ out_keys_b,
                    uint32_t* __restrict__ out_rids_b, uint64_t n, int pass, WahCtrl* ctrl,
                    uint32_t* __restrict__ lookback, uint32_t* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SortPassSmem& sm = *reinterpret_cast<SortPassSmem*>(smem_raw);

  const int src = ctrl->pass_src[pass];
  if (src < 0) return;  // trivial digit: every row in one bin, order unchanged
  const int dst = ctrl->pass_dst[pass];
  const uint32_t* __restrict__ kin = bufs.keys[src];
  const uint32_t* __restrict__ rin = bufs.rids[src];
  uint32_t* __restrict__ kout = dst == kSelA ? out_keys_a : out_keys_b;
  uint32_t* __restrict__ rout = dst == kSelA ? out_rids_a : out_rids_b;
  const int shift = pass * kRadixBits;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    sm.tile = atomicAdd(&ctrl->tile_ctr[pass], 1u);
    sm.abort = 0;
  }
  for (int i = tid; i < (kSortThreads / 32) * kRadix; i += kSortThreads)
    (&sm.whist[0][0])[i] = 0;
  __syncthreads();
  const uint32_t tile = sm.tile;
  const uint64_t base = (uint64_t)tile * kSortTile;

  // Warp-striped load: warp w owns rows [w*32*ITEMS, (w+1)*32*ITEMS) of the
  // tile, item j of lane l is row j*32 + l within it (coalesced 128 B/warp).
  uint32_t key[kSortItems], rid[kSortItems];
  const uint64_t wbase = base + (uint64_t)warp * 32 * kSortItems + lane;
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const uint64_t p = wbase + (uint64_t)j * 32;
    if (p < n) {
      key[j] = kin[p];
      rid[j] = rin ? rin[p] : (uint32_t)p;
    } else {
      key[j] = 0;
      rid[j] = 0;
    }
  }

  // Stable rank inside the warp: items in (j, lane) order == row order.
  uint32_t rank[kSortItems];
  const uint32_t lt = lanemask_lt();
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const uint64_t p = wbase + (uint64_t)j * 32;
    const uint32_t d = p < n ? (key[j] >> shift) & (kRadix - 1) : kRadix;  // kRadix: padding
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    uint32_t before = 0;
    if (d < kRadix) before = sm.whist[warp][d];
    __syncwarp();
    if (d < kRadix && lane == 31 - __clz(peers)) sm.whist[warp][d] = before + __popc(peers);
    __syncwarp();
    rank[j] = before + __popc(peers & lt);
  }
  __syncthreads();

  // Thread b owns bin b: warp prefixes and the tile's count for the bin.
  const int b = tid;
  uint32_t count = 0;
#pragma unroll
  for (int w = 0; w < kSortThreads / 32; ++w) {
    const uint32_t c = sm.whist[w][b];
    sm.whist[w][b] = count;
    count += c;
  }
  uint32_t* lb = lookback + (uint64_t)tile * kRadix + b;
  // Publish the aggregate first so later tiles can look past this one.
  st_relaxed_u32(lb, (tile == 0 ? kLbPrefix32 : kLbAggregate32) | count);

  uint32_t tile_total;
  const uint32_t lstart = block_exclusive_scan<kSortThreads>(count, &tile_total, sm.warp_tmp);
  sm.local_start[b] = lstart;

  // Decoupled look-back over earlier tiles for bin b.
  uint32_t excl = 0;
  if (tile > 0) {
    uint32_t k = tile - 1;
    uint32_t spins = 0;
    while (true) {
      const uint32_t e = ld_relaxed_u32(lookback + (uint64_t)k * kRadix + b);
      const uint32_t fl = e >> kLbFlagShift32;
      if (fl == 0) {
        if (++spins > kSpinLimit) {
          set_status(status, WAH_ETIMEOUT);
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
  sm.bin_base[b] = ctrl->bin_off[pass][b] + excl - lstart;
  __syncthreads();

  // Scatter into shared memory in tile-sorted order.
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const uint64_t p = wbase + (uint64_t)j * 32;
    if (p < n) {
      const uint32_t d = (key[j] >> shift) & (kRadix - 1);
      const uint32_t r = sm.local_start[d] + sm.whist[warp][d] + rank[j];
      sm.keys[r] = key[j];
      sm.rids[r] = rid[j];
    }
  }
  __syncthreads();
  if (sm.abort) return;  // positions unknown: write nothing

  // Coalesced-by-bin write-out: consecutive threads, consecutive positions.
  const uint32_t valid = (n - base) < (uint64_t)kSortTile ? (uint32_t)(n - base) : (uint32_t)kSortTile;
  for (uint32_t i = tid; i < valid; i += kSortThreads) {
    const uint32_t k = sm.keys[i];
    const uint32_t d = (k >> shift) & (kRadix - 1);
    const uint32_t g = sm.bin_base[d] + i;
    if (g < n) {
      kout[g] = k;
      rout[g] = sm.rids[i];
    } else {
      set_status(status, WAH_ETIMEOUT);
    }
  }
}

cudaError_t launch_sort(const SortLaunch& a, cudaStream_t s, uint32_t* launches) {
  const uint64_t n = a.n;
  // Histogram: enough CTAs to keep every SM busy with 16-byte loads in flight.
  {
    const uint64_t work = ceil_div(n / 4 + 1, (uint64_t)kHistThreads * kHistUnroll);
    const uint64_t cap = (uint64_t)a.sm_count * 8;
    const int grid = (int)(work < cap ? work : cap);
    record_phase(a.events, kPhaseHist, false, s);
    k_digit_histogram<<<grid, kHistThreads, 0, s>>>(a.values, n, a.ctrl);
    record_phase(a.events, kPhaseHist, true, s);
    ++*launches;
  }
  record_phase(a.events, kPhasePlan, false, s);
  k_sort_plan<<<1, kRadix, 0, s>>>(a.ctrl, n, a.passes, a.status);
  record_phase(a.events, kPhasePlan, true, s);
  ++*launches;
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;

  SortBufs bufs;
  bufs.keys[kSelInput] = a.values;
  bufs.rids[kSelInput] = nullptr;
  bufs.keys[kSelA] = a.buf_keys[0];
  bufs.rids[kSelA] = a.buf_rids[0];
  bufs.keys[kSelB] = a.buf_keys[1];
  bufs.rids[kSelB] = a.buf_rids[1];
  const uint64_t tiles = ceil_div(n, kSortTile);
  const size_t smem = sizeof(SortPassSmem);
  err = cudaFuncSetAttribute(k_onesweep_pass, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
  if (err != cudaSuccess) return err;
  for (int p = 0; p < kDigits; ++p) {
    if (p >= a.passes) {  // not launched: empty span keeps every event valid
      record_phase(a.events, kPhasePass0 + p, false, s);
      record_phase(a.events, kPhasePass0 + p, true, s);
      continue;
    }
    err = cudaMemsetAsync(a.lb_sort, 0, tiles * kRadix * sizeof(uint32_t), s);
    if (err != cudaSuccess) return err;
    record_phase(a.events, kPhasePass0 + p, false, s);
    k_onesweep_pass<<<(unsigned)tiles, kSortThreads, smem, s>>>(
        bufs, a.buf_keys[0], a.buf_rids[0], a.buf_keys[1], a.buf_rids[1], n, p, a.ctrl,
        a.lb_sort, a.status);
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
  const uint32_t* __restrict__ k = bufs.keys[sel];
  const uint32_t* __restrict__ r = bufs.rids[sel];
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
