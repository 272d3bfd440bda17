// wah_serve.cu -- continuous-batching index server (wah_server_*).
//
// The reference's `gpu` program keeps up to --jobs batches in flight through
// an indexer actor and merges per-batch results in a merger actor
// (src/gpu.cpp:103-261).  Here a server takes index-build requests (a host
// column each, with its arrival time), and a scheduler thread:
//   - admits arrived requests in arrival order while their device memory
//     (values, outputs, their share of a batch workspace) fits the budget of
//     one device arena,
//   - forms a batch of everything admitted and runs it with the batched
//     kernels (wah_batch.cu) on one of `streams` batch slots, so a batch's
//     upload overlaps another batch's kernels,
//   - when a batch finishes, records each request's completion time, frees
//     the batch workspace and the uploaded values, and keeps the outputs
//     (keys, offsets, index) resident on the device until the request is
//     released.
// In plain mode every request is built alone with wah_build, one at a time:
// the one-launch-sequence-per-request baseline.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "wah_common.cuh"

using namespace wah;

namespace {

using Clock = std::chrono::steady_clock;

inline double now_s() {
  return std::chrono::duration<double>(Clock::now().time_since_epoch()).count();
}

constexpr size_t kArenaAlign = 256;
inline size_t arena_round(size_t x) { return (x + kArenaAlign - 1) / kArenaAlign * kArenaAlign; }

// First-fit allocator over one device allocation (offsets), coalescing frees.
class Arena {
 public:
  void init(size_t size) {
    free_.clear();
    free_[0] = size;
    used_ = 0;
  }
  // Returns SIZE_MAX when nothing fits.
  size_t alloc(size_t bytes) {
    bytes = arena_round(std::max<size_t>(bytes, 1));
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        const size_t off = it->first, rest = it->second - bytes;
        free_.erase(it);
        if (rest) free_[off + bytes] = rest;
        used_ += bytes;
        return off;
      }
    }
    return SIZE_MAX;
  }
  void release(size_t off, size_t bytes) {
    if (bytes == 0) return;
    bytes = arena_round(bytes);
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  size_t used() const { return used_; }

 private:
  std::map<size_t, size_t> free_;
  size_t used_ = 0;
};

struct Req {
  uint64_t id = 0;
  const uint32_t* h_values = nullptr;
  uint64_t n = 0;
  uint32_t bound = 0;
  double arrival = 0, admitted = 0, done = 0;
  int state = 0;  // 0 waiting, 1 running, 2 done, 3 failed
  int status = WAH_OK;
  // arena blocks (offset, bytes)
  size_t in_off = 0, in_bytes = 0, out_off = 0, out_bytes = 0;
  uint64_t keys_cap = 0, index_cap = 0;
  wah_counts counts{};
};

struct BatchSlot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  bool busy = false;
  std::vector<uint64_t> reqs;
  size_t ws_off = 0, ws_bytes = 0;
  // pinned staging (grown as needed; reused)
  ColumnView* h_cols = nullptr;
  size_t h_cols_cap = 0;
  unsigned char* h_tables = nullptr;  // ranges + spans
  size_t h_tables_cap = 0;
  wah_counts* h_counts = nullptr;
  size_t h_counts_cap = 0;
  wah_counts* d_counts_gather = nullptr;  // inside the batch workspace
};

// Gathers each column's counters into one array for a single copy back.
__global__ void k_gather_counts(const ColumnView* __restrict__ cols, uint32_t ncols,
                                wah_counts* __restrict__ out) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncols) out[c] = *cols[c].counts;
}

template <class T>
bool grow_pinned(T** p, size_t* cap, size_t want) {
  if (*cap >= want) return true;
  if (*p) cudaFreeHost(*p);
  *p = nullptr;
  *cap = 0;
  const size_t n = std::max<size_t>(want, 2 * want);
  if (cudaMallocHost(reinterpret_cast<void**>(p), n * sizeof(T)) != cudaSuccess) return false;
  *cap = n;
  return true;
}

}  // namespace

struct wah_server {
  int device = 0;
  int mode = 0;  // 0 continuous batching, 1 plain
  int tuning = 0;  // tile shapes of its builds, 0: the process default
  uint32_t max_batch = 1;
  unsigned char* dev = nullptr;
  size_t budget = 0;
  Arena arena;
  std::vector<BatchSlot> slots;
  std::mutex mu;
  std::condition_variable cv;       // scheduler wake-ups
  std::condition_variable done_cv;  // completions
  std::unordered_map<uint64_t, Req> reqs;
  std::deque<uint64_t> waiting;  // arrival order
  // set by an admission pass that stopped because the arena had no room for
  // the first arrived request (not because nothing had arrived yet)
  bool mem_blocked = false;
  uint64_t next_id = 1;
  bool stop = false;
  std::thread worker;
  // plain mode: one workspace for the largest request seen so far
  size_t plain_ws_off = SIZE_MAX, plain_ws_bytes = 0;
  uint64_t completed = 0, rows_completed = 0;

  // Device footprint a request keeps until released (values until its batch
  // ends): values, outputs, and its share of a batch workspace.
  static void sizes(uint64_t n, uint32_t bound, size_t* in_b, size_t* out_b, uint64_t* kc,
                    uint64_t* ic) {
    wah_output_caps(std::max<uint64_t>(n, 1), bound, kc, ic);
    *in_b = arena_round(std::max<uint64_t>(n, 1) * 4);
    *out_b = arena_round(*kc * 4) * 2 + arena_round(*ic * 4) + arena_round(sizeof(wah_counts));
  }

  void fail_locked(Req& r, int st) {
    r.state = 3;
    r.status = st;
    r.done = now_s();
    done_cv.notify_all();
  }

  // Completion of finished batches.
  void reap() {
    for (BatchSlot& b : slots) {
      if (!b.busy) continue;
      const cudaError_t q = cudaEventQuery(b.done);
      if (q == cudaErrorNotReady) continue;
      const double t = now_s();
      std::lock_guard<std::mutex> lk(mu);
      for (size_t i = 0; i < b.reqs.size(); ++i) {
        Req& r = reqs[b.reqs[i]];
        r.counts = b.h_counts[i];
        r.done = t;
        r.status = q == cudaSuccess ? (int)r.counts.status : cuda_status(q);
        r.state = r.status == WAH_OK ? 2 : 3;
        arena.release(r.in_off, r.in_bytes);  // values are no longer needed
        r.in_bytes = 0;
        ++completed;
        rows_completed += r.n;
      }
      if (b.ws_bytes) arena.release(b.ws_off, b.ws_bytes);
      b.ws_bytes = 0;
      b.reqs.clear();
      b.busy = false;
      done_cv.notify_all();
    }
  }

  // Admit arrived requests (FIFO) into a new batch on a free slot.
  bool launch_batch(BatchSlot& b) {
    std::vector<uint64_t> ids;
    std::vector<Req*> rp;  // element pointers stay valid while the map grows
    std::vector<uint64_t> ns;
    std::vector<uint32_t> bounds;
    BatchLayout L;
    {
      std::lock_guard<std::mutex> lk(mu);
      const double t = now_s();
      while (!waiting.empty() && ids.size() < max_batch) {
        Req& r = reqs[waiting.front()];
        if (r.arrival > t) break;  // not arrived yet
        size_t in_b, out_b;
        sizes(r.n, r.bound, &in_b, &out_b, &r.keys_cap, &r.index_cap);
        const size_t in_off = arena.alloc(in_b);
        if (in_off == SIZE_MAX) {
          mem_blocked = ids.empty();
          break;
        }
        const size_t out_off = arena.alloc(out_b);
        if (out_off == SIZE_MAX) {
          arena.release(in_off, in_b);
          mem_blocked = ids.empty();
          break;
        }
        r.in_off = in_off;
        r.in_bytes = in_b;
        r.out_off = out_off;
        r.out_bytes = out_b;
        ids.push_back(r.id);
        ns.push_back(r.n);
        bounds.push_back(r.bound);
        waiting.pop_front();
      }
      if (ids.empty()) return false;
      // workspace of the batch (plus the counters gather array); give back
      // the newest admissions until it fits
      while (true) {
        plan_batch_layout(ns.data(), bounds.data(), (uint32_t)ns.size(), sm_count_current(), &L);
        const size_t ws = L.bytes + arena_round(sizeof(wah_counts) * ns.size());
        const size_t off = arena.alloc(ws);
        if (off != SIZE_MAX) {
          b.ws_off = off;
          b.ws_bytes = ws;
          break;
        }
        Req& r = reqs[ids.back()];
        arena.release(r.in_off, r.in_bytes);
        arena.release(r.out_off, r.out_bytes);
        r.in_bytes = r.out_bytes = 0;
        waiting.push_front(r.id);
        ids.pop_back();
        ns.pop_back();
        bounds.pop_back();
        if (ids.empty()) {
          mem_blocked = true;
          return false;
        }
      }
      for (uint64_t id : ids) {
        Req& r = reqs[id];
        r.state = 1;
        r.admitted = now_s();
        rp.push_back(&r);
      }
    }
    const uint32_t nc = (uint32_t)ids.size();
    unsigned char* ws = dev + b.ws_off;
    bool ok = grow_pinned(&b.h_cols, &b.h_cols_cap, nc) &&
              grow_pinned(&b.h_counts, &b.h_counts_cap, nc) &&
              grow_pinned(&b.h_tables, &b.h_tables_cap,
                          sizeof(RangeView) * L.nranges + L.spans.size() * 4);
    cudaError_t e = ok ? cudaSuccess : cudaErrorMemoryAllocation;
    std::vector<wah_column> cols(nc);
    for (uint32_t c = 0; c < nc && e == cudaSuccess; ++c) {
      Req& r = *rp[c];
      unsigned char* out = dev + r.out_off;
      wah_column& x = cols[c];
      x.values = reinterpret_cast<const uint32_t*>(dev + r.in_off);
      x.n = r.n;
      x.bound = r.bound;
      x.reserved = 0;
      x.keys = reinterpret_cast<uint32_t*>(out);
      x.offsets = reinterpret_cast<uint32_t*>(out + arena_round(r.keys_cap * 4));
      x.index = reinterpret_cast<uint32_t*>(out + 2 * arena_round(r.keys_cap * 4));
      x.counts = reinterpret_cast<wah_counts*>(out + 2 * arena_round(r.keys_cap * 4) +
                                               arena_round(r.index_cap * 4));
      if (r.n) e = cudaMemcpyAsync(const_cast<uint32_t*>(x.values), r.h_values, r.n * 4,
                                   cudaMemcpyHostToDevice, b.stream);
    }
    if (e == cudaSuccess) {
      fill_batch_columns(L, ws, cols.data(), b.h_cols);
      std::memcpy(b.h_tables, L.ranges.data(), sizeof(RangeView) * L.nranges);
      std::memcpy(b.h_tables + sizeof(RangeView) * L.nranges, L.spans.data(), L.spans.size() * 4);
      e = cudaMemcpyAsync(ws + L.o_cols, b.h_cols, sizeof(ColumnView) * nc,
                          cudaMemcpyHostToDevice, b.stream);
    }
    if (e == cudaSuccess && L.nranges)
      e = cudaMemcpyAsync(ws + L.o_ranges, b.h_tables, sizeof(RangeView) * L.nranges,
                          cudaMemcpyHostToDevice, b.stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(ws + L.o_spans, b.h_tables + sizeof(RangeView) * L.nranges,
                          L.spans.size() * 4, cudaMemcpyHostToDevice, b.stream);
    uint32_t launches = 0;
    if (e == cudaSuccess) e = enqueue_batch(L, ws, b.stream, &launches, tuning);
    wah_counts* gather = reinterpret_cast<wah_counts*>(ws + L.bytes);
    if (e == cudaSuccess) {
      k_gather_counts<<<(unsigned)ceil_div(nc, 256), 256, 0, b.stream>>>(
          reinterpret_cast<const ColumnView*>(ws + L.o_cols), nc, gather);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(b.h_counts, gather, sizeof(wah_counts) * nc, cudaMemcpyDeviceToHost,
                          b.stream);
    if (e == cudaSuccess) e = cudaEventRecord(b.done, b.stream);
    b.reqs = ids;
    if (e != cudaSuccess) {
      cudaStreamSynchronize(b.stream);
      std::lock_guard<std::mutex> lk(mu);
      for (uint64_t id : ids) {
        Req& r = reqs[id];
        arena.release(r.in_off, r.in_bytes);
        arena.release(r.out_off, r.out_bytes);
        r.in_bytes = r.out_bytes = 0;
        fail_locked(r, cuda_status(e));
      }
      arena.release(b.ws_off, b.ws_bytes);
      b.ws_bytes = 0;
      b.reqs.clear();
      return false;
    }
    b.busy = true;
    return true;
  }

  // Plain mode: the oldest arrived request alone, through wah_build.
  bool launch_plain(BatchSlot& b) {
    uint64_t id;
    Req* rq = nullptr;
    {
      std::lock_guard<std::mutex> lk(mu);
      if (waiting.empty()) return false;
      Req& r = reqs[waiting.front()];
      if (r.arrival > now_s()) return false;
      size_t in_b, out_b;
      sizes(r.n, r.bound, &in_b, &out_b, &r.keys_cap, &r.index_cap);
      const size_t need_ws = wah_workspace_bytes(std::max<uint64_t>(r.n, 1), r.bound);
      if (need_ws > plain_ws_bytes) {
        if (plain_ws_off != SIZE_MAX) arena.release(plain_ws_off, plain_ws_bytes);
        plain_ws_off = arena.alloc(need_ws);
        plain_ws_bytes = plain_ws_off == SIZE_MAX ? 0 : need_ws;
        if (plain_ws_off == SIZE_MAX) {
          mem_blocked = true;
          return false;
        }
      }
      const size_t in_off = arena.alloc(in_b);
      if (in_off == SIZE_MAX) {
        mem_blocked = true;
        return false;
      }
      const size_t out_off = arena.alloc(out_b);
      if (out_off == SIZE_MAX) {
        arena.release(in_off, in_b);
        mem_blocked = true;
        return false;
      }
      r.in_off = in_off;
      r.in_bytes = in_b;
      r.out_off = out_off;
      r.out_bytes = out_b;
      r.state = 1;
      r.admitted = now_s();
      id = r.id;
      rq = &r;
      waiting.pop_front();
    }
    Req& r = *rq;
    grow_pinned(&b.h_counts, &b.h_counts_cap, 1);
    unsigned char* out = dev + r.out_off;
    uint32_t* keys = reinterpret_cast<uint32_t*>(out);
    uint32_t* offs = reinterpret_cast<uint32_t*>(out + arena_round(r.keys_cap * 4));
    uint32_t* index = reinterpret_cast<uint32_t*>(out + 2 * arena_round(r.keys_cap * 4));
    wah_counts* cnt = reinterpret_cast<wah_counts*>(out + 2 * arena_round(r.keys_cap * 4) +
                                                    arena_round(r.index_cap * 4));
    uint32_t* vals = reinterpret_cast<uint32_t*>(dev + r.in_off);
    cudaError_t e = cudaSuccess;
    if (r.n) e = cudaMemcpyAsync(vals, r.h_values, r.n * 4, cudaMemcpyHostToDevice, b.stream);
    int rc = cuda_status(e);
    if (rc == WAH_OK)
      rc = wah_build_tuned(vals, r.n, r.bound, keys, offs, index, cnt, dev + plain_ws_off,
                           plain_ws_bytes, tuning, b.stream);
    if (rc == WAH_OK)
      rc = cuda_status(cudaMemcpyAsync(b.h_counts, cnt, sizeof(wah_counts),
                                       cudaMemcpyDeviceToHost, b.stream));
    if (rc == WAH_OK) rc = cuda_status(cudaEventRecord(b.done, b.stream));
    b.reqs.assign(1, id);
    b.ws_bytes = 0;
    if (rc != WAH_OK) {
      cudaStreamSynchronize(b.stream);
      std::lock_guard<std::mutex> lk(mu);
      arena.release(r.in_off, r.in_bytes);
      arena.release(r.out_off, r.out_bytes);
      r.in_bytes = r.out_bytes = 0;
      fail_locked(r, rc);
      b.reqs.clear();
      return false;
    }
    b.busy = true;
    return true;
  }

  // A request that arrived but found no room in the arena, with nothing in
  // flight: while completed results the client has not released yet hold
  // arena memory, it waits for their release (a client that reads results
  // more slowly than they complete); when none are held, or no release has
  // come for kStallFailS (a client that waits for this request while it
  // holds the results that block it), it can never be placed: fail it.  Only
  // a pass that stopped for lack of room counts; one that found nothing
  // arrived yet (the front request may arrive just after it) does not.
  static constexpr double kStallFailS = 2.0;
  double blocked_since = -1.0;  // start of the current stall, -1 when none

  void fail_unplaceable() {
    std::lock_guard<std::mutex> lk(mu);
    if (!mem_blocked || waiting.empty()) {
      blocked_since = -1.0;
      return;
    }
    const size_t ws = plain_ws_off == SIZE_MAX ? 0 : arena_round(plain_ws_bytes);
    const size_t resident = arena.used() - std::min(arena.used(), ws);
    const double t = now_s();
    if (resident > 0) {
      if (blocked_since < 0) blocked_since = t;
      if (t - blocked_since < kStallFailS) return;
    }
    blocked_since = -1.0;
    mem_blocked = false;
    Req& r = reqs[waiting.front()];
    waiting.pop_front();
    fail_locked(r, WAH_ENOMEM);
  }

  void run() {
    cudaSetDevice(device);
    while (true) {
      reap();
      {
        std::lock_guard<std::mutex> lk(mu);
        mem_blocked = false;
      }
      bool launched = false, any_busy = false;
      for (BatchSlot& b : slots) {
        if (b.busy) {
          any_busy = true;
          continue;
        }
        launched = mode == 1 ? launch_plain(b) : launch_batch(b);
        if (launched) break;  // one launch per pass, then reap again
      }
      if (!launched && !any_busy) {
        fail_unplaceable();
      } else {
        std::lock_guard<std::mutex> lk(mu);
        blocked_since = -1.0;
      }
      std::unique_lock<std::mutex> lk(mu);
      if (stop && waiting.empty() &&
          std::none_of(slots.begin(), slots.end(), [](const BatchSlot& b) { return b.busy; }))
        return;
      if (!launched) {
        // nothing to start: wait briefly for an arrival, a submit or a finish
        double wait_s = 20e-6;
        if (!waiting.empty()) {
          const double dt = reqs[waiting.front()].arrival - now_s();
          if (dt > 0) wait_s = std::min(std::max(dt, 5e-6), 1e-3);
        }
        cv.wait_for(lk, std::chrono::duration<double>(wait_s));
      }
    }
  }
};

extern "C" {

int wah_server_create(uint64_t budget_bytes, uint32_t max_batch, uint32_t streams, int plain,
                      wah_server** out) {
  return wah_server_create_tuned(budget_bytes, max_batch, streams, plain, 0, out);
}

int wah_server_create_tuned(uint64_t budget_bytes, uint32_t max_batch, uint32_t streams,
                            int plain, int tuning, wah_server** out) {
  if (!out || budget_bytes == 0 || streams == 0 || streams > 8) return WAH_EINVAL;
  *out = nullptr;
  if (tuning != 0 && !valid_tuning(tuning)) return WAH_EINVAL;
  wah_server* s = new (std::nothrow) wah_server;
  if (!s) return WAH_ENOMEM;
  s->tuning = tuning;
  s->mode = plain ? 1 : 0;
  s->max_batch = plain ? 1 : std::max<uint32_t>(max_batch, 1);
  s->budget = arena_round(budget_bytes);
  cudaGetDevice(&s->device);
  cudaError_t e = cudaMalloc(&s->dev, s->budget);
  s->slots.resize(plain ? 1 : streams);
  for (BatchSlot& b : s->slots) {
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    for (BatchSlot& b : s->slots) {
      if (b.done) cudaEventDestroy(b.done);
      if (b.stream) cudaStreamDestroy(b.stream);
    }
    cudaFree(s->dev);
    delete s;
    return cuda_status(e);
  }
  s->arena.init(s->budget);
  s->worker = std::thread([s] { s->run(); });
  *out = s;
  return WAH_OK;
}

int wah_server_submit(wah_server* s, const uint32_t* h_values, uint64_t n, uint32_t bound,
                      double arrival_delay_s, uint64_t* id) {
  if (!s || !id || (n > 0 && !h_values)) return WAH_EINVAL;
  if (n >= WAH_MAX_ROWS) return WAH_ERANGE;
  std::lock_guard<std::mutex> lk(s->mu);
  Req r;
  r.id = s->next_id++;
  r.h_values = h_values;
  r.n = n;
  r.bound = bound;
  r.arrival = now_s() + std::max(arrival_delay_s, 0.0);
  // a request that could never fit the budget alone is refused up front
  size_t in_b, out_b;
  wah_server::sizes(n, bound, &in_b, &out_b, &r.keys_cap, &r.index_cap);
  if (in_b + out_b + wah_workspace_bytes(std::max<uint64_t>(n, 1), bound) + (1u << 20) >
      s->budget)
    return WAH_ENOMEM;
  s->reqs[r.id] = r;
  s->waiting.push_back(r.id);
  *id = r.id;
  s->cv.notify_all();
  return WAH_OK;
}

int wah_server_wait(wah_server* s, uint64_t id, wah_server_result* res) {
  if (!s) return WAH_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return WAH_EINVAL;
  const Req* rp = &it->second;  // stable while other requests come and go
  s->done_cv.wait(lk, [&] { return rp->state >= 2; });
  const Req& r = *rp;
  if (res) {
    std::memset(res, 0, sizeof(*res));
    res->counts = r.counts;
    res->latency_s = r.done - r.arrival;
    res->queue_s = r.admitted - r.arrival;
    if (r.state == 2) {
      unsigned char* out = s->dev + r.out_off;
      res->keys = reinterpret_cast<uint32_t*>(out);
      res->offsets = reinterpret_cast<uint32_t*>(out + arena_round(r.keys_cap * 4));
      res->index = reinterpret_cast<uint32_t*>(out + 2 * arena_round(r.keys_cap * 4));
    }
  }
  return r.status;
}

int wah_server_release(wah_server* s, uint64_t id) {
  if (!s) return WAH_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end() || it->second.state < 2) return WAH_EINVAL;
  if (it->second.out_bytes) s->arena.release(it->second.out_off, it->second.out_bytes);
  s->reqs.erase(it);
  s->blocked_since = -1.0;  // progress: a stalled admission waits afresh
  s->cv.notify_all();
  return WAH_OK;
}

int wah_server_copy_out(wah_server* s, uint64_t id, uint32_t* d_keys, uint32_t* d_offsets,
                        uint32_t* d_index, void* stream) {
  if (!s) return WAH_EINVAL;
  Req r;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end() || it->second.state != 2) return WAH_EINVAL;
    r = it->second;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* out = s->dev + r.out_off;
  const uint64_t K = r.counts.keycnt, L = r.counts.index_len;
  cudaError_t e = cudaSuccess;
  if (K && d_keys) e = cudaMemcpyAsync(d_keys, out, K * 4, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && K && d_offsets)
    e = cudaMemcpyAsync(d_offsets, out + arena_round(r.keys_cap * 4), K * 4,
                        cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && L && d_index)
    e = cudaMemcpyAsync(d_index, out + 2 * arena_round(r.keys_cap * 4), L * 4,
                        cudaMemcpyDeviceToDevice, st);
  return cuda_status(e);
}

uint64_t wah_server_arena_used(wah_server* s) {
  if (!s) return 0;
  std::lock_guard<std::mutex> lk(s->mu);
  return s->arena.used();
}

void wah_server_destroy(wah_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (BatchSlot& b : s->slots) {
    if (b.stream) cudaStreamSynchronize(b.stream);
    if (b.h_cols) cudaFreeHost(b.h_cols);
    if (b.h_tables) cudaFreeHost(b.h_tables);
    if (b.h_counts) cudaFreeHost(b.h_counts);
    if (b.done) cudaEventDestroy(b.done);
    if (b.stream) cudaStreamDestroy(b.stream);
  }
  cudaFree(s->dev);
  delete s;
}

}  // extern "C"
