// wah_pipe.cu -- pipelined host-buffer builds (wah_pipe_*).
//
// The reference moves each column host -> device, runs the phases and reads
// the index back, one column at a time, with a host synchronisation per step
// (global_argument ... mem_ref::data, src/phases.cpp:720-1088; per batch in
// src/gpu.cpp:194-259 with --jobs in flight).  Here a pipe owns `depth`
// slots, each with its own stream and device buffers, and one completion
// thread.  A submit enqueues on its slot's stream the copy of the values in,
// the build, and a 16-byte copy of the counters to pinned memory, then hands
// the slot to the completion thread and returns.  The completion thread waits
// for each build in submit order, reads K and L and enqueues copies of
// exactly keys[K], offsets[K] and index[L] (and the counters) to the
// caller's host buffers on the copy engines.  Consecutive submits therefore
// overlap: one column's values come in while another is sorted and a third
// one's index goes out, and no SM is spent on host copies.
#include <algorithm>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "wah_common.cuh"

namespace wah {
namespace {

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t built = nullptr;  // build + counter copy done
  cudaEvent_t done = nullptr;   // outputs in host memory
  uint32_t* d_values = nullptr;
  uint32_t* d_keys = nullptr;
  uint32_t* d_offsets = nullptr;
  uint32_t* d_index = nullptr;
  wah_counts* d_counts = nullptr;
  wah_counts* h_cnt = nullptr;  // pinned copy of the counters
  void* d_ws = nullptr;
  // the submit in this slot
  uint64_t ticket = 0;
  bool busy = false;     // submitted, not yet waited for
  bool issued = false;   // output copies enqueued by the completion thread
  int error = WAH_OK;
  uint32_t* h_keys = nullptr;
  uint32_t* h_offsets = nullptr;
  uint32_t* h_index = nullptr;
  wah_counts* h_counts = nullptr;
};

int cuda_rc(cudaError_t e) {
  if (e == cudaSuccess) return WAH_OK;
  return e == cudaErrorMemoryAllocation ? WAH_ENOMEM : WAH_ECUDA;
}

}  // namespace
}  // namespace wah

using namespace wah;

struct wah_pipe {
  uint64_t max_n = 0;
  uint32_t bound = 0;
  uint64_t keys_cap = 0, index_cap = 0;
  size_t ws_bytes = 0;
  int device = 0;
  uint64_t next_ticket = 1;
  std::vector<Slot> slots;
  // completion thread
  std::mutex mu;
  std::condition_variable cv;
  std::deque<size_t> queue;  // slots whose outputs still need copying, in order
  bool stop = false;
  std::thread worker;

  void run() {
    cudaSetDevice(device);
    while (true) {
      size_t i;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return stop || !queue.empty(); });
        if (queue.empty()) return;  // stop requested and nothing left
        i = queue.front();
        queue.pop_front();
      }
      Slot& s = slots[i];
      int err = cuda_rc(cudaEventSynchronize(s.built));
      if (err == WAH_OK) {
        const wah_counts c = *s.h_cnt;
        cudaError_t e = cudaSuccess;
        if (c.status == WAH_OK) {
          const uint64_t K = std::min<uint64_t>(c.keycnt, keys_cap);
          const uint64_t L = std::min<uint64_t>(c.index_len, index_cap);
          if (L) e = cudaMemcpyAsync(s.h_index, s.d_index, L * 4, cudaMemcpyDeviceToHost, s.stream);
          if (e == cudaSuccess && K)
            e = cudaMemcpyAsync(s.h_keys, s.d_keys, K * 4, cudaMemcpyDeviceToHost, s.stream);
          if (e == cudaSuccess && K)
            e = cudaMemcpyAsync(s.h_offsets, s.d_offsets, K * 4, cudaMemcpyDeviceToHost, s.stream);
        }
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(s.h_counts, s.d_counts, sizeof(wah_counts), cudaMemcpyDeviceToHost,
                              s.stream);
        if (e == cudaSuccess) e = cudaEventRecord(s.done, s.stream);
        err = cuda_rc(e);
      }
      {
        std::lock_guard<std::mutex> lk(mu);
        s.error = err;
        s.issued = true;
      }
      cv.notify_all();
    }
  }

  // Wait until slot i's outputs are in host memory; frees the slot.
  int finish(size_t i) {
    Slot& s = slots[i];
    {
      std::unique_lock<std::mutex> lk(mu);
      cv.wait(lk, [&] { return s.issued; });
    }
    int rc = s.error;
    if (rc == WAH_OK) rc = cuda_rc(cudaEventSynchronize(s.done));
    s.busy = false;
    return rc;
  }
};

extern "C" {

void wah_pipe_destroy(wah_pipe* p) {
  if (!p) return;
  if (p->worker.joinable()) {
    {
      std::lock_guard<std::mutex> lk(p->mu);
      p->stop = true;
    }
    p->cv.notify_all();
    p->worker.join();
  }
  for (Slot& s : p->slots) {
    if (s.stream) cudaStreamSynchronize(s.stream);
    cudaFree(s.d_values);
    cudaFree(s.d_keys);
    cudaFree(s.d_offsets);
    cudaFree(s.d_index);
    cudaFree(s.d_counts);
    cudaFree(s.d_ws);
    if (s.h_cnt) cudaFreeHost(s.h_cnt);
    if (s.built) cudaEventDestroy(s.built);
    if (s.done) cudaEventDestroy(s.done);
    if (s.stream) cudaStreamDestroy(s.stream);
  }
  delete p;
}

int wah_pipe_create(uint64_t max_n, uint32_t bound, uint32_t depth, wah_pipe** out) {
  if (!out || depth == 0 || depth > 8) return WAH_EINVAL;
  *out = nullptr;
  if (max_n >= WAH_MAX_ROWS) return WAH_ERANGE;
  wah_pipe* p = new (std::nothrow) wah_pipe;
  if (!p) return WAH_ENOMEM;
  p->max_n = std::max<uint64_t>(max_n, 1);
  p->bound = bound;
  wah_output_caps(p->max_n, bound, &p->keys_cap, &p->index_cap);
  p->ws_bytes = wah_workspace_bytes(p->max_n, bound);
  cudaGetDevice(&p->device);
  p->slots.resize(depth);
  cudaError_t e = cudaSuccess;
  for (Slot& s : p->slots) {
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.built, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&s.d_values, p->max_n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&s.d_keys, p->keys_cap * 4);
    if (e == cudaSuccess) e = cudaMalloc(&s.d_offsets, p->keys_cap * 4);
    if (e == cudaSuccess) e = cudaMalloc(&s.d_index, p->index_cap * 4);
    if (e == cudaSuccess) e = cudaMalloc(&s.d_counts, sizeof(wah_counts));
    if (e == cudaSuccess) e = cudaMallocHost(&s.h_cnt, sizeof(wah_counts));
    if (e == cudaSuccess) e = cudaMalloc(&s.d_ws, p->ws_bytes);
  }
  if (e != cudaSuccess) {
    wah_pipe_destroy(p);
    return cuda_rc(e);
  }
  p->worker = std::thread([p] { p->run(); });
  *out = p;
  return WAH_OK;
}

int wah_pipe_wait(wah_pipe* p, uint64_t ticket) {
  if (!p) return WAH_EINVAL;
  for (size_t i = 0; i < p->slots.size(); ++i)
    if (p->slots[i].busy && p->slots[i].ticket == ticket) return p->finish(i);
  return WAH_OK;  // already waited for (or never submitted)
}

int wah_pipe_submit(wah_pipe* p, const uint32_t* h_values, uint64_t n, uint32_t* h_keys,
                    uint32_t* h_offsets, uint32_t* h_index, wah_counts* h_counts,
                    uint64_t* ticket) {
  if (!p || !h_counts) return WAH_EINVAL;
  if (n > p->max_n) return WAH_ERANGE;
  if (n > 0 && (!h_values || !h_keys || !h_offsets || !h_index)) return WAH_EINVAL;
  // slots are used round robin; the oldest submit's slot is reused
  const size_t i = (p->next_ticket - 1) % p->slots.size();
  Slot& s = p->slots[i];
  if (s.busy) {
    const int rc = p->finish(i);
    if (rc != WAH_OK) return rc;
  }
  cudaError_t e = cudaSuccess;
  if (n > 0) e = cudaMemcpyAsync(s.d_values, h_values, n * 4, cudaMemcpyHostToDevice, s.stream);
  if (e != cudaSuccess) return cuda_rc(e);
  const int rc = wah_build(s.d_values, n, p->bound, s.d_keys, s.d_offsets, s.d_index,
                           s.d_counts, s.d_ws, p->ws_bytes, s.stream);
  if (rc != WAH_OK) return rc;
  e = cudaMemcpyAsync(s.h_cnt, s.d_counts, sizeof(wah_counts), cudaMemcpyDeviceToHost, s.stream);
  if (e == cudaSuccess) e = cudaEventRecord(s.built, s.stream);
  if (e != cudaSuccess) return cuda_rc(e);
  s.ticket = p->next_ticket++;
  s.h_keys = h_keys;
  s.h_offsets = h_offsets;
  s.h_index = h_index;
  s.h_counts = h_counts;
  {
    std::lock_guard<std::mutex> lk(p->mu);
    s.busy = true;
    s.issued = false;
    s.error = WAH_OK;
    p->queue.push_back(i);
  }
  p->cv.notify_all();
  if (ticket) *ticket = s.ticket;
  return WAH_OK;
}

}  // extern "C"
