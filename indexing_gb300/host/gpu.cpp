// gpu -- the reference's batched actor pipeline rebuilt on the GB300 kernels
// (src/gpu.cpp:103-375).
//
//   indexer  cuts the column into batches of --batch-size x --work-groups rows
//            and keeps up to --jobs batches in flight (src/gpu.cpp:179-261);
//   worker   builds each batch on the GPU: every work-group slice of
//            --batch-size rows is indexed as its own column, all slices of a
//            batch in one batched launch (the reference runs one OpenCL
//            work-group per slice, kernel_wah_index, :356-367);
//   merger   joins the slice indexes into the index of the whole column
//            (src/gpu.cpp:103-165).
//
// The reference's merger appends each slice's words to its key's bitmap and
// so loses the zero chunks between slices; this one re-bases every slice on
// its first chunk (wahmerge::slice_merger), so the merged index is the index
// the whole column gets from wah_build / the cpu program, word for word.
// That needs slices that start on a chunk boundary: --batch-size is rounded
// down to a multiple of 31 when the column has more rows than one slice (the
// default 1023 = 33 x 31).
//
// Flags as the reference (-f, -b bound, -d device name, -p print,
// --batch-size, -j/--jobs, -w/--work-groups) plus --output FILE,
// --host-parse (the data file is parsed on the GPU by default) and
// --device-merge (slices are appended to one index on the GPU with
// wah_append, in row order, and the merged index comes back once; the
// merger takes it whole).  Prints the reference's lines ('N' values, maximum
// value, device, -p listing of keys 0..bound, Time: 'X' ms).
//
// As in the reference, the clock starts when the merger is initialised,
// after the worker exists: the column is staged in page-locked memory and the
// worker's device and page-locked buffers are set up before that; batches
// are sent as row spans of the staged column and copied to the device from
// there.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "actors.hpp"
#include "cli.hpp"
#include "merge.hpp"

using namespace wahact;

namespace {

struct init_atom {};
struct index_atom {};
struct work_atom {};
struct done_atom {};
struct add_atom {};
struct quit_atom {};
struct ready_atom {};

constexpr uint32_t kChunk = 31;

uint64_t round4(uint64_t x) { return (x + 3) & ~uint64_t(3); }

// One slice's index, rows [row_start, row_start + n).
struct slice_index {
  uint64_t row_start = 0;
  uint32_t n = 0;
  int status = WAH_OK;
  std::vector<uint32_t> keys, offsets, index;
  // The whole column's index merged on the device: its arrays stay in the
  // page-locked block `hold` (no copy into the vectors above).
  bool whole = false;
  std::shared_ptr<uint32_t> hold;
  const uint32_t *pk = nullptr, *po = nullptr, *pw = nullptr;
  uint32_t kc = 0, wc = 0;
};

// -p listing of keys 0..bound from a (keys, offsets, index) triple
// (src/gpu.cpp:153-158 prints every key up to the bound).
void print_keys_upto(uint32_t bound, const uint32_t* keys, const uint32_t* offsets, uint32_t K,
                     const uint32_t* words, uint32_t L) {
  uint32_t i = 0;
  for (uint64_t key = 0; key <= bound; ++key) {
    while (i < K && keys[i] < key) ++i;
    std::string bits;
    if (i < K && keys[i] == key) {
      const uint32_t end = i + 1 < K ? offsets[i + 1] : L;
      bits = wahcli::decoded_bitmap(words + offsets[i], end - offsets[i]);
    }
    std::printf("%llu\t%s\n", (unsigned long long)key, bits.c_str());
  }
}

// ---------------------------------------------------------------- merger --

struct merger_state {
  bool print_results = false;
  uint32_t bound = 0;
  std::string output;
  std::chrono::steady_clock::time_point start;
  wahmerge::slice_merger index{std::min(16u, std::max(1u, std::thread::hardware_concurrency()))};
  std::map<uint64_t, slice_index> pending;  // slices that arrived early
  slice_index whole;                         // --device-merge: the merged index
  bool have_whole = false;
  int status = WAH_OK;
  int* exit_code = nullptr;
};

behavior merger(actor_ctx<merger_state>& self) {
  auto& s = self.state;
  return {
      handler<init_atom, bool, uint32_t, std::string, int*>(
          [&](init_atom, bool print, uint32_t bound, std::string output, int* exit_code) {
            s.start = std::chrono::steady_clock::now();
            s.print_results = print;
            s.bound = bound;
            s.output = std::move(output);
            s.exit_code = exit_code;
          }),
      handler<add_atom, slice_index>([&](add_atom, slice_index x) {
        if (x.status != WAH_OK) {
          if (s.status == WAH_OK) s.status = x.status;
          return;
        }
        if (x.whole) {  // merged on the device already
          s.whole = std::move(x);
          s.have_whole = true;
          return;
        }
        // slices are merged in row order
        s.pending.emplace(x.row_start, std::move(x));
        while (!s.pending.empty() && s.pending.begin()->first == s.index.rows()) {
          slice_index& y = s.pending.begin()->second;
          if (!s.index.add(y.row_start, y.n, y.keys.data(), y.offsets.data(),
                           static_cast<uint32_t>(y.keys.size()), y.index.data(),
                           static_cast<uint32_t>(y.index.size())) &&
              s.status == WAH_OK)
            s.status = WAH_EINVAL;
          s.pending.erase(s.pending.begin());
        }
      }),
      handler<quit_atom, int>([&](quit_atom, int indexer_status) {
        if (s.status == WAH_OK) s.status = indexer_status;
        const uint64_t ms = wahcli::micros_since(s.start) / 1000;
        if (s.status != WAH_OK) {
          std::fprintf(stderr, "[!!!] %s\n", wah_strerror(s.status));
          *s.exit_code = 1;
          self.quit();
          return;
        }
        if (s.have_whole) {
          const slice_index& x = s.whole;
          if (s.print_results) print_keys_upto(s.bound, x.pk, x.po, x.kc, x.pw, x.wc);
          std::printf("Index has %u elements with %u keys\n", x.wc, x.kc);
          std::printf("Time: '%llu' ms\n", (unsigned long long)ms);
          if (!s.output.empty() && !wahcli::write_result(s.output, x.pk, x.po, x.kc, x.pw, x.wc)) {
            std::fprintf(stderr, "cannot write '%s'\n", s.output.c_str());
            *s.exit_code = 1;
          }
          self.quit();
          return;
        }
        std::vector<uint32_t> keys, offsets, words;
        s.index.finish(&keys, &offsets, &words);
        if (s.print_results) {
          for (uint64_t key = 0; key <= s.bound; ++key) {
            const auto* w = s.index.words(static_cast<uint32_t>(key));
            const std::string bits = w ? wahcli::decoded_bitmap(w->data(), w->size()) : "";
            std::printf("%llu\t%s\n", (unsigned long long)key, bits.c_str());
          }
        }
        std::printf("Index has %zu elements with %zu keys\n", words.size(), keys.size());
        std::printf("Time: '%llu' ms\n", (unsigned long long)ms);
        if (!s.output.empty() && !wahcli::write_result(s.output, keys, offsets, words)) {
          std::fprintf(stderr, "cannot write '%s'\n", s.output.c_str());
          *s.exit_code = 1;
        }
        self.quit();
      }),
  };
}

// ---------------------------------------------------------------- worker --

// Device and pinned buffers for one batch in flight.  Slice c of a batch sits
// at c * stride in every buffer (strides rounded to 16 bytes, as the batched
// build wants 16-byte aligned columns).
struct job_slot {
  void* stream = nullptr;
  uint32_t *d_values = nullptr, *d_keys = nullptr, *d_offsets = nullptr, *d_index = nullptr;
  wah_counts* d_counts = nullptr;
  uint32_t *h_keys = nullptr, *h_offsets = nullptr, *h_index = nullptr;
  wah_counts* h_counts = nullptr;
  void* ws = nullptr;  // one slice per batch: wah_build's workspace
  wah_batch* batch = nullptr;
  uint32_t batch_cols = 0;   // shape the batch plan is for
  uint32_t batch_last = 0;
  // the batch in flight
  uint64_t row_start = 0;
  uint32_t ncols = 0;
  std::vector<uint32_t> ns;
  int status = WAH_OK;
  bool busy = false;
};

struct worker_state {
  int device = 0;
  uint32_t wg_size = 0, wg_num = 0, bound = 0;
  uint64_t v_stride = 0, k_stride = 0, i_stride = 0;
  size_t ws_bytes = 0;
  const uint32_t* input = nullptr;  // the column, page-locked
  uint64_t total_rows = 0;
  // --device-merge: the index of rows [0, acc_rows) in acc_*[acc_cur]
  bool device_merge = false;
  uint32_t *acc_k[2] = {nullptr, nullptr}, *acc_o[2] = {nullptr, nullptr};
  uint32_t* acc_w[2] = {nullptr, nullptr};
  wah_counts* acc_counts = nullptr;    // device
  wah_counts* h_acc_counts = nullptr;  // page-locked
  uint64_t acc_rows = 0, acc_keys_cap = 0, acc_index_cap = 0;
  uint32_t acc_K = 0, acc_L = 0;
  int acc_cur = 0;
  void* app_ws = nullptr;
  size_t app_ws_bytes = 0;
  std::shared_ptr<uint32_t> out_hold;  // page-locked keys | offsets | words
  std::vector<job_slot> slots;
  actor reply_to;
  // completion thread: waits for batches in submission order
  std::mutex mu;
  std::condition_variable cv;
  std::deque<size_t> queue;
  bool stop = false;
  std::thread completer;
  actor_system* sys = nullptr;
  actor self;
  int setup_status = WAH_OK;

  int setup(uint32_t jobs) {
    uint64_t keys_cap = 0, index_cap = 0;
    wah_output_caps(wg_size, bound, &keys_cap, &index_cap);
    v_stride = round4(wg_size);
    k_stride = round4(keys_cap);
    i_stride = round4(index_cap);
    ws_bytes = wg_num == 1 ? wah_workspace_bytes(wg_size, bound) : 0;
    slots.resize(jobs);
    int rc = WAH_OK;
    auto dev = [&](size_t bytes, auto** out) {
      void* p = nullptr;
      if (rc == WAH_OK) rc = wah_dev_alloc(bytes, &p);
      *out = static_cast<std::remove_reference_t<decltype(*out)>>(p);
    };
    auto host = [&](size_t bytes, auto** out) {
      void* p = nullptr;
      if (rc == WAH_OK) rc = wah_host_alloc(bytes, &p);
      *out = static_cast<std::remove_reference_t<decltype(*out)>>(p);
    };
    for (job_slot& j : slots) {
      if (rc == WAH_OK) rc = wah_stream_create(&j.stream);
      dev(v_stride * wg_num * 4, &j.d_values);
      dev(k_stride * wg_num * 4, &j.d_keys);
      dev(k_stride * wg_num * 4, &j.d_offsets);
      dev(i_stride * wg_num * 4, &j.d_index);
      dev(sizeof(wah_counts) * wg_num, &j.d_counts);
      if (!device_merge) {  // slices come back to the host one by one
        host(k_stride * wg_num * 4, &j.h_keys);
        host(k_stride * wg_num * 4, &j.h_offsets);
        host(i_stride * wg_num * 4, &j.h_index);
      }
      host(sizeof(wah_counts) * wg_num, &j.h_counts);
      if (wg_num == 1 && rc == WAH_OK) rc = wah_dev_alloc(ws_bytes, &j.ws);
    }
    if (device_merge && rc == WAH_OK) {
      // wah_append checks its outputs against ka + kb keys and la + lb + kb
      // words (one gap word per key of the slice): the merged index's own
      // bounds plus one slice's keys
      wah_output_caps(std::max<uint64_t>(total_rows, 1), bound, &acc_keys_cap, &acc_index_cap);
      acc_keys_cap += k_stride;
      acc_index_cap = 2 * std::max<uint64_t>(total_rows, 1) + k_stride;
      for (int b = 0; b < 2; ++b) {
        dev(acc_keys_cap * 4, &acc_k[b]);
        dev(acc_keys_cap * 4, &acc_o[b]);
        dev(acc_index_cap * 4, &acc_w[b]);
      }
      dev(sizeof(wah_counts), &acc_counts);
      host(sizeof(wah_counts), &h_acc_counts);
      app_ws_bytes = wah_append_workspace_bytes(static_cast<uint32_t>(acc_keys_cap),
                                                static_cast<uint32_t>(k_stride));
      if (rc == WAH_OK) rc = wah_dev_alloc(app_ws_bytes, &app_ws);
      uint32_t* out = nullptr;
      host((2 * acc_keys_cap + acc_index_cap) * 4, &out);
      if (out) out_hold = std::shared_ptr<uint32_t>(out, [](uint32_t* q) { wah_host_free(q); });
    }
    return rc;
  }

  // Appends slice c of batch j to the merged index (device, row order).
  int append_slice(job_slot& j, uint32_t c, const wah_counts& cb) {
    const int nxt = acc_cur ^ 1;
    int rc = wah_append(acc_k[acc_cur], acc_o[acc_cur], acc_w[acc_cur], acc_K, acc_L, acc_rows,
                        j.d_keys + c * k_stride, j.d_offsets + c * k_stride,
                        j.d_index + c * i_stride, cb.keycnt, cb.index_len, acc_k[nxt],
                        acc_o[nxt], acc_w[nxt], acc_keys_cap, acc_index_cap, acc_counts, app_ws,
                        app_ws_bytes, j.stream);
    if (rc == WAH_OK) rc = wah_copy(h_acc_counts, acc_counts, sizeof(wah_counts), j.stream);
    if (rc == WAH_OK) rc = wah_stream_sync(j.stream);
    if (rc == WAH_OK) rc = static_cast<int>(h_acc_counts->status);
    if (rc == WAH_OK) {
      acc_K = h_acc_counts->keycnt;
      acc_L = h_acc_counts->index_len;
      acc_cur = nxt;
      acc_rows += j.ns[c];
    }
    return rc;
  }

  // The merged index to page-locked memory, handed on without a copy.
  int deliver(void* stream, slice_index* x) {
    uint32_t* k = out_hold.get();
    uint32_t* o = k + acc_keys_cap;
    uint32_t* w = o + acc_keys_cap;
    int rc = WAH_OK;
    if (acc_K) rc = wah_copy(k, acc_k[acc_cur], uint64_t(acc_K) * 4, stream);
    if (rc == WAH_OK && acc_K) rc = wah_copy(o, acc_o[acc_cur], uint64_t(acc_K) * 4, stream);
    if (rc == WAH_OK && acc_L) rc = wah_copy(w, acc_w[acc_cur], uint64_t(acc_L) * 4, stream);
    if (rc == WAH_OK) rc = wah_stream_sync(stream);
    x->row_start = 0;
    x->n = static_cast<uint32_t>(acc_rows);
    x->status = rc;
    x->whole = true;
    x->hold = out_hold;
    x->pk = k;
    x->po = o;
    x->pw = w;
    x->kc = acc_K;
    x->wc = acc_L;
    return rc;
  }

  void teardown() {
    if (completer.joinable()) {
      {
        std::lock_guard<std::mutex> lk(mu);
        stop = true;
      }
      cv.notify_all();
      completer.join();
    }
    for (job_slot& j : slots) {
      if (j.stream) wah_stream_sync(j.stream);
      for (void* p : {static_cast<void*>(j.d_values), static_cast<void*>(j.d_keys),
                      static_cast<void*>(j.d_offsets), static_cast<void*>(j.d_index),
                      static_cast<void*>(j.d_counts), j.ws})
        if (p) wah_dev_free(p);
      for (void* p : {static_cast<void*>(j.h_keys),
                      static_cast<void*>(j.h_offsets), static_cast<void*>(j.h_index),
                      static_cast<void*>(j.h_counts)})
        if (p) wah_host_free(p);
      if (j.batch) wah_batch_destroy(j.batch);
      if (j.stream) wah_stream_destroy(j.stream);
    }
    for (int b = 0; b < 2; ++b)
      for (void* p : {static_cast<void*>(acc_k[b]), static_cast<void*>(acc_o[b]),
                      static_cast<void*>(acc_w[b])})
        if (p) wah_dev_free(p);
    if (acc_counts) wah_dev_free(acc_counts);
    if (app_ws) wah_dev_free(app_ws);
    if (h_acc_counts) wah_host_free(h_acc_counts);
    out_hold.reset();  // freed when the merger lets go of it too
    slots.clear();
  }

  // Enqueues one batch: copy in (from the page-locked column), build every
  // slice, copy the results out.
  int launch(job_slot& j) {
    const uint32_t ncols = j.ncols;
    int rc = WAH_OK;
    for (uint32_t c = 0; c < ncols && rc == WAH_OK; ++c)
      rc = wah_copy(j.d_values + c * v_stride, input + j.row_start + uint64_t(c) * wg_size,
                    uint64_t(j.ns[c]) * 4, j.stream);
    if (rc != WAH_OK) return rc;
    if (wg_num == 1) {
      rc = wah_build(j.d_values, j.ns[0], bound, j.d_keys, j.d_offsets, j.d_index, j.d_counts,
                     j.ws, ws_bytes, j.stream);
    } else {
      const uint32_t last = j.ns[ncols - 1];
      if (!j.batch || j.batch_cols != ncols || j.batch_last != last) {
        if (j.batch) {
          wah_stream_sync(j.stream);
          wah_batch_destroy(j.batch);
          j.batch = nullptr;
        }
        std::vector<uint64_t> ns(j.ns.begin(), j.ns.end());
        std::vector<uint32_t> bounds(ncols, bound);
        rc = wah_batch_create(ns.data(), bounds.data(), ncols, &j.batch);
        if (rc != WAH_OK) return rc;
        j.batch_cols = ncols;
        j.batch_last = last;
      }
      std::vector<wah_column> cols(ncols);
      for (uint32_t c = 0; c < ncols; ++c) {
        cols[c].values = j.d_values + c * v_stride;
        cols[c].n = j.ns[c];
        cols[c].bound = bound;
        cols[c].reserved = 0;
        cols[c].keys = j.d_keys + c * k_stride;
        cols[c].offsets = j.d_offsets + c * k_stride;
        cols[c].index = j.d_index + c * i_stride;
        cols[c].counts = j.d_counts + c;
      }
      rc = wah_batch_set_columns(j.batch, cols.data(), j.stream);
      if (rc == WAH_OK) rc = wah_batch_build(j.batch, j.stream);
    }
    if (rc != WAH_OK) return rc;
    // one slice: its sizes are read first and exactly K, L words copied
    // (by the completion thread); several: whole capacity regions now
    rc = wah_copy(j.h_counts, j.d_counts, sizeof(wah_counts) * ncols, j.stream);
    if (rc == WAH_OK && ncols > 1 && !device_merge) {
      const uint64_t kw = uint64_t(ncols - 1) * k_stride + std::min<uint64_t>(k_stride, j.ns[ncols - 1]);
      const uint64_t iw = uint64_t(ncols - 1) * i_stride + 2ull * j.ns[ncols - 1];
      rc = wah_copy(j.h_keys, j.d_keys, kw * 4, j.stream);
      if (rc == WAH_OK) rc = wah_copy(j.h_offsets, j.d_offsets, kw * 4, j.stream);
      if (rc == WAH_OK) rc = wah_copy(j.h_index, j.d_index, iw * 4, j.stream);
    }
    return rc;
  }

  void complete_loop() {
    wah_device_select(device);
    while (true) {
      size_t i;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return stop || !queue.empty(); });
        if (queue.empty()) return;
        i = queue.front();
        queue.pop_front();
      }
      job_slot& j = slots[i];
      int rc = j.status;
      if (rc == WAH_OK) rc = wah_stream_sync(j.stream);
      if (device_merge) {
        // batches complete in submission order, which is row order
        std::vector<slice_index> out;
        for (uint32_t c = 0; c < j.ncols && rc == WAH_OK; ++c) {
          rc = static_cast<int>(j.h_counts[c].status);
          if (rc == WAH_OK) rc = append_slice(j, c, j.h_counts[c]);
        }
        if (rc != WAH_OK) {
          out.resize(1);
          out[0].status = rc;
        } else if (acc_rows == total_rows) {
          out.resize(1);
          deliver(j.stream, &out[0]);
        }
        uint64_t processed = 0;
        for (uint32_t c = 0; c < j.ncols; ++c) processed += j.ns[c];
        {
          std::lock_guard<std::mutex> lk(mu);
          j.busy = false;
        }
        sys->send_from(self, reply_to, done_atom{}, processed, std::move(out));
        continue;
      }
      if (rc == WAH_OK && j.ncols == 1) {
        const wah_counts c = j.h_counts[0];
        if (c.status == WAH_OK) {
          if (c.index_len) rc = wah_copy(j.h_index, j.d_index, uint64_t(c.index_len) * 4, j.stream);
          if (rc == WAH_OK && c.keycnt)
            rc = wah_copy(j.h_keys, j.d_keys, uint64_t(c.keycnt) * 4, j.stream);
          if (rc == WAH_OK && c.keycnt)
            rc = wah_copy(j.h_offsets, j.d_offsets, uint64_t(c.keycnt) * 4, j.stream);
          if (rc == WAH_OK) rc = wah_stream_sync(j.stream);
        }
      }
      std::vector<slice_index> out(j.ncols);
      uint64_t row = j.row_start;
      for (uint32_t c = 0; c < j.ncols; ++c) {
        slice_index& x = out[c];
        x.row_start = row;
        x.n = j.ns[c];
        row += j.ns[c];
        const wah_counts cnt = j.h_counts[c];
        x.status = rc != WAH_OK ? rc : static_cast<int>(cnt.status);
        if (x.status != WAH_OK) continue;
        const uint32_t* k = j.h_keys + c * k_stride;
        const uint32_t* o = j.h_offsets + c * k_stride;
        const uint32_t* w = j.h_index + c * i_stride;
        x.keys.assign(k, k + cnt.keycnt);
        x.offsets.assign(o, o + cnt.keycnt);
        x.index.assign(w, w + cnt.index_len);
      }
      const uint64_t processed = row - j.row_start;
      {
        std::lock_guard<std::mutex> lk(mu);
        j.busy = false;  // free before replying: the reply may bring the next batch
      }
      sys->send_from(self, reply_to, done_atom{}, processed, std::move(out));
    }
  }
};

behavior worker(actor_ctx<worker_state>& self) {
  auto& s = self.state;
  return {
      handler_from<init_atom, int, uint32_t, uint32_t, uint32_t, uint32_t, actor, const uint32_t*,
                   uint64_t, bool>(
          [&](const actor& from, init_atom, int device, uint32_t jobs, uint32_t wg_size,
              uint32_t wg_num, uint32_t bound, actor reply_to, const uint32_t* input,
              uint64_t total_rows, bool device_merge) {
            s.device = device;
            wah_device_select(device);
            s.wg_size = wg_size;
            s.wg_num = wg_num;
            s.bound = bound;
            s.reply_to = reply_to;
            s.input = input;
            s.total_rows = total_rows;
            s.device_merge = device_merge;
            s.sys = &self.system();
            s.self = self.self();
            s.setup_status = s.setup(jobs);
            s.completer = std::thread([&s] { s.complete_loop(); });
            self.send(from, ready_atom{}, s.setup_status);
          }),
      handler<work_atom, uint64_t, uint64_t>(
          [&](work_atom, uint64_t row_start, uint64_t rows) {
            wah_device_select(s.device);
            size_t i = 0;
            {
              std::lock_guard<std::mutex> lk(s.mu);
              while (i < s.slots.size() && s.slots[i].busy) ++i;
              if (i < s.slots.size()) s.slots[i].busy = true;
            }
            if (i == s.slots.size()) {  // more batches than --jobs: a caller bug
              std::vector<slice_index> err(1);
              err[0].status = WAH_EINVAL;
              self.send(s.reply_to, done_atom{}, rows, std::move(err));
              return;
            }
            job_slot& j = s.slots[i];
            j.row_start = row_start;
            j.ncols = static_cast<uint32_t>((rows + s.wg_size - 1) / s.wg_size);
            j.ns.assign(j.ncols, s.wg_size);
            j.ns.back() = static_cast<uint32_t>(rows - uint64_t(j.ncols - 1) * s.wg_size);
            j.status = s.setup_status != WAH_OK ? s.setup_status : s.launch(j);
            {
              std::lock_guard<std::mutex> lk(s.mu);
              s.queue.push_back(i);
            }
            s.cv.notify_all();
          }),
      handler<quit_atom>([&](quit_atom) {
        wah_device_select(s.device);
        s.teardown();
        self.quit();
      }),
  };
}

// --------------------------------------------------------------- indexer --

struct indexer_state {
  actor worker, merger;
  uint64_t n = 0;  // rows of the column (staged page-locked, read by the worker)
  uint64_t next_row = 0;   // first row not yet sent
  uint64_t remaining = 0;  // rows not yet indexed
  uint32_t in_progress = 0, jobs = 1, wg_num = 1, wg_size = 1;
  int status = WAH_OK;
};

behavior indexer(actor_ctx<indexer_state>& self) {
  auto& s = self.state;
  // copied into the handlers that call it: this function's frame is gone
  // by the time they run (the actor's context and state are not)
  auto finish = [&self, &s] {
    self.send(s.merger, quit_atom{}, s.status);
    self.send(s.worker, quit_atom{});
    self.quit();
  };
  return {
      handler<init_atom, actor, actor, uint64_t, uint32_t, uint32_t, uint32_t>(
          [&, finish](init_atom, actor w, actor m, uint64_t n, uint32_t jobs, uint32_t wg_num,
              uint32_t wg_size) {
            s.worker = w;
            s.merger = m;
            s.n = n;
            s.remaining = n;
            s.jobs = jobs;
            s.wg_num = wg_num;
            s.wg_size = wg_size;
            if (s.remaining == 0) finish();
          }),
      handler<index_atom>([&](index_atom) {
        if (s.status != WAH_OK || s.in_progress >= s.jobs || s.next_row >= s.n) return;
        const uint64_t batch = std::min<uint64_t>(s.n - s.next_row, uint64_t(s.wg_size) * s.wg_num);
        self.send(s.worker, work_atom{}, s.next_row, batch);
        s.next_row += batch;
        s.in_progress += 1;
        self.send(self.self(), index_atom{});
      }),
      handler<done_atom, uint64_t, std::vector<slice_index>>(
          [&, finish](done_atom, uint64_t processed, std::vector<slice_index> slices) {
            s.in_progress -= 1;
            s.remaining -= std::min(processed, s.remaining);
            for (auto& x : slices) {
              if (x.status != WAH_OK && s.status == WAH_OK) s.status = x.status;
              self.send(s.merger, add_atom{}, std::move(x));
            }
            if (s.status != WAH_OK || s.remaining == 0) {
              if (s.in_progress == 0) finish();
              return;
            }
            self.send(self.self(), index_atom{});
          }),
  };
}

}  // namespace

int main(int argc, char** argv) {
  std::string filename, device_name, output;
  uint32_t bound = 0, batch_size = 1023, jobs = 1, work_groups = 1;
  bool print_results = false, host_parse = false, device_merge = false;
  const std::vector<wahcli::flag> flags = {
      {"data-file", 'f', "file with test data (one value per line)", wahcli::flag::STRING, &filename},
      {"bound", 'b', "maximum value (0 will scan values)", wahcli::flag::U32, &bound},
      {"device", 'd', "device for computation (first available if empty)", wahcli::flag::STRING,
       &device_name},
      {"batch-size", 0, "values indexed per work-group slice (1023)", wahcli::flag::U32,
       &batch_size},
      {"print", 'p', "print resulting bitmap index", wahcli::flag::BOOL, &print_results},
      {"work-groups", 'w', "slices per batch (1)", wahcli::flag::U32, &work_groups},
      {"jobs", 'j', "batches in flight on the GPU (1; 0 = 4, at most 8)", wahcli::flag::U32, &jobs},
      {"output", 'o', "write K, L, keys, offsets, index (u32) to this file", wahcli::flag::STRING,
       &output},
      {"host-parse", 0, "parse the data file on the host instead of the GPU", wahcli::flag::BOOL,
       &host_parse},
      {"device-merge", 0, "append the slices on the GPU and copy the merged index back once",
       wahcli::flag::BOOL, &device_merge},
  };
  const int pf = wahcli::parse_flags(argc, argv, flags);
  if (pf != 0) return pf > 0 ? 0 : 2;
  std::vector<uint32_t> values;
  if (filename.empty()) {
    values = wahcli::builtin_values();
  } else {
    std::printf("Reading data from '%s' ... ", filename.c_str());
    std::fflush(stdout);
    std::string err;
    if (host_parse ? !wahcli::read_values(filename, &values)
                   : !wahcli::read_values_gpu(filename, &values, &err)) {
      std::fprintf(stderr, "%s\n", err.empty() ? ("cannot read '" + filename + "'").c_str()
                                                : err.c_str());
      return 2;
    }
  }
  std::printf("'%zu' values.\n", values.size());
  if (bound == 0 && !values.empty()) bound = *std::max_element(values.begin(), values.end());
  std::printf("Maximum value is '%u'.\n", bound);
  if (values.size() >= WAH_MAX_ROWS) {
    std::fprintf(stderr, "[!!!] %s\n", wah_strerror(WAH_ERANGE));
    return 1;
  }

  const int dev = wahcli::find_device(device_name, false);
  if (dev < 0) {
    std::fprintf(stderr, "Device %s not found.\n", device_name.c_str());
    return 3;
  }
  char name[256] = {0};
  if (wah_device_select(dev) != WAH_OK || wah_device_name(dev, name, sizeof name) != WAH_OK) {
    std::fprintf(stderr, "cannot select device %d\n", dev);
    return 3;
  }
  std::printf("Using device named '%s'.\n", name);

  if (jobs == 0) jobs = 4;
  jobs = std::min<uint32_t>(jobs, 8);
  work_groups = std::max<uint32_t>(work_groups, 1);
  const uint64_t n = values.size();
  uint64_t wg_size = std::max<uint64_t>(1, std::min<uint64_t>(batch_size, n));
  if (wg_size < n && wg_size % kChunk) {
    const uint64_t r = std::max<uint64_t>(kChunk, wg_size / kChunk * kChunk);
    std::printf("Batch size %llu rounded to %llu (slices start on 31-row chunks).\n",
                (unsigned long long)wg_size, (unsigned long long)r);
    wg_size = r;
  }
  const uint64_t slices = (std::max<uint64_t>(n, 1) + wg_size - 1) / wg_size;
  work_groups = static_cast<uint32_t>(std::min<uint64_t>(work_groups, slices));

  // the column in page-locked memory: batches are copied to the device from it
  wahcli::pinned_u32 column;
  if (column.alloc(n) != WAH_OK) {
    std::fprintf(stderr, "[!!!] %s\n", wah_strerror(WAH_ENOMEM));
    return 1;
  }
  if (n) std::memcpy(column.p, values.data(), n * 4);
  std::vector<uint32_t>().swap(values);

  int exit_code = 0;
  {
    actor_system system{4};
    actor m = system.spawn<merger_state>([](actor_ctx<merger_state>& self) { return merger(self); });
    actor w = system.spawn<worker_state>([](actor_ctx<worker_state>& self) { return worker(self); });
    actor x = system.spawn<indexer_state>(
        [](actor_ctx<indexer_state>& self) { return indexer(self); });
    // the worker's buffers exist before the clock starts (the reference
    // spawns its OpenCL worker before the indexer and merger, too)
    int setup = WAH_OK;
    {
      scoped_actor self{system};
      self.send(w, init_atom{}, dev, jobs, static_cast<uint32_t>(wg_size), work_groups, bound, x,
                static_cast<const uint32_t*>(column.p), n, device_merge);
      self.receive(handler<ready_atom, int>([&](ready_atom, int rc) { setup = rc; }));
    }
    if (setup != WAH_OK) std::fprintf(stderr, "[!!!] %s\n", wah_strerror(setup));
    system.send(m, init_atom{}, print_results, bound, output, &exit_code);
    system.send(x, init_atom{}, w, m, n, jobs, work_groups, static_cast<uint32_t>(wg_size));
    system.send(x, index_atom{});
    system.await_all_actors_done();
  }
  return exit_code;
}
