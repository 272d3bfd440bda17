// phases -- the reference's multi-phase GPU driver rebuilt on the GB300
// kernels (src/phases.cpp:356-1136).
//
// A device actor owns the column's device buffers and one stream; the main
// thread is a scoped actor that drives the phases one request/reply round
// trip at a time and prints the host time each one took, as the reference's
// SHOW_TIME_CONSUMPTION build does ("N us" per line, src/phases.cpp:714-1127):
//
//   Transfer to     values host -> device         (global_argument, :720)
//   Sort            stable radix sort carrying row ids (:730-813)
//   Index           chunk ids + literals, OR-merge, fills, fuse, column
//                   lengths, offsets, keys -- one fused pass here (:817-1083)
//   Transfer back   keys, offsets, index device -> host (mem_ref::data, :1087-1093)
//   Total
//
// Flags as the reference (-f data file, -b bound, -d device name, -p print)
// plus --describe (label each line, the reference's WITH_DESCRIPTION build),
// --output FILE (binary result: K, L, keys, offsets, index) and --host-parse
// (read the data file on the host; by default its bytes are parsed on the
// GPU by wah_parse_text, before the timed phases as in the reference).  Unlike the
// reference, -p prints the index as the cpu program does, and the keys are
// produced (the reference's phases never materialises them).
#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "actors.hpp"
#include "cli.hpp"

using namespace wahact;

namespace {

struct transfer_to_atom {};
struct sort_atom {};
struct index_atom {};
struct transfer_back_atom {};
struct quit_atom {};

struct device_state {
  int device = 0;  // made current at the start of every handler: handlers
                   // run on whichever worker thread the system picks
  void* stream = nullptr;
  uint64_t n = 0;
  uint32_t bound = 0;
  uint64_t keys_cap = 0, index_cap = 0;
  size_t ws_bytes = 0;
  uint32_t *values = nullptr, *sorted = nullptr, *rids = nullptr, *keys = nullptr,
           *offsets = nullptr, *index = nullptr, *status = nullptr;
  wah_counts* counts = nullptr;
  void* ws = nullptr;
  wah_counts host_counts{};

  int allocate(uint64_t rows, uint32_t b) {
    n = rows;
    bound = b;
    wah_output_caps(n, bound, &keys_cap, &index_cap);
    ws_bytes = wah_workspace_bytes(n, bound);
    int rc = wah_stream_create(&stream);
    const uint64_t n1 = std::max<uint64_t>(n, 1);
    void* p = nullptr;
    auto alloc = [&](size_t bytes, void** out) {
      if (rc == WAH_OK) rc = wah_dev_alloc(bytes, out);
    };
    alloc(n1 * 4, &p);
    values = static_cast<uint32_t*>(p);
    alloc(n1 * 4, &p);
    sorted = static_cast<uint32_t*>(p);
    alloc(n1 * 4, &p);
    rids = static_cast<uint32_t*>(p);
    alloc(std::max<uint64_t>(keys_cap, 1) * 4, &p);
    keys = static_cast<uint32_t*>(p);
    alloc(std::max<uint64_t>(keys_cap, 1) * 4, &p);
    offsets = static_cast<uint32_t*>(p);
    alloc(std::max<uint64_t>(index_cap, 1) * 4, &p);
    index = static_cast<uint32_t*>(p);
    alloc(16, &p);
    status = static_cast<uint32_t*>(p);
    alloc(sizeof(wah_counts), &p);
    counts = static_cast<wah_counts*>(p);
    alloc(ws_bytes, &ws);
    return rc;
  }
  void release() {
    if (stream) wah_stream_sync(stream);
    for (void* p : {static_cast<void*>(values), static_cast<void*>(sorted),
                    static_cast<void*>(rids), static_cast<void*>(keys),
                    static_cast<void*>(offsets), static_cast<void*>(index),
                    static_cast<void*>(status), static_cast<void*>(counts), ws})
      if (p) wah_dev_free(p);
    if (stream) wah_stream_destroy(stream);
    stream = nullptr;
  }
};

int sync_rc(int rc, void* stream) { return rc != WAH_OK ? rc : wah_stream_sync(stream); }

// The device actor: one handler per phase, each replying when its work is
// finished on the device (the reference's kernel actors reply when their
// OpenCL event completes).
behavior device_actor(actor_ctx<device_state>& self) {
  auto& s = self.state;
  return {
      handler_from<transfer_to_atom, const uint32_t*, uint64_t, uint32_t>(
          [&](const actor& from, transfer_to_atom, const uint32_t* values, uint64_t n,
              uint32_t bound) {
            wah_device_select(s.device);
            int rc = s.allocate(n, bound);
            if (rc == WAH_OK && n) rc = wah_copy(s.values, values, n * 4, s.stream);
            self.send(from, transfer_to_atom{}, sync_rc(rc, s.stream));
          }),
      handler_from<sort_atom>([&](const actor& from, sort_atom) {
        wah_device_select(s.device);
        uint32_t status = WAH_OK;
        int rc = wah_sort_rids_by_value(s.values, s.n, s.bound, s.sorted, s.rids, s.status, s.ws,
                                        s.ws_bytes, s.stream);
        if (rc == WAH_OK) rc = wah_copy(&status, s.status, 4, s.stream);
        rc = sync_rc(rc, s.stream);
        if (rc == WAH_OK && s.n > 0) rc = static_cast<int>(status);
        self.send(from, sort_atom{}, rc);
      }),
      handler_from<index_atom>([&](const actor& from, index_atom) {
        wah_device_select(s.device);
        int rc = wah_build_sorted(s.sorted, s.rids, s.n, s.keys, s.offsets, s.index, s.counts,
                                  s.ws, s.ws_bytes, s.stream);
        if (rc == WAH_OK) rc = wah_copy(&s.host_counts, s.counts, sizeof(wah_counts), s.stream);
        rc = sync_rc(rc, s.stream);
        if (rc == WAH_OK) rc = static_cast<int>(s.host_counts.status);
        self.send(from, index_atom{}, rc, s.host_counts);
      }),
      // keys[K], offsets[K], index[L] into the caller's page-locked buffers
      handler_from<transfer_back_atom, uint32_t*, uint32_t*, uint32_t*>(
          [&](const actor& from, transfer_back_atom, uint32_t* keys, uint32_t* offsets,
              uint32_t* index) {
            wah_device_select(s.device);
            const wah_counts c = s.host_counts;
            int rc = WAH_OK;
            if (c.index_len) rc = wah_copy(index, s.index, uint64_t(c.index_len) * 4, s.stream);
            if (rc == WAH_OK && c.keycnt)
              rc = wah_copy(offsets, s.offsets, uint64_t(c.keycnt) * 4, s.stream);
            if (rc == WAH_OK && c.keycnt)
              rc = wah_copy(keys, s.keys, uint64_t(c.keycnt) * 4, s.stream);
            self.send(from, transfer_back_atom{}, sync_rc(rc, s.stream));
          }),
      handler<quit_atom>([&](quit_atom) {
        wah_device_select(s.device);
        s.release();
        self.quit();
      }),
  };
}

}  // namespace

int main(int argc, char** argv) {
  std::string filename, device_name, output;
  uint32_t bound = 0;
  bool print_results = false, describe = false, host_parse = false;
  const std::vector<wahcli::flag> flags = {
      {"data-file", 'f', "file with test data (one value per line)", wahcli::flag::STRING, &filename},
      {"bound", 'b', "maximum value (0 will scan values)", wahcli::flag::U32, &bound},
      {"device", 'd', "device for computation (first available if not found)",
       wahcli::flag::STRING, &device_name},
      {"print", 'p', "print resulting bitmap index", wahcli::flag::BOOL, &print_results},
      {"describe", 0, "label each timing line", wahcli::flag::BOOL, &describe},
      {"host-parse", 0, "parse the data file on the host instead of the GPU", wahcli::flag::BOOL,
       &host_parse},
      {"output", 'o', "write K, L, keys, offsets, index (u32) to this file", wahcli::flag::STRING,
       &output},
  };
  const int pf = wahcli::parse_flags(argc, argv, flags);
  if (pf != 0) return pf > 0 ? 0 : 2;
  if (filename.empty()) {
    std::printf("A filename with test data is required, see --help for details.\n");
    return 2;
  }
  const int dev = wahcli::find_device(device_name, true);
  if (dev < 0) {
    std::fprintf(stderr, "No device found.\n");
    return 3;
  }
  if (wah_device_select(dev) != WAH_OK) {
    std::fprintf(stderr, "cannot select device %d\n", dev);
    return 3;
  }
  // reading the file is not timed (the reference reads it before its clock)
  std::vector<uint32_t> values;
  std::string err;
  if (host_parse ? !wahcli::read_values(filename, &values)
                 : !wahcli::read_values_gpu(filename, &values, &err)) {
    std::fprintf(stderr, "%s\n", err.empty() ? ("cannot read '" + filename + "'").c_str()
                                              : err.c_str());
    return 2;
  }
  if (bound == 0 && !values.empty()) bound = *std::max_element(values.begin(), values.end());

  auto line = [&](const char* label, uint64_t us) {
    if (describe)
      std::printf("%-16s%llu us\n", label, (unsigned long long)us);
    else
      std::printf("%llu us\n", (unsigned long long)us);
  };
  // page-locked host buffers for the column and the index, set up before
  // the clock starts (the reference's buffers are ready before it, too)
  const uint64_t n = values.size();
  uint64_t keys_cap = 0, index_cap = 0;
  wah_output_caps(n, bound, &keys_cap, &index_cap);
  wahcli::pinned_u32 h_values, h_keys, h_offsets, h_index;
  int rc = h_values.alloc(n);
  if (rc == WAH_OK) rc = h_keys.alloc(keys_cap);
  if (rc == WAH_OK) rc = h_offsets.alloc(keys_cap);
  if (rc == WAH_OK) rc = h_index.alloc(index_cap);
  if (rc != WAH_OK) {
    std::fprintf(stderr, "[!!!] %s\n", wah_strerror(rc));
    return 1;
  }
  std::copy(values.begin(), values.end(), h_values.p);
  std::vector<uint32_t>().swap(values);
  wah_counts counts{};
  {
    actor_system system{2};
    actor device = system.spawn<device_state>([dev](actor_ctx<device_state>& self) {
      self.state.device = dev;
      return device_actor(self);
    });
    scoped_actor self{system};
    const auto start = std::chrono::steady_clock::now();
    auto from = start;
    auto expect_ok = [&](int r) {
      if (r != WAH_OK && rc == WAH_OK) rc = r;
      return rc == WAH_OK;
    };

    self.send(device, transfer_to_atom{}, static_cast<const uint32_t*>(h_values.p), n, bound);
    self.receive(handler<transfer_to_atom, int>([&](transfer_to_atom, int r) { expect_ok(r); }));
    line("Transfer to:", wahcli::micros_since(from));
    from = std::chrono::steady_clock::now();

    if (rc == WAH_OK) {
      self.send(device, sort_atom{});
      self.receive(handler<sort_atom, int>([&](sort_atom, int r) { expect_ok(r); }));
      line("Sort:", wahcli::micros_since(from));
      from = std::chrono::steady_clock::now();
    }
    if (rc == WAH_OK) {
      self.send(device, index_atom{});
      self.receive(handler<index_atom, int, wah_counts>([&](index_atom, int r, wah_counts c) {
        expect_ok(r);
        counts = c;
      }));
      line("Index:", wahcli::micros_since(from));
      from = std::chrono::steady_clock::now();
    }
    if (rc == WAH_OK) {
      self.send(device, transfer_back_atom{}, h_keys.p, h_offsets.p, h_index.p);
      self.receive(handler<transfer_back_atom, int>(
          [&](transfer_back_atom, int r) { expect_ok(r); }));
      line("Transfer back:", wahcli::micros_since(from));
    }
    line("Total:", wahcli::micros_since(start));
    self.send(device, quit_atom{});
  }
  if (rc != WAH_OK) {
    std::fprintf(stderr, "[!!!] %s\n", wah_strerror(rc));
    return 1;
  }
  std::printf("Index has %u elements with %u keys\n", counts.index_len, counts.keycnt);
  if (print_results)
    wahcli::print_index(h_keys.p, h_offsets.p, counts.keycnt, h_index.p, counts.index_len);
  if (!output.empty() && !wahcli::write_result(output, h_keys.p, h_offsets.p, counts.keycnt,
                                               h_index.p, counts.index_len)) {
    std::fprintf(stderr, "cannot write '%s'\n", output.c_str());
    return 1;
  }
  return 0;
}
