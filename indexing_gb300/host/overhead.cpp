// overhead -- launch-overhead measurements (src/overhead_benchmark.cpp:64-148).
//
// The reference sends an empty kernel through CAF's OpenCL actor facade and
// reports the mean round trip ("Took X us on average over N runs.").  The
// same round trip is measured here -- a scoped actor sends to a device actor,
// which launches the empty kernel through the C ABI, waits for it and
// replies -- together with what explains the gap between per-column and
// batched builds:
//
//   actor      scoped actor -> device actor -> wah_noop -> sync -> reply
//   direct     wah_noop + stream sync from the calling thread
//   stream     K empty launches back to back, one sync: cost per launch
//   graph      the K launches captured once in a CUDA graph, replayed
//   build      wah_build of one small column + sync (about ten kernels)
//   batched    C columns of the same size in one replayed batched build
//              (wah_batch_launch_graph): cost per column
//
// Flags: -i/--iterations (1000), -d/--device, -k/--launches (K, 1000),
// --rows (rows of the small column, 4096), --columns (C, 256).  Prints the
// reference's line for the actor round trip, then one JSON line with every
// figure in microseconds.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <numeric>
#include <string>
#include <vector>

#include "actors.hpp"
#include "cli.hpp"

using namespace wahact;

namespace {

struct launch_atom {};
struct quit_atom {};

struct device_state {
  int device = 0;
  void* stream = nullptr;
};

behavior device_actor(actor_ctx<device_state>& self) {
  auto& s = self.state;
  return {
      handler_from<launch_atom>([&](const actor& from, launch_atom) {
        wah_device_select(s.device);
        int rc = wah_noop(s.stream);
        if (rc == WAH_OK) rc = wah_stream_sync(s.stream);
        self.send(from, launch_atom{}, rc);
      }),
      handler<quit_atom>([&](quit_atom) { self.quit(); }),
  };
}

double now_us() {
  return std::chrono::duration<double, std::micro>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

struct stats {
  double mean, p50, p99;
};
stats summarize(std::vector<double> v) {
  if (v.empty()) return {0, 0, 0};
  std::sort(v.begin(), v.end());
  const double mean = std::accumulate(v.begin(), v.end(), 0.0) / v.size();
  return {mean, v[v.size() / 2], v[std::min(v.size() - 1, v.size() * 99 / 100)]};
}

// The small column: row i has value (i * 2654435761) mod 4096.
std::vector<uint32_t> small_column(uint64_t rows) {
  std::vector<uint32_t> v(rows);
  for (uint64_t i = 0; i < rows; ++i) v[i] = (uint32_t)((i * 2654435761ull) & 4095u);
  return v;
}

}  // namespace

int main(int argc, char** argv) {
  std::string device_name;
  uint64_t iterations = 1000, launches = 1000, rows = 4096, columns = 256;
  const std::vector<wahcli::flag> flags = {
      {"iterations", 'i', "measurements (1000)", wahcli::flag::U64, &iterations},
      {"device", 'd', "device for computation (first available if not found)",
       wahcli::flag::STRING, &device_name},
      {"launches", 'k', "launches per stream / graph measurement (1000)", wahcli::flag::U64,
       &launches},
      {"rows", 0, "rows of the small column (4096)", wahcli::flag::U64, &rows},
      {"columns", 0, "columns of the batched build (256)", wahcli::flag::U64, &columns},
  };
  const int pf = wahcli::parse_flags(argc, argv, flags);
  if (pf != 0) return pf > 0 ? 0 : 2;
  iterations = std::max<uint64_t>(iterations, 1);
  launches = std::max<uint64_t>(launches, 1);
  rows = std::max<uint64_t>(rows, 1);
  columns = std::max<uint64_t>(columns, 1);
  const int dev = wahcli::find_device(device_name, true);
  if (dev < 0 || wah_device_select(dev) != WAH_OK) {
    std::fprintf(stderr, "No device found.\n");
    return 3;
  }
  void* stream = nullptr;
  if (wah_stream_create(&stream) != WAH_OK) return 1;
  int rc = WAH_OK;
  auto ok = [&](int r) {
    if (r != WAH_OK && rc == WAH_OK) rc = r;
    return r == WAH_OK;
  };

  // actor round trip
  std::vector<double> t_actor;
  {
    actor_system system{2};
    actor device = system.spawn<device_state>([&](actor_ctx<device_state>& self) {
      self.state.device = dev;
      self.state.stream = stream;
      return device_actor(self);
    });
    scoped_actor self{system};
    for (uint64_t i = 0; i < iterations + 10; ++i) {
      const double t0 = now_us();
      self.send(device, launch_atom{});
      self.receive(handler<launch_atom, int>([&](launch_atom, int r) { ok(r); }));
      if (i >= 10) t_actor.push_back(now_us() - t0);  // the first ones warm up
    }
    self.send(device, quit_atom{});
  }
  // direct launch + sync
  std::vector<double> t_direct;
  for (uint64_t i = 0; i < iterations + 10 && rc == WAH_OK; ++i) {
    const double t0 = now_us();
    ok(wah_noop(stream));
    ok(wah_stream_sync(stream));
    if (i >= 10) t_direct.push_back(now_us() - t0);
  }
  // back-to-back launches, one sync; then the same launches as a graph
  double stream_us = 0, graph_us = 0;
  for (int rep = 0; rep < 2 && rc == WAH_OK; ++rep) {  // the first pass warms up
    const double t0 = now_us();
    for (uint64_t i = 0; i < launches; ++i) ok(wah_noop(stream));
    ok(wah_stream_sync(stream));
    stream_us = (now_us() - t0) / launches;
  }
  {
    wah_noop_graph* g = nullptr;
    if (rc == WAH_OK && ok(wah_noop_graph_create((uint32_t)launches, &g))) {
      for (int rep = 0; rep < 2 && rc == WAH_OK; ++rep) {
        const double t0 = now_us();
        ok(wah_noop_graph_launch(g, stream));
        ok(wah_stream_sync(stream));
        graph_us = (now_us() - t0) / launches;
      }
      wah_noop_graph_destroy(g);
    }
  }
  // one small build + sync, and the batched build per column
  std::vector<double> t_build;
  double batched_us = 0;
  uint32_t build_launches = 0;
  {
    const std::vector<uint32_t> host = small_column(rows);
    const uint32_t bound = 4095;
    uint64_t keys_cap = 0, index_cap = 0;
    wah_output_caps(rows, bound, &keys_cap, &index_cap);
    const uint64_t vs = (rows + 3) & ~3ull, ks = (keys_cap + 3) & ~3ull,
                   is = (index_cap + 3) & ~3ull;
    void *d_vals = nullptr, *d_keys = nullptr, *d_offs = nullptr, *d_index = nullptr,
         *d_counts = nullptr, *d_ws = nullptr;
    const size_t ws_bytes = wah_workspace_bytes(rows, bound);
    ok(wah_dev_alloc(vs * 4 * columns, &d_vals));
    ok(wah_dev_alloc(ks * 4 * columns, &d_keys));
    ok(wah_dev_alloc(ks * 4 * columns, &d_offs));
    ok(wah_dev_alloc(is * 4 * columns, &d_index));
    ok(wah_dev_alloc(16 * columns, &d_counts));
    ok(wah_dev_alloc(ws_bytes, &d_ws));
    for (uint64_t c = 0; c < columns && rc == WAH_OK; ++c)
      ok(wah_copy(static_cast<uint32_t*>(d_vals) + c * vs, host.data(), rows * 4, stream));
    if (rc == WAH_OK) ok(wah_stream_sync(stream));
    for (uint64_t i = 0; i < iterations + 10 && rc == WAH_OK; ++i) {
      const double t0 = now_us();
      ok(wah_build(static_cast<uint32_t*>(d_vals), rows, bound, static_cast<uint32_t*>(d_keys),
                   static_cast<uint32_t*>(d_offs), static_cast<uint32_t*>(d_index),
                   static_cast<wah_counts*>(d_counts), d_ws, ws_bytes, stream));
      build_launches = wah_last_launch_count();
      ok(wah_stream_sync(stream));
      if (i >= 10) t_build.push_back(now_us() - t0);
    }
    std::vector<uint64_t> ns(columns, rows);
    std::vector<uint32_t> bounds(columns, bound);
    wah_batch* b = nullptr;
    if (rc == WAH_OK && ok(wah_batch_create(ns.data(), bounds.data(), (uint32_t)columns, &b))) {
      std::vector<wah_column> cols(columns);
      for (uint64_t c = 0; c < columns; ++c) {
        cols[c].values = static_cast<uint32_t*>(d_vals) + c * vs;
        cols[c].n = rows;
        cols[c].bound = bound;
        cols[c].reserved = 0;
        cols[c].keys = static_cast<uint32_t*>(d_keys) + c * ks;
        cols[c].offsets = static_cast<uint32_t*>(d_offs) + c * ks;
        cols[c].index = static_cast<uint32_t*>(d_index) + c * is;
        cols[c].counts = static_cast<wah_counts*>(d_counts) + c;
      }
      ok(wah_batch_set_columns(b, cols.data(), stream));
      const uint64_t reps = std::max<uint64_t>(iterations / 10, 3);
      for (int pass = 0; pass < 2 && rc == WAH_OK; ++pass) {  // the first pass captures
        const double t0 = now_us();
        for (uint64_t r = 0; r < reps; ++r) ok(wah_batch_launch_graph(b, stream));
        ok(wah_stream_sync(stream));
        batched_us = (now_us() - t0) / (reps * columns);
      }
      wah_stream_sync(stream);
      wah_batch_destroy(b);
    }
    for (void* p : {d_vals, d_keys, d_offs, d_index, d_counts, d_ws})
      if (p) wah_dev_free(p);
  }
  wah_stream_destroy(stream);
  if (rc != WAH_OK) {
    std::fprintf(stderr, "[!!!] %s\n", wah_strerror(rc));
    return 1;
  }
  const stats a = summarize(t_actor), d = summarize(t_direct), b = summarize(t_build);
  std::printf("Took %.0fus on average over %zu runs.\n", a.mean, t_actor.size());
  std::printf(
      "{\"actor_us\": {\"mean\": %.2f, \"p50\": %.2f, \"p99\": %.2f}, "
      "\"direct_us\": {\"mean\": %.2f, \"p50\": %.2f, \"p99\": %.2f}, "
      "\"stream_us_per_launch\": %.3f, \"graph_us_per_launch\": %.3f, "
      "\"build_us\": {\"mean\": %.2f, \"p50\": %.2f, \"p99\": %.2f, \"rows\": %llu, "
      "\"launches\": %u}, \"batched_us_per_column\": %.3f, \"columns\": %llu}\n",
      a.mean, a.p50, a.p99, d.mean, d.p50, d.p99, stream_us, graph_us, b.mean, b.p50, b.p99,
      (unsigned long long)rows, build_launches, batched_us, (unsigned long long)columns);
  return 0;
}
