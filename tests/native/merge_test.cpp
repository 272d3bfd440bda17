// merge_test -- the slice merger of the `gpu` program against the oracle.
//
// Test code: links the oracle (oracle/wah_oracle.c).  Random columns are cut
// into slices whose sizes are multiples of 31, each slice is indexed by the
// oracle on its own, the slice indexes are merged, and the result must equal
// the oracle's index of the whole column word for word.  Also checks that the
// reference's plain append (no re-basing) differs on such inputs.
#include <cstdio>
#include <cstdlib>
#include <map>
#include <vector>

#include "merge.hpp"
#include "wah_oracle.h"

namespace {

struct built {
  std::vector<uint32_t> keys, offsets, index;
};

built oracle_build(const uint32_t* v, size_t n) {
  built b;
  const size_t cap = n ? n : 1;
  b.keys.resize(cap);
  b.offsets.resize(cap);
  b.index.resize(2 * cap);
  size_t K = 0, L = 0, k = 0;
  if (wah_oracle_build(v, n, WAH_ORACLE_SORT_STABLE, b.keys.data(), b.offsets.data(),
                       b.index.data(), &K, &L, &k) != 0) {
    std::fprintf(stderr, "oracle failed\n");
    std::exit(2);
  }
  b.keys.resize(K);
  b.offsets.resize(K);
  b.index.resize(L);
  return b;
}

uint64_t state = 0x1234567;
uint32_t next_u32() {
  uint64_t z = (state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return static_cast<uint32_t>((z ^ (z >> 31)) >> 32);
}

}  // namespace

int main() {
  int failures = 0, cases = 0, append_differs = 0;
  const size_t sizes[] = {1, 30, 31, 32, 500, 1023, 1024, 5000, 40000};
  const uint32_t cards[] = {1, 2, 3, 16, 1000, 65536};
  const size_t slice_sizes[] = {31, 62, 1023, 3100};
  for (size_t n : sizes)
    for (uint32_t card : cards)
      for (int layout = 0; layout < 2; ++layout)
        for (size_t slice : slice_sizes) {
          std::vector<uint32_t> v(n);
          for (size_t i = 0; i < n; ++i) {
            if (layout == 0)
              v[i] = next_u32() % card;
            else  // runs of ~100 equal values: long fills between slices
              v[i] = ((i / 100) * 7919u + (i % 97 == 0 ? 1 : 0)) % card;
          }
          const built whole = oracle_build(v.data(), n);
          wahmerge::slice_merger m;
          for (size_t start = 0; start < n; start += slice) {
            const size_t len = std::min(slice, n - start);
            const built part = oracle_build(v.data() + start, len);
            if (!m.add(start, len, part.keys.data(), part.offsets.data(),
                       static_cast<uint32_t>(part.keys.size()), part.index.data(),
                       static_cast<uint32_t>(part.index.size()))) {
              std::fprintf(stderr, "add refused at row %zu\n", start);
              ++failures;
            }
          }
          built merged;
          m.finish(&merged.keys, &merged.offsets, &merged.index);
          // the reference merger's plain per-key append (src/gpu.cpp:140-149)
          {
            std::map<uint32_t, std::vector<uint32_t>> app;
            for (size_t start = 0; start < n; start += slice) {
              const size_t len = std::min(slice, n - start);
              const built part = oracle_build(v.data() + start, len);
              for (size_t i = 0; i < part.keys.size(); ++i) {
                const size_t e = i + 1 < part.keys.size() ? part.offsets[i + 1] : part.index.size();
                auto& dst = app[part.keys[i]];
                dst.insert(dst.end(), part.index.begin() + part.offsets[i], part.index.begin() + e);
              }
            }
            std::vector<uint32_t> flat;
            for (auto& kv : app) flat.insert(flat.end(), kv.second.begin(), kv.second.end());
            if (flat != whole.index) ++append_differs;
          }
          ++cases;
          if (merged.keys != whole.keys || merged.offsets != whole.offsets ||
              merged.index != whole.index) {
            std::fprintf(stderr, "mismatch: n=%zu card=%u layout=%d slice=%zu\n", n, card, layout,
                         slice);
            ++failures;
          }
        }
  // large slices merged by several threads (the parallel path), against the
  // whole column and against the one-thread merge
  {
    const size_t n = 3000000, slice = 31 * 40000;
    std::vector<uint32_t> v(n);
    for (size_t i = 0; i < n; ++i) v[i] = next_u32() % 1000;
    const built whole = oracle_build(v.data(), n);
    wahmerge::slice_merger par(4), one(1);
    for (size_t start = 0; start < n; start += slice) {
      const size_t len = std::min(slice, n - start);
      const built part = oracle_build(v.data() + start, len);
      for (wahmerge::slice_merger* m : {&par, &one})
        m->add(start, len, part.keys.data(), part.offsets.data(),
               static_cast<uint32_t>(part.keys.size()), part.index.data(),
               static_cast<uint32_t>(part.index.size()));
    }
    built a, b;
    par.finish(&a.keys, &a.offsets, &a.index);
    one.finish(&b.keys, &b.offsets, &b.index);
    ++cases;
    if (a.keys != whole.keys || a.offsets != whole.offsets || a.index != whole.index ||
        b.index != whole.index) {
      std::fprintf(stderr, "mismatch: threaded merge of 3M rows\n");
      ++failures;
    }
  }
  // a slice that does not start on a chunk boundary is refused
  {
    wahmerge::slice_merger m;
    const uint32_t k = 5, o = 0, w = 0x80000001u;
    if (m.add(30, 1, &k, &o, 1, &w, 1)) {
      std::fprintf(stderr, "unaligned slice accepted\n");
      ++failures;
    }
  }
  if (append_differs == 0) {
    std::fprintf(stderr, "plain append never differed: the cases do not exercise slice gaps\n");
    ++failures;
  }
  if (failures) {
    std::fprintf(stderr, "merge: %d of %d cases failed\n", failures, cases);
    return 1;
  }
  std::printf("merge: all %d cases passed (plain append differs in %d)\n", cases, append_differs);
  return 0;
}
