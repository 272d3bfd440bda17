// ref_cpu_shim.cpp -- exposes the reference's own WAH functions as a C ABI.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile, in the development
// container where the reference sources are mounted, into oracle/_ref/
// (git-ignored).  It #includes the reference file src/cpu.cpp as it lies (the
// include path points at the reference checkout) together with the CAF
// stand-in under oracle/caf_stub/, so the functions called below are the
// reference's code, not a restatement.  Used to pin the C restatement
// (oracle/wah_oracle.c) and to generate the golden vectors in tests/golden/.
#include <cstdint>
#include <cstring>
#include <utility>

#include "src/cpu.cpp"

namespace {
// src/phases.cpp:143-160 (compiled only under WITH_CPU_TESTS there, and that
// file needs CAF's OpenCL module, so it cannot be built here): rids = iota,
// std::stable_sort of (value, rid) pairs comparing the value only.
void ref_stable_sort_rids(std::vector<uint32_t>& input,
                          std::vector<uint32_t>& rids) {
  const size_t size = input.size();
  rids.resize(size);
  std::vector<std::pair<uint32_t, uint32_t>> view;
  view.reserve(size);
  for (size_t i = 0; i < size; ++i) view.emplace_back(input[i], uint32_t(i));
  std::stable_sort(view.begin(), view.end(),
                   [](const std::pair<uint32_t, uint32_t>& l,
                      const std::pair<uint32_t, uint32_t>& r) {
                     return l.first < r.first;
                   });
  for (size_t i = 0; i < size; ++i) {
    input[i] = view[i].first;
    rids[i] = view[i].second;
  }
}
}  // namespace

extern "C" {

// Runs src/cpu.cpp:314-326 (bubble = 1 uses the reference's own O(n^2)
// sort_rids_by_value, src/cpu.cpp:180-197).  Output capacities: keys/offsets
// >= n, index >= 2n.  n == 0 is undefined in the reference and refused here.
int ref_wah_build(const uint32_t* values, uint64_t n, int bubble,
                  uint32_t* keys, uint32_t* offsets, uint32_t* index,
                  uint64_t* keycnt, uint64_t* index_len, uint64_t* merged) {
  if (n == 0) return -1;
  std::vector<uint32_t> input(values, values + n);
  std::vector<uint32_t> rids(n), chids(n), lits(n);
  if (bubble)
    sort_rids_by_value(input, rids);
  else
    ref_stable_sort_rids(input, rids);
  produce_chunk_id_literals(rids, chids, lits);
  auto k = merged_lit_by_val_chids(input, chids, lits);
  produce_fills(input, chids, k);
  std::vector<uint32_t> idx(2 * k);
  auto L = fuse_fill_literals(chids, lits, idx, k);
  std::vector<uint32_t> offs(k);
  auto K = compute_colum_length(input, chids, offs, k);
  std::memcpy(index, idx.data(), L * sizeof(uint32_t));
  std::memcpy(keys, input.data(), K * sizeof(uint32_t));
  std::memcpy(offsets, offs.data(), K * sizeof(uint32_t));
  *keycnt = K;
  *index_len = L;
  *merged = k;
  return 0;
}

// src/cpu.cpp:47-74.  Copies at most cap-1 characters plus NUL; returns the
// full length.
uint64_t ref_decoded_bitmap(const uint32_t* words, uint64_t len, char* out,
                            uint64_t cap) {
  std::vector<uint32_t> bm(words, words + len);
  std::string s = decoded_bitmap(bm);
  if (cap > 0) {
    size_t c = s.size() < cap - 1 ? s.size() : cap - 1;
    std::memcpy(out, s.data(), c);
    out[c] = '\0';
  }
  return s.size();
}

}  // extern "C"
