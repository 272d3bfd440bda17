// merge.hpp -- joins the indexes of consecutive row slices of one column into
// the index of the whole column.
//
// The reference's `gpu` merger appends each slice's words to its key's
// bitmap (src/gpu.cpp:140-149).  A slice's bitmap is relative to the slice's
// first row and ends at its last literal, so plain appending loses the zero
// chunks between a key's last row in one slice and its first row in a later
// one.  Here each slice is re-based on its first chunk: its leading fill (the
// zero chunks before the key's first row in the slice, when there are any) is
// replaced by the zero chunks since the key's last literal in earlier slices
// and the rest is appended.  The result is word for word the index of the
// whole column (src/cpu.cpp:223-257 semantics: fill = chunk gap, no 1-fills,
// no trailing fill), provided every slice starts on a 31-row chunk boundary
// and slices are added in row order.
#pragma once

#include <algorithm>
#include <cstdint>
#include <unordered_map>
#include <vector>

namespace wahmerge {

class slice_merger {
 public:
  // Adds the index of rows [row_start, row_start + n): keys[K] ascending,
  // offsets[K], index[L].  row_start must be a multiple of 31 and not below
  // the previous slice's end.  Returns false (and adds nothing) otherwise.
  bool add(uint64_t row_start, uint64_t n, const uint32_t* keys, const uint32_t* offsets,
           uint32_t K, const uint32_t* index, uint32_t L) {
    if (row_start % 31 || row_start < next_row_) return false;
    const uint64_t first_chunk = row_start / 31;
    for (uint32_t i = 0; i < K; ++i) {
      const uint32_t begin = offsets[i];
      const uint32_t end = (i + 1 < K) ? offsets[i + 1] : L;
      if (end <= begin) continue;
      const uint32_t* w = index + begin;
      const uint32_t len = end - begin;
      bitmap& b = keys_[keys[i]];
      uint32_t at = 0;
      uint64_t lead = 0;  // zero chunks before the key's first row in the slice
      if (!(w[0] & 0x80000000u)) {
        lead = w[0] & 0x3FFFFFFFu;
        at = 1;
      }
      const uint64_t gap = first_chunk + lead - b.next_chunk;
      if (gap) b.words.push_back(static_cast<uint32_t>(gap));
      b.words.insert(b.words.end(), w + at, w + len);
      uint64_t covered = lead;
      for (uint32_t j = at; j < len; ++j)
        covered += (w[j] & 0x80000000u) ? 1u : (w[j] & 0x3FFFFFFFu);
      b.next_chunk = first_chunk + covered;
    }
    next_row_ = row_start + n;
    return true;
  }

  // Rows covered so far (the end of the last slice added).
  uint64_t rows() const { return next_row_; }

  // One key's merged words (nullptr if the key never occurred).
  const std::vector<uint32_t>* words(uint32_t key) const {
    auto it = keys_.find(key);
    return it == keys_.end() ? nullptr : &it->second.words;
  }

  // The whole index: keys ascending, offsets, concatenated words.
  void finish(std::vector<uint32_t>* keys, std::vector<uint32_t>* offsets,
              std::vector<uint32_t>* index) const {
    keys->clear();
    keys->reserve(keys_.size());
    for (const auto& kv : keys_) keys->push_back(kv.first);
    std::sort(keys->begin(), keys->end());
    offsets->assign(keys->size(), 0);
    index->clear();
    for (size_t i = 0; i < keys->size(); ++i) {
      (*offsets)[i] = static_cast<uint32_t>(index->size());
      const auto& w = keys_.at((*keys)[i]).words;
      index->insert(index->end(), w.begin(), w.end());
    }
  }

 private:
  struct bitmap {
    std::vector<uint32_t> words;
    uint64_t next_chunk = 0;  // first chunk after the key's last literal
  };
  std::unordered_map<uint32_t, bitmap> keys_;
  uint64_t next_row_ = 0;
};

}  // namespace wahmerge
