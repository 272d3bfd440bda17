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
#include <thread>
#include <unordered_map>
#include <vector>

namespace wahmerge {

class slice_merger {
 public:
  // threads: host threads a large slice is merged with (keys are independent)
  explicit slice_merger(unsigned threads = 1) : threads_(threads ? threads : 1) {}

  // Adds the index of rows [row_start, row_start + n): keys[K] ascending,
  // offsets[K], index[L].  row_start must be a multiple of 31 and not below
  // the previous slice's end.  Returns false (and adds nothing) otherwise.
  bool add(uint64_t row_start, uint64_t n, const uint32_t* keys, const uint32_t* offsets,
           uint32_t K, const uint32_t* index, uint32_t L) {
    if (row_start % 31 || row_start < next_row_) return false;
    const uint64_t first_chunk = row_start / 31;
    // the keys' entries first (map insertion is not thread-safe; references
    // to elements stay valid), then the keys merged independently
    std::vector<bitmap*> slot(K);
    for (uint32_t i = 0; i < K; ++i) slot[i] = &keys_[keys[i]];
    auto run = [&](uint32_t lo, uint32_t hi) {
      for (uint32_t i = lo; i < hi; ++i) {
        const uint32_t begin = offsets[i];
        const uint32_t end = (i + 1 < K) ? offsets[i + 1] : L;
        if (end > begin) merge_key(*slot[i], first_chunk, index + begin, end - begin);
      }
    };
    parallel_for(K, L, run);
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
    const uint32_t K = static_cast<uint32_t>(keys->size());
    std::vector<const std::vector<uint32_t>*> src(K);
    offsets->assign(K, 0);
    uint64_t total = 0;
    for (uint32_t i = 0; i < K; ++i) {
      src[i] = &keys_.at((*keys)[i]).words;
      (*offsets)[i] = static_cast<uint32_t>(total);
      total += src[i]->size();
    }
    index->resize(total);
    uint32_t* out = index->data();
    const uint32_t* off = offsets->data();
    parallel_for(K, total, [&](uint32_t lo, uint32_t hi) {
      for (uint32_t i = lo; i < hi; ++i) std::copy(src[i]->begin(), src[i]->end(), out + off[i]);
    });
  }

 private:
  struct bitmap {
    std::vector<uint32_t> words;
    uint64_t next_chunk = 0;  // first chunk after the key's last literal
  };

  static void merge_key(bitmap& b, uint64_t first_chunk, const uint32_t* w, uint32_t len) {
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
    for (uint32_t j = at; j < len; ++j) covered += (w[j] & 0x80000000u) ? 1u : (w[j] & 0x3FFFFFFFu);
    b.next_chunk = first_chunk + covered;
  }

  // fn(lo, hi) over [0, count) in threads_ chunks when the work (words) is
  // large enough to pay for the threads, else on this thread.
  template <class F>
  void parallel_for(uint32_t count, uint64_t work, F fn) const {
    const unsigned t = (work >= (1u << 20) && count >= 256) ? threads_ : 1u;
    if (t <= 1) {
      fn(0, count);
      return;
    }
    std::vector<std::thread> pool;
    const uint32_t per = (count + t - 1) / t;
    for (unsigned k = 1; k < t; ++k) {
      const uint32_t lo = k * per, hi = std::min<uint32_t>(count, lo + per);
      if (lo < hi) pool.emplace_back(fn, lo, hi);
    }
    fn(0, std::min<uint32_t>(count, per));
    for (auto& th : pool) th.join();
  }

  std::unordered_map<uint32_t, bitmap> keys_;
  uint64_t next_row_ = 0;
  unsigned threads_;
};

}  // namespace wahmerge
