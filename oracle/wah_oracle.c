/*
 * wah_oracle.c -- CPU restatement of the reference WAH index build.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path (tests, smoke
 * check, CPU-baseline leg of the benchmark).  Never linked into the product.
 *
 * Every function restates one step of the reference's sequential program
 * src/cpu.cpp (file:line given per function).  Word format (src/cpu.cpp:
 * 207-208, :55-69): a literal word has bit 31 set and bit (row % 31) for each
 * row of its 31-row chunk; a fill word has bit 31 clear, bit 30 = fill bit
 * (always 0 here, only zero-fills are produced) and bits 0..29 = number of
 * all-zero chunks.  No one-fills and no trailing fills are produced
 * (src/cpu.cpp:223-257).
 *
 * Plain C99, no platform intrinsics: builds and gives the same results on
 * x86-64 and aarch64.
 */
#include "wah_oracle.h"

#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* a1: sort_rids_by_value                                                    */
/* ------------------------------------------------------------------------ */

/* Bubble sort exactly as src/cpu.cpp:180-197: swaps only on strict '>', so it
 * is stable; O(n^2), usable only for small n. */
static void bubble_sort_rids(uint32_t* input, uint32_t* rids, size_t n) {
  for (size_t i = 0; i < n; ++i) rids[i] = (uint32_t)i;
  if (n < 2) return;
  for (size_t i = n - 1; i > 0; --i) {
    for (size_t j = 0; j < i; ++j) {
      if (input[j] > input[j + 1]) {
        uint32_t t = input[j];
        input[j] = input[j + 1];
        input[j + 1] = t;
        t = rids[j];
        rids[j] = rids[j + 1];
        rids[j + 1] = t;
      }
    }
  }
}

/* Stable sort by value carrying row ids, as src/phases.cpp:143-160 does with
 * std::stable_sort over (value, rid) pairs compared on the value only.  A
 * bottom-up merge sort on packed (value << 32 | rid) words; merges compare the
 * value half only and take the left run on ties, which is what makes it
 * stable.  Its output equals the bubble sort's (both are the unique stable
 * order). */
static int stable_sort_rids(uint32_t* input, uint32_t* rids, size_t n) {
  if (n == 0) return 0;
  uint64_t* a = (uint64_t*)malloc(n * sizeof(uint64_t));
  uint64_t* b = (uint64_t*)malloc(n * sizeof(uint64_t));
  if (!a || !b) {
    free(a);
    free(b);
    return -1;
  }
  for (size_t i = 0; i < n; ++i) a[i] = ((uint64_t)input[i] << 32) | (uint64_t)i;
  /* insertion sort of runs of 32 (stable: shifts only strictly greater) */
  const size_t RUN = 32;
  for (size_t s = 0; s < n; s += RUN) {
    size_t e = s + RUN < n ? s + RUN : n;
    for (size_t i = s + 1; i < e; ++i) {
      uint64_t x = a[i];
      uint32_t xv = (uint32_t)(x >> 32);
      size_t j = i;
      while (j > s && (uint32_t)(a[j - 1] >> 32) > xv) {
        a[j] = a[j - 1];
        --j;
      }
      a[j] = x;
    }
  }
  for (size_t width = RUN; width < n; width *= 2) {
    for (size_t lo = 0; lo < n; lo += 2 * width) {
      size_t mid = lo + width < n ? lo + width : n;
      size_t hi = lo + 2 * width < n ? lo + 2 * width : n;
      size_t i = lo, j = mid, o = lo;
      while (i < mid && j < hi) {
        /* take right only when strictly smaller: stability */
        if ((uint32_t)(a[j] >> 32) < (uint32_t)(a[i] >> 32))
          b[o++] = a[j++];
        else
          b[o++] = a[i++];
      }
      while (i < mid) b[o++] = a[i++];
      while (j < hi) b[o++] = a[j++];
    }
    uint64_t* t = a;
    a = b;
    b = t;
  }
  for (size_t i = 0; i < n; ++i) {
    input[i] = (uint32_t)(a[i] >> 32);
    rids[i] = (uint32_t)a[i];
  }
  free(a);
  free(b);
  return 0;
}

int wah_oracle_sort_rids_by_value(uint32_t* input, uint32_t* rids, size_t n,
                                  int sort_mode) {
  if (sort_mode == WAH_ORACLE_SORT_BUBBLE) {
    bubble_sort_rids(input, rids, n);
    return 0;
  }
  return stable_sort_rids(input, rids, n);
}

/* ------------------------------------------------------------------------ */
/* a2: produce_chunk_id_literals, src/cpu.cpp:201-211                        */
/* ------------------------------------------------------------------------ */
void wah_oracle_produce_chunk_id_literals(const uint32_t* rids, uint32_t* chids,
                                          uint32_t* lits, size_t n) {
  for (size_t i = 0; i < n; ++i) {
    lits[i] = (UINT32_C(1) << (rids[i] % 31)) | (UINT32_C(1) << 31);
    chids[i] = rids[i] / 31;
  }
}

/* ------------------------------------------------------------------------ */
/* a3: merged_lit_by_val_chids = reduce_by_key (OR), src/cpu.cpp:78-116,     */
/*     :215-219.  Runs of equal (value, chid) collapse to one entry whose     */
/*     literal is the OR of the run.  In place; returns k.                    */
/* ------------------------------------------------------------------------ */
size_t wah_oracle_merged_lit_by_val_chids(uint32_t* input, uint32_t* chids,
                                          uint32_t* lits, size_t n) {
  size_t from = 0, k = 0;
  while (from < n) {
    uint32_t v = input[from], c = chids[from];
    size_t to = from;
    uint32_t merged = 0;
    while (to < n && input[to] == v && chids[to] == c) merged |= lits[to++];
    input[k] = v;
    chids[k] = c;
    lits[k] = merged;
    ++k;
    from = to;
  }
  return k;
}

/* ------------------------------------------------------------------------ */
/* a4: produce_fills, src/cpu.cpp:223-241.  Entry e is a head when e == 0 or  */
/*     its value differs from entry e-1 (adjacent_difference with front = 1). */
/*     Head: fill = chid.  Otherwise fill = chid - prev_chid - 1 (u32).       */
/* ------------------------------------------------------------------------ */
void wah_oracle_produce_fills(const uint32_t* input, uint32_t* chids, size_t k) {
  if (k == 0) return;
  /* walk backwards so chids[i-1] is still the chunk id when entry i reads it */
  for (size_t i = k; i-- > 1;) {
    if (input[i] == input[i - 1]) chids[i] = chids[i] - chids[i - 1] - 1;
  }
  /* entry 0 is always a head: fill = chid, unchanged */
}

/* ------------------------------------------------------------------------ */
/* a5: fuse_fill_literals + stream_compaction(index, 0),                      */
/*     src/cpu.cpp:245-257, :170-174.  index = [fill_0, lit_0, fill_1, ...]   */
/*     with every zero word removed (only fills can be zero).                 */
/* ------------------------------------------------------------------------ */
size_t wah_oracle_fuse_fill_literals(const uint32_t* fills, const uint32_t* lits,
                                     uint32_t* index, size_t k) {
  size_t L = 0;
  for (size_t i = 0; i < k; ++i) {
    if (fills[i] != 0) index[L++] = fills[i];
    if (lits[i] != 0) index[L++] = lits[i];
  }
  return L;
}

/* ------------------------------------------------------------------------ */
/* a6: compute_colum_length, src/cpu.cpp:261-272.  tmp_e = 1 + (fill_e != 0) */
/*     (:264-266); reduce_by_key SUM keyed by value (:119-148) gives the      */
/*     distinct keys and per-key word counts; offsets = exclusive_scan of the */
/*     counts in u32 arithmetic (:160-168).  Returns K.                        */
/* ------------------------------------------------------------------------ */
size_t wah_oracle_compute_colum_length(const uint32_t* input,
                                       const uint32_t* fills, uint32_t* keys,
                                       uint32_t* offsets, size_t k) {
  size_t K = 0;
  uint32_t running = 0;
  size_t from = 0;
  while (from < k) {
    uint32_t v = input[from];
    uint32_t cnt = 0;
    size_t to = from;
    while (to < k && input[to] == v) {
      cnt += 1u + (fills[to] == 0 ? 0u : 1u);
      ++to;
    }
    keys[K] = v;
    offsets[K] = running;
    running += cnt;
    ++K;
    from = to;
  }
  return K;
}

/* ------------------------------------------------------------------------ */
/* Whole pipeline, in the order of src/cpu.cpp:318-326.                       */
/* ------------------------------------------------------------------------ */
int wah_oracle_build(const uint32_t* values, size_t n, int sort_mode,
                     uint32_t* keys, uint32_t* offsets, uint32_t* index,
                     size_t* keycnt, size_t* index_len, size_t* merged) {
  *keycnt = 0;
  *index_len = 0;
  if (merged) *merged = 0;
  if (n == 0) return 0;
  uint32_t* input = (uint32_t*)malloc(n * sizeof(uint32_t));
  uint32_t* rids = (uint32_t*)malloc(n * sizeof(uint32_t));
  uint32_t* chids = (uint32_t*)malloc(n * sizeof(uint32_t));
  uint32_t* lits = (uint32_t*)malloc(n * sizeof(uint32_t));
  int rc = -1;
  if (!input || !rids || !chids || !lits) goto out;
  memcpy(input, values, n * sizeof(uint32_t));
  if (wah_oracle_sort_rids_by_value(input, rids, n, sort_mode) != 0) goto out;
  wah_oracle_produce_chunk_id_literals(rids, chids, lits, n);
  {
    size_t k = wah_oracle_merged_lit_by_val_chids(input, chids, lits, n);
    wah_oracle_produce_fills(input, chids, k);
    *index_len = wah_oracle_fuse_fill_literals(chids, lits, index, k);
    *keycnt = wah_oracle_compute_colum_length(input, chids, keys, offsets, k);
    if (merged) *merged = k;
  }
  rc = 0;
out:
  free(input);
  free(rids);
  free(chids);
  free(lits);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* a7: decoded_bitmap, src/cpu.cpp:47-74.  Literal (bit 31 set): 31 bits,     */
/*     LSB first.  Fill: (bits 0..29) chunks of 31 copies of bit 30.          */
/*     Trailing '0's are trimmed.                                             */
/* ------------------------------------------------------------------------ */
size_t wah_oracle_decoded_bitmap(const uint32_t* words, size_t len, char* out,
                                 size_t cap) {
  size_t pos = 0, last_one = 0; /* last_one = 1 + index of last '1' */
  for (size_t w = 0; w < len; ++w) {
    uint32_t block = words[w];
    if (block & (UINT32_C(1) << 31)) {
      for (int i = 0; i < 31; ++i) {
        char c = (block >> i) & 1u ? '1' : '0';
        if (pos + 1 < cap) out[pos] = c;
        ++pos;
        if (c == '1') last_one = pos;
      }
    } else {
      char bit = (block & (UINT32_C(1) << 30)) ? '1' : '0';
      uint32_t times = block & ~(UINT32_C(3) << 30);
      for (uint32_t t = 0; t < times; ++t) {
        for (int j = 0; j < 31; ++j) {
          if (pos + 1 < cap) out[pos] = bit;
          ++pos;
          if (bit == '1') last_one = pos;
        }
      }
    }
  }
  if (cap > 0) out[last_one < cap ? last_one : cap - 1] = '\0';
  return last_one;
}
