/*
 * wah_oracle.h -- CPU restatement of the reference WAH index build.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the CUDA path is compared
 * against (tests, smoke check, and the CPU-baseline leg of the benchmark).
 * The product library never links, loads or calls it; there is no CPU
 * fallback in the product path.
 *
 * Each step restates one function of the reference's sequential `cpu`
 * program (src/cpu.cpp) and cites the lines it follows.  Parity of this
 * restatement is pinned against the reference source itself, compiled
 * unmodified through oracle/ref_cpu_shim.cpp, and against the golden vectors
 * in tests/golden/.
 */
#ifndef WAH_ORACLE_H
#define WAH_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Sort modes for wah_oracle_build. */
#define WAH_ORACLE_SORT_STABLE 0 /* stable merge sort, src/phases.cpp:143-160 */
#define WAH_ORACLE_SORT_BUBBLE 1 /* O(n^2) bubble sort, src/cpu.cpp:180-197   */

/*
 * Builds the WAH bitmap index of values[0..n) exactly as the reference `cpu`
 * program does (src/cpu.cpp:314-326).
 *
 * Outputs (caller-allocated):
 *   keys[K]     distinct values, ascending             (cap >= n)
 *   offsets[K]  first word of each key's bitmap        (cap >= n)
 *   index[L]    concatenated 32-bit WAH words          (cap >= 2n)
 *   *keycnt = K, *index_len = L, *merged = k (merged (value, chunk) entries)
 *
 * n == 0 yields K = L = k = 0 (the reference is undefined there).
 * Returns 0 on success, -1 when scratch memory cannot be allocated.
 */
int wah_oracle_build(const uint32_t* values, size_t n, int sort_mode,
                     uint32_t* keys, uint32_t* offsets, uint32_t* index,
                     size_t* keycnt, size_t* index_len, size_t* merged);

/* The individual steps, exposed for per-phase tests. */

/* src/cpu.cpp:180-197 (bubble) / src/phases.cpp:143-160 (stable sort). */
int wah_oracle_sort_rids_by_value(uint32_t* input, uint32_t* rids, size_t n,
                                  int sort_mode);

/* src/cpu.cpp:201-211. */
void wah_oracle_produce_chunk_id_literals(const uint32_t* rids, uint32_t* chids,
                                          uint32_t* lits, size_t n);

/* src/cpu.cpp:78-116 + :215-219: OR-reduce runs of equal (value, chid) in
 * place; returns k. */
size_t wah_oracle_merged_lit_by_val_chids(uint32_t* input, uint32_t* chids,
                                          uint32_t* lits, size_t n);

/* src/cpu.cpp:223-241: chids[0..k) become fill counts in place. */
void wah_oracle_produce_fills(const uint32_t* input, uint32_t* chids, size_t k);

/* src/cpu.cpp:245-257 + :170-174: interleave (fill, literal) into
 * index[0..2k), drop zero words; returns L. */
size_t wah_oracle_fuse_fill_literals(const uint32_t* fills, const uint32_t* lits,
                                     uint32_t* index, size_t k);

/* src/cpu.cpp:261-272 + :119-148 + :160-168: keys[K] and offsets[K]; returns K. */
size_t wah_oracle_compute_colum_length(const uint32_t* input,
                                       const uint32_t* fills, uint32_t* keys,
                                       uint32_t* offsets, size_t k);

/*
 * src/cpu.cpp:47-74: decodes one key's words into a '0'/'1' string with
 * trailing zeros trimmed.  Writes at most cap-1 characters plus a NUL into
 * out and returns the full decoded length (before truncation to cap).
 */
size_t wah_oracle_decoded_bitmap(const uint32_t* words, size_t len, char* out,
                                 size_t cap);

#ifdef __cplusplus
}
#endif

#endif /* WAH_ORACLE_H */
