/*
 * wah.h -- C ABI of the GB300 WAH bitmap index builder.
 *
 * One call builds the WAH bitmap index of a uint32 column on the GPU:
 *   keys[K]     the distinct values, ascending
 *   offsets[K]  position of each key's first word in index (u32)
 *   index[L]    the concatenated 32-bit WAH words of all keys
 * bit-exact with the reference's sequential `cpu` program
 * (src/cpu.cpp:314-326).  Word format (src/cpu.cpp:201-211, :47-74): a literal
 * has bit 31 set and bit (row % 31) for each row of its 31-row chunk; a fill
 * has bit 31 clear and its low 30 bits count all-zero chunks.  Only zero
 * fills are produced, never a trailing fill, and a full chunk stays a
 * 0xFFFFFFFF literal.
 *
 * The reference drives the same path through CAF's OpenCL actor facade
 * (caf::opencl::manager::spawn(program, kernel, nd_range, in/out tags...),
 * src/phases.cpp:480-712, and the single-kernel variant src/gpu.cpp:356-367),
 * moving data with dev->global_argument / mem_ref::data (src/phases.cpp:720,
 * :1087-1088).  These entry points replace that facade: plain pointers and
 * sizes, caller-owned device buffers, stream-ordered, never aborting.
 *
 * All device pointers must be 16-byte aligned (cudaMalloc gives 256).
 * Functions return a WAH_* status; asynchronous device-side errors land in
 * wah_counts.status and are valid after the stream is synchronised.
 */
#ifndef WAH_WAH_H
#define WAH_WAH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference exits the process on any failure
 * (valid_or_exit, src/phases.cpp:102-112); here every failure is a code. */
#define WAH_OK 0
#define WAH_EINVAL 1    /* null/misaligned pointer, bad size               */
#define WAH_ENOMEM 2    /* workspace too small / allocation failed          */
#define WAH_ECUDA 3     /* a CUDA runtime call failed                       */
#define WAH_ETIMEOUT 4  /* a bounded device-side wait gave up               */
#define WAH_ERANGE 5    /* n >= 2^31, or a value above the stated bound     */
#define WAH_EOVERFLOW 6 /* an output would exceed the caller's capacity     */
#define WAH_ENODEV 7    /* no usable sm_103 device                          */
#define WAH_ECORRUPT 8  /* index words do not describe the stated rows      */

/* Largest column one call accepts (rows).  Offsets and index positions are
 * u32 as in the reference (src/cpu.cpp:261-272); with n < 2^31 rows a
 * column's index holds L <= 2n < 2^32 words, so every row, word and key
 * position stays within u32. */
#define WAH_MAX_ROWS ((uint64_t)1 << 31)

/* Device-written result counters (16 bytes). */
typedef struct wah_counts {
  uint32_t keycnt;    /* K: distinct values (keycount, src/phases.cpp:1052)   */
  uint32_t index_len; /* L: index words (index_length, src/phases.cpp:974)     */
  uint32_t merged;    /* k: merged (value, chunk) entries (src/cpu.cpp:320)    */
  uint32_t status;    /* WAH_OK or the first device-side error                 */
} wah_counts;

/* Human-readable name of a status code. */
const char* wah_strerror(int status);

/* Output capacities a caller must provide for a column of n rows whose
 * values are all <= bound (bound == 0: unknown, any uint32).
 * keys_cap = offsets_cap = min(n, bound + 1) (n when bound == 0);
 * index_cap = 2n (L <= 2k <= 2n).  Replaces the reference's size lambdas
 * (k_double, fills_k, ..., src/phases.cpp:405-438). */
void wah_output_caps(uint64_t n, uint32_t bound, uint64_t* keys_cap,
                     uint64_t* index_cap);

/* Device workspace bytes wah_build needs for n rows.  Replaces the
 * reference's scratch_argument buffers (src/phases.cpp:749-753). */
size_t wah_workspace_bytes(uint64_t n, uint32_t bound);

/*
 * Builds the index of d_values[0..n) (device memory) on `stream`
 * (a cudaStream_t; NULL = legacy default stream).  The whole of
 * src/cpu.cpp:318-326 / src/phases.cpp:730-1077: sort_rids_by_value,
 * produce_chunk_id_literals, merged_lit_by_val_chids, produce_fills,
 * fuse_fill_literals, compute_colum_length.
 *
 * bound: largest value in the column, or 0 to let the device find out
 * (the reference's -b/--bound flag, src/cpu.cpp:306-310).  With a bound the
 * sort runs ceil(bits(bound)/8) digit passes; values above it are reported
 * as WAH_ERANGE in d_counts->status.
 * d_keys/d_offsets: capacity from wah_output_caps; d_index: 2n words.
 * d_counts: device wah_counts (16-byte aligned), cleared by the build's
 * first kernel and written at its end; a call that returns an error code
 * before enqueueing anything leaves it untouched.
 * The call enqueues work and returns; nothing is synchronised.
 * n == 0 writes K = L = 0 (the reference is undefined there).
 */
int wah_build(const uint32_t* d_values, uint64_t n, uint32_t bound,
              uint32_t* d_keys, uint32_t* d_offsets, uint32_t* d_index,
              wah_counts* d_counts, void* d_workspace, size_t workspace_bytes,
              void* stream);

/*
 * wah_build with the tile shapes of this call given (the reference's radix
 * shape is fixed, src/phases.cpp:445-453): `tuning` is a tuning word as
 * wah_set_tuning takes -- for instance the one wah_autotune_workload chose
 * for this kind of column -- or 0 for the process default.  Builds with
 * different words may run at the same time.  WAH_EINVAL for a word that
 * wah_set_tuning would refuse.
 */
int wah_build_tuned(const uint32_t* d_values, uint64_t n, uint32_t bound,
                    uint32_t* d_keys, uint32_t* d_offsets, uint32_t* d_index,
                    wah_counts* d_counts, void* d_workspace,
                    size_t workspace_bytes, int tuning, void* stream);

/*
 * wah_build for callers that cannot allocate device memory (no counterpart in
 * the reference).  An ingest plugin whose host engine owns the device memory
 * pool, or a serving loop that cannot afford the device synchronisation of
 * cudaMalloc/cudaFree, passes only the column and the output buffers; the
 * build's scratch memory is a fixed array in the library's device image
 * (24 MiB, held by every GPU that loads the library until exit).  Columns of
 * up to WAH_NOALLOC_MAX_ROWS rows; larger n returns WAH_ERANGE without
 * enqueueing anything (d_counts is left untouched then, so it does not hold
 * this call's result).  Calls no allocator.  All calls share the array:
 * calls whose work overlaps on the GPU (unordered streams or host threads)
 * race.  The array has its own address in every CUDA context (primary or
 * created by the caller); each call looks it up in the context current on
 * the calling thread.  The first call in a context may load the library's
 * device code there; make it before any stream capture.
 */
#define WAH_NOALLOC_MAX_ROWS ((uint64_t)1 << 20)
int wah_build_noalloc(const uint32_t* d_values, uint64_t n, uint32_t bound,
                      uint32_t* d_keys, uint32_t* d_offsets, uint32_t* d_index,
                      wah_counts* d_counts, void* stream);

/*
 * Phase a1 alone: stable sort of d_values by value carrying row ids
 * (src/cpu.cpp:180-197 semantics; src/phases.cpp:730-773 on the GPU).
 * Writes d_sorted_values[n] and d_rids[n].  Same bound and workspace rules as
 * wah_build.  d_status (optional, device u32) receives WAH_OK / error.
 */
int wah_sort_rids_by_value(const uint32_t* d_values, uint64_t n,
                           uint32_t bound, uint32_t* d_sorted_values,
                           uint32_t* d_rids, uint32_t* d_status,
                           void* d_workspace, size_t workspace_bytes,
                           void* stream);

/*
 * Phases a2-a6 fused, on an already sorted (value, rid) stream
 * (src/cpu.cpp:319-326; src/phases.cpp:817-1077): chunk ids and literals,
 * OR-merge per (value, chunk), fills, compaction into index, per-key counts
 * and offsets.  Workspace: wah_workspace_bytes(n, bound) suffices.
 */
int wah_build_sorted(const uint32_t* d_sorted_values, const uint32_t* d_rids,
                     uint64_t n, uint32_t* d_keys, uint32_t* d_offsets,
                     uint32_t* d_index, wah_counts* d_counts,
                     void* d_workspace, size_t workspace_bytes, void* stream);

/*
 * Host-buffer convenience path: the reference `phases` flow end to end
 * (global_argument -> phases -> mem_ref::data, src/phases.cpp:720-1088).
 * A context owns device buffers sized for columns up to max_n rows, a
 * stream and a copy of the result counters.  Host buffers may be pageable or
 * pinned (pinned is faster).  wah_ctx_build_host copies values in, builds,
 * and copies keys[K], offsets[K], index[L] out; it returns when they are in
 * host memory.  Host capacities as wah_output_caps.
 */
typedef struct wah_ctx wah_ctx;
int wah_ctx_create(uint64_t max_n, uint32_t bound, wah_ctx** out);
int wah_ctx_build_host(wah_ctx* ctx, const uint32_t* h_values, uint64_t n,
                       uint32_t* h_keys, uint32_t* h_offsets, uint32_t* h_index,
                       wah_counts* h_counts);
void wah_ctx_destroy(wah_ctx* ctx);

/*
 * Batched builds: many columns, each indexed exactly as wah_build would index
 * it alone, with every kernel of the pipeline launched once for the whole
 * batch (the reference's single-kernel batch path, kernel_wah_index in
 * include/kernel_wah_bitindex.cl:43-91 driven by src/gpu.cpp:194-259,
 * indexes each <=1,023-row batch separately).  wah_batch_create plans a batch
 * for given row counts and bounds (host arrays) and allocates its device
 * memory; wah_batch_set_columns sets the columns' device buffers (their n and
 * bound must match the plan; values 16-byte aligned; outputs with
 * wah_output_caps capacities; counts 16-byte aligned) by an upload enqueued
 * on `stream`; wah_batch_build enqueues the build (no allocation, no host
 * synchronisation); wah_batch_launch_graph captures that build into a CUDA
 * graph on its first call and replays it, so new columns of the same sizes
 * need only wah_batch_set_columns + a replay.  Results and errors are in each
 * column's counts.
 */
typedef struct wah_column {
  const uint32_t* values; /* device, n values                         */
  uint64_t n;
  uint32_t bound;         /* largest value, 0 = unknown               */
  uint32_t reserved;
  uint32_t* keys;         /* device outputs                           */
  uint32_t* offsets;
  uint32_t* index;
  wah_counts* counts;     /* device                                   */
} wah_column;

typedef struct wah_batch wah_batch;
int wah_batch_create(const uint64_t* ns, const uint32_t* bounds, uint32_t ncols,
                     wah_batch** out);
/* The same with the batch's own tuning word (0 = the process default). */
int wah_batch_create_tuned(const uint64_t* ns, const uint32_t* bounds,
                           uint32_t ncols, int tuning, wah_batch** out);
int wah_batch_set_columns(wah_batch* batch, const wah_column* cols, void* stream);
int wah_batch_build(wah_batch* batch, void* stream);
int wah_batch_launch_graph(wah_batch* batch, void* stream);
size_t wah_batch_device_bytes(const wah_batch* batch);
uint32_t wah_batch_ranges(const wah_batch* batch);
void wah_batch_destroy(wah_batch* batch);

/*
 * Continuous-batching index server.  Requests (a host column each, with an
 * arrival delay from now) are admitted in arrival order while their device
 * memory fits `budget_bytes` (one device arena, allocated at create), batched
 * into the batched build (up to max_batch columns per batch, `streams`
 * batches in flight), and completed asynchronously; the outputs stay
 * resident on the device until released.  The reference's `gpu` program
 * keeps --jobs batches in flight between its indexer and merger actors
 * (src/gpu.cpp:103-261).  plain != 0 builds every request alone with
 * wah_build, one at a time (the per-request baseline).  h_values must stay
 * valid until the request completes.  A request that cannot fit the budget
 * even alone is refused with WAH_ENOMEM.  An arrived request that finds no
 * room waits for batches to finish and for results to be released; with
 * nothing in flight it fails with WAH_ENOMEM once no released result can
 * make room (none held, or none released for 2 s while it waits: a client
 * waiting for it while holding the results that block it).  Releasing each
 * result once read keeps the arena free.  wah_server_wait blocks until the
 * request is done and fills `result` (device pointers valid until
 * wah_server_release; latency = completion - arrival).
 */
typedef struct wah_server wah_server;
typedef struct wah_server_result {
  wah_counts counts;
  uint32_t* keys; /* device */
  uint32_t* offsets;
  uint32_t* index;
  double latency_s; /* completion - arrival */
  double queue_s;   /* admission - arrival */
} wah_server_result;
int wah_server_create(uint64_t budget_bytes, uint32_t max_batch, uint32_t streams,
                      int plain, wah_server** out);
/* The same with the server's own tuning word for all its builds (0 = the
 * process default). */
int wah_server_create_tuned(uint64_t budget_bytes, uint32_t max_batch,
                            uint32_t streams, int plain, int tuning,
                            wah_server** out);
int wah_server_submit(wah_server* server, const uint32_t* h_values, uint64_t n,
                      uint32_t bound, double arrival_delay_s, uint64_t* id);
int wah_server_wait(wah_server* server, uint64_t id, wah_server_result* result);
int wah_server_release(wah_server* server, uint64_t id);
/* Copies a completed request's keys[K], offsets[K], index[L] into caller
 * device buffers on `stream` (before releasing it). */
int wah_server_copy_out(wah_server* server, uint64_t id, uint32_t* d_keys,
                        uint32_t* d_offsets, uint32_t* d_index, void* stream);
uint64_t wah_server_arena_used(wah_server* server);
void wah_server_destroy(wah_server* server);

/*
 * Pipelined host-buffer builds: the reference's per-column flow
 * (global_argument -> phases -> mem_ref::data, src/phases.cpp:720-1088) with
 * several columns in flight, like `gpu --jobs` (src/gpu.cpp:194-259).  A pipe
 * owns `depth` (1..8) slots of device buffers for columns of up to max_n
 * rows, each with its own stream, and a completion thread.  wah_pipe_submit
 * enqueues the copy of h_values in and the build, and returns a ticket
 * without waiting (unless every slot is busy: then it first waits for the
 * oldest build); the completion thread copies exactly keys[K], offsets[K],
 * index[L] and the counters out once the build's sizes are known.
 * Consecutive submits overlap on the GPU and on the host link.  h_values
 * must stay unchanged, and the output buffers (capacities as
 * wah_output_caps) untouched, until wah_pipe_wait(ticket) returns; the
 * outputs are valid when it returns WAH_OK and h_counts->status == WAH_OK.
 * Pinned host buffers (cudaHostAlloc / cudaMallocHost / cudaHostRegister)
 * copy fastest; pageable ones work.  A pipe is driven by one host thread.
 */
typedef struct wah_pipe wah_pipe;
int wah_pipe_create(uint64_t max_n, uint32_t bound, uint32_t depth,
                    wah_pipe** out);
int wah_pipe_submit(wah_pipe* pipe, const uint32_t* h_values, uint64_t n,
                    uint32_t* h_keys, uint32_t* h_offsets, uint32_t* h_index,
                    wah_counts* h_counts, uint64_t* ticket);
int wah_pipe_wait(wah_pipe* pipe, uint64_t ticket);
void wah_pipe_destroy(wah_pipe* pipe);

/*
 * Thin device helpers so host programs need only this header: device
 * discovery and selection (the reference picks a device by name or the first
 * available one, src/phases.cpp:376-388), device/pinned allocation, copies in
 * either direction (cudaMemcpyDefault semantics; global_argument and
 * mem_ref::data, src/phases.cpp:720, :1087-1088) and streams.
 */
int wah_device_count(void);
int wah_device_name(int device, char* out, size_t cap);
int wah_device_select(int device);
int wah_dev_alloc(size_t bytes, void** out);
void wah_dev_free(void* ptr);
int wah_host_alloc(size_t bytes, void** out);
void wah_host_free(void* ptr);
int wah_copy(void* dst, const void* src, size_t bytes, void* stream);
int wah_stream_create(void** out);
int wah_stream_sync(void* stream);
void wah_stream_destroy(void* stream);

/*
 * Decoding a built index on the device: the reference's decoded_bitmap
 * (src/cpu.cpp:47-74; src/gpu.cpp:65-94) reads one key's words into a
 * '0'/'1' string on the host; wah_decode reads every key's words at once.
 * Inputs: keys[K], offsets[K], index[L] of a column of n rows (device).
 * Optional outputs (device, NULL to skip):
 *   d_rows[n]        row ids, keys ascending, rows ascending within a key
 *                    (the stable sort's rid order)
 *   d_row_values[n]  the key of each of those rows (the sorted column)
 *   d_column[n]      the column itself: d_column[row] = its value
 *   d_key_rows[K]    position in d_rows of each key's first row
 * d_status (device u32): WAH_OK, or WAH_ECORRUPT when a row falls outside
 * [0, n) or the words hold a number of rows other than n.  Workspace:
 * wah_decode_workspace_bytes().  Enqueues on `stream`, no synchronisation.
 */
size_t wah_decode_workspace_bytes(void);
int wah_decode(const uint32_t* d_keys, const uint32_t* d_offsets,
               const uint32_t* d_index, uint32_t keycnt, uint32_t index_len,
               uint64_t n, uint32_t* d_rows, uint32_t* d_row_values,
               uint32_t* d_column, uint32_t* d_key_rows, uint32_t* d_status,
               void* d_workspace, size_t workspace_bytes, void* stream);

/*
 * Queries on a built index (no counterpart in the reference, which stops at
 * decoding).  Term A = rows whose value is in [a_lo, a_hi]; with op
 * WAH_QUERY_OR / _AND / _ANDNOT, term B = [b_lo, b_hi] combines with it
 * (A|B, A&B, A&~B); WAH_QUERY_KEYS is A alone.  A single key is
 * [v, v]; a value range is a range of keys.  Outputs (device, NULL to skip):
 *   d_words[words]  the result as a WAH bitmap in the index's format
 *                   (literal per non-empty chunk, fills for gaps, no
 *                   trailing fill): for one key, exactly its own words;
 *                   capacity 2 * ceil(n / 31) always suffices
 *   d_rows[rows]    the result's row ids, ascending; capacity n suffices
 * d_result (device, 16-byte aligned) receives words, rows and a status
 * (WAH_EOVERFLOW when a capacity was too small: counts stay exact, the
 * outputs are cut).  Workspace: wah_query_workspace_bytes(n).
 */
#define WAH_QUERY_KEYS 0
#define WAH_QUERY_OR 1
#define WAH_QUERY_AND 2
#define WAH_QUERY_ANDNOT 3
typedef struct wah_query_result {
  uint32_t words;
  uint32_t rows;
  uint32_t status;
  uint32_t reserved;
} wah_query_result;
size_t wah_query_workspace_bytes(uint64_t n);
int wah_query(const uint32_t* d_keys, const uint32_t* d_offsets,
              const uint32_t* d_index, uint32_t keycnt, uint32_t index_len,
              uint64_t n, uint32_t a_lo, uint32_t a_hi, int op, uint32_t b_lo,
              uint32_t b_hi, uint32_t* d_words, uint64_t words_cap,
              uint32_t* d_rows, uint64_t rows_cap, wah_query_result* d_result,
              void* d_workspace, size_t workspace_bytes, void* stream);

/*
 * Text ingest on the device.  The reference reads its columns from text
 * files, one value per line, with `while (source >> next)`
 * (src/cpu.cpp:297-302; files from src/generate_test_data.cpp:45-53).
 * wah_parse_text parses d_text[0..bytes) (device, 16-byte aligned) the same
 * way: tokens are separated by whitespace (space, \t \n \v \f \r); a token
 * of decimal digits whose value fits in 32 bits is a value (leading zeros
 * allowed; signs are not); parsing stops at the first token that is not
 * one.  Value i goes to d_values[i] (capacity `capacity`; more values set
 * WAH_EOVERFLOW, the count stays exact).  d_result (device, 16-byte
 * aligned) receives the number of values, of tokens, the largest value and
 * a status.  Workspace: wah_parse_workspace_bytes().  Enqueues on `stream`.
 */
typedef struct wah_parse_result {
  uint64_t values;    /* values parsed (tokens before the first invalid one) */
  uint64_t tokens;    /* all tokens                                          */
  uint32_t max_value; /* largest of the values (0 if none)                   */
  uint32_t status;    /* WAH_OK or WAH_EOVERFLOW                             */
  uint64_t reserved;
} wah_parse_result;
size_t wah_parse_workspace_bytes(void);
int wah_parse_text(const void* d_text, uint64_t bytes, uint32_t* d_values,
                   uint64_t capacity, wah_parse_result* d_result,
                   void* d_workspace, size_t workspace_bytes, void* stream);

/*
 * Launch-overhead measurements (the reference's overhead_benchmark sends an
 * empty kernel through the actor facade, src/overhead_benchmark.cpp:64-148,
 * include/empty_kernel.cl): wah_noop enqueues one empty kernel on `stream`;
 * a noop graph holds `count` empty kernels captured once into a CUDA graph,
 * replayed by wah_noop_graph_launch.
 */
typedef struct wah_noop_graph wah_noop_graph;
int wah_noop(void* stream);
int wah_noop_graph_create(uint32_t count, wah_noop_graph** out);
int wah_noop_graph_launch(wah_noop_graph* graph, void* stream);
void wah_noop_graph_destroy(wah_noop_graph* graph);

/*
 * Incremental append on the device.  A = the index (keys, offsets, index) of
 * rows [0, rows_a) of a column, B = the index of the next rows [rows_a,
 * rows_a + n) built alone (rows_a a multiple of 31).  wah_append writes the
 * index of all rows_a + n rows -- word for word what one build of the whole
 * column gives -- to out_* (keys_cap >= keycnt_a + keycnt_b, index_cap >=
 * index_len_a + index_len_b + keycnt_b).  The reference's `gpu` merger
 * appends slice bitmaps without re-basing their leading fills
 * (src/gpu.cpp:103-165); here B's leading fill per key becomes the zero
 * chunks since the key's last row in A.  d_counts receives K, L and a
 * status (WAH_ECORRUPT when A has rows at or past rows_a).  All pointers are
 * device memory; workspace wah_append_workspace_bytes(keycnt_a, keycnt_b).
 * out_index past the result's L words is scratch during the call (a table
 * of index_len_a / 4,096 words sits at its end before the words are
 * written).
 */
size_t wah_append_workspace_bytes(uint32_t keycnt_a, uint32_t keycnt_b);
int wah_append(const uint32_t* a_keys, const uint32_t* a_offsets,
               const uint32_t* a_index, uint32_t keycnt_a, uint32_t index_len_a,
               uint64_t rows_a, const uint32_t* b_keys, const uint32_t* b_offsets,
               const uint32_t* b_index, uint32_t keycnt_b, uint32_t index_len_b,
               uint32_t* out_keys, uint32_t* out_offsets, uint32_t* out_index,
               uint64_t keys_cap, uint64_t index_cap, wah_counts* d_counts,
               void* d_workspace, size_t workspace_bytes, void* stream);

/* Number of kernels the last wah_build/wah_ctx_build_host on this thread
 * enqueued (launch accounting for benchmarks). */
uint32_t wah_last_launch_count(void);

/* Tile shape of the radix digit passes: rows per thread (8, 12 or 16;
 * 256 threads per tile), optionally OR WAH_TUNE_MATCH to build the digit
 * peer masks with match.any instead of ballots, or WAH_TUNE_HYBRID to build
 * 3/8 of them with match.any and the rest with ballots.  That shape applies
 * to digit pass 0; WAH_TUNE_LATER(shape) ORed in gives one-column index
 * builds (wah_build and its host-buffer forms; not the sort alone) a
 * different shape for the later passes (0: the same).  Process-wide; set by
 * the autotuner or the caller before builds are enqueued; the default is
 * 16 | WAH_TUNE_HYBRID | WAH_TUNE_LATER(12 | WAH_TUNE_HYBRID).  The reference
 * hard-codes its radix shape (src/phases.cpp:445-453). */
#define WAH_TUNE_MATCH 0x100
#define WAH_TUNE_HYBRID 0x200
/* In the shape of digit pass 0: one-column index builds whose keys all fit
 * 16 bits exchange one packed word per row between the two digit passes
 * (row offset in its pass-0 range and high digit) whatever the length of
 * pass 0's runs; without it they do so only when pass-0 ranges hold at least
 * 65,536 rows, and a 16-bit key beside a row id otherwise. */
#define WAH_TUNE_PACK 0x400
#define WAH_TUNE_LATER(shape) ((shape) << 16)
int wah_set_tuning(int sort_items);
int wah_get_tuning(void);

/*
 * Autotuner: times every tile shape for all digit passes, then every other
 * shape for the passes after the first (WAH_TUNE_LATER), then the packed
 * exchange (WAH_TUNE_PACK) on and off, by index builds of a synthetic column
 * of n rows with values uniform up to bound (the reference's radix shape is
 * fixed, src/phases.cpp:445-453; its radix test program takes it as flags,
 * src/radix.cpp:161-184), applies the fastest as the process default, and
 * appends it to the text file cache_path (NULL: no cache) under the key
 * (device name, workload "uniform", floor(log2 n), digit passes, format tag
 * "t3").  When the cache already holds the key, its entry is applied without
 * timing and *from_cache is 1.  Allocates and frees its own device memory;
 * synchronises.  *chosen receives the tuning applied.  Candidates are timed
 * with the word passed per build, so concurrent builds keep their own shapes.
 */
int wah_autotune(uint64_t n, uint32_t bound, const char* cache_path, int* chosen,
                 int* from_cache);

/*
 * Autotuning for one kind of workload, applied nowhere: *chosen receives the
 * tuning word to pass to wah_build_tuned, wah_batch_create_tuned or
 * wah_server_create_tuned.  workload: WAH_WORKLOAD_UNIFORM (one column of n
 * rows, values uniform in [0, bound]), WAH_WORKLOAD_SKEWED (one column, a
 * power law over [0, bound]: a few values hold most rows) or
 * WAH_WORKLOAD_BATCH (a batch of ncols columns of about n rows in all, row
 * counts log-uniform, each column's values uniform below its own log-uniform
 * cardinality; the batch uses the shape of digit pass 0 for every pass).
 * Times every tile shape (one-column workloads: then every other shape for
 * the later passes, and the packed exchange on and off) and caches the
 * choice under (device, workload, size bucket, digit passes) in cache_path
 * like wah_autotune.  Allocates and frees its own device memory; synchronises.
 */
#define WAH_WORKLOAD_UNIFORM 0
#define WAH_WORKLOAD_SKEWED 1
#define WAH_WORKLOAD_BATCH 2
int wah_autotune_workload(int workload, uint64_t n, uint32_t bound, uint32_t ncols,
                          const char* cache_path, int* chosen, int* from_cache);

/*
 * Per-phase device timing, the counterpart of the reference's
 * SHOW_TIME_CONSUMPTION "N us" lines (src/phases.cpp:714-1127), measured with
 * CUDA events on the build's own stream instead of host clocks around
 * synchronisations.  wah_build_timed is wah_build plus event records around
 * each kernel: events[2p] before and events[2p+1] after phase p, for the
 * WAH_TIMED_PHASES phases: 0 histogram, 1 plan, 2..5 digit passes 0..3
 * (count, scan and scatter), 6 index build (count, scan, emit), and single
 * kernels inside them: 7..10 the scatter kernel of passes 0..3, 11 the
 * build's emit kernel (a pass that is not launched gets empty spans).
 * Events come from wah_events_create; durations from wah_events_elapsed
 * after a sync.
 */
#define WAH_TIMED_PHASES 12
int wah_events_create(uint32_t count, void** events);
void wah_events_destroy(uint32_t count, void** events);
int wah_events_elapsed(void* start, void* end, float* ms);
int wah_build_timed(const uint32_t* d_values, uint64_t n, uint32_t bound,
                    uint32_t* d_keys, uint32_t* d_offsets, uint32_t* d_index,
                    wah_counts* d_counts, void* d_workspace,
                    size_t workspace_bytes, void* stream, void** events);

#ifdef __cplusplus
}
#endif

#endif /* WAH_WAH_H */
