// wah_tune.cu -- autotuner of the radix tile shape, with a cache file.
//
// The reference hard-codes its radix parameters (src/phases.cpp:445-453:
// 4-bit digits, 8 blocks of 1024 threads); its stale `radix` test program
// exposes them as flags (src/radix.cpp:161-184).  Here every compiled tile
// shape of the digit passes -- rows per thread 8, 12 or 16, peer masks from
// ballots, match.any or half of each -- is timed on a synthetic column of the
// caller's size and bound, then every other shape for the passes after the
// first one; the fastest is applied (wah_set_tuning), and the
// choice is remembered per (device, size bucket, digit passes) in a text
// cache file, so later processes apply it without timing.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "wah_common.cuh"

namespace wah {
namespace {

// Row i of the synthetic column: a hash of i, folded below bound + 1.
__global__ void k_tune_column(uint32_t* v, uint64_t n, uint32_t bound) {
  const uint64_t range = (uint64_t)bound + 1;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t z = i + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    v[i] = bound == 0 ? (uint32_t)z : (uint32_t)((z >> 32) * range >> 32);
  }
}

// Every tuning value wah_set_tuning accepts.
const int kCandidates[] = {16, 12, 8, 16 | WAH_TUNE_MATCH, 12 | WAH_TUNE_MATCH,
                           8 | WAH_TUNE_MATCH, 16 | WAH_TUNE_HYBRID, 12 | WAH_TUNE_HYBRID,
                           8 | WAH_TUNE_HYBRID};

std::mutex g_tune_mu;

std::string cache_key(int device, uint64_t n, uint32_t bound) {
  cudaDeviceProp p;
  std::string name = cudaGetDeviceProperties(&p, device) == cudaSuccess ? p.name : "unknown";
  for (char& c : name)
    if (c == ' ' || c == '\t') c = '_';
  int bucket = 0;
  while (bucket < 63 && (2ull << bucket) <= n) ++bucket;  // floor(log2 n)
  // "t2": entries that hold a later-pass shape (older entries are timed again)
  return name + " " + std::to_string(bucket) + " " + std::to_string(passes_for_bound(bound)) +
         " t2";
}

bool cache_lookup(const char* path, const std::string& key, int* tuning) {
  FILE* f = path ? std::fopen(path, "r") : nullptr;
  if (!f) return false;
  char line[512];
  bool found = false;
  while (std::fgets(line, sizeof line, f)) {
    const size_t len = std::strlen(line);
    if (len <= key.size() || std::strncmp(line, key.c_str(), key.size()) != 0 ||
        line[key.size()] != ' ')
      continue;
    int t = 0;
    if (std::sscanf(line + key.size() + 1, "%d", &t) == 1) {
      *tuning = t;  // the last entry of a key wins
      found = true;
    }
  }
  std::fclose(f);
  return found;
}

int timed_build(const uint32_t* v, uint64_t n, uint32_t bound, uint32_t* keys, uint32_t* offs,
                uint32_t* index, wah_counts* counts, void* ws, size_t ws_bytes, cudaStream_t s,
                cudaEvent_t a, cudaEvent_t b, int reps, float* ms) {
  int rc = wah_build(v, n, bound, keys, offs, index, counts, ws, ws_bytes, s);  // warm-up
  if (rc != WAH_OK) return rc;
  cudaError_t e = cudaEventRecord(a, s);
  for (int r = 0; r < reps && rc == WAH_OK && e == cudaSuccess; ++r)
    rc = wah_build(v, n, bound, keys, offs, index, counts, ws, ws_bytes, s);
  if (rc != WAH_OK) return rc;
  if (e == cudaSuccess) e = cudaEventRecord(b, s);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, a, b);
  *ms /= reps;
  return cuda_status(e);
}

}  // namespace
}  // namespace wah

using namespace wah;

extern "C" {

int wah_autotune(uint64_t n, uint32_t bound, const char* cache_path, int* chosen,
                 int* from_cache) {
  if (n == 0 || n >= WAH_MAX_ROWS) return WAH_ERANGE;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_status(e);
  const std::string key = cache_key(device, n, bound);
  int tuning = 0;
  if (cache_lookup(cache_path, key, &tuning) && wah_set_tuning(tuning) == WAH_OK) {
    if (chosen) *chosen = tuning;
    if (from_cache) *from_cache = 1;
    return WAH_OK;
  }
  const int before = wah_get_tuning();
  uint64_t keys_cap = 0, index_cap = 0;
  wah_output_caps(n, bound, &keys_cap, &index_cap);
  const size_t ws_bytes = wah_workspace_bytes(n, bound);
  uint32_t *v = nullptr, *keys = nullptr, *offs = nullptr, *index = nullptr;
  wah_counts* counts = nullptr;
  void* ws = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  e = cudaMalloc(&v, n * 4);
  if (e == cudaSuccess) e = cudaMalloc(&keys, keys_cap * 4);
  if (e == cudaSuccess) e = cudaMalloc(&offs, keys_cap * 4);
  if (e == cudaSuccess) e = cudaMalloc(&index, index_cap * 4);
  if (e == cudaSuccess) e = cudaMalloc(&counts, sizeof(wah_counts));
  if (e == cudaSuccess) e = cudaMalloc(&ws, ws_bytes);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  int rc = cuda_status(e);
  if (rc == WAH_OK) {
    k_tune_column<<<sm_count_current() * 4, 256, 0, s>>>(v, n, bound);
    rc = cuda_status(cudaGetLastError());
  }
  // each candidate timed over enough builds for ~20 ms, at least 2
  const int reps = n >= (1ull << 26) ? 2 : n >= (1ull << 22) ? 8 : 32;
  // First every shape for all passes, then, with the best of those for digit
  // pass 0, every other shape for the later passes.
  float best_ms = 0;
  int best = before;
  auto consider = [&](int t) {
    if (rc != WAH_OK || wah_set_tuning(t) != WAH_OK) return;
    float ms = 0;
    rc = timed_build(v, n, bound, keys, offs, index, counts, ws, ws_bytes, s, a, b, reps, &ms);
    if (rc == WAH_OK && (best_ms == 0 || ms < best_ms)) {
      best_ms = ms;
      best = t;
    }
  };
  for (int t : kCandidates) consider(t);
  const int first = best & 0xffff;
  if (passes_for_bound(bound) > 1)
    for (int t : kCandidates)
      if (t != first) consider(first | WAH_TUNE_LATER(t));
  if (rc == WAH_OK) {
    wah_counts c{};
    e = cudaMemcpy(&c, counts, sizeof c, cudaMemcpyDeviceToHost);
    rc = e == cudaSuccess ? (int)c.status : cuda_status(e);
  }
  if (s) cudaStreamSynchronize(s);
  cudaFree(v);
  cudaFree(keys);
  cudaFree(offs);
  cudaFree(index);
  cudaFree(counts);
  cudaFree(ws);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (s) cudaStreamDestroy(s);
  if (rc != WAH_OK) {
    wah_set_tuning(before);
    return rc;
  }
  wah_set_tuning(best);
  if (cache_path) {
    if (FILE* f = std::fopen(cache_path, "a")) {
      std::fprintf(f, "%s %d %.4f\n", key.c_str(), best, best_ms);
      std::fclose(f);
    }
  }
  if (chosen) *chosen = best;
  if (from_cache) *from_cache = 0;
  return WAH_OK;
}

}  // extern "C"
