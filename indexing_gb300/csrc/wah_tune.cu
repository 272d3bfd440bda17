// wah_tune.cu -- autotuner of the radix tile shapes, with a cache file.
//
// The reference hard-codes its radix parameters (src/phases.cpp:445-453:
// 4-bit digits, 8 blocks of 1024 threads); its stale `radix` test program
// exposes them as flags (src/radix.cpp:161-184).  Here every compiled tile
// shape of the digit passes -- rows per thread 8, 12 or 16, peer masks from
// ballots, match.any or 3/8 match.any -- is timed on synthetic data of the
// workload the caller names (one uniform column, one skewed column, or a
// batch of many columns of uneven size), then, for one-column workloads,
// every other shape for the passes after the first and the packed exchange
// between the two digit passes on and off.  Builds are timed with the
// candidate word passed per call (wah_build_tuned, wah_batch_create_tuned):
// nothing process-wide changes while timing, so other callers' builds keep
// their own shapes.  The choice is remembered per (device, workload, size
// bucket, digit passes) in a text cache file, so later processes take it
// without timing.  wah_autotune is the uniform workload, applied as the
// process default.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "wah_common.cuh"

namespace wah {
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Row i of a synthetic column: a hash of (seed, i) folded below bound + 1;
// skewed: a power law, value = (bound + 1)^u - 1 with u uniform in [0, 1)
// (the small values hold most rows).
__global__ void k_tune_column(uint32_t* v, uint64_t n, uint32_t bound, uint64_t seed,
                              int skewed) {
  const uint64_t range = (uint64_t)bound + 1;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t z = mix64(i + seed * 0x9E3779B97F4A7C15ull + 0x9E3779B97F4A7C15ull);
    uint32_t x;
    if (bound == 0) {
      x = (uint32_t)z;
    } else if (skewed) {
      const double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
      const double e = exp(u * log((double)range)) - 1.0;
      x = e < 0 ? 0u : (uint32_t)fmin(e, (double)bound);
    } else {
      x = (uint32_t)((z >> 32) * range >> 32);
    }
    v[i] = x;
  }
}

// Every tile shape wah_set_tuning accepts.
const int kCandidates[] = {16, 12, 8, 16 | WAH_TUNE_MATCH, 12 | WAH_TUNE_MATCH,
                           8 | WAH_TUNE_MATCH, 16 | WAH_TUNE_HYBRID, 12 | WAH_TUNE_HYBRID,
                           8 | WAH_TUNE_HYBRID};

std::mutex g_tune_mu;

std::string cache_key(int device, int workload, uint32_t ncols, uint64_t n, uint32_t bound) {
  cudaDeviceProp p;
  std::string name = cudaGetDeviceProperties(&p, device) == cudaSuccess ? p.name : "unknown";
  for (char& c : name)
    if (c == ' ' || c == '\t') c = '_';
  int bucket = 0;
  while (bucket < 63 && (2ull << bucket) <= n) ++bucket;  // floor(log2 n)
  std::string w = workload == WAH_WORKLOAD_SKEWED  ? "skewed"
                  : workload == WAH_WORKLOAD_BATCH ? "batch" + std::to_string(ncols)
                                                    : "uniform";
  // "t3": entries of the per-workload tuner (later-pass shape and packing)
  return name + " " + w + " " + std::to_string(bucket) + " " +
         std::to_string(passes_for_bound(bound)) + " t3";
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
    if (std::sscanf(line + key.size() + 1, "%d", &t) == 1 && valid_tuning(t)) {
      *tuning = t;  // the last entry of a key wins
      found = true;
    }
  }
  std::fclose(f);
  return found;
}

// Device memory of one tuning run, freed by the destructor.
struct TuneMem {
  std::vector<void*> blocks;
  cudaStream_t s = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t alloc(void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 16));
    if (e == cudaSuccess) blocks.push_back(*p);
    return e;
  }
  ~TuneMem() {
    if (s) cudaStreamSynchronize(s);
    for (void* p : blocks) cudaFree(p);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (s) cudaStreamDestroy(s);
  }
};

// Mean ms of `reps` calls of fn() on stream s after one warm-up call.
template <class F>
int time_calls(F fn, cudaStream_t s, cudaEvent_t a, cudaEvent_t b, int reps, float* ms) {
  int rc = fn();
  if (rc != WAH_OK) return rc;
  cudaError_t e = cudaEventRecord(a, s);
  for (int r = 0; r < reps && rc == WAH_OK && e == cudaSuccess; ++r) rc = fn();
  if (rc != WAH_OK) return rc;
  if (e == cudaSuccess) e = cudaEventRecord(b, s);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, a, b);
  *ms /= reps;
  return cuda_status(e);
}

// The candidate list is timed with `timed(word, &ms)`; returns the fastest.
template <class T>
int search(T timed, bool one_column, bool two_passes, int* best, float* best_ms) {
  int rc = WAH_OK;
  *best = 0;
  *best_ms = 0;
  // margin: a candidate must be this much faster to replace the best
  auto consider = [&](int t, float margin) {
    if (rc != WAH_OK) return;
    float ms = 0;
    rc = timed(t, &ms);
    if (rc == WAH_OK && (*best_ms == 0 || ms < *best_ms * margin)) {
      *best_ms = ms;
      *best = t;
    }
  };
  for (int t : kCandidates) consider(t, 1.0f);
  if (one_column && two_passes) {
    // with the best of those for digit pass 0: every other shape for the
    // later passes, then the packed exchange forced on (kept only when it
    // gains 2%: where the size alone already selects it, forcing it changes
    // nothing, and the flag would then force it on other sizes that share
    // the word)
    const int first = *best & 0xffff;
    for (int t : kCandidates)
      if (t != first) consider(first | WAH_TUNE_LATER(t), 1.0f);
    consider(*best | WAH_TUNE_PACK, 0.98f);
  }
  return rc;
}

int tune_one_column(int workload, uint64_t n, uint32_t bound, int* best, float* best_ms) {
  uint64_t keys_cap = 0, index_cap = 0;
  wah_output_caps(n, bound, &keys_cap, &index_cap);
  const size_t ws_bytes = wah_workspace_bytes(n, bound);
  TuneMem m;
  uint32_t *v = nullptr, *keys = nullptr, *offs = nullptr, *index = nullptr;
  wah_counts* counts = nullptr;
  void* ws = nullptr;
  cudaError_t e = m.alloc((void**)&v, n * 4);
  if (e == cudaSuccess) e = m.alloc((void**)&keys, keys_cap * 4);
  if (e == cudaSuccess) e = m.alloc((void**)&offs, keys_cap * 4);
  if (e == cudaSuccess) e = m.alloc((void**)&index, index_cap * 4);
  if (e == cudaSuccess) e = m.alloc((void**)&counts, sizeof(wah_counts));
  if (e == cudaSuccess) e = m.alloc(&ws, ws_bytes);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m.s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&m.a);
  if (e == cudaSuccess) e = cudaEventCreate(&m.b);
  if (e != cudaSuccess) return cuda_status(e);
  k_tune_column<<<sm_count_current() * 4, 256, 0, m.s>>>(v, n, bound, 1,
                                                         workload == WAH_WORKLOAD_SKEWED);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e);
  // each candidate timed over enough builds for ~20 ms, at least 2
  const int reps = n >= (1ull << 26) ? 2 : n >= (1ull << 22) ? 8 : 32;
  auto timed = [&](int t, float* ms) {
    return time_calls(
        [&] {
          return wah_build_tuned(v, n, bound, keys, offs, index, counts, ws, ws_bytes, t, m.s);
        },
        m.s, m.a, m.b, reps, ms);
  };
  int rc = search(timed, true, passes_for_bound(bound) > 1, best, best_ms);
  if (rc == WAH_OK) {
    wah_counts c{};
    e = cudaMemcpy(&c, counts, sizeof c, cudaMemcpyDeviceToHost);
    rc = e == cudaSuccess ? (int)c.status : cuda_status(e);
  }
  return rc;
}

int tune_batch(uint64_t n, uint32_t bound, uint32_t ncols, int* best, float* best_ms) {
  // Column sizes log-uniform in [1,024, 4,194,304] scaled to n rows in all,
  // cardinalities log-uniform in [2, min(bound + 1, 65,536)] (a fixed LCG).
  std::vector<uint64_t> ns(ncols);
  std::vector<uint32_t> bounds(ncols);
  const double cmax = bound == 0 ? 65536.0 : std::min<double>((double)bound + 1, 65536.0);
  uint64_t st = 0x853c49e6748fea9bull;
  auto uni = [&] {
    st = st * 6364136223846793005ull + 1442695040888963407ull;
    return (double)(st >> 11) * (1.0 / 9007199254740992.0);
  };
  double sum = 0;
  std::vector<double> raw(ncols);
  for (uint32_t c = 0; c < ncols; ++c) {
    raw[c] = std::exp(std::log(1024.0) + uni() * (std::log(4194304.0) - std::log(1024.0)));
    sum += raw[c];
    const double card = std::exp(std::log(2.0) + uni() * (std::log(cmax) - std::log(2.0)));
    bounds[c] = (uint32_t)std::max(1.0, std::floor(card) - 1);
  }
  uint64_t total = 0;
  for (uint32_t c = 0; c < ncols; ++c) {
    ns[c] = std::max<uint64_t>(1, (uint64_t)(raw[c] * (double)n / sum));
    total += ns[c];
  }
  if (total >= (1ull << 32)) return WAH_ERANGE;
  TuneMem m;
  cudaError_t e = cudaStreamCreateWithFlags(&m.s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&m.a);
  if (e == cudaSuccess) e = cudaEventCreate(&m.b);
  std::vector<wah_column> cols(ncols);
  for (uint32_t c = 0; c < ncols && e == cudaSuccess; ++c) {
    uint64_t kc = 0, ic = 0;
    wah_output_caps(ns[c], bounds[c], &kc, &ic);
    wah_column& x = cols[c];
    std::memset(&x, 0, sizeof x);
    x.n = ns[c];
    x.bound = bounds[c];
    void *v = nullptr, *k = nullptr, *o = nullptr, *i = nullptr, *cnt = nullptr;
    e = m.alloc(&v, ns[c] * 4);
    if (e == cudaSuccess) e = m.alloc(&k, kc * 4);
    if (e == cudaSuccess) e = m.alloc(&o, kc * 4);
    if (e == cudaSuccess) e = m.alloc(&i, ic * 4);
    if (e == cudaSuccess) e = m.alloc(&cnt, sizeof(wah_counts));
    if (e == cudaSuccess) {
      k_tune_column<<<64, 256, 0, m.s>>>(static_cast<uint32_t*>(v), ns[c], bounds[c], c + 2, 0);
      e = cudaGetLastError();
    }
    x.values = static_cast<const uint32_t*>(v);
    x.keys = static_cast<uint32_t*>(k);
    x.offsets = static_cast<uint32_t*>(o);
    x.index = static_cast<uint32_t*>(i);
    x.counts = static_cast<wah_counts*>(cnt);
  }
  if (e != cudaSuccess) return cuda_status(e);
  const int reps = total >= (1ull << 28) ? 2 : 4;
  auto timed = [&](int t, float* ms) {
    wah_batch* b = nullptr;
    int rc = wah_batch_create_tuned(ns.data(), bounds.data(), ncols, t, &b);
    if (rc == WAH_OK) rc = wah_batch_set_columns(b, cols.data(), m.s);
    if (rc == WAH_OK) rc = time_calls([&] { return wah_batch_build(b, m.s); }, m.s, m.a, m.b,
                                      reps, ms);
    if (b) {
      cudaStreamSynchronize(m.s);
      wah_batch_destroy(b);
    }
    return rc;
  };
  return search(timed, false, false, best, best_ms);
}

}  // namespace
}  // namespace wah

using namespace wah;

extern "C" {

int wah_autotune_workload(int workload, uint64_t n, uint32_t bound, uint32_t ncols,
                          const char* cache_path, int* chosen, int* from_cache) {
  if (workload != WAH_WORKLOAD_UNIFORM && workload != WAH_WORKLOAD_SKEWED &&
      workload != WAH_WORKLOAD_BATCH)
    return WAH_EINVAL;
  if (workload == WAH_WORKLOAD_BATCH ? (ncols == 0 || n < ncols) : (n == 0 || n >= WAH_MAX_ROWS))
    return WAH_ERANGE;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_status(e);
  const std::string key = cache_key(device, workload, ncols, n, bound);
  int tuning = 0;
  if (cache_lookup(cache_path, key, &tuning)) {
    if (chosen) *chosen = tuning;
    if (from_cache) *from_cache = 1;
    return WAH_OK;
  }
  int best = 0;
  float best_ms = 0;
  const int rc = workload == WAH_WORKLOAD_BATCH ? tune_batch(n, bound, ncols, &best, &best_ms)
                                                : tune_one_column(workload, n, bound, &best,
                                                                  &best_ms);
  if (rc != WAH_OK) return rc;
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

int wah_autotune(uint64_t n, uint32_t bound, const char* cache_path, int* chosen,
                 int* from_cache) {
  int t = 0, cached = 0;
  const int rc = wah_autotune_workload(WAH_WORKLOAD_UNIFORM, n, bound, 0, cache_path, &t,
                                       &cached);
  if (rc != WAH_OK) return rc;
  const int set = wah_set_tuning(t);
  if (set != WAH_OK) return set;
  if (chosen) *chosen = t;
  if (from_cache) *from_cache = cached;
  return WAH_OK;
}

}  // extern "C"
