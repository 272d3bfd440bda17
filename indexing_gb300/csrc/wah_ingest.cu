// wah_ingest.cu -- parsing the reference's text data files on the GPU.
//
// The reference reads its columns from text files with one value per line
// (`generate` writes them, src/generate_test_data.cpp:45-53) through
// `while (source >> next) values.push_back(next)` (src/cpu.cpp:297-302,
// src/phases.cpp:363-366, src/gpu.cpp:298-303), one character at a time on
// one host thread.  Here the raw bytes go to the device and are parsed there:
//
//   token    a maximal run of non-whitespace bytes (whitespace: space and
//            \t \n \v \f \r, the stream's separators)
//   value    a token of decimal digits only whose value fits in 32 bits
//            (leading zeros allowed)
//   stop     parsing ends at the first token that is not a value, as the
//            stream's extraction fails there; the values before it are the
//            column
//
// The bytes are cut into equal ranges, one persistent CTA per range (the
// builds' look-back-free layout): k_parse_count counts token starts per
// range (16 bytes per thread per step, whitespace found with SIMD byte
// compares), k_parse_scan turns the counts into each range's first token
// number, and k_parse_emit re-reads the range step by step through shared
// memory (32 bytes per thread per step: half the per-step scan and barrier
// work per token of 16), parses every token that starts in it and writes
// value i to values[i].  A token of up to 16 characters is converted eight digits at a
// time in 64-bit registers (SWAR); longer ones (leading zeros) character by
// character.  Invalid tokens lower a device-wide "first invalid token" with
// atomicMin.  The largest value is reduced while parsing; only when an
// invalid token cuts the column is it recomputed over the values before it.
#include "wah_common.cuh"

namespace wah {
namespace {

constexpr int kPThreads = 256;
constexpr uint32_t kPStep = kPThreads * 16;   // bytes per CTA step of the count
constexpr uint32_t kPEStep = kPThreads * 32;  // bytes per CTA step of the emit
constexpr uint32_t kMaxParseRanges = 4096;
constexpr uint64_t kNoInvalid = ~0ull;

struct ParseCtrl {
  unsigned long long first_invalid;  // token number, kNoInvalid if none
  unsigned long long tokens;         // all tokens
  uint32_t max_value;       // over every valid token (k_parse_emit)
  uint32_t done_blocks;     // k_parse_finish blocks that have finished
  uint32_t recomputed_max;  // over the tokens before the first invalid one
  uint32_t pad;
};

struct ParseRange {
  unsigned long long starts;  // tokens starting in the range
  unsigned long long base;    // tokens before the range (scan)
};

// Bit 7 of each byte of x set where the byte is whitespace (space, \t..\r),
// exactly, with carry-free byte arithmetic (SWAR): bytes in [9, 13] are
// those >= 9 and not >= 14 among bytes below 0x80; spaces are the zero bytes
// of x ^ 0x20202020.
__device__ __forceinline__ uint32_t ws_flags4(uint32_t x) {
  const uint32_t lo = x & 0x7F7F7F7Fu;
  const uint32_t ge9 = (lo + 0x77777777u) & 0x80808080u;
  const uint32_t ge14 = (lo + 0x72727272u) & 0x80808080u;
  const uint32_t ctl = ge9 & ~ge14 & ~x & 0x80808080u;
  const uint32_t y = x ^ 0x20202020u;
  const uint32_t sp = ~(((y & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | y) & 0x80808080u;
  return ctl | sp;
}

// One bit per byte (bit i = byte i) of the 16 bytes in q that are not
// whitespace: each word's four byte flags are gathered into four bits by
// one multiply (the partial products land on distinct bits).
__device__ __forceinline__ uint32_t nonws_mask16(uint4 q) {
  const uint32_t w[4] = {q.x, q.y, q.z, q.w};
  uint32_t m = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const uint32_t f = (ws_flags4(w[k]) >> 7) & 0x01010101u;
    m |= ((f * 0x10204080u) >> 28) << (4 * k);
  }
  return ~m & 0xFFFFu;
}

__device__ __forceinline__ bool is_ws(uint32_t c) { return c == 0x20u || (c >= 9u && c <= 13u); }

struct ParseIn {
  const unsigned char* text;
  uint64_t bytes;
  uint64_t range_bytes;  // multiple of kPEStep (and so of kPStep)
  uint32_t ranges;
};

// Loads the 16 bytes at p (p a multiple of 16); bytes past the end of the
// text read as spaces.
__device__ __forceinline__ uint4 load16(const ParseIn& in, uint64_t p) {
  if (p + 16 <= in.bytes) return *reinterpret_cast<const uint4*>(in.text + p);
  unsigned char b[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) b[i] = p + i < in.bytes ? in.text[p + i] : 0x20;
  uint4 q;
  q.x = b[0] | b[1] << 8 | b[2] << 16 | (uint32_t)b[3] << 24;
  q.y = b[4] | b[5] << 8 | b[6] << 16 | (uint32_t)b[7] << 24;
  q.z = b[8] | b[9] << 8 | b[10] << 16 | (uint32_t)b[11] << 24;
  q.w = b[12] | b[13] << 8 | b[14] << 16 | (uint32_t)b[15] << 24;
  return q;
}

// Token starts among the 16 bytes at p: non-whitespace bytes whose
// predecessor is whitespace (or the start of the text).
__device__ __forceinline__ uint32_t starts16(const ParseIn& in, uint64_t p, uint4 q) {
  const uint32_t nw = nonws_mask16(q);
  const uint32_t prev_nonws = (p > 0 && !is_ws(in.text[p - 1])) ? 1u : 0u;
  return nw & ~((nw << 1) | prev_nonws) & 0xFFFFu;
}

__global__ void __launch_bounds__(kPThreads) k_parse_count(ParseIn in, ParseRange* rng) {
  __shared__ unsigned long long s_red[kPThreads / 32];
  const uint64_t lo = (uint64_t)blockIdx.x * in.range_bytes;
  const uint64_t hi = lo + in.range_bytes < in.bytes ? lo + in.range_bytes : in.bytes;
  unsigned long long cnt = 0;
  for (uint64_t p = lo + threadIdx.x * 16ull; p < hi; p += kPStep)
    cnt += __popc(starts16(in, p, load16(in, p)));
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, d);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < kPThreads / 32; ++w) t += s_red[w];
    rng[blockIdx.x].starts = t;
  }
}

constexpr int kPScanThreads = 1024;
__global__ void __launch_bounds__(kPScanThreads) k_parse_scan(ParseRange* rng, uint32_t ranges,
                                                              ParseCtrl* ctrl) {
  __shared__ uint64_t s_w[kPScanThreads / 32 + 1];
  constexpr uint32_t PER = kMaxParseRanges / kPScanThreads;
  const uint32_t base = threadIdx.x * PER;
  uint64_t sum = 0;
  for (uint32_t i = 0; i < PER; ++i)
    if (base + i < ranges) sum += rng[base + i].starts;
  uint64_t total;
  uint64_t ex = block_exclusive_scan64<kPScanThreads>(sum, &total, s_w);
  for (uint32_t i = 0; i < PER; ++i)
    if (base + i < ranges) {
      rng[base + i].base = ex;
      ex += rng[base + i].starts;
    }
  if (threadIdx.x == 0) {
    ctrl->tokens = total;
    ctrl->first_invalid = kNoInvalid;
    ctrl->max_value = 0;
    ctrl->done_blocks = 0;
    ctrl->recomputed_max = 0;
  }
}

// Bytes an emit step keeps in shared memory: its own 8192 (32 per thread)
// and the 64 after them, so tokens that start in the step and end shortly
// after it are read from shared memory too; longer ones continue from
// global memory.
constexpr uint32_t kPWindow = kPEStep + 64;

// Parses the token starting at byte p (a token start) of the step at s,
// character by character.  Returns false if the token is not a 32-bit
// decimal value.
__device__ __forceinline__ bool parse_token(const ParseIn& in, const unsigned char* s_text,
                                            uint64_t s, uint64_t p, uint32_t* out) {
  uint64_t v = 0;
  bool ok = true;
  for (uint64_t i = p; i < in.bytes; ++i) {
    const uint64_t o = i - s;
    const uint32_t c = o < kPWindow ? (uint32_t)s_text[o] : (uint32_t)in.text[i];
    if (is_ws(c)) break;
    const uint32_t d = c - '0';
    if (d > 9) {
      ok = false;
      break;
    }
    v = v * 10 + d;
    if (v > 0xFFFFFFFFull) {
      ok = false;
      break;
    }
  }
  *out = (uint32_t)v;
  return ok;
}

// The 8 bytes of s_text at byte offset o (any alignment), little endian.
__device__ __forceinline__ uint64_t load8(const unsigned char* s_text, uint32_t o) {
  const uint64_t* w = reinterpret_cast<const uint64_t*>(s_text + (o & ~7u));
  const uint32_t sh = (o & 7u) * 8u;
  return sh ? (w[0] >> sh) | (w[1] << (64u - sh)) : w[0];
}

// Up to 8 characters as a number: x holds them in its low `len` bytes
// (first character lowest).  They are right-aligned behind '0's, checked to
// be digits, and combined pairwise (SWAR: 2, 4, then 8 digits per lane).
__device__ __forceinline__ bool swar_digits(uint64_t x, uint32_t len, uint64_t* out) {
  const uint32_t pad = 8u - len;
  x = (x << (8u * pad)) | (pad ? 0x3030303030303030ull >> (8u * len) : 0ull);
  const uint64_t t = x ^ 0x3030303030303030ull;  // digits become 0..9
  if (((t + 0x7676767676767676ull) | t) & 0x8080808080808080ull) return false;
  uint64_t y = ((t * 10u) + (t >> 8)) & 0x00FF00FF00FF00FFull;
  y = ((y * 100u) + (y >> 16)) & 0x0000FFFF0000FFFFull;
  y = ((y * 10000u) + (y >> 32)) & 0xFFFFFFFFull;
  *out = y;
  return true;
}

__global__ void __launch_bounds__(kPThreads) k_parse_emit(ParseIn in, const ParseRange* rng,
                                                          uint32_t* values, uint64_t cap,
                                                          ParseCtrl* ctrl) {
  __shared__ uint32_t s_w[kPThreads / 32 + 1];
  __shared__ uint32_t s_max[kPThreads / 32];
  __shared__ __align__(16) unsigned char s_text[kPWindow];
  const uint64_t lo = (uint64_t)blockIdx.x * in.range_bytes;
  const uint64_t hi = lo + in.range_bytes < in.bytes ? lo + in.range_bytes : in.bytes;
  if (lo >= hi) return;
  const uint32_t lane = threadIdx.x & 31;
  uint64_t carry = rng[blockIdx.x].base;
  uint32_t vmax = 0;
  for (uint64_t s = lo; s < hi; s += kPEStep) {
    // this thread's 32 bytes (two 16-byte loads); bytes past the range are
    // loaded too (whitespace past the text's end)
    const uint64_t p = s + threadIdx.x * 32ull;
    const uint4 q0 = load16(in, p), q1 = load16(in, p + 16);
    reinterpret_cast<uint4*>(s_text)[2 * threadIdx.x] = q0;
    reinterpret_cast<uint4*>(s_text)[2 * threadIdx.x + 1] = q1;
    if (threadIdx.x < 4)
      reinterpret_cast<uint4*>(s_text + kPEStep)[threadIdx.x] =
          load16(in, s + kPEStep + 16ull * threadIdx.x);
    const uint32_t nw = nonws_mask16(q0) | (nonws_mask16(q1) << 16);
    // the next 32 bytes' mask: the next lane's, or (last lane) computed here
    uint32_t nw_next = __shfl_down_sync(0xffffffffu, nw, 1);
    const uint32_t prev_last = __shfl_up_sync(0xffffffffu, nw >> 31, 1);
    __syncthreads();
    if (lane == 31) {
      const uint4* nx = reinterpret_cast<const uint4*>(s_text) + 2 * (threadIdx.x + 1);
      nw_next = nonws_mask16(nx[0]) | (nonws_mask16(nx[1]) << 16);
    }
    uint32_t st = 0;
    if (p < hi) {
      uint32_t prev_nonws;
      if (lane > 0)
        prev_nonws = prev_last & 1u;
      else if (threadIdx.x > 0)
        prev_nonws = !is_ws(s_text[threadIdx.x * 32 - 1]);
      else
        prev_nonws = p > 0 && !is_ws(in.text[p - 1]);
      st = nw & ~((nw << 1) | prev_nonws);
    }
    uint32_t tot;
    const uint32_t ex = block_exclusive_scan<kPThreads>(__popc(st), &tot, s_w);
    uint64_t idx = carry + ex;
    const uint64_t nw64 = (uint64_t)nw | ((uint64_t)nw_next << 32);
    uint32_t m = st;
    while (m) {
      const uint32_t b = __ffs(m) - 1;
      m &= m - 1;
      // token length from the 64-byte non-whitespace mask, if it ends there
      const uint64_t after = ~nw64 >> b;
      const uint32_t len = after ? (uint32_t)__ffsll((long long)after) - 1 : 64u;
      const uint32_t o = threadIdx.x * 32u + b;
      uint64_t v = 0;
      bool ok;
      if (len <= 8) {
        ok = swar_digits(load8(s_text, o), len, &v);
      } else if (len <= 16) {
        uint64_t h = 0, l = 0;
        ok = swar_digits(load8(s_text, o), len - 8, &h) &&
             swar_digits(load8(s_text, o + len - 8), 8, &l);
        v = h * 100000000ull + l;
        ok = ok && v <= 0xFFFFFFFFull;
      } else {
        uint32_t w;
        ok = parse_token(in, s_text, s, p + b, &w);  // long token (leading zeros)
        v = w;
      }
      if (ok) {
        if (idx < cap) values[idx] = (uint32_t)v;
        vmax = (uint32_t)v > vmax ? (uint32_t)v : vmax;
      } else {
        atomicMin(&ctrl->first_invalid, (unsigned long long)idx);
      }
      ++idx;
    }
    carry += tot;
    __syncthreads();  // s_text is rewritten by the next step
  }
  // largest value of every valid token (k_parse_finish redoes it over the
  // tokens before the first invalid one when there is one)
  vmax = __reduce_max_sync(0xffffffffu, vmax);
  if (lane == 0) s_max[threadIdx.x >> 5] = vmax;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t b = 0;
    for (int w = 0; w < kPThreads / 32; ++w) b = s_max[w] > b ? s_max[w] : b;
    atomicMax(&ctrl->max_value, b);
  }
}

// The result record.  Without an invalid token the largest value is the one
// k_parse_emit reduced; otherwise it is recomputed over the values before the
// first invalid token (four 16-byte loads in flight per thread).
__global__ void __launch_bounds__(kPThreads) k_parse_finish(const uint32_t* values, uint64_t cap,
                                                            ParseCtrl* ctrl,
                                                            wah_parse_result* res) {
  __shared__ uint32_t s_max[kPThreads / 32];
  const uint64_t fi = ctrl->first_invalid;
  const uint64_t count = ctrl->tokens < fi ? ctrl->tokens : fi;
  const bool recompute = fi != kNoInvalid;
  uint32_t m = 0;
  if (recompute) {
    const uint64_t stored = count < cap ? count : cap;
    const uint64_t n4 = stored / 4;
    const uint4* v4 = reinterpret_cast<const uint4*>(values);
    const uint64_t stride = (uint64_t)gridDim.x * kPThreads;
    uint64_t i = (uint64_t)blockIdx.x * kPThreads + threadIdx.x;
    for (; i + 3 * stride < n4; i += 4 * stride) {
      uint4 a[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = v4[i + u * stride];
#pragma unroll
      for (int u = 0; u < 4; ++u)
        m = max(m, max(max(a[u].x, a[u].y), max(a[u].z, a[u].w)));
    }
    for (; i < n4; i += stride) {
      const uint4 a = v4[i];
      m = max(m, max(max(a.x, a.y), max(a.z, a.w)));
    }
    if (blockIdx.x == 0 && threadIdx.x < (stored & 3)) m = max(m, values[n4 * 4 + threadIdx.x]);
  }
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t b = 0;
    for (int w = 0; w < kPThreads / 32; ++w) b = s_max[w] > b ? s_max[w] : b;
    if (recompute) atomicMax(&ctrl->recomputed_max, b);
    __threadfence();
    const uint32_t done = atomicAdd(&ctrl->done_blocks, 1u);
    if (done == gridDim.x - 1) {
      __threadfence();
      res->values = count;
      res->tokens = ctrl->tokens;
      res->max_value = recompute ? atomicAdd(&ctrl->recomputed_max, 0u) : ctrl->max_value;
      res->status = count > cap ? WAH_EOVERFLOW : WAH_OK;
      res->reserved = 0;
    }
  }
}

constexpr size_t kAlign = 256;
size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

}  // namespace
}  // namespace wah

using namespace wah;

extern "C" {

size_t wah_parse_workspace_bytes(void) {
  return align_up(sizeof(ParseCtrl)) + align_up(sizeof(ParseRange) * kMaxParseRanges);
}

int wah_parse_text(const void* d_text, uint64_t bytes, uint32_t* d_values, uint64_t capacity,
                   wah_parse_result* d_result, void* d_workspace, size_t workspace_bytes,
                   void* stream) {
  if (!d_result || (reinterpret_cast<uintptr_t>(d_result) & 15)) return WAH_EINVAL;
  if (bytes > 0 && (!d_text || (reinterpret_cast<uintptr_t>(d_text) & 15))) return WAH_EINVAL;
  if (capacity > 0 && (!d_values || (reinterpret_cast<uintptr_t>(d_values) & 15)))
    return WAH_EINVAL;
  if (!d_workspace || workspace_bytes < wah_parse_workspace_bytes() ||
      (reinterpret_cast<uintptr_t>(d_workspace) & 15))
    return WAH_ENOMEM;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char* ws = static_cast<unsigned char*>(d_workspace);
  ParseCtrl* ctrl = reinterpret_cast<ParseCtrl*>(ws);
  ParseRange* rng = reinterpret_cast<ParseRange*>(ws + align_up(sizeof(ParseCtrl)));
  const int sms = sm_count_current();
  uint32_t ranges = (uint32_t)(sms * 4);
  if (ranges > kMaxParseRanges) ranges = kMaxParseRanges;
  ParseIn in;
  in.text = static_cast<const unsigned char*>(d_text);
  in.bytes = bytes;
  const uint64_t rb = ceil_div(bytes ? bytes : 1, ranges);
  in.range_bytes = ceil_div(rb, kPEStep) * kPEStep;
  in.ranges = ranges;
  k_parse_count<<<ranges, kPThreads, 0, s>>>(in, rng);
  k_parse_scan<<<1, kPScanThreads, 0, s>>>(rng, ranges, ctrl);
  k_parse_emit<<<ranges, kPThreads, 0, s>>>(in, rng, d_values, capacity, ctrl);
  k_parse_finish<<<(unsigned)(sms * 2), kPThreads, 0, s>>>(d_values, capacity, ctrl, d_result);
  *last_launches_slot() = 4;
  return cuda_status(cudaGetLastError());
}

}  // extern "C"
