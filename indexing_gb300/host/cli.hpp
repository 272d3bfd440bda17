// cli.hpp -- what the host programs share: flag parsing, reading the
// one-value-per-line data files, the WAH decoder used for printing, and the
// binary result file the tests read.
//
// Flags follow the reference programs' CAF option groups: long form
// `--name=value` or `--name value`, short form `-x value`, booleans without a
// value (src/cpu.cpp:274-285, src/phases.cpp:332-348, src/gpu.cpp:264-285,
// src/generate_test_data.cpp:18-31).
#pragma once

#include <cerrno>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "wah/wah.h"

namespace wahcli {

struct flag {
  const char* long_name;
  char short_name;  // 0 = none
  const char* help;
  enum kind_t { STRING, U32, U64, BOOL } kind;
  void* target;
};

inline void print_help(const char* prog, const std::vector<flag>& flags) {
  std::printf("%s options:\n", prog);
  for (const auto& f : flags) {
    if (f.short_name)
      std::printf("  -%c, --%-16s %s\n", f.short_name, f.long_name, f.help);
    else
      std::printf("      --%-16s %s\n", f.long_name, f.help);
  }
}

inline bool parse_number(const char* s, uint64_t max, uint64_t* out) {
  if (!s || !*s) return false;
  errno = 0;
  char* end = nullptr;
  unsigned long long v = std::strtoull(s, &end, 10);
  if (errno || *end || v > max || s[0] == '-') return false;
  *out = v;
  return true;
}

// Returns 0 on success, 1 when help was printed, -1 on a bad command line.
inline int parse_flags(int argc, char** argv, const std::vector<flag>& flags) {
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    if (a == "-h" || a == "--help" || a == "-?") {
      print_help(argv[0], flags);
      return 1;
    }
    const flag* f = nullptr;
    std::string value;
    bool has_value = false;
    if (a.rfind("--", 0) == 0) {
      std::string name = a.substr(2);
      const auto eq = name.find('=');
      if (eq != std::string::npos) {
        value = name.substr(eq + 1);
        name = name.substr(0, eq);
        has_value = true;
      }
      for (const auto& c : flags)
        if (name == c.long_name) f = &c;
    } else if (a.size() == 2 && a[0] == '-') {
      for (const auto& c : flags)
        if (c.short_name == a[1]) f = &c;
    }
    if (!f) {
      std::fprintf(stderr, "unknown option '%s' (see --help)\n", a.c_str());
      return -1;
    }
    if (f->kind == flag::BOOL) {
      bool v = true;
      if (has_value) v = !(value == "false" || value == "0");
      *static_cast<bool*>(f->target) = v;
      continue;
    }
    if (!has_value) {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "option '%s' needs a value\n", a.c_str());
        return -1;
      }
      value = argv[++i];
    }
    if (f->kind == flag::STRING) {
      *static_cast<std::string*>(f->target) = value;
      continue;
    }
    uint64_t v = 0;
    const uint64_t max = f->kind == flag::U32 ? 0xFFFFFFFFull : ~0ull;
    if (!parse_number(value.c_str(), max, &v)) {
      std::fprintf(stderr, "option '%s': '%s' is not a valid number\n", a.c_str(), value.c_str());
      return -1;
    }
    if (f->kind == flag::U32)
      *static_cast<uint32_t*>(f->target) = static_cast<uint32_t>(v);
    else
      *static_cast<uint64_t*>(f->target) = v;
  }
  return 0;
}

// Reads whitespace-separated decimal values, like `while (source >> next)`
// (src/cpu.cpp:297-302): reading stops at the first token that is not an
// unsigned 32-bit number.  Returns false if the file cannot be opened.
inline bool read_values(const std::string& path, std::vector<uint32_t>* out) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  out->clear();
  std::vector<char> buf(1 << 22);
  uint64_t cur = 0;
  bool in_num = false, stop = false;
  while (!stop) {
    const size_t got = std::fread(buf.data(), 1, buf.size(), f);
    if (got == 0) break;
    for (size_t i = 0; i < got; ++i) {
      const unsigned char c = static_cast<unsigned char>(buf[i]);
      if (c >= '0' && c <= '9') {
        cur = cur * 10 + (c - '0');
        if (cur > 0xFFFFFFFFull) {
          stop = true;  // the stream's failbit on overflow
          in_num = false;
          break;
        }
        in_num = true;
      } else if (c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\v' || c == '\f') {
        if (in_num) out->push_back(static_cast<uint32_t>(cur));
        cur = 0;
        in_num = false;
      } else {
        stop = true;  // not a number: the stream fails here
        in_num = false;
        break;
      }
    }
  }
  if (in_num) out->push_back(static_cast<uint32_t>(cur));
  std::fclose(f);
  return true;
}

// The same reading on the device: the file's bytes are copied to the GPU
// and parsed there by wah_parse_text (same rule as read_values), then the
// values come back.  Returns false with a message in *err on failure.
inline bool read_values_gpu(const std::string& path, std::vector<uint32_t>* out,
                            std::string* err) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    *err = "cannot open '" + path + "'";
    return false;
  }
  std::fseek(f, 0, SEEK_END);
  const long len = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  const uint64_t bytes = len > 0 ? static_cast<uint64_t>(len) : 0;
  const uint64_t cap = (bytes + 1) / 2;
  void *h_text = nullptr, *d_text = nullptr, *d_vals = nullptr, *d_res = nullptr, *d_ws = nullptr,
       *stream = nullptr;
  const size_t ws_bytes = wah_parse_workspace_bytes();
  int rc = wah_host_alloc(bytes ? bytes : 1, &h_text);
  if (rc == WAH_OK && bytes && std::fread(h_text, 1, bytes, f) != bytes) rc = WAH_EINVAL;
  std::fclose(f);
  if (rc == WAH_OK) rc = wah_dev_alloc((bytes + 16) & ~uint64_t(15), &d_text);
  if (rc == WAH_OK) rc = wah_dev_alloc((cap ? cap : 1) * 4, &d_vals);
  if (rc == WAH_OK) rc = wah_dev_alloc(sizeof(wah_parse_result), &d_res);
  if (rc == WAH_OK) rc = wah_dev_alloc(ws_bytes, &d_ws);
  if (rc == WAH_OK) rc = wah_stream_create(&stream);
  if (rc == WAH_OK && bytes) rc = wah_copy(d_text, h_text, bytes, stream);
  if (rc == WAH_OK)
    rc = wah_parse_text(d_text, bytes, static_cast<uint32_t*>(d_vals), cap,
                        static_cast<wah_parse_result*>(d_res), d_ws, ws_bytes, stream);
  wah_parse_result res{};
  if (rc == WAH_OK) rc = wah_copy(&res, d_res, sizeof res, stream);
  if (rc == WAH_OK) rc = wah_stream_sync(stream);
  if (rc == WAH_OK) rc = static_cast<int>(res.status);
  if (rc == WAH_OK) {
    out->resize(res.values);
    if (res.values) rc = wah_copy(out->data(), d_vals, res.values * 4, stream);
    if (rc == WAH_OK) rc = wah_stream_sync(stream);
  }
  if (stream) wah_stream_destroy(stream);
  for (void* p : {d_text, d_vals, d_res, d_ws})
    if (p) wah_dev_free(p);
  if (h_text) wah_host_free(h_text);
  if (rc != WAH_OK) {
    *err = std::string("parsing '") + path + "' on the GPU: " + wah_strerror(rc);
    return false;
  }
  return true;
}

// The reference's built-in 32-value fixture (src/cpu.cpp:292-295).
inline std::vector<uint32_t> builtin_values() {
  return {10, 7, 22, 6, 7, 1, 9, 42, 2, 5, 13, 3, 2, 1, 0, 1,
          18, 18, 3, 13, 5, 9, 0, 3, 2, 19, 5, 23, 22, 10, 6, 22};
}

// Bit string of one key's words, trailing zeros trimmed (src/cpu.cpp:47-74).
inline std::string decoded_bitmap(const uint32_t* words, size_t count) {
  std::string s;
  for (size_t w = 0; w < count; ++w) {
    const uint32_t block = words[w];
    if (block & 0x80000000u) {
      for (int i = 0; i < 31; ++i) s.push_back((block >> i) & 1u ? '1' : '0');
    } else {
      const char bit = (block & 0x40000000u) ? '1' : '0';
      const uint32_t times = block & 0x3FFFFFFFu;
      s.append(static_cast<size_t>(times) * 31, bit);
    }
  }
  const auto last = s.find_last_not_of('0');
  s.erase(last == std::string::npos ? 0 : last + 1);
  return s;
}

// The cpu program's -p listing: keys 0..max present key, an absent key as
// "j\t" (src/cpu.cpp:329-351).
inline void print_index(const uint32_t* keys, const uint32_t* offsets, size_t K,
                        const uint32_t* index, size_t L) {
  uint64_t next = 0;
  for (size_t i = 0; i < K; ++i) {
    const uint64_t key = keys[i];
    const size_t begin = offsets[i];
    const size_t end = (i + 1 < K) ? offsets[i + 1] : L;
    for (uint64_t j = next; j < key; ++j) std::printf("%llu\t\n", (unsigned long long)j);
    std::printf("%llu\t%s\n", (unsigned long long)key,
                decoded_bitmap(index + begin, end - begin).c_str());
    next = key + 1;
  }
}
inline void print_index(const std::vector<uint32_t>& keys, const std::vector<uint32_t>& offsets,
                        const std::vector<uint32_t>& index) {
  print_index(keys.data(), offsets.data(), keys.size(), index.data(), index.size());
}

// Result file: u32 K, u32 L, keys[K], offsets[K], index[L] (little endian).
inline bool write_result(const std::string& path, const uint32_t* keys, const uint32_t* offsets,
                         size_t K, const uint32_t* index, size_t L) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  const uint32_t head[2] = {static_cast<uint32_t>(K), static_cast<uint32_t>(L)};
  bool ok = std::fwrite(head, 4, 2, f) == 2;
  ok = ok && std::fwrite(keys, 4, K, f) == K;
  ok = ok && std::fwrite(offsets, 4, K, f) == K;
  ok = ok && std::fwrite(index, 4, L, f) == L;
  return std::fclose(f) == 0 && ok;
}
inline bool write_result(const std::string& path, const std::vector<uint32_t>& keys,
                         const std::vector<uint32_t>& offsets, const std::vector<uint32_t>& index) {
  return write_result(path, keys.data(), offsets.data(), keys.size(), index.data(), index.size());
}

// Page-locked host array of u32 (copies to and from it run at link speed).
struct pinned_u32 {
  uint32_t* p = nullptr;
  size_t n = 0;
  pinned_u32() = default;
  pinned_u32(const pinned_u32&) = delete;
  pinned_u32& operator=(const pinned_u32&) = delete;
  ~pinned_u32() {
    if (p) wah_host_free(p);
  }
  int alloc(size_t count) {
    void* q = nullptr;
    const int rc = wah_host_alloc((count ? count : 1) * 4, &q);
    p = static_cast<uint32_t*>(q);
    n = count;
    return rc;
  }
};

// Device by exact name, else (when fallback) the first device; -1 if none.
inline int find_device(const std::string& name, bool fallback) {
  const int count = wah_device_count();
  char buf[256];
  if (!name.empty()) {
    for (int d = 0; d < count; ++d)
      if (wah_device_name(d, buf, sizeof buf) == WAH_OK && name == buf) return d;
    if (!fallback) return -1;
  }
  return count > 0 ? 0 : -1;
}

inline uint64_t micros_since(std::chrono::steady_clock::time_point t) {
  return static_cast<uint64_t>(std::chrono::duration_cast<std::chrono::microseconds>(
                                   std::chrono::steady_clock::now() - t)
                                   .count());
}

}  // namespace wahcli
