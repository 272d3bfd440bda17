// generate -- test data in the reference's text format: `amount` values,
// uniform in [from, to], separated by `separator` (default newline), with a
// final newline (src/generate_test_data.cpp:18-55).
//
// The reference seeds std::mt19937 from std::random_device, so its files are
// not reproducible, and std::uniform_int_distribution's mapping differs
// between standard libraries.  Here the stream is SplitMix64 from --seed,
// mapped to [from, to] by Lemire's multiply-and-reject method (unbiased), so
// one seed gives the same file on every machine.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cli.hpp"

namespace {

struct splitmix64 {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
};

// Uniform in [0, range) for range <= 2^32, from the high 32 bits of each draw.
uint32_t bounded(splitmix64& g, uint64_t range) {
  if (range == (1ull << 32)) return static_cast<uint32_t>(g.next() >> 32);
  uint64_t m = (g.next() >> 32) * range;
  uint32_t low = static_cast<uint32_t>(m);
  if (low < range) {
    const uint32_t threshold = static_cast<uint32_t>((1ull << 32) % range);
    while (low < threshold) {
      m = (g.next() >> 32) * range;
      low = static_cast<uint32_t>(m);
    }
  }
  return static_cast<uint32_t>(m >> 32);
}

}  // namespace

int main(int argc, char** argv) {
  uint64_t from = 0, to = 65535, amount = 268500000, seed = 0x5EED;
  std::string separator = "\n", output;
  const std::vector<wahcli::flag> flags = {
      {"from", 'f', "minimum value (0)", wahcli::flag::U64, &from},
      {"to", 't', "maximum value (65535)", wahcli::flag::U64, &to},
      {"amount", 'a', "number of values (268 500 000)", wahcli::flag::U64, &amount},
      {"separator", 's', "separator between numbers (\\n)", wahcli::flag::STRING, &separator},
      {"seed", 0, "SplitMix64 seed (0x5EED)", wahcli::flag::U64, &seed},
      {"output", 'o', "write to this file instead of stdout", wahcli::flag::STRING, &output},
  };
  const int pf = wahcli::parse_flags(argc, argv, flags);
  if (pf != 0) return pf > 0 ? 0 : 2;
  if (to > 0xFFFFFFFFull || from > to) {
    std::fprintf(stderr, "need from <= to <= 4294967295\n");
    return 2;
  }
  if (separator == "\\n") separator = "\n";
  FILE* out = output.empty() ? stdout : std::fopen(output.c_str(), "wb");
  if (!out) {
    std::fprintf(stderr, "cannot open '%s'\n", output.c_str());
    return 2;
  }
  splitmix64 g{seed};
  const uint64_t range = to - from + 1;
  std::vector<char> buf;
  buf.reserve(1 << 22);
  char digits[16];
  for (uint64_t i = 0; i < amount; ++i) {
    uint64_t v = from + bounded(g, range);
    int d = 0;
    do {
      digits[d++] = static_cast<char>('0' + v % 10);
      v /= 10;
    } while (v);
    while (d) buf.push_back(digits[--d]);
    if (i + 1 < amount) buf.insert(buf.end(), separator.begin(), separator.end());
    if (buf.size() > (1u << 22) - 64) {
      if (std::fwrite(buf.data(), 1, buf.size(), out) != buf.size()) return 1;
      buf.clear();
    }
  }
  buf.push_back('\n');
  if (std::fwrite(buf.data(), 1, buf.size(), out) != buf.size()) return 1;
  if (out != stdout && std::fclose(out) != 0) return 1;
  return 0;
}
