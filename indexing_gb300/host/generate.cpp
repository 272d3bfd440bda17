// generate -- test data in the reference's text format: `amount` values,
// uniform in [from, to], separated by `separator` (default newline), with a
// final newline (src/generate_test_data.cpp:18-55).
//
// The reference seeds std::mt19937 from std::random_device, so its files are
// not reproducible, and std::uniform_int_distribution's mapping differs
// between standard libraries.  Here the stream is SplitMix64 from --seed,
// mapped to [from, to] by Lemire's multiply-and-reject method (unbiased), so
// one seed gives the same file on every machine.  Besides the reference's
// uniform values it writes the other columns of the benchmark workloads
// (--dist zipf: value from + r - 1 with weight r^-s, by a double-precision
// inverse-CDF table; few: `distinct` values uniform; runs: geometric runs of
// mean --run-mean with uniform values) and, with --trace, a Poisson serving
// trace (arrival time, log-uniform rows, distribution per request).
#include <algorithm>
#include <cmath>
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

// Uniform double in (0, 1] from the top 53 bits of a draw.
double unit(splitmix64& g) { return ((g.next() >> 11) + 1) * (1.0 / 9007199254740992.0); }

// Decimal digits of v into buf.
void put_u64(std::vector<char>& buf, uint64_t v) {
  char digits[24];
  int d = 0;
  do {
    digits[d++] = static_cast<char>('0' + v % 10);
    v /= 10;
  } while (v);
  while (d) buf.push_back(digits[--d]);
}

bool parse_double(const std::string& s, double* out) {
  char* end = nullptr;
  *out = std::strtod(s.c_str(), &end);
  return end && *end == '\0' && !s.empty();
}

}  // namespace

int main(int argc, char** argv) {
  uint64_t from = 0, to = 65535, amount = 268500000, seed = 0x5EED, distinct = 16, run_mean = 1000,
           trace = 0, min_rows = 10000, max_rows = 16777216;
  std::string separator = "\n", output, dist = "uniform", zipf_s = "1.1", rate = "1000";
  const std::vector<wahcli::flag> flags = {
      {"from", 'f', "minimum value (0)", wahcli::flag::U64, &from},
      {"to", 't', "maximum value (65535)", wahcli::flag::U64, &to},
      {"amount", 'a', "number of values (268 500 000)", wahcli::flag::U64, &amount},
      {"separator", 's', "separator between numbers (\\n)", wahcli::flag::STRING, &separator},
      {"seed", 0, "SplitMix64 seed (0x5EED)", wahcli::flag::U64, &seed},
      {"output", 'o', "write to this file instead of stdout", wahcli::flag::STRING, &output},
      {"dist", 0, "uniform | zipf | few | runs (uniform)", wahcli::flag::STRING, &dist},
      {"zipf-s", 0, "zipf exponent; value from + r - 1 has weight r^-s (1.1)",
       wahcli::flag::STRING, &zipf_s},
      {"distinct", 0, "few: values uniform in [from, from + distinct - 1] (16)",
       wahcli::flag::U64, &distinct},
      {"run-mean", 0, "runs: geometric run lengths of this mean, run values uniform (1000)",
       wahcli::flag::U64, &run_mean},
      {"trace", 0, "instead of values: this many serving requests, one per line "
                   "(arrival seconds, rows, distribution)", wahcli::flag::U64, &trace},
      {"rate", 0, "trace: Poisson arrivals per second (1000)", wahcli::flag::STRING, &rate},
      {"min-rows", 0, "trace: rows log-uniform from (10000)", wahcli::flag::U64, &min_rows},
      {"max-rows", 0, "trace: rows log-uniform to (16777216)", wahcli::flag::U64, &max_rows},
  };
  const int pf = wahcli::parse_flags(argc, argv, flags);
  if (pf != 0) return pf > 0 ? 0 : 2;
  if (to > 0xFFFFFFFFull || from > to) {
    std::fprintf(stderr, "need from <= to <= 4294967295\n");
    return 2;
  }
  const uint64_t range = to - from + 1;
  double s_exp = 0, lambda = 0;
  if (dist != "uniform" && dist != "zipf" && dist != "few" && dist != "runs") {
    std::fprintf(stderr, "unknown --dist '%s'\n", dist.c_str());
    return 2;
  }
  if (!parse_double(zipf_s, &s_exp) || s_exp <= 0 || !parse_double(rate, &lambda) || lambda <= 0 ||
      distinct == 0 || run_mean == 0 || min_rows == 0 || max_rows < min_rows) {
    std::fprintf(stderr, "bad --zipf-s, --rate, --distinct, --run-mean or row range\n");
    return 2;
  }
  if (dist == "zipf" && range > (1ull << 26)) {
    std::fprintf(stderr, "zipf needs to - from < 2^26 (its inverse-CDF table)\n");
    return 2;
  }
  if (separator == "\\n") separator = "\n";
  FILE* out = output.empty() ? stdout : std::fopen(output.c_str(), "wb");
  if (!out) {
    std::fprintf(stderr, "cannot open '%s'\n", output.c_str());
    return 2;
  }
  splitmix64 g{seed};
  std::vector<char> buf;
  buf.reserve(1 << 22);
  auto flush = [&](bool force) {
    if ((force || buf.size() > (1u << 22) - 256) && !buf.empty()) {
      if (std::fwrite(buf.data(), 1, buf.size(), out) != buf.size()) return false;
      buf.clear();
    }
    return true;
  };

  if (trace) {
    // serving trace: Poisson arrivals, rows log-uniform, uniform / zipf /
    // runs with probability 1/3 each (the batched-serving workload)
    static const char* kinds[3] = {"uniform", "zipf", "runs"};
    const double lo = std::log((double)min_rows), hi = std::log((double)max_rows);
    double t = 0;
    for (uint64_t i = 0; i < trace; ++i) {
      t += -std::log(unit(g)) / lambda;
      uint64_t rows = (uint64_t)std::llround(std::exp(lo + (hi - lo) * (unit(g) - 0x1p-53)));
      rows = std::min(std::max(rows, min_rows), max_rows);
      const char* kind = kinds[bounded(g, 3)];
      char line[128];
      const int len = std::snprintf(line, sizeof line, "%.9f %llu %s\n", t,
                                    (unsigned long long)rows, kind);
      buf.insert(buf.end(), line, line + len);
      if (!flush(false)) return 1;
    }
    if (!flush(true)) return 1;
    if (out != stdout && std::fclose(out) != 0) return 1;
    return 0;
  }

  std::vector<double> cdf;  // zipf: cumulative weights of ranks 1..range
  if (dist == "zipf") {
    cdf.resize(range);
    double acc = 0;
    for (uint64_t r = 0; r < range; ++r) cdf[r] = acc += std::pow((double)(r + 1), -s_exp);
    for (double& c : cdf) c /= acc;
  }
  const uint64_t few = std::min<uint64_t>(distinct, range);
  const double log_q = std::log(1.0 - 1.0 / (double)run_mean);
  uint64_t run_left = 0, run_value = 0;
  for (uint64_t i = 0; i < amount; ++i) {
    uint64_t v;
    if (dist == "uniform") {
      v = from + bounded(g, range);
    } else if (dist == "few") {
      v = from + bounded(g, few);
    } else if (dist == "zipf") {
      const double u = unit(g);
      v = from + (uint64_t)(std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
      if (v > to) v = to;
    } else {  // runs
      if (run_left == 0) {
        run_value = from + bounded(g, range);
        // geometric length >= 1 with mean run_mean
        run_left = run_mean == 1 ? 1 : 1 + (uint64_t)(std::log(unit(g)) / log_q);
      }
      v = run_value;
      --run_left;
    }
    put_u64(buf, v);
    if (i + 1 < amount) buf.insert(buf.end(), separator.begin(), separator.end());
    if (!flush(false)) return 1;
  }
  buf.push_back('\n');
  if (!flush(true)) return 1;
  if (out != stdout && std::fclose(out) != 0) return 1;
  return 0;
}
