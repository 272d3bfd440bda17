/*
 * cpu -- the reference's sequential `cpu` program (src/cpu.cpp:274-352) over
 * the oracle's C restatement.
 *
 * TEST INFRASTRUCTURE ONLY: the tests run it beside the GPU programs and
 * compare outputs.  Flags as the reference: -f/--data-file, -b/--bound,
 * -p/--print; plus --bubble (the reference's O(n^2) sort instead of the
 * stable sort; same output) and -o/--output FILE (binary result: u32 K, L,
 * keys[K], offsets[K], index[L]).  Without -f it indexes the reference's
 * built-in 32 values (src/cpu.cpp:292-295).  Output lines are the
 * reference's: 'N' values, maximum value, "Merged to k values", "Index has L
 * elements with K keys", and with -p one line per key 0..max key.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "wah_oracle.h"

static int read_values(const char* path, uint32_t** out, size_t* n) {
  FILE* f = fopen(path, "rb");
  size_t cap = 1 << 16, len = 0;
  uint32_t* v;
  unsigned long long cur = 0;
  int in_num = 0, c;
  if (!f) return -1;
  v = (uint32_t*)malloc(cap * sizeof *v);
  if (!v) {
    fclose(f);
    return -1;
  }
  /* whitespace-separated decimals; stop at the first token that is not an
   * unsigned 32-bit number, as `while (source >> next)` does */
  while ((c = fgetc(f)) != EOF) {
    if (c >= '0' && c <= '9') {
      cur = cur * 10 + (unsigned)(c - '0');
      if (cur > 0xFFFFFFFFull) {
        in_num = 0;
        break;
      }
      in_num = 1;
    } else if (c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\v' || c == '\f') {
      if (in_num) {
        if (len == cap) {
          uint32_t* w = (uint32_t*)realloc(v, 2 * cap * sizeof *v);
          if (!w) {
            free(v);
            fclose(f);
            return -1;
          }
          v = w;
          cap *= 2;
        }
        v[len++] = (uint32_t)cur;
      }
      cur = 0;
      in_num = 0;
    } else {
      in_num = 0;
      break;
    }
  }
  if (in_num) {
    if (len == cap) {
      uint32_t* w = (uint32_t*)realloc(v, (cap + 1) * sizeof *v);
      if (!w) {
        free(v);
        fclose(f);
        return -1;
      }
      v = w;
    }
    v[len++] = (uint32_t)cur;
  }
  fclose(f);
  *out = v;
  *n = len;
  return 0;
}

int main(int argc, char** argv) {
  static const uint32_t builtin[32] = {10, 7, 22, 6, 7, 1, 9, 42, 2, 5, 13, 3, 2, 1, 0, 1,
                                       18, 18, 3, 13, 5, 9, 0, 3, 2, 19, 5, 23, 22, 10, 6, 22};
  const char* file = NULL;
  const char* output = NULL;
  unsigned long bound = 0;
  int print = 0, bubble = 0, i;
  uint32_t* values = NULL;
  size_t n = 0, K = 0, L = 0, k = 0, cap;
  uint32_t *keys, *offsets, *index;

  for (i = 1; i < argc; ++i) {
    const char* a = argv[i];
    if (!strcmp(a, "-f") || !strcmp(a, "--data-file")) {
      if (++i >= argc) return 2;
      file = argv[i];
    } else if (!strncmp(a, "--data-file=", 12)) {
      file = a + 12;
    } else if (!strcmp(a, "-b") || !strcmp(a, "--bound")) {
      if (++i >= argc) return 2;
      bound = strtoul(argv[i], NULL, 10);
    } else if (!strncmp(a, "--bound=", 8)) {
      bound = strtoul(a + 8, NULL, 10);
    } else if (!strcmp(a, "-p") || !strcmp(a, "--print")) {
      print = 1;
    } else if (!strcmp(a, "--bubble")) {
      bubble = 1;
    } else if (!strcmp(a, "-o") || !strcmp(a, "--output")) {
      if (++i >= argc) return 2;
      output = argv[i];
    } else if (!strncmp(a, "--output=", 9)) {
      output = a + 9;
    } else {
      fprintf(stderr, "unknown option '%s'\n", a);
      return 2;
    }
  }
  if (file) {
    printf("Reading data from '%s' ... ", file);
    fflush(stdout);
    if (read_values(file, &values, &n) != 0) {
      fprintf(stderr, "cannot read '%s'\n", file);
      return 2;
    }
  } else {
    n = 32;
    values = (uint32_t*)malloc(sizeof builtin);
    if (!values) return 1;
    memcpy(values, builtin, sizeof builtin);
  }
  printf("'%zu' values.\n", n);
  if (bound == 0) {
    size_t j;
    for (j = 0; j < n; ++j)
      if (values[j] > bound) bound = values[j];
  }
  printf("Maximum value is '%lu'.\n", bound);

  cap = n ? n : 1;
  keys = (uint32_t*)malloc(cap * 4);
  offsets = (uint32_t*)malloc(cap * 4);
  index = (uint32_t*)malloc(2 * cap * 4);
  if (!keys || !offsets || !index ||
      wah_oracle_build(values, n, bubble ? WAH_ORACLE_SORT_BUBBLE : WAH_ORACLE_SORT_STABLE, keys,
                       offsets, index, &K, &L, &k) != 0) {
    fprintf(stderr, "out of memory\n");
    return 1;
  }
  printf("Merged to %zu values\n", k);
  printf("Index has %zu elements with %zu keys\n", L, K);
  if (print) {
    size_t next = 0, j, bits_cap = 1024;
    char* bits = (char*)malloc(bits_cap);
    if (!bits) return 1;
    for (j = 0; j < K; ++j) {
      const size_t begin = offsets[j];
      const size_t end = (j + 1 < K) ? offsets[j + 1] : L;
      size_t need = wah_oracle_decoded_bitmap(index + begin, end - begin, bits, bits_cap);
      if (need + 1 > bits_cap) {
        char* b2 = (char*)realloc(bits, need + 1);
        if (!b2) return 1;
        bits = b2;
        bits_cap = need + 1;
        wah_oracle_decoded_bitmap(index + begin, end - begin, bits, bits_cap);
      }
      for (; next < keys[j]; ++next) printf("%zu\t\n", next);
      printf("%u\t%s\n", keys[j], bits);
      next = (size_t)keys[j] + 1;
    }
    free(bits);
  }
  if (output) {
    FILE* f = fopen(output, "wb");
    uint32_t head[2];
    int ok;
    head[0] = (uint32_t)K;
    head[1] = (uint32_t)L;
    ok = f && fwrite(head, 4, 2, f) == 2 && fwrite(keys, 4, K, f) == K &&
         fwrite(offsets, 4, K, f) == K && fwrite(index, 4, L, f) == L;
    if (f && fclose(f) != 0) ok = 0;
    if (!ok) {
      fprintf(stderr, "cannot write '%s'\n", output);
      return 1;
    }
  }
  free(values);
  free(keys);
  free(offsets);
  free(index);
  return 0;
}
