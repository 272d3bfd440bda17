"""A numpy model of the GPU build's integer arithmetic, checked against the
oracle on the CPU (no GPU; the CUDA kernels themselves are checked by the
-m gpu parity tests).  It restates, per sorted row:

* key-start mode (indexing_gb300/csrc/wah_sort.cu, k_range_count +
  k_key_starts): the rows of every 16-bit key, counted over the whole column,
  scanned in key order, mark where each key starts in the stable sorted
  order; the keys come out in order and the sorted keys themselves are never
  needed;
* the word count of k_build_count (indexing_gb300/csrc/wah_index.cu,
  count_words): x = c + 1 at a key start, else the chunk step c - pc; a row
  adds min(x, 2) words and min(x, 1) segments;
* the words of k_build_emit: every row with x != 0 heads a segment, writes
  the fill x - 1 when it is not zero, then the literal, bit 31 plus the OR of
  1 << (rid % 31) over the segment's rows.

The model is test infrastructure: it proves the formulas, the oracle proves
the model (src/cpu.cpp:176-272 restated in oracle/wah_oracle.c).
"""
import numpy as np
import pytest

from oracle import oracle as O


def model_build(v: np.ndarray):
    v = np.asarray(v, dtype=np.uint32)
    n = v.size
    if n == 0:
        return np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.uint32), 0
    assert int(v.max()) < 65536, "key-start mode needs every key below 2^16"
    # stable LSD sort by the low, then the high digit: the row ids
    rid = np.argsort(v & 0xFF, kind="stable")
    rid = rid[np.argsort(v[rid] >> 8, kind="stable")].astype(np.int64)
    # key starts from the full-key counts (no sorted keys read)
    counts = np.bincount(v, minlength=65536).astype(np.int64)
    present = np.flatnonzero(counts)
    first_row = np.concatenate([[0], np.cumsum(counts)[:-1]])[present]
    start = np.zeros(n, dtype=bool)
    start[first_row] = True
    keys = present.astype(np.uint32)
    # words and segments per row
    c = rid // 31
    pc = np.concatenate([[0], c[:-1]])
    x = np.where(start, c + 1, c - pc)
    assert (x >= 0).all(), "chunks ascend within a key"
    head = x != 0
    words_per_row = np.minimum(x, 2)
    merged = int(np.minimum(x, 1).sum())
    # literals: OR of the segment's row bits, bit 31 set
    seg = np.cumsum(head) - 1
    bits = (np.uint64(1) << (rid % 31).astype(np.uint64)).astype(np.uint64)
    lits = np.zeros(int(head.sum()), dtype=np.uint64)
    np.bitwise_or.at(lits, seg, bits)
    lits = (lits | np.uint64(0x80000000)).astype(np.uint32)
    fills = (x[head] - 1).astype(np.uint32)
    # interleave [fill if nonzero, literal] per head
    nw = np.where(fills != 0, 2, 1)
    pos = np.concatenate([[0], np.cumsum(nw)[:-1]])
    index = np.zeros(int(nw.sum()), dtype=np.uint32)
    has_fill = fills != 0
    index[pos[has_fill]] = fills[has_fill]
    index[pos + nw - 1] = lits
    assert index.size == int(words_per_row.sum())
    # offsets: the first word of each key's first segment
    head_rows = np.flatnonzero(head)
    key_head = start[head_rows]
    offsets = pos[key_head].astype(np.uint32)
    assert offsets.size == keys.size
    return keys, offsets, index, merged


def gen(kind, n, rng):
    if kind == "uniform16":
        return rng.integers(0, 65536, size=n, dtype=np.uint32)
    if kind == "few":
        return rng.integers(300, 320, size=n, dtype=np.uint32)
    if kind == "runs":
        runs = rng.geometric(1 / 200, size=n // 100 + 2)
        vals = rng.integers(0, 65536, size=runs.size, dtype=np.uint32)
        return np.repeat(vals, runs)[:n]
    if kind == "zipf":
        w = 1.0 / np.arange(1, 65537, dtype=np.float64) ** 1.1
        cdf = np.cumsum(w) / w.sum()
        return np.minimum(np.searchsorted(cdf, rng.random(n)), 65535).astype(np.uint32)
    raise ValueError(kind)


@pytest.mark.parametrize("kind", ["uniform16", "few", "runs", "zipf"])
@pytest.mark.parametrize("n", [1, 2, 30, 31, 32, 62, 63, 1000, 4097, 65_537])
def test_model_matches_oracle(kind, n):
    rng = np.random.default_rng(hash((kind, n)) & 0xFFFFFFFF)
    v = gen(kind, n, rng)
    keys, offsets, index, merged = model_build(v)
    ref = O.build(v)
    assert np.array_equal(keys, ref.keys)
    assert np.array_equal(offsets, ref.offsets)
    assert np.array_equal(index, ref.index)
    assert merged == ref.merged


def test_model_matches_golden_vectors(golden):
    for name, case in golden.items():
        v = case["values"]
        if v.size == 0 or int(v.max()) >= 65536:
            continue  # key-start mode covers 16-bit columns only
        keys, offsets, index, merged = model_build(v)
        assert np.array_equal(keys, case["keys"]), name
        assert np.array_equal(offsets, case["offsets"]), name
        assert np.array_equal(index, case["index"]), name
        assert merged == int(case["merged"][0]), name
