"""A numpy model of the packed exchange between the two digit passes of a
key-start-mode build, checked on the CPU.

Digit pass 0 sorts each row range stably by the low digit and writes, for
every row, one word: (row offset in its pass-0 range) << 8 | high digit.
Its output is bin-major: for each low digit, the ranges' runs in range
order; seg0[b][r] is where the run of (bin b, range r) starts.  Digit pass 1
sees only the words; a row's pass-0 run is the last run start (in that
bin-major order) at or before the row's position, and its row id is
range * range_rows + offset.  The model rebuilds the row ids that way and
checks them against the true pass-0 order, then checks that the stable
pass-1 order equals a stable sort by key -- for uniform keys, few keys,
empty runs (ranges and bins without rows) and a ragged last range.
The kernels doing this are scatter_pack0 / scatter_pack1 in wah_sort.cu;
the GPU tests check their output against the oracle.
"""
import numpy as np
import pytest


def pass0_packed(keys: np.ndarray, range_rows: int):
    n = keys.size
    ranges = -(-n // range_rows)
    lo = keys & 0xFF
    counts = np.zeros((256, ranges), np.int64)  # rows of bin b in range r
    r_of = np.arange(n) // range_rows
    np.add.at(counts, (lo, r_of), 1)
    starts = np.concatenate([[0], np.cumsum(counts.ravel())[:-1]]).reshape(256, ranges)
    order = np.empty(n, np.int64)  # pass-0 output position -> row
    words = np.empty(n, np.uint32)
    nxt = starts.copy()
    for i in range(n):  # stable: rows in row order within each run
        b, r = lo[i], r_of[i]
        p = nxt[b, r]
        nxt[b, r] += 1
        order[p] = i
        words[p] = ((i - r * range_rows) << 8) | (keys[i] >> 8)
    return order, words, starts


def rows_from_words(words: np.ndarray, starts: np.ndarray, range_rows: int):
    flat = starts.ravel()  # bin-major run starts, ascending
    ranges = starts.shape[1]
    pos = np.arange(words.size)
    run = np.searchsorted(flat, pos, side="right") - 1  # last start <= pos
    r = run % ranges
    return r * range_rows + (words >> 8).astype(np.int64)


@pytest.mark.parametrize("n,range_rows,kind", [
    (5000, 700, "uniform"), (5000, 700, "few"), (4097, 1024, "uniform"),
    (3000, 3000, "uniform"), (2500, 64, "sparse"), (1, 8, "uniform")])
def test_packed_words_recover_rows_and_order(n, range_rows, kind):
    rng = np.random.default_rng(n + range_rows)
    if kind == "uniform":
        keys = rng.integers(0, 65536, n).astype(np.uint32)
    elif kind == "few":
        keys = rng.choice(np.array([3, 259, 515, 65535], np.uint32), n)
    else:  # most bins empty in most ranges
        keys = rng.choice(np.array([0x0101, 0x0201, 0xff07], np.uint32), n)
    order, words, starts = pass0_packed(keys, range_rows)
    rows = rows_from_words(words, starts, range_rows)
    assert np.array_equal(rows, order)
    # pass 1: stable by the high digit, carried in the low byte of the word
    p1 = np.argsort(words & 0xFF, kind="stable")
    assert np.array_equal(rows[p1], np.argsort(keys, kind="stable"))
    # the offset fits 24 bits when a range holds fewer than 2^24 rows
    assert range_rows < (1 << 24)
