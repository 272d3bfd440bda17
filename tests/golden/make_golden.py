"""Generates tests/golden/golden.npz from the reference's own code.

Runs in the development container only: it needs oracle/_ref/libref_cpu.so,
which oracle/Makefile compiles from the reference's unmodified src/cpu.cpp
(`make -C oracle ref`).  Each case stores the input column and the
reference's keys / offsets / index / merged count.  Small columns go through
the reference's own bubble sort (src/cpu.cpp:180-197), larger ones through
the stable sort of src/phases.cpp:143-160.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402


def cases():
    rng = np.random.default_rng(20170101)
    c = {}
    # KAT-1: the built-in column of src/cpu.cpp:292-295 (no fill words)
    c["kat1_builtin32"] = np.array(
        [10, 7, 22, 6, 7, 1, 9, 42, 2, 5, 13, 3, 2, 1, 0, 1, 18, 18, 3, 13,
         5, 9, 0, 3, 2, 19, 5, 23, 22, 10, 6, 22], np.uint32)
    # KAT-2: fills, 0xFFFFFFFF literals and OR-merges
    c["kat2_fills300"] = np.array(
        [1 if i % 97 == 0 else (2 if (i // 40) % 2 else 3) for i in range(300)], np.uint32)
    c["single_row"] = np.array([7], np.uint32)
    c["single_zero"] = np.array([0], np.uint32)
    c["n31_all_equal"] = np.full(31, 5, np.uint32)
    c["n32_all_equal"] = np.full(32, 5, np.uint32)
    c["n62_two_chunks"] = (np.arange(62) // 31).astype(np.uint32)
    c["all_equal_1000"] = np.full(1000, 123456, np.uint32)
    c["descending_2000"] = np.arange(2000, 0, -1).astype(np.uint32)
    c["ascending_2000"] = np.arange(2000).astype(np.uint32)
    c["max_uint32_mix"] = rng.choice(np.array([0, 1, 0xFFFFFFFF, 0xFFFFFFFE, 0x80000000],
                                              np.uint32), size=1500)
    c["full_u32_random_3000"] = rng.integers(0, 2 ** 32, size=3000, dtype=np.uint64).astype(
        np.uint32)
    c["uniform16_5000"] = rng.integers(0, 65536, size=5000, dtype=np.uint32)
    c["uniform16_70000"] = rng.integers(0, 65536, size=70000, dtype=np.uint32)
    c["few16_10000"] = rng.integers(0, 16, size=10000, dtype=np.uint32)
    c["two_values_4093"] = rng.integers(0, 2, size=4093, dtype=np.uint32)
    # run-clustered: geometric run lengths (mean 100), uniform run values
    runs = rng.geometric(1 / 100, size=400)
    vals = rng.integers(0, 65536, size=400, dtype=np.uint32)
    c["runs_mean100"] = np.repeat(vals, runs)[:30000]
    # 31-row aligned runs -> full 0xFFFFFFFF literals and long fills
    c["aligned_runs_31"] = np.repeat(rng.integers(0, 8, size=300, dtype=np.uint32), 31)
    # sparse value among zeros -> long zero fills
    sp = np.zeros(50000, np.uint32)
    sp[rng.choice(50000, size=40, replace=False)] = 9
    c["sparse_fills_50000"] = sp
    # Zipf s=1.1 over 65536 values via inverse CDF
    w = 1.0 / np.arange(1, 65537, dtype=np.float64) ** 1.1
    cdf = np.cumsum(w) / w.sum()
    c["zipf11_20000"] = np.searchsorted(cdf, rng.random(20000)).astype(np.uint32)
    # sizes around the GPU tile edges (2048-row build tiles, 4096-row sort tiles)
    for n in (2047, 2048, 2049, 4095, 4096, 4097, 8193):
        c[f"edge_{n}"] = rng.integers(0, 300, size=n, dtype=np.uint32)
    return c


def main():
    O.make(ref=True)
    out = {}
    for name, v in cases().items():
        r = O.ref_build(v, bubble=v.size <= 2000)
        out[f"{name}/values"] = v
        out[f"{name}/keys"] = r.keys
        out[f"{name}/offsets"] = r.offsets
        out[f"{name}/index"] = r.index
        out[f"{name}/merged"] = np.array([r.merged], np.uint64)
    path = os.path.join(HERE, "golden.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {len(out) // 5} cases, {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
