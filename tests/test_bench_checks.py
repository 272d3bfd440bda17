"""The benchmark's parity machinery, on the CPU: the oracle comparison finds
a planted difference, and the 64-bit result fingerprint used for the served
requests tells different indexes apart and equal ones together."""
import numpy as np
import pytest

import bench

torch = pytest.importorskip("torch")


def _oracle_result(v):
    from oracle import oracle as O
    r = O.build(v)
    return (0, len(r.keys), len(r.index), r.merged, r.keys.copy(), r.offsets.copy(),
            r.index.copy())


def test_check_columns_finds_a_planted_difference():
    rng = np.random.default_rng(3)
    cols = [rng.integers(0, 1000, size=n, dtype=np.uint32) for n in (1, 31, 5000, 20000)]
    jobs = [(v, _oracle_result(v)) for v in cols]
    assert bench.check_columns(jobs, 2) == ([], 4)
    st, K, L, k, keys, offs, index = jobs[2][1]
    index = index.copy()
    index[L // 2] ^= 1  # one flipped bit in one word
    jobs[2] = (cols[2], (st, K, L, k, keys, offs, index))
    assert bench.check_columns(jobs, 2) == ([2], 4)
    # a wrong merged count and a nonzero status are differences too
    jobs[2] = (cols[2], (st, K, L, k + 1, keys, offs, _oracle_result(cols[2])[6]))
    assert bench.check_columns(jobs, 1)[0] == [2]
    jobs[2] = (cols[2], (5,) + _oracle_result(cols[2])[1:])
    assert bench.check_columns(jobs, 1)[0] == [2]


def test_result_fingerprint():
    mult = bench.hash_multipliers(torch, "cpu", 1 << 14, 11)
    rng = np.random.default_rng(4)
    v = rng.integers(0, 300, size=3000, dtype=np.uint32)
    _, K, L, k, keys, offs, index = _oracle_result(v)

    def h(keys, offs, index, K=K, L=L, k=k):
        t = [torch.from_numpy(a.view(np.int32).copy()) for a in (keys, offs, index)]
        return int(bench.result_hash(torch, *t, K, L, k, mult))
    base = h(keys, offs, index)
    assert base == h(keys.copy(), offs.copy(), index.copy())
    flipped = index.copy()
    flipped[7] ^= 1 << 30
    assert h(keys, offs, flipped) != base
    swapped = index.copy()
    swapped[[3, 4]] = swapped[[4, 3]]
    assert h(keys, offs, swapped) != base
    assert h(keys, offs, index, k=k + 1) != base
    shifted = offs.copy()
    shifted[1] += 1
    assert h(keys, shifted, index) != base


def test_build_bytes_follows_the_library_geometry():
    """The benchmark's algorithmic bytes per phase: the 268,435,456-row
    16-bit column exchanges packed words (8 B/row per digit pass, 32.4n +
    4L + 8K in all), the 1,048,576-row column keeps the 16-bit exchange, a
    one-byte column takes one pass, and full 32-bit keys four."""
    n, sms = 268_435_456, 152
    L, K = 2 * n - 1000, 65_536
    alg, passes, mid16, derive, packed = bench.build_bytes(n, 65_536, L, K, 524, sms)
    assert (passes, mid16, derive, packed) == (2, True, True, True)
    assert alg["scatter0"] == alg["scatter1"] == 8 * n
    assert alg["pass2"] == alg["pass3"] == 0
    total = sum(alg[p] for p in ("histogram", "pass0", "pass1", "build"))
    assert total == 4 * n + (8 * n + n // 8) + (8 * n + 4 * n + 4 * K) + \
        2 * (4 * n + n // 8) + 4 * L + 4 * K
    assert abs((total - 4 * L - 8 * K) / n - 32.375) < 1e-9
    # C1: pass-0 ranges of one 2,048- or 3,072-row tile, below 2^16 rows
    n1 = 1 << 20
    for tuning in (8, 524):
        alg1, _, _, derive1, packed1 = bench.build_bytes(n1, 65_536, 2 * n1, K, tuning, sms)
        assert derive1 and not packed1
        assert alg1["scatter0"] == alg1["scatter1"] == 10 * n1
    # the packed exchange forced by the tuning word
    assert bench.build_bytes(n1, 65_536, 2 * n1, K, 524 | 0x400, sms)[4]
    # values below 256: one pass, no key starts
    alg2, passes2, _, derive2, packed2 = bench.build_bytes(n, 256, n, 256, 524, sms)
    assert (passes2, derive2, packed2) == (1, False, False)
    assert alg2["scatter0"] == 12 * n and alg2["scatter1"] == 0
    # full 32-bit keys: four passes of 32-bit keys and row ids
    alg3, passes3, mid3, derive3, _ = bench.build_bytes(n, 1 << 32, n, n, 524, sms)
    assert (passes3, mid3, derive3) == (4, False, False)
    assert [alg3[f"scatter{p}"] for p in range(4)] == [12 * n, 16 * n, 16 * n, 16 * n]
