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
