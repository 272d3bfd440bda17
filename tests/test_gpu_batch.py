"""Batched builds (wah_batch_*): every column equals the oracle's index of
that column alone; graph replays on new columns of the same sizes too."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def wah():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import indexing_gb300 as w
    w._lib.load()
    return w


def mixed_columns(rng, ncols, max_n):
    sizes, bounds, cols = [], [], []
    for c in range(ncols):
        n = int(np.exp(rng.uniform(0, np.log(max_n))))
        if c % 17 == 0:
            n = 0
        card = int(np.exp(rng.uniform(np.log(2), np.log(65536))))
        kind = c % 4
        if kind == 0:
            v = rng.integers(0, card, size=n, dtype=np.uint32)
        elif kind == 1:
            runs = rng.geometric(1 / 100, size=n // 50 + 2)
            v = np.repeat(rng.integers(0, card, size=runs.size, dtype=np.uint32), runs)[:n]
        elif kind == 2:
            v = rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)
            card = 0
        else:
            v = np.full(n, rng.integers(0, card), np.uint32)
        sizes.append(n)
        bounds.append(0 if card == 0 or c % 3 == 0 else card - 1)
        cols.append(v)
    return sizes, bounds, cols


def check(results, cols):
    for c, (r, v) in enumerate(zip(results, cols)):
        g = r.numpy()
        ref = O.build(v)
        assert np.array_equal(g.keys, ref.keys), f"column {c}: keys"
        assert np.array_equal(g.offsets, ref.offsets), f"column {c}: offsets"
        assert np.array_equal(g.index, ref.index), f"column {c}: index"
        assert g.merged == ref.merged, f"column {c}: k"


def test_batch_matches_oracle(wah):
    rng = np.random.default_rng(40)
    sizes, bounds, cols = mixed_columns(rng, 60, 300_000)
    b = wah.Batch(sizes, bounds)
    dev = [torch.from_numpy(v.view(np.int32)).cuda() for v in cols]
    b.set_columns(dev)
    b.build()
    check(b.results(), cols)
    b.close()


def test_batch_graph_replay_new_columns(wah):
    rng = np.random.default_rng(41)
    sizes, bounds, cols = mixed_columns(rng, 40, 200_000)
    b = wah.Batch(sizes, bounds)
    for rep in range(3):
        if rep:
            # new data, same sizes and bounds
            cols = [(rng.integers(0, max(bd, 1) + 1, size=n, dtype=np.uint64).astype(np.uint32)
                     if bd else rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32))
                    for n, bd in zip(sizes, bounds)]
        dev = [torch.from_numpy(v.view(np.int32)).cuda() for v in cols]
        b.set_columns(dev)
        b.launch_graph()
        check(b.results(), cols)
    b.close()


def test_batch_large_and_tiny_columns(wah):
    # one column spanning many ranges beside single-range ones
    rng = np.random.default_rng(42)
    cols = [rng.integers(0, 65536, size=3_000_000, dtype=np.uint32),
            rng.integers(0, 5, size=1024, dtype=np.uint32),
            np.zeros(0, np.uint32),
            rng.integers(0, 65536, size=4097, dtype=np.uint32)]
    b = wah.Batch([v.size for v in cols], [65535, 4, 0, 65535])
    b.set_columns([torch.from_numpy(v.view(np.int32)).cuda() for v in cols])
    b.build()
    check(b.results(), cols)
    b.close()
