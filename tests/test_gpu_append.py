"""Incremental append on the GPU (wah_append): a column indexed slice by
slice and appended on the device equals the oracle's index of the whole
column, word for word (the reference's plain per-key append does not: its
slices' leading fills are never re-based).  Integer work: bit-exact."""
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


def u32(t):
    return t.cpu().numpy().view(np.uint32)


def columns():
    rng = np.random.default_rng(5)
    yield "kat2", np.array([(1 if i % 97 == 0 else (2 if (i // 40) % 2 else 3))
                            for i in range(300)], np.uint32)
    yield "uniform16", rng.integers(0, 65536, size=200_003, dtype=np.uint32)
    yield "few", rng.integers(0, 5, size=150_001, dtype=np.uint32)
    yield "u32", rng.integers(0, 2 ** 32, size=90_000, dtype=np.uint64).astype(np.uint32)
    runs = rng.geometric(1 / 2000, size=200)
    yield "runs", np.repeat(rng.integers(0, 300, size=200, dtype=np.uint32), runs)[:240_000]
    sparse = np.zeros(300_000, np.uint32)
    sparse[rng.choice(300_000, 40, replace=False)] = rng.integers(1, 6, size=40, dtype=np.uint32)
    yield "sparse", sparse


def assert_index(got, ref, what):
    g = got.numpy()
    assert np.array_equal(g.keys, ref.keys), f"{what}: keys"
    assert np.array_equal(g.offsets, ref.offsets), f"{what}: offsets"
    assert g.index.size == ref.index.size, f"{what}: L {g.index.size} != {ref.index.size}"
    assert np.array_equal(g.index, ref.index), f"{what}: words"


@pytest.mark.parametrize("name,v", list(columns()))
def test_slices_appended_equal_whole_column(wah, name, v):
    n = v.size
    rng = np.random.default_rng(n)
    ref = O.build(v)
    for parts in (2, 5):
        cuts = sorted(set(int(c) // 31 * 31 for c in rng.integers(1, n, size=parts - 1)))
        bounds = [0] + [c for c in cuts if 0 < c < n] + [n]
        acc = wah.build_index(v[bounds[0]:bounds[1]])
        for lo, hi in zip(bounds[1:-1], bounds[2:]):
            acc = wah.append(acc, lo, wah.build_index(v[lo:hi]))
        assert_index(acc, ref, f"{name} cut at {bounds}")


def test_append_edges(wah):
    rng = np.random.default_rng(8)
    v = rng.integers(0, 100, size=31 * 1000 + 7, dtype=np.uint32)
    whole = O.build(v)
    empty = wah.build_index(np.zeros(0, np.uint32))
    # empty + B = B; A + empty = A
    b = wah.build_index(v)
    assert_index(wah.append(empty, 0, b), whole, "empty + B")
    assert_index(wah.append(b, 31 * 1001, empty), whole, "A + empty")
    # one-chunk slices, and a slice made of keys A never had
    w2 = np.concatenate([v[:3100], np.full(31, 7777, np.uint32), v[3131:6200]])
    acc = wah.build_index(w2[:3100])
    acc = wah.append(acc, 3100, wah.build_index(w2[3100:3131]))
    acc = wah.append(acc, 3131, wah.build_index(w2[3131:]))
    assert_index(acc, O.build(w2), "one-chunk slice of a new key")


def test_append_errors(wah):
    v = np.arange(93, dtype=np.uint32) % 5
    a = wah.build_index(v[:62])
    b = wah.build_index(v[62:])
    with pytest.raises(wah.WahError) as e:
        wah.append(a, 61, b)  # not a multiple of 31
    assert e.value.status == wah.WAH_ERANGE
    with pytest.raises(wah.WahError) as e:
        wah.append(a, 31, b)  # A has rows past 31: B's rows would overlap them
    assert e.value.status == wah.WAH_ECORRUPT


def test_append_large(wah):
    """268,435,456 rows in four slices appended on the device equal one build
    of the whole column (compared with the GPU's own whole-column build)."""
    n = 268_435_456
    g = torch.Generator(device="cuda")
    g.manual_seed(12)
    col = torch.randint(0, 65536, (n,), device="cuda", dtype=torch.int32, generator=g)
    whole = wah.build_index(col, bound=65535)
    step = (n // 4) // 124 * 124  # slices start on 31-row chunks
    acc = wah.build_index(col[:step], bound=65535)
    for lo in (step, 2 * step, 3 * step):
        hi = lo + step if lo < 3 * step else n
        acc = wah.append(acc, lo, wah.build_index(col[lo:hi], bound=65535))
    assert torch.equal(acc.keys, whole.keys)
    assert torch.equal(acc.offsets, whole.offsets)
    assert torch.equal(acc.index, whole.index)
