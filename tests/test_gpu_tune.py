"""The autotuner: it picks one of the compiled tile shapes, records it in
its cache file, applies the cached entry without timing on the next call,
and builds after tuning still match the oracle.  Integer work: bit-exact."""
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


def test_autotune_cache_and_parity(wah, tmp_path):
    lib = wah._lib.load()
    before = lib.wah_get_tuning()
    cache = str(tmp_path / "tune.txt")
    try:
        t, cached = wah.autotune(1 << 21, 65535, cache)
        assert not cached
        assert t & 0xff in (8, 12, 16)
        assert lib.wah_get_tuning() == t
        lines = open(cache).read().splitlines()
        assert len(lines) == 1 and int(lines[0].split()[-2]) == t
        # a different size in the same power-of-two bucket: from the cache
        lib.wah_set_tuning(16)
        t2, cached2 = wah.autotune((1 << 21) + 12345, 65535, cache)
        assert cached2 and t2 == t and lib.wah_get_tuning() == t
        rng = np.random.default_rng(5)
        v = rng.integers(0, 65536, size=(1 << 21) + 77, dtype=np.uint32)
        got = wah.build_index(v, bound=65535).numpy()
        ref = O.build(v)
        assert np.array_equal(got.keys, ref.keys)
        assert np.array_equal(got.offsets, ref.offsets)
        assert np.array_equal(got.index, ref.index)
        with pytest.raises(wah.WahError):
            wah.autotune(0, 10)
    finally:
        lib.wah_set_tuning(before)


# ---------------------------------------------------------------------------
# Per-call tuning words.
# ---------------------------------------------------------------------------
from test_gpu_parity import assert_same, gen  # noqa: E402


@pytest.mark.parametrize("shape", [16 | 0x200, 12 | 0x200, 8, 16 | 0x100])
@pytest.mark.parametrize("kind", ["uniform16", "few16", "zipf", "runs", "two"])
@pytest.mark.parametrize("n", [4097, 100_003, 1 << 20, (1 << 22) + 5])
def test_packed_exchange_forced(wah, shape, kind, n):
    """WAH_TUNE_PACK: the packed words between the two digit passes even
    where pass-0 runs are short (many run starts per tile and per warp slice:
    the search fallbacks), with a 16-bit bound; per-call word."""
    rng = np.random.default_rng(hash((shape, kind, n)) & 0xFFFFFFFF)
    v = gen(kind, n, rng)
    t = shape | wah.TUNE_PACK | wah.tune_later(12 | 0x200)
    assert_same(wah.build_index(v, bound=65535, tuning=t), O.build(v), f"{kind}/{n}/{t:#x}")


def test_invalid_word_is_refused_per_call(wah):
    lib = wah._lib.load()
    before = lib.wah_get_tuning()
    v = np.arange(1000, dtype=np.uint32)
    for bad in (7, 16 | later_pack(), 16 | 0x800, -3):
        with pytest.raises(wah.WahError) as e:
            wah.build_index(v, tuning=bad)
        assert e.value.status == wah.WAH_EINVAL
    assert lib.wah_get_tuning() == before  # nothing process-wide changed


def later_pack():
    return (12 | 0x400) << 16  # WAH_TUNE_PACK is refused in a later-pass shape


def test_concurrent_callers_with_different_words(wah):
    """Two host threads build at the same time on their own streams, each
    with its own tuning word; every result equals the oracle."""
    import threading
    rng = np.random.default_rng(12)
    cols = [gen("uniform16", 2_000_003, rng), gen("zipf", 1_500_001, rng),
            gen("runs", 1_000_000, rng), gen("few16", 777_777, rng)]
    refs = [O.build(v) for v in cols]
    words = [16 | 0x200 | wah.tune_later(12 | 0x200) | wah.TUNE_PACK, 8 | wah.tune_later(16)]
    errors = []

    def worker(w):
        try:
            s = torch.cuda.Stream()
            for rep in range(3):
                for v, ref in zip(cols, refs):
                    with torch.cuda.stream(s):
                        got = wah.build_index(v, bound=65535, stream=s, tuning=w)
                    assert_same(got, ref, f"word {w:#x} rep {rep}")
        except Exception as ex:  # reported in the main thread
            errors.append(ex)
    ths = [threading.Thread(target=worker, args=(w,)) for w in words]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    assert not errors, errors[0]


@pytest.mark.parametrize("workload", ["skewed", "batch"])
def test_autotune_workload(wah, workload, tmp_path):
    """The per-workload tuner returns a valid word without applying it,
    caches it per workload, and builds with that word equal the oracle."""
    lib = wah._lib.load()
    before = lib.wah_get_tuning()
    cache = str(tmp_path / "tune.txt")
    if workload == "skewed":
        t, cached = wah.autotune_workload(wah.WORKLOAD_SKEWED, 1 << 21, 65535, 0, cache)
    else:
        t, cached = wah.autotune_workload(wah.WORKLOAD_BATCH, 1 << 24, 65535, 64, cache)
    assert not cached and t & 0xff in (8, 12, 16)
    assert lib.wah_get_tuning() == before
    line = open(cache).read().splitlines()[-1]
    assert ("skewed" if workload == "skewed" else "batch64") in line
    assert int(line.split()[-2]) == t
    if workload == "skewed":
        t2, c2 = wah.autotune_workload(wah.WORKLOAD_SKEWED, (1 << 21) + 99, 65535, 0, cache)
        assert c2 and t2 == t
        v = gen("zipf", 1_234_567, np.random.default_rng(3))
        assert_same(wah.build_index(v, bound=65535, tuning=t), O.build(v), "tuned zipf")
    else:
        t2, c2 = wah.autotune_workload(wah.WORKLOAD_BATCH, 1 << 24, 65535, 64, cache)
        assert c2 and t2 == t
        rng = np.random.default_rng(4)
        cols = [gen("uniform16", int(n), rng) for n in (5000, 70_001, 300_000, 31)]
        b = wah.Batch([c.size for c in cols], [65535] * 4, tuning=t)
        b.set_columns([torch.from_numpy(c.view(np.int32)).cuda() for c in cols])
        b.build()
        for got, v in zip(b.results(), cols):
            assert_same(got, O.build(v), "tuned batch")
        b.close()
