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
