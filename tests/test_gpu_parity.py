"""Parity of the CUDA path (through the C ABI) with the oracle and with the
golden vectors made by the reference's own code.  Integer work: bit-exact."""
import ctypes

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


def assert_same(gpu_idx, ref, name=""):
    g = gpu_idx.numpy()
    assert np.array_equal(g.keys, ref.keys), f"{name}: keys differ"
    assert np.array_equal(g.offsets, ref.offsets), f"{name}: offsets differ"
    assert g.index.size == ref.index.size, f"{name}: L {g.index.size} != {ref.index.size}"
    assert np.array_equal(g.index, ref.index), f"{name}: index words differ"
    assert g.merged == ref.merged, f"{name}: k {g.merged} != {ref.merged}"


def test_golden_vectors(wah, golden):
    for name, case in golden.items():
        ref = O.Index(case["keys"], case["offsets"], case["index"], int(case["merged"][0]))
        assert_same(wah.build_index(case["values"]), ref, name)
        # with the exact bound as the -b flag
        bound = int(case["values"].max())
        assert_same(wah.build_index(case["values"], bound=bound), ref, name + "/bound")


def gen(kind, n, rng):
    if kind == "uniform16":
        return rng.integers(0, 65536, size=n, dtype=np.uint32)
    if kind == "few16":
        return rng.integers(0, 16, size=n, dtype=np.uint32)
    if kind == "u32":
        return rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)
    if kind == "zipf":
        w = 1.0 / np.arange(1, 65537, dtype=np.float64) ** 1.1
        cdf = np.cumsum(w) / w.sum()
        return np.minimum(np.searchsorted(cdf, rng.random(n)), 65535).astype(np.uint32)
    if kind == "runs":
        runs = rng.geometric(1 / 1000, size=n // 500 + 2)
        vals = rng.integers(0, 65536, size=runs.size, dtype=np.uint32)
        return np.repeat(vals, runs)[:n]
    if kind == "const":
        return np.full(n, 77, np.uint32)
    if kind == "two":
        return rng.integers(0, 2, size=n, dtype=np.uint32)
    raise ValueError(kind)


@pytest.mark.parametrize("kind", ["uniform16", "few16", "u32", "zipf", "runs", "const", "two"])
@pytest.mark.parametrize("n", [1, 30, 31, 33, 1000, 2048, 4096, 4097, 100_003, 1 << 20])
def test_random_columns(wah, kind, n):
    rng = np.random.default_rng(hash((kind, n)) & 0xFFFFFFFF)
    v = gen(kind, n, rng)
    assert_same(wah.build_index(v), O.build(v), f"{kind}/{n}")


@pytest.mark.parametrize("kind", ["uniform16", "few16", "zipf", "runs", "const", "two"])
@pytest.mark.parametrize("n", [1, 30, 31, 33, 1000, 2048, 4096, 4097, 100_003, 1 << 20])
def test_random_columns_bound16(wah, kind, n):
    # a 16-bit bound: two digit passes; where both digits vary the build
    # takes key starts from the full-key counts instead of reading keys
    rng = np.random.default_rng(hash((kind, n, 16)) & 0xFFFFFFFF)
    v = gen(kind, n, rng)
    assert_same(wah.build_index(v, bound=65535), O.build(v), f"{kind}/{n}/b16")


def test_config1_uniform_1m_with_bound(wah):
    # 1,048,576 uniform [0, 65535], seeded; bound given as the reference's -b
    rng = np.random.default_rng(1)
    v = rng.integers(0, 65536, size=1 << 20, dtype=np.uint32)
    ref = O.build(v)
    assert_same(wah.build_index(v, bound=65535), ref, "c1")
    assert_same(wah.build_index(v, bound=0), ref, "c1/scan")


@pytest.mark.parametrize("kind", ["uniform16", "runs", "two"])
def test_many_tiles_per_range(wah, kind):
    # 16M rows: every range owns many tiles, so both halves of each double
    # buffer are reused many times; the first range's first window is read
    # without a bulk copy
    rng = np.random.default_rng(16)
    v = gen(kind, 1 << 24, rng)
    assert_same(wah.build_index(v, bound=65535), O.build(v), f"16M/{kind}")


def test_sort_phase_matches_stable_sort(wah):
    rng = np.random.default_rng(3)
    for n, m in ((1, 5), (5000, 7), (300_000, 65536), (70_001, 2 ** 32)):
        v = rng.integers(0, m, size=n, dtype=np.uint64).astype(np.uint32)
        sv, sr = wah.sort_rids_by_value(v)
        ev, er = O.sort_rids_by_value(v)
        assert np.array_equal(sv.cpu().numpy().view(np.uint32), ev)
        assert np.array_equal(sr.cpu().numpy().view(np.uint32), er)


def test_sort_phase_with_bound(wah):
    # two digit passes with 16-bit keys between them: the sort alone still
    # returns every sorted key (key starts are an index-build mode only)
    rng = np.random.default_rng(31)
    for n, m in ((4097, 65536), (300_000, 65536), (1 << 20, 40_000), (77_777, 300)):
        v = rng.integers(0, m, size=n, dtype=np.uint32)
        sv, sr = wah.sort_rids_by_value(v, bound=65535)
        ev, er = O.sort_rids_by_value(v)
        assert np.array_equal(sv.cpu().numpy().view(np.uint32), ev), (n, m)
        assert np.array_equal(sr.cpu().numpy().view(np.uint32), er), (n, m)


def test_build_sorted_phase(wah):
    rng = np.random.default_rng(4)
    v = rng.integers(0, 1000, size=123_457, dtype=np.uint32)
    ev, er = O.sort_rids_by_value(v)
    assert_same(wah.build_sorted(ev, er), O.build(v), "build_sorted")


def test_host_context_roundtrip(wah):
    rng = np.random.default_rng(6)
    with wah.HostContext(1 << 18) as ctx:
        for n in (0, 1, 999, 1 << 18):
            v = rng.integers(0, 5000, size=n, dtype=np.uint32)
            got = ctx.build(v)
            ref = O.build(v)
            assert np.array_equal(got.keys, ref.keys)
            assert np.array_equal(got.offsets, ref.offsets)
            assert np.array_equal(got.index, ref.index)


def test_empty_column(wah):
    r = wah.build_index(np.zeros(0, np.uint32))
    assert r.keycnt == 0 and r.index_len == 0


def test_value_above_bound_is_reported(wah):
    v = np.array([1, 2, 70000, 3], np.uint32)  # needs 3 digits, bound says 1
    with pytest.raises(wah.WahError) as e:
        wah.build_index(v, bound=255)
    assert e.value.status == wah.WAH_ERANGE


def test_decoded_bitmaps_match_rows(wah):
    rng = np.random.default_rng(8)
    v = gen("runs", 50_000, rng)
    idx = wah.build_index(v).numpy()
    for i in range(0, idx.keycnt, max(1, idx.keycnt // 20)):
        rows = np.flatnonzero(v == idx.keys[i])
        s = wah.decoded_bitmap(idx.bitmap(i))
        assert [j for j, ch in enumerate(s) if ch == "1"] == rows.tolist()


def later(shape):
    """WAH_TUNE_LATER: the tile shape of the digit passes after the first."""
    return shape << 16


@pytest.mark.parametrize("items", [8, 12, 16, 8 | 0x100, 12 | 0x100, 16 | 0x100,
                                   8 | 0x200, 16 | 0x200,
                                   16 | 0x200 | later(12 | 0x200), 16 | later(8),
                                   8 | 0x100 | later(16 | 0x200), 12 | later(16 | 0x100)])
def test_every_sort_tile_shape(wah, items):
    lib = wah._lib.load()
    old = lib.wah_get_tuning()
    assert lib.wah_set_tuning(items) == 0
    try:
        rng = np.random.default_rng(items)
        for kind, n in (("uniform16", 300_001), ("u32", 77_777), ("runs", 200_000),
                        ("few16", 5_003)):
            v = gen(kind, n, rng)
            assert_same(wah.build_index(v), O.build(v), f"{kind}/{n}/items{items}")
            if kind != "u32":  # two digit passes (key starts where both vary)
                assert_same(wah.build_index(v, bound=65535), O.build(v),
                            f"{kind}/{n}/items{items}/b16")
    finally:
        lib.wah_set_tuning(old)


def test_rejects_unknown_tuning(wah):
    lib = wah._lib.load()
    old = lib.wah_get_tuning()
    for bad in (7, 20, 16 | 0x300, 16 | later(7), 16 | later(12 | 0x300), 16 | later(0x200),
                16 | later(12 | 0x400), 16 | 0x800, 0, -1):
        assert lib.wah_set_tuning(bad) == wah.WAH_EINVAL, bad
    assert lib.wah_get_tuning() == old


def test_pipeline_matches_oracle(wah):
    # several columns in flight; every result equals the oracle's
    rng = np.random.default_rng(21)
    cols = [gen(k, n, rng) for k, n in (("uniform16", 300_000), ("runs", 1 << 20),
                                        ("few16", 77_777), ("zipf", 500_000),
                                        ("two", 4097), ("const", 1))]
    pinned = []
    for v in cols:
        t = torch.empty(v.size, dtype=torch.int32, pin_memory=True)
        t.numpy()[:] = v.view(np.int32)
        pinned.append(t)
    with wah.Pipeline(1 << 20, bound=65535, depth=3) as pipe:
        tickets = []
        for i, t in enumerate(pinned):
            tickets.append(pipe.submit(t))
            if i >= 2:  # take results while later columns are in flight
                j = i - 2
                r = pipe.result(tickets[j])
                ref = O.build(cols[j])
                assert np.array_equal(r.keys, ref.keys) and np.array_equal(r.index, ref.index)
                assert np.array_equal(r.offsets, ref.offsets)
        for j in range(len(pinned) - 2, len(pinned)):
            r = pipe.result(tickets[j])
            ref = O.build(cols[j])
            assert np.array_equal(r.keys, ref.keys) and np.array_equal(r.index, ref.index)


def test_pipeline_pageable_buffers_and_errors(wah):
    lib = wah._lib.load()
    h = ctypes.c_void_p()
    assert lib.wah_pipe_create(1024, 0, 2, ctypes.byref(h)) == 0
    try:
        v = np.arange(100, 0, -1, dtype=np.uint32)
        keys = np.empty(1024, np.uint32)
        offs = np.empty(1024, np.uint32)
        index = np.empty(2048, np.uint32)
        cnt = np.zeros(4, dtype=np.uint32)
        t = ctypes.c_uint64()
        assert lib.wah_pipe_submit(h, v.ctypes.data, 100, keys.ctypes.data, offs.ctypes.data,
                                   index.ctypes.data, cnt.ctypes.data, ctypes.byref(t)) == 0
        assert lib.wah_pipe_wait(h, t.value) == 0
        ref = O.build(v)
        assert cnt[3] == 0 and cnt[0] == len(ref.keys) and cnt[1] == len(ref.index)
        assert np.array_equal(index[:cnt[1]], ref.index)
        # too long for the pipe
        assert lib.wah_pipe_submit(h, v.ctypes.data, 2000, keys.ctypes.data, offs.ctypes.data,
                                   index.ctypes.data, cnt.ctypes.data,
                                   ctypes.byref(t)) == wah.WAH_ERANGE
    finally:
        lib.wah_pipe_destroy(h)
