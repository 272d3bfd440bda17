"""Decoding and querying a built index on the GPU.

Decode parity: the row ids per key are the stable sort's rid order (the
oracle's sort_rids_by_value), the per-row values the sorted column, the
reconstructed column the input itself, and each key's rows are the '1's of
the oracle's decoded_bitmap (src/cpu.cpp:47-74).  At the full 268,435,456-row
size the oracle is too slow, so the round trip build -> decode -> column is
checked as a property: the column comes back bit for bit and each key's row
count equals the column's histogram.  Queries are checked against numpy on
the same column and, as WAH bitmaps, against the oracle's index of the
result's indicator column.  Integer work: bit-exact."""
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
    rng = np.random.default_rng(77)
    yield "kat2", np.array([(1 if i % 97 == 0 else (2 if (i // 40) % 2 else 3))
                            for i in range(300)], np.uint32)
    yield "one", np.array([5], np.uint32)
    yield "n31", np.full(31, 9, np.uint32)
    yield "uniform16", rng.integers(0, 65536, size=200_003, dtype=np.uint32)
    yield "few", rng.integers(0, 7, size=150_001, dtype=np.uint32)
    yield "u32", rng.integers(0, 2 ** 32, size=90_000, dtype=np.uint64).astype(np.uint32)
    runs = rng.geometric(1 / 700, size=600)
    yield "runs", np.repeat(rng.integers(0, 500, size=600, dtype=np.uint32), runs)[:250_000]
    sparse = np.zeros(300_000, np.uint32)
    sparse[rng.choice(300_000, 50, replace=False)] = rng.integers(1, 5, size=50, dtype=np.uint32)
    yield "sparse", sparse


@pytest.mark.parametrize("name,v", list(columns()))
def test_decode_matches_oracle(wah, name, v):
    n = v.size
    idx = wah.build_index(v)
    d = wah.decode(idx, n, rows=True, values=True, column=True, key_rows=True)
    sv, sr = O.sort_rids_by_value(v)
    assert np.array_equal(u32(d["rows"]), sr), f"{name}: row ids"
    assert np.array_equal(u32(d["values"]), sv), f"{name}: row values"
    assert np.array_equal(u32(d["column"]), v), f"{name}: column"
    keys = u32(idx.keys)
    counts = np.array([np.count_nonzero(v == k) for k in keys[:50]])
    starts = u32(d["key_rows"])
    assert starts[0] == 0
    m = min(len(keys) - 1, 49)
    assert np.array_equal(np.diff(starts)[:m], counts[:m]), f"{name}: key row starts"
    # the '1's of the reference decoder, key by key (a sample of keys)
    h = idx.numpy()
    for i in range(0, h.keycnt, max(1, h.keycnt // 25)):
        bits = O.decoded_bitmap(h.bitmap(i))
        ones = [j for j, ch in enumerate(bits) if ch == "1"]
        end = starts[i + 1] if i + 1 < h.keycnt else n
        assert u32(d["rows"])[starts[i]:end].tolist() == ones, f"{name}: key {i}"


@pytest.mark.parametrize("name,v", list(columns()))
def test_decode_rows_only_matches_oracle(wah, name, v):
    """Row ids alone (and with each key's first position) take the decoder's
    lean path: the same row ids as the oracle's stable sort."""
    n = v.size
    idx = wah.build_index(v)
    sv, sr = O.sort_rids_by_value(v)
    d = wah.decode(idx, n)
    assert np.array_equal(u32(d["rows"]), sr), f"{name}: row ids"
    d2 = wah.decode(idx, n, rows=True, key_rows=True)
    assert np.array_equal(u32(d2["rows"]), sr), f"{name}: row ids (with key starts)"
    starts = u32(d2["key_rows"])
    keys = u32(idx.keys)
    assert np.array_equal(starts, np.searchsorted(sv, keys)), f"{name}: key row starts"


def test_decode_empty_and_launches(wah):
    idx = wah.build_index(np.zeros(0, np.uint32))
    d = wah.decode(idx, 0, rows=True, column=True)
    assert d["rows"].numel() == 0 and d["column"].numel() == 0
    v = np.arange(1000, dtype=np.uint32) % 13
    wah.decode(wah.build_index(v), v.size)
    assert wah.last_launch_count() >= 4


def test_decode_reports_wrong_row_count(wah):
    """Words that hold more or fewer rows than stated are WAH_ECORRUPT;
    rows past n are never written."""
    v = np.random.default_rng(2).integers(0, 100, size=10_000, dtype=np.uint32)
    idx = wah.build_index(v)
    for n in (9_000, 12_000):
        with pytest.raises(wah.WahError) as e:
            wah.decode(idx, n, rows=True, column=True)
        assert e.value.status == wah.WAH_ECORRUPT
        with pytest.raises(wah.WahError) as e:  # the row-ids-only path
            wah.decode(idx, n)
        assert e.value.status == wah.WAH_ECORRUPT


@pytest.mark.parametrize("kind", ["uniform16", "zipf", "runs"])
def test_full_size_round_trip(wah, kind):
    """268,435,456 rows: build, then decode back to the column on the GPU;
    the column must return bit for bit and every key's row count must equal
    the column's histogram (size-independent properties in place of the
    oracle, which needs minutes at this size)."""
    n = 268_435_456
    g = torch.Generator(device="cuda")
    g.manual_seed({"uniform16": 1, "zipf": 2, "runs": 3}[kind])
    if kind == "uniform16":
        col = torch.randint(0, 65536, (n,), device="cuda", dtype=torch.int32, generator=g)
    elif kind == "zipf":
        # ranks by inverse CDF of s = 1.1 over 65,536 values
        w = 1.0 / torch.arange(1, 65537, device="cuda", dtype=torch.float64) ** 1.1
        cdf = torch.cumsum(w, 0) / w.sum()
        u = torch.rand(n, device="cuda", dtype=torch.float64, generator=g)
        col = torch.clamp(torch.searchsorted(cdf, u), max=65535).to(torch.int32)
        del u
    else:
        # runs of mean length ~1000: a new run where a uniform draw < 1/1000
        u = torch.rand(n, device="cuda", generator=g)
        new_run = (u < 1e-3).to(torch.int32)
        del u
        run_id = torch.cumsum(new_run, 0, dtype=torch.int32)
        del new_run
        vals = torch.randint(0, 65536, (int(run_id[-1].item()) + 1,), device="cuda",
                             dtype=torch.int32, generator=g)
        col = vals[run_id.long()]
        del run_id, vals
    idx = wah.build_index(col, bound=65535)
    d = wah.decode(idx, n, rows=False, column=True, key_rows=True)
    assert torch.equal(d["column"], col), f"{kind}: column differs after decode"
    hist = torch.bincount(col.long(), minlength=65536)
    keys = idx.keys.long()
    starts = d["key_rows"].long()
    ends = torch.cat([starts[1:], torch.tensor([n], device="cuda")])
    assert torch.equal(ends - starts, hist[keys]), f"{kind}: rows per key"
    assert int(hist[keys].sum().item()) == n
    # keys ascending, offsets ascending, index length consistent
    assert bool((keys[1:] > keys[:-1]).all())
    offs = idx.offsets.long()
    assert bool((offs[1:] > offs[:-1]).all()) and int(offs[0].item()) == 0


def indicator_bitmap(mask):
    """The oracle's WAH words for the rows where mask is True: the bitmap of
    key 1 in the index of the indicator column."""
    ind = mask.astype(np.uint32)
    if not ind.any():
        return np.zeros(0, np.uint32)
    ref = O.build(ind)
    i = int(np.searchsorted(ref.keys, 1))
    end = ref.offsets[i + 1] if i + 1 < ref.keys.size else ref.index.size
    return ref.index[ref.offsets[i]:end]


@pytest.mark.parametrize("name,v", [c for c in columns() if c[0] in
                                    ("kat2", "uniform16", "few", "runs", "sparse", "u32")])
def test_queries_match_numpy_and_oracle(wah, name, v):
    n = v.size
    idx = wah.build_index(v)
    h = idx.numpy()
    rng = np.random.default_rng(n)
    picks = [int(h.keys[0]), int(h.keys[-1]), int(h.keys[h.keycnt // 2])]
    # one key: its own words
    for key in picks:
        words, rows = wah.query(idx, n, key)
        i = int(np.searchsorted(h.keys, key))
        assert np.array_equal(u32(words), h.bitmap(i)), f"{name}: words of key {key}"
        assert np.array_equal(u32(rows), np.flatnonzero(v == key)), f"{name}: rows of {key}"
    # a value absent from the column
    lo_gap = int(h.keys[-1]) + 1 if h.keys[-1] < 2 ** 32 - 1 else None
    if lo_gap is not None:
        words, rows = wah.query(idx, n, lo_gap)
        assert words.numel() == 0 and rows.numel() == 0
    vmax = int(v.max())
    cases = []
    for _ in range(4):
        a = sorted(int(x) for x in rng.integers(0, vmax + 1, size=2, dtype=np.uint64))
        b = sorted(int(x) for x in rng.integers(0, vmax + 1, size=2, dtype=np.uint64))
        cases.append((tuple(a), tuple(b)))
    ma = lambda t: (v >= t[0]) & (v <= t[1])  # noqa: E731
    for a, b in cases:
        for op, fn in ((wah.QUERY_KEYS, lambda x, y: x), (wah.QUERY_OR, np.logical_or),
                       (wah.QUERY_AND, np.logical_and),
                       (wah.QUERY_ANDNOT, lambda x, y: x & ~y)):
            mask = fn(ma(a), ma(b))
            words, rows = wah.query(idx, n, a, op, b)
            assert np.array_equal(u32(rows), np.flatnonzero(mask)), f"{name}: op {op} {a} {b}"
            assert np.array_equal(u32(words), indicator_bitmap(mask)), f"{name}: op {op} words"


def test_query_output_capacity_is_reported(wah):
    lib = wah._lib.load()
    v = np.random.default_rng(9).integers(0, 4, size=5000, dtype=np.uint32)
    idx = wah.build_index(v)
    n = v.size
    keys, offsets, index = idx.keys, idx.offsets, idx.index
    rows = torch.empty(10, dtype=torch.int32, device="cuda")
    res = torch.zeros(4, dtype=torch.int32, device="cuda")
    wsb = int(lib.wah_query_workspace_bytes(n))
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    rc = lib.wah_query(keys.data_ptr(), offsets.data_ptr(), index.data_ptr(), len(keys),
                       len(index), n, 0, 3, wah.QUERY_KEYS, 0, 0, None, 0, rows.data_ptr(), 10,
                       res.data_ptr(), ws.data_ptr(), wsb, None)
    assert rc == 0
    torch.cuda.synchronize()
    r = u32(res)
    assert r[1] == n and r[2] == wah.WAH_EOVERFLOW
    assert np.array_equal(u32(rows), np.arange(10, dtype=np.uint32))
    # bad op and too small a workspace are refused before any launch
    assert lib.wah_query(keys.data_ptr(), offsets.data_ptr(), index.data_ptr(), len(keys),
                         len(index), n, 0, 3, 9, 0, 0, None, 0, None, 0, res.data_ptr(),
                         ws.data_ptr(), wsb, None) == wah.WAH_EINVAL
    assert lib.wah_query(keys.data_ptr(), offsets.data_ptr(), index.data_ptr(), len(keys),
                         len(index), n, 0, 3, 0, 0, 0, None, 0, None, 0, res.data_ptr(),
                         ws.data_ptr(), 16, None) == wah.WAH_ENOMEM


def test_largest_column(wah):
    """The largest column one call accepts, 2^31 - 1 rows (every row, word
    and key position stays within u32: L <= 2n < 2^32): built and decoded back
    to the column bit for bit on the GPU; 2^31 rows are refused with
    WAH_ERANGE before any work."""
    n = (1 << 31) - 1
    g = torch.Generator(device="cuda")
    g.manual_seed(30)
    col = torch.randint(0, 65536, (n,), device="cuda", dtype=torch.int32, generator=g)
    idx = wah.build_index(col, bound=65535)
    assert len(idx.keys) == 65536
    assert n < len(idx.index) < 2 * n
    d = wah.decode(idx, n, rows=False, column=True, key_rows=True)
    assert torch.equal(d["column"], col)
    starts = d["key_rows"].long()
    assert int(starts[0].item()) == 0 and bool((starts[1:] > starts[:-1]).all())
    del d, idx, starts
    torch.cuda.empty_cache()
    # 2^31 rows through the C ABI: refused before anything is read or written
    lib = wah._lib.load()
    counts = torch.zeros(4, dtype=torch.int32, device="cuda")
    dummy = torch.zeros(4, dtype=torch.int32, device="cuda")
    p = dummy.data_ptr()
    rc = lib.wah_build(p, 1 << 31, 65535, p, p, p, counts.data_ptr(), p, 16, None)
    assert rc == wah.WAH_ERANGE
