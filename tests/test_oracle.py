"""The oracle (CPU restatement of src/cpu.cpp) against the golden vectors
generated from the reference's own code, and against that code directly when
it is built here."""
import numpy as np
import pytest

from oracle import oracle as O


def test_golden_vectors(golden):
    assert len(golden) >= 20
    for name, case in golden.items():
        r = O.build(case["values"])
        assert np.array_equal(r.keys, case["keys"]), name
        assert np.array_equal(r.offsets, case["offsets"]), name
        assert np.array_equal(r.index, case["index"]), name
        assert r.merged == int(case["merged"][0]), name


def test_kat1_known_answer(golden):
    # KAT-1 (src/cpu.cpp:292-295): 16 words, 15 keys, no fills
    c = golden["kat1_builtin32"]
    assert c["keys"].tolist() == [0, 1, 2, 3, 5, 6, 7, 9, 10, 13, 18, 19, 22, 23, 42]
    assert c["offsets"].tolist() == [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 14, 15]
    assert [f"{w:08x}" for w in c["index"]] == [
        "80404000", "8000a020", "81001100", "80840800", "84100200", "c0000008",
        "80000012", "80200040", "a0000001", "80080400", "80030000", "82000000",
        "90000004", "80000001", "88000000", "80000080"]


def test_kat2_known_answer(golden):
    c = golden["kat2_fills300"]
    assert c["keys"].tolist() == [1, 2, 3]
    assert c["offsets"].tolist() == [0, 7, 17]
    assert len(c["index"]) == 27 and int(c["merged"][0]) == 21
    assert c["index"][:4].tolist() == [0x80000001, 2, 0x80000010, 2]


def test_bubble_equals_stable():
    rng = np.random.default_rng(5)
    for n in (1, 2, 31, 100, 1000, 3000):
        for m in (2, 50, 65536):
            v = rng.integers(0, m, size=n, dtype=np.uint32)
            assert O.build(v, O.SORT_BUBBLE) == O.build(v, O.SORT_STABLE)


def test_empty_column():
    r = O.build(np.zeros(0, np.uint32))
    assert r.keys.size == 0 and r.index.size == 0 and r.merged == 0


def test_decoded_bitmap_matches_rows():
    rng = np.random.default_rng(9)
    v = rng.integers(0, 20, size=2000, dtype=np.uint32)
    r = O.build(v)
    for i, key in enumerate(r.keys):
        s = O.decoded_bitmap(r.bitmap(i))
        rows = np.flatnonzero(v == key)
        expect = np.zeros(rows[-1] + 1, np.uint8)
        expect[rows] = 1
        assert s == "".join(map(str, expect))


@pytest.mark.skipif(not O.ref_available(), reason="reference shim not built here")
def test_against_reference_code_random():
    rng = np.random.default_rng(11)
    for t in range(200):
        n = int(rng.integers(1, 4000))
        m = int(rng.choice([1, 2, 3, 16, 100, 65536, 1 << 31]))
        v = rng.integers(0, m, size=n, dtype=np.uint64).astype(np.uint32)
        a = O.ref_build(v, bubble=n < 1500)
        b = O.build(v)
        assert a == b and a.merged == b.merged, (t, n, m)
        for i in range(min(3, len(a.keys))):
            assert O.decoded_bitmap(a.bitmap(i)) == O.ref_decoded_bitmap(a.bitmap(i))


@pytest.mark.skipif(not O.ref_available(), reason="reference shim not built here")
def test_against_reference_code_1m():
    rng = np.random.default_rng(12)
    v = rng.integers(0, 65536, size=1 << 20, dtype=np.uint32)
    assert O.ref_build(v) == O.build(v)
