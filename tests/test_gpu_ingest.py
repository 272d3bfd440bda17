"""Text ingest on the GPU (wah_parse_text) against a plain-Python reading of
the same bytes with the reference's rule: whitespace-separated tokens,
`while (source >> next)` stops at the first token that is not an unsigned
32-bit number (src/cpu.cpp:297-302).  Integer work: bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

WS = b" \t\n\v\f\r"


def _tokens(data: bytes):
    for c in b"\t\n\v\f\r":
        data = data.replace(bytes([c]), b" ")
    return [t for t in data.split(b" ") if t]


def reference_read(data: bytes):
    """Values before the first token that is not a 32-bit decimal number,
    and the number of tokens."""
    toks = _tokens(data)
    out = []
    for tok in toks:
        digits = tok.lstrip(b"0") or b"0"
        if not tok.isdigit() or len(digits) > 10 or int(digits) > 0xFFFFFFFF:
            break
        out.append(int(digits))
    return np.array(out, dtype=np.uint64).astype(np.uint32), len(toks)


@pytest.fixture(scope="module")
def wah():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import indexing_gb300 as w
    w._lib.load()
    return w


def check(wah, data: bytes, name=""):
    ref, tokens = reference_read(data)
    got, info = wah.parse_text(data)
    assert info["values"] == ref.size, name
    assert info["tokens"] == tokens, name
    assert np.array_equal(got.cpu().numpy().view(np.uint32), ref), name
    assert info["max_value"] == (int(ref.max()) if ref.size else 0), name


def test_generate_format(wah):
    rng = np.random.default_rng(1)
    for n in (0, 1, 2, 31, 4095, 4096, 4097, 100_000, 1_000_003):
        v = rng.integers(0, 65536, size=n, dtype=np.uint32)
        data = ("\n".join(map(str, v.tolist())) + ("\n" if n else "")).encode()
        check(wah, data, f"n={n}")


def test_separators_and_edges(wah):
    cases = [
        b"", b"\n\n\n", b"   ", b"7", b"7\n", b"  7  ", b"0", b"00000000000000000000042\n",
        b"4294967295", b"4294967296 1 2", b"1 2 4294967296 3", b"12abc 5", b"5 12abc 6",
        b"1\r\n2\r\n3\r\n", b"1\t2\v3\f4\r5 6\n7", b"-1 2", b"+3 4", b"9" * 40 + b" 1",
        b"1 " * 5000 + b"x" + b" 2" * 10, b"0" * 5000 + b"17 18",
        b"99999999 100000000 4294967295 0000000004294967295 00000004294967296",
    ]
    for c in cases:
        check(wah, c, repr(c[:40]))


def test_random_layouts_across_ranges(wah):
    """Tokens and long whitespace runs crossing 16-byte, 4096-byte and range
    boundaries, long leading-zero tokens, values up to 2^32-1."""
    rng = np.random.default_rng(7)
    for trial in range(6):
        parts = []
        for _ in range(20_000):
            kind = rng.integers(0, 10)
            if kind < 6:
                parts.append(str(int(rng.integers(0, 2 ** 32, dtype=np.uint64))).encode())
            elif kind < 8:
                parts.append(b"0" * int(rng.integers(1, 70)) +
                             str(int(rng.integers(0, 1000))).encode())
            else:
                parts.append(str(int(rng.integers(0, 10))).encode())
            ws = rng.choice(list(WS), size=int(rng.integers(1, 40))).astype(np.uint8)
            parts.append(bytes(ws))
        data = b"".join(parts)
        if trial % 2:
            pos = int(rng.integers(0, len(data)))
            data = data[:pos] + b"#" + data[pos:]
        check(wah, data, f"trial {trial}")


def test_capacity_overflow_is_reported(wah):
    data = b"1 2 3 4 5 6 7 8\n"
    with pytest.raises(wah.WahError) as e:
        wah.parse_text(data, capacity=3)
    assert e.value.status == wah.WAH_EOVERFLOW


def test_parse_then_build_matches_oracle(wah):
    from oracle import oracle as O
    rng = np.random.default_rng(3)
    v = rng.integers(0, 65536, size=300_000, dtype=np.uint32)
    data = ("\n".join(map(str, v.tolist())) + "\n").encode()
    col, info = wah.parse_text(data)
    idx = wah.build_index(col, bound=info["max_value"]).numpy()
    ref = O.build(v)
    assert np.array_equal(idx.keys, ref.keys)
    assert np.array_equal(idx.index, ref.index)
