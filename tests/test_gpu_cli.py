"""The `phases` and `gpu` programs (actor drivers over the C ABI) on a GPU:
their result files against the oracle, their -p listings against the
oracle's `cpu` program, and their error handling.  Integer work: bit-exact."""
import os
import subprocess

import numpy as np
import pytest

from indexing_gb300 import _lib
from oracle import oracle as O

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(REPO, "oracle")


@pytest.fixture(scope="module")
def progs():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.build()
    p = _lib.build_host(["phases", "gpu", "generate"])
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "bin/cpu"], check=True)
    p["cpu"] = os.path.join(ORACLE_DIR, "bin", "cpu")
    return p


def run(cmd):
    return subprocess.run(cmd, capture_output=True, text=True, timeout=600)


def write_values(path, v):
    with open(path, "w") as f:
        f.write("\n".join(map(str, v.tolist())))
        f.write("\n")


def read_result(path):
    got = np.fromfile(path, dtype=np.uint32)
    K, L = int(got[0]), int(got[1])
    return got[2:2 + K], got[2 + K:2 + 2 * K], got[2 + 2 * K:2 + 2 * K + L]


def assert_matches_oracle(path, v, what):
    keys, offsets, index = read_result(path)
    ref = O.build(v)
    assert np.array_equal(keys, ref.keys), f"{what}: keys differ"
    assert np.array_equal(offsets, ref.offsets), f"{what}: offsets differ"
    assert index.size == ref.index.size, f"{what}: L {index.size} != {ref.index.size}"
    assert np.array_equal(index, ref.index), f"{what}: index words differ"


def listing(stdout):
    """Lines of a -p listing ("key<TAB>bits")."""
    return [ln for ln in stdout.splitlines() if "\t" in ln]


@pytest.mark.parametrize("kind,n", [("uniform16", 100_000), ("few", 250_000),
                                    ("runs", 300_000), ("u32", 50_000)])
def test_phases_result_matches_oracle(progs, tmp_path, kind, n):
    rng = np.random.default_rng(n)
    if kind == "uniform16":
        v = rng.integers(0, 65536, size=n, dtype=np.uint32)
    elif kind == "few":
        v = rng.integers(0, 5, size=n, dtype=np.uint32)
    elif kind == "runs":
        v = np.repeat(rng.integers(0, 65536, size=n // 300 + 1, dtype=np.uint32), 300)[:n]
    else:
        v = rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)
    data, out = tmp_path / "v.txt", tmp_path / "r.bin"
    write_values(data, v)
    r = run([progs["phases"], "-f", str(data), "-o", str(out), "--describe"])
    assert r.returncode == 0, r.stderr
    for label in ("Transfer to:", "Sort:", "Index:", "Transfer back:", "Total:"):
        assert any(ln.startswith(label) and ln.endswith(" us") for ln in r.stdout.splitlines())
    assert_matches_oracle(out, v, f"phases {kind}")


def test_phases_listing_equals_cpu_program(progs, tmp_path):
    rng = np.random.default_rng(3)
    v = rng.integers(0, 40, size=700, dtype=np.uint32)
    v[rng.integers(0, 700, size=20)] = 63
    data = tmp_path / "v.txt"
    write_values(data, v)
    a = run([progs["phases"], "-f", str(data), "-p"])
    b = run([progs["cpu"], "-f", str(data), "-p"])
    assert a.returncode == 0 and b.returncode == 0, a.stderr + b.stderr
    assert listing(a.stdout) == listing(b.stdout)
    # plain timing lines: "N us", the reference's default format
    assert sum(ln.endswith(" us") for ln in a.stdout.splitlines()) == 5


def test_phases_bound_too_small_is_an_error(progs, tmp_path):
    data = tmp_path / "v.txt"
    write_values(data, np.array([1, 2, 300, 4], np.uint32))
    r = run([progs["phases"], "-f", str(data), "-b", "255"])
    assert r.returncode == 1
    assert "[!!!]" in r.stderr


def test_phases_needs_a_file(progs):
    r = run([progs["phases"]])
    assert r.returncode == 2 and "filename" in r.stdout


def test_gpu_builtin_fixture_listing(progs):
    """No -f: the reference's built-in 32 values; the listing (keys 0..bound)
    equals the cpu program's."""
    a = run([progs["gpu"], "-p"])
    b = run([progs["cpu"], "-p"])
    assert a.returncode == 0, a.stderr
    assert "'32' values." in a.stdout and "Maximum value is '42'." in a.stdout
    assert "Using device named" in a.stdout and "Time: '" in a.stdout
    assert listing(a.stdout) == listing(b.stdout)


@pytest.mark.parametrize("merge", ["host", "device"])
@pytest.mark.parametrize("batch,groups,jobs", [
    (1023, 1, 1), (1023, 1, 3), (31, 4, 2), (1023, 64, 2), (4096, 8, 3),
    (100_000, 1, 2), (65_534, 3, 4), (1 << 20, 1, 1)])
def test_gpu_merged_index_matches_whole_column(progs, tmp_path, batch, groups, jobs, merge):
    """Slices built separately (alone or many per batched launch) and merged
    with re-based fills -- on the host, or appended on the device
    (--device-merge) -- give the whole column's index (the reference's merger
    does not)."""
    rng = np.random.default_rng(batch + groups + jobs)
    n = 200_003
    v = rng.integers(0, 3000, size=n, dtype=np.uint32)
    v[50_000:90_000] = 7  # long runs: fills that cross slices
    data, out = tmp_path / "v.txt", tmp_path / "r.bin"
    write_values(data, v)
    r = run([progs["gpu"], "-f", str(data), "--batch-size", str(batch), "-w", str(groups),
             "-j", str(jobs), "-o", str(out)] + (["--device-merge"] if merge == "device" else []))
    assert r.returncode == 0, r.stderr
    if batch % 31 and batch < n:
        assert "rounded to" in r.stdout
    assert_matches_oracle(out, v, f"gpu batch={batch} groups={groups} jobs={jobs}")


def test_gpu_sparse_keys_across_many_slices(progs, tmp_path):
    rng = np.random.default_rng(11)
    n = 120_000
    v = np.zeros(n, np.uint32)
    hits = rng.choice(n, size=40, replace=False)
    v[hits] = rng.integers(1, 4, size=40, dtype=np.uint32)
    data, out = tmp_path / "v.txt", tmp_path / "r.bin"
    write_values(data, v)
    r = run([progs["gpu"], "-f", str(data), "--batch-size", "1023", "-w", "16", "-j", "2",
             "-o", str(out)])
    assert r.returncode == 0, r.stderr
    assert_matches_oracle(out, v, "gpu sparse")


@pytest.mark.parametrize("extra", [[], ["--device-merge"]])
def test_gpu_single_value_and_empty(progs, tmp_path, extra):
    data, out = tmp_path / "v.txt", tmp_path / "r.bin"
    write_values(data, np.array([12345], np.uint32))
    r = run([progs["gpu"], "-f", str(data), "-o", str(out)] + extra)
    assert r.returncode == 0, r.stderr
    assert_matches_oracle(out, np.array([12345], np.uint32), "gpu single")
    data.write_text("")
    r = run([progs["gpu"], "-f", str(data), "-o", str(out)] + extra)
    assert r.returncode == 0, r.stderr
    keys, offsets, index = read_result(out)
    assert keys.size == 0 and index.size == 0


def test_gpu_device_merge_listing_equals_cpu_program(progs, tmp_path):
    """-p with --device-merge lists keys 0..bound from the merged index, as
    the cpu program does."""
    a = run([progs["gpu"], "-p", "--device-merge", "--batch-size", "31"])
    b = run([progs["cpu"], "-p"])
    assert a.returncode == 0, a.stderr
    assert listing(a.stdout) == listing(b.stdout)


def test_gpu_unknown_device_is_an_error(progs):
    r = run([progs["gpu"], "-d", "no such device"])
    assert r.returncode == 3 and "not found" in r.stderr


def test_generate_then_phases_and_gpu(progs, tmp_path):
    """The reference's workflow: generate a file, index it with both drivers."""
    data = tmp_path / "g.txt"
    assert run([progs["generate"], "-a", "1000000", "--seed", "3", "-o", str(data)]).returncode == 0
    v = np.loadtxt(data, dtype=np.uint32)
    a, b = tmp_path / "a.bin", tmp_path / "b.bin"
    assert run([progs["phases"], "-f", str(data), "-o", str(a)]).returncode == 0
    r = run([progs["gpu"], "-f", str(data), "--batch-size", "262143", "-w", "2", "-j", "2",
             "-o", str(b)])
    assert r.returncode == 0, r.stderr
    assert_matches_oracle(a, v, "phases generated")
    assert_matches_oracle(b, v, "gpu generated")


def test_gpu_and_host_parsing_agree(progs, tmp_path):
    """The data file read on the GPU (default) and on the host (--host-parse)
    gives the same column: separators of every kind, leading zeros, and a
    token that ends the stream."""
    rng = np.random.default_rng(21)
    parts = []
    for i in range(30_000):
        parts.append(("0" * int(i % 3)) + str(int(rng.integers(0, 70_000))))
        parts.append(["\n", "\r\n", " ", "\t", "  \n"][i % 5])
    parts.insert(40_001, "oops ")
    data = tmp_path / "v.txt"
    data.write_text("".join(parts))
    a, b = tmp_path / "a.bin", tmp_path / "b.bin"
    ra = run([progs["phases"], "-f", str(data), "-o", str(a)])
    rb = run([progs["phases"], "-f", str(data), "-o", str(b), "--host-parse"])
    assert ra.returncode == 0 and rb.returncode == 0, ra.stderr + rb.stderr
    assert a.read_bytes() == b.read_bytes()
    # "oops" is glued to value 20,001, so that token ends the stream: the
    # column is the first 20,000 values
    v = np.array([int(x) for x in "".join(parts[:40_000]).split()], dtype=np.uint32)
    assert v.size == 20_000
    assert_matches_oracle(a, v, "phases parsed")


def test_overhead_program(tmp_path):
    """The launch-overhead program runs and reports every figure."""
    import json
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.build()
    prog = _lib.build_host(["overhead"])["overhead"]
    r = run([prog, "-i", "200", "-k", "500", "--rows", "4096", "--columns", "64"])
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    assert lines[0].startswith("Took ") and lines[0].endswith(" runs.")
    d = json.loads(lines[1])
    for k in ("actor_us", "direct_us", "build_us"):
        assert d[k]["mean"] > 0
    assert d["stream_us_per_launch"] > 0 and d["graph_us_per_launch"] > 0
    assert d["build_us"]["launches"] >= 5
    assert d["batched_us_per_column"] > 0
