"""Host-side programs without a GPU: the actor runtime, the slice merger of the
`gpu` program (against the oracle), the `generate` program and the oracle's
`cpu` program (against the golden vectors)."""
import os
import subprocess

import numpy as np
import pytest

from indexing_gb300 import _lib
from oracle import oracle as O

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(REPO, "oracle")


@pytest.fixture(scope="module")
def progs(tmp_path_factory):
    progs = _lib.build_host(["generate"])
    exe = tmp_path_factory.mktemp("native") / "actors_test"
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-Wall", "-Wextra",
                    "-I" + _lib.HOST_DIR, os.path.join(REPO, "tests", "native", "actors_test.cpp"),
                    "-o", str(exe)], check=True)
    progs["actors_test"] = str(exe)
    return progs


@pytest.fixture(scope="module")
def cpu_prog():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "bin/cpu"], check=True)
    return os.path.join(ORACLE_DIR, "bin", "cpu")


def run(cmd, **kw):
    return subprocess.run(cmd, capture_output=True, text=True, timeout=120, **kw)


def test_actor_runtime_repeated(progs):
    # repeated runs shake out ordering races in the scheduler
    for _ in range(10):
        r = run([progs["actors_test"]])
        assert r.returncode == 0, r.stderr
        assert "all checks passed" in r.stdout


def test_slice_merger_matches_whole_column_index(tmp_path):
    obj = tmp_path / "wah_oracle.o"
    exe = tmp_path / "merge_test"
    subprocess.run(["gcc", "-O2", "-std=c99", "-c", os.path.join(ORACLE_DIR, "wah_oracle.c"),
                    "-o", str(obj)], check=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-I" + _lib.HOST_DIR, "-I" + ORACLE_DIR,
                    os.path.join(REPO, "tests", "native", "merge_test.cpp"), str(obj),
                    "-o", str(exe)], check=True)
    r = run([str(exe)])
    assert r.returncode == 0, r.stderr
    assert "all" in r.stdout and "passed" in r.stdout


def splitmix_lemire(seed, n, lo, hi):
    """Python restatement of generate's recipe: SplitMix64, high 32 bits,
    Lemire's multiply-and-reject into [lo, hi]."""
    mask = (1 << 64) - 1
    s = seed
    rng = hi - lo + 1
    out = []

    def nxt():
        nonlocal s
        s = (s + 0x9E3779B97F4A7C15) & mask
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
        return z ^ (z >> 31)

    for _ in range(n):
        if rng == 1 << 32:
            out.append(lo + (nxt() >> 32))
            continue
        m = (nxt() >> 32) * rng
        low = m & 0xFFFFFFFF
        if low < rng:
            t = (1 << 32) % rng
            while low < t:
                m = (nxt() >> 32) * rng
                low = m & 0xFFFFFFFF
        out.append(lo + (m >> 32))
    return out


def test_generate_recipe_and_format(progs, tmp_path):
    r = run([progs["generate"], "-a", "1000", "--seed", "7", "-f", "3", "-t", "40000"])
    assert r.returncode == 0
    assert r.stdout.endswith("\n") and not r.stdout.endswith("\n\n")
    vals = [int(x) for x in r.stdout.split()]
    assert vals == splitmix_lemire(7, 1000, 3, 40000)
    # separator and the full uint32 range
    r = run([progs["generate"], "-a", "50", "--seed", "1", "-s", ",", "-t", "4294967295"])
    vals = [int(x) for x in r.stdout.strip().split(",")]
    assert vals == splitmix_lemire(1, 50, 0, 2 ** 32 - 1)
    # same seed, same file
    out = tmp_path / "a.txt"
    assert run([progs["generate"], "-a", "20000", "--seed", "9", "-o", str(out)]).returncode == 0
    again = run([progs["generate"], "-a", "20000", "--seed", "9"]).stdout
    assert out.read_text() == again
    v = np.array(again.split(), dtype=np.uint64)
    assert v.size == 20000 and v.max() <= 65535
    # bad ranges are refused
    assert run([progs["generate"], "-f", "9", "-t", "3"]).returncode != 0
    assert run([progs["generate"], "--nope"]).returncode != 0


def test_cpu_program_builtin_fixture(cpu_prog, golden):
    """The oracle's `cpu` program on the reference's built-in 32 values:
    the reference's output lines and the KAT-1 index."""
    r = run([cpu_prog, "-p"])
    assert r.returncode == 0
    lines = r.stdout.splitlines()
    assert lines[0] == "'32' values."
    assert lines[1] == "Maximum value is '42'."
    assert lines[2] == "Merged to 16 values"
    assert lines[3] == "Index has 16 elements with 15 keys"
    listing = lines[4:]
    assert len(listing) == 43  # keys 0..42, absent ones as "j\t"
    kat = golden["kat1_builtin32"] if "kat1_builtin32" in golden else None
    values = [10, 7, 22, 6, 7, 1, 9, 42, 2, 5, 13, 3, 2, 1, 0, 1,
              18, 18, 3, 13, 5, 9, 0, 3, 2, 19, 5, 23, 22, 10, 6, 22]
    for key in range(43):
        rows = [i for i, x in enumerate(values) if x == key]
        bits = "".join("1" if i in rows else "0" for i in range(max(rows) + 1)) if rows else ""
        assert listing[key] == f"{key}\t{bits}"
    if kat is not None:
        assert np.array_equal(kat["values"], np.array(values, np.uint32))


def test_cpu_program_output_file_matches_golden(cpu_prog, golden, tmp_path):
    for name, case in golden.items():
        data = tmp_path / f"{name}.txt"
        data.write_text("\n".join(str(int(x)) for x in case["values"]) + "\n")
        out = tmp_path / f"{name}.bin"
        r = run([cpu_prog, "-f", str(data), "-o", str(out)])
        assert r.returncode == 0, r.stderr
        got = np.fromfile(out, dtype=np.uint32)
        K, L = int(got[0]), int(got[1])
        assert np.array_equal(got[2:2 + K], case["keys"]), name
        assert np.array_equal(got[2 + K:2 + 2 * K], case["offsets"]), name
        assert np.array_equal(got[2 + 2 * K:2 + 2 * K + L], case["index"]), name


def test_cpu_program_bubble_equals_stable(cpu_prog, tmp_path):
    rng = np.random.default_rng(5)
    v = rng.integers(0, 50, size=3000, dtype=np.uint32)
    data = tmp_path / "v.txt"
    data.write_text("\n".join(map(str, v)) + "\n")
    a = run([cpu_prog, "-f", str(data), "-p"]).stdout
    b = run([cpu_prog, "-f", str(data), "-p", "--bubble"]).stdout
    assert a == b
    ref = O.build(v)
    assert f"Index has {ref.index.size} elements with {ref.keys.size} keys" in a


def test_text_reading_stops_like_a_stream(cpu_prog, tmp_path):
    """`while (source >> next)` stops at the first token that is not a
    number; values around it are kept up to there."""
    data = tmp_path / "v.txt"
    data.write_text("5 6\n7\tx 8 9\n")
    r = run([cpu_prog, "-f", str(data)])
    assert "'3' values." in r.stdout
    data.write_text("1 4294967296 2\n")  # overflow ends the stream too
    r = run([cpu_prog, "-f", str(data)])
    assert "'1' values." in r.stdout


def test_generate_workload_distributions(progs):
    """The benchmark workloads' columns from `generate`: Zipf frequencies
    follow r^-s, `few` has exactly the requested distinct values, runs have
    the requested mean length; all seeded and within [from, to]."""
    g = progs["generate"]
    n = 400_000
    z = np.array(run([g, "-a", str(n), "--dist", "zipf", "--zipf-s", "1.1", "--seed", "3"])
                 .stdout.split(), dtype=np.int64)
    assert z.size == n and z.min() >= 0 and z.max() <= 65535
    w = 1.0 / np.arange(1, 65537, dtype=np.float64) ** 1.1
    p = w / w.sum()
    for r in (0, 1, 9):  # ranks 1, 2, 10
        assert abs(np.mean(z == r) - p[r]) < 5 * np.sqrt(p[r] / n) + 1e-4
    again = run([g, "-a", "1000", "--dist", "zipf", "--seed", "3"]).stdout
    assert again.split() == [str(x) for x in z[:1000]]
    f = np.array(run([g, "-a", "50000", "--dist", "few", "--distinct", "16", "-f", "100",
                      "-t", "65535"]).stdout.split(), dtype=np.int64)
    assert set(np.unique(f)) == set(range(100, 116))
    r = np.array(run([g, "-a", str(n), "--dist", "runs", "--run-mean", "500"]).stdout.split(),
                 dtype=np.int64)
    runs = 1 + np.count_nonzero(np.diff(r))
    assert 0.85 * 500 < n / runs < 1.15 * 500
    assert run([g, "--dist", "nope"]).returncode != 0
    assert run([g, "--dist", "zipf", "-t", "4294967295"]).returncode != 0


def test_generate_serving_trace(progs):
    lines = run([progs["generate"], "--trace", "5000", "--rate", "200", "--seed", "9"]) \
        .stdout.splitlines()
    assert len(lines) == 5000
    t = np.array([float(x.split()[0]) for x in lines])
    rows = np.array([int(x.split()[1]) for x in lines])
    kinds = {x.split()[2] for x in lines}
    assert (np.diff(t) > 0).all()
    assert 0.9 / 200 < t[-1] / 5000 < 1.1 / 200
    assert rows.min() >= 10_000 and rows.max() <= 16_777_216
    # log-uniform sizes: the median near the geometric mean of the bounds
    assert 0.7 < np.median(rows) / np.sqrt(10_000 * 16_777_216) < 1.4
    assert kinds == {"uniform", "zipf", "runs"}
