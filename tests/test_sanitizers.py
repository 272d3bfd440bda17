"""Host code under AddressSanitizer and UndefinedBehaviorSanitizer (no GPU):
the actor runtime's self-checks, the slice merger against the oracle, and
the oracle's `cpu` program on a data file, each built with
-fsanitize=address,undefined and required to run clean."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from indexing_gb300 import _lib

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(REPO, "oracle")
SAN = ["-fsanitize=address,undefined", "-fno-omit-frame-pointer", "-fno-sanitize-recover=all",
       "-g", "-O1"]
ENV = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=1",
           UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")


def _have_sanitizers(tmp_path):
    src = tmp_path / "t.c"
    src.write_text("int main(void) { return 0; }\n")
    r = subprocess.run(["gcc", *SAN, str(src), "-o", str(tmp_path / "t")], capture_output=True)
    return r.returncode == 0 and subprocess.run([str(tmp_path / "t")], env=ENV).returncode == 0


@pytest.fixture(scope="module")
def san_dir(tmp_path_factory):
    d = tmp_path_factory.mktemp("san")
    if shutil.which("gcc") is None or not _have_sanitizers(d):
        pytest.skip("no sanitizer runtime here")
    return d


def test_actor_runtime_sanitized(san_dir):
    exe = san_dir / "actors_test"
    subprocess.run(["g++", "-std=c++17", "-pthread", *SAN, "-I" + _lib.HOST_DIR,
                    os.path.join(REPO, "tests", "native", "actors_test.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, env=ENV, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "all checks passed" in r.stdout


def test_slice_merger_sanitized(san_dir):
    obj = san_dir / "wah_oracle.o"
    exe = san_dir / "merge_test"
    subprocess.run(["gcc", "-std=c99", *SAN, "-c", os.path.join(ORACLE, "wah_oracle.c"),
                    "-o", str(obj)], check=True)
    subprocess.run(["g++", "-std=c++17", "-pthread", *SAN, "-I" + _lib.HOST_DIR, "-I" + ORACLE,
                    os.path.join(REPO, "tests", "native", "merge_test.cpp"), str(obj),
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, env=ENV, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]


def test_cpu_program_sanitized(san_dir):
    exe = san_dir / "cpu"
    subprocess.run(["gcc", "-std=c99", *SAN, os.path.join(ORACLE, "cpu_main.c"),
                    os.path.join(ORACLE, "wah_oracle.c"), "-o", str(exe)], check=True)
    rng = np.random.default_rng(4)
    v = rng.integers(0, 300, size=20_000, dtype=np.uint32)
    data = san_dir / "v.txt"
    data.write_text("\n".join(map(str, v.tolist())) + "\n")
    for extra in ([], ["-p"], ["--bubble"]):
        r = subprocess.run([str(exe), "-f", str(data), "-o", str(san_dir / "r.bin"), *extra],
                           capture_output=True, text=True, env=ENV, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([str(exe), "-p"], capture_output=True, text=True, env=ENV)
    assert r.returncode == 0 and "Index has 16 elements with 15 keys" in r.stdout
