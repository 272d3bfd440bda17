"""The GPU host programs (`gpu`, `phases`) built with AddressSanitizer and
run on the device: actor handlers, worker threads and the page-locked
buffers must run clean (use after return and use after scope included).
CUDA's own allocations are not leak-checked and the shadow gap stays
unprotected, as ASan needs next to the CUDA driver."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from indexing_gb300 import _lib

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

ASAN = ["-fsanitize=address", "-fno-omit-frame-pointer", "-g", "-O1"]
ENV = dict(os.environ, ASAN_OPTIONS="protect_shadow_gap=0:detect_leaks=0:"
                                    "detect_stack_use_after_return=1:abort_on_error=1")


@pytest.fixture(scope="module")
def progs(tmp_path_factory):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    _lib.build()
    d = tmp_path_factory.mktemp("asan")
    out = {}
    for name in ("gpu", "phases"):
        exe = d / name
        r = subprocess.run(["g++", "-std=c++17", "-pthread", *ASAN, "-I" + _lib.INCLUDE,
                            os.path.join(_lib.HOST_DIR, name + ".cpp"), "-o", str(exe),
                            "-L" + _lib.PKG_DIR, "-l:libwah_gb300.so",
                            "-Wl,-rpath," + _lib.PKG_DIR], capture_output=True, text=True)
        if r.returncode != 0:
            pytest.skip("no AddressSanitizer build here: " + r.stderr[-300:])
        out[name] = str(exe)
    return out


def run(args):
    return subprocess.run(args, capture_output=True, text=True, env=ENV, timeout=300)


@pytest.mark.parametrize("extra", [[], ["--device-merge"]])
def test_gpu_program_clean(progs, tmp_path, extra):
    # the built-in fixture in two slices, then a file over several batches
    r = run([progs["gpu"], "-p", "--batch-size", "31"] + extra)
    assert r.returncode == 0 and "AddressSanitizer" not in r.stderr, r.stderr[-3000:]
    v = np.random.default_rng(5).integers(0, 500, size=20_000, dtype=np.uint32)
    data = tmp_path / "v.txt"
    data.write_text("\n".join(map(str, v.tolist())) + "\n")
    r = run([progs["gpu"], "-f", str(data), "--batch-size", "1023", "-w", "4", "-j", "3",
             "-o", str(tmp_path / "r.bin")] + extra)
    assert r.returncode == 0 and "AddressSanitizer" not in r.stderr, r.stderr[-3000:]


def test_phases_program_clean(progs, tmp_path):
    v = np.random.default_rng(6).integers(0, 65536, size=50_000, dtype=np.uint32)
    data = tmp_path / "v.txt"
    data.write_text("\n".join(map(str, v.tolist())) + "\n")
    r = run([progs["phases"], "-f", str(data), "--describe"])
    assert r.returncode == 0 and "AddressSanitizer" not in r.stderr, r.stderr[-3000:]
