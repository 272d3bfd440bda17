"""The bounded device-side waits give up with WAH_ETIMEOUT and leave the
context usable.

Every wait of the library's kernels on an mbarrier (the scatter's and the
emit's bulk-copied tiles) goes through mbar_wait_bounded: after a clock limit
it returns false, the kernel records WAH_ETIMEOUT in the build's status word
and returns instead of spinning.  The reference has no such path: it exits
the process on any error (src/phases.cpp:102-112).  A test-only kernel
(tests/native/wait_timeout.cu) makes that wait run out on purpose in the
only way that cannot hang or fault: an mbarrier that nothing arrives at, no
copy in flight, and a limit of 10^5 clocks.  Afterwards the same stream
builds an index that must equal the oracle's.
"""
import ctypes
import os
import subprocess
import time

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WAH_ETIMEOUT = 4


@pytest.fixture(scope="module")
def waitlib(tmp_path_factory):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from indexing_gb300 import _lib
    out = tmp_path_factory.mktemp("timeout") / "libwait_timeout.so"
    subprocess.run([_lib.nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                    "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-I" + _lib.INCLUDE,
                    "-I" + _lib.CSRC, os.path.join(REPO, "tests", "native", "wait_timeout.cu"),
                    "-o", str(out)], check=True)
    lib = ctypes.CDLL(str(out))
    lib.test_wait_on_nobody.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong,
                                        ctypes.c_int, ctypes.c_void_p]
    lib.test_wait_on_nobody.restype = ctypes.c_int
    return lib


@pytest.mark.parametrize("threads", [32, 256])
def test_wait_gives_up_with_etimeout(waitlib, threads):
    import indexing_gb300 as wah
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    completed = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    assert waitlib.test_wait_on_nobody(status.data_ptr(), completed.data_ptr(), 100_000,
                                       threads, stream.cuda_stream) == 0
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t0
    assert int(status.item()) == WAH_ETIMEOUT
    assert int(completed.item()) == 0
    assert elapsed < 5.0  # gave up after its limit (10^5 clocks), did not spin
    # the context and the stream stay usable: a build on the same stream
    rng = np.random.default_rng(9)
    v = rng.integers(0, 65536, size=200_000, dtype=np.uint32)
    got = wah.build_index(v, bound=65535, stream=stream).numpy()
    ref = O.build(v)
    assert np.array_equal(got.keys, ref.keys)
    assert np.array_equal(got.offsets, ref.offsets)
    assert np.array_equal(got.index, ref.index)
