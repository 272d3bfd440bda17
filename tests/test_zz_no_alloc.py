"""wah_build_noalloc: the build for callers that cannot allocate device memory.

An engine that owns the whole device memory pool, or a serving loop that
cannot pay for cudaMalloc's device synchronisation, hands the library only the
column and the output buffers; the scratch memory comes from a fixed array in
the library.  This checks, through the C ABI, that two calls in a row give
exactly what the regular wah_build gives (integer output: bit-exact), with
and without a 16-bit bound, that the array's leftover contents from the first
call do not leak into the second, that a call takes no device memory, and
that a column over the limit is refused.  The file name makes pytest collect
it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

MAX_ROWS = 1 << 20


def _buffers(n):
    kc, ic = max(n, 1), max(2 * n, 1)
    return (torch.empty(kc, dtype=torch.int32, device="cuda"),
            torch.empty(kc, dtype=torch.int32, device="cuda"),
            torch.empty(ic, dtype=torch.int32, device="cuda"),
            torch.zeros(4, dtype=torch.int32, device="cuda"))


def _result(keys, offs, index, counts):
    c = counts.cpu().numpy().view(np.uint32)
    K, L = int(c[0]), int(c[1])
    return (c[3], c[2], keys[:K].cpu().numpy().view(np.uint32),
            offs[:K].cpu().numpy().view(np.uint32), index[:L].cpu().numpy().view(np.uint32))


@pytest.mark.parametrize("bound", [0, 65535])
def test_noalloc_matches_wah_build_twice(bound):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from indexing_gb300 import _lib
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(77 + bound)
    # two different columns in a row: the second must not see the first's scratch
    cols = [rng.integers(0, 65536, size=MAX_ROWS, dtype=np.uint32),
            np.repeat(rng.integers(0, 300, size=5000, dtype=np.uint32), 97)[:123_457]]
    for call, v in enumerate(cols):
        n = v.size
        d_v = torch.from_numpy(v.view(np.int32)).cuda()
        # regular entry point with its own workspace
        ref = _buffers(n)
        wsb = lib.wah_workspace_bytes(n, bound)
        ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
        assert lib.wah_build(d_v.data_ptr(), n, bound, ref[0].data_ptr(), ref[1].data_ptr(),
                             ref[2].data_ptr(), ref[3].data_ptr(), ws.data_ptr(), wsb,
                             stream) == 0
        # allocation-free entry point; from the second call on, the device's
        # free memory must not move across the call
        got = _buffers(n)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        assert lib.wah_build_noalloc(d_v.data_ptr(), n, bound, got[0].data_ptr(),
                                     got[1].data_ptr(), got[2].data_ptr(),
                                     got[3].data_ptr(), stream) == 0
        torch.cuda.synchronize()
        if call > 0:
            assert torch.cuda.mem_get_info()[0] == free_before
        a, b = _result(*ref), _result(*got)
        assert a[0] == 0 and b[0] == 0
        assert a[1] == b[1]
        for x, y in zip(a[2:], b[2:]):
            assert np.array_equal(x, y)
        # and word for word what the oracle builds
        from oracle import oracle as O
        o = O.build(v)
        assert b[1] == o.merged
        assert np.array_equal(b[2], o.keys) and np.array_equal(b[3], o.offsets)
        assert np.array_equal(b[4], o.index)


def test_noalloc_refuses_oversize():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from indexing_gb300 import _lib
    lib = _lib.load()
    rc = lib.wah_build_noalloc(ctypes.c_void_p(256), MAX_ROWS + 1, 0, ctypes.c_void_p(256),
                               ctypes.c_void_p(256), ctypes.c_void_p(256),
                               ctypes.c_void_p(256), None)
    assert rc == 5  # WAH_ERANGE, before anything is enqueued
