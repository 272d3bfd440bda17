"""One-column builds captured into a CUDA graph and replayed with new data.

Every kernel of a one-column build is launched as a programmatic dependent
of the kernel before it, so a captured build holds programmatic edges.  Each
replay here runs after the next column has been copied into the same input
buffer on the replay stream; the result of every replay must equal the
oracle word for word (keys, offsets, index, merged count).  Sizes: a
1,048,576-row column (16-bit exchange between the digit passes) and a
33,554,432-row column (ranges long enough for the packed exchange), with
16-bit keys (key-start mode) and without a bound.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def env():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import indexing_gb300 as wah
    lib = wah._lib.load()
    return wah, lib


def _result(b):
    c = b.counts.cpu().numpy().view(np.uint32)
    K, L = int(c[0]), int(c[1])
    return (int(c[3]), b.keys[:K].cpu().numpy().view(np.uint32),
            b.offsets[:K].cpu().numpy().view(np.uint32),
            b.index[:L].cpu().numpy().view(np.uint32), int(c[2]))


@pytest.mark.parametrize("n,bound", [(1 << 20, 65535), (1 << 20, 0), (1 << 25, 65535)])
def test_replayed_build_equals_oracle(env, n, bound):
    wah, lib = env
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(n + bound)
    cols = [rng.integers(0, 65536, n, dtype=np.uint32),
            np.repeat(rng.integers(0, 65536, n // 1000 + 1, dtype=np.uint32), 1000)[:n],
            rng.zipf(1.3, n).astype(np.uint32) % 65536]
    d_v = torch.empty(n, dtype=torch.int32, device=dev)
    b = wah._Buffers(n, bound, dev)
    g = torch.cuda.CUDAGraph()
    cs = torch.cuda.Stream(dev)
    d_v.copy_(torch.from_numpy(cols[0].view(np.int32)))
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=cs, capture_error_mode="thread_local"):
        rc = lib.wah_build(d_v.data_ptr(), n, bound, b.keys.data_ptr(), b.offsets.data_ptr(),
                           b.index.data_ptr(), b.counts.data_ptr(), b.ws.data_ptr(), b.ws_bytes,
                           cs.cuda_stream)
    assert rc == 0
    for v in cols:
        with torch.cuda.stream(cs):
            d_v.copy_(torch.from_numpy(v.view(np.int32)))
            g.replay()
        cs.synchronize()
        status, keys, offs, index, merged = _result(b)
        assert status == 0
        ref = O.build(v)
        assert np.array_equal(keys, ref.keys)
        assert np.array_equal(offs, ref.offsets)
        assert index.size == ref.index.size and np.array_equal(index, ref.index)
        assert merged == ref.merged
