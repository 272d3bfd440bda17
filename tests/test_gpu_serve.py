"""Continuous-batching server: every request's index is the same as built
alone (the oracle), whatever mix of requests it was batched with; plain mode
too; the arena is empty again after release."""
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


def requests(rng, count, max_n):
    out = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(1000), np.log(max_n))))
        kind = i % 3
        if kind == 0:
            v = rng.integers(0, 65536, size=n, dtype=np.uint32)
        elif kind == 1:
            w_ = 1.0 / np.arange(1, 65537, dtype=np.float64) ** 1.1
            v = np.minimum(np.searchsorted(np.cumsum(w_) / w_.sum(), rng.random(n)),
                           65535).astype(np.uint32)
        else:
            runs = rng.geometric(1 / 1000, size=n // 500 + 2)
            v = np.repeat(rng.integers(0, 65536, size=runs.size, dtype=np.uint32), runs)[:n]
        t = torch.empty(n, dtype=torch.int32, pin_memory=True)
        t.numpy()[:] = v.view(np.int32)
        out.append((v, t))
    return out


@pytest.mark.parametrize("plain", [False, True])
def test_server_results_equal_alone(wah, plain):
    rng = np.random.default_rng(50 + plain)
    reqs = requests(rng, 60, 400_000)
    srv = wah.Server(budget_bytes=2 << 30, max_batch=16, streams=2, plain=plain)
    ids = [srv.submit(t, bound=65535, delay=0.0002 * i) for i, (_, t) in enumerate(reqs)]
    for (v, _), rid in zip(reqs, ids):
        got = srv.result(rid).numpy()
        ref = O.build(v)
        assert np.array_equal(got.keys, ref.keys)
        assert np.array_equal(got.offsets, ref.offsets)
        assert np.array_equal(got.index, ref.index)
        assert got.merged == ref.merged
    assert srv.arena_used == 0 or plain  # plain keeps its workspace
    srv.close()


def test_server_small_budget_still_progresses(wah):
    # budget for only a few requests at a time: admission waits for releases
    rng = np.random.default_rng(52)
    reqs = requests(rng, 20, 200_000)
    srv = wah.Server(budget_bytes=64 << 20, max_batch=8, streams=2)
    ids = [srv.submit(t, bound=65535) for _, t in reqs]
    for (v, _), rid in zip(reqs, ids):
        got = srv.result(rid).numpy()
        assert np.array_equal(got.index, O.build(v).index)
    srv.close()


def test_server_refuses_oversized(wah):
    srv = wah.Server(budget_bytes=16 << 20, max_batch=4, streams=1)
    t = torch.empty(1 << 20, dtype=torch.int32, pin_memory=True)
    with pytest.raises(wah.WahError) as e:
        srv.submit(t, bound=65535)
    assert e.value.status == wah.WAH_ENOMEM
    srv.close()
