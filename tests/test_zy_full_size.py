"""Bit-exact parity at the sizes the benchmark quotes its numbers on.

The reference checks every phase against its CPU code at the run's own size
(src/phases.cpp:775-807, :1097-1123, built WITH_CPU_TESTS).  Here the GPU
results of the benchmark's own inputs are compared word for word (keys,
offsets, index, merged-entry count) with the oracle, the plain-C
restatement of the reference `cpu` program, run on host threads:

* the 268,435,456-row uniform [0, 65535] column (seed 20170101, bound 65535);
* the three 268,435,456-row skewed / clustered columns (Zipf s=1.1, 16
  distinct values, runs of mean length 1,000);
* every column of the 4,096-column batched mix, built by a replayed graph;
* the 20,000-request serving trace: every request served in the mix equals
  the same request built alone (a 64-bit fingerprint of its keys, offsets
  and index, taken on the device), and a seeded sample equals the oracle
  word for word;
* a column of 2^30 + 4,099 rows, above the row limit of earlier builds.

The inputs come from the benchmark's own generators.  The file name makes
pytest collect it after the other GPU tests and before the allocation-free
entry point's test.
"""
import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

N = 268_435_456
SEED = 20170101


@pytest.fixture(scope="module")
def env():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import indexing_gb300 as wah
    lib = wah._lib.load()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    return wah, lib, dev


def _build(lib, wah, d_values, n, bound, dev):
    b = wah._Buffers(n, bound, dev)
    rc = lib.wah_build(d_values.data_ptr(), n, bound, b.keys.data_ptr(), b.offsets.data_ptr(),
                       b.index.data_ptr(), b.counts.data_ptr(), b.ws.data_ptr(), b.ws_bytes,
                       torch.cuda.current_stream(dev).cuda_stream)
    assert rc == 0
    got = bench.result_numpy(b.keys, b.offsets, b.index, b.counts)
    del b
    torch.cuda.empty_cache()
    return got


def test_full_size_single_columns(env):
    """C2 and the three C3 columns, 268,435,456 rows each."""
    wah, lib, dev = env
    jobs, names = [], []
    v = bench.gen_uniform(N, 65536, SEED)
    d = torch.from_numpy(v.view(np.int32)).to(dev)
    jobs.append((v, _build(lib, wah, d, N, 65535, dev)))
    names.append("uniform")
    del d
    for kind in ("zipf1.1", "distinct16", "runs1000"):
        d = bench.gen_skewed(kind, N, SEED, torch, dev)
        got = _build(lib, wah, d, N, 65535, dev)
        jobs.append((d.cpu().numpy().view(np.uint32), got))
        names.append(kind)
        del d
        torch.cuda.empty_cache()
    for name, (_, got) in zip(names, jobs):
        assert got[0] == 0, f"{name}: device status {got[0]}"
    bad, count = bench.check_columns(jobs, bench.oracle_threads(N, len(jobs)))
    assert count == 4
    assert not bad, f"columns differing from the oracle: {[names[i] for i in bad]}"


def test_batched_mix_every_column(env):
    """C4: all 4,096 columns of the batched mix, from a replayed graph."""
    wah, lib, dev = env
    stream = torch.cuda.current_stream(dev)
    sizes, cards, cols = bench.gen_batched(4096, SEED + 4, torch, dev)
    b = wah.Batch(sizes.tolist(), [int(c) - 1 for c in cards])
    outs = b.set_columns(cols, stream=stream)
    b.launch_graph(stream)
    b.launch_graph(stream)  # a replay of the captured graph
    torch.cuda.synchronize()
    status = torch.stack([o[3] for o in outs]).cpu().numpy().view(np.uint32)[:, 3]
    assert (status == 0).all()
    bad, count = bench.check_batched_columns(outs, cols, bench.oracle_threads(4194304, 16))
    b.close()
    assert count == 4096
    assert not bad, f"{len(bad)} columns differ from the oracle, first {bad[:10]}"


def test_serving_trace_each_request_equal_alone(env):
    """C5: the 20,000-request trace at a fixed offered load (30 G rows/s,
    about 80% of the server's measured capacity on GB300), 64 GB budget;
    every request as served has the fingerprint of the same request built
    alone, and 64 of them equal the oracle word for word."""
    wah, lib, dev = env
    nreq = 20_000
    rng, sizes, kinds, pools, dpools = bench.gen_serving(nreq, SEED + 5, torch, dev)
    rate = 30e9 / float(sizes.mean())
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
    out = bench.verify_serving(lib, wah, torch, dev, sizes, kinds, pools, dpools, arrivals,
                               nreq, 64, 64, SEED + 55,
                               bench.oracle_threads(bench.SERVE_MAX_ROWS, 16))
    assert out["equal_alone"] == nreq, f"differ from alone: {out['differ_alone'][:10]}"
    assert out["oracle_checked"] == 64
    assert not out["oracle_differ"], f"differ from the oracle: {out['oracle_differ']}"


def test_column_above_two_to_the_thirty(env):
    """A column just above 2^30 rows (the limit before u32 positions were
    shown to hold up to 2^31 rows), against the oracle word for word."""
    wah, lib, dev = env
    n = (1 << 30) + 4099
    v = bench.gen_uniform(n, 65536, SEED + 30)
    d = torch.from_numpy(v.view(np.int32)).to(dev)
    got = _build(lib, wah, d, n, 65535, dev)
    del d
    torch.cuda.empty_cache()
    assert got[0] == 0
    bad, count = bench.check_columns([(v, got)], 1)
    assert count == 1 and not bad
