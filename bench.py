#!/usr/bin/env python3
"""Benchmark of the WAH index build on GB300.

Default workload (one GPU): one column of 268,435,456 uint32 values, i.i.d.
uniform in [0, 65535] from a seeded PRNG (numpy PCG64), bound = 65535 (the
reference's -b).  A step is one full index build of that column: digit
histogram, plan, two radix digit passes (per-range counts and scatter), fused
index build.

Printed: one JSON line on stdout.  Per-phase "N us" lines (the reference's
SHOW_TIME_CONSUMPTION output, src/phases.cpp:714-1127) go to stderr.

  value       rows/s with the column resident in HBM (CUDA events around K
              builds on the launching stream; the 1 GiB input and 6+ GiB of
              traffic per build exceed the 129 MB L2, so no flush is needed)
  e2e         rows/s through the pipelined host-buffer API (wah_pipe_*) with
              pinned host buffers: H2D of the values, build, D2H of
              keys/offsets/index, every step; consecutive steps overlap
  roofline    the dominant kernel's algorithmic bytes / its mean event-timed
              duration, against the measured HBM copy bandwidth
  column_roofline  the whole build on the scope table's byte formula
              (40n + 24k + 4L + 8K) over the build time, same peak
  autotune    the radix tile shapes timed and applied before the run (digit
              pass 0's shape, and the later passes' in the upper 16 bits)
  cpu_baseline  the oracle (plain-C restatement of the reference `cpu`
              program) on a bounded sample, host cores of this machine
  decode      the built index decoded back to row ids on the device, and
              one-key / 1,000-key range queries
  ingest      the column as a one-value-per-line text file parsed on the
              device (resident text, and from pinned host memory)
  c1          a 1,048,576-row column: device build latency and the build
              through the host-buffer context API
  append      the index of the first ~3/4 of the column and the index of the
              rest appended on the device (wah_append), checked word for word
              against the whole-column build

--impl reference times the reference CPU implementation (the oracle port:
the reference's own sources are not on the GPU machine) on all host threads.
Multi-GPU (torchrun): independent replicas, one column per rank, no
collective on the data path ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "rows/s & HBM GB/s at 256M u32; batched rows/s + p50/p99 vs plain, bit-exact"
# wah_build_timed spans: phases, then single kernels inside them
PHASES = ["histogram", "plan", "pass0", "pass1", "pass2", "pass3", "build",
          "scatter0", "scatter1", "scatter2", "scatter3", "emit"]
KERNELS = ["histogram", "scatter0", "scatter1", "scatter2", "scatter3", "emit"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=268_435_456)
    ap.add_argument("--card", type=int, default=65536, help="values uniform in [0, card)")
    ap.add_argument("--bound", type=int, default=None,
                    help="bound given to the build (default card - 1; 0: the build scans "
                         "the column for its largest value)")
    ap.add_argument("--seed", type=int, default=20170101)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-skewed", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batch-cols", type=int, default=4096)
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip timing every radix tile shape on this size before the run")
    ap.add_argument("--tune-cache", default=None, help="autotuner cache file")
    ap.add_argument("--no-ingest", action="store_true")
    ap.add_argument("--no-decode", action="store_true")
    ap.add_argument("--no-append", action="store_true")
    ap.add_argument("--no-c1", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=20000)
    ap.add_argument("--serve-budget-gb", type=int, default=64)
    ap.add_argument("--pipe-depth", type=int, default=3,
                    help="builds in flight in the end-to-end leg")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sort-items", type=int, default=0,
                    help="radix scatter tuning: rows per thread | peer-mask flags, optionally "
                         "| (later passes' shape << 16) (0: library default)")
    ap.add_argument("--cpu-sample", type=int, default=1 << 23,
                    help="rows per oracle build in the CPU legs")
    return ap.parse_args()


def gen_uniform(n: int, card: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).integers(0, card, size=n, dtype=np.uint32)


def load_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def replica_throughput(elapsed_ms: float, rows_per_step: int, steps: int, dist=None,
                       device="cpu"):
    """Replicas only: every rank builds its own column, no collective on the
    data path.  The job's time is the slowest rank's (max over ranks); the
    job's throughput counts every rank's rows.  Returns (max_ms, rows/s)."""
    import torch
    world = 1
    max_ms = elapsed_ms
    if dist is not None and dist.is_initialized():
        world = dist.get_world_size()
        t = torch.tensor([elapsed_ms], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        max_ms = float(t.item())
    return max_ms, world * rows_per_step * steps / (max_ms / 1e3)


def time_events(fn, steps, torch, stream):
    """Mean ms of fn() over steps, CUDA events on `stream`."""
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(steps):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def gen_skewed(kind: str, n: int, seed: int, torch, dev):
    """Seeded device columns of the skewed / clustered workloads."""
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    if kind == "zipf1.1":
        w = 1.0 / np.arange(1, 65537, dtype=np.float64) ** 1.1
        cdf = torch.from_numpy(np.cumsum(w) / w.sum()).to(dev)
        u = torch.rand(n, generator=g, device=dev, dtype=torch.float64)
        return torch.searchsorted(cdf, u).clamp_(max=65535).to(torch.int32)
    if kind == "distinct16":
        return torch.randint(0, 16, (n,), generator=g, device=dev, dtype=torch.int32)
    if kind == "runs1000":
        rng = np.random.default_rng(seed)
        runs = rng.geometric(1 / 1000, size=n // 1000 * 2 + 16)
        cum = np.cumsum(runs)
        m = int(np.searchsorted(cum, n)) + 1
        runs = runs[:m]
        runs[-1] -= int(cum[m - 1] - n)
        vals = torch.from_numpy(rng.integers(0, 65536, size=m, dtype=np.int64)).to(dev)
        return torch.repeat_interleave(vals, torch.from_numpy(runs).to(dev)).to(torch.int32)
    raise ValueError(kind)


def bench_skewed(args, lib, wah, torch, dev, stream):
    """C3: skewed and clustered single columns of args.n rows, bound 65535."""
    out = {}
    for kind in ("zipf1.1", "distinct16", "runs1000"):
        v = gen_skewed(kind, args.n, args.seed, torch, dev)
        bufs = wah._Buffers(args.n, 65535, dev)
        sh = stream.cuda_stream

        def step():
            rc = lib.wah_build(v.data_ptr(), args.n, 65535, bufs.keys.data_ptr(),
                               bufs.offsets.data_ptr(), bufs.index.data_ptr(),
                               bufs.counts.data_ptr(), bufs.ws.data_ptr(), bufs.ws_bytes, sh)
            assert rc == 0
        step()
        ms = time_events(step, max(3, args.steps // 5), torch, stream)
        c = bufs.counts.cpu().numpy().view(np.uint32)
        assert c[3] == 0
        out[kind] = {"rows_per_s": args.n / (ms / 1e3), "ms": ms, "keycnt": int(c[0]),
                     "index_len": int(c[1]), "merged": int(c[2])}
        del v, bufs
        torch.cuda.empty_cache()
    return out


def bench_batched(args, lib, wah, torch, dev, stream):
    """C4: 4,096 columns, rows log-uniform in [1,024, 4,194,304], cardinality
    log-uniform in [2, 65,536], values uniform within it.  Batched (one
    launch sequence, replayed CUDA graph) against the plain path (one
    wah_build per column on the same stream)."""
    rng = np.random.default_rng(args.seed + 4)
    ncols = args.batch_cols
    sizes = np.rint(np.exp(rng.uniform(np.log(1024), np.log(4194304), ncols))).astype(np.int64)
    cards = np.rint(np.exp(rng.uniform(np.log(2), np.log(65536), ncols))).astype(np.int64)
    g = torch.Generator(device=dev)
    g.manual_seed(args.seed + 4)
    cols = [torch.randint(0, int(c), (int(n),), generator=g, device=dev, dtype=torch.int32)
            for n, c in zip(sizes, cards)]
    bounds = [int(c) - 1 for c in cards]
    b = wah.Batch(sizes.tolist(), bounds)
    outs = b.set_columns(cols, stream=stream)
    b.launch_graph(stream)
    ms_batched = time_events(lambda: b.launch_graph(stream), 3, torch, stream)
    counts_b = torch.stack([o[3] for o in outs]).cpu().numpy().view(np.uint32).copy()
    assert (counts_b[:, 3] == 0).all()
    # plain path into the same outputs, one workspace sized for the largest column
    nmax = int(sizes.max())
    wsb = wah.workspace_bytes(nmax, 0)
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    sh = stream.cuda_stream

    def plain():
        for c in range(ncols):
            keys, offs, index, cnt = outs[c]
            rc = lib.wah_build(cols[c].data_ptr(), int(sizes[c]), bounds[c], keys.data_ptr(),
                               offs.data_ptr(), index.data_ptr(), cnt.data_ptr(),
                               ws.data_ptr(), wsb, sh)
            assert rc == 0
    plain()
    ms_plain = time_events(plain, 2, torch, stream)
    counts_p = torch.stack([o[3] for o in outs]).cpu().numpy().view(np.uint32)
    same = bool((counts_p == counts_b).all())
    total = int(sizes.sum())
    b.close()
    del cols, outs, ws
    torch.cuda.empty_cache()
    return {"columns": ncols, "rows": total, "ranges": None,
            "rows_per_s_batched": total / (ms_batched / 1e3), "ms_batched": ms_batched,
            "rows_per_s_plain": total / (ms_plain / 1e3), "ms_plain": ms_plain,
            "speedup": ms_plain / ms_batched, "same_counts_as_plain": same}


def column_text(col, max_digits, torch):
    """The column as the reference's data file (`generate` format: one value
    per line), built on the device: digits are scattered to each value's
    offset in the text."""
    v = col.to(torch.int64)
    ndig = torch.ones_like(v)
    t = v // 10
    for _ in range(max_digits - 1):
        ndig += (t > 0).to(torch.int64)
        t //= 10
    del t
    ends = torch.cumsum(ndig + 1, 0)
    starts = ends - ndig - 1
    text = torch.full((int(ends[-1].item()),), 10, dtype=torch.uint8, device=col.device)
    last = starts + ndig - 1
    del ends, starts
    x = v
    for d in range(max_digits):
        m = ndig > d
        text[last[m] - d] = (x[m] % 10 + 48).to(torch.uint8)
        x = x // 10
    return text


def bench_ingest(args, lib, torch, dev, stream, d_values, n):
    """Text ingest: the column written as a one-value-per-line data file
    (the reference's `generate` format), parsed by wah_parse_text from device
    memory (value) and from pinned host memory with the copy in the timed
    region (e2e).  The parsed column must equal the original."""
    digits = len(str(args.card - 1))
    text = column_text(d_values, digits, torch)
    nbytes = text.numel()
    out = torch.empty((nbytes + 1) // 2, dtype=torch.int32, device=dev)
    res = torch.zeros(4, dtype=torch.int64, device=dev)
    wsb = int(lib.wah_parse_workspace_bytes())
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    sh = stream.cuda_stream

    def parse_dev(src=text):
        rc = lib.wah_parse_text(src.data_ptr(), nbytes, out.data_ptr(), out.numel(),
                                res.data_ptr(), ws.data_ptr(), wsb, sh)
        assert rc == 0
    parse_dev()
    torch.cuda.synchronize()
    count = int(res.cpu().numpy()[0])
    same = count == n and bool(torch.equal(out[:n], d_values))
    steps = max(3, args.steps // 5)
    ms = time_events(parse_dev, steps, torch, stream)
    host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    host.copy_(text)
    staging = torch.empty_like(text)

    def parse_host():
        staging.copy_(host, non_blocking=True)
        parse_dev(staging)
    parse_host()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        parse_host()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    del text, out, staging, host
    torch.cuda.empty_cache()
    return {"text_bytes": nbytes, "values": count, "parsed_equals_column": same,
            "ms": ms, "rows_per_s": n / (ms / 1e3), "text_gb_per_s": nbytes / (ms / 1e3) / 1e9,
            "alg_bytes": nbytes + 4 * n,
            "e2e": {"rows_per_s": n / dt, "ms": dt * 1e3, "h2d_bytes_per_step": nbytes}}


def bench_decode(args, lib, torch, dev, stream, bufs, n, K, L):
    """Decode of the built index back to row ids on the device (wah_decode),
    and one-key / value-range queries (wah_query)."""
    rows = torch.empty(n, dtype=torch.int32, device=dev)
    st = torch.zeros(4, dtype=torch.int32, device=dev)
    wsb = int(lib.wah_decode_workspace_bytes())
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    sh = stream.cuda_stream

    def dec():
        rc = lib.wah_decode(bufs.keys.data_ptr(), bufs.offsets.data_ptr(), bufs.index.data_ptr(),
                            K, L, n, rows.data_ptr(), None, None, None, st.data_ptr(),
                            ws.data_ptr(), wsb, sh)
        assert rc == 0
    dec()
    ms = time_events(dec, max(3, args.steps // 5), torch, stream)
    assert int(st[0].item()) == 0
    qws_b = int(lib.wah_query_workspace_bytes(n))
    qws = torch.empty(qws_b, dtype=torch.uint8, device=dev)
    qrows = torch.empty(n, dtype=torch.int32, device=dev)
    qwords = torch.empty(2 * ((n + 30) // 31), dtype=torch.int32, device=dev)
    qres = torch.zeros(4, dtype=torch.int32, device=dev)
    out = {"decode_rows_per_s": n / (ms / 1e3), "decode_ms": ms,
           "decode_alg_bytes": 4 * L + 4 * n}
    for name, lo, hi in (("one_key", 1234, 1234), ("range_1000_keys", 0, 999)):
        def q():
            rc = lib.wah_query(bufs.keys.data_ptr(), bufs.offsets.data_ptr(),
                               bufs.index.data_ptr(), K, L, n, lo, hi, 0, 0, 0,
                               qwords.data_ptr(), qwords.numel(), qrows.data_ptr(), n,
                               qres.data_ptr(), qws.data_ptr(), qws_b, sh)
            assert rc == 0
        q()
        qms = time_events(q, 5, torch, stream)
        r = qres.cpu().numpy()
        out[name] = {"ms": qms, "rows": int(r[1]), "words": int(r[0])}
    del rows, qws, qrows, qwords
    torch.cuda.empty_cache()
    return out


def bench_append(args, lib, wah, torch, dev, stream, d_values, n, bound, bufs, K, L):
    """Incremental build: the index of the column's first R rows (R about
    3/4 of n, a multiple of 124 so both slices start 16-byte aligned) and the
    index of the remaining n - R rows, appended on the device (wah_append);
    the result is checked word for word against the whole-column build."""
    sh = stream.cuda_stream
    R = (3 * n // 4) // 124 * 124
    parts = []
    for start, rows in ((0, R), (R, n - R)):
        b = wah._Buffers(rows, bound, dev)
        rc = lib.wah_build(d_values.data_ptr() + 4 * start, rows, bound, b.keys.data_ptr(),
                           b.offsets.data_ptr(), b.index.data_ptr(), b.counts.data_ptr(),
                           b.ws.data_ptr(), b.ws_bytes, sh)
        assert rc == 0
        c = b.counts.cpu().numpy().view(np.uint32)
        assert c[3] == 0
        parts.append((b, int(c[0]), int(c[1])))
    (a, ka, la), (b, kb, lb) = parts
    kc, ic = ka + kb, la + lb + kb
    out_k = torch.empty(kc, dtype=torch.int32, device=dev)
    out_o = torch.empty(kc, dtype=torch.int32, device=dev)
    out_i = torch.empty(ic, dtype=torch.int32, device=dev)
    cnt = torch.zeros(4, dtype=torch.int32, device=dev)
    wsb = int(lib.wah_append_workspace_bytes(ka, kb))
    ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=dev)

    def app():
        rc = lib.wah_append(a.keys.data_ptr(), a.offsets.data_ptr(), a.index.data_ptr(), ka, la, R,
                            b.keys.data_ptr(), b.offsets.data_ptr(), b.index.data_ptr(), kb, lb,
                            out_k.data_ptr(), out_o.data_ptr(), out_i.data_ptr(), kc, ic,
                            cnt.data_ptr(), ws.data_ptr(), wsb, sh)
        assert rc == 0
    app()
    ms = time_events(app, max(3, args.steps // 5), torch, stream)
    c = cnt.cpu().numpy().view(np.uint32)
    assert c[3] == 0
    Ko, Lo = int(c[0]), int(c[1])
    exact = (Ko == K and Lo == L and torch.equal(out_k[:K], bufs.keys[:K])
             and torch.equal(out_o[:K], bufs.offsets[:K]) and torch.equal(out_i[:L], bufs.index[:L]))
    # algorithmic bytes: A's words walked once for every key's end chunk,
    # A's and B's words read and the merged words written, keys and offsets
    # of A and B read and of the result written
    alg = 4 * la + 4 * (la + lb) + 4 * Lo + 8 * (ka + kb) + 8 * Ko
    out = {"rows_a": R, "rows_b": n - R, "words_a": la, "words_b": lb, "words_out": Lo,
           "ms": ms, "appended_rows_per_s": (n - R) / (ms / 1e3),
           "alg_bytes": alg, "hbm_gbs": alg / (ms / 1e3) / 1e9,
           "equals_whole_build": bool(exact)}
    del a, b, parts, out_k, out_o, out_i, ws
    torch.cuda.empty_cache()
    return out


def bench_c1(args, lib, wah, torch, dev, stream):
    """The scope table's C1 column: 1,048,576 uint32 uniform [0, 65535]
    (seeded).  Device-resident build latency (CUDA events over repeated
    builds on the stream), and the same build through the host-buffer
    context API (values in from page-locked host memory, keys, offsets and
    index back to page-locked memory, wall clock per call)."""
    n = 1 << 20
    v = gen_uniform(n, 65536, args.seed + 1)
    d_v = torch.from_numpy(v.view(np.int32)).to(dev)
    b = wah._Buffers(n, 65535, dev)
    sh = stream.cuda_stream

    def build():
        rc = lib.wah_build(d_v.data_ptr(), n, 65535, b.keys.data_ptr(), b.offsets.data_ptr(),
                           b.index.data_ptr(), b.counts.data_ptr(), b.ws.data_ptr(), b.ws_bytes,
                           sh)
        assert rc == 0
    for _ in range(5):
        build()
    reps = 200
    ms = time_events(build, reps, torch, stream)
    c = b.counts.cpu().numpy().view(np.uint32)
    assert c[3] == 0
    kc, ic = wah.output_caps(n, 65535)
    pin = {name: torch.empty(size, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
           for name, size in (("v", n), ("k", kc), ("o", kc), ("i", ic))}
    pin["v"][:] = v
    with wah.HostContext(n, 65535) as ctx:
        for _ in range(5):
            ctx.build_into(pin["v"], pin["k"], pin["o"], pin["i"])
        t0 = time.perf_counter()
        for _ in range(50):
            cnt = ctx.build_into(pin["v"], pin["k"], pin["o"], pin["i"])
        host_ms = (time.perf_counter() - t0) * 1e3 / 50
    assert int(cnt.keycnt) == int(c[0]) and int(cnt.index_len) == int(c[1])
    return {"rows": n, "device_us": ms * 1e3, "device_rows_per_s": n / (ms / 1e3),
            "host_api_us": host_ms * 1e3, "host_api_rows_per_s": n / (host_ms / 1e3),
            "keycnt": int(c[0]), "index_len": int(c[1]), "merged": int(c[2])}


def bench_serving(args, wah, torch, dev):
    """C5: Poisson arrivals of index-build requests (one pinned host column
    each), rows log-uniform in [10,000, 16,777,216], values uniform [0,65535],
    Zipf s=1.1 over 65,536 or run-clustered (mean run 1,000), 1/3 each;
    64 GB device budget, results kept on the device.  Offered load: 80% of
    the batching server's capacity measured on a saturating prefix of the
    trace.  The continuous-batching server and the plain per-request server
    replay the same trace."""
    rng = np.random.default_rng(args.seed + 5)
    nreq = args.serve_requests
    max_rows = 16_777_216
    sizes = np.rint(np.exp(rng.uniform(np.log(10_000), np.log(max_rows), nreq))).astype(np.int64)
    kinds = rng.integers(0, 3, nreq)
    pools = []
    for kind in ("uniform", "zipf1.1", "runs1000"):
        v = gen_skewed(kind, max_rows, args.seed + 5, torch, dev) if kind != "uniform" else \
            torch.randint(0, 65536, (max_rows,), device=dev, dtype=torch.int32)
        h = torch.empty(max_rows, dtype=torch.int32, pin_memory=True)
        h.copy_(v)
        pools.append(h)
    del v
    torch.cuda.empty_cache()

    def run(plain, arrivals, count):
        srv = wah.Server(budget_bytes=args.serve_budget_gb << 30, max_batch=512, streams=3,
                         plain=plain)
        ids = [srv.submit(pools[int(kinds[i])][:int(sizes[i])], bound=65535,
                          delay=float(arrivals[i])) for i in range(count)]
        t0 = time.perf_counter()
        lat = np.empty(count)
        for i, rid in enumerate(ids):
            r = srv.wait(rid)
            lat[i] = r.latency_s
            srv.release(rid)
        wall = time.perf_counter() - t0
        srv.close()
        rows = int(sizes[:count].sum())
        return {"requests": count, "rows": rows, "wall_s": wall,
                "rows_per_s": rows / wall,
                "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "mean_ms": float(lat.mean() * 1e3)}

    # capacity: a saturating prefix, everything arriving at once
    cal = min(nreq, max(200, nreq // 10))
    cap = run(False, np.zeros(cal), cal)["rows_per_s"]
    rate = 0.8 * cap / float(sizes.mean())  # requests per second
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
    batched = run(False, arrivals, nreq)
    plain = run(True, arrivals, nreq)
    return {"requests": nreq, "offered_rows_per_s": 0.8 * cap, "capacity_rows_per_s": cap,
            "arrival_rate_per_s": rate, "budget_gb": args.serve_budget_gb,
            "batched": batched, "plain": plain,
            "rows_per_s_ratio": batched["rows_per_s"] / plain["rows_per_s"],
            "results_on_device": True}


def cpu_oracle_rate(values: np.ndarray, sample: int, threads: int, repeats: int):
    """Oracle builds of `threads` disjoint slices of `sample` rows, in parallel
    (ctypes releases the GIL).  Returns rows/s and the wall time."""
    from oracle import oracle as O
    O._load()
    slices = [values[(i * sample) % max(values.size - sample + 1, 1):][:sample]
              for i in range(threads)]
    t0 = time.perf_counter()
    for _ in range(repeats):
        ths = [threading.Thread(target=O.build, args=(s,)) for s in slices]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
    dt = time.perf_counter() - t0
    return threads * sample * repeats / dt, dt


def host_cpu():
    """nproc and the CPU model of this host (for the CPU baselines)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if model is None:
        import platform
        model = platform.processor() or platform.machine()
    return {"nproc": os.cpu_count(), "cpu_model": model}


def cpu_bubble_time(values: np.ndarray, n: int):
    """The reference `cpu` program as written sorts by bubble sort
    (src/cpu.cpp:180-197): the oracle's bubble-sort build of n rows, 1 thread,
    seconds (timed only at small n; it grows as n^2)."""
    from oracle import oracle as O
    O._load()
    v = np.ascontiguousarray(values[:n])
    t0 = time.perf_counter()
    O.build(v, sort_mode=O.SORT_BUBBLE)
    return time.perf_counter() - t0


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    O.make()
    n = args.n
    card = args.card
    values = gen_uniform(min(n, max(args.cpu_sample * 4, 1 << 22)), card, args.seed)
    threads = os.cpu_count() or 1
    sample = min(args.cpu_sample, values.size)
    for _ in range(max(args.warmup, 0)):
        cpu_oracle_rate(values, sample, threads, 1)
    times = []
    for _ in range(args.steps):
        r, dt = cpu_oracle_rate(values, sample, threads, 1)
        times.append(dt)
    total = sum(times)
    rate = threads * sample * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "rows/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"one column, {n} uint32 uniform [0,{card - 1}], seed "
                               f"{args.seed}", "rows": n, "bound": card - 1},
        "cpu_baseline": {"value": rate, "unit": "rows/s", "cores": threads, "kind": "port",
                         "sample": f"{threads} threads x one oracle build each of {sample} "
                                   f"rows (disjoint slices of the seeded column) per step",
                         "host": host_cpu()},
        "e2e": {"value": rate, "unit": "rows/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    import indexing_gb300 as wah
    from indexing_gb300 import _lib

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    lib = _lib.load()
    if args.sort_items:
        if lib.wah_set_tuning(args.sort_items) != 0:
            raise SystemExit(f"unsupported --sort-items {args.sort_items}")
    n, card = args.n, args.card
    bound = card - 1 if args.bound is None else args.bound
    tuned = None
    if not args.no_autotune and not args.sort_items:
        t, cached = wah.autotune(n, bound, args.tune_cache)
        tuned = {"tuning": t, "from_cache": cached}
    values_np = gen_uniform(n, card, args.seed + rank)
    d_values = torch.from_numpy(values_np.view(np.int32)).to(dev)
    bufs = wah._Buffers(n, bound, dev)
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream

    def step(events=None):
        if events is None:
            rc = lib.wah_build(d_values.data_ptr(), n, bound, bufs.keys.data_ptr(),
                               bufs.offsets.data_ptr(), bufs.index.data_ptr(),
                               bufs.counts.data_ptr(), bufs.ws.data_ptr(), bufs.ws_bytes, sh)
        else:
            rc = lib.wah_build_timed(d_values.data_ptr(), n, bound, bufs.keys.data_ptr(),
                                     bufs.offsets.data_ptr(), bufs.index.data_ptr(),
                                     bufs.counts.data_ptr(), bufs.ws.data_ptr(), bufs.ws_bytes,
                                     sh, events)
        if rc != 0:
            raise wah.WahError(rc, "wah_build")

    # Per-phase events for every timed step (recorded on the build's stream).
    n_ev = 2 * len(PHASES)
    ev_arrays = []
    for _ in range(args.steps):
        arr = (ctypes.c_void_p * n_ev)()
        if lib.wah_events_create(n_ev, arr) != 0:
            raise RuntimeError("event creation failed")
        ev_arrays.append(arr)

    with ClockSampler(local) as clocks:
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        launches = 0
        t_start.record(stream)
        for i in range(args.steps):
            step(ev_arrays[i])
            launches += wah.last_launch_count()
        t_end.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
    elapsed_ms = t_start.elapsed_time(t_end)
    c = bufs.counts.cpu().numpy().view(np.uint32)
    if c[3] != 0:
        raise wah.WahError(int(c[3]), "wah_build (device)")
    K, L, k = int(c[0]), int(c[1]), int(c[2])

    # per-phase mean durations over the timed steps
    phase_ms = {p: 0.0 for p in PHASES}
    f = ctypes.c_float()
    for arr in ev_arrays:
        for j, p in enumerate(PHASES):
            lib.wah_events_elapsed(arr[2 * j], arr[2 * j + 1], ctypes.byref(f))
            phase_ms[p] += f.value / args.steps
    for arr in ev_arrays:
        lib.wah_events_destroy(n_ev, arr)

    max_ms, value = replica_throughput(elapsed_ms, n, args.steps, dist, dev)
    ms_per_step = max_ms / args.steps

    # Algorithmic bytes per build: histogram 4n; digit pass 0 12n (read key,
    # write key + rid), later passes 16n -- with two passes the key between
    # them is 16-bit: pass 0 10n, pass 1 14n (2 + 4 in, 4 + 4 out); build
    # 8n + 4L + 8K (read sorted key + rid, write words, keys, offsets).  When
    # both digits of a two-pass column vary, key-start bits (one per row)
    # replace the sorted keys: pass 1 writes rids and the bits (10n + n/8)
    # and the build reads rids and bits (4n + n/8 + 4L + 8K).  A phase
    # (count + scan + kernel) and its main kernel are credited the same
    # bytes; the roofline is taken on the longest single kernel.
    passes = max(1, -(-(card - 1).bit_length() // 8))
    mid16 = passes == 2
    derive = mid16 and card > 256
    alg = {"histogram": 4 * n, "plan": 0,
           "build": (4 * n + n // 8 if derive else 8 * n) + 4 * L + 8 * K}
    alg["emit"] = alg["build"]
    for p in range(4):
        if p >= passes:
            a = 0
        elif mid16:
            a = 10 * n if p == 0 else (10 * n + n // 8 if derive else 14 * n)
        else:
            a = 12 * n if p == 0 else 16 * n
        alg[f"pass{p}"] = a
        alg[f"scatter{p}"] = a
    # DRAM bytes per row of each kernel (dram__bytes_read.sum +
    # dram__bytes_write.sum, one ncu capture of a 67,108,864-row uniform
    # 16-bit column with the same tile shape); traffic grows with rows.
    traffic_per_row = {"histogram": 4.05, "scatter0": 13.03, "scatter1": 11.05, "emit": 11.28}
    per_unit = {"histogram": "4 B/row",
                "scatter0": ("10 B/row (key in, 16-bit key + rid out)" if mid16
                             else "12 B/row (key in, key + rid out)"),
                "scatter1": ("10 B/row + 1 bit (16-bit key + rid in, rid out, key-start bit)"
                             if derive else
                             "14 B/row (16-bit key + rid in, key + rid out)" if mid16
                             else "16 B/row (key + rid in and out)"),
                "emit": ("4 B/row + 1 bit + 4 B/word + 8 B/key" if derive
                         else "8 B/row + 4 B/word + 8 B/key")}
    dom = max(KERNELS, key=lambda p: phase_ms[p])
    peak, peak_kind = load_peaks()
    ach = alg[dom] / (phase_ms[dom] / 1e3) / 1e9 if phase_ms[dom] > 0 else 0.0
    total_alg = sum(alg[p] for p in ("histogram", "pass0", "pass1", "pass2", "pass3", "build"))
    for p in PHASES:
        if rank == 0:
            gbs = alg[p] / (phase_ms[p] / 1e3) / 1e9 if phase_ms[p] > 0 and alg[p] else 0
            print(f"{p}:\t{phase_ms[p] * 1e3:.0f} us\t{gbs:.0f} GB/s", file=sys.stderr)

    # End to end: host values in, host index out, through the public
    # pipelined host-buffer API (wah_pipe_*): every step copies its column in
    # from pinned host memory and its keys/offsets/index out to pinned host
    # memory; consecutive steps overlap (depth builds in flight).  It runs
    # before the other legs, whose pinned host buffers stay cached by torch.
    e2e = None
    if not args.no_e2e:
        pin_v = torch.empty(n, dtype=torch.int32, pin_memory=True)
        pin_v.numpy()[:] = values_np.view(np.int32)
        pipe = wah.Pipeline(n, bound, depth=args.pipe_depth)
        e2e_steps = max(3, min(args.steps, 20))
        for _ in range(max(1, args.warmup)):
            pipe.result(pipe.submit(pin_v))
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        tickets = [pipe.submit(pin_v) for _ in range(e2e_steps)]
        for t in tickets[:-1]:
            pipe.wait(t)
        last = pipe.result(tickets[-1])
        dt = time.perf_counter() - t0
        if dist:
            t = torch.tensor([dt], device=dev, dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            dt = float(t.item())
        assert last.keycnt == K and last.index_len == L and last.merged == k
        e2e = {"value": world * n * e2e_steps / dt, "unit": "rows/s",
               "h2d_bytes_per_step": 4 * n,
               "d2h_bytes_per_step": 16 + 8 * K + 4 * L,
               "ms_per_step": 1e3 * dt / e2e_steps, "steps": e2e_steps,
               "pipeline_depth": args.pipe_depth}
        pipe.close()
        del pipe, pin_v

    decode = None if args.no_decode else bench_decode(args, lib, torch, dev, stream, bufs, n, K, L)
    append = (None if args.no_append else
              bench_append(args, lib, wah, torch, dev, stream, d_values, n, bound, bufs, K, L))
    ingest = None if args.no_ingest else bench_ingest(args, lib, torch, dev, stream, d_values, n)
    c1 = None if args.no_c1 else bench_c1(args, lib, wah, torch, dev, stream)

    skewed = None if args.no_skewed else bench_skewed(args, lib, wah, torch, dev, stream)
    batched = None if args.no_batched else bench_batched(args, lib, wah, torch, dev, stream)
    serving = None if args.no_serving else bench_serving(args, wah, torch, dev)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sample = min(args.cpu_sample, n)
        rate, dt = cpu_oracle_rate(values_np, sample, 1, 1)
        reps = max(1, min(5, int(10.0 / max(dt, 1e-3))))
        if reps > 1:
            rate, dt = cpu_oracle_rate(values_np, sample, 1, reps)
        nb = min(16384, n)
        tb = cpu_bubble_time(values_np, nb)
        cpu = {"value": rate, "unit": "rows/s", "cores": 1, "kind": "port",
               "sample": f"{reps} oracle build(s) of the first {sample} rows of the same "
                         f"column, 1 thread ({dt:.1f} s)",
               "host": host_cpu(),
               "bubble_sort_cpu": {"rows": nb, "seconds": tb,
                                   "extrapolated_seconds_at_n": tb * (n / nb) ** 2,
                                   "note": "the reference cpu program as written (O(n^2) "
                                           "bubble sort), 1 thread; n^2 extrapolation"}}

    if rank == 0:
        cl = clocks.summary()
        line = {
            "metric": METRIC, "value": value, "unit": "rows/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u32", "data": "synthetic",
            "config": {"workload": f"plain method, one column of {n} uint32 i.i.d. uniform "
                                   f"[0,{card - 1}] (seed {args.seed}+rank), bound {bound}",
                       "rows": n, "bound": bound, "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (1 GiB column), no flush"},
            "outputs": {"keycnt": K, "index_len": L, "merged": k},
            "sort_items": int(lib.wah_get_tuning()),
            "autotune": tuned,
            "hbm_gbs_pipeline": total_alg / (ms_per_step / 1e3) / 1e9,
            # whole-column figure on the scope table's formula (P = 2 digit
            # passes; the reference's k-sized intermediates included), and the
            # compulsory I/O (values in, index words, keys and offsets out)
            "column_roofline": {
                "formula": "40n + 24k + 4L + 8K",
                "alg_bytes": 40 * n + 24 * k + 4 * L + 8 * K,
                "achieved": (40 * n + 24 * k + 4 * L + 8 * K) / (ms_per_step / 1e3) / 1e9,
                "peak": peak, "unit": "GB/s",
                "frac": (40 * n + 24 * k + 4 * L + 8 * K) / (ms_per_step / 1e3) / 1e9 / peak,
                "compulsory_io_bytes": 4 * n + 4 * L + 8 * K,
                "compulsory_io_gbs": (4 * n + 4 * L + 8 * K) / (ms_per_step / 1e3) / 1e9},
            "phase_us": {p: round(phase_ms[p] * 1e3, 1) for p in PHASES},
            "roofline": {"bound": "hbm", "kernel": {"scatter0": "k_radix_scatter (pass 0)",
                                                    "scatter1": "k_radix_scatter (pass 1)",
                                                    "emit": "k_build_emit",
                                                    "histogram": "k_digit_histogram"}.get(dom, dom),
                         "per_unit": per_unit.get(dom),
                         "achieved": ach, "peak": peak, "unit": "GB/s",
                         "frac": ach / peak, "peak_kind": peak_kind,
                         "traffic": (traffic_per_row[dom] * n
                                     if card == 65536 and dom in traffic_per_row else None),
                         "traffic_source": "ncu capture at 67,108,864 rows, scaled by rows"},
            "gpu_launches": launches,
            "clocks": cl,
            "e2e": e2e,
            "skewed": skewed,
            "batched": batched,
            "serving": serving,
            "decode": decode,
            "append": append,
            "c1": c1,
            "ingest": ingest,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
