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
    ap.add_argument("--no-link", action="store_true", help="skip the copy-only host-link leg")
    ap.add_argument("--no-cub", action="store_true", help="skip the CUB sort speed reference")
    ap.add_argument("--serve-requests", type=int, default=20000)
    ap.add_argument("--serve-budget-gb", type=int, default=64)
    ap.add_argument("--serve-verify", type=int, default=2000,
                    help="requests of the trace served again and checked against the same "
                         "request built alone (the GPU tests check all of them)")
    ap.add_argument("--pipe-depth", type=int, default=3,
                    help="builds in flight in the end-to-end leg")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the oracle checks of the C2, C3, C4 and C5 results (run after "
                         "every timed leg)")
    ap.add_argument("--sort-items", type=int, default=0,
                    help="radix scatter tuning: rows per thread | peer-mask flags, optionally "
                         "| (later passes' shape << 16) (0: library default)")
    ap.add_argument("--cpu-sample", type=int, default=1 << 23,
                    help="rows per oracle build in the CPU-baseline leg")
    ap.add_argument("--ref-sample", type=int, default=1 << 25,
                    help="rows per step of --impl reference (a slice of the same column)")
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


def build_bytes(n: int, card: int, L: int, K: int, tuning: int, sms: int):
    """Algorithmic bytes of each phase and main kernel of one index build of
    n rows with `card` possible values (the bound + 1), L index words and K
    keys, as the library runs it with tuning word `tuning` on `sms` SMs.
    Returns (bytes by phase/kernel name, digit passes, 16-bit keys between
    the passes, key-start mode, packed exchange).

    The packed exchange runs when a pass-0 range -- a whole number of tiles
    of 256 x items rows, SMs x resident scatter CTAs ranges -- holds 2^16 to
    2^24 rows (or the word forces it), as launch_sort_one decides."""
    passes = max(1, -(-(card - 1).bit_length() // 8))
    mid16 = passes == 2
    derive = mid16 and card > 256
    rows_in = 4 * n + n // 8 if derive else 8 * n
    alg = {"histogram": 4 * n, "plan": 0,
           "emit": rows_in + 4 * L + (4 * K if derive else 8 * K)}
    alg["build"] = alg["emit"] + rows_in  # the build count reads the same rows first
    items = tuning & 0xFF
    ranges = sms * {8: 4, 12: 3, 16: 2}.get(items, 2)
    quantum = 256 * max(items, 1)
    range_rows = max(-(-(-(-n // ranges)) // quantum) * quantum, quantum)
    packed = bool(derive and range_rows < (1 << 24)
                  and (range_rows >= (1 << 16) or tuning & 0x400))
    for p in range(4):
        if p >= passes:
            a = 0
        elif packed:
            a = 8 * n  # pass 0: key in, packed word out; pass 1: packed word in, rid out
        elif derive:
            a = 10 * n  # pass 0: key in, 16-bit key + rid out; pass 1: both in, rid out
        elif mid16:
            a = 10 * n if p == 0 else 14 * n
        else:
            a = 12 * n if p == 0 else 16 * n
        alg[f"pass{p}"] = a
        alg[f"scatter{p}"] = a
    if derive:
        alg["pass0"] += n // 8  # the range scan zeroes the key-start bits
        # the count over the pass-0 output; the key starts write the keys
        alg["pass1"] += (4 * n if packed else 2 * n) + 4 * K
    return alg, passes, mid16, derive, packed


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


def bench_skewed(args, lib, wah, torch, dev, stream, keep=None):
    """C3: skewed and clustered single columns of args.n rows, bound 65535.
    keep (a list) receives (kind, host values, host result) of each column
    for the oracle check after every timed leg."""
    out = {}
    tuning = 0
    if not args.no_autotune and not args.sort_items:
        # tile shapes timed on a synthetic skewed column of the same size
        tuning, cached = wah.autotune_workload(wah.WORKLOAD_SKEWED, args.n, 65535, 0,
                                               args.tune_cache)
        out["autotune"] = {"workload": "skewed", "tuning": tuning, "from_cache": cached}
    for kind in ("zipf1.1", "distinct16", "runs1000"):
        v = gen_skewed(kind, args.n, args.seed, torch, dev)
        bufs = wah._Buffers(args.n, 65535, dev)
        sh = stream.cuda_stream

        def step():
            rc = lib.wah_build_tuned(v.data_ptr(), args.n, 65535, bufs.keys.data_ptr(),
                                     bufs.offsets.data_ptr(), bufs.index.data_ptr(),
                                     bufs.counts.data_ptr(), bufs.ws.data_ptr(), bufs.ws_bytes,
                                     tuning, sh)
            assert rc == 0
        step()
        ms = time_events(step, max(3, args.steps // 5), torch, stream)
        c = bufs.counts.cpu().numpy().view(np.uint32)
        assert c[3] == 0
        out[kind] = {"rows_per_s": args.n / (ms / 1e3), "ms": ms, "keycnt": int(c[0]),
                     "index_len": int(c[1]), "merged": int(c[2])}
        if keep is not None:
            keep.append((kind, v.cpu().numpy().view(np.uint32),
                         result_numpy(bufs.keys, bufs.offsets, bufs.index, bufs.counts)))
        del v, bufs
        torch.cuda.empty_cache()
    return out


def _cpulist(ids) -> str:
    ids = sorted(ids)
    out, i = [], 0
    while i < len(ids):
        j = i
        while j + 1 < len(ids) and ids[j + 1] == ids[j] + 1:
            j += 1
        out.append(str(ids[i]) if i == j else f"{ids[i]}-{ids[j]}")
        i = j + 1
    return ",".join(out)


def numa_info(torch, dev, host_ptr=None) -> dict:
    """Where the GPU, this process's CPUs and a pinned host buffer sit
    (sysfs and /proc/self/numa_maps; best effort, None where unknown)."""
    import glob
    info = {"gpu_numa_node": None, "nodes": {}, "process_cpus": None, "buffer_pages_by_node": None}
    try:
        p = torch.cuda.get_device_properties(dev)
        bus = f"{p.pci_domain_id:04x}:{p.pci_bus_id:02x}:{p.pci_device_id:02x}.0"
        with open(f"/sys/bus/pci/devices/{bus}/numa_node") as f:
            info["gpu_numa_node"] = int(f.read())
        info["gpu_pci"] = bus
    except Exception:
        pass
    for d in sorted(glob.glob("/sys/devices/system/node/node[0-9]*")):
        node = int(d.rsplit("node", 1)[1])
        entry = {}
        try:
            with open(d + "/cpulist") as f:
                entry["cpus"] = f.read().strip()
            with open(d + "/meminfo") as f:
                for line in f:
                    if "MemTotal" in line:
                        entry["mem_gb"] = round(int(line.split()[-2]) / 2**20, 1)
        except OSError:
            pass
        info["nodes"][node] = entry
    try:
        info["process_cpus"] = _cpulist(os.sched_getaffinity(0))
    except Exception:
        pass
    if host_ptr:
        try:
            start = None
            with open("/proc/self/maps") as f:
                for line in f:
                    a, b = (int(x, 16) for x in line.split()[0].split("-"))
                    if a <= host_ptr < b:
                        start = a
                        break
            with open("/proc/self/numa_maps") as f:
                for line in f:
                    parts = line.split()
                    if start is not None and int(parts[0], 16) == start:
                        info["buffer_pages_by_node"] = {
                            x.split("=")[0]: int(x.split("=")[1]) for x in parts
                            if x.startswith("N") and "=" in x}
                        info["buffer_policy"] = parts[1]
        except Exception:
            pass
    return info


def bench_link(torch, dev, h2d_bytes: int, d2h_bytes: int, reps: int = 5):
    """Copy-only leg with the end-to-end step's bytes: pinned host ->
    device alone, device -> pinned host alone, and both at once on two
    streams (CUDA events); the last is the host-link floor of one step."""
    hb = torch.empty(max(h2d_bytes, d2h_bytes), dtype=torch.uint8, pin_memory=True)
    hb2 = torch.empty(d2h_bytes, dtype=torch.uint8, pin_memory=True)
    db = torch.empty(max(h2d_bytes, d2h_bytes), dtype=torch.uint8, device=dev)
    db2 = torch.empty(d2h_bytes, dtype=torch.uint8, device=dev)
    s1, s2 = torch.cuda.Stream(dev), torch.cuda.Stream(dev)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        cur = torch.cuda.current_stream(dev)
        a.record(cur)
        s1.wait_stream(cur)
        s2.wait_stream(cur)
        for _ in range(reps):
            fn()
        cur.wait_stream(s1)
        cur.wait_stream(s2)
        b.record(cur)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    def h2d():
        with torch.cuda.stream(s1):
            db[:h2d_bytes].copy_(hb[:h2d_bytes], non_blocking=True)

    def d2h():
        with torch.cuda.stream(s2):
            hb2.copy_(db2, non_blocking=True)

    def both():
        h2d()
        d2h()
    ms_h2d, ms_d2h, ms_both = timed(h2d), timed(d2h), timed(both)
    out = {"h2d_bytes": h2d_bytes, "d2h_bytes": d2h_bytes,
           "h2d_gbs": h2d_bytes / ms_h2d / 1e6, "d2h_gbs": d2h_bytes / ms_d2h / 1e6,
           "both_ms": ms_both, "both_gbs": (h2d_bytes + d2h_bytes) / ms_both / 1e6,
           "numa": numa_info(torch, dev, hb.data_ptr())}
    del hb, hb2, db, db2
    torch.cuda.empty_cache()
    return out


def bench_cub_sort(torch, dev, d_values, n: int, reps: int = 3):
    """External speed reference for the sort phase: CUB's DeviceRadixSort
    SortPairs of (value, row id) over the same column, (a) 32-bit keys
    sorted on bits [0, 16) and (b) the keys as 16-bit integers, all bits; two
    8-bit digit passes each (CUB's onesweep).  Event-timed, inputs resident."""
    import ctypes as C
    from indexing_gb300 import _lib
    if not os.path.exists(_lib.SPEEDREF_PATH):
        return None
    lib = C.CDLL(_lib.SPEEDREF_PATH)
    lib.speedref_sort_pairs_u32_bytes.restype = C.c_size_t
    lib.speedref_sort_pairs_u32_bytes.argtypes = [C.c_uint64]
    lib.speedref_sort_pairs_u16_bytes.restype = C.c_size_t
    lib.speedref_sort_pairs_u16_bytes.argtypes = [C.c_uint64]
    vp = C.c_void_p
    lib.speedref_sort_pairs_u32.argtypes = [vp, vp, vp, vp, C.c_uint64, C.c_int, C.c_int, vp,
                                            C.c_size_t, vp]
    lib.speedref_sort_pairs_u16.argtypes = [vp, vp, vp, vp, C.c_uint64, vp, C.c_size_t, vp]
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    rids = torch.arange(n, dtype=torch.int32, device=dev)
    vals_out = torch.empty(n, dtype=torch.int32, device=dev)
    out = {}
    tb = int(lib.speedref_sort_pairs_u32_bytes(n))
    temp = torch.empty(tb, dtype=torch.uint8, device=dev)
    keys_out = torch.empty(n, dtype=torch.int32, device=dev)

    def s32():
        assert lib.speedref_sort_pairs_u32(d_values.data_ptr(), keys_out.data_ptr(),
                                           rids.data_ptr(), vals_out.data_ptr(), n, 0, 16,
                                           temp.data_ptr(), tb, sh) == 0
    s32()
    out["u32_keys_bits_0_16_ms"] = time_events(s32, reps, torch, stream)
    same = bool(torch.equal(keys_out, torch.sort(d_values, stable=True)[0])) if n <= 1 << 28 else None
    del temp, keys_out
    k16 = d_values.to(torch.int16)
    k16_out = torch.empty_like(k16)
    tb = int(lib.speedref_sort_pairs_u16_bytes(n))
    temp = torch.empty(tb, dtype=torch.uint8, device=dev)

    def s16():
        assert lib.speedref_sort_pairs_u16(k16.data_ptr(), k16_out.data_ptr(), rids.data_ptr(),
                                           vals_out.data_ptr(), n, temp.data_ptr(), tb, sh) == 0
    s16()
    out["u16_keys_ms"] = time_events(s16, reps, torch, stream)
    out["sorted_keys_check"] = same
    del temp, k16, k16_out, rids, vals_out
    torch.cuda.empty_cache()
    return out


def gen_batched(ncols: int, seed: int, torch, dev):
    """C4 columns: rows log-uniform in [1,024, 4,194,304], cardinality
    log-uniform in [2, 65,536], values uniform within it (seeded, on the
    device).  Returns (sizes, cards, device columns)."""
    rng = np.random.default_rng(seed)
    sizes = np.rint(np.exp(rng.uniform(np.log(1024), np.log(4194304), ncols))).astype(np.int64)
    cards = np.rint(np.exp(rng.uniform(np.log(2), np.log(65536), ncols))).astype(np.int64)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    cols = [torch.randint(0, int(c), (int(n),), generator=g, device=dev, dtype=torch.int32)
            for n, c in zip(sizes, cards)]
    return sizes, cards, cols


def batch_tuning(args, wah, total_rows: int, ncols: int):
    """Tile shapes for batches of many uneven columns: timed on a synthetic
    mix of 512 columns with the same mean rows per column (the batch runs
    the shape of digit pass 0 for every pass)."""
    if args.no_autotune or args.sort_items:
        return None
    tcols = min(ncols, 512)
    t, cached = wah.autotune_workload(wah.WORKLOAD_BATCH, total_rows * tcols // ncols, 65535,
                                      tcols, args.tune_cache)
    return {"workload": f"batch of {tcols} columns", "tuning": t, "from_cache": cached}


def bench_batched(args, lib, wah, torch, dev, stream, verify=False):
    """C4: 4,096 columns, rows log-uniform in [1,024, 4,194,304], cardinality
    log-uniform in [2, 65,536], values uniform within it.  Batched (one
    launch sequence, replayed CUDA graph) against the plain path (one
    wah_build per column on the same stream)."""
    ncols = args.batch_cols
    sizes, cards, cols = gen_batched(ncols, args.seed + 4, torch, dev)
    bounds = [int(c) - 1 for c in cards]
    tuned = batch_tuning(args, wah, int(sizes.sum()), ncols)
    b = wah.Batch(sizes.tolist(), bounds, tuning=tuned["tuning"] if tuned else 0)
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
    parity = None
    if verify:
        # the batched build once more into the outputs (the plain path wrote
        # them last), then every column against the oracle
        b.launch_graph(stream)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bad, count = check_batched_columns(outs, cols, oracle_threads(4194304, 16))
        parity = {"columns_checked": count, "columns_differ": bad, "ok": not bad and count == ncols,
                  "seconds": time.perf_counter() - t0}
    b.close()
    del cols, outs, ws
    torch.cuda.empty_cache()
    return {"columns": ncols, "rows": total, "ranges": None,
            "rows_per_s_batched": total / (ms_batched / 1e3), "ms_batched": ms_batched,
            "rows_per_s_plain": total / (ms_plain / 1e3), "ms_plain": ms_plain,
            "speedup": ms_plain / ms_batched, "same_counts_as_plain": same, "parity": parity,
            "autotune": tuned}


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
    tuning, tuned = 0, None
    if not args.no_autotune and not args.sort_items:  # shapes of this size, per call
        tuning, cached = wah.autotune_workload(wah.WORKLOAD_UNIFORM, n, 65535, 0, args.tune_cache)
        tuned = {"workload": "uniform", "tuning": tuning, "from_cache": cached}

    def build():
        rc = lib.wah_build_tuned(d_v.data_ptr(), n, 65535, b.keys.data_ptr(),
                                 b.offsets.data_ptr(), b.index.data_ptr(), b.counts.data_ptr(),
                                 b.ws.data_ptr(), b.ws_bytes, tuning, sh)
        assert rc == 0
    for _ in range(5):
        build()
    reps = 200
    ms = time_events(build, reps, torch, stream)
    c = b.counts.cpu().numpy().view(np.uint32)
    assert c[3] == 0
    # the same build captured once into a CUDA graph and replayed (a caller
    # that rebuilds columns of one size in the same buffers)
    graph_ms = None
    try:
        g = torch.cuda.CUDAGraph()
        cs = torch.cuda.Stream(dev)
        with torch.cuda.graph(g, stream=cs, capture_error_mode="thread_local"):
            rc = lib.wah_build_tuned(d_v.data_ptr(), n, 65535, b.keys.data_ptr(),
                                     b.offsets.data_ptr(), b.index.data_ptr(),
                                     b.counts.data_ptr(), b.ws.data_ptr(), b.ws_bytes, tuning,
                                     cs.cuda_stream)
        assert rc == 0
        for _ in range(5):
            g.replay()
        graph_ms = time_events(g.replay, reps, torch, torch.cuda.current_stream(dev))
        cg = b.counts.cpu().numpy().view(np.uint32)
        assert cg[3] == 0 and int(cg[1]) == int(c[1])
    except Exception as ex:  # reported, not fatal: the stream figure stands
        graph_ms = f"graph capture failed: {ex}"
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
    return {"rows": n, "autotune": tuned, "device_us": ms * 1e3,
            "device_rows_per_s": n / (ms / 1e3),
            "graph_replay_us": graph_ms * 1e3 if isinstance(graph_ms, float) else graph_ms,
            "launches": int(lib.wah_last_launch_count()),
            "host_api_us": host_ms * 1e3, "host_api_rows_per_s": n / (host_ms / 1e3),
            "keycnt": int(c[0]), "index_len": int(c[1]), "merged": int(c[2])}


SERVE_MAX_ROWS = 16_777_216
SERVE_KINDS = ("uniform", "zipf1.1", "runs1000")


def gen_serving(nreq: int, seed: int, torch, dev):
    """C5 trace: per request, rows log-uniform in [10,000, 16,777,216] and
    one of three value distributions (uniform [0, 65535], Zipf s=1.1 over
    65,536, run-clustered with mean run 1,000), 1/3 each.  A request's column
    is the first rows of its distribution's 16,777,216-value pool (seeded).
    Returns (rng, sizes, kinds, pinned host pools, device pools); rng then
    draws the arrival gaps."""
    rng = np.random.default_rng(seed)
    sizes = np.rint(np.exp(rng.uniform(np.log(10_000), np.log(SERVE_MAX_ROWS),
                                       nreq))).astype(np.int64)
    kinds = rng.integers(0, 3, nreq)
    host, devp = [], []
    for kind in SERVE_KINDS:
        if kind == "uniform":
            g = torch.Generator(device=dev)
            g.manual_seed(seed)
            v = torch.randint(0, 65536, (SERVE_MAX_ROWS,), generator=g, device=dev,
                              dtype=torch.int32)
        else:
            v = gen_skewed(kind, SERVE_MAX_ROWS, seed, torch, dev)
        h = torch.empty(SERVE_MAX_ROWS, dtype=torch.int32, pin_memory=True)
        h.copy_(v)
        host.append(h)
        devp.append(v)
    return rng, sizes, kinds, host, devp


def serve_trace(wah, sizes, kinds, pools, arrivals, count, plain, budget_gb, on_result=None,
                tuning=0):
    """Replays the first `count` requests of a trace through a server
    (continuous batching, or plain per-request builds); on_result(i, rid,
    res, server), if given, sees every completed request before it is
    released."""
    srv = wah.Server(budget_bytes=budget_gb << 30, max_batch=512, streams=3, plain=plain,
                     tuning=tuning)
    ids = [srv.submit(pools[int(kinds[i])][:int(sizes[i])], bound=65535,
                      delay=float(arrivals[i])) for i in range(count)]
    t0 = time.perf_counter()
    lat = np.empty(count)
    for i, rid in enumerate(ids):
        r = srv.wait(rid)
        lat[i] = r.latency_s
        if on_result is not None:
            on_result(i, rid, r, srv)
        srv.release(rid)
    wall = time.perf_counter() - t0
    srv.close()
    rows = int(sizes[:count].sum())
    return {"requests": count, "rows": rows, "wall_s": wall, "rows_per_s": rows / wall,
            "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3)}


class _DeviceWords:
    """A device buffer of n 32-bit words seen by torch without a copy."""

    def __init__(self, ptr: int, n: int):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<i4", "data": (ptr, False),
                                         "version": 3, "strides": None}


def result_hash(torch, keys, offsets, index, K: int, L: int, k: int, mult):
    """64-bit fingerprint of one index (a 0-d int64 device tensor, nothing
    synchronised): every word times a fixed random odd multiplier of its
    position, summed in wrapping int64 arithmetic (exact and order-free), for
    index, keys and offsets, mixed with K, L and k."""
    def part(t, n, base):
        if n == 0:
            return torch.zeros((), dtype=torch.int64, device=mult.device)
        return (t[:n].to(torch.int64) * mult[base:base + n]).sum()
    return (part(index, L, 0) * 3 + part(keys, K, 7) * 5 + part(offsets, K, 13) * 7
            + (K * 11 + L * 13 + k * 17))


def hash_multipliers(torch, dev, n: int, seed: int):
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    return torch.randint(-2**62, 2**62, (n + 16,), generator=g, device=dev,
                         dtype=torch.int64) | 1


def verify_serving(lib, wah, torch, dev, sizes, kinds, pools, dpools, arrivals, count,
                   budget_gb, oracle_sample: int, seed: int, threads: int, tuning: int = 0):
    """Every request of the trace served again by the continuous-batching
    server and fingerprinted on the device as it completes (result_hash,
    before its release), then every request built alone with wah_build and
    fingerprinted the same way: the two must agree for every request.  A
    seeded sample of served results is also compared word for word with the
    oracle.  Returns the counts checked and the mismatches."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle as O
    O._load()
    kc, ic = wah.output_caps(SERVE_MAX_ROWS, 65535)
    mult = hash_multipliers(torch, dev, ic, seed)
    served_h = torch.zeros(count, dtype=torch.int64, device=dev)
    alone_h = torch.zeros(count, dtype=torch.int64, device=dev)
    status = np.zeros(count, dtype=np.int64)
    # the fingerprints run while the server's persistent batch kernels hold
    # the SMs: a high-priority stream gets them the next free slots
    stream = torch.cuda.Stream(dev, priority=-1)
    sh = stream.cuda_stream
    pick = set(np.random.default_rng(seed).choice(count, size=min(oracle_sample, count),
                                                  replace=False).tolist())
    jobs = []
    ex = ThreadPoolExecutor(max_workers=threads)

    def on_result(i, rid, res, srv):
        c = res.counts
        K, L, k = int(c.keycnt), int(c.index_len), int(c.merged)
        status[i] = c.status
        keys = torch.as_tensor(_DeviceWords(res.keys, K), device=dev) if K else None
        offs = torch.as_tensor(_DeviceWords(res.offsets, K), device=dev) if K else None
        index = torch.as_tensor(_DeviceWords(res.index, L), device=dev) if L else None
        with torch.cuda.stream(stream):
            served_h[i] = result_hash(torch, keys, offs, index, K, L, k, mult)
        if i in pick:
            got = (int(c.status), K, L, k,
                   *(np.empty(0, np.uint32) if t is None else t.cpu().numpy().view(np.uint32)
                     for t in (keys, offs, index)))
            n, kind = int(sizes[i]), int(kinds[i])
            jobs.append((i, ex.submit(same_as_oracle, pools[kind][:n].numpy().view(np.uint32),
                                      got)))
        stream.synchronize()  # the arena memory is reused once released

    serve_trace(wah, sizes, kinds, pools, arrivals, count, False, budget_gb, on_result,
                tuning=tuning)
    # every request alone, fingerprinted the same way
    alone = wah._Buffers(SERVE_MAX_ROWS, 65535, dev)
    for i in range(count):
        n, kind = int(sizes[i]), int(kinds[i])
        rc = lib.wah_build(dpools[kind].data_ptr(), n, 65535, alone.keys.data_ptr(),
                           alone.offsets.data_ptr(), alone.index.data_ptr(),
                           alone.counts.data_ptr(), alone.ws.data_ptr(), alone.ws_bytes, sh)
        assert rc == 0
        with torch.cuda.stream(stream):
            c = alone.counts.cpu().numpy().view(np.uint32)
            if c[3] != 0:
                alone_h[i] = -1
                continue
            alone_h[i] = result_hash(torch, alone.keys, alone.offsets, alone.index, int(c[0]),
                                     int(c[1]), int(c[2]), mult)
    torch.cuda.synchronize()
    same = (served_h == alone_h).cpu().numpy() & (status == 0)
    differ = np.flatnonzero(~same).tolist()
    oracle_bad = [i for i, f in jobs if not f.result()]
    ex.shutdown()
    del alone, served_h, alone_h, mult
    torch.cuda.empty_cache()
    return {"requests": count, "equal_alone": int(same.sum()), "differ_alone": differ[:20],
            "compare": "64-bit fingerprint of keys, offsets, index, K, L, k per request",
            "oracle_checked": len(jobs), "oracle_differ": oracle_bad,
            "ok": not differ and not oracle_bad}


def bench_serving(args, lib, wah, torch, dev, verify: bool):
    """C5: Poisson arrivals of index-build requests (one pinned host column
    each, the trace of gen_serving); 64 GB device budget, results kept on the
    device.  Offered load: 80% of the batching server's capacity measured on
    a saturating prefix of the trace.  The continuous-batching server and the
    plain per-request server replay the same trace; then (outside the timed
    replays) every request is served again and compared with itself built
    alone, and a sample with the oracle."""
    nreq = args.serve_requests
    rng, sizes, kinds, pools, dpools = gen_serving(nreq, args.seed + 5, torch, dev)
    torch.cuda.empty_cache()
    budget = args.serve_budget_gb
    # capacity: a saturating prefix, everything arriving at once
    cal = min(nreq, max(200, nreq // 10))
    tuned = batch_tuning(args, wah, int(sizes.sum()), nreq)
    t = tuned["tuning"] if tuned else 0
    cap = serve_trace(wah, sizes, kinds, pools, np.zeros(cal), cal, False, budget,
                      tuning=t)["rows_per_s"]
    rate = 0.8 * cap / float(sizes.mean())  # requests per second
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
    batched = serve_trace(wah, sizes, kinds, pools, arrivals, nreq, False, budget, tuning=t)
    plain = serve_trace(wah, sizes, kinds, pools, arrivals, nreq, True, budget)
    out = {"requests": nreq, "offered_rows_per_s": 0.8 * cap, "capacity_rows_per_s": cap,
           "arrival_rate_per_s": rate, "budget_gb": budget,
           "batched": batched, "plain": plain,
           "rows_per_s_ratio": batched["rows_per_s"] / plain["rows_per_s"],
           "results_on_device": True, "autotune": tuned}
    if verify:
        t0 = time.perf_counter()
        count = min(nreq, args.serve_verify)
        out["parity"] = verify_serving(lib, wah, torch, dev, sizes, kinds, pools, dpools,
                                       arrivals, count, budget, 64, args.seed + 55,
                                       oracle_threads(SERVE_MAX_ROWS, 16), tuning=t)
        out["parity"]["seconds"] = time.perf_counter() - t0
    del pools, dpools
    torch.cuda.empty_cache()
    return out


# ---------------------------------------------------------------------------
# Parity checks against the oracle, outside every timed region.  The oracle
# (the plain-C restatement of the reference `cpu` program) runs on host
# threads (ctypes releases the GIL); each column's GPU result is compared
# word for word: keys, offsets, index, and the merged-entry count.
# ---------------------------------------------------------------------------
def host_mem_available() -> int:
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


def oracle_threads(max_rows: int, want: int) -> int:
    """Concurrent oracle builds of up to max_rows rows that fit in host
    memory (about 56 bytes per row each, with the GPU result held beside it)."""
    avail = host_mem_available()
    fit = int(avail * 0.7 // max(56 * max_rows, 1)) if avail else 1
    return max(1, min(want, fit, os.cpu_count() or 1))


def result_numpy(keys, offsets, index, counts):
    """(status, K, L, k, keys[K], offsets[K], index[L]) of one device result."""
    c = counts.cpu().numpy().view(np.uint32)
    K, L = int(c[0]), int(c[1])
    return (int(c[3]), K, L, int(c[2]), keys[:K].cpu().numpy().view(np.uint32),
            offsets[:K].cpu().numpy().view(np.uint32), index[:L].cpu().numpy().view(np.uint32))


def same_as_oracle(values: np.ndarray, got) -> bool:
    """got = result_numpy(...); True when it equals the oracle's index of values."""
    from oracle import oracle as O
    status, K, L, k, keys, offs, index = got
    ref = O.build(values)
    return (status == 0 and k == ref.merged and np.array_equal(keys, ref.keys)
            and np.array_equal(offs, ref.offsets) and np.array_equal(index, ref.index))


def check_columns(jobs, threads: int):
    """jobs: iterable of (values numpy, got) pairs, or of callables returning
    one; oracle builds on `threads` host threads.  Returns the indexes of the
    columns that differ and the number checked."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle as O
    O._load()

    def one(job):
        v, got = job() if callable(job) else job
        return same_as_oracle(v, got)
    bad, count = [], 0
    with ThreadPoolExecutor(max_workers=threads) as ex:
        for i, ok in enumerate(ex.map(one, jobs)):
            count += 1
            if not ok:
                bad.append(i)
    return bad, count


def check_batched_columns(outs, cols, threads: int, group_rows: int = 1 << 28):
    """Every column of a batch against the oracle: inputs and outputs come to
    the host a group of columns at a time (bounded host memory)."""
    bad, count, i = [], 0, 0
    while i < len(cols):
        j, rows = i, 0
        while j < len(cols) and (j == i or rows + cols[j].numel() <= group_rows):
            rows += cols[j].numel()
            j += 1
        jobs = [(cols[c].cpu().numpy().view(np.uint32), result_numpy(*outs[c]))
                for c in range(i, j)]
        b, n = check_columns(jobs, threads)
        bad += [i + x for x in b]
        count += n
        i = j
    return bad, count


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


def workload_config(args, n: int, card: int, bound: int, world: int) -> dict:
    """The `config` of the default workload, the same on both arms."""
    return {"workload": f"plain method, one column of {n} uint32 i.i.d. uniform "
                        f"[0,{card - 1}] (seed {args.seed}+rank), bound {bound}",
            "rows": n, "bound": bound, "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (1 GiB column), no flush"}


def run_reference(args):
    """The reference's CPU implementation of the path on this host: the
    oracle port of the reference `cpu` program (its own sources do not
    travel to the GPU machine), which is sequential, so one thread.  Each step
    builds the index of a contiguous slice of --ref-sample rows of the same
    seeded column as the GPU arm (slices taken in turn), so that the whole
    run stays within a few minutes; rows/s = rows built / time.  A labelled
    extra figure runs one slice per host thread at once."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    O.make()
    O._load()
    n, card = args.n, args.card
    bound = card - 1 if args.bound is None else args.bound
    world = int(os.environ.get("WORLD_SIZE", "1"))
    values = gen_uniform(n, card, args.seed)
    sample = min(args.ref_sample, n)
    nslices = max(n // sample, 1)

    def one(step):
        lo = (step % nslices) * sample
        t0 = time.perf_counter()
        O.build(values[lo:lo + sample])
        return time.perf_counter() - t0
    for i in range(max(args.warmup, 0)):
        one(i)
    times = [one(args.warmup + i) for i in range(args.steps)]
    total = sum(times)
    rate = sample * args.steps / total
    threads = os.cpu_count() or 1
    par_rate, par_dt = cpu_oracle_rate(values, sample, threads, 1)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "rows/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": workload_config(args, n, card, bound, world),
        "cpu_baseline": {"value": rate, "unit": "rows/s", "cores": 1, "kind": "port",
                         "sample": f"per step one oracle build (1 thread, as the reference cpu "
                                   f"program runs) of a contiguous {sample}-row slice of the "
                                   f"seeded {n}-row column, slices in turn",
                         "host": host_cpu()},
        "e2e": {"value": rate, "unit": "rows/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "extra_all_threads": {"rows_per_s": par_rate, "threads": threads, "seconds": par_dt,
                              "note": f"{threads} oracle builds at once, each of its own "
                                      f"{sample}-row slice of the column (not the reference's "
                                      f"sequential program: a parallel upper bound for it)"},
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
    # them is 16-bit: pass 0 10n, pass 1 14n (2 + 4 in, 4 + 4 out); emit
    # 8n + 4L + 8K (read sorted key + rid, write words, keys, offsets), and
    # the build count before it reads the same 8n.  When both digits of a
    # two-pass column vary (key-start mode), pass 0 writes one packed word
    # per row (row offset in its range and high digit: 8n; the range scan
    # before it zeroes the n/8 bytes of key-start bits), the pass-1 count
    # reads those words (4n), the key starts write the keys (4K), pass 1
    # reads the words and writes row ids (8n), and the build count and the
    # emit each read row ids and bits (4n + n/8; the emit writes 4L + 4K).
    # Short pass-0 ranges keep the 16-bit exchange (10n per pass).  A phase
    # (count + scan + kernel) and its main kernel are credited the same
    # bytes, except the pass-1 count and the build count; the roofline is
    # taken on the longest single kernel.
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    alg, passes, mid16, derive, packed = build_bytes(n, card, L, K, int(lib.wah_get_tuning()),
                                                     sms)
    # DRAM bytes per row of each kernel (dram__bytes_read.sum +
    # dram__bytes_write.sum, one ncu capture of a 67,108,864-row uniform
    # 16-bit column with the same tile shape); traffic grows with rows.
    traffic_per_row = {"histogram": 4.05, "scatter0": 8.85, "scatter1": 8.87, "emit": 11.28}
    # DRAM bytes per row of each phase (every kernel of it), same capture
    phase_dram_per_row = {"histogram": 4.05, "pass0": 8.86, "pass1": 13.02, "build": 15.45}
    dram_bytes = (sum(phase_dram_per_row.values()) * n
                  if card == 65536 and packed else None)
    per_unit = {"histogram": "4 B/row",
                "scatter0": ("8 B/row (key in, packed row offset + high digit out)" if packed
                             else "10 B/row (key in, 16-bit key + rid out)" if mid16
                             else "12 B/row (key in, key + rid out)"),
                "scatter1": ("8 B/row (packed word in, rid out)" if packed
                             else "10 B/row (16-bit key + rid in, rid out)" if derive
                             else "14 B/row (16-bit key + rid in, key + rid out)" if mid16
                             else "16 B/row (key + rid in and out)"),
                "emit": ("4 B/row + 1 bit + 4 B/word + 4 B/key (offsets; the key starts "
                         "write the keys)" if derive
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

    link = None
    if not args.no_link:
        link = bench_link(torch, dev, 4 * n, 16 + 8 * K + 4 * L)
        if e2e is not None:
            e2e["link"] = {"h2d_gbs": link["h2d_gbs"], "d2h_gbs": link["d2h_gbs"],
                           "both_gbs": link["both_gbs"], "floor_ms": link["both_ms"],
                           "ms_over_floor": e2e["ms_per_step"] / link["both_ms"]}
    cub = None if args.no_cub else bench_cub_sort(torch, dev, d_values, n)
    if cub is not None:
        ours = sum(phase_ms[p] for p in ("histogram", "plan", "pass0", "pass1", "pass2", "pass3"))
        cub["ours_sort_phase_ms"] = ours
        cub["note"] = ("ours: histogram + digit passes of the index build (one packed word per "
                       "row between the passes where key-start mode packs, else 16-bit keys; row "
                       "ids and key-start bits out of the last); CUB: SortPairs of the column's "
                       "(value, row id)")
    decode = None if args.no_decode else bench_decode(args, lib, torch, dev, stream, bufs, n, K, L)
    append = (None if args.no_append else
              bench_append(args, lib, wah, torch, dev, stream, d_values, n, bound, bufs, K, L))
    ingest = None if args.no_ingest else bench_ingest(args, lib, torch, dev, stream, d_values, n)
    c1 = None if args.no_c1 else bench_c1(args, lib, wah, torch, dev, stream)

    verify = not args.no_parity and rank == 0
    c3_keep = [] if verify else None
    skewed = (None if args.no_skewed else
              bench_skewed(args, lib, wah, torch, dev, stream, c3_keep))
    batched = (None if args.no_batched else
               bench_batched(args, lib, wah, torch, dev, stream, verify))
    serving = (None if args.no_serving else
               bench_serving(args, lib, wah, torch, dev, not args.no_parity))

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

    # Oracle checks of the C2 column and the C3 columns (the C4 and C5 checks
    # ran inside their legs, after their timed parts); nothing here is timed.
    parity = None
    if verify:
        t0 = time.perf_counter()
        c2_got = result_numpy(bufs.keys, bufs.offsets, bufs.index, bufs.counts)
        jobs = [(values_np, c2_got)] + [(v, got) for _, v, got in (c3_keep or [])]
        names = ["c2"] + [f"c3_{kind}" for kind, _, _ in (c3_keep or [])]
        bad, _ = check_columns(jobs, oracle_threads(n, len(jobs)))
        parity = {name: i not in bad for i, name in enumerate(names)}
        if batched is not None and batched.get("parity"):
            bp = batched["parity"]
            parity["c4_columns_checked"] = bp["columns_checked"]
            parity["c4"] = bp["ok"]
        if serving is not None and serving.get("parity"):
            sp = serving["parity"]
            parity["c5_requests_checked"] = sp["requests"]
            parity["c5_requests_equal_alone"] = sp["equal_alone"]
            parity["c5_oracle_checked"] = sp["oracle_checked"]
            parity["c5"] = sp["ok"]
        parity["ok"] = all(v for k, v in parity.items() if isinstance(v, bool))
        parity["oracle"] = ("oracle/wah_oracle.c (plain-C restatement of the reference cpu "
                            "program, pinned to its golden vectors), host threads")
        parity["seconds"] = time.perf_counter() - t0
        del jobs, c2_got, c3_keep

    if rank == 0:
        cl = clocks.summary()
        line = {
            "metric": METRIC, "value": value, "unit": "rows/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u32", "data": "synthetic",
            "config": workload_config(args, n, card, bound, world),
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
                "compulsory_io_gbs": (4 * n + 4 * L + 8 * K) / (ms_per_step / 1e3) / 1e9,
                # what the DRAM actually moves: ncu's dram bytes per row of
                # every phase (a 67,108,864-row capture of the same column
                # and kernels) times n, over the same build time
                "dram_bytes": dram_bytes,
                "dram_bytes_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per row "
                                     "and phase at 67,108,864 rows, scaled by rows",
                "dram_gbs": (dram_bytes / (ms_per_step / 1e3) / 1e9 if dram_bytes else None),
                "dram_frac": (dram_bytes / (ms_per_step / 1e3) / 1e9 / peak
                              if dram_bytes else None)},
            "phase_us": {p: round(phase_ms[p] * 1e3, 1) for p in PHASES},
            "roofline": {"bound": "hbm", "kernel": {"scatter0": "k_radix_scatter (pass 0)",
                                                    "scatter1": "k_radix_scatter (pass 1)",
                                                    "emit": "k_build_emit",
                                                    "histogram": "k_digit_histogram"}.get(dom, dom),
                         "per_unit": per_unit.get(dom),
                         "achieved": ach, "peak": peak, "unit": "GB/s",
                         "frac": ach / peak, "peak_kind": peak_kind,
                         "traffic": (traffic_per_row[dom] * n
                                     if card == 65536 and packed and dom in traffic_per_row
                                     else None),
                         "traffic_source": "ncu capture at 67,108,864 rows (12-row tiles in "
                                           "both digit passes), scaled by rows"},
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
            "link": link,
            "cub_sort_reference": cub,
            "cpu_baseline": cpu,
            "parity": parity,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
