"""Loader and build recipe for the native library ``libwah_gb300.so``.

The library holds the CUDA kernels and the C ABI declared in
``include/wah/wah.h``.  It is built in-tree by ``nvcc`` for sm_103a only; the
Python side never falls back to anything else: if the library is missing or
cannot be loaded, importing the functions that need it raises.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
OBJ_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libwah_gb300.so")

CUDA_SOURCES = ["wah_sort.cu", "wah_index.cu", "wah_api.cu", "wah_batch.cu", "wah_pipe.cu",
                "wah_serve.cu", "wah_noalloc.cu", "wah_query.cu", "wah_ingest.cu",
                "wah_tune.cu", "wah_append.cu"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo",
              "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def build(verbose: bool = False, force: bool = False, report=None) -> str:
    """Compile every CUDA source (in parallel) and link libwah_gb300.so.

    Without ``force`` an object newer than its source and every header is
    reused; ``force=True`` compiles every source and relinks whatever is on
    disk (a copied tree can carry objects built elsewhere).  ``report``, a
    list, receives the sources compiled and whether the library was linked.
    """
    os.makedirs(OBJ_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "wah", "wah.h"))
    newest_header = max(os.path.getmtime(h) for h in headers)

    def compile_one(src: str):
        obj = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
        path = os.path.join(CSRC, src)
        if (not force and os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(path)
                and os.path.getmtime(obj) >= newest_header):
            return obj, False
        cmd = [nvcc(), *NVCC_FLAGS, "-c", path, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        subprocess.run(cmd, check=True)
        return obj, True

    with ThreadPoolExecutor(max_workers=len(CUDA_SOURCES)) as ex:
        done = list(ex.map(compile_one, CUDA_SOURCES))
    objs = [o for o, _ in done]
    linked = (force or not os.path.exists(LIB_PATH)
              or any(os.path.getmtime(o) > os.path.getmtime(LIB_PATH) for o in objs))
    if linked:
        subprocess.run([nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-shared",
                        *objs, "-o", LIB_PATH], check=True)
    if report is not None:
        report.extend(src for src, (_, built) in zip(CUDA_SOURCES, done) if built)
        report.append(("linked", linked))
    return LIB_PATH


SPEEDREF_PATH = os.path.join(PKG_DIR, "libwah_speedref.so")


def build_speedref(force: bool = False) -> str:
    """Compile libwah_speedref.so: CUB's radix sort as an external speed
    reference for the benchmark (not part of the library's ABI)."""
    src = os.path.join(CSRC, "speedref_cub.cu")
    if (force or not os.path.exists(SPEEDREF_PATH)
            or os.path.getmtime(SPEEDREF_PATH) < os.path.getmtime(src)):
        subprocess.run([nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                        "-std=c++17", "-Xcompiler", "-fPIC", "-shared", src, "-o",
                        SPEEDREF_PATH], check=True)
    return SPEEDREF_PATH


HOST_DIR = os.path.join(PKG_DIR, "host")
BIN_DIR = os.path.join(PKG_DIR, "bin")
# host programs: (source, links libwah_gb300.so)
HOST_PROGRAMS = [("phases.cpp", True), ("gpu.cpp", True), ("overhead.cpp", True),
                 ("generate.cpp", False)]
CXX_FLAGS = ["-O2", "-std=c++17", "-pthread", "-Wall", "-Wextra", "-I" + INCLUDE]


def build_host(names=None, force: bool = False) -> dict:
    """Compile the C++ host programs into indexing_gb300/bin/ with g++.

    phases, gpu and overhead link libwah_gb300.so (found next to the package
    through an $ORIGIN rpath); generate needs no GPU library.  `names` limits
    the build to some programs (e.g. ["generate"]); ``force`` recompiles
    programs that look up to date.  Plain g++ without -march flags, so the
    same recipe builds on x86-64 and aarch64.
    """
    os.makedirs(BIN_DIR, exist_ok=True)
    headers = [os.path.join(HOST_DIR, f) for f in os.listdir(HOST_DIR) if f.endswith(".hpp")]
    headers.append(os.path.join(INCLUDE, "wah", "wah.h"))
    newest_header = max(os.path.getmtime(h) for h in headers)
    cxx = os.environ.get("CXX", "g++")

    def compile_one(item):
        src, link = item
        out = os.path.join(BIN_DIR, src[:-4])
        path = os.path.join(HOST_DIR, src)
        deps = [os.path.getmtime(path), newest_header]
        if link:
            deps.append(os.path.getmtime(LIB_PATH))
        if not force and os.path.exists(out) and all(os.path.getmtime(out) >= t for t in deps):
            return out
        cmd = [cxx, *CXX_FLAGS, path, "-o", out]
        if link:
            cmd += ["-L" + PKG_DIR, "-l:libwah_gb300.so", "-Wl,-rpath,$ORIGIN/.."]
        subprocess.run(cmd, check=True)
        return out

    todo = [p for p in HOST_PROGRAMS if names is None or p[0][:-4] in names]
    with ThreadPoolExecutor(max_workers=len(todo)) as ex:
        outs = list(ex.map(compile_one, todo))
    return {src[:-4]: out for (src, _), out in zip(todo, outs)}


def program(name: str) -> str:
    """Path of a built host program (raises if it has not been built)."""
    path = os.path.join(BIN_DIR, name)
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: run build_host()")
    return path


class wah_counts(ctypes.Structure):
    _fields_ = [("keycnt", ctypes.c_uint32), ("index_len", ctypes.c_uint32),
                ("merged", ctypes.c_uint32), ("status", ctypes.c_uint32)]


class wah_server_result(ctypes.Structure):
    _fields_ = [("counts", wah_counts), ("keys", ctypes.c_void_p), ("offsets", ctypes.c_void_p),
                ("index", ctypes.c_void_p), ("latency_s", ctypes.c_double),
                ("queue_s", ctypes.c_double)]


class wah_column(ctypes.Structure):
    _fields_ = [("values", ctypes.c_void_p), ("n", ctypes.c_uint64), ("bound", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("keys", ctypes.c_void_p),
                ("offsets", ctypes.c_void_p), ("index", ctypes.c_void_p),
                ("counts", ctypes.c_void_p)]


# Exported symbols and their signatures (must match include/wah/wah.h).
_vp = ctypes.c_void_p
_u64 = ctypes.c_uint64
_u32 = ctypes.c_uint32
SIGNATURES = {
    "wah_strerror": ([ctypes.c_int], ctypes.c_char_p),
    "wah_output_caps": ([_u64, _u32, ctypes.POINTER(_u64), ctypes.POINTER(_u64)], None),
    "wah_workspace_bytes": ([_u64, _u32], ctypes.c_size_t),
    "wah_build": ([_vp, _u64, _u32, _vp, _vp, _vp, _vp, _vp, ctypes.c_size_t, _vp],
                  ctypes.c_int),
    "wah_build_noalloc": ([_vp, _u64, _u32, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "wah_sort_rids_by_value": ([_vp, _u64, _u32, _vp, _vp, _vp, _vp, ctypes.c_size_t, _vp],
                               ctypes.c_int),
    "wah_build_sorted": ([_vp, _vp, _u64, _vp, _vp, _vp, _vp, _vp, ctypes.c_size_t, _vp],
                         ctypes.c_int),
    "wah_ctx_create": ([_u64, _u32, ctypes.POINTER(_vp)], ctypes.c_int),
    "wah_ctx_build_host": ([_vp, _vp, _u64, _vp, _vp, _vp, ctypes.POINTER(wah_counts)],
                           ctypes.c_int),
    "wah_ctx_destroy": ([_vp], None),
    "wah_batch_create": ([ctypes.POINTER(_u64), ctypes.POINTER(_u32), _u32,
                          ctypes.POINTER(_vp)], ctypes.c_int),
    "wah_batch_set_columns": ([_vp, _vp, _vp], ctypes.c_int),
    "wah_batch_build": ([_vp, _vp], ctypes.c_int),
    "wah_batch_launch_graph": ([_vp, _vp], ctypes.c_int),
    "wah_batch_device_bytes": ([_vp], ctypes.c_size_t),
    "wah_batch_ranges": ([_vp], _u32),
    "wah_batch_destroy": ([_vp], None),
    "wah_server_create": ([_u64, _u32, _u32, ctypes.c_int, ctypes.POINTER(_vp)], ctypes.c_int),
    "wah_server_submit": ([_vp, _vp, _u64, _u32, ctypes.c_double, ctypes.POINTER(_u64)],
                          ctypes.c_int),
    "wah_server_wait": ([_vp, _u64, ctypes.POINTER(wah_server_result)], ctypes.c_int),
    "wah_server_release": ([_vp, _u64], ctypes.c_int),
    "wah_server_arena_used": ([_vp], _u64),
    "wah_server_copy_out": ([_vp, _u64, _vp, _vp, _vp, _vp], ctypes.c_int),
    "wah_server_destroy": ([_vp], None),
    "wah_pipe_create": ([_u64, _u32, _u32, ctypes.POINTER(_vp)], ctypes.c_int),
    "wah_pipe_submit": ([_vp, _vp, _u64, _vp, _vp, _vp, _vp, ctypes.POINTER(_u64)],
                        ctypes.c_int),
    "wah_pipe_wait": ([_vp, _u64], ctypes.c_int),
    "wah_pipe_destroy": ([_vp], None),
    "wah_decode_workspace_bytes": ([], ctypes.c_size_t),
    "wah_decode": ([_vp, _vp, _vp, _u32, _u32, _u64, _vp, _vp, _vp, _vp, _vp, _vp,
                    ctypes.c_size_t, _vp], ctypes.c_int),
    "wah_query_workspace_bytes": ([_u64], ctypes.c_size_t),
    "wah_query": ([_vp, _vp, _vp, _u32, _u32, _u64, _u32, _u32, ctypes.c_int, _u32, _u32,
                   _vp, _u64, _vp, _u64, _vp, _vp, ctypes.c_size_t, _vp], ctypes.c_int),
    "wah_parse_workspace_bytes": ([], ctypes.c_size_t),
    "wah_parse_text": ([_vp, _u64, _vp, _u64, _vp, _vp, ctypes.c_size_t, _vp], ctypes.c_int),
    "wah_noop": ([_vp], ctypes.c_int),
    "wah_noop_graph_create": ([_u32, ctypes.POINTER(_vp)], ctypes.c_int),
    "wah_noop_graph_launch": ([_vp, _vp], ctypes.c_int),
    "wah_noop_graph_destroy": ([_vp], None),
    "wah_append_workspace_bytes": ([_u32, _u32], ctypes.c_size_t),
    "wah_append": ([_vp, _vp, _vp, _u32, _u32, _u64, _vp, _vp, _vp, _u32, _u32, _vp, _vp, _vp,
                    _u64, _u64, _vp, _vp, ctypes.c_size_t, _vp], ctypes.c_int),
    "wah_last_launch_count": ([], _u32),
    "wah_device_count": ([], ctypes.c_int),
    "wah_device_name": ([ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
    "wah_device_select": ([ctypes.c_int], ctypes.c_int),
    "wah_dev_alloc": ([ctypes.c_size_t, ctypes.POINTER(_vp)], ctypes.c_int),
    "wah_dev_free": ([_vp], None),
    "wah_host_alloc": ([ctypes.c_size_t, ctypes.POINTER(_vp)], ctypes.c_int),
    "wah_host_free": ([_vp], None),
    "wah_copy": ([_vp, _vp, ctypes.c_size_t, _vp], ctypes.c_int),
    "wah_stream_create": ([ctypes.POINTER(_vp)], ctypes.c_int),
    "wah_stream_sync": ([_vp], ctypes.c_int),
    "wah_stream_destroy": ([_vp], None),
    "wah_set_tuning": ([ctypes.c_int], ctypes.c_int),
    "wah_get_tuning": ([], ctypes.c_int),
    "wah_autotune": ([_u64, _u32, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int),
                      ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "wah_autotune_workload": ([ctypes.c_int, _u64, _u32, _u32, ctypes.c_char_p,
                               ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
                              ctypes.c_int),
    "wah_build_tuned": ([_vp, _u64, _u32, _vp, _vp, _vp, _vp, _vp, ctypes.c_size_t, ctypes.c_int,
                         _vp], ctypes.c_int),
    "wah_batch_create_tuned": ([ctypes.POINTER(_u64), ctypes.POINTER(_u32), _u32, ctypes.c_int,
                                ctypes.POINTER(_vp)], ctypes.c_int),
    "wah_server_create_tuned": ([_u64, _u32, _u32, ctypes.c_int, ctypes.c_int,
                                 ctypes.POINTER(_vp)], ctypes.c_int),
    "wah_events_create": ([_u32, ctypes.POINTER(_vp)], ctypes.c_int),
    "wah_events_destroy": ([_u32, ctypes.POINTER(_vp)], None),
    "wah_events_elapsed": ([_vp, _vp, ctypes.POINTER(ctypes.c_float)], ctypes.c_int),
    "wah_build_timed": ([_vp, _u64, _u32, _vp, _vp, _vp, _vp, _vp, ctypes.c_size_t, _vp,
                         ctypes.POINTER(_vp)], ctypes.c_int),
}

_lib = None


def load() -> ctypes.CDLL:
    """Load libwah_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
    return _lib
