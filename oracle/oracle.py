"""ctypes bindings for the oracle (TEST INFRASTRUCTURE ONLY).

Two checkers live here:

* ``build``/``decoded_bitmap`` call ``liboracle.so``, the plain-C restatement
  of the reference's sequential ``cpu`` program (src/cpu.cpp:176-272, with the
  stable sort of src/phases.cpp:143-160).  It builds on any host with gcc.
* ``ref_build``/``ref_decoded_bitmap`` call ``_ref/libref_cpu.so``, the
  reference's own src/cpu.cpp compiled unmodified (see ``Makefile``); it exists
  only where the reference sources were available at build time.

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module; the product never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libref_cpu.so")
REFERENCE_ROOT = "/root/reference"

SORT_STABLE = 0
SORT_BUBBLE = 1

_u32p = ctypes.POINTER(ctypes.c_uint32)
_lib = None
_ref = None


def make(ref: bool = False) -> None:
    """Compile liboracle.so (and, with ref=True, the reference shim)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REFERENCE_ROOT}"],
                       check=True)


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            make()
        lib = ctypes.CDLL(LIB_PATH)
        lib.wah_oracle_build.argtypes = [
            _u32p, ctypes.c_size_t, ctypes.c_int, _u32p, _u32p, _u32p,
            ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t),
            ctypes.POINTER(ctypes.c_size_t)]
        lib.wah_oracle_build.restype = ctypes.c_int
        lib.wah_oracle_decoded_bitmap.argtypes = [
            _u32p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t]
        lib.wah_oracle_decoded_bitmap.restype = ctypes.c_size_t
        lib.wah_oracle_sort_rids_by_value.argtypes = [
            _u32p, _u32p, ctypes.c_size_t, ctypes.c_int]
        lib.wah_oracle_sort_rids_by_value.restype = ctypes.c_int
        _lib = lib
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_LIB_PATH)


def _load_ref():
    global _ref
    if _ref is None:
        if not ref_available():
            raise FileNotFoundError(
                f"{REF_LIB_PATH} not built (needs the reference sources: "
                "make -C oracle ref)")
        lib = ctypes.CDLL(REF_LIB_PATH)
        lib.ref_wah_build.argtypes = [
            _u32p, ctypes.c_uint64, ctypes.c_int, _u32p, _u32p, _u32p,
            ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
            ctypes.POINTER(ctypes.c_uint64)]
        lib.ref_wah_build.restype = ctypes.c_int
        lib.ref_decoded_bitmap.argtypes = [
            _u32p, ctypes.c_uint64, ctypes.c_char_p, ctypes.c_uint64]
        lib.ref_decoded_bitmap.restype = ctypes.c_uint64
        _ref = lib
    return _ref


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_u32p)


class Index:
    """(keys, offsets, index, merged) of one column, numpy uint32 arrays."""

    def __init__(self, keys, offsets, index, merged):
        self.keys = keys
        self.offsets = offsets
        self.index = index
        self.merged = merged

    def __eq__(self, other):
        return (np.array_equal(self.keys, other.keys)
                and np.array_equal(self.offsets, other.offsets)
                and np.array_equal(self.index, other.index))

    def bitmap(self, i: int) -> np.ndarray:
        """Words of the i-th key (offsets[i] .. offsets[i+1] or L)."""
        end = self.offsets[i + 1] if i + 1 < len(self.offsets) else len(self.index)
        return self.index[self.offsets[i]:end]


def build(values: np.ndarray, sort_mode: int = SORT_STABLE) -> Index:
    """The C restatement of the reference `cpu` pipeline."""
    lib = _load()
    v = np.ascontiguousarray(values, dtype=np.uint32)
    n = v.size
    keys = np.empty(max(n, 1), np.uint32)
    offs = np.empty(max(n, 1), np.uint32)
    index = np.empty(max(2 * n, 1), np.uint32)
    K, L, k = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
    rc = lib.wah_oracle_build(_ptr(v), n, sort_mode, _ptr(keys), _ptr(offs),
                              _ptr(index), ctypes.byref(K), ctypes.byref(L),
                              ctypes.byref(k))
    if rc != 0:
        raise MemoryError("oracle build failed")
    return Index(keys[:K.value].copy(), offs[:K.value].copy(),
                 index[:L.value].copy(), k.value)


def sort_rids_by_value(values: np.ndarray, sort_mode: int = SORT_STABLE):
    lib = _load()
    v = np.array(values, dtype=np.uint32, copy=True)
    rids = np.empty(v.size, np.uint32)
    if lib.wah_oracle_sort_rids_by_value(_ptr(v), _ptr(rids), v.size, sort_mode):
        raise MemoryError("oracle sort failed")
    return v, rids


def ref_build(values: np.ndarray, bubble: bool = False) -> Index:
    """The reference's own src/cpu.cpp functions (unmodified source)."""
    lib = _load_ref()
    v = np.ascontiguousarray(values, dtype=np.uint32)
    n = v.size
    keys = np.empty(max(n, 1), np.uint32)
    offs = np.empty(max(n, 1), np.uint32)
    index = np.empty(max(2 * n, 1), np.uint32)
    K, L, k = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
    rc = lib.ref_wah_build(_ptr(v), n, int(bubble), _ptr(keys), _ptr(offs),
                           _ptr(index), ctypes.byref(K), ctypes.byref(L),
                           ctypes.byref(k))
    if rc != 0:
        raise ValueError("reference build refused the input (n == 0)")
    return Index(keys[:K.value].copy(), offs[:K.value].copy(),
                 index[:L.value].copy(), k.value)


def _decode(fn, words: np.ndarray) -> str:
    w = np.ascontiguousarray(words, dtype=np.uint32)
    full = fn(_ptr(w), w.size, None, 0)
    buf = ctypes.create_string_buffer(int(full) + 1)
    fn(_ptr(w), w.size, buf, int(full) + 1)
    return buf.value.decode()


def decoded_bitmap(words: np.ndarray) -> str:
    return _decode(_load().wah_oracle_decoded_bitmap, words)


def ref_decoded_bitmap(words: np.ndarray) -> str:
    return _decode(_load_ref().ref_decoded_bitmap, words)
