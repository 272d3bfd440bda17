"""The C-ABI library loads and exports every symbol include/wah/wah.h
declares; host-only entry points behave without a GPU."""
import ctypes
import os
import re

import pytest

from indexing_gb300 import _lib

HEADER = os.path.join(_lib.INCLUDE, "wah", "wah.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w\s\*]*?\b(wah_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        _lib.build()
    return _lib.load()


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("wah_build", "wah_workspace_bytes", "wah_strerror", "wah_sort_rids_by_value",
                 "wah_build_sorted", "wah_ctx_create", "wah_ctx_build_host",
                 "wah_ctx_destroy", "wah_output_caps"):
        assert must in names


def test_every_declared_symbol_is_exported(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"


def declared_parameter_counts():
    """Parameters of every function the header declares (void -> 0)."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(wah_\w+)\s*\(([^;]*?)\)\s*;", text,
                         flags=re.M | re.S):
        params = " ".join(m.group(2).split())
        out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_ctypes_signatures_match_the_header():
    """Every binding in the Python signature table takes as many arguments as
    the header declares, so a parameter added on one side only fails here
    on the CPU instead of corrupting a call on the GPU."""
    counts = declared_parameter_counts()
    assert set(counts) == set(declared_functions())
    for name, n in counts.items():
        argtypes = _lib.SIGNATURES[name][0]
        assert len(argtypes) == n, f"{name}: header {n} parameters, ctypes {len(argtypes)}"


def test_strerror(lib):
    assert lib.wah_strerror(0) == b"ok"
    assert b"range" in lib.wah_strerror(5)
    assert lib.wah_strerror(999) == b"unknown status"


def test_output_caps_and_workspace(lib):
    kc, ic = ctypes.c_uint64(), ctypes.c_uint64()
    lib.wah_output_caps(1000, 0, ctypes.byref(kc), ctypes.byref(ic))
    assert (kc.value, ic.value) == (1000, 2000)
    lib.wah_output_caps(1 << 20, 65535, ctypes.byref(kc), ctypes.byref(ic))
    assert (kc.value, ic.value) == (65536, 1 << 21)
    ws = lib.wah_workspace_bytes(1 << 20, 0)
    assert ws >= 16 * (1 << 20)  # four ping-pong columns
    assert lib.wah_workspace_bytes(1 << 20, 0) < lib.wah_workspace_bytes(1 << 21, 0)


def test_rejects_oversize_without_touching_device(lib):
    # n >= 2^31 is refused before any CUDA call
    rc = lib.wah_build(None, 1 << 31, 0, None, None, None, ctypes.c_void_p(16), None, 0, None)
    assert rc == 5


def test_tuning_encoding(lib):
    # host-only: the tile shape of digit pass 0 in the low 16 bits, that of
    # the later passes in the high 16 (0: the same); bad shapes are refused
    # and leave the tuning unchanged
    old = lib.wah_get_tuning()
    try:
        for good in (8, 12, 16, 16 | 0x100, 12 | 0x200, (16 | 0x200) | ((12 | 0x200) << 16),
                     8 | (16 << 16)):
            assert lib.wah_set_tuning(good) == 0, good
            assert lib.wah_get_tuning() == good
        cur = lib.wah_get_tuning()
        for bad in (0, 7, 20, 16 | 0x300, 16 | 0x800, 16 | (7 << 16), 16 | (0x200 << 16),
                    16 | ((12 | 0x300) << 16), -1):
            assert lib.wah_set_tuning(bad) == 1, bad  # WAH_EINVAL
            assert lib.wah_get_tuning() == cur
    finally:
        lib.wah_set_tuning(old)


def test_tuning_words_are_validated_on_the_host(lib):
    """Tuning words: rows per thread 8/12/16, one peer mode, the packed flag
    only in the first shape; a bad word is refused before any device work."""
    before = lib.wah_get_tuning()
    for bad in (0, -1, 7, 16 | 0x300, 16 | ((12 | 0x400) << 16), 16 | 0x800, 16 | (5 << 16)):
        assert lib.wah_set_tuning(bad) == 1, bad
        if bad != 0:  # 0 in a call means the process default
            assert lib.wah_build_tuned(None, 1000, 0, None, None, None, ctypes.c_void_p(16), None,
                                       0, bad, None) == 1, bad
    assert lib.wah_get_tuning() == before
    for good in (16, 12 | 0x100, 8 | 0x200 | 0x400, 16 | 0x200 | ((12 | 0x200) << 16)):
        assert lib.wah_set_tuning(good) == 0, good
    lib.wah_set_tuning(before)
