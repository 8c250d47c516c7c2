"""The C ABI library loads on a host without a GPU and exports exactly the
entry points that include/mtcheck.h declares; the host-only helpers work."""
import ctypes
import os
import re

import numpy as np

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "mtcheck.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mtc_[a-z_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(mtc):
    lib = ctypes.CDLL(mtc.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(mtc.SIGNATURES), set(names) ^ set(mtc.SIGNATURES)


def test_host_digest_matches_oracle(mtc, oracle):
    rng = np.random.default_rng(9)
    for n in (0, 1, 15, 16, 17, 63, 64, 65, 1000, 4096, 100003):
        d = rng.integers(0, 256, n, dtype=np.uint8)
        assert mtc.digest_host(d, mtc.MURMUR3) == oracle.digest(d, oracle.MURMUR3)
        assert mtc.digest_host(d, mtc.MD5) == oracle.digest(d, oracle.MD5)


def test_digest_hex_format(mtc):
    s = mtc.digest_hex(bytes(range(16)))
    assert s == "00010203 04050607 08090A0B 0C0D0E0F "


def test_bad_arguments_fail_without_gpu(mtc):
    lib = mtc.load()
    h = ctypes.c_void_p()
    assert lib.mtc_create(99, 0, 128, ctypes.byref(h)) == 1
    assert lib.mtc_create(4, 7, 128, ctypes.byref(h)) == 1
    assert lib.mtc_create(4, 0, 0, ctypes.byref(h)) == 1
    assert b"chunk size" in lib.mtc_last_error()
    # NULL handles are refused before any CUDA call
    assert lib.mtc_release_restart_buffers(None) == 1
    assert b"NULL" in lib.mtc_last_error()
