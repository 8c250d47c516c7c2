"""The oracle's digest functions against the reference's own hash headers.

Golden vectors (tests/golden/hash_vectors.json) were produced by the
reference's include/kokkos_murmur3.hpp and include/kokkos_md5.hpp compiled on
the host (tests/golden/make_golden.py); where the reference is mounted the
compiled headers are also called directly on fresh random inputs.
"""
import hashlib
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "hash_vectors.json")


def test_oracle_matches_golden_vectors(oracle):
    vecs = json.load(open(GOLDEN))["vectors"]
    assert len(vecs) > 100
    for v in vecs:
        data = bytes.fromhex(v["data"])
        assert oracle.digest(data, oracle.MURMUR3).hex() == v["murmur3"], v["len"]
        assert oracle.digest(data, oracle.MD5).hex() == v["md5"], v["len"]


def test_md5_is_rfc1321_below_int_max(oracle):
    rng = np.random.default_rng(5)
    for n in (0, 1, 55, 56, 63, 64, 65, 127, 128, 1000):
        d = rng.integers(0, 256, n, dtype=np.uint8).tobytes()
        assert oracle.digest(d, oracle.MD5).hex() == hashlib.md5(d).hexdigest()


def test_murmur3_is_not_canonical(oracle):
    # the reference's rotl64 truncates to 32 bits, so a full 16-byte block
    # gives a different digest from canonical MurmurHash3_x64_128
    gold = {v["len"]: v for v in json.load(open(GOLDEN))["vectors"]}
    assert gold[16]["murmur3"] != gold[16]["md5"]


def test_oracle_matches_compiled_reference(oracle):
    ref = oracle.ref_lib()
    if ref is None:
        pytest.skip("reference sources not mounted on this host")
    import ctypes
    rng = np.random.default_rng(11)
    for n in list(range(0, 70)) + [511, 512, 4096, 12345]:
        d = rng.integers(0, 256, n, dtype=np.uint8)
        for kind, fn in ((oracle.MURMUR3, ref.ref_murmur3_hash), (oracle.MD5, ref.ref_md5_hash)):
            out = (ctypes.c_uint8 * 16)()
            fn(d.ctypes.data, n, out)
            assert oracle.digest(d, kind) == bytes(out)


def test_whole_buffer_digest_above_int_max(mtc, oracle):
    # calculate_digest_host over more than INT_MAX bytes: the reference's MD5
    # then feeds 128-byte pieces and cuts the last one to len % 128 bytes
    # (include/kokkos_md5.hpp:293-301).  The golden digests come from the
    # reference's own headers; the library's host digest (the restart check)
    # and the oracle must reproduce them.
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(os.path.dirname(GOLDEN),
                                                                              "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    vecs = json.load(open(os.path.join(os.path.dirname(GOLDEN), "long_hash_vectors.json")))["vectors"]
    assert [v["len"] for v in vecs] == mg.LONG_LENGTHS
    for v in vecs:
        data = mg.long_pattern(v["len"])
        assert mtc.digest_host(data, mtc.MD5).hex() == v["md5"], v["len"]
        assert oracle.digest(data, oracle.MD5).hex() == v["md5"], v["len"]
        assert mtc.digest_host(data, mtc.MURMUR3).hex() == v["murmur3"], v["len"]
        del data
