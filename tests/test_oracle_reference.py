"""The oracle against the reference's own code.

The reference's tree, list and basic deduplicators (src/{tree,list,basic}_approach.cpp)
are compiled from where they lie against the serial Kokkos stand-in in
oracle/kokkos_serial (oracle/build.py) where the reference is mounted.  Their
diffs must equal the oracle's byte for byte on seeded series, and their
restarts must equal the oracle's restarts.  This pins the byte order of the
incremental checkpoints, and the restart, to the reference code itself run
with serial Kokkos semantics.  The reference computes Murmur3 chunk digests
(its hash(), include/hash_functions.hpp:17-20).
"""
import json
import os

import numpy as np
import pytest

from mtcheck_gb300 import workloads

SHAPES = [  # (pattern, bytes, chunk size)
    (1, 1 << 18, 128),
    (2, (1 << 18) + 77, 64),   # ragged last chunk, leaf count not a power of two
    (2, 1 << 19, 512),
    (1, 3 * 64 * 1000, 64),
    (2, 64 * 1024 + 5, 24),
]


@pytest.fixture(scope="module")
def ref(oracle):
    if oracle.ref_dedup_lib() is None:
        pytest.skip("reference sources not mounted on this host")
    return oracle


def series(pattern, nbytes, cs, steps, seed):
    if pattern == 1:
        return [s.copy() for s in workloads.pattern1(nbytes, cs, steps, seed=seed)]
    z = (nbytes // 4, nbytes // 4 + nbytes // 8)
    return [s.copy() for s in workloads.pattern2(nbytes, cs, steps, seed=seed, zero_range=z)]


@pytest.mark.parametrize("approach", [2, 3, 4], ids=["basic", "list", "tree"])
@pytest.mark.parametrize("pattern,nbytes,cs", SHAPES)
def test_checkpoints_equal_the_reference_code(ref, approach, pattern, nbytes, cs):
    seq = series(pattern, nbytes, cs, 5, seed=nbytes % 991 + approach)
    r = ref.RefDeduplicator(approach, cs)
    o = ref.Deduplicator(approach, cs)
    diffs = []
    for i, s in enumerate(seq):
        want = r.checkpoint(s, i == 0)
        assert o.checkpoint(s, i == 0) == want, i
        diffs.append(want)
    # restart through the reference's restart_chkpt (its tree restart reads
    # out of bounds unless the chunk count is a power of two)
    n = (nbytes + cs - 1) // cs
    if approach == 4 and (n & (n - 1) or nbytes % cs):
        return
    for i in range(len(seq)):
        a = np.full(nbytes, 0x5A, np.uint8)
        assert ref.ref_restart(approach, cs, diffs, i, a) == 0
        b = np.full(nbytes, 0x5A, np.uint8)
        assert ref.restart(approach, diffs, i, b) == 0
        assert np.array_equal(a, b), i


def test_known_answers_through_the_reference_code(ref):
    # the ten tests of test/test_case_*.cpp, run on the reference code: the
    # header counts of the second checkpoint
    cases = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "tree_kat.json")))["cases"]
    for c in cases:
        r = ref.RefDeduplicator(4, c["chunk_size"])
        r.checkpoint(np.frombuffer(c["step0"].encode(), np.uint8), True)
        d = r.checkpoint(np.frombuffer(c["step1"].encode(), np.uint8), False)
        hdr = np.frombuffer(d[:32], np.uint32)
        assert (int(hdr[5]), int(hdr[7])) == (c["num_first_ocur"], c["num_shift_dupl"]), c["name"]


def test_reference_fixtures_are_current(ref):
    # the committed fixture (tests/golden/reference_series.npz) is what the
    # reference code gives today
    import importlib.util
    here = os.path.join(os.path.dirname(__file__), "golden")
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(here, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    fx = np.load(os.path.join(here, "reference_series.npz"))
    fresh = mg.reference_series()
    assert sorted(fx.files) == sorted(fresh)
    for k in fx.files:
        assert np.array_equal(fx[k], fresh[k]), k
