"""Oracle self-consistency: every approach restarts every checkpoint of a
chain to the original buffer (the property test/{tree,list,basic,full}_chkpt.cpp
check), on the two update patterns at small sizes."""
import numpy as np
import pytest

from mtcheck_gb300 import workloads


def states(pattern, nbytes, cs, steps, seed):
    if pattern == 1:
        g = workloads.pattern1(nbytes, cs, steps, seed=seed)
    else:
        g = workloads.pattern2(nbytes, cs, steps, seed=seed, zero_range=(nbytes // 4, nbytes // 4 + nbytes // 8))
    return [s.copy() for s in g]


@pytest.mark.parametrize("approach", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("pattern,nbytes,cs", [(1, 1 << 18, 128), (2, 1 << 19, 512), (2, (1 << 18), 64)])
@pytest.mark.parametrize("hash_kind", [0, 1])
def test_restart_roundtrip(oracle, approach, pattern, nbytes, cs, hash_kind):
    seq = states(pattern, nbytes, cs, 6, seed=7)
    d = oracle.Deduplicator(approach, cs, hash_kind)
    diffs = []
    for i, s in enumerate(seq):
        diffs.append(d.checkpoint(s, i == 0))
        out = np.zeros(nbytes, np.uint8)
        assert oracle.restart(approach, diffs, i, out) == 0
        assert np.array_equal(out, s), (approach, i)


def test_diff_layout_invariants(oracle):
    seq = states(2, 1 << 19, 256, 5, seed=3)
    d = oracle.Deduplicator(4, 256)
    for i, s in enumerate(seq):
        diff = d.checkpoint(s, i == 0)
        h = np.frombuffer(diff[:32], dtype=np.uint32)
        F, P, S = int(h[5]), int(h[6]), int(h[7])
        assert int(h[1]) == i and int(h[0]) == 0
        assert (F, S) == (d.num_first_ocur(), d.num_shift_dupl())
        # shift entries are sorted by source checkpoint (the repeat table order)
        table = np.frombuffer(diff[32 + 4 * F:32 + 4 * F + 8 * P], dtype=np.uint32).reshape(-1, 2)
        assert list(table[:, 0]) == sorted(table[:, 0])
        assert int(table[:, 1].sum()) == S


def test_non_power_of_two_tree_loses_chunks(oracle):
    # num_leaf_descendents/leftmost_leaf (include/kokkos_merkle_tree.hpp:102-142)
    # are exact only for a power-of-two leaf count: with 3 chunks the root
    # region covers chunks 1..2 and chunk 0 is never restored.
    data = np.arange(3 * 64, dtype=np.uint8)
    d = oracle.Deduplicator(4, 64)
    diff = d.checkpoint(data, True)
    out = np.zeros_like(data)
    assert oracle.restart(4, [diff], 0, out) == 0
    assert not np.array_equal(out, data)
    assert np.array_equal(out[64:], data[64:])
