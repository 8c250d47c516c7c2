"""The reference's ten known-answer tests (test/test_case_01..10.cpp) on the oracle.

Each case checkpoints two 8-byte buffers with 1-byte chunks and checks the
number of first-occurrence and shifted-duplicate regions of the second
checkpoint, and that both checkpoints restart to their input.
"""
import json
import os

import numpy as np
import pytest

CASES = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "tree_kat.json")))["cases"]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
@pytest.mark.parametrize("approach", [4, 5], ids=["tree", "tree-low-offset-ref"])
def test_kat(oracle, case, approach):
    d = oracle.Deduplicator(approach, case["chunk_size"])
    s0 = np.frombuffer(case["step0"].encode(), np.uint8).copy()
    s1 = np.frombuffer(case["step1"].encode(), np.uint8).copy()
    diffs = [d.checkpoint(s0, True)]
    out = np.zeros(8, np.uint8)
    assert oracle.restart(approach, diffs, 0, out) == 0
    assert oracle.digest(out) == oracle.digest(s0)
    diffs.append(d.checkpoint(s1, False))
    assert (d.num_first_ocur(), d.num_shift_dupl()) == (case["num_first_ocur"], case["num_shift_dupl"])
    assert oracle.restart(approach, diffs, 1, out) == 0
    assert oracle.digest(out) == oracle.digest(s1)
