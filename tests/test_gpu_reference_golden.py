"""GPU checkpoints against diffs made by the reference's own code.

tests/golden/reference_series.npz holds a seeded series and the diffs that the
reference's basic, list and tree deduplicators (src/*_approach.cpp compiled
against a serial Kokkos stand-in, tests/golden/make_golden.py) wrote for it.
The GPU path must give the same bytes, without the oracle in between, and
restart every checkpoint of the list and basic chains to the original state.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(__file__), "golden", "reference_series.npz")


@pytest.mark.parametrize("approach,name", [(2, "basic"), (3, "list"), (4, "tree")])
def test_gpu_equals_reference_code(cuda, mtc, approach, name):
    fx = np.load(FIX)
    states = [fx["state%d" % i] for i in range(sum(1 for k in fx.files if k.startswith("state")))]
    cs = 64
    d = mtc.Deduplicator(cs, 0, approach=approach)
    diffs = []
    for i, s in enumerate(states):
        got = d.checkpoint(cuda.from_numpy(s).cuda(), i == 0)
        assert got == fx["%s_diff%d" % (name, i)].tobytes(), (name, i)
        diffs.append(got)
    if approach != 4:  # the leaf count is not a power of two: the tree restart loses chunks by design
        for i, s in enumerate(states):
            out = cuda.zeros(s.size, dtype=cuda.uint8, device="cuda")
            d.restart(out, diffs, i)
            assert np.array_equal(out.cpu().numpy(), s), (name, i)
    d.close()
