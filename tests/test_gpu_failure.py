"""Failure detection on the GPU without a GPU fault.

Every device wait of the chunk-hashing pipeline is bounded.  A test hook makes
the pipeline's copy producer issue nothing, so the consumers' waits run out:
the call must come back with MTC_ETIMEOUT (no trap, no hang, no copy left in
flight), the GPU context must stay usable, and the same handle must go on.
Its next checkpoint is taken as a baseline (its digest state may have been
partly written by the failed launch), and it and every later checkpoint must
equal the oracle's, which makes a baseline at the same id.  The chain then
restarts byte for byte.
"""
import numpy as np
import pytest

from mtcheck_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("approach", [2, 3, 4, 5], ids=["basic", "list", "tree", "tree-ref"])
def test_bounded_wait_runs_out_and_handle_recovers(cuda, mtc, oracle, approach):
    nbytes, cs = 1 << 21, 512
    seq = [s.copy() for s in workloads.pattern2(nbytes, cs, 5, seed=17, zero_range=(nbytes // 4, nbytes // 2))]
    ref = oracle.Deduplicator(approach, cs)
    gpu = mtc.Deduplicator(cs, approach=approach)
    dev = [cuda.from_numpy(s).cuda() for s in seq]
    diffs = []
    for i in (0, 1):
        want = ref.checkpoint(seq[i], i == 0)
        assert gpu.checkpoint(dev[i], i == 0) == want
        diffs.append(want)
    gpu.inject_stall(1)
    with pytest.raises(mtc.MtcError) as e:
        gpu.checkpoint(dev[2], False)
    assert e.value.code == 4, str(e.value)           # MTC_ETIMEOUT
    assert gpu.current_id == 2                       # the failed call did not advance the id
    assert gpu.info().device_error & 2               # DERR_SPIN, read back by the host
    # the context is usable: an unrelated CUDA operation works
    assert int(cuda.arange(10, device="cuda").sum().item()) == 45
    # the same handle goes on; the retried checkpoint is a baseline
    for i in (2, 3, 4):
        want = ref.checkpoint(seq[i], i == 2)
        got = gpu.checkpoint(dev[i], False)
        assert got == want, i
        diffs.append(want)
    hdr = np.frombuffer(diffs[2][:8], np.uint32)
    assert tuple(hdr) == (2, 2)                      # ref_id = chkpt_id = 2: a baseline
    out = cuda.zeros(nbytes, dtype=cuda.uint8, device="cuda")
    gpu.restart(out, diffs, 4)
    assert np.array_equal(out.cpu().numpy(), seq[4])
    gpu.close()

