"""Parity at the workloads' full sizes, byte for byte against the oracle.

* 64 MiB of seeded random bytes in 128 B chunks, Murmur3, 10 checkpoints
  (20% of the first state's chunks are copies of other chunks, then 1% of the
  chunks rewritten per step in runs of 1-32), for the tree approach, the tree
  with the serial reference labelling (include/reference_impl.hpp:16-132),
  the list and the basic approach, and a restart of every checkpoint;
* 4 GiB in 512 B chunks with Murmur3 and 1 GiB with MD5: a baseline and three
  incremental checkpoints of the scale-up update pattern (0.1-5% of the chunks
  change per step, half sparse, half in runs of up to 4096 chunks, a further
  10% shifted duplicates of earlier offsets, [1/4, 3/8) of the buffer zero);
* 4 GiB in 256 B chunks (2^24 chunks): the chunk compaction and the other
  scans over more than 2^23 entries take their three-launch form;
* the same three-launch forms, and the root compaction's, on small inputs
  through the MTCHECK_REDUCE_TILES hook.

The oracle runs on the host cores; the largest case takes about a minute.
"""
import numpy as np
import pytest

from mtcheck_gb300 import workloads

pytestmark = pytest.mark.gpu


def compare(got, want, what):
    if got == want:
        return
    g, w = np.frombuffer(got, np.uint8), np.frombuffer(want, np.uint8)
    n = min(g.size, w.size)
    bad = np.nonzero(g[:n] != w[:n])[0]
    raise AssertionError("%s differs: %d vs %d bytes, %d differ, first at %s" % (what, g.size, w.size, bad.size,
                                                                              bad[:1].tolist()))


@pytest.mark.parametrize("approach", [4, 5, 3, 2], ids=["tree", "tree-ref", "list", "basic"])
def test_64mib_128b_ten_checkpoints(cuda, mtc, oracle, approach):
    nbytes, cs = 64 << 20, 128
    seq = [s.copy() for s in workloads.pattern1(nbytes, cs, 10, seed=101)]
    ref = oracle.Deduplicator(approach, cs)
    gpu = mtc.Deduplicator(cs, approach=approach)
    diffs = []
    for i, s in enumerate(seq):
        want = ref.checkpoint(s, i == 0)
        compare(gpu.checkpoint(cuda.from_numpy(s).cuda(), i == 0), want, "checkpoint %d" % i)
        assert (gpu.num_first_ocur(), gpu.num_shift_dupl()) == (ref.num_first_ocur(), ref.num_shift_dupl())
        diffs.append(want)
    out = cuda.empty(nbytes, dtype=cuda.uint8, device="cuda")
    for i in range(len(seq)):
        out.fill_(0x5A)
        gpu.restart(out, diffs, i)
        assert np.array_equal(out.cpu().numpy(), seq[i]), "restart of checkpoint %d" % i
    gpu.close()


@pytest.mark.parametrize("nbytes,cs,kind,approach", [
    (4 << 30, 512, 0, 4),   # 4 GiB / 512 B, Murmur3, tree
    (1 << 30, 512, 1, 4),   # the same pattern with MD5 at 1 GiB
    (4 << 30, 256, 0, 3),   # 2^24 chunks, list
    (4 << 30, 256, 0, 4),   # 2^24 chunks, tree
], ids=["4GiB-512B-murmur3-tree", "1GiB-512B-md5-tree", "4GiB-256B-list", "4GiB-256B-tree"])
def test_scale_up_full_size(cuda, mtc, oracle, nbytes, cs, kind, approach):
    zero = (nbytes // 4, nbytes // 4 + nbytes // 8)
    rng = np.random.default_rng(nbytes // cs + kind)
    state = cuda.empty(nbytes, dtype=cuda.uint8, device="cuda")
    workloads.init_device(state, seed=7 + kind, zero_range=zero)
    ref = oracle.Deduplicator(approach, cs, kind)
    gpu = mtc.Deduplicator(cs, kind, approach=approach)
    diffs = []
    for i in range(4):
        if i:
            workloads.mutate_device(state, cs, float(rng.uniform(0.001, 0.05)), seed=1000 * i + kind,
                                    zero_range=zero)
        got = gpu.checkpoint(state, i == 0)
        host = state.cpu().numpy()
        compare(got, ref.checkpoint(host, i == 0), "checkpoint %d" % i)
        assert (gpu.num_first_ocur(), gpu.num_shift_dupl()) == (ref.num_first_ocur(), ref.num_shift_dupl())
        diffs.append(got)
        del host
    out = cuda.zeros(nbytes, dtype=cuda.uint8, device="cuda")
    gpu.restart(out, diffs, 3)
    assert bool(cuda.equal(out, state)), "restart of checkpoint 3"
    gpu.close()
    del out, state
    cuda.cuda.empty_cache()


@pytest.mark.parametrize("approach", [2, 3, 4, 5], ids=["basic", "list", "tree", "tree-ref"])
@pytest.mark.parametrize("kind", [0, 1], ids=["murmur3", "md5"])
def test_three_launch_scans_on_small_inputs(cuda, mtc, oracle, monkeypatch, approach, kind):
    # every scan of more than one tile, and the root compaction of more than
    # one tile (more than 32768 nodes), takes the three-launch form
    monkeypatch.setenv("MTCHECK_REDUCE_TILES", "1")
    nbytes, cs = (4 << 20) + 100, 64
    z = (nbytes // 4, nbytes // 4 + nbytes // 8)
    seq = [s.copy() for s in workloads.pattern2(nbytes, cs, 5, seed=55 + kind, zero_range=z)]
    ref = oracle.Deduplicator(approach, cs, kind)
    gpu = mtc.Deduplicator(cs, kind, approach=approach)
    diffs = []
    for i, s in enumerate(seq):
        want = ref.checkpoint(s, i == 0)
        compare(gpu.checkpoint(cuda.from_numpy(s).cuda(), i == 0), want, "checkpoint %d" % i)
        diffs.append(want)
    out = cuda.full((nbytes,), 0x5A, dtype=cuda.uint8, device="cuda")
    gpu.restart(out, diffs, len(seq) - 1)
    want = np.full(nbytes, 0x5A, np.uint8)
    assert oracle.restart(approach, diffs, len(seq) - 1, want) == 0
    assert np.array_equal(out.cpu().numpy(), want)
    gpu.close()
