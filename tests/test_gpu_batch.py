"""Batched checkpoints (mtc_batch_*) and launch tuning give exactly the bytes of
lone handles: every member's diff, header counters and restart are those of a
deduplicator driven one call at a time on the same buffers, whether the step
ran eagerly or as a replayed CUDA graph, and whatever launch shape or map load
factor is set."""
import numpy as np
import pytest

from mtcheck_gb300 import workloads

pytestmark = pytest.mark.gpu

# (approach, hash, chunk size, bytes): uneven sizes, every chunk size of the
# batched workload, all approaches, both digests, ragged tails
MIX = [
    (4, 0, 64, (1 << 18) + 64 * 37),
    (4, 1, 128, 1 << 19),
    (4, 0, 512, (1 << 20) + 300),
    (4, 1, 4096, 3 << 20),
    (3, 0, 128, 700 * 1000),
    (2, 1, 512, 1 << 20),
    (5, 0, 64, 1 << 17),
    (1, 0, 4096, 1 << 18),
    (4, 0, 4096, 4096 * 5 + 17),
    (3, 1, 64, 3 * 64 * 1000),
]
STEPS = 5


def member_states(i, approach, kind, cs, nbytes):
    z = (nbytes // 4, nbytes // 4 + nbytes // 8)
    return [s.copy() for s in workloads.pattern2(nbytes, cs, STEPS, seed=100 + i, rate=(0.001, 0.1),
                                                 run_max=64, zero_range=z)]


@pytest.fixture(scope="module")
def states():
    return [member_states(i, *m[:3], m[3]) for i, m in enumerate(MIX)]


def lone_diffs(cuda, mtc, states):
    """Per-member diffs of lone handles: the one-buffer-per-call path."""
    out = []
    for (approach, kind, cs, nbytes), seq in zip(MIX, states):
        d = mtc.Deduplicator(cs, kind, approach=approach)
        out.append([d.checkpoint(cuda.from_numpy(s).cuda(), i == 0) for i, s in enumerate(seq)])
        d.close()
    return out


@pytest.fixture(scope="module")
def lone(cuda, mtc, states):
    return lone_diffs(cuda, mtc, states)


def member_diff(mtc, m):
    p, n = m.diff_device()
    host = np.empty(n, np.uint8)
    m.copy_diff(host)
    return host.tobytes()


@pytest.mark.parametrize("use_graph,leaf_launch", [(True, False), (True, True), (False, False)],
                         ids=["graph", "graph-one-leaf-launch", "eager"])
def test_batch_equals_lone_handles(cuda, mtc, states, lone, use_graph, leaf_launch, monkeypatch):
    # leaf_launch: every member's leaves in one persistent launch driven by a
    # device work queue (MTCHECK_BATCH_LEAF=1) instead of a leaf kernel per member
    monkeypatch.setenv("MTCHECK_BATCH_LEAF", "1" if leaf_launch else "0")
    b = mtc.Batch([m[:3] for m in MIX])
    b.set_options(use_graph=use_graph)
    bufs = [cuda.empty(m[3], dtype=cuda.uint8, device="cuda") for m in MIX]
    for step in range(STEPS):
        for buf, seq in zip(bufs, states):
            buf.copy_(cuda.from_numpy(seq[step]))
        sizes = b.checkpoint(bufs, make_baseline=(step == 0))
        info = b.info()
        assert info.last_used_graph == (1 if (use_graph and step > 0) else 0)
        # graph steps hash every member's leaves in one persistent launch
        # driven by a device work queue (all members but the full approach,
        # which has no leaves)
        if info.last_used_graph:
            assert info.batched_leaf_members == (sum(1 for m in MIX if m[0] != 1) if leaf_launch else 0)
        for i, m in enumerate(b.members):
            got = member_diff(mtc, m)
            assert sizes[i] == len(got)
            assert got == lone[i][step], "member %d step %d differs" % (i, step)
            assert m.current_id == step + 1
    if use_graph:
        info = b.info()
        assert info.graph_captures >= 1 and info.graph_nodes > 0 and info.kernels_per_step > 0
    b.close()


def test_graph_replayed_without_recapture(cuda, mtc, states, lone):
    # buffers written in place: after the first incremental step a member is
    # captured again only when its map grows
    b = mtc.Batch([m[:3] for m in MIX])
    bufs = [cuda.empty(m[3], dtype=cuda.uint8, device="cuda") for m in MIX]
    for step in range(STEPS):
        for buf, seq in zip(bufs, states):
            buf.copy_(cuda.from_numpy(seq[step]))
        b.checkpoint(bufs, make_baseline=(step == 0))
        if step == 1:
            first = b.info().graph_captures
            assert first == len(MIX)
    assert b.info().graph_captures <= first + len(MIX)
    b.close()


def test_graph_recaptured_when_buffers_move(cuda, mtc, states, lone):
    b = mtc.Batch([m[:3] for m in MIX])
    for step in range(STEPS):
        # fresh device buffers every step: the captured graph must be rebuilt
        bufs = [cuda.from_numpy(seq[step]).cuda() for seq in states]
        b.checkpoint(bufs, make_baseline=(step == 0))
        for i, m in enumerate(b.members):
            assert member_diff(mtc, m) == lone[i][step]
    # one graph per member, captured again at every step
    assert b.info().graph_captures == (STEPS - 1) * len(MIX)
    b.close()


FILL = 0x5A


def test_batch_member_restart(cuda, mtc, oracle, states):
    # a member restarts its chain like a lone handle: equal to the oracle's
    # restart, and to the original state wherever the reference round-trips
    # (every approach but the tree with a leaf count that is not a power of two)
    b = mtc.Batch([m[:3] for m in MIX])
    bufs = [cuda.empty(m[3], dtype=cuda.uint8, device="cuda") for m in MIX]
    chains = [[] for _ in MIX]
    for step in range(STEPS):
        for buf, seq in zip(bufs, states):
            buf.copy_(cuda.from_numpy(seq[step]))
        b.checkpoint(bufs, make_baseline=(step == 0))
        for i, m in enumerate(b.members):
            chains[i].append(member_diff(mtc, m))
    for i, (m, (approach, kind, cs, nbytes)) in enumerate(zip(b.members, MIX)):
        n = -(-nbytes // cs)
        exact = approach in (1, 2, 3) or (n & (n - 1) == 0 and nbytes % cs == 0)
        for target in (STEPS - 1, 2):
            want = np.full(nbytes, FILL, np.uint8)
            assert oracle.restart(approach, chains[i][:target + 1], target, want) == 0
            out = cuda.full((nbytes,), FILL, dtype=cuda.uint8, device="cuda")
            m.restart(out, chains[i][:target + 1], target)
            got = out.cpu().numpy()
            assert np.array_equal(got, want), (i, target)
            if exact:
                assert np.array_equal(got, states[i][target]), (i, target)
    b.close()


def test_member_handles_are_owned(cuda, mtc):
    b = mtc.Batch([(4, 0, 128), (3, 1, 512)])
    with pytest.raises(mtc.MtcError):
        mtc._check(mtc.load().mtc_destroy(b.members[0].h))
    with pytest.raises(mtc.MtcError):
        b.members[0].set_stream(0)
    b.close()


@pytest.mark.parametrize("tune", [
    dict(rows=128), dict(rows=256, ctas_per_sm=1), dict(rows=128, ctas_per_sm=4), dict(direct=1),
    dict(max_load=0.5), dict(max_load=0.9), dict(rows=128, ctas_per_sm=2, max_load=0.6), dict(eager=1),
    dict(direct=1, eager=1), dict(threads_per_chunk=32), dict(threads_per_chunk=32, eager=1),
])
def test_tuning_does_not_change_output(cuda, mtc, states, lone, tune):
    for i in (0, 1, 3, 4, 5, 6):
        approach, kind, cs, nbytes = MIX[i]
        d = mtc.Deduplicator(cs, kind, approach=approach)
        d.set_tuning(**tune)
        got = [d.checkpoint(cuda.from_numpy(s).cuda(), k == 0) for k, s in enumerate(states[i])]
        assert got == lone[i], (i, tune)
        d.close()


def test_autotune(cuda, mtc):
    t, best, dflt = mtc.autotune(4, 0, 512, 16 << 20)
    assert t["rows"] in (128, 256) and 0.1 < t["max_load"] <= 0.95
    assert 0 < best <= dflt
    # 4096 B chunks: the warp-per-chunk shape is among the candidates
    t, best, dflt = mtc.autotune(4, 1, 4096, 16 << 20)
    assert t["threads_per_chunk"] in (1, 32) and 0 < best <= dflt


@pytest.mark.parametrize("cs,nbytes", [(4096, (1 << 20) + 1000), (24, 64 * 1024 + 5), (1, 3000)])
@pytest.mark.parametrize("kind", [0, 1], ids=["murmur3", "md5"])
def test_warp_per_chunk_matches_oracle(cuda, mtc, oracle, cs, nbytes, kind):
    # one warp per chunk (coalesced loads, one lane hashing) gives the oracle's bytes
    seq = [s.copy() for s in workloads.pattern2(nbytes, cs, 4, seed=cs, zero_range=(nbytes // 4, nbytes // 2))]
    for approach in (2, 3, 4):
        ref = oracle.Deduplicator(approach, cs, kind)
        d = mtc.Deduplicator(cs, kind, approach=approach)
        d.set_tuning(threads_per_chunk=32)
        for i, s in enumerate(seq):
            assert d.checkpoint(cuda.from_numpy(s).cuda(), i == 0) == ref.checkpoint(s, i == 0), (approach, i)
        d.close()


def test_batch_autotune_keeps_output(cuda, mtc, states, lone):
    b = mtc.Batch([m[:3] for m in MIX])
    bufs = [cuda.empty(m[3], dtype=cuda.uint8, device="cuda") for m in MIX]
    b.autotune(bufs)
    for step in range(STEPS):
        for buf, seq in zip(bufs, states):
            buf.copy_(cuda.from_numpy(seq[step]))
        b.checkpoint(bufs, make_baseline=(step == 0))
        for i, m in enumerate(b.members):
            assert member_diff(mtc, m) == lone[i][step]
    b.close()


def test_batch_reserve_keeps_output(cuda, mtc, states, lone):
    # memory reserved for the members' state before the first step: the same
    # bytes, and at least the state of the largest member reserved
    b = mtc.Batch([m[:3] for m in MIX])
    bufs = [cuda.empty(m[3], dtype=cuda.uint8, device="cuda") for m in MIX]
    reserved = b.reserve(bufs)
    assert reserved > max(m[3] for m in MIX)
    for step in range(STEPS):
        for buf, seq in zip(bufs, states):
            buf.copy_(cuda.from_numpy(seq[step]))
        b.checkpoint(bufs, make_baseline=(step == 0))
        for i, m in enumerate(b.members):
            assert member_diff(mtc, m) == lone[i][step]
    b.close()


@pytest.mark.parametrize("kind", [0, 1], ids=["murmur3", "md5"])
@pytest.mark.parametrize("cs", [16, 32, 64, 128, 512])
@pytest.mark.parametrize("rows,ctas", [(128, 0), (128, 1), (128, 3), (256, 1), (256, 0)])
def test_leaf_shapes_persistent_loop(cuda, mtc, kind, cs, rows, ctas):
    # enough chunks that every CTA of the persistent grid loops over many tiles
    nbytes = cs * 152 * 4 * 256 * 3 + 5
    seq = [s.copy() for s in workloads.pattern2(nbytes, cs, 3, seed=cs + rows, rate=(0.01, 0.05), run_max=256)]
    base = mtc.TreeDeduplicator(cs, kind)
    want = [base.checkpoint(cuda.from_numpy(s).cuda(), i == 0) for i, s in enumerate(seq)]
    d = mtc.TreeDeduplicator(cs, kind)
    d.set_tuning(rows=rows, ctas_per_sm=ctas)
    got = [d.checkpoint(cuda.from_numpy(s).cuda(), i == 0) for i, s in enumerate(seq)]
    for i in range(len(seq)):
        assert got[i] == want[i], (i, len(got[i]), len(want[i]))


@pytest.mark.parametrize("kind", [1, 0], ids=["md5", "murmur3"])
@pytest.mark.parametrize("nbytes", [19340567, 64 * (152 * 3 * 128 * 5 + 77) + 23, 64 * 128 * 457])
@pytest.mark.parametrize("rows,ctas", [(128, 3), (128, 0), (256, 0)])
def test_leaf_shapes_ragged_tiles(cuda, mtc, kind, nbytes, rows, ctas):
    # partial last tile, uneven tiles per CTA: lone tuned handle vs default
    cs = 64
    rng = np.random.default_rng(nbytes % 1000)
    s0 = rng.integers(0, 256, nbytes, dtype=np.uint8)
    base = mtc.TreeDeduplicator(cs, kind)
    want = base.checkpoint(cuda.from_numpy(s0).cuda(), True)
    d = mtc.TreeDeduplicator(cs, kind)
    d.set_tuning(rows=rows, ctas_per_sm=ctas)
    got = d.checkpoint(cuda.from_numpy(s0).cuda(), True)
    assert len(got) == len(want) and got == want


@pytest.mark.parametrize("rows,ctas", [(128, 3), (256, 0)])
def test_leaf_shapes_concurrent_members(cuda, mtc, rows, ctas):
    # the same shape inside a batch, members overlapping on the device
    cs, nbytes = 64, 19340567
    rng = np.random.default_rng(7)
    bufs_h = [rng.integers(0, 256, nbytes + k * 4099, dtype=np.uint8) for k in range(4)]
    want = []
    for h in bufs_h:
        d = mtc.TreeDeduplicator(cs, 1)
        want.append(d.checkpoint(cuda.from_numpy(h).cuda(), True))
    b = mtc.Batch([(4, 1, cs)] * 4)
    for m in b.members:
        m.set_tuning(rows=rows, ctas_per_sm=ctas)
    bufs = [cuda.from_numpy(h).cuda() for h in bufs_h]
    b.checkpoint(bufs, make_baseline=True)
    for i, m in enumerate(b.members):
        assert member_diff(mtc, m) == want[i], i
