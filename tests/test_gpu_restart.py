"""Restart on the GPU against the oracle's restart of the same chain.

The output buffer starts with the same fill pattern on both sides, so chunks
that the reference never writes (the power-of-two defect of the tree
arithmetic, chunks outside the chain) are compared too."""
import os

import numpy as np
import pytest

from mtcheck_gb300 import workloads

pytestmark = pytest.mark.gpu
FILL = 0x5A


def series(pattern, nbytes, cs, steps, seed):
    if pattern == 1:
        return [s.copy() for s in workloads.pattern1(nbytes, cs, steps, seed=seed)]
    z = (nbytes // 4, nbytes // 4 + nbytes // 8)
    return [s.copy() for s in workloads.pattern2(nbytes, cs, steps, seed=seed, zero_range=z)]


def chain(cuda, mtc, approach, kind, seq, cs):
    gpu = mtc.Deduplicator(cs, kind, approach=approach)
    return gpu, [gpu.checkpoint(cuda.from_numpy(s).cuda(), i == 0) for i, s in enumerate(seq)]


def oracle_restart(oracle, approach, diffs, i, n):
    out = np.full(n, FILL, np.uint8)
    assert oracle.restart(approach, diffs, i, out) == 0
    return out


@pytest.mark.parametrize("approach", [1, 2, 3, 4, 5], ids=["full", "basic", "list", "tree", "tree-ref"])
@pytest.mark.parametrize("kind", [0, 1], ids=["murmur3", "md5"])
@pytest.mark.parametrize("pattern,nbytes,cs", [(1, 1 << 20, 128), (2, 1 << 21, 512), (2, (1 << 20) + 77, 256),
                                               (1, 3 * 64 * 1000, 64)])
def test_restart_matches_oracle(cuda, mtc, oracle, approach, kind, pattern, nbytes, cs):
    seq = series(pattern, nbytes, cs, 6, seed=nbytes % 997 + pattern)
    gpu, diffs = chain(cuda, mtc, approach, kind, seq, cs)
    pow2 = (nbytes // cs) & ((nbytes // cs) - 1) == 0 and nbytes % cs == 0
    for i in range(len(seq)):
        want = oracle_restart(oracle, approach, diffs, i, nbytes)
        out = cuda.full((nbytes,), FILL, dtype=cuda.uint8, device="cuda")
        gpu.restart(out, diffs, i)
        got = out.cpu().numpy()
        assert np.array_equal(got, want), (i, int(np.count_nonzero(got != want)))
        if approach in (1, 2, 3) or pow2:
            assert np.array_equal(got, seq[i])


def test_restart_device_resident_chain(cuda, mtc, oracle):
    seq = series(2, 1 << 21, 256, 8, seed=4)
    gpu = mtc.TreeDeduplicator(256)
    dev = []
    for i, s in enumerate(seq):
        gpu.checkpoint_device(cuda.from_numpy(s).cuda(), i == 0)
        p, n = gpu.diff_device()
        keep = cuda.empty(n, dtype=cuda.uint8, device="cuda")
        host = np.empty(n, np.uint8)
        gpu.copy_diff(host)
        keep.copy_(cuda.from_numpy(host))
        dev.append(keep)
    for i in (0, 3, 7):
        out = cuda.zeros(1 << 21, dtype=cuda.uint8, device="cuda")
        gpu.restart_device(out, [(t.data_ptr(), t.numel()) for t in dev], i)
        assert np.array_equal(out.cpu().numpy(), seq[i])


def test_restart_from_files_and_logs(cuda, mtc, tmp_path):
    seq = series(1, 1 << 19, 128, 4, seed=8)
    gpu = mtc.TreeDeduplicator(128)
    names = []
    for i, s in enumerate(seq):
        f = str(tmp_path / ("ckpt%d.hashtree.incr_chkpt" % i))
        gpu.checkpoint_file(cuda.from_numpy(s).cuda(), f, str(tmp_path / "log"), i == 0)
        names.append(f)
    assert gpu.current_id == 4
    out = cuda.zeros(1 << 19, dtype=cuda.uint8, device="cuda")
    gpu.restart_files(out, names, 3)
    assert np.array_equal(out.cpu().numpy(), seq[3])
    rows = open(str(tmp_path / "log") + ".chunk_size.128.csv").read().splitlines()
    assert rows[0].startswith("Approach,Chkpt ID,Chunk Size") and len(rows) == 5
    assert rows[1].split(",")[:4] == ["Tree", "0", "128", str(1 << 19)]
    size_rows = open(str(tmp_path / "log") + ".chunk_size.128.size.csv").read().splitlines()
    assert len(size_rows) == 4 and size_rows[0].startswith("Tree,0,128,")


def test_corrupt_checkpoints_are_rejected(cuda, mtc):
    seq = series(1, 1 << 18, 128, 3, seed=9)
    gpu, diffs = chain(cuda, mtc, 4, 0, seq, 128)
    out = cuda.zeros(1 << 18, dtype=cuda.uint8, device="cuda")
    # truncated inside the metadata
    bad = [diffs[0], diffs[1], diffs[2][:40]]
    with pytest.raises(mtc.MtcError) as e:
        gpu.restart(out, bad, 2)
    assert e.value.code in (1, 2)
    # wrong datalen
    with pytest.raises(mtc.MtcError) as e:
        gpu.restart(cuda.zeros(1000, dtype=cuda.uint8, device="cuda"), diffs, 2)
    assert e.value.code == 1
    # node id out of range in the first-occurrence list
    b = bytearray(diffs[1])
    if int.from_bytes(b[20:24], "little") > 0:
        b[32:36] = (0xFFFFFFF0).to_bytes(4, "little")
        with pytest.raises(mtc.MtcError) as e:
            gpu.restart(out, [diffs[0], bytes(b), diffs[2]], 1)
        assert e.value.code == 2
    # repeat table naming a later checkpoint
    b = bytearray(diffs[2])
    F, P = int.from_bytes(b[20:24], "little"), int.from_bytes(b[24:28], "little")
    if P:
        off = 32 + 4 * F
        b[off:off + 4] = (77).to_bytes(4, "little")
        with pytest.raises(mtc.MtcError) as e:
            gpu.restart(out, [diffs[0], diffs[1], bytes(b)], 2)
        assert e.value.code == 2
    # the handle keeps working after an error
    gpu.restart(out, diffs, 2)
    assert np.array_equal(out.cpu().numpy(), seq[2])


@pytest.mark.parametrize("approach", [3, 4], ids=["list", "tree"])
def test_long_chain_restart(cuda, mtc, oracle, approach):
    # 40 checkpoints: the per-key step masks of the chain span two words
    nbytes, cs = (1 << 17) + 77, 128
    seq = series(2, nbytes, cs, 40, seed=21)
    gpu, diffs = chain(cuda, mtc, approach, 0, seq, cs)
    for i in (39, 33, 32, 31, 5):
        want = oracle_restart(oracle, approach, diffs, i, nbytes)
        out = cuda.full((nbytes,), FILL, dtype=cuda.uint8, device="cuda")
        gpu.restart(out, diffs, i)
        assert np.array_equal(out.cpu().numpy(), want), i


def test_restart_handle_reused_across_chains(cuda, mtc, oracle):
    # one restarting handle alternates between chains of different lengths and
    # buffer sizes (its chain tables keep cells of earlier restarts; once they
    # are freed and allocated again), and writes into an output that is not
    # 16-byte aligned
    cs = 128
    sa, sb = series(2, 1 << 18, cs, 6, seed=31), series(1, (1 << 17) + 77, cs, 4, seed=32)
    _, da = chain(cuda, mtc, 4, 0, sa, cs)
    _, db = chain(cuda, mtc, 4, 0, sb, cs)
    r = mtc.TreeDeduplicator(cs)
    for seqs, diffs, i in ((sa, da, 5), (sb, db, 3), (sa, da, 2), (sb, db, 1), (sa, da, 5)):
        n = len(seqs[0])
        want = oracle_restart(oracle, 4, diffs, i, n)
        buf = cuda.full((n + 16,), FILL, dtype=cuda.uint8, device="cuda")
        for view in (buf[:n], buf[3:3 + n]):
            view.fill_(FILL)
            r.restart(view, diffs, i)
            assert np.array_equal(view.cpu().numpy(), want), (n, i, view.data_ptr() % 16)
        if i == 3:
            r.release_restart_buffers()


@pytest.mark.parametrize("cs", [3, 24, 4096])
def test_restart_odd_chunk_sizes(cuda, mtc, oracle, cs):
    # chunk sizes that are not multiples of 16 (byte-wise copy) and a large one
    nbytes = 64 * 1024 + 5
    seq = series(2, nbytes, cs, 4, seed=cs + 40)
    for approach in (2, 3, 4):
        gpu, diffs = chain(cuda, mtc, approach, 0, seq, cs)
        for i in range(len(seq)):
            want = oracle_restart(oracle, approach, diffs, i, nbytes)
            out = cuda.full((nbytes,), FILL, dtype=cuda.uint8, device="cuda")
            gpu.restart(out, diffs, i)
            assert np.array_equal(out.cpu().numpy(), want), (approach, i)
