"""Incremental checkpoints from the GPU path are byte-identical to the oracle's
(header, metadata in serial push order, data) for every approach, both
digests, both update patterns, power-of-two and ragged sizes."""
import json
import os

import numpy as np
import pytest

from mtcheck_gb300 import workloads

pytestmark = pytest.mark.gpu

APPROACHES = {"full": 1, "basic": 2, "list": 3, "tree": 4, "tree-ref": 5}
KAT = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "tree_kat.json")))["cases"]


def series(pattern, nbytes, cs, steps, seed):
    if pattern == 1:
        return [s.copy() for s in workloads.pattern1(nbytes, cs, steps, seed=seed)]
    z = (nbytes // 4, nbytes // 4 + nbytes // 8)
    return [s.copy() for s in workloads.pattern2(nbytes, cs, steps, seed=seed, zero_range=z)]


def run_both(cuda, mtc, oracle, approach, kind, seq, cs):
    ref = oracle.Deduplicator(approach, cs, kind)
    gpu = mtc.Deduplicator(cs, kind, approach=approach)
    for i, s in enumerate(seq):
        want = ref.checkpoint(s, i == 0)
        got = gpu.checkpoint(cuda.from_numpy(s).cuda(), i == 0)
        assert len(got) == len(want), (i, len(got), len(want))
        if got != want:
            diff = np.nonzero(np.frombuffer(got, np.uint8) != np.frombuffer(want, np.uint8))[0]
            raise AssertionError("checkpoint %d differs at %d bytes, first %d" % (i, diff.size, diff[0]))
        if approach != 1:
            assert (gpu.num_first_ocur(), gpu.num_shift_dupl()) == (ref.num_first_ocur(), ref.num_shift_dupl())
            assert gpu.info().data_size == ref.datasizes()[0] and gpu.info().metadata_size == ref.datasizes()[1]
    return gpu


@pytest.mark.parametrize("approach", list(APPROACHES.values()), ids=list(APPROACHES))
@pytest.mark.parametrize("kind", [0, 1], ids=["murmur3", "md5"])
@pytest.mark.parametrize("pattern,nbytes,cs", [
    (1, 1 << 20, 128),          # 64 MiB / 128 B series, scaled down
    (2, 1 << 21, 512),          # 4 GiB / 512 B series, scaled down
    (2, (1 << 20) + 77, 256),   # ragged last chunk, non-power-of-two leaves
    (1, 3 * 64 * 1000, 64),
])
def test_series_matches_oracle(cuda, mtc, oracle, approach, kind, pattern, nbytes, cs):
    seq = series(pattern, nbytes, cs, 5, seed=nbytes % 1000 + pattern)
    run_both(cuda, mtc, oracle, approach, kind, seq, cs)


@pytest.mark.parametrize("cs", [1, 3, 24, 4096])
def test_odd_chunk_sizes(cuda, mtc, oracle, cs):
    seq = series(2, 64 * 1024 + 5, cs, 4, seed=cs)
    for approach in (2, 3, 4, 5):
        run_both(cuda, mtc, oracle, approach, 0, seq, cs)


@pytest.mark.parametrize("case", KAT, ids=[c["name"] for c in KAT])
def test_known_answer(cuda, mtc, case):
    gpu = mtc.TreeDeduplicator(case["chunk_size"])
    s0 = np.frombuffer(case["step0"].encode(), np.uint8).copy()
    s1 = np.frombuffer(case["step1"].encode(), np.uint8).copy()
    gpu.checkpoint(cuda.from_numpy(s0).cuda(), True)
    gpu.checkpoint(cuda.from_numpy(s1).cuda(), False)
    assert (gpu.num_first_ocur(), gpu.num_shift_dupl()) == (case["num_first_ocur"], case["num_shift_dupl"])


def test_heavy_duplication_and_zero_region(cuda, mtc, oracle):
    # many equal digests hit one map slot (the zero-filled range of the 4 GiB series)
    rng = np.random.default_rng(1)
    base = rng.integers(0, 256, 1 << 20, dtype=np.uint8)
    base[1 << 18: 3 << 18] = 0
    seq = [base.copy()]
    nxt = base.copy()
    nxt[:4096] = nxt[8192:12288]
    nxt[5 << 16:(5 << 16) + 2048] = 0
    seq.append(nxt)
    for approach in (3, 4, 5):
        run_both(cuda, mtc, oracle, approach, 0, seq, 128)


@pytest.mark.parametrize("kind", [0, 1], ids=["murmur3", "md5"])
@pytest.mark.parametrize("nbytes,cs", [(1 << 20, 128), ((1 << 20) + 300, 256)])
def test_new_content_repeated_in_one_checkpoint(cuda, mtc, oracle, kind, nbytes, cs):
    # Fresh bytes written at several places in one incremental checkpoint: the
    # later copies' leaves are demoted to shifted duplicates, and the aligned
    # copy's interior pairs hash to first-occurrence digests inserted by the
    # same checkpoint, so the duplicate pass has to follow the first-occurrence
    # pass.  The next checkpoint repeats no new content (one traversal), with
    # shifted duplicates of old content.
    rng = np.random.default_rng(nbytes + kind)
    s0 = rng.integers(0, 256, nbytes, dtype=np.uint8)
    s1 = s0.copy()
    run = 64 * cs
    fresh = rng.integers(0, 256, run, dtype=np.uint8)
    for at in (128 * cs, 1024 * cs, 2048 * cs + 5 * cs):
        s1[at:at + run] = fresh
    s2 = s1.copy()
    s2[512 * cs:512 * cs + run] = rng.integers(0, 256, run, dtype=np.uint8)
    s2[3000 * cs:3007 * cs] = s1[100 * cs:107 * cs]
    s2[3100 * cs:3164 * cs] = s1[1024 * cs:1088 * cs]
    for approach in (4, 5):
        run_both(cuda, mtc, oracle, approach, kind, [s0, s1, s2], cs)


def test_epochs_rebased_near_their_limit(cuda, mtc, oracle, monkeypatch):
    # launch epochs start just below the 26-bit epoch field of a map entry:
    # the map's entries go back to epoch 0 at the third checkpoint and every
    # diff stays equal to the oracle's
    monkeypatch.setenv("MTCHECK_EPOCH_START", str((1 << 26) - 8))
    seq = series(2, 1 << 20, 128, 6, seed=5)
    for approach in (3, 4):
        run_both(cuda, mtc, oracle, approach, 0, seq, 128)


@pytest.mark.parametrize("kind", [0, 1], ids=["murmur3", "md5"])
@pytest.mark.parametrize("approach", [3, 4], ids=["list", "tree"])
@pytest.mark.parametrize("issue", ["in_place", "alternating", "eager", "untimed"])
def test_graph_replay_matches_oracle(cuda, mtc, oracle, kind, approach, issue):
    # the single-call path replays a captured launch sequence: on the same
    # buffer rewritten in place, on two buffers taking turns (the sequence
    # retargeted to the other input), and issued eagerly
    nbytes, cs = (1 << 20) + 77, 256
    seq = series(2, nbytes, cs, 7, seed=11 + kind)
    ref = oracle.Deduplicator(approach, cs, kind)
    gpu = mtc.Deduplicator(cs, kind, approach=approach)
    if issue == "eager":
        gpu.set_tuning(eager=1)
    if issue == "untimed":
        gpu.set_tuning(untimed=1)
    bufs = [cuda.empty(nbytes, dtype=cuda.uint8, device="cuda") for _ in range(2)]
    for i, s in enumerate(seq):
        buf = bufs[i % 2] if issue in ("alternating", "untimed") else bufs[0]
        buf.copy_(cuda.from_numpy(s))
        assert gpu.checkpoint(buf, i == 0) == ref.checkpoint(s, i == 0), (issue, i)
        if issue == "untimed" and i > 0:
            # one graph without the phase events: no phase times
            assert list(gpu.info().phase_times) == [0.0, 0.0, 0.0]
    assert gpu.tuning()["eager"] == (1 if issue == "eager" else 0)
    assert gpu.tuning()["untimed"] == (1 if issue == "untimed" else 0)
    gpu.close()


def test_same_id_header_overload(cuda, mtc, oracle):
    # checkpoint(header_t&, ...) does not advance current_id
    seq = series(1, 1 << 18, 128, 3, seed=2)
    ref = oracle.Deduplicator(4, 128)
    gpu = mtc.TreeDeduplicator(128)
    for i, s in enumerate(seq):
        want = ref.checkpoint(s, i == 0, increment=False)
        got = gpu.checkpoint(cuda.from_numpy(s).cuda(), i == 0, advance=False)
        assert got == want


def test_length_change_requires_baseline(cuda, mtc):
    gpu = mtc.TreeDeduplicator(128)
    gpu.checkpoint(cuda.zeros(1 << 16, dtype=cuda.uint8, device="cuda"), True)
    with pytest.raises(mtc.MtcError) as e:
        gpu.checkpoint(cuda.zeros(1 << 15, dtype=cuda.uint8, device="cuda"), False)
    assert e.value.code == 1


def test_same_id_many_equal_chunks(cuda, mtc, oracle):
    # Header overload (the id is not advanced): a run of 2^20 chunks rewritten
    # to one content whose digest already has an entry of this id.  Every one
    # of them lowers that entry's node at once; the lowest chunk must win, as
    # the reference's atomic_min gives (src/tree_approach.cpp:337-339), and
    # the rest become shifted duplicates.
    cs, nbytes = 64, 1 << 27
    rng = np.random.default_rng(23)
    s0 = rng.integers(0, 256, nbytes, dtype=np.uint8)
    s0[-(1 << 22):] = 0
    s1 = s0.copy()
    s1[(1 << 20):(1 << 20) + (1 << 26)] = 0
    s2 = s1.copy()
    s2[:1 << 16] = 0
    s2[1 << 26:(1 << 26) + 4096] = rng.integers(0, 256, 4096, dtype=np.uint8)
    for approach in (4, 5):
        ref = oracle.Deduplicator(approach, cs)
        gpu = mtc.Deduplicator(cs, approach=approach)
        for i, s in enumerate((s0, s1, s2)):
            want = ref.checkpoint(s, i == 0, increment=False)
            got = gpu.checkpoint(cuda.from_numpy(s).cuda(), i == 0, advance=False)
            assert got == want, (approach, i)
        gpu.close()
