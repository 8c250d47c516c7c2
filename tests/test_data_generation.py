"""The seven perturbation modes of the reference's data generator
(include/data_generation.hpp:13-95) as seeded series: each mode's rule, the
command line, and deduplication of every mode's series (oracle on the CPU,
the CUDA library against it on the GPU)."""
import os
import subprocess
import sys

import numpy as np
import pytest

from mtcheck_gb300 import data_generation as dg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def steps(mode, n=1 << 14, k=1000, count=3, seed=5):
    return [b.copy() for b in dg.series(n, count, mode, k, seed=seed)]


def test_random_and_beginning_identical():
    r = steps("R")
    assert np.count_nonzero(r[0] != r[1]) > 0.98 * r[0].size
    b = steps("B")
    assert np.array_equal(b[0][:1000], b[1][:1000]) and np.count_nonzero(b[0][1000:] != b[1][1000:]) > 0.98 * (b[0].size - 1000)


@pytest.mark.parametrize("mode", ["C", "Z"])
def test_contiguous_region(mode):
    s = steps(mode)
    d = np.nonzero(s[0] != s[1])[0]
    assert d.size > 0 and d[-1] - d[0] < 1000
    if mode == "Z":
        assert np.all(s[1][d] == 0)


def test_identical_and_sparse():
    i = steps("I")
    assert all(np.array_equal(i[0], x) for x in i)
    s = steps("S", k=500)
    changed = np.count_nonzero(s[0] != s[1])
    assert 400 < changed <= 500  # every drawn position changes; repeats change once


def test_swap():
    w = steps("W", n=1 << 14, k=256)
    a, b = w[0], w[1]
    moved = np.nonzero(a != b)[0]
    off = moved[moved >= 256][0] // 128 * 128
    assert off % 128 == 0 and off >= 256
    assert np.array_equal(b[:256], a[off:off + 256]) and np.array_equal(b[off:off + 256], a[:256])
    with pytest.raises(ValueError):
        list(dg.series(300, 2, "W", 256))


def test_command_line(tmp_path):
    r = subprocess.run([sys.executable, "-m", "mtcheck_gb300.data_generation", "4096", "3", "C", "100",
                        str(tmp_path / "gen")], capture_output=True, text=True, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    assert "Mode: C" in r.stdout and "Num changes: 100" in r.stdout
    for i in range(3):
        assert (tmp_path / ("gen.%d.chkpt" % i)).stat().st_size == 4096


@pytest.mark.parametrize("mode", list(dg.MODES))
def test_every_mode_round_trips_on_the_oracle(oracle, mode):
    n, cs = 1 << 15, 128  # power-of-two chunk count: the tree restart is exact
    seq = [b.copy() for b in dg.series(n, 4, mode, 1024, seed=7)]
    for approach in (2, 3, 4):
        d = oracle.Deduplicator(approach, cs, 0)
        diffs = [d.checkpoint(s, i == 0) for i, s in enumerate(seq)]
        out = np.zeros(n, np.uint8)
        assert oracle.restart(approach, diffs, 3, out) == 0
        assert np.array_equal(out, seq[3]), (mode, approach)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", list(dg.MODES))
def test_every_mode_on_the_gpu(cuda, mtc, oracle, mode):
    n, cs = (1 << 16) + 77, 64
    seq = [b.copy() for b in dg.series(n, 5, mode, 2048, seed=11)]
    for approach, kind in ((4, 0), (3, 1), (2, 0), (5, 1)):
        ref = oracle.Deduplicator(approach, cs, kind)
        gpu = mtc.Deduplicator(cs, kind, approach=approach)
        for i, s in enumerate(seq):
            assert gpu.checkpoint(cuda.from_numpy(s).cuda(), i == 0) == ref.checkpoint(s, i == 0), (mode, approach, i)
        gpu.close()


def test_repeated_copy_destinations_keep_the_last_source():
    # the update series copy chunks onto random destinations; a destination
    # drawn twice takes the later source, on numpy and torch buffers alike
    torch = pytest.importorskip("torch")
    from mtcheck_gb300.workloads import _copy_chunks
    cs, n = 4, 8
    base = np.arange(n * cs, dtype=np.uint8)
    dst, src = np.array([5, 2, 5, 5, 1]), np.array([0, 3, 1, 4, 6])
    want = base.copy().reshape(n, cs)
    want[2], want[1], want[5] = base.reshape(n, cs)[3], base.reshape(n, cs)[6], base.reshape(n, cs)[4]
    a = base.copy()
    _copy_chunks(a, cs, dst, src, n * cs, prev=base.copy())
    t = torch.from_numpy(base.copy())
    _copy_chunks(t, cs, dst, src, n * cs, prev=torch.from_numpy(base.copy()))
    assert np.array_equal(a.reshape(n, cs), want)
    assert np.array_equal(t.numpy().reshape(n, cs), want)
