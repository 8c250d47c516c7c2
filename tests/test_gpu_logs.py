"""The CSV logs written beside each checkpoint file, column by column.

Every column but the timers is compared with the rows the reference's log
writers give for the oracle's checkpoints (restated in oracle.pyoracle.log_rows
from src/utils.cpp:38-124 and each approach's write_chkpt_log), for every
approach, over a series with shifted duplicates from several earlier
checkpoints and a second baseline in the middle.
"""
import csv
import os

import numpy as np
import pytest

from mtcheck_gb300 import workloads

pytestmark = pytest.mark.gpu


def rows(path):
    with open(path) as f:
        return [r for r in csv.reader(f)]


@pytest.mark.parametrize("approach", [1, 2, 3, 4, 5], ids=["full", "basic", "list", "tree", "tree-ref"])
def test_logs_match_the_reference_writers(cuda, mtc, oracle, tmp_path, approach):
    nbytes, cs = (1 << 20) + 77, 128
    z = (nbytes // 4, nbytes // 4 + nbytes // 8)
    seq = [s.copy() for s in workloads.pattern2(nbytes, cs, 7, seed=77, zero_range=z)]
    baselines = {0, 4}
    ref = oracle.Deduplicator(approach, cs)
    gpu = mtc.Deduplicator(cs, approach=approach)
    log = str(tmp_path / "run")
    want_csv, want_size, want_timing = [], [], []
    baseline_id = 0
    for i, s in enumerate(seq):
        diff = ref.checkpoint(s, i in baselines)
        if i in baselines:
            baseline_id = i
        f = str(tmp_path / ("c%d" % i))
        gpu.checkpoint_file(cuda.from_numpy(s).cuda(), f, log, i in baselines)
        assert open(f, "rb").read() == diff, i
        c, z_, t = oracle.log_rows(approach, cs, i, baseline_id, nbytes, ref.datasizes(), diff)
        want_csv.append(c)
        want_size.append(z_)
        want_timing.append(t)
    base = log + ".chunk_size.%d" % cs
    got_csv = rows(base + ".csv")
    assert got_csv[0] == ("Approach,Chkpt ID,Chunk Size,Uncompressed Size,Compressed Size,Data Size,Metadata Size,"
                          "Setup Time,Comparison Time,Gather Time,Write Time").split(",")
    assert len(got_csv) == len(seq) + 1
    for i, r in enumerate(got_csv[1:]):
        assert r[:7] == [str(v) for v in want_csv[i]], i
        assert len(r) == 11 and all(float(x) >= 0 for x in r[7:]), i
    got_size = rows(base + ".size.csv")
    assert [r for r in got_size] == [[str(v) for v in w] for w in want_size]
    got_timing = rows(base + ".timing.csv")
    assert len(got_timing) == len(seq)
    for i, r in enumerate(got_timing):
        assert r[:len(want_timing[i])] == [str(v) for v in want_timing[i]], i
        assert len(r) == 6
    gpu.close()
