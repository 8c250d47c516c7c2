"""Per-rank file selection of the multi-rank driver (src/dedup_files_mpi.cpp:54-65):
the filter itself, a world_size-2 gloo run on the CPU (dry run: selection and
barriers, no GPU), and on the GPU the ranks' chains served on one device,
byte-identical to the oracle per rank."""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

from mtcheck_gb300 import ranks, workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_substring_filter():
    files = ["a/ckpt.Rank0.0", "a/ckpt.Rank1.0", "a/ckpt.Rank10.0", "a/other.0"]
    assert ranks.rank_files(files, 0) == ["a/ckpt.Rank0.0"]
    # the reference's substring test: Rank1 also selects Rank10
    assert ranks.rank_files(files, 1) == ["a/ckpt.Rank1.0", "a/ckpt.Rank10.0"]
    assert ranks.rank_files(files, 2) == []


def test_single_process_dry_run():
    files = ["x.Rank0.%d" % i for i in range(3)] + ["x.Rank1.%d" % i for i in range(3)]
    r = subprocess.run([sys.executable, "-m", "mtcheck_gb300.ranks", "128", "6", "--run-tree-chkpt", "--ranks",
                        "2", "--dry-run"] + files, capture_output=True, text=True, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    assert "rank 0: x.Rank0.0 x.Rank0.1 x.Rank0.2" in r.stdout and "rank 1: x.Rank1.0" in r.stdout


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_world_size_two_gloo_dry_run():
    files = ["y.Rank0.%d" % i for i in range(2)] + ["y.Rank1.%d" % i for i in range(2)]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), "-m", "mtcheck_gb300.ranks",
           "128", "4", "--run-list-chkpt", "--dry-run"] + files
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=ROOT, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "MPI COMM SIZE: 2, MPI_RANK: 0" in r.stdout and "MPI COMM SIZE: 2, MPI_RANK: 1" in r.stdout
    assert "rank 0: y.Rank0.0 y.Rank0.1" in r.stdout and "rank 1: y.Rank1.0 y.Rank1.1" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("flag,approach", [("--run-tree-chkpt", 4), ("--run-list-chkpt", 3),
                                           ("--run-basic-chkpt", 2)])
def test_ranks_served_on_one_gpu(mtc, oracle, tmp_path, flag, approach):
    files, seqs = [], []
    for r in range(3):
        seq = [s.copy() for s in workloads.pattern2((1 << 19) + 64 * r, 128, 4, seed=40 + r, run_max=64)]
        seqs.append(seq)
        for i, s in enumerate(seq):
            p = tmp_path / ("ckpt.Rank%d.%d.dat" % (r, i))
            p.write_bytes(s.tobytes())
            files.append(str(p))
    res = subprocess.run([sys.executable, "-m", "mtcheck_gb300.ranks", "128", str(len(files)), flag, "--ranks", "3"]
                         + files, capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    suffix = ranks.SUFFIX.get(approach, ".hashtree.incr_chkpt")
    for r in range(3):
        ref = oracle.Deduplicator(approach, 128, 0)
        for i, s in enumerate(seqs[r]):
            want = ref.checkpoint(s, i == 0)
            got = open(str(tmp_path / ("ckpt.Rank%d.%d.dat" % (r, i))) + suffix, "rb").read()
            assert got == want, (r, i)
