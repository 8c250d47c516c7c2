"""The command-line drivers dedup_chkpt_files / restart_chkpt_files (the
reference's src/dedup_files.cpp and src/restart_chkpt_files.cpp): files,
logs and printed digests."""
import os
import subprocess

import numpy as np
import pytest

from mtcheck_gb300 import workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "mtcheck_gb300", "_build")
SUFFIX = {"--run-full-chkpt": ".full_chkpt", "--run-basic-chkpt": ".basic.incr_chkpt",
          "--run-list-chkpt": ".hashlist.incr_chkpt", "--run-tree-chkpt": ".hashtree.incr_chkpt"}
APPROACH = {"--run-full-chkpt": 1, "--run-basic-chkpt": 2, "--run-list-chkpt": 3, "--run-tree-chkpt": 4}
LABEL = {"--run-full-chkpt": "Full chkpt digest:", "--run-basic-chkpt": "Basic Hashlist digest:",
         "--run-list-chkpt": "Hashlist digest:", "--run-tree-chkpt": "Hashtree digest:"}


@pytest.fixture(scope="module")
def clis(mtc):
    for name in ("dedup_chkpt_files", "restart_chkpt_files"):
        assert os.access(os.path.join(BUILD, name), os.X_OK), name
    return BUILD


def run(clis, name, *args, cwd=None):
    return subprocess.run([os.path.join(clis, name)] + [str(a) for a in args], capture_output=True, text=True,
                          cwd=cwd, timeout=300)


def test_usage_and_bad_mode(clis):
    r = run(clis, "dedup_chkpt_files")
    assert r.returncode == 2 and "--run-tree-chkpt" in r.stdout
    r = run(clis, "dedup_chkpt_files", 128, 1, "--run-nothing", "x")
    assert r.returncode == 2 and "ERROR: Incorrect mode" in r.stdout
    r = run(clis, "restart_chkpt_files", 0, 1, 1, 128, "--run-tree-chkpt")
    assert r.returncode == 2


def test_missing_file_fails_loudly(clis, tmp_path):
    r = run(clis, "dedup_chkpt_files", 128, 1, "--run-tree-chkpt", str(tmp_path / "nope"))
    assert r.returncode == 1 and r.stderr.startswith("dedup_chkpt_files:")


def write_series(tmp_path, nbytes, cs, steps, seed):
    z = (nbytes // 4, nbytes // 4 + nbytes // 8)
    seq = [s.copy() for s in workloads.pattern2(nbytes, cs, steps, seed=seed, zero_range=z, run_max=64)]
    paths = []
    for i, s in enumerate(seq):
        p = tmp_path / ("state_%02d.dat" % i)
        p.write_bytes(s.tobytes())
        paths.append(str(p))
    return seq, paths


@pytest.mark.gpu
@pytest.mark.parametrize("flag", list(SUFFIX))
@pytest.mark.parametrize("nbytes,cs", [(1 << 20, 128), ((1 << 19) + 333, 256)])
def test_files_logs_and_restart_digest(clis, oracle, tmp_path, flag, nbytes, cs):
    seq, paths = write_series(tmp_path, nbytes, cs, 5, seed=nbytes % 97)
    r = run(clis, "dedup_chkpt_files", cs, len(paths), flag, *paths, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    ref = oracle.Deduplicator(APPROACH[flag], cs, 0)
    diffs = []
    for i, s in enumerate(seq):
        want = ref.checkpoint(s, i == 0)
        got = open(paths[i] + SUFFIX[flag], "rb").read()
        assert got == want, (flag, i)
        diffs.append(want)
    if flag != "--run-full-chkpt":
        for i in range(len(paths)):
            base = os.path.basename(paths[i]) + ".chunk_size.%d" % cs
            for ext in (".csv", ".size.csv", ".timing.csv"):
                assert (tmp_path / (base + ext)).exists(), base + ext
    for rid in (len(paths) - 1, 2):
        r = run(clis, "restart_chkpt_files", rid, len(paths), 2, cs, flag, *paths, cwd=tmp_path)
        assert r.returncode == 0, r.stderr
        lines = [ln for ln in r.stdout.splitlines() if ln.startswith(LABEL[flag])]
        assert len(lines) == 2
        out = np.zeros(nbytes, np.uint8)
        assert oracle.restart(APPROACH[flag], diffs[:rid + 1], rid, out) == 0
        want = oracle.digest(out.tobytes(), 0)
        hexd = " ".join(want.hex().upper()[k:k + 8] for k in range(0, 32, 8)) + " "
        assert lines[0][len(LABEL[flag]):].strip() == hexd.strip()
        assert (tmp_path / (os.path.basename(paths[rid]) + ".chunk_size.%d.restart_timing.csv" % cs)).exists()
