"""Host-side plumbing of bench.py, without a GPU: the served and batched
sections run in processes of their own, and the closing summary reads every
section's headline figures.  A misspelt option or a section that fails must
show in the bench line as an error, not break it."""
import json
import subprocess
import sys

import pytest

import bench


def _fake_run(captured, stdout="", returncode=0, stderr=""):
    def run(args, capture_output=True, text=True, env=None):
        captured["args"] = args
        captured["env"] = env
        return subprocess.CompletedProcess(args, returncode, stdout=stdout, stderr=stderr)
    return run


@pytest.mark.parametrize("flag,key", [("--only-serve", "served"), ("--only-batch", "batched")])
def test_section_process_gets_every_option_and_returns_its_object(monkeypatch, flag, key):
    monkeypatch.setattr(sys, "argv", ["bench.py", "--serve-seconds", "3", "--batch-count", "12"])
    a = bench.parse()
    captured = {}
    line = json.dumps({key: {"value": 1.5}})
    monkeypatch.setattr(bench.subprocess, "run", _fake_run(captured, stdout="noise\n" + line + "\n"))
    got = bench.section_in_subprocess(flag, key, a)
    assert got == {"value": 1.5}
    args = captured["args"]
    assert args[0] == sys.executable and args[1].endswith("bench.py") and args[2] == flag
    # every option handed to the section process is one that bench.py parses,
    # with the value of this run
    monkeypatch.setattr(sys, "argv", ["bench.py"] + args[3:])
    b = bench.parse()
    assert b.serve_seconds == 3.0 and b.batch_count == 12 and b.hash == a.hash
    assert captured["env"]["WORLD_SIZE"] == "1" and captured["env"]["RANK"] == "0"


def test_section_process_failure_is_an_error_object(monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse()
    monkeypatch.setattr(bench.subprocess, "run", _fake_run({}, returncode=3, stderr="boom\nlast line"))
    got = bench.section_in_subprocess("--only-serve", "served", a)
    assert "error" in got and "exited 3" in got["error"] and "last line" in got["error"]
    monkeypatch.setattr(bench.subprocess, "run", _fake_run({}, stdout="no json here\n"))
    assert "error" in bench.section_in_subprocess("--only-batch", "batched", a)


def test_summary_reads_present_sections_and_tolerates_missing_ones():
    empty = bench.summary_of({"value": 4700.0})
    assert empty["dedup_4gib_512b_murmur3_gbs"] == 4700.0
    assert empty["served_p99_ms"] is None and empty["restart_1gib_256b_gbs"] is None
    line = {"value": 4700.0, "e2e": {"value": 205.0, "link_frac": 0.98},
            "restart": {"value": 1620.0, "roofline_frac": 0.48},
            "served": {"latency_ms": {"p50": 0.45, "p99": 1.3}, "saturation": {"speedup_vs_per_call": 2.8}},
            "batched": {"error": "section process exited 1"}}
    s = bench.summary_of(line)
    assert s["e2e_gbs"] == 205.0 and s["e2e_frac_of_link"] == 0.98
    assert s["restart_1gib_256b_gbs"] == 1620.0 and s["served_p99_ms"] == 1.3
    assert s["served_capacity_vs_per_call"] == 2.8
    assert s["batched_speedup_job"] is None  # a failed section reads as absent
