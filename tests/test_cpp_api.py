"""The C++ interface (include/mtcheck/deduplicator.hpp) compiles, and on the GPU
passes the reference's known-answer and round-trip tests restated in C++."""
import json
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "api_test.cpp")


def test_header_compiles_without_cuda():
    r = subprocess.run(["g++", "-std=c++14", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), "-x", "c++", "-"],
                       input='#include "mtcheck/deduplicator.hpp"\nint main(){return 0;}\n', text=True,
                       capture_output=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_cpp_api_on_gpu(mtc, tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "api_test")
    lib_dir = os.path.dirname(mtc.LIB_PATH)
    subprocess.check_call([nvcc, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
                           "-L", lib_dir, "-lmtcheck_gb300", "-Xlinker", "-rpath=" + lib_dir])
    cases = json.load(open(os.path.join(ROOT, "tests", "golden", "tree_kat.json")))["cases"]
    stdin = "".join("%d %s %s %d %d\n" % (c["chunk_size"], c["step0"], c["step1"], c["num_first_ocur"],
                                          c["num_shift_dupl"]) for c in cases)
    r = subprocess.run([exe], input=stdin, text=True, capture_output=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failures" in r.stdout


def test_leaf_range_closed_form_equals_reference_loop(tmp_path):
    # host-only program over the kernels' own header: no GPU needed
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = os.path.join(ROOT, "tests", "cpp", "leaf_range_test.cu")
    exe = str(tmp_path / "leaf_range_test")
    subprocess.check_call([nvcc, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           "-I", os.path.join(ROOT, "mtcheck_gb300", "csrc"), src, "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout
