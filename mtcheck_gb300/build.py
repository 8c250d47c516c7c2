"""In-tree build of the CUDA library ``mtcheck_gb300/_build/libmtcheck_gb300.so``.

Compiles every ``csrc/*.cu`` for sm_103a only (one ``-gencode``), in parallel,
and links one shared library that exports the C ABI of ``include/mtcheck.h``.
No CMake; nvcc and the host compiler only.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmtcheck_gb300.so")
CLI_DIR = os.path.join(HERE, "cli")
# command-line drivers of the reference (src/dedup_files.cpp,
# src/restart_chkpt_files.cpp), built next to the library
CLIS = ["dedup_chkpt_files", "restart_chkpt_files"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _deps():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.hpp")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))


def _compile(src, extra):
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    newest_dep = max([os.path.getmtime(d) for d in _deps()] + [os.path.getmtime(src)])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj
    cmd = [nvcc()] + ARCH + FLAGS + extra + ["-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose=False, extra=()):
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcuda"] * 0
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(LIB + ".tmp", LIB)
    _build_clis()
    if verbose:
        print(LIB)
    return LIB


def _build_clis():
    """The CLI drivers: host C++ over include/mtcheck/deduplicator.hpp, linked
    to the library with an $ORIGIN rpath."""
    for name in CLIS:
        src = os.path.join(CLI_DIR, name + ".cpp")
        out = os.path.join(OUT_DIR, name)
        deps = [src, LIB] + glob.glob(os.path.join(ROOT, "include", "*.h")) + \
            glob.glob(os.path.join(ROOT, "include", "mtcheck", "*.hpp"))
        if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(d) for d in deps):
            continue
        cmd = [nvcc(), "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), src, "-o", out + ".tmp",
               "-L", OUT_DIR, "-lmtcheck_gb300", "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        os.replace(out + ".tmp", out)


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
