"""Regenerate the golden fixtures in this folder from the reference itself.

* ``tree_kat.json``: the ten known-answer tests of the reference
  (test/test_case_01.cpp .. test_case_10.cpp): the two 8-byte checkpoints
  (chunk size 1), and the expected number of first-occurrence and
  shifted-duplicate regions after the second checkpoint.  Parsed from the
  test sources as text.
* ``hash_vectors.json``: digests of seeded byte strings of many lengths,
  computed by the reference's own hash headers (include/kokkos_murmur3.hpp,
  include/kokkos_md5.hpp) compiled by ``oracle/build.py`` into oracle/_ref.

* ``reference_series.npz``: a seeded series (inputs) checkpointed by the
  reference's own basic, list and tree deduplicators, compiled by
  ``oracle/build.py`` against the serial Kokkos stand-in (``<approach>_diff<i>``).
* ``long_hash_vectors.json``: whole-buffer digests of inputs longer than
  INT_MAX bytes (a fixed arithmetic byte pattern, ``long_pattern``), where the
  reference's MD5 takes its 128-byte-piece branch
  (include/kokkos_md5.hpp:293-301), computed by the same compiled headers.

Run from the repository root where the reference sources are mounted
(``MTCHECK_REFERENCE``, default /root/reference):
    python tests/golden/make_golden.py
"""
import ctypes
import json
import os
import re
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
REF = os.environ.get("MTCHECK_REFERENCE", "/root/reference")
OUT = os.path.dirname(os.path.abspath(__file__))

# lengths: every tail length, block boundaries, and the chunk sizes in use
HASH_LENGTHS = sorted(set(list(range(0, 130)) + [255, 256, 257, 511, 512, 513, 1000, 4095, 4096, 4097]))
HASH_SEED = 20260101


def kat_cases():
    cases = []
    for i in range(1, 11):
        path = os.path.join(REF, "test", "test_case_%02d.cpp" % i)
        src = open(path).read()
        steps = {0: {}, 1: {}}
        for step, idx, ch in re.findall(r"step([01])_h\((\d)\)\s*=\s*static_cast<uint8_t>\('(.)'\)", src):
            steps[int(step)][int(idx)] = ch
        chunk = int(re.search(r"TreeDeduplicator deduplicator\((\d+)\)", src).group(1))
        m = re.search(r"num_first_ocur\(\) != (\d+) \|\| deduplicator.num_shift_dupl\(\) != (\d+)", src)
        cases.append({
            "name": "test_case_%02d" % i,
            "source": "test/test_case_%02d.cpp" % i,
            "chunk_size": chunk,
            "step0": "".join(steps[0][k] for k in range(8)),
            "step1": "".join(steps[1][k] for k in range(8)),
            "num_first_ocur": int(m.group(1)),
            "num_shift_dupl": int(m.group(2)),
        })
    return cases


def hash_vectors():
    from oracle import build
    lib = ctypes.CDLL(build.build_ref(force=True))
    rng = np.random.default_rng(HASH_SEED)
    vecs = []
    for n in HASH_LENGTHS:
        data = rng.integers(0, 256, n, dtype=np.uint8)
        ent = {"len": n, "data": data.tobytes().hex()}
        for name, fn in (("murmur3", lib.ref_murmur3_hash), ("md5", lib.ref_md5_hash)):
            out = (ctypes.c_uint8 * 16)()
            fn(ctypes.c_void_p(data.ctypes.data), ctypes.c_uint64(n), out)
            ent[name] = bytes(out).hex()
        vecs.append(ent)
    return vecs


# lengths above INT_MAX: len % 128 = 77 (a short last piece) and 0 (an
# empty last piece)
LONG_LENGTHS = [(1 << 31) + 77, (1 << 31) + 128]


def long_pattern(n, block=64 << 20):
    """n bytes: byte i = ((i * 2654435761) mod 2^32) >> 24."""
    out = np.empty(n, dtype=np.uint8)
    for s in range(0, n, block):
        x = np.arange(s, min(n, s + block), dtype=np.uint32)
        out[s:s + x.size] = ((x * np.uint32(2654435761)) >> np.uint32(24)).astype(np.uint8)
    return out


def long_vectors():
    from oracle import build
    lib = ctypes.CDLL(build.build_ref())
    vecs = []
    for n in LONG_LENGTHS:
        data = long_pattern(n)
        ent = {"len": n}
        for name, fn in (("murmur3", lib.ref_murmur3_hash), ("md5", lib.ref_md5_hash)):
            out = (ctypes.c_uint8 * 16)()
            fn(ctypes.c_void_p(data.ctypes.data), ctypes.c_uint64(n), out)
            ent[name] = bytes(out).hex()
        vecs.append(ent)
    return vecs


# series checkpointed by the reference's own code (oracle/_ref/libref_dedup.so)
# for the GPU tests: inputs, diffs per approach, restarted states
REF_SERIES = {"nbytes": 32 * 1024 + 77, "chunk_size": 64, "steps": 4, "seed": 1234}


def reference_series():
    from oracle import pyoracle
    from mtcheck_gb300 import workloads
    n, cs, steps = REF_SERIES["nbytes"], REF_SERIES["chunk_size"], REF_SERIES["steps"]
    z = (n // 4, n // 4 + n // 8)
    states = [s.copy() for s in workloads.pattern2(n, cs, steps, seed=REF_SERIES["seed"], zero_range=z)]
    out = {"state%d" % i: s for i, s in enumerate(states)}
    for approach, name in ((2, "basic"), (3, "list"), (4, "tree")):
        r = pyoracle.RefDeduplicator(approach, cs)
        for i, s in enumerate(states):
            out["%s_diff%d" % (name, i)] = np.frombuffer(r.checkpoint(s, i == 0), np.uint8).copy()
    return out


if __name__ == "__main__":
    with open(os.path.join(OUT, "tree_kat.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": kat_cases()}, f, indent=1)
    with open(os.path.join(OUT, "hash_vectors.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "seed": HASH_SEED, "vectors": hash_vectors()}, f)
    with open(os.path.join(OUT, "long_hash_vectors.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "pattern": "long_pattern",
                   "vectors": long_vectors()}, f, indent=1)
    np.savez_compressed(os.path.join(OUT, "reference_series.npz"), **reference_series())
    print("wrote", os.listdir(OUT))
