"""Build recipe for the oracle (test infrastructure, never part of the product).

* ``oracle/_build/liboracle.so``: the C restatement in ``mtc_oracle.c``.
* ``oracle/_ref/libref_dedup.so``: the reference's own tree, list and basic
  deduplicators (``src/{tree,list,basic}_approach.cpp``, ``src/utils.cpp``)
  compiled from where they lie against the serial Kokkos stand-in in
  ``oracle/kokkos_serial``; built only where the reference is mounted.
* ``oracle/_ref/libref_hash.so``: the reference's own digest headers compiled
  from where they lie (``$MTCHECK_REFERENCE/include``, by default
  /root/reference/include) against the macro stub in
  ``oracle/ref_stub``.  Built only where the reference is mounted; the files
  travel with the repository snapshot but ``.so`` files are rebuilt per host.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# where the reference sources are mounted (only in the development container)
REFERENCE = os.environ.get("MTCHECK_REFERENCE", "/root/reference")
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_hash.so")


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force=False):
    src = os.path.join(HERE, "mtc_oracle.c")
    if force or _stale(ORACLE_SO, [src]):
        os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fvisibility=hidden",
                               "-Wall", "-o", ORACLE_SO + ".tmp", src])
        os.replace(ORACLE_SO + ".tmp", ORACLE_SO)
    return ORACLE_SO


def build_ref(force=False):
    inc = os.path.join(REFERENCE, "include")
    if not os.path.isdir(inc):
        return None
    src = os.path.join(HERE, "ref_hash_shim.cpp")
    if force or _stale(REF_SO, [src]):
        os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
        subprocess.check_call(["g++", "-O2", "-std=c++14", "-fPIC", "-shared", "-w",
                               "-I", os.path.join(HERE, "ref_stub"), "-I", inc,
                               "-o", REF_SO + ".tmp", src])
        os.replace(REF_SO + ".tmp", REF_SO)
    return REF_SO


REF_DEDUP_SO = os.path.join(HERE, "_ref", "libref_dedup.so")
KOKKOS_SERIAL = os.path.join(HERE, "kokkos_serial")
REF_DEDUP_SOURCES = ["src/tree_approach.cpp", "src/list_approach.cpp", "src/basic_approach.cpp", "src/utils.cpp"]


def build_ref_dedup(force=False):
    """The reference's own deduplicators (REF_DEDUP_SOURCES, compiled from
    where they lie) against the serial Kokkos stand-in in kokkos_serial/,
    behind the C-linkage driver ref_dedup_shim.cpp: oracle/_ref/libref_dedup.so.
    None where the reference is not mounted."""
    inc = os.path.join(REFERENCE, "include")
    if not os.path.isdir(inc):
        return None
    srcs = [os.path.join(REFERENCE, f) for f in REF_DEDUP_SOURCES] + [os.path.join(HERE, "ref_dedup_shim.cpp")]
    deps = srcs + [os.path.join(KOKKOS_SERIAL, f) for f in os.listdir(KOKKOS_SERIAL) if f.endswith(".hpp")]
    if force or _stale(REF_DEDUP_SO, deps):
        os.makedirs(os.path.dirname(REF_DEDUP_SO), exist_ok=True)
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-w", "-fvisibility=hidden",
                               "-I", KOKKOS_SERIAL, "-I", inc, "-o", REF_DEDUP_SO + ".tmp"] + srcs)
        os.replace(REF_DEDUP_SO + ".tmp", REF_DEDUP_SO)
    return REF_DEDUP_SO


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_oracle(force))
    print(build_ref(force))
    print(build_ref_dedup(force))
