"""ctypes binding of the C oracle (``oracle/mtc_oracle.c``).

Test infrastructure: imported only by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``.  The product library never loads it.
"""
import ctypes
import struct
import os

import numpy as np

from . import build as _build

FULL, BASIC, LIST, TREE, TREE_LOW_OFFSET_REF, TREE_LOW_OFFSET = 1, 2, 3, 4, 5, 6
MURMUR3, MD5 = 0, 1
APPROACH_NAMES = {FULL: "full", BASIC: "basic", LIST: "list", TREE: "tree",
                  TREE_LOW_OFFSET_REF: "tree-low-offset-ref", TREE_LOW_OFFSET: "tree-low-offset"}

_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint32]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_checkpoint.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_uint64)]
        L.orc_free.argtypes = [ctypes.c_void_p]
        L.orc_restart.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_uint64),
                                  ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint64]
        L.orc_hash.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
        for f in ("orc_num_first_ocur", "orc_num_shift_dupl", "orc_current_id"):
            getattr(L, f).restype = ctypes.c_uint32
            getattr(L, f).argtypes = [ctypes.c_void_p]
        L.orc_datasizes.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]
        L.orc_labels.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        _lib = L
    return _lib


def ref_lib():
    """The reference's own hash headers compiled on this host, or None."""
    global _ref
    if _ref is None:
        path = _build.build_ref()
        if path is None:
            return None
        _ref = ctypes.CDLL(path)
        for f in (_ref.ref_murmur3_hash, _ref.ref_md5_hash):
            f.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
    return _ref


_refd = None


def ref_dedup_lib():
    """The reference's own deduplicators compiled on this host, or None."""
    global _refd
    if _refd is None:
        path = _build.build_ref_dedup()
        if path is None:
            return None
        L = ctypes.CDLL(path)
        L.refd_create.restype = ctypes.c_void_p
        L.refd_create.argtypes = [ctypes.c_int, ctypes.c_uint32]
        L.refd_destroy.argtypes = [ctypes.c_void_p]
        L.refd_checkpoint.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_uint64)]
        L.refd_free.argtypes = [ctypes.c_void_p]
        L.refd_restart.argtypes = [ctypes.c_int, ctypes.c_uint32, ctypes.POINTER(ctypes.c_void_p),
                                   ctypes.POINTER(ctypes.c_uint64), ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p,
                                   ctypes.c_uint64]
        _refd = L
    return _refd


class RefDeduplicator:
    """A deduplicator of the reference's own code (Murmur3, the reference's
    hash()): BASIC, LIST or TREE."""

    def __init__(self, approach, chunk_size):
        self.h = ref_dedup_lib().refd_create(approach, chunk_size)
        if not self.h:
            raise ValueError("approach not available in the reference build")

    def __del__(self):
        if getattr(self, "h", None):
            ref_dedup_lib().refd_destroy(self.h)
            self.h = None

    def checkpoint(self, data, make_baseline):
        a = _buf(data)
        p, n = ctypes.c_void_p(), ctypes.c_uint64()
        ref_dedup_lib().refd_checkpoint(self.h, a.ctypes.data, a.size, int(make_baseline), ctypes.byref(p),
                                        ctypes.byref(n))
        out = ctypes.string_at(p.value, n.value)
        ref_dedup_lib().refd_free(p)
        return out


def ref_restart(approach, chunk_size, diffs, chkpt_id, out):
    """The reference's restart_chkpt of checkpoint ``chkpt_id`` into ``out``
    (in place).  Its tree restart reads out of bounds for chunk counts that
    are not powers of two: callers keep to power-of-two tree chains."""
    bufs = [np.frombuffer(d, dtype=np.uint8) for d in diffs]
    ptrs = (ctypes.c_void_p * len(bufs))(*[b.ctypes.data for b in bufs])
    lens = (ctypes.c_uint64 * len(bufs))(*[b.size for b in bufs])
    return ref_dedup_lib().refd_restart(approach, chunk_size, ptrs, lens, len(bufs), chkpt_id, out.ctypes.data,
                                        out.size)


def _buf(data):
    a = np.ascontiguousarray(np.frombuffer(data, dtype=np.uint8) if isinstance(data, (bytes, bytearray)) else data,
                             dtype=np.uint8)
    return a


def digest(data, kind=MURMUR3):
    a = _buf(data)
    out = (ctypes.c_uint8 * 16)()
    lib().orc_hash(kind, a.ctypes.data if a.size else None, a.size, out)
    return bytes(out)


class Deduplicator:
    """Serial restatement of one reference deduplicator (tree/list/basic/full)."""

    def __init__(self, approach, chunk_size, hash_kind=MURMUR3):
        self.approach = approach
        self.h = lib().orc_create(approach, hash_kind, chunk_size)
        if not self.h:
            raise ValueError("bad oracle arguments")

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def checkpoint(self, data, make_baseline, increment=True):
        a = _buf(data)
        p = ctypes.c_void_p()
        n = ctypes.c_uint64()
        rc = lib().orc_checkpoint(self.h, a.ctypes.data, a.size, int(make_baseline), int(increment),
                                  ctypes.byref(p), ctypes.byref(n))
        if rc != 0:
            raise RuntimeError(f"oracle checkpoint failed: {rc}")
        if n.value < (1 << 31):
            out = ctypes.string_at(p.value, n.value)
        else:  # string_at takes a C int size
            a = np.empty(n.value, dtype=np.uint8)
            ctypes.memmove(a.ctypes.data, p.value, n.value)
            out = a.tobytes()
            del a
        lib().orc_free(p)
        return out

    def num_first_ocur(self):
        return lib().orc_num_first_ocur(self.h)

    def num_shift_dupl(self):
        return lib().orc_num_shift_dupl(self.h)

    def datasizes(self):
        v = (ctypes.c_uint64 * 2)()
        lib().orc_datasizes(self.h, v)
        return int(v[0]), int(v[1])


def restart(approach, diffs, chkpt_id, out):
    """Restart checkpoint ``chkpt_id`` of ``diffs`` into the uint8 array ``out`` (in place)."""
    bufs = [np.frombuffer(d, dtype=np.uint8) for d in diffs]
    ptrs = (ctypes.c_void_p * len(bufs))(*[b.ctypes.data for b in bufs])
    lens = (ctypes.c_uint64 * len(bufs))(*[b.size for b in bufs])
    rc = lib().orc_restart(approach, ptrs, lens, len(bufs), chkpt_id, out.ctypes.data, out.size)
    return rc


# ---------------------------------------------------------------------------
# CSV logs of one checkpoint, restated from the reference's writers: the
# values of every column except the timers.
# ---------------------------------------------------------------------------
LOG_NAMES = {FULL: "Full", BASIC: "Basic", LIST: "List", TREE: "Tree", TREE_LOW_OFFSET_REF: "Tree",
             TREE_LOW_OFFSET: "Tree"}


def metadata_breakdown(diff, num_chkpts):
    """write_metadata_breakdown (src/utils.cpp:38-124): header bytes, distinct
    metadata bytes, repeat-map bytes, then one column per checkpoint (the
    bytes of shifted-duplicate entries taken from it, by repeat-map row)."""
    ref_id, chkpt_id, _datalen, _cs, nfo, nprior, nshift = struct.unpack_from("<IIQIIII", diff, 0)
    cols = [32, nfo * 4]
    if ref_id != chkpt_id:                                      # :98-116
        cols.append(8 * nprior)
        for i in range(num_chkpts):
            if i < nprior:
                off = 32 + nfo * 4 + i * 8
                num = struct.unpack_from("<I", diff, off + 4)[0]
                cols.append(num * 8)
            else:
                cols.append(0)
    else:                                                       # :117-123
        cols.append(0)
        cols.append(nshift * 8)
        cols.extend([0] * max(0, num_chkpts - 1))
    return cols


def log_rows(approach, chunk_size, current_id, baseline_id, data_len, datasizes, diff):
    """The rows that write_chkpt_log appends for checkpoint `current_id`
    (src/tree_approach.cpp:1854-1896, src/list_approach.cpp:1014-1052,
    src/basic_approach.cpp:632-673, src/full_approach.cpp:187-234), with the
    timer columns left out: (.csv row without its four timers, .size.csv row,
    .timing.csv row without its timers)."""
    name = LOG_NAMES[approach]
    d, m = datasizes
    csv = [name, current_id, chunk_size, data_len, d + m, d, m]
    timing = [name, current_id, chunk_size]
    if approach == FULL:
        size = [name, current_id, chunk_size, d, 0, 0, 0, 0] + [0] * current_id
        timing += ["0.0", "0.0"]
        return csv, size, timing
    # the basic approach passes current_id - baseline_id + 1 checkpoints
    # (src/basic_approach.cpp:672), the others current_id
    n = current_id - baseline_id + 1 if approach == BASIC else current_id
    size = [name, current_id, chunk_size, d, m] + metadata_breakdown(diff, n)
    return csv, size, timing
