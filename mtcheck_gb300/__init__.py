"""mtcheck_gb300 -- GB300 incremental-checkpoint deduplicator (Python binding).

The product is the CUDA library ``_build/libmtcheck_gb300.so`` behind the C ABI
of ``include/mtcheck.h``; this module binds it with ctypes and mirrors the
reference's deduplicator classes (``TreeDeduplicator``, ``ListDeduplicator``,
``BasicDeduplicator``, ``FullDeduplicator`` of TauferLab/MTCheck,
include/deduplicator_interface.hpp:14-184).  Device buffers are torch CUDA
tensors (uint8) or raw device addresses.  There is no CPU fallback: every
call fails loudly when the library or a GPU is missing.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libmtcheck_gb300.so")

# approaches: DedupMode values (include/utils.hpp:39-49)
FULL, BASIC, LIST, TREE, TREE_LOW_OFFSET_REF, TREE_LOW_OFFSET = 1, 2, 3, 4, 5, 6
MURMUR3, MD5 = 0, 1
STATUS = {0: "MTC_OK", 1: "MTC_EINVAL", 2: "MTC_ECORRUPT", 3: "MTC_ENOMEM", 4: "MTC_ETIMEOUT", 5: "MTC_ECUDA",
          6: "MTC_EINTERNAL", 7: "MTC_ENOTSUP"}
FILE_SUFFIX = {FULL: ".full_chkpt", BASIC: ".basic.incr_chkpt", LIST: ".hashlist.incr_chkpt",
               TREE: ".hashtree.incr_chkpt", TREE_LOW_OFFSET_REF: ".hashtree.incr_chkpt",
               TREE_LOW_OFFSET: ".hashtree.incr_chkpt"}


class MtcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg))
        self.code = code


class Header(ctypes.Structure):
    """header_t, include/utils.hpp:29-37."""
    _fields_ = [("ref_id", ctypes.c_uint32), ("chkpt_id", ctypes.c_uint32), ("datalen", ctypes.c_uint64),
                ("chunk_size", ctypes.c_uint32), ("num_first_ocur", ctypes.c_uint32),
                ("num_prior_chkpts", ctypes.c_uint32), ("num_shift_dupl", ctypes.c_uint32)]


class Info(ctypes.Structure):
    _fields_ = [("current_id", ctypes.c_uint32), ("baseline_id", ctypes.c_uint32), ("chunk_size", ctypes.c_uint32),
                ("num_first_ocur", ctypes.c_uint32), ("num_shift_dupl", ctypes.c_uint32),
                ("num_prior_chkpts", ctypes.c_uint32), ("data_len", ctypes.c_uint64),
                ("diff_len", ctypes.c_uint64), ("data_size", ctypes.c_uint64), ("metadata_size", ctypes.c_uint64),
                ("timers", ctypes.c_double * 4), ("restart_timers", ctypes.c_double * 2),
                ("phase_times", ctypes.c_double * 3),
                ("device_error", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_uint64), ("graph_captures", ctypes.c_uint64), ("graph_nodes", ctypes.c_uint64),
                ("kernels_per_step", ctypes.c_uint64), ("last_device_ms", ctypes.c_double),
                ("last_call_ms", ctypes.c_double), ("host_ms", ctypes.c_double * 5),
                ("last_used_graph", ctypes.c_int32),
                ("batched_leaf_members", ctypes.c_uint32)]


class Tune(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32), ("direct", ctypes.c_int32),
                ("eager", ctypes.c_int32), ("max_load", ctypes.c_double), ("threads_per_chunk", ctypes.c_int32),
                ("untimed", ctypes.c_int32)]

    def as_dict(self):
        return {"rows": self.rows, "ctas_per_sm": self.ctas_per_sm, "direct": self.direct,
                "eager": self.eager, "max_load": self.max_load, "threads_per_chunk": self.threads_per_chunk,
                "untimed": self.untimed}


class ServerOptions(ctypes.Structure):
    _fields_ = [("hbm_budget", ctypes.c_uint64), ("max_inflight", ctypes.c_uint32), ("id_headroom", ctypes.c_uint32),
                ("use_graph", ctypes.c_int32), ("reserve_hbm", ctypes.c_int32), ("pinned_reserve", ctypes.c_uint64)]


class Completion(ctypes.Structure):
    _fields_ = [("ticket", ctypes.c_uint64), ("pid", ctypes.c_uint32), ("kind", ctypes.c_int32),
                ("status", ctypes.c_int32), ("chkpt_id", ctypes.c_uint32), ("diff_len", ctypes.c_uint64),
                ("t_submit_ms", ctypes.c_double), ("t_admit_ms", ctypes.c_double), ("t_done_ms", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "submitted", "completed", "failed", "checkpoints", "restarts", "bytes_checkpointed", "bytes_restarted",
        "spilled_diffs", "spilled_states", "restored_states", "staged_diffs", "spilled_bytes", "graph_captures",
        "graph_replays", "hbm_used", "hbm_peak", "pinned_reserved", "deferred_admissions", "pool_reserved_high",
        "pool_used_high")] + \
        [("inflight_peak", ctypes.c_uint32), ("pinned_sync_grows", ctypes.c_uint32),
         ("worker_ms", ctypes.c_double * 4), ("worker_max_ms", ctypes.c_double * 3)]

    def as_dict(self):
        d = {n: getattr(self, n) for n, _ in self._fields_ if n not in ("worker_ms", "worker_max_ms")}
        d["worker_ms"] = {k: round(self.worker_ms[j], 2) for j, k in enumerate(("start", "finish", "room", "wait"))}
        d["worker_max_ms"] = {k: round(self.worker_max_ms[j], 2) for j, k in enumerate(("start", "finish", "room"))}
        return d


# every symbol of include/mtcheck.h with its ctypes signature
_VP, _U32, _U64, _I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
SIGNATURES = {
    "mtc_create": (_I, [_I, _I, _U32, ctypes.POINTER(_VP)]),
    "mtc_destroy": (_I, [_VP]),
    "mtc_set_stream": (_I, [_VP, _VP]),
    "mtc_checkpoint_header": (_I, [_VP, ctypes.POINTER(Header), _VP, _U64, _I, ctypes.POINTER(_U64)]),
    "mtc_checkpoint": (_I, [_VP, _VP, _U64, _I, ctypes.POINTER(_U64)]),
    "mtc_advance": (_I, [_VP]),
    "mtc_inject_stall": (_I, [_VP, _U32]),
    "mtc_diff_copy": (_I, [_VP, _VP, _U64]),
    "mtc_diff_device": (_I, [_VP, ctypes.POINTER(_VP), ctypes.POINTER(_U64)]),
    "mtc_checkpoint_alloc": (_I, [_VP, _VP, _U64, _I, ctypes.POINTER(_VP), ctypes.POINTER(_U64)]),
    "mtc_free": (None, [_VP]),
    "mtc_checkpoint_file": (_I, [_VP, _VP, _U64, ctypes.c_char_p, ctypes.c_char_p, _I]),
    "mtc_restart": (_I, [_VP, _VP, _U64, ctypes.POINTER(_VP), ctypes.POINTER(_U64), _U32, _U32]),
    "mtc_restart_device": (_I, [_VP, _VP, _U64, ctypes.POINTER(_VP), ctypes.POINTER(_U64), _U32, _U32]),
    "mtc_release_restart_buffers": (_I, [_VP]),
    "mtc_restart_files": (_I, [_VP, _VP, _U64, ctypes.POINTER(ctypes.c_char_p), _U32, _U32]),
    "mtc_get_info": (_I, [_VP, ctypes.POINTER(Info)]),
    "mtc_write_chkpt_log": (_I, [_VP, ctypes.POINTER(Header), _VP, _U64, ctypes.c_char_p]),
    "mtc_write_restart_log": (_I, [_VP, _U32, ctypes.c_char_p]),
    "mtc_hash_chunks": (_I, [_I, _VP, _U64, _U32, _VP, _VP]),
    "mtc_digest_host": (_I, [_I, _VP, _U64, _VP]),
    "mtc_digest_hex": (_I, [_VP, ctypes.c_char_p]),
    "mtc_basic_checkpoint_noalloc": (_I, [_I, _VP, _U64, _U32, _VP, _U32, _U32, _I, _VP, _U64,
                                         ctypes.POINTER(_U64), _VP]),
    "mtc_batch_create": (_I, [_U32, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_U32),
                              ctypes.POINTER(_VP)]),
    "mtc_batch_destroy": (_I, [_VP]),
    "mtc_batch_member": (_I, [_VP, _U32, ctypes.POINTER(_VP)]),
    "mtc_batch_checkpoint": (_I, [_VP, ctypes.POINTER(_VP), ctypes.POINTER(_U64), _I, ctypes.POINTER(_U64)]),
    "mtc_batch_set_options": (_I, [_VP, _I, _U32]),
    "mtc_batch_get_info": (_I, [_VP, ctypes.POINTER(BatchInfo)]),
    "mtc_batch_autotune": (_I, [_VP, ctypes.POINTER(_U64)]),
    "mtc_batch_reserve": (_I, [_VP, ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    "mtc_server_create": (_I, [ctypes.POINTER(ServerOptions), ctypes.POINTER(_VP)]),
    "mtc_server_destroy": (_I, [_VP]),
    "mtc_server_add_process": (_I, [_VP, _I, _I, _U32, ctypes.POINTER(_U32)]),
    "mtc_server_submit_checkpoint": (_I, [_VP, _U32, _VP, _U64, _I, ctypes.POINTER(_U64)]),
    "mtc_server_submit_restart": (_I, [_VP, _U32, _U32, _VP, _U64, ctypes.POINTER(_U64)]),
    "mtc_server_poll": (_I, [_VP, ctypes.POINTER(Completion), _U32, ctypes.POINTER(_U32), ctypes.c_double]),
    "mtc_server_drain": (_I, [_VP, ctypes.c_double]),
    "mtc_server_chain_length": (_I, [_VP, _U32, ctypes.POINTER(_U32)]),
    "mtc_server_copy_diff": (_I, [_VP, _U32, _U32, _VP, _U64, ctypes.POINTER(_U64)]),
    "mtc_server_get_stats": (_I, [_VP, ctypes.POINTER(ServerStats)]),
    "mtc_now_ms": (ctypes.c_double, []),
    "mtc_set_tuning": (_I, [_VP, ctypes.POINTER(Tune)]),
    "mtc_get_tuning": (_I, [_VP, ctypes.POINTER(Tune)]),
    "mtc_autotune": (_I, [_I, _I, _U32, _U64, ctypes.POINTER(Tune), ctypes.POINTER(ctypes.c_double),
                          ctypes.POINTER(ctypes.c_double)]),
    "mtc_launch_count": (_U64, []),
    "mtc_last_error": (ctypes.c_char_p, []),
}

_lib = None


def load(path=LIB_PATH):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise ImportError("mtcheck_gb300 CUDA library missing: %s (run __graft_entry__.build())" % path)
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise MtcError(rc, (load().mtc_last_error() or b"").decode())


def _dev_ptr(buf):
    """(address, nbytes) of a torch CUDA tensor, or pass (int address, nbytes)."""
    if isinstance(buf, tuple):
        return int(buf[0]), int(buf[1])
    if not getattr(buf, "is_cuda", False):
        raise TypeError("expected a CUDA tensor or an (address, nbytes) pair")
    if not buf.is_contiguous():
        raise ValueError("tensor must be contiguous")
    return int(buf.data_ptr()), int(buf.numel() * buf.element_size())


def launch_count():
    return int(load().mtc_launch_count())


def hash_chunks(kind, buf, chunk_size, out=None, stream=0):
    """Digests of every chunk of a device buffer (16 bytes each)."""
    import torch
    ptr, n = _dev_ptr(buf)
    nchunks = (n + chunk_size - 1) // chunk_size
    if out is None:
        out = torch.empty(nchunks * 16, dtype=torch.uint8, device="cuda")
    _check(load().mtc_hash_chunks(kind, ptr, n, chunk_size, out.data_ptr(), stream))
    return out


def digest_host(data, kind=MURMUR3):
    """calculate_digest_host's 16-byte digest of a host buffer."""
    a = np.ascontiguousarray(np.frombuffer(data, dtype=np.uint8) if isinstance(data, (bytes, bytearray)) else data,
                             dtype=np.uint8)
    out = (ctypes.c_uint8 * 16)()
    _check(load().mtc_digest_host(kind, a.ctypes.data if a.size else None, a.size, out))
    return bytes(out)


def digest_hex(d):
    out = ctypes.create_string_buffer(37)
    _check(load().mtc_digest_hex(ctypes.c_char_p(d), out))
    return out.value.decode()


class Deduplicator:
    """Common base: BaseDeduplicator (include/deduplicator_interface.hpp:14-184)."""
    approach = TREE

    def __init__(self, chunk_size, hash=MURMUR3, approach=None):
        L = load()
        if approach is not None:
            self.approach = approach
        self.chunk_size = chunk_size
        h = _VP()
        _check(L.mtc_create(self.approach, hash, chunk_size, ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            load().mtc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream):
        _check(load().mtc_set_stream(self.h, int(stream)))

    # -- checkpoint ------------------------------------------------------
    def checkpoint_device(self, buf, make_baseline, advance=True):
        """Deduplicate a device buffer; the diff stays in device memory.  Returns its size."""
        ptr, n = _dev_ptr(buf)
        out = _U64()
        if advance:
            _check(load().mtc_checkpoint(self.h, ptr, n, int(make_baseline), ctypes.byref(out)))
        else:
            _check(load().mtc_checkpoint_header(self.h, None, ptr, n, int(make_baseline), ctypes.byref(out)))
        return int(out.value)

    def checkpoint(self, buf, make_baseline, advance=True):
        """checkpoint(uint8_t*, size_t, HostMirror& diff_h, bool): returns the diff as bytes."""
        n = self.checkpoint_device(buf, make_baseline, advance)
        host = np.empty(n, dtype=np.uint8)
        _check(load().mtc_diff_copy(self.h, host.ctypes.data, n))
        return host.tobytes()

    def copy_diff(self, host_array):
        _check(load().mtc_diff_copy(self.h, host_array.ctypes.data, host_array.nbytes))

    def diff_device(self):
        p, n = _VP(), _U64()
        _check(load().mtc_diff_device(self.h, ctypes.byref(p), ctypes.byref(n)))
        return int(p.value or 0), int(n.value)

    def checkpoint_file(self, buf, filename, logname=None, make_baseline=False):
        ptr, n = _dev_ptr(buf)
        _check(load().mtc_checkpoint_file(self.h, ptr, n, filename.encode(),
                                          logname.encode() if logname else None, int(make_baseline)))

    # -- restart ---------------------------------------------------------
    def restart(self, out, chkpts, chkpt_id):
        """restart(View data, std::vector<HostMirror>& chkpts, logname, id) into device buffer `out`."""
        ptr, n = _dev_ptr(out)
        bufs = [np.frombuffer(c, dtype=np.uint8) for c in chkpts]
        ptrs = (_VP * len(bufs))(*[b.ctypes.data if b.size else 0 for b in bufs])
        lens = (_U64 * len(bufs))(*[b.size for b in bufs])
        _check(load().mtc_restart(self.h, ptr, n, ptrs, lens, len(bufs), chkpt_id))

    def restart_device(self, out, dev_chkpts, chkpt_id):
        """Restart from a chain resident in device memory: list of (address, nbytes)."""
        ptr, n = _dev_ptr(out)
        ptrs = (_VP * len(dev_chkpts))(*[int(p) for p, _ in dev_chkpts])
        lens = (_U64 * len(dev_chkpts))(*[int(l) for _, l in dev_chkpts])
        _check(load().mtc_restart_device(self.h, ptr, n, ptrs, lens, len(dev_chkpts), chkpt_id))

    def inject_stall(self, checkpoints=1):
        """Fault injection for tests: the next checkpoints' hashing kernel
        times out on the device (MTC_ETIMEOUT); the one after is a baseline."""
        _check(load().mtc_inject_stall(self.h, checkpoints))

    def release_restart_buffers(self):
        """Free the restart tables kept between restarts (reallocated by the next one)."""
        _check(load().mtc_release_restart_buffers(self.h))

    def restart_files(self, out, filenames, chkpt_id):
        ptr, n = _dev_ptr(out)
        names = (ctypes.c_char_p * len(filenames))(*[f.encode() for f in filenames])
        _check(load().mtc_restart_files(self.h, ptr, n, names, len(filenames), chkpt_id))

    # -- counters ----------------------------------------------------------
    def info(self):
        i = Info()
        _check(load().mtc_get_info(self.h, ctypes.byref(i)))
        return i

    def num_first_ocur(self):
        return self.info().num_first_ocur

    def num_shift_dupl(self):
        return self.info().num_shift_dupl

    @property
    def current_id(self):
        return self.info().current_id

    def write_restart_log(self, select_chkpt, logname):
        _check(load().mtc_write_restart_log(self.h, select_chkpt, logname.encode()))

    # -- tuning ------------------------------------------------------------
    def set_tuning(self, rows=None, ctas_per_sm=None, direct=None, max_load=None, eager=None,
                   threads_per_chunk=None, untimed=None):
        """Set the given fields of the launch tuning; the others keep their values."""
        cur = self.tuning()
        pick = lambda v, k: cur[k] if v is None else v
        t = Tune(pick(rows, "rows"), pick(ctas_per_sm, "ctas_per_sm"), pick(direct, "direct"), pick(eager, "eager"),
                 pick(max_load, "max_load"), pick(threads_per_chunk, "threads_per_chunk"), pick(untimed, "untimed"))
        _check(load().mtc_set_tuning(self.h, ctypes.byref(t)))

    def tuning(self):
        t = Tune()
        _check(load().mtc_get_tuning(self.h, ctypes.byref(t)))
        return t.as_dict()


class TreeDeduplicator(Deduplicator):
    approach = TREE


class TreeLowOffsetRefDeduplicator(Deduplicator):
    approach = TREE_LOW_OFFSET_REF


class ListDeduplicator(Deduplicator):
    approach = LIST


class BasicDeduplicator(Deduplicator):
    approach = BASIC


class FullDeduplicator(Deduplicator):
    approach = FULL


class _Member(Deduplicator):
    """A batch member: an ordinary handle owned by its batch."""

    def __init__(self, handle, approach, chunk_size, owner):
        self.h = handle
        self.approach = approach
        self.chunk_size = chunk_size
        self._owner = owner  # keeps the batch alive

    def close(self):
        self.h = None


class Batch:
    """Many deduplicators checkpointed in one call (mtc_batch_*): the baseline
    step overlaps every member's kernels on separate streams, later steps
    replay one CUDA graph.  `members` is a list of (approach, hash, chunk_size)."""

    def __init__(self, members):
        L = load()
        n = len(members)
        ap = (_I * n)(*[int(m[0]) for m in members])
        hs = (_I * n)(*[int(m[1]) for m in members])
        cs = (_U32 * n)(*[int(m[2]) for m in members])
        b = _VP()
        _check(L.mtc_batch_create(n, ap, hs, cs, ctypes.byref(b)))
        self.b = b
        self.members = []
        for i, m in enumerate(members):
            h = _VP()
            _check(L.mtc_batch_member(b, i, ctypes.byref(h)))
            self.members.append(_Member(h, int(m[0]), int(m[2]), self))

    def __len__(self):
        return len(self.members)

    def close(self):
        if getattr(self, "b", None):
            for m in self.members:
                m.h = None
            load().mtc_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_options(self, use_graph=True, id_headroom=64):
        _check(load().mtc_batch_set_options(self.b, int(use_graph), int(id_headroom)))

    def autotune(self, bufs):
        lens = (_U64 * len(bufs))(*[_dev_ptr(x)[1] for x in bufs])
        _check(load().mtc_batch_autotune(self.b, lens))

    def reserve(self, bufs):
        """Reserve device memory for every member's state on these buffers;
        returns the bytes reserved."""
        lens = (_U64 * len(bufs))(*[_dev_ptr(x)[1] for x in bufs])
        out = _U64()
        _check(load().mtc_batch_reserve(self.b, lens, ctypes.byref(out)))
        return int(out.value)

    def checkpoint(self, bufs, make_baseline=False):
        """One checkpoint of every member; returns the list of diff sizes."""
        n = len(bufs)
        pl = [_dev_ptr(x) for x in bufs]
        ptrs = (_VP * n)(*[p for p, _ in pl])
        lens = (_U64 * n)(*[l for _, l in pl])
        out = (_U64 * n)()
        _check(load().mtc_batch_checkpoint(self.b, ptrs, lens, int(make_baseline), out))
        return [int(x) for x in out]

    def info(self):
        i = BatchInfo()
        _check(load().mtc_batch_get_info(self.b, ctypes.byref(i)))
        return i


class Server:
    """Request-serving loop (mtc_server_*): processes submit checkpoint and
    restart requests; a worker thread admits them continuously under an HBM
    budget, spilling cold state to pinned host memory."""

    def __init__(self, hbm_budget=0, max_inflight=0, id_headroom=0, use_graph=False, reserve_hbm=False,
                 pinned_reserve=0):
        o = ServerOptions(int(hbm_budget), int(max_inflight), int(id_headroom), int(use_graph), int(reserve_hbm),
                          int(pinned_reserve))
        s = _VP()
        _check(load().mtc_server_create(ctypes.byref(o), ctypes.byref(s)))
        self.s = s
        self._buf = (Completion * 256)()

    def close(self):
        if getattr(self, "s", None):
            load().mtc_server_destroy(self.s)
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_process(self, approach, hash, chunk_size):
        pid = _U32()
        _check(load().mtc_server_add_process(self.s, approach, hash, chunk_size, ctypes.byref(pid)))
        return int(pid.value)

    def submit_checkpoint(self, pid, buf, make_baseline=False):
        ptr, n = _dev_ptr(buf)
        t = _U64()
        _check(load().mtc_server_submit_checkpoint(self.s, pid, ptr, n, int(make_baseline), ctypes.byref(t)))
        return int(t.value)

    def submit_restart(self, pid, chkpt_id, out):
        ptr, n = _dev_ptr(out)
        t = _U64()
        _check(load().mtc_server_submit_restart(self.s, pid, chkpt_id, ptr, n, ctypes.byref(t)))
        return int(t.value)

    def poll(self, wait_ms=0.0):
        """List of completions (dicts), waiting up to wait_ms for the first."""
        n = _U32()
        _check(load().mtc_server_poll(self.s, self._buf, len(self._buf), ctypes.byref(n), float(wait_ms)))
        out = []
        for i in range(n.value):
            c = self._buf[i]
            out.append({"ticket": c.ticket, "pid": c.pid, "kind": c.kind, "status": c.status,
                        "chkpt_id": c.chkpt_id, "diff_len": c.diff_len, "t_submit_ms": c.t_submit_ms,
                        "t_admit_ms": c.t_admit_ms, "t_done_ms": c.t_done_ms})
        return out

    def drain(self, timeout_ms=600000.0):
        _check(load().mtc_server_drain(self.s, float(timeout_ms)))

    def chain_length(self, pid):
        n = _U32()
        _check(load().mtc_server_chain_length(self.s, pid, ctypes.byref(n)))
        return int(n.value)

    def diff(self, pid, chkpt_id):
        n = _U64()
        _check(load().mtc_server_copy_diff(self.s, pid, chkpt_id, None, 0, ctypes.byref(n)))
        host = np.empty(n.value, np.uint8)
        _check(load().mtc_server_copy_diff(self.s, pid, chkpt_id, host.ctypes.data, n.value, ctypes.byref(n)))
        return host.tobytes()

    def stats(self):
        s = ServerStats()
        _check(load().mtc_server_get_stats(self.s, ctypes.byref(s)))
        return s.as_dict()


def now_ms():
    return float(load().mtc_now_ms())


def autotune(approach, hash, chunk_size, nbytes):
    """Fastest launch shape for one configuration: (tuning dict, best ms, default ms)."""
    t = Tune()
    best, dflt = ctypes.c_double(), ctypes.c_double()
    _check(load().mtc_autotune(approach, hash, chunk_size, nbytes, ctypes.byref(t), ctypes.byref(best),
                               ctypes.byref(dflt)))
    return t.as_dict(), best.value, dflt.value
