"""mtc_basic_checkpoint_noalloc: the checkpoint for callers that cannot allocate.

Out-of-memory and crash handlers, and runtimes whose pool owns the whole GPU,
cannot call cudaMalloc; this entry point works from caller-owned buffers and a
fixed scratch array inside the library.  It is called through the C ABI a
first time and then twice in a row, and each .basic checkpoint must equal,
byte for byte, the oracle's basic approach and the regular basic-approach
deduplicator on the same buffers, while the device's free memory stays the
same across the calls after the first.  This file is collected last on
purpose, so that a run stopping at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

from mtcheck_gb300 import workloads

pytestmark = pytest.mark.gpu


def _noalloc(lib, kind, data_ptr, nbytes, cs, digests, step, diff, cap):
    n = ctypes.c_uint64()
    rc = lib.mtc_basic_checkpoint_noalloc(kind, data_ptr, nbytes, cs, digests.data_ptr(), 0, step,
                                          1 if step == 0 else 0, diff.data_ptr(), cap, ctypes.byref(n), None)
    assert rc == 0, lib.mtc_last_error()
    return n.value


@pytest.mark.parametrize("nbytes,cs,kind,offset", [
    ((1 << 20) + 300, 128, 0, 0),   # ragged last chunk, TMA path
    (1 << 21, 512, 1, 0),           # MD5
    ((64 << 10) + 5, 24, 0, 0),     # chunk size not a multiple of 16: per-thread path, byte copies
    ((1 << 20) + 7, 256, 0, 3),     # input 3 bytes past an aligned address
])
def test_noalloc_matches_basic_deduplicator(cuda, mtc, oracle, nbytes, cs, kind, offset):
    seq = [s.copy() for s in workloads.pattern2(nbytes, cs, 3, seed=31, zero_range=(nbytes // 4, nbytes // 2))]
    ref = oracle.Deduplicator(oracle.BASIC, cs, kind)
    want = [ref.checkpoint(s, i == 0) for i, s in enumerate(seq)]
    gpu = mtc.BasicDeduplicator(cs, kind)
    assert [gpu.checkpoint(cuda.from_numpy(s).cuda(), i == 0) for i, s in enumerate(seq)] == want
    gpu.close()

    lib = mtc.load()
    nchunks = (nbytes + cs - 1) // cs
    cap = 32 + nchunks * (4 + cs)
    # every device buffer is made before the calls: nothing is allocated between them
    inputs = []
    for s in seq:
        base = cuda.zeros(nbytes + 64, dtype=cuda.uint8, device="cuda")
        base[offset:offset + nbytes].copy_(cuda.from_numpy(s))
        inputs.append(base)
    digests = cuda.zeros(nchunks * 16, dtype=cuda.uint8, device="cuda")
    diffs = [cuda.empty(cap, dtype=cuda.uint8, device="cuda") for _ in seq]
    cuda.cuda.synchronize()

    lens = [_noalloc(lib, kind, inputs[0].data_ptr() + offset, nbytes, cs, digests, 0, diffs[0], cap)]
    free_after_first = cuda.cuda.mem_get_info()[0]
    for i in range(1, len(seq)):   # two calls in a row after the first
        lens.append(_noalloc(lib, kind, inputs[i].data_ptr() + offset, nbytes, cs, digests, i, diffs[i], cap))
    assert cuda.cuda.mem_get_info()[0] == free_after_first, "device memory changed across the calls"
    for i in range(len(seq)):
        got = diffs[i][:lens[i]].cpu().numpy().tobytes()
        assert got == want[i], i


def test_noalloc_rejects_oversize_and_bad_buffers(cuda, mtc):
    lib = mtc.load()
    data = cuda.zeros(1 << 16, dtype=cuda.uint8, device="cuda")
    dig = cuda.zeros(16 * 1024 + 16, dtype=cuda.uint8, device="cuda")
    out = cuda.zeros(64, dtype=cuda.uint8, device="cuda")
    n = ctypes.c_uint64()
    rc = lib.mtc_basic_checkpoint_noalloc(0, data.data_ptr(), 1 << 16, 64, dig.data_ptr(), 0, 0, 1,
                                          out.data_ptr(), 64, ctypes.byref(n), None)
    assert rc == 1 and b"diff buffer" in lib.mtc_last_error()
    rc = lib.mtc_basic_checkpoint_noalloc(0, data.data_ptr(), (1 << 22) * 2 + 1, 2, dig.data_ptr(), 0, 0, 1,
                                          out.data_ptr(), 1 << 40, ctypes.byref(n), None)
    assert rc == 7 and b"4194304" in lib.mtc_last_error()
    rc = lib.mtc_basic_checkpoint_noalloc(0, data.data_ptr(), 1 << 16, 64, dig.data_ptr() + 4, 0, 0, 1,
                                          out.data_ptr(), 1 << 40, ctypes.byref(n), None)
    assert rc == 1 and b"16-byte" in lib.mtc_last_error()
