"""mtc_basic_checkpoint_noalloc: the checkpoint for callers that cannot allocate.

It is called through the C ABI with caller-owned buffers only, twice in a row
(a first checkpoint, then an incremental one), and its .basic checkpoints must
equal, byte for byte, those of the regular basic-approach deduplicator on the
same buffers.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from mtcheck_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nbytes,cs,kind", [((1 << 20) + 300, 128, 0), (1 << 21, 512, 1)])
def test_noalloc_matches_basic_deduplicator(cuda, mtc, nbytes, cs, kind):
    seq = [s.copy() for s in workloads.pattern2(nbytes, cs, 2, seed=31, zero_range=(nbytes // 4, nbytes // 2))]
    ref = mtc.BasicDeduplicator(cs, kind)
    want = [ref.checkpoint(cuda.from_numpy(s).cuda(), i == 0) for i, s in enumerate(seq)]

    lib = mtc.load()
    nchunks = (nbytes + cs - 1) // cs
    digests = cuda.zeros(nchunks * 16, dtype=cuda.uint8, device="cuda")
    cap = 32 + nchunks * (4 + cs)
    diff = cuda.empty(cap, dtype=cuda.uint8, device="cuda")
    for i, s in enumerate(seq):
        data = cuda.from_numpy(s).cuda()
        n = ctypes.c_uint64()
        rc = lib.mtc_basic_checkpoint_noalloc(kind, data.data_ptr(), nbytes, cs, digests.data_ptr(), 0, i,
                                              1 if i == 0 else 0, diff.data_ptr(), cap, ctypes.byref(n), None)
        assert rc == 0, lib.mtc_last_error()
        got = diff[:n.value].cpu().numpy().tobytes()
        assert got == want[i], i


def test_noalloc_rejects_oversize_and_small_buffers(cuda, mtc):
    lib = mtc.load()
    data = cuda.zeros(1 << 16, dtype=cuda.uint8, device="cuda")
    dig = cuda.zeros(16 * 1024, dtype=cuda.uint8, device="cuda")
    out = cuda.zeros(64, dtype=cuda.uint8, device="cuda")
    n = ctypes.c_uint64()
    rc = lib.mtc_basic_checkpoint_noalloc(0, data.data_ptr(), 1 << 16, 64, dig.data_ptr(), 0, 0, 1,
                                          out.data_ptr(), 64, ctypes.byref(n), None)
    assert rc == 1 and b"diff buffer" in lib.mtc_last_error()
    rc = lib.mtc_basic_checkpoint_noalloc(0, data.data_ptr(), (1 << 22) * 2 + 1, 2, dig.data_ptr(), 0, 0, 1,
                                          out.data_ptr(), 1 << 40, ctypes.byref(n), None)
    assert rc == 7 and b"4194304" in lib.mtc_last_error()
