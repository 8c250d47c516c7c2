"""Chunk hashing on the GPU (TMA pipeline and direct kernel) against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def oracle_digests(oracle, data, cs, kind):
    n = (len(data) + cs - 1) // cs
    return b"".join(oracle.digest(data[i * cs:(i + 1) * cs], kind) for i in range(n))


@pytest.mark.parametrize("kind", [0, 1], ids=["murmur3", "md5"])
@pytest.mark.parametrize("cs", [1, 7, 16, 32, 48, 64, 100, 128, 256, 512, 640, 4096])
def test_hash_chunks(cuda, mtc, oracle, kind, cs):
    rng = np.random.default_rng(cs * 3 + kind)
    for nchunks, tail in ((1, 0), (3, 0), (257, 0), (700, 5), (1025, cs - 1)):
        n = nchunks * cs + (tail if tail < cs else 0)
        data = rng.integers(0, 256, n, dtype=np.uint8)
        dev = cuda.from_numpy(data).cuda()
        out = mtc.hash_chunks(kind, dev, cs).cpu().numpy().tobytes()
        assert out == oracle_digests(oracle, data, cs, kind), (cs, nchunks, tail)


@pytest.mark.parametrize("kind", [0, 1])
def test_hash_unaligned_buffer(cuda, mtc, oracle, kind):
    # the buffer starts `off` bytes past a 16-byte aligned address: offsets 0
    # and 16 take the TMA path, the others the direct per-thread path (4-byte
    # aligned words for 4, 8 and 12, byte loads for 1 and 3)
    rng = np.random.default_rng(3)
    data = rng.integers(0, 256, 128 * 300 + 17, dtype=np.uint8)
    want = oracle_digests(oracle, data, 128, kind)
    for off in (0, 1, 3, 4, 8, 12, 16):
        base = cuda.zeros(len(data) + 64, dtype=cuda.uint8, device="cuda")
        assert base.data_ptr() % 16 == 0
        base[off:off + len(data)].copy_(cuda.from_numpy(data))
        out = mtc.hash_chunks(kind, (base.data_ptr() + off, len(data)), 128).cpu().numpy().tobytes()
        assert out == want, off
