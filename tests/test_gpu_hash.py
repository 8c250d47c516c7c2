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
    rng = np.random.default_rng(3)
    data = rng.integers(0, 256, 128 * 300 + 17, dtype=np.uint8)
    base = cuda.from_numpy(np.concatenate([np.zeros(16, np.uint8), data])).cuda()
    for off in (1, 4, 8):
        view = (base.data_ptr() + 16 - off + off, len(data))  # aligned control
        out = mtc.hash_chunks(kind, view, 128).cpu().numpy().tobytes()
        assert out == oracle_digests(oracle, data, 128, kind)
    shifted = cuda.from_numpy(np.concatenate([np.zeros(3, np.uint8), data])).cuda()
    out = mtc.hash_chunks(kind, (shifted.data_ptr() + 3, len(data)), 128).cpu().numpy().tobytes()
    assert out == oracle_digests(oracle, data, 128, kind)
