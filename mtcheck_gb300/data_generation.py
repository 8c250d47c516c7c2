"""Checkpoint-series generator with the seven modes of the reference's
data_generation tool (include/data_generation.hpp:13-95,
src/data_generation.cpp:112-156).

    python -m mtcheck_gb300.data_generation data_len num_chkpts mode num_changes filename

writes filename.0.chkpt ... filename.<num_chkpts-1>.chkpt: an initial buffer
of uniform random bytes, then one perturbation per file:

  R  every byte drawn anew
  B  bytes [num_changes, data_len) drawn anew, the first num_changes kept
  C  num_changes contiguous bytes at a uniform random offset drawn anew
  I  nothing changes
  S  num_changes random positions each get a byte different from the old one
  Z  num_changes contiguous bytes at a uniform random offset set to zero
  W  the first num_changes bytes swap places with num_changes bytes at a
     random 128-byte-aligned offset that does not overlap them

The reference draws from Kokkos' XorShift64 pool and std::default_random_engine
(seed 1931); those generators are not available here, so the series follow the
same rules from numpy's seeded generator (same seed by default) and are not
byte-equal to the reference's files.  Sparse positions that repeat within one
step change once.
"""
import sys

import numpy as np

MODES = "RBCISZW"


def perturb(buf, mode, num_changes, rng):
    """One step of `mode` applied in place to the uint8 array `buf`."""
    n = buf.size
    k = int(num_changes)
    if mode == "R":
        buf[:] = rng.integers(0, 256, n, dtype=np.uint8)
    elif mode == "B":
        if k < n:
            buf[k:] = rng.integers(0, 256, n - k, dtype=np.uint8)
    elif mode in ("C", "Z"):
        if k > n:
            raise ValueError("num_changes larger than the buffer")
        off = int(rng.integers(0, n - k + 1))
        buf[off:off + k] = 0 if mode == "Z" else rng.integers(0, 256, k, dtype=np.uint8)
    elif mode == "I":
        pass
    elif mode == "S":
        pos = np.unique(rng.integers(0, n, k))
        # a new value that differs from the old one: old + 1..255 (mod 256)
        step = rng.integers(1, 256, pos.size).astype(np.uint16)
        buf[pos] = ((buf[pos].astype(np.uint16) + step) & 0xFF).astype(np.uint8)
    elif mode == "W":
        starts = np.arange(0, n - k + 1, 128, dtype=np.int64)
        starts = starts[starts >= k]
        if k == 0 or starts.size == 0:
            raise ValueError("no 128-byte-aligned region of num_changes bytes after the first one")
        b = int(starts[int(rng.integers(0, starts.size))])
        a = buf[:k].copy()
        buf[:k] = buf[b:b + k]
        buf[b:b + k] = a
    else:
        raise ValueError("unknown mode %r (one of %s)" % (mode, MODES))
    return buf


def series(data_len, num_chkpts, mode, num_changes, seed=1931):
    """Yield the num_chkpts successive buffers (the same array, updated in place)."""
    if mode not in MODES:
        raise ValueError("unknown mode %r (one of %s)" % (mode, MODES))
    rng = np.random.default_rng(seed)
    buf = rng.integers(0, 256, int(data_len), dtype=np.uint8)
    yield buf
    for _ in range(1, num_chkpts):
        yield perturb(buf, mode, num_changes, rng)


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) < 5:
        print("usage: python -m mtcheck_gb300.data_generation data_len num_chkpts mode num_changes filename")
        return 2
    data_len = int(argv[0], 0)
    num_chkpts = int(argv[1])
    mode = argv[2][:1]
    num_changes = int(argv[3], 0)
    name = argv[4] + "."
    print("Data length: %d" % data_len)
    print("Number of checkpoints: %d" % num_chkpts)
    print("Mode: %s" % mode)
    print("Num changes: %d" % num_changes)
    print("File name: %s" % name)
    for i, buf in enumerate(series(data_len, num_chkpts, mode, num_changes)):
        with open(name + "%d.chkpt" % i, "wb") as f:
            f.write(buf.tobytes())
    return 0


if __name__ == "__main__":
    sys.exit(main())
