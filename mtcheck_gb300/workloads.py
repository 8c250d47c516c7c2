"""Seeded synthetic checkpoint series with the shapes of the benchmark configs.

Each generator yields the successive states of one application buffer.  The
same code runs on numpy (host, used by the parity tests) and on torch CUDA
tensors (used by the benchmark at full size); the two are not bit-identical to
each other, each is deterministic for its seed.

* ``pattern1``: uniform random bytes; 20% of chunks in the first state are byte
  copies of other randomly chosen chunks; every later state rewrites 1% of
  chunks in contiguous runs of 1-32 chunks with fresh random bytes.
* ``pattern2``: per step 0.1-5% of chunks change, half as sparse single chunks
  and half as runs of up to 4096 chunks; a further 10% of the changed count are
  shifted duplicates copied from earlier offsets of the previous state; an
  optional byte range is zero-filled in every state.
"""
import numpy as np


class _NpOps:
    def __init__(self, seed):
        self.rng = np.random.default_rng(seed)

    def random_bytes(self, n):
        return self.rng.integers(0, 256, n, dtype=np.uint8)

    def integers(self, lo, hi, n):
        return self.rng.integers(lo, hi, n, dtype=np.int64)

    def uniform(self, lo, hi):
        return float(self.rng.uniform(lo, hi))

    def uniform_array(self, n):
        return self.rng.random(n)


class _TorchOps:
    def __init__(self, seed, device):
        import torch
        self.torch = torch
        self.device = device
        self.gen = torch.Generator(device=device)
        self.gen.manual_seed(seed)
        self.cpu = np.random.default_rng(seed)

    def random_bytes(self, n):
        return self.torch.randint(0, 256, (n,), dtype=self.torch.uint8, device=self.device, generator=self.gen)

    def integers(self, lo, hi, n):
        return self.cpu.integers(lo, hi, n, dtype=np.int64)

    def uniform(self, lo, hi):
        return float(self.cpu.uniform(lo, hi))

    def uniform_array(self, n):
        return self.cpu.random(n)


def _ops(seed, device):
    return _NpOps(seed) if device is None else _TorchOps(seed, device)


def _rows(buf, cs, nbytes):
    """2-D view [full chunks, cs] of the buffer."""
    full = nbytes // cs
    return buf[:full * cs].reshape(full, cs) if hasattr(buf, "reshape") else buf[:full * cs].view(full, cs)


def _is_torch(buf):
    return type(buf).__module__.split(".")[0] == "torch"


def _index(buf, idx):
    if _is_torch(buf):
        import torch
        return torch.from_numpy(np.ascontiguousarray(idx)).to(buf.device)
    return idx


def _copy_chunks(buf, cs, dst, src, nbytes, prev=None):
    """buf[chunk d] = (prev or buf)[chunk s] for whole chunks (partial last chunk skipped)."""
    full = nbytes // cs
    dst = np.asarray(dst, dtype=np.int64)
    src = np.asarray(src, dtype=np.int64)
    keep = (dst < full) & (src < full)
    dst, src = dst[keep], src[keep]
    if dst.size == 0:
        return
    rows = _rows(buf, cs, nbytes)
    srows = rows if prev is None else _rows(prev, cs, nbytes)
    vals = srows[_index(buf, src)]
    rows[_index(buf, dst)] = vals


def _fill_random(ops, buf, cs, chunks, nbytes):
    """Fresh random bytes in the given chunks."""
    chunks = np.unique(np.asarray(chunks, dtype=np.int64))
    if chunks.size == 0:
        return
    full = nbytes // cs
    body = chunks[chunks < full]
    if body.size:
        rows = _rows(buf, cs, nbytes)
        rnd = ops.random_bytes(int(body.size) * cs)
        rows[_index(buf, body)] = rnd.reshape(int(body.size), cs)
    if full * cs < nbytes and chunks[-1] >= full:
        buf[full * cs:nbytes] = ops.random_bytes(nbytes - full * cs)


def pattern1(nbytes, cs, steps, seed=1, device=None, dup_frac=0.2, rate=0.01, run_max=32):
    """States of the 64 MiB / 128 B series (and its scaled-down versions)."""
    ops = _ops(seed, device)
    n = (nbytes + cs - 1) // cs
    buf = ops.random_bytes(nbytes)
    ndup = int(dup_frac * n)
    if ndup and n > 1:
        dst = ops.integers(0, n, ndup)
        src = ops.integers(0, n, ndup)
        _copy_chunks(buf, cs, dst, src, nbytes)
    yield buf
    for _ in range(1, steps):
        target = max(1, int(round(rate * n)))
        chunks = []
        while len(chunks) < target:
            ln = int(ops.integers(1, run_max + 1, 1)[0])
            st = int(ops.integers(0, n, 1)[0])
            chunks.extend(range(st, min(n, st + ln)))
        _fill_random(ops, buf, cs, chunks[:target], nbytes)
        yield buf


def pattern2(nbytes, cs, steps, seed=2, device=None, rate=(0.001, 0.05), run_max=4096, shift_frac=0.1,
             zero_range=None):
    """States of the 4 GiB / 512 B series (and of the restart-chain series)."""
    ops = _ops(seed, device)
    n = (nbytes + cs - 1) // cs
    buf = ops.random_bytes(nbytes)
    if zero_range:
        buf[zero_range[0]:zero_range[1]] = 0
    yield buf
    for _ in range(1, steps):
        prev = buf.clone() if hasattr(buf, "clone") else buf.copy()
        nchg = max(2, int(ops.uniform(*rate) * n))
        sparse = ops.integers(0, n, nchg // 2)
        runs = []
        left = nchg - nchg // 2
        while left > 0:
            ln = int(min(left, ops.integers(1, run_max + 1, 1)[0]))
            st = int(ops.integers(0, max(1, n - ln), 1)[0])
            runs.extend(range(st, st + ln))
            left -= ln
        _fill_random(ops, buf, cs, np.concatenate([sparse, np.asarray(runs, dtype=np.int64)]), nbytes)
        nshift = max(1, int(shift_frac * nchg))
        dst = ops.integers(1, n, nshift)
        src = np.floor(ops.uniform_array(nshift) * dst).astype(np.int64)
        _copy_chunks(buf, cs, dst, src, nbytes, prev=prev)
        if zero_range:
            buf[zero_range[0]:zero_range[1]] = 0
        yield buf


def batch_mix(count=96, seed=4, median_mib=72.0, sigma=1.2, lo_mib=1, hi_mib=512,
              chunk_sizes=(64, 128, 512, 4096), rate=(0.001, 0.10)):
    """Members of the batched workload: sizes log-normal (median `median_mib`,
    log-sigma `sigma`) clipped to [lo_mib, hi_mib] MiB, chunk size uniform over
    `chunk_sizes`, Murmur3 and MD5 alternating, one change rate per member
    drawn uniformly from `rate`.  Returns a list of dicts."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        mib = float(np.clip(rng.lognormal(np.log(median_mib), sigma), lo_mib, hi_mib))
        cs = int(rng.choice(chunk_sizes))
        nbytes = int(mib * (1 << 20))
        out.append({"nbytes": nbytes, "chunk_size": cs, "hash": i % 2, "rate": float(rng.uniform(*rate)),
                    "seed": int(seed * 1000 + i)})
    return out
