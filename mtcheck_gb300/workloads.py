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
    # one source per destination, the last one, as numpy's assignment keeps
    # it (a CUDA index_put with repeated indices keeps an arbitrary one)
    _, last = np.unique(dst[::-1], return_index=True)
    pick = dst.size - 1 - last
    dst, src = dst[pick], src[pick]
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


# ---------------------------------------------------------------------------
# On-device update pattern for request streams: one call per checkpoint,
# a handful of kernel launches, deterministic for (seed, step).
# ---------------------------------------------------------------------------
def init_device(buf, seed, zero_range=None):
    """Fill a torch CUDA uint8 buffer with seeded random bytes."""
    import torch
    g = torch.Generator(device=buf.device)
    g.manual_seed(int(seed) & 0x7FFFFFFFFFFFFFFF)
    buf.copy_(torch.randint(0, 256, (buf.numel(),), dtype=torch.uint8, device=buf.device, generator=g))
    if zero_range:
        buf[zero_range[0]:zero_range[1]] = 0
    return buf


def mutate_device(buf, cs, rate, seed, run_max=4096, shift_frac=0.1, zero_range=None):
    """One step of the 4 GiB update pattern applied in place to a torch CUDA
    buffer: `rate` of the chunks change, half as sparse single chunks and half
    as runs of up to `run_max` chunks (fresh random bytes); a further
    `shift_frac` of the changed count become copies of chunks at earlier
    offsets of the previous state; `zero_range` stays zero."""
    import torch
    dev = buf.device
    nbytes = buf.numel()
    full = nbytes // cs
    if full < 2:
        return buf
    rng = np.random.default_rng(int(seed) & 0x7FFFFFFFFFFFFFFF)
    g = torch.Generator(device=dev)
    g.manual_seed(int(rng.integers(1 << 62)))
    nchg = max(2, int(rate * full))
    rows = buf[:full * cs].view(full, cs)
    # shifted duplicates read the previous state: gather them first.  Every
    # index set is made unique so that no two writes race (the result is the
    # same on every run)
    nshift = max(1, int(shift_frac * nchg))
    dst = torch.unique(torch.randint(1, full, (nshift,), device=dev, generator=g))
    src = (torch.rand(dst.numel(), device=dev, generator=g) * dst).long()
    shifted = rows[src].clone()
    # sparse chunks
    sparse = torch.randint(0, full, (nchg // 2,), device=dev, generator=g)
    # runs: lengths on the host, starts and expansion on the device
    left = nchg - nchg // 2
    lens = []
    while left > 0:
        ln = int(min(left, rng.integers(1, run_max + 1)))
        lens.append(ln)
        left -= ln
    L = torch.tensor(lens, dtype=torch.long, device=dev)
    hi = torch.clamp(full - L, min=1)
    starts = (torch.rand(len(lens), device=dev, generator=g) * hi).long()
    offs = torch.cumsum(L, 0) - L
    total = int(sum(lens))
    within = torch.arange(total, device=dev) - torch.repeat_interleave(offs, L, output_size=total)
    runs = torch.repeat_interleave(starts, L, output_size=total) + within
    idx = torch.unique(torch.cat([sparse, runs]))
    rows[idx] = torch.randint(0, 256, (idx.numel(), cs), dtype=torch.uint8, device=dev, generator=g)
    rows[dst] = shifted
    if zero_range:
        buf[zero_range[0]:zero_range[1]] = 0
    return buf


def serve_mix(count=256, seed=5, lo_log2=22, hi_log2=28, cs=128, rate=(0.005, 0.05)):
    """Processes of the served workload: buffer sizes 2^k bytes with k uniform
    over the integers [lo_log2, hi_log2] (4 MiB .. 256 MiB: a power-of-two
    chunk count, for which the reference's tree restart is exact), chunk size
    `cs`, one change-rate range for all."""
    rng = np.random.default_rng(seed)
    return [{"nbytes": 1 << int(rng.integers(lo_log2, hi_log2 + 1)), "chunk_size": cs, "rate": rate,
             "seed": int(seed * 100000 + i)} for i in range(count)]


class DeviceUpdates:
    """Pre-generated steps of the 4 GiB update pattern for one device buffer,
    for request streams where the update itself must cost little host time.
    `count` variants are drawn once (changed chunk ids -- half sparse, half
    runs of up to `run_max` chunks --, their new bytes, and `shift_frac` as
    many shifted-duplicate destinations with earlier sources).  apply(step)
    writes variant step % count, its bytes XOR-ed with the low byte of the
    step so that repeated variants still write new content; four kernel
    launches.  Deterministic for (seed, step)."""

    def __init__(self, buf, cs, rate, seed, count=4, run_max=4096, shift_frac=0.1, zero_range=None):
        import torch
        self.cs = cs
        self.full = buf.numel() // cs
        self.zero_range = zero_range
        dev = buf.device
        rng = np.random.default_rng(int(seed) & 0x7FFFFFFFFFFFFFFF)
        g = torch.Generator(device=dev)
        g.manual_seed(int(rng.integers(1 << 62)))
        full = self.full
        self.variants = []
        for _ in range(count):
            nchg = max(2, int(rate * full))
            sparse = torch.randint(0, full, (nchg // 2,), device=dev, generator=g)
            left, lens = nchg - nchg // 2, []
            while left > 0:
                ln = int(min(left, rng.integers(1, run_max + 1)))
                lens.append(ln)
                left -= ln
            L = torch.tensor(lens, dtype=torch.long, device=dev)
            starts = (torch.rand(len(lens), device=dev, generator=g) * torch.clamp(full - L, min=1)).long()
            total = int(sum(lens))
            offs = torch.cumsum(L, 0) - L
            runs = torch.repeat_interleave(starts, L, output_size=total) + \
                torch.arange(total, device=dev) - torch.repeat_interleave(offs, L, output_size=total)
            idx = torch.unique(torch.cat([sparse, runs]))
            payload = torch.randint(0, 256, (idx.numel(), cs), dtype=torch.uint8, device=dev, generator=g)
            dst = torch.unique(torch.randint(1, full, (max(1, int(shift_frac * nchg)),), device=dev, generator=g))
            src = (torch.rand(dst.numel(), device=dev, generator=g) * dst).long()
            self.variants.append((idx, payload, dst, src))

    def apply(self, buf, step):
        import torch
        idx, payload, dst, src = self.variants[step % len(self.variants)]
        rows = buf[:self.full * self.cs].view(self.full, self.cs)
        shifted = rows[src]                         # earlier offsets of the previous state
        rows[idx] = torch.bitwise_xor(payload, step & 0xFF)
        rows[dst] = shifted
        if self.zero_range:
            buf[self.zero_range[0]:self.zero_range[1]] = 0
        return buf
