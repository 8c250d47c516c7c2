"""Benchmark of the GB300 incremental-checkpoint deduplicator.

Default workload: tree approach (lowest-offset rule), Murmur3, one 4 GiB
buffer in 512-byte chunks, seeded synthetic states with the 4 GiB update
pattern (0.1-5% of chunks change per step, half sparse, half runs of up to
4096 chunks, 10% shifted duplicates, [1 GiB, 1.5 GiB) zero-filled).  A step is
one incremental checkpoint of the whole buffer.

  value : buffer bytes / device time per checkpoint, inputs resident in HBM,
          diff assembled in HBM (GB/s, whole job over all ranks)
  e2e   : the same through the C ABI with pinned host buffers: H2D of the
          state, checkpoint, D2H of the diff inside the timed region (the
          next state's upload overlaps the current checkpoint)

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun every rank deduplicates its own buffer (replicas, no
collective on the data path); value = all ranks' bytes / max rank time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# more hardware work queues than the default 8, so that the kernels of many
# concurrent streams (batch members, served processes) are not funnelled into
# false dependencies; a per-process runtime setting, read at context creation
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = "Dedup & restart GB/s on 1 GB300, % HBM roofline; batched vs per-call; p99 ms"
GIB = 1 << 30


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--hash", default="murmur3", choices=["murmur3", "md5"])
    p.add_argument("--size-gib", type=float, default=4.0)
    p.add_argument("--chunk", type=int, default=512)
    p.add_argument("--pattern", default="4gib", choices=["4gib", "64mib"],
                   help="update series: the 4 GiB one (sparse chunks, runs, shifted copies, a zero range) or the "
                        "64 MiB one (20%% duplicated chunks at first, then 1%% rewritten per step in runs of 1-32)")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-sections", action="store_true",
                   help="skip the MD5 and the 64 MiB / 128 B sections")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-restart", action="store_true")
    p.add_argument("--restart-gib", type=float, default=1.0)
    p.add_argument("--restart-chunk", type=int, default=256)
    p.add_argument("--restart-chain", type=int, default=31)
    p.add_argument("--no-batch", action="store_true")
    p.add_argument("--batch-count", type=int, default=96)
    p.add_argument("--batch-median-mib", type=float, default=72.0)
    p.add_argument("--batch-steps", type=int, default=5)
    p.add_argument("--batch-no-tune", action="store_true")
    p.add_argument("--only-batch", action="store_true")
    p.add_argument("--no-serve", action="store_true")
    p.add_argument("--only-serve", action="store_true")
    p.add_argument("--only-restart", action="store_true")
    p.add_argument("--serve-procs", type=int, default=256)
    p.add_argument("--serve-rate", type=float, default=2000.0)
    p.add_argument("--serve-seconds", type=float, default=8.0)
    p.add_argument("--serve-budget-gb", type=float, default=120.0)
    p.add_argument("--serve-inflight", type=int, default=64)
    p.add_argument("--serve-verify-procs", type=int, default=4)
    p.add_argument("--serve-pinned-gb", type=float, default=32.0)
    p.add_argument("--serve-trace", default=None,
                   help="write one CSV row per request of the timed stream to this file")
    p.add_argument("--serve-sat-procs", type=int, default=64,
                   help="processes the capacity run draws its requests from (both arms)")
    p.add_argument("--serve-sat-requests", type=int, default=3000,
                   help="requests of the capacity run (all arriving at once), also run one call at a time")
    return p.parse_args()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic():
    """Per-chunk DRAM traffic of the leaf kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "leaf_kernel_traffic.json")
    if os.path.exists(path):
        try:
            return json.load(open(path))
        except Exception:
            return None
    return None


class ClockSampler:
    """nvidia-smi clock and throttle samples during the timed region."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx.append(float(s[1]))
            except ValueError:
                continue
            for n, v in zip(names, s[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(torch, x, device, ws):
    """The slowest rank's time (every rank gets it): the job ends when the
    last replica does."""
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    if ws > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(bytes_per_rank, seconds, ws):
    """GB/s of the whole job: every replica's bytes over the slowest time."""
    return bytes_per_rank * ws / seconds / 1e9


PATTERN_NAME = {"4gib": "the 4 GiB update pattern", "64mib": "the 64 MiB update pattern"}


def series(pattern, nbytes, cs, count, seed, device=None):
    """States of one of the two update series (generator)."""
    from mtcheck_gb300 import workloads
    if pattern == "64mib":
        return workloads.pattern1(nbytes, cs, count, seed=seed, device=device)
    z = (GIB, GIB + GIB // 2) if nbytes >= 2 * GIB else (nbytes // 4, nbytes // 4 + nbytes // 8)
    return workloads.pattern2(nbytes, cs, count, seed=seed, device=device, zero_range=z)


def make_states(torch, nbytes, cs, count, seed, device, pattern="4gib"):
    return [s.clone() for s in series(pattern, nbytes, cs, count, seed, device)]


def restart_bench(torch, mc, dev, a, kind, approach=None):
    """Restart of the last checkpoint of a chain (1 GiB, 256 B chunks, 30
    incrementals after a baseline, 4 GiB update pattern); tree approach unless
    `approach` is given."""
    from mtcheck_gb300 import workloads
    approach = approach or mc.TREE
    nbytes = int(a.restart_gib * GIB) // a.restart_chunk * a.restart_chunk
    z = (nbytes // 4, nbytes // 4 + nbytes // 8)
    d = mc.Deduplicator(a.restart_chunk, kind, approach=approach)
    chain_dev, chain_host, last = [], [], None
    for i, s in enumerate(workloads.pattern2(nbytes, a.restart_chunk, a.restart_chain, seed=303, device=dev,
                                             zero_range=z)):
        n = d.checkpoint_device(s, i == 0)
        keep = torch.empty(n, dtype=torch.uint8, device=dev)
        host = torch.empty(n, dtype=torch.uint8).pin_memory()
        d.copy_diff(host.numpy())
        keep.copy_(host)
        chain_dev.append(keep)
        chain_host.append(host)
        last = s.clone()
    torch.cuda.synchronize()
    out = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    ptrs = [(t.data_ptr(), t.numel()) for t in chain_dev]
    rid = len(chain_dev) - 1
    r = mc.Deduplicator(a.restart_chunk, kind, approach=approach)
    r.restart_device(out, ptrs, rid)  # warm-up
    ok = bool(torch.equal(out, last))
    reps = 5
    times, dev_times = [], []
    for _ in range(reps):
        out.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r.restart_device(out, ptrs, rid)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
        dev_times.append(r.info().restart_timers[1])
        ok = ok and bool(torch.equal(out, last))
    dev_t = statistics.median(dev_times)
    call_t = statistics.median(times)
    chain_bytes = sum(t.numel() for t in chain_dev)
    # B_restart = D (written) + the chain bytes read: every chunk's data once
    # (D) and the metadata of every checkpoint of the chain (headers, region
    # lists, repeat tables, shift entries)
    import struct
    meta = 0
    for h in chain_host:
        _r, _c, _dl, _cs, nfo, nprior, nshift = struct.unpack_from("<IIQIIII", h[:32].numpy().tobytes(), 0)
        meta += 32 + 4 * nfo + (0 if approach == mc.BASIC else 8 * nprior + 8 * nshift)
    b_restart = 2 * nbytes + meta
    # chain in pinned host memory: H2D inside the call (mtc_restart)
    host_list = [h.numpy().tobytes() for h in chain_host]
    e2e_t = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r.restart(out, host_list, rid)
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t0)
        ok = ok and bool(torch.equal(out, last))
    # the reference's restart check: hash() of the whole restored buffer
    # (calculate_digest_host), against the same digest of the original state
    dig = mc.digest_hex(mc.digest_host(out.cpu().numpy(), kind))
    dig_ok = dig == mc.digest_hex(mc.digest_host(last.cpu().numpy(), kind))
    name = {mc.TREE: "tree", mc.LIST: "list", mc.BASIC: "basic"}.get(approach, str(approach))
    return {"workload": "restart of checkpoint %d of a %s chain, %.3g GiB buffer, %d B chunks, 4 GiB update "
                        "pattern" % (rid, name, a.restart_gib, a.restart_chunk),
            "value": round(nbytes / dev_t / 1e9, 3), "unit": "GB/s", "ms": round(dev_t * 1e3, 3),
            "roofline_frac": round(b_restart / dev_t / 1e9 / load_peaks()[0], 4),
            "b_restart_bytes": int(b_restart),
            "call_ms": round(call_t * 1e3, 3),
            "chain_bytes": int(chain_bytes), "verified_byte_identical": ok,
            "restart_digest": dig.strip(), "digest_matches_original": dig_ok,
            "host_chain_value": round(nbytes / statistics.median(e2e_t) / 1e9, 3),
            "host_chain_ms": round(statistics.median(e2e_t) * 1e3, 3),
            "note": "value: device time with the chain resident in HBM; call_ms adds the host side of the call; "
                    "host_chain_value: chain in pageable host memory, copied to HBM inside the call"}


def series_bench(torch, mc, dev, states, cs, kind, W, flush=None, untimed=False):
    """Incremental checkpoints of resident device states through one handle:
    states[0] is the baseline, the next W are warm-up, the rest are timed.
    With `flush`, each step is timed alone after a write of `flush` (larger
    than L2); without it, the whole loop between two events.  Returns the
    device seconds per step and the per-step counters."""
    d = mc.TreeDeduplicator(cs, kind)
    if untimed:
        d.set_tuning(untimed=1)
    d.checkpoint_device(states[0], True)
    for s in states[1:1 + W]:
        d.checkpoint_device(s, False)
    timed = states[1 + W:]
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in timed]
    leaf, sdata, smeta = [], [], []
    torch.cuda.synchronize()
    for i, s in enumerate(timed):
        if flush is not None:
            flush.zero_()
        if flush is not None or i == 0:
            evs[i][0].record()
        d.checkpoint_device(s, False)
        if flush is not None or i == len(timed) - 1:
            evs[i][1].record()
        info = d.info()
        leaf.append(info.phase_times[0])
        sdata.append(info.data_size)
        smeta.append(info.metadata_size)
    torch.cuda.synchronize()
    if flush is not None:
        t = sum(e0.elapsed_time(e1) for e0, e1 in evs) / 1e3 / len(timed)
    else:
        t = evs[0][0].elapsed_time(evs[-1][1]) / 1e3 / len(timed)
    d.close()
    return t, sum(leaf) / len(leaf), sum(sdata) / len(sdata), sum(smeta) / len(smeta)


def link_section(torch, dev, nbytes=GIB, reps=3):
    """The host link's ceiling: pinned 1 GiB copies host->device and
    device->host, split over 1, 2 and 4 streams (best of `reps`), timed by
    events on the current stream that every copy stream joins."""
    host = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    devb = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    devb.copy_(host)  # first pass over the newly pinned pages
    host.copy_(devb)
    torch.cuda.synchronize()
    streams = [torch.cuda.Stream(device=dev) for _ in range(4)]
    out = {}
    for name, to_dev in (("h2d_gbs", True), ("d2h_gbs", False)):
        out[name] = {}
        for ns in (1, 2, 4):
            part = nbytes // ns
            best = None
            for _ in range(reps):
                cur = torch.cuda.current_stream()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(cur)
                for k in range(ns):
                    streams[k].wait_event(e0)
                    with torch.cuda.stream(streams[k]):
                        if to_dev:
                            devb[k * part:(k + 1) * part].copy_(host[k * part:(k + 1) * part], non_blocking=True)
                        else:
                            host[k * part:(k + 1) * part].copy_(devb[k * part:(k + 1) * part], non_blocking=True)
                for k in range(ns):
                    cur.wait_stream(streams[k])
                e1.record(cur)
                e1.synchronize()
                ms = e0.elapsed_time(e1)
                best = ms if best is None else min(best, ms)
            out[name][str(ns)] = round(nbytes / (best * 1e-3) / 1e9, 1)
    del host, devb
    return out


def small_series_section(torch, mc, dev, peak):
    """The 64 MiB / 128 B series (tree, Murmur3, 10 checkpoints: a baseline and
    9 incremental ones, each timed alone after a 256 MiB write that flushes
    L2): once as a warm-up, once with the phase events (for the leaf time),
    once replayed as one graph without them (the value)."""
    nbytes, cs = 64 << 20, 128
    N = nbytes // cs
    states = make_states(torch, nbytes, cs, 10, seed=64, device=dev, pattern="64mib")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    series_bench(torch, mc, dev, states, cs, mc.MURMUR3, 0, flush)
    t_timed, leaf, sd, sm = series_bench(torch, mc, dev, states, cs, mc.MURMUR3, 0, flush)
    t, _, _, _ = series_bench(torch, mc, dev, states, cs, mc.MURMUR3, 0, flush, untimed=True)
    b = nbytes + 32 * N + 2 * sd + sm
    del states, flush
    return {"workload": "tree dedup, Murmur3, 64 MiB buffer, 128 B chunks, 10 checkpoints of the 64 MiB update "
                        "pattern (9 incremental timed, L2 flushed before each)",
            "value": round(nbytes / t / 1e9, 3), "unit": "GB/s", "ms": round(t * 1e3, 4),
            "ms_with_phase_events": round(t_timed * 1e3, 4),
            "leaf_ms": round(leaf * 1e3, 4),
            "roofline_frac": round(b / t / 1e9 / peak, 4),
            "note": "value and ms: replayed as one graph (mtc_tune_t.untimed); ms_with_phase_events: the default "
                    "five graph launches with events between the phases, which the leaf time comes from; "
                    "roofline_frac: B_dedup = D + 32 N + 2 S_data + S_meta per device-timed checkpoint over the "
                    "measured HBM copy bandwidth"}


def md5_section(torch, mc, dev, states, cs, W, peak):
    """The same 4 GiB states checkpointed with MD5 chunk digests."""
    nbytes = states[0].numel()
    N = (nbytes + cs - 1) // cs
    t, leaf, sd, sm = series_bench(torch, mc, dev, states, cs, mc.MD5, W)
    return {"workload": "tree dedup, MD5, %.3g GiB buffer, %d B chunks, incremental checkpoints of the 4 GiB update "
                        "pattern" % (nbytes / GIB, cs),
            "value": round(nbytes / t / 1e9, 3), "unit": "GB/s", "ms": round(t * 1e3, 4),
            "leaf_ms": round(leaf * 1e3, 4),
            "leaf_hbm_frac": round(N * (cs + 32) / leaf / 1e9 / peak, 4),
            "leaf_alu_pipe_frac_ncu": MD5_ALU_PIPE,
            "note": "MD5 is bound by the integer ALU pipe; leaf_alu_pipe_frac_ncu is the ALU pipe's share of peak "
                    "in the committed ncu capture of this kernel (profiles/leaf_tma_kernel_md5_512B.md)"}


# ALU pipe utilisation of leaf_tma_kernel<MD5> at 512 B chunks, from the
# committed ncu capture (sm__inst_executed_pipe_alu over its peak)
MD5_ALU_PIPE = 0.797


def cpu_sample(kind, cs, pattern="4gib", nbytes=GIB):
    """Single-thread oracle on a sample of the same pattern (at most 1 GiB): baseline + incrementals."""
    from oracle import pyoracle
    n = min(nbytes, GIB) // cs * cs
    seq = series(pattern, n, cs, 4, seed=123)
    d = pyoracle.Deduplicator(pyoracle.TREE, cs, kind)
    first = next(seq).copy()
    d.checkpoint(first, True)
    times = []
    for s in seq:
        t0 = time.perf_counter()
        d.checkpoint(s, False)
        times.append(time.perf_counter() - t0)
    return n / (sum(times) / len(times)) / 1e9, len(times)


def reference_worker(args):
    """One host thread of the CPU reference arm: oracle dedup of an independent slice."""
    sys.path.insert(0, ROOT)
    nbytes, cs, kind, steps, warmup, seed, pattern = args
    from oracle import pyoracle
    seq = [s.copy() for s in series(pattern, nbytes, cs, 1 + warmup + steps, seed)]
    d = pyoracle.Deduplicator(pyoracle.TREE, cs, kind)
    d.checkpoint(seq[0], True)
    for s in seq[1:1 + warmup]:
        d.checkpoint(s, False)
    t0 = time.perf_counter()
    for s in seq[1 + warmup:]:
        d.checkpoint(s, False)
    return time.perf_counter() - t0


def run_reference(a, ws, rank):
    if rank != 0:
        return 0
    import multiprocessing as mp
    kind = 1 if a.hash == "md5" else 0
    cores = os.cpu_count() or 1
    total = int(a.size_gib * GIB)
    # bounded sample: every host thread deduplicates an independent slice of
    # the buffer; the aggregate covers the whole configured size
    per = max(a.chunk, (total // cores) // a.chunk * a.chunk)
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        t = pool.map(reference_worker, [(per, a.chunk, kind, a.steps, a.warmup, 1000 + i, a.pattern)
                                        for i in range(cores)])
    elapsed = max(t)
    value = per * cores * a.steps / elapsed / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": ws,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(elapsed / a.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": "tree dedup, %s, %.3g GiB buffer, %d B chunks, %s"
                   % (a.hash, a.size_gib, a.chunk, PATTERN_NAME[a.pattern]), "approach": "tree", "hash": a.hash},
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": cores, "kind": "port",
                         "sample": "%d host processes, each deduplicating an independent %d MiB slice (own map and "
                                   "tree) for %d timed incremental checkpoints after a baseline and %d warm-up"
                                   % (cores, per >> 20, a.steps, a.warmup)},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


class _DevView:
    """A device address range as a torch tensor (via __cuda_array_interface__)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (int(n),), "typestr": "|u1", "data": (int(ptr), False),
                                         "version": 3}


def batch_bench(torch, mc, dev, a):
    """96 buffers of log-normal sizes (1-512 MiB, about 12 GiB), chunk sizes
    {64, 128, 512, 4096}, Murmur3/MD5 alternating, tree approach, 5 checkpoints
    of the 4 GiB update pattern with a per-buffer change rate of 0.1-10%:
    (i) one buffer per call through lone handles, (ii) one batched call per
    step (eager baseline, CUDA graph replays after), on the same device
    buffers; every member's diff compared byte for byte on the device."""
    from mtcheck_gb300 import workloads
    mix = workloads.batch_mix(count=a.batch_count, median_mib=a.batch_median_mib)
    total = sum(m["nbytes"] for m in mix)
    gens, bufs = [], []
    for m in mix:
        z = (m["nbytes"] // 4, m["nbytes"] // 4 + m["nbytes"] // 8)
        g = workloads.pattern2(m["nbytes"], m["chunk_size"], a.batch_steps, seed=m["seed"], device=dev,
                               rate=(m["rate"], m["rate"]), zero_range=z)
        gens.append(g)
        bufs.append(next(g))
    lone = [mc.TreeDeduplicator(m["chunk_size"], m["hash"]) for m in mix]
    b = mc.Batch([(mc.TREE, m["hash"], m["chunk_size"]) for m in mix])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if not a.batch_no_tune:
        b.autotune(bufs)
    tune_s = time.perf_counter() - t0
    tunes = [m.tuning() for m in b.members]
    # the members' state reserved in one allocation of their pool; timed and
    # counted in the batched job (in its baseline step)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reserved = b.reserve(bufs)
    reserve_s = time.perf_counter() - t0
    per_call, batched, batched_dev, identical, diff_total = [], [], [], True, 0
    per_call_dev, host_parts, mismatches = [], [], []
    all_pc, all_b = [], []
    l0 = mc.launch_count()
    for step in range(a.batch_steps):
        if step:
            for i, g in enumerate(gens):
                bufs[i] = next(g)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lens, pdev = [], 0.0
        for d, x in zip(lone, bufs):
            lens.append(d.checkpoint_device(x, step == 0))
            pdev += sum(d.info().timers[:3])
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        blens = b.checkpoint(bufs, make_baseline=(step == 0))
        t2 = time.perf_counter()
        info = b.info()
        all_pc.append(t1 - t0)
        all_b.append(t2 - t1 + (reserve_s if step == 0 else 0.0))
        if step == 0:
            baseline_host = [round(x, 3) for x in info.host_ms]
        if step:
            per_call.append(t1 - t0)
            per_call_dev.append(pdev)
            batched.append(t2 - t1)
            batched_dev.append(info.last_device_ms / 1e3)
            host_parts.append(list(info.host_ms))
        for i, (d, mem, n, bn) in enumerate(zip(lone, b.members, lens, blens)):
            pa, na = d.diff_device()
            pb, nb = mem.diff_device()
            same = na == nb and n == bn
            if same:
                ta = torch.as_tensor(_DevView(pa, na), device=dev)
                tb = torch.as_tensor(_DevView(pb, nb), device=dev)
                same = bool(torch.equal(ta, tb))
                if not same and len(mismatches) < 8:
                    first = int(torch.nonzero(ta != tb)[0].item())
                    mismatches.append({"member": i, "step": step, "len": na, "first_byte": first,
                                       "chunk_size": mix[i]["chunk_size"], "hash": mix[i]["hash"],
                                       "nbytes": mix[i]["nbytes"], "tune": tunes[i]})
            elif len(mismatches) < 8:
                mismatches.append({"member": i, "step": step, "len": [n, na, bn, nb],
                                   "chunk_size": mix[i]["chunk_size"], "hash": mix[i]["hash"],
                                   "nbytes": mix[i]["nbytes"], "tune": tunes[i]})
            identical = identical and same
            diff_total += nb
    launches = mc.launch_count() - l0
    info = b.info()
    inc = a.batch_steps - 1
    pc = sum(per_call) / inc
    bt = sum(batched) / inc
    steady = sum(batched[1:]) / max(1, inc - 1)
    res = {
        "workload": "%d buffers, log-normal sizes %.0f MiB median clipped to [1, 512] MiB (%.2f GiB total), chunk "
                    "sizes {64,128,512,4096}, Murmur3/MD5 alternating, tree approach, %d checkpoints, change rate "
                    "0.1-10%% per buffer, 4 GiB update pattern" % (len(mix), a.batch_median_mib, total / GIB,
                                                                   a.batch_steps),
        "unit": "GB/s",
        "per_call_value": round(total / pc / 1e9, 3),
        "batched_value": round(total / bt / 1e9, 3),
        "batched_steady_value": round(total / steady / 1e9, 3),
        "batched_device_value": round(total / (sum(batched_dev) / inc) / 1e9, 3),
        "speedup": round(sum(all_pc) / sum(all_b), 3),
        "speedup_incremental": round(pc / bt, 3),
        "speedup_steady": round(pc / steady, 3),
        "job_s": {"per_call": round(sum(all_pc), 4), "batched": round(sum(all_b), 4)},
        "baseline_s": {"per_call": round(all_pc[0], 4), "batched": round(all_b[0], 4)},
        "reserve": {"seconds": round(reserve_s, 4), "bytes": reserved,
                    "note": "mtc_batch_reserve before the first step; counted in the batched baseline step"},
        "baseline_host_ms": dict(zip(("prepare", "capture", "issue", "wait", "complete"), baseline_host)),
        "per_call_ms": round(pc * 1e3, 3), "batched_ms": round(bt * 1e3, 3),
        "batched_steady_ms": round(steady * 1e3, 3),
        "identical_to_per_call": identical,
        "mismatches": mismatches,
        "per_call_device_ms": round(sum(per_call_dev) / inc * 1e3, 3),
        "batched_host_ms": {k: round(sum(h[j] for h in host_parts) / inc, 3)
                            for j, k in enumerate(["prepare", "capture", "issue", "wait", "complete"])},
        "diff_bytes_total": int(diff_total),
        "graph": {"captures": int(info.graph_captures), "nodes": int(info.graph_nodes),
                  "kernels_per_step": int(info.kernels_per_step)},
        "autotune": {"seconds": round(tune_s, 2),
                     "distinct_choices": sorted({json.dumps(t, sort_keys=True) for t in tunes})},
        "gpu_launches": int(launches),
        "note": "per_call: one mtc_checkpoint per buffer through lone handles (host wall time incl. its "
                "synchronisation); batched: one mtc_batch_checkpoint per step (wall time; the first incremental "
                "step includes the graph capture). speedup: whole job (all checkpoints, baseline included); "
                "*_value, speedup_incremental: incremental steps; steady: incremental steps after the first; "
                "device: fork-to-join CUDA events of the batched step",
    }
    for d in lone:
        d.close()
    b.close()
    return res


def _digest2(mc, kind, buf):
    """A 16-byte digest of a device buffer: the digests of its 4 KiB pieces,
    then of 4 KiB pieces of those, until one piece is left (a few short
    launches with a thread per piece, so that the verification does not hold
    the default stream that the requests are ordered after)."""
    d = mc.hash_chunks(kind, buf, 4096)
    while d.numel() > 4096:
        d = mc.hash_chunks(kind, d, 4096)
    return mc.hash_chunks(kind, d, d.numel())


def serve_bench(torch, mc, dev, a):
    """256 processes with buffers of 2^k bytes, k uniform in 22..28 (4-256 MiB),
    128 B chunks, Murmur3, tree approach.  Requests arrive as a Poisson stream
    at --serve-rate per second for --serve-seconds; 5% are restarts of a random
    earlier checkpoint of the process; a checkpoint first applies one step of
    the 4 GiB update pattern (change rate 0.5-5%).  A process has at most one
    request on the server; later arrivals for it wait, and latency runs from
    the arrival time to completion.  Before the timed stream every process
    makes one incremental checkpoint and every buffer size one restart
    (warm-up).  The update steps are drawn before the
    stream starts (DeviceUpdates) so that the client loop keeps up with the rate.
    Every restart is verified against a digest of the state it restores; a
    sample of processes is replayed alone through lone handles and compared
    byte for byte with the served chain."""
    from collections import deque
    import numpy as np
    from mtcheck_gb300 import workloads
    mix = workloads.serve_mix(count=a.serve_procs)
    P = len(mix)
    kind = mc.MURMUR3
    srv = mc.Server(hbm_budget=int(a.serve_budget_gb * 1e9), max_inflight=a.serve_inflight, use_graph=True,
                    reserve_hbm=True, pinned_reserve=int(a.serve_pinned_gb * (1 << 30)))
    pids = [srv.add_process(mc.TREE, kind, m["chunk_size"]) for m in mix]
    assert pids == list(range(P))
    zr = [(m["nbytes"] // 4, m["nbytes"] // 4 + m["nbytes"] // 8) for m in mix]
    bufs = [workloads.init_device(torch.empty(m["nbytes"], dtype=torch.uint8, device=dev), m["seed"], zr[i])
            for i, m in enumerate(mix)]
    maxn = max(m["nbytes"] for m in mix)
    outs = [torch.empty(maxn, dtype=torch.uint8, device=dev) for _ in range(8)]
    free_outs = list(range(len(outs)))
    rng = np.random.default_rng(11)
    rates = [float(rng.uniform(*m["rate"])) for m in mix]
    plans = [workloads.DeviceUpdates(bufs[i], m["chunk_size"], rates[i], m["seed"], zero_range=zr[i])
             for i, m in enumerate(mix)]
    # baselines (not timed)
    t_base = time.perf_counter()
    for i, pid in enumerate(pids):
        srv.submit_checkpoint(pid, bufs[i], make_baseline=True)
    srv.drain()
    base = srv.poll(0)
    while len(base) < P:
        base += srv.poll(100)
    assert all(c["status"] == 0 for c in base)
    base_s = time.perf_counter() - t_base
    step = [1] * P
    pending_checks = []
    # warm-up, not timed: one incremental checkpoint per process, then one
    # restart per buffer size (first use of every kernel, of the allocator
    # sizes of the update step, of the restart scratch)
    for p in range(P):
        plans[p].apply(bufs[p], 1)
        srv.submit_checkpoint(pids[p], bufs[p])
    got = []
    while len(got) < P:
        got += srv.poll(100)
    assert all(c["status"] == 0 for c in got)
    step = [2] * P
    for nb in sorted(set(m["nbytes"] for m in mix)):
        p = next(i for i, m in enumerate(mix) if m["nbytes"] == nb)
        srv.submit_restart(pids[p], 1, outs[0][:nb])
        srv.drain()
        c = srv.poll(100)
        assert len(c) == 1 and c[0]["status"] == 0, c
        pending_checks.append((p, 1, _digest2(mc, kind, outs[0][:nb])))
    rst_ok, rst_checked = True, 0

    def stream(arr, is_rst, who, trace=None, stalls=None):
        """Requests arriving at offsets `arr` (ms); returns the latencies,
        (arrival offset, latency) pairs, bytes served and the wall time from
        the first arrival to the last completion.  `trace`, a list, receives
        one row per request: arrival, submission, admission and completion
        (ms from the start), kind, process, buffer bytes; `stalls`, a dict,
        the longest single call of each kind the client made (ms, at ms)."""
        def timed_call(name, f, *args):
            if stalls is None:
                return f(*args)
            t = mc.now_ms()
            r = f(*args)
            dt = mc.now_ms() - t
            if dt > stalls.get(name, (0.0, 0.0))[0]:
                stalls[name] = (round(dt, 3), round(t - t0, 1))
            return r

        n_req = len(arr)
        queues = [deque() for _ in range(P)]
        busy = [None] * P
        ready = set()
        lat = {"checkpoint": [], "restart": []}
        lat_t = []
        nbytes_done = 0
        t0 = mc.now_ms() + 20.0
        i = 0
        t_last = t0
        outstanding = 0
        while i < n_req or outstanding or ready:
            now = mc.now_ms()
            while i < n_req and t0 + arr[i] <= now:
                p = int(who[i])
                queues[p].append((t0 + arr[i], bool(is_rst[i])))
                if busy[p] is None:
                    ready.add(p)
                i += 1
            for p in list(ready):
                arrival, r = queues[p][0]
                if r:
                    if not free_outs:
                        continue
                    slot = free_outs.pop()
                    target = int(rng.integers(0, step[p]))
                    n = mix[p]["nbytes"]
                    timed_call("submit_restart", srv.submit_restart, pids[p], target, outs[slot][:n])
                    busy[p] = ("restart", arrival, target, slot)
                else:
                    timed_call("apply_update", plans[p].apply, bufs[p], step[p])
                    timed_call("submit_checkpoint", srv.submit_checkpoint, pids[p], bufs[p])
                    busy[p] = ("checkpoint", arrival, step[p], None)
                    step[p] += 1
                queues[p].popleft()
                ready.discard(p)
                outstanding += 1
            t_poll = mc.now_ms()
            done = srv.poll(0.0 if (ready or (i < n_req and t0 + arr[i] <= mc.now_ms() + 0.05)) else 0.2)
            if stalls is not None and done:
                dt = mc.now_ms() - t_poll
                if dt > stalls.get("poll", (0.0, 0.0))[0]:
                    stalls["poll"] = (round(dt, 3), round(t_poll - t0, 1))
            for c in done:
                p = c["pid"]  # this server's process ids are 0..P-1 in order
                what, arrival, target, slot = busy[p]
                assert c["status"] == 0, c
                lat[what].append(c["t_done_ms"] - arrival)
                lat_t.append((arrival - t0, c["t_done_ms"] - arrival))
                if trace is not None:
                    trace.append((round(arrival - t0, 3), round(c["t_submit_ms"] - t0, 3),
                                  round(c["t_admit_ms"] - t0, 3), round(c["t_done_ms"] - t0, 3), what, p,
                                  mix[p]["nbytes"]))
                nbytes_done += mix[p]["nbytes"]
                t_last = max(t_last, c["t_done_ms"])
                if what == "restart":
                    pending_checks.append((p, target, timed_call("verify_digest", _digest2, mc, kind,
                                                                 outs[slot][:mix[p]["nbytes"]])))
                    free_outs.append(slot)
                busy[p] = None
                outstanding -= 1
                if queues[p]:
                    ready.add(p)
        return lat, lat_t, nbytes_done, (t_last - t0) / 1e3

    # the request stream: Poisson arrivals at the configured rate
    n_req = int(a.serve_rate * a.serve_seconds)
    arr = np.cumsum(rng.exponential(1.0 / a.serve_rate, n_req)) * 1e3
    trace = [] if a.serve_trace else None
    client_max = {}
    lat, lat_t, nbytes_done, wall = stream(arr, rng.random(n_req) < 0.05, rng.integers(0, P, n_req), trace,
                                           client_max)
    st_stream = srv.stats()
    if trace is not None:
        with open(a.serve_trace, "w") as f:
            f.write("arrival_ms,submit_ms,admit_ms,done_ms,kind,process,bytes\n")
            for row in trace:
                f.write(",".join(str(x) for x in row) + "\n")
    # capacity: the same kind of requests all arriving at once (each process
    # still has one request on the server at a time)
    n_sat = a.serve_sat_requests
    P_sat = min(P, a.serve_sat_procs)
    sat_rst = rng.random(n_sat) < 0.05
    sat_who = rng.integers(0, P_sat, n_sat)
    lat_s, _, bytes_s, wall_s = stream(np.zeros(n_sat), sat_rst, sat_who)
    sat_lat = lat_s["checkpoint"] + lat_s["restart"]
    # the one-buffer-per-call path on the same requests: one lone handle per
    # process (a baseline of the process's current state first, untimed),
    # every request a synchronous call in arrival order, each new checkpoint
    # kept in HBM for the restarts as the server keeps its chains
    pc_bufs = [b.clone() for b in bufs[:P_sat]]
    lones = [mc.TreeDeduplicator(m["chunk_size"], kind) for m in mix[:P_sat]]
    pc_chain = [[] for _ in range(P_sat)]

    def keep_diff(p):
        ptr, ln = lones[p].diff_device()
        pc_chain[p].append(torch.as_tensor(_DevView(ptr, ln), device=dev).clone())

    for p in range(P_sat):
        lones[p].checkpoint_device(pc_bufs[p], True)
        keep_diff(p)
    pc_step = list(step)
    rng_pc = np.random.default_rng(12)
    torch.cuda.synchronize()
    t_pc = time.perf_counter()
    for r, p in zip(sat_rst, sat_who):
        p = int(p)
        if r:
            target = int(rng_pc.integers(0, len(pc_chain[p])))
            lones[p].restart_device(outs[0][:mix[p]["nbytes"]],
                                    [(x.data_ptr(), x.numel()) for x in pc_chain[p]], target)
        else:
            plans[p].apply(pc_bufs[p], pc_step[p])
            pc_step[p] += 1
            lones[p].checkpoint_device(pc_bufs[p], False)
            keep_diff(p)
    torch.cuda.synchronize()
    wall_pc = time.perf_counter() - t_pc
    for d in lones:
        d.close()
    del lones, pc_bufs, pc_chain
    torch.cuda.empty_cache()
    saturation = {
        "requests": n_sat, "restarts": int(sat_rst.sum()), "processes": P_sat,
        "served_rate": round(n_sat / wall_s, 1), "served_gbs": round(bytes_s / wall_s / 1e9, 3),
        "per_call_rate": round(n_sat / wall_pc, 1),
        "speedup_vs_per_call": round(wall_pc / wall_s, 3),
        "served_latency_ms": {"p50": round(float(np.percentile(sat_lat, 50)), 3),
                              "p99": round(float(np.percentile(sat_lat, 99)), 3)},
        "note": "all requests arrive at once, for the first `processes` processes; served: the request server "
                "(continuous admission, overlapped on the device); per_call: one synchronous call per request "
                "through one lone handle per process, starting from a baseline of the same states, each "
                "checkpoint kept in HBM",
    }
    st = srv.stats()
    # every restart against the state it restores: replay each process's
    # updates (deterministic per seed and step) into a scratch buffer
    need = {}
    for p, target, got in pending_checks:
        need.setdefault(p, []).append((target, got))
    scratch = torch.empty(maxn, dtype=torch.uint8, device=dev)
    for p, items in need.items():
        m = mix[p]
        b = workloads.init_device(scratch[:m["nbytes"]], m["seed"], zr[p])
        for k in range(max(t for t, _ in items) + 1):
            if k:
                plans[p].apply(b, k)
            exp = None
            for t, got in items:
                if t == k:
                    exp = _digest2(mc, kind, b) if exp is None else exp
                    rst_checked += 1
                    rst_ok = rst_ok and bool(torch.equal(got, exp))
    del scratch
    # a sample of processes alone, through lone handles: byte-identical chains
    alone_ok, alone_checked = True, 0
    sample = sorted(set(int(x) for x in np.linspace(0, P - 1, a.serve_verify_procs)))
    for p in sample:
        m = mix[p]
        b = workloads.init_device(torch.empty(m["nbytes"], dtype=torch.uint8, device=dev), m["seed"], zr[p])
        d = mc.TreeDeduplicator(m["chunk_size"], kind)
        for k in range(step[p]):
            if k:
                plans[p].apply(b, k)
            alone_ok = alone_ok and d.checkpoint(b, k == 0) == srv.diff(pids[p], k)
            alone_checked += 1
        d.close()
        del b
    srv.close()

    def pct(v, q):
        return round(float(np.percentile(v, q)), 3) if v else None
    allv = lat["checkpoint"] + lat["restart"]
    late = [v for t, v in lat_t if t >= 1000.0]
    per_s = {}
    for t, v in lat_t:
        per_s.setdefault(int(t // 1000), []).append(v)
    return {
        "workload": "%d processes, buffers 2^k B with k uniform in 22..28 (%.1f GiB), 128 B chunks, Murmur3, tree "
                    "approach; Poisson arrivals at %.0f requests/s for %.1f s, 5%% restarts of a random earlier "
                    "checkpoint, change rate 0.5-5%% per checkpoint (4 GiB update pattern); %.0f GB HBM budget; "
                    "timed after one untimed incremental checkpoint per process"
                    % (P, sum(m["nbytes"] for m in mix) / GIB, a.serve_rate, a.serve_seconds, a.serve_budget_gb),
        "value": round(nbytes_done / wall / 1e9, 3), "unit": "GB/s",
        "requests": n_req, "achieved_rate": round(len(allv) / wall, 1),
        "latency_ms": {"p50": pct(allv, 50), "p99": pct(allv, 99), "mean": round(float(np.mean(allv)), 3),
                       "checkpoint_p50": pct(lat["checkpoint"], 50), "checkpoint_p99": pct(lat["checkpoint"], 99),
                       "restart_p50": pct(lat["restart"], 50), "restart_p99": pct(lat["restart"], 99),
                       "after_first_second_p50": pct(late, 50), "after_first_second_p99": pct(late, 99),
                       "p99_per_second": [pct(per_s[k], 99) for k in sorted(per_s)]},
        "saturation": saturation,
        "restarts_verified": rst_checked, "restarts_identical": rst_ok,
        "alone_vs_mix": {"processes": len(sample), "checkpoints": alone_checked, "identical": alone_ok},
        "baseline_s": round(base_s, 2),
        "cuda_device_max_connections": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"),
        "server": {k: st[k] for k in ("inflight_peak", "graph_captures", "graph_replays", "spilled_diffs",
                                      "spilled_bytes", "spilled_states", "restored_states", "staged_diffs",
                                      "hbm_peak", "pinned_reserved", "pinned_sync_grows", "deferred_admissions",
                                      "failed", "worker_ms", "worker_max_ms", "pool_reserved_high",
                                      "pool_used_high")},
        "torch_allocator": {k: torch.cuda.memory_stats().get(k) for k in ("num_alloc_retries", "num_device_alloc",
                                                                         "num_device_free")},
        "client_max_ms": {k: {"ms": v[0], "at_ms": v[1]} for k, v in sorted(client_max.items())},
        "server_after_stream": {k: st_stream[k] for k in ("spilled_diffs", "spilled_bytes", "spilled_states",
                                                          "restored_states", "staged_diffs", "hbm_peak",
                                                          "deferred_admissions", "worker_max_ms")},
        "note": "value: bytes of all completed requests (checkpointed and restarted buffers) / time from the first "
                "arrival to the last completion; latency: arrival to completion (diff archived in HBM, or "
                "restarted buffer written)",
    }


def summary_of(line):
    """The headline figures of every section in one small object, printed
    last on the line."""
    def g(d, *ks):
        for k in ks:
            if not isinstance(d, dict) or d.get(k) is None:
                return None
            d = d[k]
        return d
    return {
        "dedup_4gib_512b_murmur3_gbs": line["value"],
        "dedup_checkpoint_roofline_frac": g(line, "config", "checkpoint_roofline_frac"),
        "leaf_kernel_roofline_frac": g(line, "roofline", "frac"),
        "e2e_gbs": g(line, "e2e", "value"),
        "e2e_frac_of_link": g(line, "e2e", "link_frac"),
        "dedup_4gib_512b_md5_gbs": g(line, "md5", "value"),
        "md5_leaf_alu_pipe_frac": g(line, "md5", "leaf_alu_pipe_frac_ncu"),
        "dedup_64mib_128b_gbs": g(line, "series_64mib", "value"),
        "dedup_64mib_128b_ms": g(line, "series_64mib", "ms"),
        "dedup_64mib_128b_roofline_frac": g(line, "series_64mib", "roofline_frac"),
        "restart_1gib_256b_gbs": g(line, "restart", "value"),
        "restart_roofline_frac": g(line, "restart", "roofline_frac"),
        "restart_host_chain_gbs": g(line, "restart", "host_chain_value"),
        "restart_verified": g(line, "restart", "verified_byte_identical"),
        "batched_speedup_job": g(line, "batched", "speedup"),
        "batched_speedup_incremental": g(line, "batched", "speedup_incremental"),
        "batched_identical": g(line, "batched", "identical_to_per_call"),
        "served_gbs": g(line, "served", "value"),
        "served_p50_ms": g(line, "served", "latency_ms", "p50"),
        "served_p99_ms": g(line, "served", "latency_ms", "p99"),
        "served_capacity_vs_per_call": g(line, "served", "saturation", "speedup_vs_per_call"),
    }


def section_in_subprocess(flag, key, a):
    """Run one section (`--only-serve`, `--only-batch`) in a fresh process of
    this script with the section's options, and return its object.  The
    served stream and the batch each measured worse in a process that had
    run the other first (worker calls six times slower after the batch;
    the batch's first allocations 35 times slower after the server), so
    each is measured as a user would run it, in a process of its own."""
    args = [sys.executable, os.path.abspath(__file__), flag]
    for name in ("serve_procs", "serve_rate", "serve_seconds", "serve_budget_gb", "serve_inflight",
                 "serve_verify_procs", "serve_pinned_gb", "serve_sat_procs", "serve_sat_requests",
                 "batch_count", "batch_median_mib", "batch_steps"):
        args += ["--" + name.replace("_", "-"), str(getattr(a, name))]
    args += ["--hash", a.hash]
    if a.batch_no_tune:
        args.append("--batch-no-tune")
    if a.serve_trace:
        args += ["--serve-trace", a.serve_trace]
    env = dict(os.environ, RANK="0", LOCAL_RANK=os.environ.get("LOCAL_RANK", "0"), WORLD_SIZE="1")
    r = subprocess.run(args, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        return {"error": "section process exited %d: %s" % (r.returncode, r.stderr.strip().splitlines()[-1:])}
    for line in reversed(r.stdout.strip().splitlines()):
        if line.startswith("{"):
            return json.loads(line).get(key)
    return {"error": "section process printed no result"}


def bind_local_cpus(torch, local):
    """Pin this process to the CPUs next to the GPU (sysfs local_cpulist of
    its PCI function), so that pinned host buffers are allocated on the GPU's
    own memory node.  Returns the CPU list, or None when sysfs does not say."""
    try:
        p = torch.cuda.get_device_properties(local)
        path = "/sys/bus/pci/devices/%04x:%02x:%02x.0/local_cpulist" % (p.pci_domain_id, p.pci_bus_id,
                                                                          p.pci_device_id)
        spec = open(path).read().strip()
        cpus = set()
        for part in spec.split(","):
            lo, _, hi = part.partition("-")
            cpus.update(range(int(lo), int(hi or lo) + 1))
        if not cpus or not hasattr(os, "sched_setaffinity"):
            return None
        os.sched_setaffinity(0, cpus & os.sched_getaffinity(0) or cpus)
        return spec
    except (OSError, ValueError, AttributeError):
        return None


def main():
    a = parse()
    ws, rank, local = dist_setup()
    if a.impl == "reference":
        return run_reference(a, ws, rank)
    import numpy as np
    import torch
    import mtcheck_gb300 as mc

    torch.cuda.set_device(local)
    host_cpus = bind_local_cpus(torch, local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    mc.load()
    kind = mc.MD5 if a.hash == "md5" else mc.MURMUR3
    if a.only_batch:
        print(json.dumps({"batched": batch_bench(torch, mc, torch.device("cuda", local), a)}), flush=True)
        return 0
    if a.only_serve:
        print(json.dumps({"served": serve_bench(torch, mc, torch.device("cuda", local), a)}), flush=True)
        return 0
    if a.only_restart:
        print(json.dumps({"restart": restart_bench(torch, mc, torch.device("cuda", local), a, kind)}), flush=True)
        return 0
    cs = a.chunk
    nbytes = int(a.size_gib * GIB) // cs * cs
    N = (nbytes + cs - 1) // cs
    dev = torch.device("cuda", local)
    K, W = a.steps, a.warmup
    states = make_states(torch, nbytes, cs, 1 + W + K, seed=77 + rank, device=dev, pattern=a.pattern)
    torch.cuda.synchronize()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- device-resident timing -------------------------------------------
    dd = mc.TreeDeduplicator(cs, kind)
    dd.checkpoint_device(states[0], True)
    for s in states[1:1 + W]:
        dd.checkpoint_device(s, False)
    leaf_t, tree_t, asm_t, ckpt_t, sizes, sdata, smeta = [], [], [], [], [], [], []
    # inputs that fit in L2 (129 MB) several times over: every step timed on
    # its own, after a 256 MiB write that flushes L2 (outside its events)
    small = nbytes < (512 << 20)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev) if small else None
    step_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    l0 = mc.launch_count()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        start.record()
        for i, s in enumerate(states[1 + W:]):
            if small:
                flush.zero_()
                step_ev[i][0].record()
            n = dd.checkpoint_device(s, False)
            if small:
                step_ev[i][1].record()
            info = dd.info()
            leaf_t.append(info.phase_times[0])
            tree_t.append(info.phase_times[1])
            asm_t.append(info.timers[2])
            ckpt_t.append(sum(info.timers[:3]))
            sizes.append(n)
            sdata.append(info.data_size)
            smeta.append(info.metadata_size)
        stop.record()
        barrier()
    launches = mc.launch_count() - l0
    if small:
        timed = sum(e0.elapsed_time(e1) for e0, e1 in step_ev) / 1e3
    else:
        timed = start.elapsed_time(stop) / 1e3
    elapsed = max_over_ranks(torch, timed, dev, ws)
    value = whole_job_rate(nbytes * K, elapsed, ws)

    # roofline of the dominant kernel (leaf hashing): per chunk the chunk bytes,
    # the previous leaf digest read and the new leaf digest write
    peak, peak_kind = load_peaks()
    leaf_bytes = N * (cs + 32)
    leaf_avg = sum(leaf_t) / len(leaf_t)
    achieved = leaf_bytes / leaf_avg / 1e9
    tr = load_traffic()
    traffic = None
    if tr and tr.get("chunk_size") == cs and tr.get("hash") == a.hash:
        traffic = int(round(tr["dram_bytes_per_chunk"] * N))
    # whole checkpoint: B_dedup = D + 32 N + 2 S_data + S_meta
    b_dedup = nbytes + 32 * N + 2 * (sum(sdata) / K) + sum(smeta) / K
    ckpt_frac = b_dedup / (elapsed / K) / 1e9 / peak

    # ---- end to end through the C ABI with host buffers --------------------
    e2e = None
    if not a.no_e2e:
        host = [s.cpu().pin_memory() for s in states[1 + W:]]
        devbuf = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        # two device input buffers: step i+1 uploads on a side stream while
        # step i is checkpointed (every upload stays inside the timed region)
        bufs = [devbuf, torch.empty(nbytes, dtype=torch.uint8, device=dev)]
        side = torch.cuda.Stream(device=dev)
        ready = [torch.cuda.Event(), torch.cuda.Event()]
        # one pinned result buffer for the largest diff a checkpoint can have
        # (header, region and repeat metadata, every chunk), allocated before
        # the timed region
        max_diff = nbytes + 12 * (N + 1) + 32 + 8 * 4096
        pinned_out = torch.empty(max_diff, dtype=torch.uint8).pin_memory()
        out_view = pinned_out.numpy()
        de = mc.TreeDeduplicator(cs, kind)
        # the handle works on its own stream, ordered after each upload by an
        # event, so that the next upload runs beside it
        work = torch.cuda.Stream(device=dev)
        de.set_stream(work.cuda_stream)
        devbuf.copy_(states[W])
        work.wait_stream(torch.cuda.current_stream())
        de.checkpoint_device(devbuf, True)
        # the copy engines' first pass over newly pinned pages runs at a
        # fraction of the link rate; every host buffer is moved once before
        # timing, as staging buffers reused from step to step would have been
        for h in host:
            bufs[1].copy_(h, non_blocking=True)
        pinned_out[:nbytes].copy_(bufs[1], non_blocking=True)
        # W untimed steps through the same path (upload, checkpoint, copy out),
        # then the handle starts again from the same baseline
        for i in range(W):
            bufs[i % 2].copy_(host[i % len(host)], non_blocking=True)
            work.wait_stream(torch.cuda.current_stream())
            n = de.checkpoint_device(bufs[i % 2], False)
            de.copy_diff(out_view[:n])
        devbuf.copy_(states[W])
        work.wait_stream(torch.cuda.current_stream())
        de.checkpoint_device(devbuf, True)
        barrier()

        def upload(i):
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                bufs[i % 2].copy_(host[i], non_blocking=True)
                ready[i % 2].record(side)

        t0 = time.perf_counter()
        d2h = 0
        marks = []
        upload(0)
        for i in range(len(host)):
            work.wait_event(ready[i % 2])
            if i + 1 < len(host):
                upload(i + 1)  # the other buffer's last checkpoint has returned
            n = de.checkpoint_device(bufs[i % 2], False)
            de.copy_diff(out_view[:n])
            d2h += n
            marks.append(time.perf_counter())
        barrier()
        te = max_over_ranks(torch, time.perf_counter() - t0, dev, ws)
        e2e = {"value": round(whole_job_rate(nbytes * K, te, ws), 3), "unit": "GB/s", "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": int(d2h / K),
               "host_buffers": "pinned; each input and the result buffer moved once, then W untimed steps through "
                               "the same path, before timing",
               "step_ms": [round((b - a) * 1e3, 2) for a, b in zip([t0] + marks[:-1], marks)]}
        del host, pinned_out, out_view, bufs

    # the served stream and the batch run in processes of their own
    srvd = None
    if not a.no_serve and rank == 0:
        torch.cuda.empty_cache()
        srvd = section_in_subprocess("--only-serve", "served", a)

    md5 = small = None
    if rank == 0 and not a.no_sections:
        md5 = md5_section(torch, mc, dev, states[:1 + W + K], cs, W, peak)
    if rank == 0 and e2e is not None:
        # the link bounds e2e: every input byte crosses it once
        link = link_section(torch, dev)
        h2d = max(link["h2d_gbs"].values())
        e2e["link"] = dict(link, note="pinned 1 GiB copies split over 1, 2 and 4 streams; kernels reading pinned "
                                      "or pageable host memory directly measured the same ceiling")
        e2e["link_frac"] = round(e2e["value"] / h2d, 3)
    rst = None
    if not a.no_restart and rank == 0:
        del states
        torch.cuda.empty_cache()
        rst = restart_bench(torch, mc, dev, a, kind)
        torch.cuda.empty_cache()
        rst["other_approaches"] = {}
        for name, ap in (("list", mc.LIST), ("basic", mc.BASIC)):
            r2 = restart_bench(torch, mc, dev, a, kind, ap)
            rst["other_approaches"][name] = {k: r2[k] for k in ("value", "ms", "verified_byte_identical",
                                                                 "digest_matches_original", "host_chain_value",
                                                                 "chain_bytes")}
            torch.cuda.empty_cache()

    if rank == 0 and not a.no_sections:
        torch.cuda.empty_cache()
        small = small_series_section(torch, mc, dev, peak)
        torch.cuda.empty_cache()

    bat = None
    if not a.no_batch and rank == 0:
        torch.cuda.empty_cache()
        bat = section_in_subprocess("--only-batch", "batched", a)

    cpu = None
    if rank == 0 and ws == 1 and not a.no_cpu:
        v, nsteps = cpu_sample(1 if a.hash == "md5" else 0, cs, a.pattern, nbytes)
        cpu = {"value": round(v, 3), "unit": "GB/s", "cores": 1, "kind": "port",
               "sample": "oracle restatement, one host thread, %d MiB buffer of the same update pattern and chunk "
                         "size, mean of %d incremental checkpoints after a baseline" % (min(nbytes, GIB) >> 20,
                                                                                      nsteps)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": ws, "steps": K, "warmup": W,
            "ms_per_step": round(elapsed / K * 1e3, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": "tree dedup (lowest offset), %s, %.3g GiB buffer, %d B chunks, incremental "
                                   "checkpoints of %s" % (a.hash, a.size_gib, cs, PATTERN_NAME[a.pattern]),
                       "approach": "tree", "hash": a.hash, "buffer_bytes": nbytes, "chunk_size": cs,
                       "chunks": N,
                       "l2": ("L2 flushed before every step (256 MiB write outside the step's events)" if small
                              else "inputs (%d MiB) larger than L2" % (nbytes >> 20)),
                       "parallelism": "replicas" if ws > 1 else "single GPU",
                       "host_cpus": host_cpus,
                       "diff_bytes_mean": int(sum(sizes) / K),
                       "checkpoint_roofline_frac": round(ckpt_frac, 4),
                       "phase_ms_mean": {"leaf_hash": round(leaf_avg * 1e3, 4),
                                         "labels_forest_roots": round(sum(tree_t) / K * 1e3, 4),
                                         "diff_assembly": round(sum(asm_t) / K * 1e3, 4),
                                         "checkpoint_device": round(sum(ckpt_t) / K * 1e3, 4)}},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic,
                         "kernel": "leaf_tma_kernel (chunk hashing + classification)",
                         "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                         else "fallback 6.8 TB/s"},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "md5": md5,
            "series_64mib": small,
            "restart": rst,
            "batched": bat,
            "served": srvd,
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
        }
        line["summary"] = summary_of(line)
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
