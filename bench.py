"""Benchmark of the GB300 incremental-checkpoint deduplicator.

Default workload: tree approach (lowest-offset rule), Murmur3, one 4 GiB
buffer in 512-byte chunks, seeded synthetic states with the 4 GiB update
pattern (0.1-5% of chunks change per step, half sparse, half runs of up to
4096 chunks, 10% shifted duplicates, [1 GiB, 1.5 GiB) zero-filled).  A step is
one incremental checkpoint of the whole buffer.

  value : buffer bytes / device time per checkpoint, inputs resident in HBM,
          diff assembled in HBM (GB/s, whole job over all ranks)
  e2e   : the same through the C ABI with pinned host buffers: H2D of the
          state, checkpoint, D2H of the diff inside the timed region

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
    p.add_argument("--no-e2e", action="store_true")
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


def make_states(torch, nbytes, cs, count, seed, device):
    from mtcheck_gb300 import workloads
    z = (GIB, GIB + GIB // 2) if nbytes >= 2 * GIB else (nbytes // 4, nbytes // 4 + nbytes // 8)
    states = []
    for s in workloads.pattern2(nbytes, cs, count, seed=seed, device=device, zero_range=z):
        states.append(s.clone())
    return states


def restart_bench(torch, mc, dev, a, kind):
    """Restart of the last checkpoint of a chain (1 GiB, 256 B chunks, 30
    incrementals after a baseline, 4 GiB update pattern), tree approach."""
    from mtcheck_gb300 import workloads
    nbytes = int(a.restart_gib * GIB) // a.restart_chunk * a.restart_chunk
    z = (nbytes // 4, nbytes // 4 + nbytes // 8)
    d = mc.TreeDeduplicator(a.restart_chunk, kind)
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
    r = mc.TreeDeduplicator(a.restart_chunk, kind)
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
    return {"workload": "restart of checkpoint %d of a tree chain, %.3g GiB buffer, %d B chunks, 4 GiB update "
                        "pattern" % (rid, a.restart_gib, a.restart_chunk),
            "value": round(nbytes / dev_t / 1e9, 3), "unit": "GB/s", "ms": round(dev_t * 1e3, 3),
            "call_ms": round(call_t * 1e3, 3),
            "chain_bytes": int(chain_bytes), "verified_byte_identical": ok,
            "host_chain_value": round(nbytes / statistics.median(e2e_t) / 1e9, 3),
            "host_chain_ms": round(statistics.median(e2e_t) * 1e3, 3),
            "note": "value: device time with the chain resident in HBM; call_ms adds the host side of the call; "
                    "host_chain_value: chain in pageable host memory, copied to HBM inside the call"}


def cpu_sample(kind, cs, seconds_hint=20.0):
    """Single-thread oracle on a 1 GiB sample of the same pattern: baseline + incrementals."""
    import numpy as np
    from mtcheck_gb300 import workloads
    from oracle import pyoracle
    n = GIB
    z = (n // 4, n // 4 + n // 8)
    seq = workloads.pattern2(n, cs, 4, seed=123, zero_range=z)
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
    nbytes, cs, kind, steps, warmup, seed = args
    from mtcheck_gb300 import workloads
    from oracle import pyoracle
    z = (nbytes // 4, nbytes // 4 + nbytes // 8)
    seq = [s.copy() for s in workloads.pattern2(nbytes, cs, 1 + warmup + steps, seed=seed, zero_range=z)]
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
        t = pool.map(reference_worker, [(per, a.chunk, kind, a.steps, a.warmup, 1000 + i) for i in range(cores)])
    elapsed = max(t)
    value = per * cores * a.steps / elapsed / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": ws,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(elapsed / a.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": "tree dedup, %s, %.3g GiB buffer, %d B chunks, 4 GiB update pattern"
                   % (a.hash, a.size_gib, a.chunk), "approach": "tree", "hash": a.hash},
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
        all_b.append(t2 - t1)
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


def main():
    a = parse()
    ws, rank, local = dist_setup()
    if a.impl == "reference":
        return run_reference(a, ws, rank)
    import numpy as np
    import torch
    import mtcheck_gb300 as mc

    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    mc.load()
    kind = mc.MD5 if a.hash == "md5" else mc.MURMUR3
    if a.only_batch:
        print(json.dumps({"batched": batch_bench(torch, mc, torch.device("cuda", local), a)}), flush=True)
        return 0
    cs = a.chunk
    nbytes = int(a.size_gib * GIB) // cs * cs
    N = (nbytes + cs - 1) // cs
    dev = torch.device("cuda", local)
    K, W = a.steps, a.warmup
    states = make_states(torch, nbytes, cs, 1 + W + K, seed=77 + rank, device=dev)
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
    leaf_t, ckpt_t, sizes, sdata, smeta = [], [], [], [], []
    l0 = mc.launch_count()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        start.record()
        for s in states[1 + W:]:
            n = dd.checkpoint_device(s, False)
            info = dd.info()
            leaf_t.append(info.phase_times[0])
            ckpt_t.append(sum(info.timers[:3]))
            sizes.append(n)
            sdata.append(info.data_size)
            smeta.append(info.metadata_size)
        stop.record()
        barrier()
    launches = mc.launch_count() - l0
    elapsed = start.elapsed_time(stop) / 1e3
    tmax = torch.tensor([elapsed], device=dev)
    if ws > 1:
        torch.distributed.all_reduce(tmax, op=torch.distributed.ReduceOp.MAX)
    elapsed = float(tmax.item())
    value = nbytes * K * ws / elapsed / 1e9

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
        outs = [np.empty(sz, dtype=np.uint8) for sz in sizes]
        pinned_out = [torch.empty(sz, dtype=torch.uint8).pin_memory() for sz in sizes]
        de = mc.TreeDeduplicator(cs, kind)
        devbuf.copy_(states[W])
        de.checkpoint_device(devbuf, True)
        barrier()
        t0 = time.perf_counter()
        d2h = 0
        for i, h in enumerate(host):
            devbuf.copy_(h, non_blocking=True)
            n = de.checkpoint_device(devbuf, False)
            if pinned_out[i].numel() < n:
                pinned_out[i] = torch.empty(n, dtype=torch.uint8).pin_memory()
            de.copy_diff(pinned_out[i].numpy())
            d2h += n
        barrier()
        te = time.perf_counter() - t0
        te_t = torch.tensor([te], device=dev)
        if ws > 1:
            torch.distributed.all_reduce(te_t, op=torch.distributed.ReduceOp.MAX)
        te = float(te_t.item())
        e2e = {"value": round(nbytes * K * ws / te / 1e9, 3), "unit": "GB/s", "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": int(d2h / K)}
        del host, pinned_out, outs

    rst = None
    if not a.no_restart and rank == 0:
        del states
        torch.cuda.empty_cache()
        rst = restart_bench(torch, mc, dev, a, kind)

    bat = None
    if not a.no_batch and rank == 0:
        torch.cuda.empty_cache()
        bat = batch_bench(torch, mc, dev, a)
        torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and ws == 1 and not a.no_cpu:
        v, nsteps = cpu_sample(1 if a.hash == "md5" else 0, cs)
        cpu = {"value": round(v, 3), "unit": "GB/s", "cores": 1, "kind": "port",
               "sample": "oracle restatement, one host thread, 1 GiB buffer of the same update pattern and chunk "
                         "size, mean of %d incremental checkpoints after a baseline" % nsteps}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": ws, "steps": K, "warmup": W,
            "ms_per_step": round(elapsed / K * 1e3, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": "tree dedup (lowest offset), %s, %.3g GiB buffer, %d B chunks, incremental "
                                   "checkpoints of the 4 GiB update pattern" % (a.hash, a.size_gib, cs),
                       "approach": "tree", "hash": a.hash, "buffer_bytes": nbytes, "chunk_size": cs,
                       "chunks": N, "l2": "inputs (%d MiB) larger than L2" % (nbytes >> 20),
                       "parallelism": "replicas" if ws > 1 else "single GPU",
                       "diff_bytes_mean": int(sum(sizes) / K),
                       "checkpoint_roofline_frac": round(ckpt_frac, 4),
                       "phase_ms_mean": {"leaf_hash": round(leaf_avg * 1e3, 4),
                                         "checkpoint_device": round(sum(ckpt_t) / K * 1e3, 4)}},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic,
                         "kernel": "leaf_tma_kernel (chunk hashing + classification)",
                         "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                         else "fallback 6.8 TB/s"},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "restart": rst,
            "batched": bat,
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
