"""The request-serving loop (mtc_server_*): every process's incremental
checkpoints and restarts are byte-identical to a lone handle's on the same
buffers, alone or in a mix of processes whose requests overlap on the GPU,
with or without spilling to pinned host memory under a small HBM budget."""
import numpy as np
import pytest

from mtcheck_gb300 import workloads

pytestmark = pytest.mark.gpu
FILL = 0x5A
STEPS = 6

# (approach, hash, chunk size, bytes)
PROCS = [
    (4, 0, 128, 1 << 20),
    (4, 1, 64, (1 << 19) + 64 * 11),
    (3, 0, 512, 3 << 19),
    (2, 1, 256, 1 << 20),
    (5, 0, 128, 1 << 19),
    (1, 0, 4096, 1 << 18),
    (4, 0, 4096, (4096 * 300) + 9),
    (3, 1, 128, 700 * 1000),
    (4, 1, 512, 1 << 21),
    (4, 0, 64, 1 << 18),
]


def proc_states(i, cs, nbytes):
    z = (nbytes // 4, nbytes // 4 + nbytes // 8)
    return [s.copy() for s in workloads.pattern2(nbytes, cs, STEPS, seed=500 + i, rate=(0.005, 0.05),
                                                 run_max=128, zero_range=z)]


def plan(i):
    """Checkpoints 0..STEPS-1 with restarts of earlier checkpoints in between."""
    acts = []
    for k in range(STEPS):
        acts.append(("ckpt", k))
        if k in (2, 4):
            acts.append(("restart", (k * 7 + i) % (k + 1)))
    return acts


@pytest.fixture(scope="module")
def states():
    return [proc_states(i, p[2], p[3]) for i, p in enumerate(PROCS)]


@pytest.fixture(scope="module")
def lone(cuda, mtc, states):
    """Per process: lone-handle diffs, and restarts of every checkpoint."""
    out = []
    for (approach, kind, cs, nbytes), seq in zip(PROCS, states):
        d = mtc.Deduplicator(cs, kind, approach=approach)
        diffs = [d.checkpoint(cuda.from_numpy(s).cuda(), k == 0) for k, s in enumerate(seq)]
        rst = []
        for k in range(STEPS):
            o = cuda.full((nbytes,), FILL, dtype=cuda.uint8, device="cuda")
            d.restart(o, diffs[:k + 1], k)
            rst.append(o.cpu().numpy())
        out.append((diffs, rst))
        d.close()
    return out


def serve(cuda, mtc, states, procs, srv):
    """Drive every process's plan through the server; a process submits its
    next request once the previous one completed.  Returns restart outputs."""
    pids = [srv.add_process(a, h, cs) for a, h, cs, _ in procs]
    bufs = [cuda.empty(n, dtype=cuda.uint8, device="cuda") for *_, n in procs]
    outs = [cuda.empty(n, dtype=cuda.uint8, device="cuda") for *_, n in procs]
    todo = [list(plan(i)) for i in range(len(procs))]
    busy = [None] * len(procs)
    restarts = {}
    while any(todo) or any(b is not None for b in busy):
        for i, pid in enumerate(pids):
            if busy[i] is None and todo[i]:
                act = todo[i].pop(0)
                if act[0] == "ckpt":
                    bufs[i].copy_(cuda.from_numpy(states[i][act[1]]))
                    srv.submit_checkpoint(pid, bufs[i], make_baseline=(act[1] == 0))
                else:
                    outs[i].fill_(FILL)
                    srv.submit_restart(pid, act[1], outs[i])
                busy[i] = act
        for c in srv.poll(wait_ms=100):
            i = pids.index(c["pid"])
            assert c["status"] == 0, (i, busy[i], c)
            if busy[i][0] == "restart":
                # complete on the GPU: read it on the legacy stream, no device-wide sync
                restarts[(i, busy[i][1])] = outs[i].cpu().numpy()
            else:
                assert c["chkpt_id"] == busy[i][1]
            assert c["t_submit_ms"] <= c["t_admit_ms"] <= c["t_done_ms"]
            busy[i] = None
    return pids, restarts


def check(mtc, srv, pids, restarts, lone):
    for i, pid in enumerate(pids):
        diffs, rst = lone[i]
        assert srv.chain_length(pid) == STEPS
        for k in range(STEPS):
            assert srv.diff(pid, k) == diffs[k], (i, k)
    for (i, k), got in restarts.items():
        assert np.array_equal(got, lone[i][1][k]), (i, k)


@pytest.mark.parametrize("use_graph", [True, False], ids=["graph", "eager"])
def test_mix_equals_lone_handles(cuda, mtc, states, lone, use_graph):
    srv = mtc.Server(max_inflight=16, use_graph=use_graph)
    pids, restarts = serve(cuda, mtc, states, PROCS, srv)
    check(mtc, srv, pids, restarts, lone)
    st = srv.stats()
    assert st["completed"] == st["submitted"] == len(PROCS) * (STEPS + 2) and st["failed"] == 0
    assert st["inflight_peak"] > 1          # requests of different processes overlapped
    assert (st["graph_replays"] > 0) == use_graph
    srv.close()


def test_each_process_alone(cuda, mtc, states, lone):
    # the same plans, one process per server: results equal the mix's
    for i in (0, 2, 3):
        srv = mtc.Server()
        pids, restarts = serve(cuda, mtc, [states[i]], [PROCS[i]], srv)
        check(mtc, srv, pids, restarts, [lone[i]])
        srv.close()


def test_spill_under_small_budget(cuda, mtc, states, lone):
    # about one process's state fits: the others spill and come back
    srv = mtc.Server(hbm_budget=12 << 20, max_inflight=4, use_graph=True)
    pids, restarts = serve(cuda, mtc, states, PROCS, srv)
    check(mtc, srv, pids, restarts, lone)
    st = srv.stats()
    assert st["spilled_diffs"] > 0 and st["spilled_states"] > 0 and st["restored_states"] > 0
    assert st["failed"] == 0
    srv.close()


def test_spill_without_graphs(cuda, mtc, states, lone):
    # the six processes' states total about 12.5 MB: 8 MiB forces state spills
    srv = mtc.Server(hbm_budget=8 << 20, max_inflight=8)
    pids, restarts = serve(cuda, mtc, states[:6], PROCS[:6], srv)
    check(mtc, srv, pids, restarts, lone[:6])
    st = srv.stats()
    assert st["graph_replays"] == 0 and st["spilled_states"] > 0
    srv.close()


def test_request_larger_than_budget_fails(cuda, mtc):
    srv = mtc.Server(hbm_budget=1 << 20)
    pid = srv.add_process(4, 0, 128)
    buf = cuda.zeros(16 << 20, dtype=cuda.uint8, device="cuda")
    srv.submit_checkpoint(pid, buf, make_baseline=True)
    srv.drain()
    c = srv.poll()
    assert len(c) == 1 and c[0]["status"] == 3  # MTC_ENOMEM
    srv.close()


def test_bad_arguments(cuda, mtc):
    srv = mtc.Server()
    with pytest.raises(mtc.MtcError):
        srv.add_process(9, 0, 128)
    buf = cuda.zeros(4096, dtype=cuda.uint8, device="cuda")
    with pytest.raises(mtc.MtcError):
        srv.submit_checkpoint(3, buf)
    pid = srv.add_process(4, 0, 128)
    srv.submit_restart(pid, 5, buf)  # no checkpoint 5 yet: the request fails
    srv.drain()
    c = srv.poll()
    assert c[0]["status"] == 1
    srv.close()


def test_device_update_pattern_is_deterministic(cuda, mtc):
    # the request-stream generator replays to the same states (no racing writes)
    a = workloads.init_device(cuda.empty(3 << 20, dtype=cuda.uint8, device="cuda"), 9, (1 << 20, 3 << 19))
    b = workloads.init_device(cuda.empty(3 << 20, dtype=cuda.uint8, device="cuda"), 9, (1 << 20, 3 << 19))
    assert cuda.equal(a, b)
    for k in range(1, 6):
        workloads.mutate_device(a, 128, 0.05, seed=100 + k, run_max=512, zero_range=(1 << 20, 3 << 19))
        workloads.mutate_device(b, 128, 0.05, seed=100 + k, run_max=512, zero_range=(1 << 20, 3 << 19))
        assert cuda.equal(a, b), k
