"""Multi-rank checkpoint files: the per-rank file selection of the reference's
MPI driver (src/dedup_files_mpi.cpp:26-128) on one GB300.

    python -m mtcheck_gb300.ranks chunk_size num_chkpts <mode> [--ranks R] [--dry-run] files...

Rank r deduplicates, in order, the files whose path contains "Rank<r>"
(a substring test, as in the reference: "Rank1" also matches "Rank10"),
the first as its baseline, and writes <file> + the approach's suffix; one
process per rank also writes the CSV logs under the file's base name, like
dedup_chkpt_files.

* Under torchrun (WORLD_SIZE > 1) every rank is a process with its own
  handle; the ranks only meet at barriers (gloo), as the reference's ranks meet
  at MPI_Barrier, and no data moves between them.
* In one process, --ranks R serves all R ranks' chains through one request
  server (mtc_server_*): each rank is a server process, and their checkpoints
  overlap on the GPU.
* --dry-run prints each rank's selection and stops (no GPU needed).

The reference iterates over num_chkpts entries of the filtered list, which
runs past its end whenever the filter drops files; here each rank runs the
files it selected.
"""
import os
import sys

import numpy as np

FLAGS = {"--run-full-chkpt": 1, "--run-basic-chkpt": 2, "--run-list-chkpt": 3, "--run-tree-chkpt": 4,
         "--run-tree-low-offset-ref-chkpt": 5, "--run-tree-low-offset-chkpt": 6,
         "--run-tree-low-root-ref-chkpt": 7, "--run-tree-low-root-chkpt": 8}
SUFFIX = {1: ".full_chkpt", 2: ".basic.incr_chkpt", 3: ".hashlist.incr_chkpt"}


def rank_files(files, rank):
    """The files rank `rank` reads (src/dedup_files_mpi.cpp:54-65)."""
    tag = "Rank%d" % rank
    return [f for f in files if tag in f]


def _approach(mode):
    # the reference driver runs every tree flag on the tree deduplicator
    return mode if mode in (1, 2, 3) else 4


def _parse(argv):
    if len(argv) < 3:
        raise SystemExit("usage: python -m mtcheck_gb300.ranks chunk_size num_chkpts <mode> "
                         "[--ranks R] [--dry-run] files...")
    cs, num = int(argv[0]), int(argv[1])
    mode, ranks, dry, files = 0, None, False, []
    it = iter(argv[2:])
    for a in it:
        if a in FLAGS:
            mode = FLAGS[a]
        elif a == "--ranks":
            ranks = int(next(it))
        elif a == "--dry-run":
            dry = True
        else:
            files.append(a)
    if mode == 0:
        raise SystemExit("ERROR: Incorrect mode")
    return cs, num, mode, ranks, dry, files[:num]


def _checkpoint_lone(cs, approach, files):
    import torch
    import mtcheck_gb300 as mc
    d = mc.Deduplicator(cs, mc.MURMUR3, approach=approach)
    for i, path in enumerate(files):
        data = np.fromfile(path, dtype=np.uint8)
        buf = torch.from_numpy(data).cuda()
        d.checkpoint_file(buf, path + SUFFIX.get(approach, ".hashtree.incr_chkpt"), os.path.basename(path), i == 0)
    d.close()


def _checkpoint_served(cs, approach, per_rank):
    """All ranks' chains through one server; files written after draining."""
    import torch
    import mtcheck_gb300 as mc
    srv = mc.Server()
    pids = [srv.add_process(approach, mc.MURMUR3, cs) for _ in per_rank]
    bufs = [None] * len(per_rank)
    nxt = [0] * len(per_rank)
    busy = [False] * len(per_rank)
    while any(nxt[r] < len(f) for r, f in enumerate(per_rank)) or any(busy):
        for r, f in enumerate(per_rank):
            if not busy[r] and nxt[r] < len(f):
                bufs[r] = torch.from_numpy(np.fromfile(f[nxt[r]], dtype=np.uint8)).cuda()
                srv.submit_checkpoint(pids[r], bufs[r], make_baseline=(nxt[r] == 0))
                busy[r] = True
        for c in srv.poll(wait_ms=50):
            if c["status"] != 0:
                raise RuntimeError("rank %d checkpoint failed (status %d)" % (c["pid"], c["status"]))
            busy[c["pid"]] = False
            nxt[c["pid"]] += 1
    for r, f in enumerate(per_rank):
        for k, path in enumerate(f):
            with open(path + SUFFIX.get(approach, ".hashtree.incr_chkpt"), "wb") as out:
                out.write(srv.diff(pids[r], k))
    srv.close()


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    cs, num, mode, ranks, dry, files = _parse(argv)
    approach = _approach(mode)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        rank = int(os.environ["RANK"])
        dist.init_process_group("gloo")
        print("MPI COMM SIZE: %d, MPI_RANK: %d" % (world, rank), flush=True)
        dist.barrier()
        mine = rank_files(files, rank)
        if dry:
            print("rank %d: %s" % (rank, " ".join(mine)), flush=True)
        else:
            _checkpoint_lone(cs, approach, mine)
        dist.barrier()
        dist.destroy_process_group()
        return 0
    n = ranks or 1
    per_rank = [rank_files(files, r) for r in range(n)]
    if dry:
        for r, f in enumerate(per_rank):
            print("rank %d: %s" % (r, " ".join(f)))
        return 0
    _checkpoint_served(cs, approach, [f for f in per_rank if f])
    return 0


if __name__ == "__main__":
    sys.exit(main())
