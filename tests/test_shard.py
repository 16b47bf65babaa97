"""Region sharding across ranks (gloo, world size 2, CPU): the partition
covers every region exactly once and the concatenated per-rank records equal
the single-process records.  The per-rank compute here is the oracle (the
data path needs no GPU to test the host logic)."""
import os
import socket

import torch.distributed as dist
import torch.multiprocessing as mp


def test_partition_properties():
    from rabbitvar_gb300.shard import partition
    w = [5, 1, 9, 9, 3, 0, 7, 2, 2, 8]
    for n in (1, 2, 3, 4, 7):
        parts = partition(w, n)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(w)))
        loads = [sum(max(w[i], 1) for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(w)
    assert partition(w, 3) == partition(w, 3)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "oracle"))
    import oracle as O
    from rabbitvar_gb300 import synth
    from rabbitvar_gb300.shard import estimate_reads, shard_regions
    g, vs, rs = synth.dense_multi(length=30_000, depth=30.0)
    regions = [(1 + 3000 * i, 3000 * (i + 1)) for i in range(10)]
    w = estimate_reads(rs.pos, regions)
    mine, idx = shard_regions(regions, w, rank, world)
    n, text = O.run_regions(rs, g, mine, params=O.default_params(local_realign=0))
    gathered = [None] * world
    dist.all_gather_object(gathered, (idx, text))
    if rank == 0:
        out.put(gathered)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_shards_equal_single_process():
    import oracle as O
    from rabbitvar_gb300 import synth
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    g, vs, rs = synth.dense_multi(length=30_000, depth=30.0)
    regions = [(1 + 3000 * i, 3000 * (i + 1)) for i in range(10)]
    _, single = O.run_regions(rs, g, regions, params=O.default_params(local_realign=0))
    merged = sorted(l for _, t in gathered for l in t.splitlines())
    assert merged == sorted(single.splitlines())
    covered = sorted(i for idx, _ in gathered for i in idx)
    assert covered == list(range(10))
