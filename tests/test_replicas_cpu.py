"""The multi-GPU form of the benchmark is replicas (one independent batch per
GPU, no data-path collective): whole-job throughput = all ranks' solves over
the slowest rank's time.  The rank logic runs here as two gloo processes."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank r solved 10 + r systems in 1 + r seconds
    v = bench.replica_throughput(10 + rank, 1.0 + rank, world)
    out.put((rank, v))
    dist.destroy_process_group()


def test_replica_throughput_two_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # (10 + 11) solves over the slowest rank's 2 s, the same number on every rank
    assert res[0] == pytest.approx(10.5) and res[1] == pytest.approx(10.5)


def test_replica_throughput_one_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_throughput(512, 0.5, 1) == 1024.0


def test_heldout_seeds_are_disjoint_across_ranks():
    """Each replica solves its own block of held-out instances: the work is
    sharded, not repeated, and no rank's block overlaps the training seeds."""
    sys.path.insert(0, ROOT)
    import bench
    blocks = [set(bench.heldout_seeds(r).tolist()) for r in range(8)]
    for r, b in enumerate(blocks):
        assert len(b) == bench.NEVAL
        assert min(b) >= bench.NTRAIN
        for q in range(r):
            assert not (b & blocks[q])


def test_batch_bytes_counts_shared_tables_once():
    """The index tables of the shared grid are charged once per round of the
    batched loop, so doubling the systems doubles only the per-system part."""
    sys.path.insert(0, ROOT)
    import types
    import bench
    info = {"nnodes": 66049, "nedges": 197120, "nblocks": 460289}
    h = [types.SimpleNamespace(nnewton=3, nlin=90 + i % 7) for i in range(8)]
    tot1, sys1, sh1 = bench.batch_bytes(info, h, 196)
    tot2, sys2, sh2 = bench.batch_bytes(info, h + h, 196)
    assert tot1 == sys1 + sh1 and tot2 == sys2 + sh2
    assert sys2 == 2 * sys1 and sh2 == sh1
