"""The multi-GPU path of bench.py (replicas only): one process per GPU, each
rank on the GPU of its LOCAL_RANK, a host-side gloo group for the barriers
and the reductions (work summed, time maximised).  Two ranks on the CPU."""
import multiprocessing as mp
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="3,5")
    import bench
    r = bench.Ranks()
    r.barrier()
    out = (rank, r.sum(10.0 * (rank + 1)), r.max(1.0 + rank), os.environ["CUDA_VISIBLE_DEVICES"], r.world)
    r.barrier()
    r.close()
    q.put(out)


def test_ranks_take_their_gpu_and_reduce_over_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(i, port, q)) for i in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 30.0, 2.0, "3", 2), (1, 30.0, 2.0, "5", 2)]


def test_single_process_needs_no_group():
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    r = bench.Ranks()
    assert r.world == 1 and r.dist is None
    r.barrier()
    assert r.sum(3.5) == 3.5 and r.max(2.0) == 2.0
