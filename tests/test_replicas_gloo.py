"""The multi-rank path of bench.py on CPU: two gloo ranks (one process each,
as torchrun launches them) agree on the max-over-ranks time, meet at the
barriers, and the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    d.barrier()
    m = d.max(float(10 * (rank + 1)))
    d.barrier()

    class Args:
        warmup, steps, gpus = 1, 1, world
    rc = bench.run_reference(Args, d) if rank == 1 else 0  # rank > 0 returns without work
    d.close()
    out.put((rank, m, rc))


def test_two_gloo_ranks_max_and_barrier():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert [r[1] for r in res] == [20.0, 20.0]
    assert [r[2] for r in res] == [0, 0]


def test_each_rank_sees_only_its_gpu(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "4,5")
    assert bench.bind_gpu() == "5" and os.environ["CUDA_VISIBLE_DEVICES"] == "5"
    monkeypatch.delenv("CUDA_VISIBLE_DEVICES")
    assert bench.bind_gpu() == "1" and os.environ["CUDA_VISIBLE_DEVICES"] == "1"
    monkeypatch.setenv("WORLD_SIZE", "1")
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "3")
    assert bench.bind_gpu() == "3" and os.environ["CUDA_VISIBLE_DEVICES"] == "3"
