"""The multi-GPU (replica) path of bench.py on CPU: two gloo ranks, the
barrier and max-over-ranks timing, the whole-job rate, and the reference arm
printing on rank 0 only. No GPU and no data-path collective are involved."""
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
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench

    rep = bench.Replicas()
    assert (rep.rank, rep.world) == (rank, world)
    rep.barrier()
    t = rep.max(10.0 + rank)  # each rank's own timing; the job is as slow as the slowest
    rate = bench.aggregate_rate(1000, rep.world, 5, t)
    rep.barrier()
    rep.close()
    with open(os.path.join(out, f"r{rank}"), "w") as f:
        f.write(f"{t} {rate}")


def test_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as tmp

    port = _free_port()
    tmp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        t, rate = map(float, (tmp_path / f"r{r}").read_text().split())
        assert t == 11.0
        assert rate == pytest.approx(1000 * 2 * 5 / 0.011)


def test_reference_arm_prints_on_rank0_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    assert bench.run_reference(None) is None
