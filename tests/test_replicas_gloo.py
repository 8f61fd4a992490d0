"""Independent replicas across ranks (cs_afqmc_gb300.replicas) on the CPU: two gloo ranks
spawned as processes (127.0.0.1), the max-over-ranks timing of the benchmark and the
per-block gather of driver.py:262-296 (every rank's weight, energy and observable in rank
order and the population's block energy sum(w E) / sum(w)); and the one-process path."""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str):
    import torch
    import torch.distributed as dist

    from cs_afqmc_gb300 import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        m = replicas.max_over_ranks(1.5 + rank)
        w, e, o, be = replicas.gather_block(1.0 + rank, -10.0 - rank, 0.5 * rank)
        torch.save({"max": m, "w": w, "e": e, "o": o, "be": be}, os.path.join(out_dir, f"r{rank}.pt"))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    import torch
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    for rank in range(world):
        r = torch.load(tmp_path / f"r{rank}.pt")
        assert r["max"] == 2.5
        assert r["w"].tolist() == [1.0, 2.0]
        assert r["e"].tolist() == [-10.0, -11.0]
        assert r["o"].tolist() == [0.0, 0.5]
        assert r["be"] == pytest.approx((1.0 * -10.0 + 2.0 * -11.0) / 3.0, rel=1e-15)


def test_single_process():
    from cs_afqmc_gb300 import replicas
    assert replicas.max_over_ranks(3.25) == 3.25
    w, e, o, be = replicas.gather_block(2.0, -7.0, 1.0)
    assert w.tolist() == [2.0] and e.tolist() == [-7.0] and o.tolist() == [1.0] and be == -7.0
