"""The N > 1 host path of bench.py on CPU: two gloo ranks on 127.0.0.1.

The commit path does not shard across GPUs (one replica per GPU, no data
exchange), so what runs across ranks is the bench's own bookkeeping: the
whole-job throughput is the units of all ranks over the slowest rank's time,
and the reference arm runs on rank 0 only."""
import json
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        units = [100.0, 300.0][rank]
        ms = [10.0, 20.0][rank]
        value, max_ms = bench.job_throughput(units, ms)
        ws, r, local = bench.dist_info()

        class A:
            steps, warmup, gpus = 1, 0, world
        ref_rc = bench.run_reference(A) if rank == 1 else None
        dist.barrier()
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump({"value": value, "max_ms": max_ms, "ws": ws, "rank": r, "local": local,
                       "ref_rc": ref_rc}, f)
    finally:
        dist.destroy_process_group()


def test_two_rank_throughput_and_rank0_only_reference(tmp_path, capfd):
    mp = pytest.importorskip("torch.multiprocessing")
    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    for r, d in enumerate(res):
        assert d["ws"] == 2 and d["rank"] == r and d["local"] == r
        assert d["max_ms"] == 20.0
        assert d["value"] == pytest.approx(400.0 / 0.020)
    # rank 1 of the reference arm does no work and prints nothing
    assert res[1]["ref_rc"] == 0
    assert '"impl": "reference"' not in capfd.readouterr().out


def test_single_process_throughput_needs_no_process_group():
    sys.path.insert(0, REPO)
    import bench
    value, ms = bench.job_throughput(50.0, 5.0)
    assert ms == 5.0 and value == pytest.approx(10000.0)
