"""The N-GPU bench path on CPU: world_size-2 gloo ranks run the bench's own
host logic (max-over-ranks step time, whole-job throughput, per-rank seeds),
the bench's replica launcher (``python bench.py --gpus N`` without torchrun)
end to end, and the reference arm's rank gating.  No GPU is involved."""

import os
import socket
import sys

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    import bench
    from jaxtronomy_gb300 import workloads as W
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms_local = 3.0 + rank  # rank 1 is the slow one
        ms = bench.max_over_ranks(ms_local, dist, "cpu")
        value = bench.job_rate(1024, world, ms)
        _, lens, _, _, _ = W.batch_epl(seed=bench.rank_seed(1001, rank), batch=4, num_pix=16,
                                       kernel_size=5)
        dist.barrier()
        out[rank] = (ms, value, float(lens[0]["theta_E"][0]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_share_the_slowest_step_time():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 4.0  # max over ranks
    assert res[0][1] == res[1][1] == pytest.approx(1024 * 2 / 4.0e-3)
    assert res[0][2] != res[1][2]  # each replica has its own batch


def test_single_rank_helpers():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(2.5) == 2.5
    assert bench.job_rate(1024, 1, 3.5) == pytest.approx(1024 / 3.5e-3)
    assert bench.rank_seed(1001, 3) == 1004


def test_reference_arm_other_ranks_do_no_work(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")

    class A:
        steps, warmup, gpus = 1, 1, 2
    assert bench.reference_arm(A()) == 0
    assert capsys.readouterr().out == ""


def _launcher_worker(out_path):
    """A replica of the launcher test: joins the group from the environment the
    launcher set, takes the max over ranks of a per-rank step time and lets rank
    0 write one bench-style line."""
    import json
    sys.path.insert(0, ROOT)
    import bench
    rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
    assert os.environ["LOCAL_RANK"] == str(rank)
    dist.init_process_group("gloo")
    try:
        ms = bench.max_over_ranks(2.0 + rank, dist, "cpu")
        if rank == 0:
            with open(out_path, "w") as f:
                f.write(json.dumps({"n_gpus": world, "value": bench.job_rate(1024, world, ms),
                                    "ms_per_step": ms}) + "\n")
    finally:
        dist.destroy_process_group()
    return 0


def test_replica_launcher_runs_two_ranks(tmp_path):
    import json
    sys.path.insert(0, ROOT)
    import bench
    out = tmp_path / "line.json"
    assert bench.launch_replicas(2, _launcher_worker, str(out)) == 0
    lines = out.read_text().splitlines()
    assert len(lines) == 1
    rec = json.loads(lines[0])
    assert rec["n_gpus"] == 2 and rec["ms_per_step"] == 3.0
    assert rec["value"] == pytest.approx(1024 * 2 / 3.0e-3)
