"""Replica path of bench.py at world_size 2 on the gloo backend (CPU).

The path does not shard: each rank advances its own simulation, so the only
cross-rank traffic is the barrier around the timed region and the max of
the ranks' times. Checked here: both ranks see the slowest rank's time, the
whole-job rate counts every rank's points over that time, and the
reference arm runs on rank 0 alone.
"""
import contextlib
import io
import json
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    r, w, dist = bench.dist_init()
    assert (r, w) == (rank, world) and dist is not None
    assert dist.get_backend() == "gloo"
    bench.barrier(dist)
    ms = 10.0 * (rank + 1)                       # rank 1 is the slow replica
    ms_max = bench.max_over_ranks(dist, ms)
    buf = io.StringIO()
    if rank != 0:
        with contextlib.redirect_stdout(buf):
            bench.run_reference(None, rank, world)
    bench.barrier(dist)
    dist.destroy_process_group()
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
        json.dump({"ms_max": ms_max, "ref_stdout": buf.getvalue()}, f)


@pytest.mark.timeout(120)
def test_two_replicas(tmp_path):
    world = 2
    mp.start_processes(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    res = [json.load(open(tmp_path / ("rank%d.json" % r))) for r in range(world)]
    assert [x["ms_max"] for x in res] == [20.0, 20.0]
    assert res[1]["ref_stdout"] == ""


def test_job_rate():
    import bench
    pts = 1025 * 193 * 32
    one = bench.job_rate(1, pts, 10, 1.0)
    assert one == pytest.approx(pts * 10 / 1e6)
    assert bench.job_rate(2, pts, 10, 1.0) == pytest.approx(2 * one)
    assert bench.job_rate(2, pts, 10, 2.0) == pytest.approx(one)
