"""The N > 1 host logic of bench.py on CPU: two gloo ranks (replicas only,
one independent instance per rank) reduce their times to the maximum, and
the reference arm prints from rank 0 alone."""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, _ = bench.dist_env()
    got = bench.max_over_ranks(10.0 + 5.0 * rank, w)
    with open(os.path.join(outdir, "rank%d.json" % rank), "w") as f:
        json.dump({"world": w, "rank": r, "max": got,
                   "seed": bench.replica_seed(3, r)}, f)
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_to_the_maximum(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    out = [json.load(open(tmp_path / ("rank%d.json" % r))) for r in range(2)]
    assert [o["world"] for o in out] == [2, 2] and [o["rank"] for o in out] == [0, 1]
    assert [o["max"] for o in out] == [15.0, 15.0]
    assert [o["seed"] for o in out] == [3, 4]  # one independent instance per rank


def test_single_rank_needs_no_process_group(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.delenv("RANK", raising=False)
    assert bench.dist_env()[:2] == (1, 0)
    assert bench.max_over_ranks(7.5, 1) == 7.5


def test_reference_arm_is_silent_off_rank_zero(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    assert bench.run_reference(bench.parse()) == 0
    assert capsys.readouterr().out == ""
