"""The multi-GPU form of the bench is independent replicas (one process per GPU, no
collective on the data path): rank setup, the barrier around the timed region and the
max-over-ranks timing, run here as two gloo ranks on CPU."""
import json
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    os.environ.update({"WORLD_SIZE": str(world), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench
    w, r, local = bench.dist_setup()
    bench.barrier(w)
    # rank r took (r + 1) ms per step on 1 GB: the job runs at the slowest rank's pace
    value, ms = bench.replica_throughput(1e9, float(r + 1), w)
    m = bench.max_over_ranks(10.0 * (r + 1), w)
    bench.barrier(w)
    (Path(out_dir) / f"rank{r}.json").write_text(json.dumps(
        {"world": w, "rank": r, "local": local, "backend": dist.get_backend(), "value": value, "ms": ms, "max": m}))
    dist.destroy_process_group()


def test_two_gloo_replicas(tmp_path):
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r in range(2):
        d = json.loads((tmp_path / f"rank{r}.json").read_text())
        assert d["world"] == 2 and d["rank"] == r and d["local"] == r and d["backend"] == "gloo"
        assert d["ms"] == 2.0 and d["max"] == 20.0
        assert abs(d["value"] - 2 * 1e9 / 2e-3 / 1e9) < 1e-9  # 2 ranks x 1 GB in 2 ms = 1000 GB/s


def test_reference_arm_other_ranks_exit_without_work(capsys):
    sys.path.insert(0, str(ROOT))
    import argparse

    import bench
    args = argparse.Namespace(gpus=2, steps=1, warmup=3)
    assert bench.run_reference(args, 2, 1) == 0
    assert capsys.readouterr().out == ""
