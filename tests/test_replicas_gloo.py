"""The multi-rank path of the benchmark on CPU: two gloo ranks each solve the
same scene with the CPU oracle (no data-path collective), then aggregate
substeps (sum), time (max) and state checksums (gather) exactly as the
benchmark does over NCCL."""
import json
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, oracle, out):
    sys.path[:0] = [str(REPO / "kami-hair-solver_gb300"), str(REPO / "tests")]
    import time

    import khs_native as kn
    import replicas
    import scenes

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lib = kn.Library(oracle)
    lib.lib.khsOracleSetThreads(1)
    sc = scenes.sphere_scene(motion=True, frames=1)
    s = kn.HairSolver(lib)
    scenes.load_into(s, sc)
    t0 = time.perf_counter()
    assert s._library.khsStepAnimationFrame(s.handle, 1, sc.frame_dt) == kn.OK
    seconds = time.perf_counter() - t0
    sub = s.stats().substeps
    agg = replicas.aggregate(sub, seconds, replicas.state_checksum(s.state()[0]), dist, "cpu")
    s.close()
    if rank == 0:
        Path(out).write_text(json.dumps(dict(agg, local_substeps=sub, local_seconds=seconds)))
    dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_replicas(oracle_path, tmp_path):
    out = tmp_path / "agg.json"
    mp.spawn(_rank, args=(2, _free_port(), str(oracle_path), str(out)), nprocs=2, join=True)
    agg = json.loads(out.read_text())
    assert agg["world"] == 2
    assert agg["substeps"] == 2 * agg["local_substeps"]
    assert agg["max_seconds"] >= agg["local_seconds"]
    assert agg["value"] == pytest.approx(agg["substeps"] / agg["max_seconds"])
    assert agg["checksums"][0] == agg["checksums"][1]  # identical replica trajectories
