"""The strand-sharded solve on two and three gloo ranks (CPU oracle, see
tests/sharded.py): every rank steps its own strands, the global scalars are
combined by all-reduce, and the gathered state, the step statistics and the
per-substep records are bit-identical to one rank stepping every strand.
The scene has contacts, so the exchanged counts and bounds are exercised; a
second scene drives the steepest-descent retries and trust-radius scaling.
One rank with the partition hook stays within 1e-6 of the oracle's default
serial sums."""
import os
import pickle
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _scene(name):
    import failure_cases
    import scenes

    if name == "contact":
        return scenes.ellipsoid_scene(strands=24, node_range=(20, 40), frames=2)
    sc = failure_cases.steepest_heavy(strands=12, frames=1)
    sc.desc["substeps"] = 2
    return sc


def _rank(rank, world, port, oracle, scene_name, out):
    sys.path[:0] = [str(REPO / "kami-hair-solver_gb300"), str(REPO / "tests")]
    import khs_native as kn
    import sharded

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lib = kn.Library(oracle)
    lib.lib.khsOracleSetThreads(1)
    res = sharded.run(lib, _scene(scene_name), rank, world, dist)
    parts = [None] * world
    dist.all_gather_object(parts, res)
    if rank == 0:
        Path(out).write_bytes(pickle.dumps(parts))
    dist.destroy_process_group()


def _sharded(oracle_path, tmp_path, world, scene_name):
    out = tmp_path / f"parts{world}.pkl"
    mp.spawn(_rank, args=(world, _free_port(), str(oracle_path), scene_name, str(out)), nprocs=world, join=True)
    parts = pickle.loads(out.read_bytes())
    q = np.concatenate([p["q"] for p in parts])
    v = np.concatenate([p["v"] for p in parts])
    assert [p["nodes"][0] for p in parts[1:]] == [p["nodes"][1] for p in parts[:-1]]  # contiguous cover
    return q, v, parts


@pytest.mark.parametrize("scene_name", ["contact", "fallbacks"])
def test_sharded_ranks_match_one_rank_bit_for_bit(oracle_lib, oracle_path, tmp_path, scene_name):
    import sharded

    oracle_lib.lib.khsOracleSetThreads(1)
    one = sharded.run(oracle_lib, _scene(scene_name))
    for world in (2, 3):
        q, v, parts = _sharded(oracle_path, tmp_path, world, scene_name)
        assert np.array_equal(q, one["q"]) and np.array_equal(v, one["v"]), world
        for p in parts:
            assert p["frames"] == one["frames"], world  # identical stats and substep records on every rank
    if scene_name == "contact":
        assert sum(fr["stats"]["active_contact_count"] for fr in one["frames"]) > 0
    else:
        recs = [r for fr in one["frames"] for r in fr["records"]]
        assert sum(r[2] for r in recs) > 0  # steepest-descent retries were exchanged


def test_partitioned_sums_stay_within_tolerance_of_serial(oracle_lib):
    import parity
    import sharded

    oracle_lib.lib.khsOracleSetThreads(1)
    one = sharded.run(oracle_lib, _scene("contact"))
    serial = parity.run(oracle_lib, _scene("contact"))
    dq = np.abs(one["q"] - serial[-1]["q"])
    assert dq[:, :3].max() <= 1e-6 and dq[:, 3:].max() <= 1e-6
    assert [fr["stats"]["newton_iterations"] for fr in one["frames"]] == \
        [fr["stats"].newton_iterations for fr in serial]
