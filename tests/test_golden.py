"""Committed oracle trajectories (tests/golden/oracle_trajectories.npz, made
by tests/golden/make_golden.py): the oracle reproduces them, and the GB300
library follows them within the FP64 tolerance."""
from pathlib import Path

import numpy as np
import pytest

import khs_native as kn
import scenes

GOLDEN = np.load(Path(__file__).resolve().parent / "golden" / "oracle_trajectories.npz")
CASES = {"sphere_moving": lambda: scenes.sphere_scene(motion=True, frames=3),
         "ellipsoid40": lambda: scenes.ellipsoid_scene(strands=40, frames=2)}


def _run(lib, scene, mode=None):
    s = kn.HairSolver(lib)
    scenes.load_into(s, scene)
    if mode is not None:
        s.set_solve_mode(mode)
    q, stats, contacts = [], [], []
    for f in range(1, scene.frames):
        assert s._library.khsStepAnimationFrame(s.handle, f, scene.frame_dt) == kn.OK, s.last_error()
        st = s.stats()
        q.append(s.state()[0])
        stats.append([st.substeps, st.newton_iterations, st.line_search_evaluations, st.contact_candidate_count,
                      st.active_contact_count])
        contacts.append(s.contact_records())
    s.close()
    return np.stack(q), np.asarray(stats, dtype=np.uint64), np.stack(contacts)


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_golden(oracle_lib, name):
    q, stats, c = _run(oracle_lib, CASES[name]())
    assert np.array_equal(stats, GOLDEN[f"{name}_stats"])
    # Bit-exact on the machine that made them; 1e-12 absorbs another libm.
    assert np.max(np.abs(q - GOLDEN[f"{name}_q"])) <= 1e-12
    for field in ("candidate_count", "closest_triangle", "active"):
        assert np.array_equal(c[field], GOLDEN[f"{name}_{field}"]), field
    has = GOLDEN[f"{name}_closest_triangle"] != 0xFFFFFFFF
    assert np.max(np.abs(c["gap"][has] - GOLDEN[f"{name}_gap"][has]), initial=0.0) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [kn.MODE_PLAIN_FP64, kn.MODE_MIXED])
def test_gpu_follows_golden_sphere(gpu_lib, mode):
    q, stats, _ = _run(gpu_lib, CASES["sphere_moving"](), mode)
    assert np.array_equal(stats, GOLDEN["sphere_moving_stats"])
    dq = np.abs(q - GOLDEN["sphere_moving_q"])
    assert dq[..., :3].max() <= 1e-6 and dq[..., 3:].max() <= 1e-6
