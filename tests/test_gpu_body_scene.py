"""The benchmark's full-size workload (body scene: 6,757 strands, 265,108
nodes, 449,940 collider triangles) on the GB300, checked through properties
that do not need a CPU trajectory of that size:

* the mixed form's trajectory is bit-identical to the plain FP64 form's;
* at the GPU's own final state the CPU oracle's broad + narrow phase gives
  the same per-element candidate counts, closest triangles, active flags and
  gap bits as the GPU's last evaluation (integer contact work bit-exact);
* no element ends inside the minimum gap, and every frame converged.
"""
import os

import numpy as np
import pytest

import khs_native as kn
import parity
import scenes

pytestmark = pytest.mark.gpu

FRAMES = 5  # frames 1-4: the first contacts arrive in frame 4


def _run(lib, mode):
    sc = scenes.body_scene(frames=FRAMES)
    s = kn.HairSolver(lib)
    scenes.load_into(s, sc)
    s.set_solve_mode(mode)
    for f in range(1, FRAMES):
        assert s._library.khsStepAnimationFrame(s.handle, f, sc.frame_dt) == kn.OK, s.last_error()
    q, v = s.state()
    out = dict(q=q, v=v, contacts=s.contact_records(), stats=s.stats(), min_gap=s.desc.minimum_gap)
    s.close()
    return out


def test_body_scene_mixed_equals_plain_and_contacts_match_oracle(gpu_lib, oracle_lib):
    mixed = _run(gpu_lib, kn.MODE_MIXED)
    plain = _run(gpu_lib, kn.MODE_PLAIN_FP64)
    assert np.array_equal(mixed["q"], plain["q"]) and np.array_equal(mixed["v"], plain["v"])
    assert mixed["stats"].active_contact_count > 0
    # The oracle classifies every element at the GPU's own state, against
    # the collider as the last substep left it (the frame-4 vertices): the
    # oracle steps the same frames (its own trajectory) to get there.
    sc = scenes.body_scene(frames=FRAMES)
    oracle_lib.lib.khsOracleSetThreads(os.cpu_count() or 1)
    o = kn.HairSolver(oracle_lib)
    scenes.load_into(o, sc)
    for f in range(1, FRAMES):
        assert o._library.khsStepAnimationFrame(o.handle, f, sc.frame_dt) == kn.OK, o.last_error()
    ref = o.query_contacts(mixed["q"])
    o.close()
    mism = parity.records_equal(mixed["contacts"], ref)
    assert all(v == 0 for v in mism.values()), mism
    gaps = mixed["contacts"]["gap"][mixed["contacts"]["closest_triangle"] != 0xFFFFFFFF]
    assert gaps.min() > mixed["min_gap"]
