"""Serving on the GB300: requests run concurrently on their own streams give
results identical to running each alone; the device-resident rollback ring
restores earlier frames exactly."""
import numpy as np
import pytest

import khs_native as kn
import scenes
import serving

pytestmark = pytest.mark.gpu


def test_concurrent_requests_match_solo_runs(gpu_lib):
    reqs = serving.make_stream(4, rate=50.0, seed=3, strand_range=(100, 400), frames=3)
    server = serving.Server(gpu_lib, budget_bytes=int(40e9), max_slots=4, mode=kn.MODE_MIXED, ring_slots=4)
    mixed = server.run(reqs)
    assert server.peak_slots >= 2  # the requests overlapped
    for req, res in zip(reqs, mixed):
        assert res.status == kn.OK, res.error
        solo = serving.run_request(gpu_lib, req, kn.MODE_MIXED, 0)
        assert solo.status == kn.OK, solo.error
        assert np.array_equal(solo.q, res.q), req.rid
    s = serving.summary(mixed, server.makespan)
    assert s["completed"] == 4 and s["p99_frame_ms"] >= s["p50_frame_ms"] > 0


def test_rollback_ring_restores_frames(gpu_lib):
    sc = scenes.sphere_scene(motion=True, frames=4)
    s = kn.HairSolver(gpu_lib)
    scenes.load_into(s, sc)
    s.set_rollback_ring(3)  # holds frame 0 now
    states = {}
    for f in range(1, 4):
        assert s._library.khsStepAnimationFrame(s.handle, f, sc.frame_dt) == kn.OK
        states[f] = s.state()
    # Frames 1-3 are held; frame 0 was overwritten by frame 3.
    assert s._library.khsxRollbackToFrame(s.handle, 0) == kn.ERROR_INVALID_ARGUMENT
    s.rollback_to_frame(1)
    q, v = s.state()
    assert np.array_equal(q, states[1][0]) and np.array_equal(v, states[1][1])
    # Re-stepping from the restored frame reproduces the trajectory.
    assert s._library.khsStepAnimationFrame(s.handle, 2, sc.frame_dt) == kn.OK
    q, v = s.state()
    assert np.array_equal(q, states[2][0]) and np.array_equal(v, states[2][1])
    s.close()


def test_restored_checkpoint_resets_rollback_ring(gpu_lib):
    """Restoring a checkpoint forgets the ring's later frames and puts the
    restored state in the checkpoint frame's slot."""
    sc = scenes.sphere_scene(motion=True, frames=6)
    s = kn.HairSolver(gpu_lib)
    scenes.load_into(s, sc)
    s.set_rollback_ring(6)
    checkpoints = {}
    for f in range(1, 6):
        assert s._library.khsStepAnimationFrame(s.handle, f, sc.frame_dt) == kn.OK
        checkpoints[f] = s.save_checkpoint()
    s.restore_checkpoint(checkpoints[2])
    assert s._library.khsxRollbackToFrame(s.handle, 4) == kn.ERROR_INVALID_ARGUMENT
    assert s._library.khsxRollbackToFrame(s.handle, 3) == kn.ERROR_INVALID_ARGUMENT
    s.rollback_to_frame(2)
    assert s.save_checkpoint() == checkpoints[2]
    # A checkpoint from another trajectory: its state, not the ring's, is frame 2's.
    other = bytearray(checkpoints[2])
    header = 24
    q = np.frombuffer(bytes(other[header:]), dtype=np.float64).copy()
    q[len(q) // 2 - 1] += 1e-9  # the last node's rotation z (q, then v)
    other[header:] = q.tobytes()
    s.restore_checkpoint(bytes(other))
    assert s._library.khsStepAnimationFrame(s.handle, 3, sc.frame_dt) == kn.OK
    s.rollback_to_frame(2)
    assert s.save_checkpoint() == bytes(other)
    s.close()
