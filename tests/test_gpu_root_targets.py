"""Root targets on the device (k_root_tangents, k_root_frames,
k_root_rotations) against the oracle's restatement of
Solver::compute_root_targets (src/solver.cpp:416-447), through
khsxComputeRootTargets, and the error behaviour of the three entry points
that compute them (khsUpdateRootTargets, khsSetRootAnimationFrame and
khsxComputeRootTargets; solver.cpp:802-824).

Positions, tangents and frames are evaluated with the same correctly
rounded operations on both sides (no FMA contraction), so the positions
must agree bit for bit.  The rotation vectors go through atan2, whose device
and host versions may differ in the last bits: within 1e-14 rad.
"""
import ctypes

import numpy as np
import pytest

import khs_native as kn
import scenes

pytestmark = pytest.mark.gpu

ROT_TOL = 1e-14


def _built(lib, scene):
    s = kn.HairSolver(lib)
    scenes.load_into(s, scene, animation=False)
    return s


def _compare(gpu_lib, oracle_lib, scene, frames):
    g, o = _built(gpu_lib, scene), _built(oracle_lib, scene)
    try:
        worst = 0.0
        for f in frames:
            pts = scene.root_points_at(f)
            gp, gr = g.compute_root_targets(pts)
            op, orr = o.compute_root_targets(pts)
            assert np.array_equal(gp, op), (f, np.abs(gp - op).max())
            err = float(np.abs(gr - orr).max())
            assert err <= ROT_TOL, (f, err)
            worst = max(worst, err)
        return worst, float(np.abs(orr).max())
    finally:
        g.close()
        o.close()


def test_root_targets_rotating_ellipsoid(gpu_lib, oracle_lib):
    """1,000 helical strands whose roots ride an ellipsoid turning about z
    at 2 rad/s: every frame has non-trivial rotation targets."""
    sc = scenes.ellipsoid_scene(frames=10)
    worst, largest = _compare(gpu_lib, oracle_lib, sc, [0, 1, 5, 9])
    print(f"rotation difference {worst:.3e} rad, largest rotation {largest:.3f} rad")
    assert largest > 0.1


def test_root_targets_moving_sphere(gpu_lib, oracle_lib):
    sc = scenes.sphere_scene(motion=True, frames=3)
    _compare(gpu_lib, oracle_lib, sc, [0, 1, 2])


def test_root_targets_body_scene(gpu_lib, oracle_lib):
    """6,757 strands / 265,108 nodes, one swayed frame."""
    sc = scenes.body_scene(frames=4)
    _compare(gpu_lib, oracle_lib, sc, [3])


def _codes(lib, scene, points, frame):
    """Result codes of the three entry points for one set of points."""
    s = kn.HairSolver(lib)
    try:
        scenes.load_into(s, scene, animation=False)
        s.allocate_animation(2)
        pts = np.ascontiguousarray(points, dtype=np.float64)
        n = len(pts)
        nodes = s.build_stats().internal_node_count
        pos = np.zeros((nodes, 3))
        rot = np.zeros((nodes, 3))
        p = ctypes.c_void_p(pts.ctypes.data)
        return (int(s._library.khsUpdateRootTargets(s.handle, p, n)),
                int(s._library.khsSetRootAnimationFrame(s.handle, frame, p, n)),
                int(s._library.khsxComputeRootTargets(s.handle, p, n, ctypes.c_void_p(pos.ctypes.data),
                                                      ctypes.c_void_p(rot.ctypes.data), nodes)),
                int(s._library.khsxComputeRootTargets(s.handle, p, n, ctypes.c_void_p(pos.ctypes.data),
                                                      ctypes.c_void_p(rot.ctypes.data), nodes - 1)))
    finally:
        s.close()


def test_root_target_errors_match_oracle(gpu_lib, oracle_lib):
    sc = scenes.sphere_scene(motion=True, frames=2)
    good = sc.root_points_at(1)
    nan = good.copy()
    nan[5, 1] = np.nan
    # Every point of the first strand at its root: zero tangents.
    degenerate = good.copy()
    degenerate[sc.offsets[0]:sc.offsets[1]] = good[sc.offsets[0]]
    cases = {
        "valid": (good, 1),
        "short": (good[:-1], 1),
        "non-finite": (nan, 1),
        "degenerate": (degenerate, 1),
        "frame out of range": (good, 7),
        "degenerate, frame out of range": (degenerate, 7),
    }
    expected = {
        "valid": (kn.OK, kn.OK, kn.OK, kn.ERROR_INVALID_ARGUMENT),
        "short": (kn.ERROR_INVALID_ARGUMENT,) * 4,
        "non-finite": (kn.ERROR_INVALID_HAIR,) * 4,
        "degenerate": (kn.ERROR_INVALID_HAIR, kn.ERROR_INVALID_HAIR, kn.ERROR_INVALID_HAIR, kn.ERROR_INVALID_ARGUMENT),
        "frame out of range": (kn.OK, kn.ERROR_INVALID_ARGUMENT, kn.OK, kn.ERROR_INVALID_ARGUMENT),
        "degenerate, frame out of range": (kn.ERROR_INVALID_HAIR, kn.ERROR_INVALID_HAIR, kn.ERROR_INVALID_HAIR,
                                           kn.ERROR_INVALID_ARGUMENT),
    }
    for name, (pts, frame) in cases.items():
        got = _codes(gpu_lib, sc, pts, frame)
        ref = _codes(oracle_lib, sc, pts, frame)
        assert got == ref == expected[name], (name, got, ref)


def test_failed_update_keeps_pending_targets(gpu_lib, oracle_lib):
    """A rejected khsUpdateRootTargets leaves the previous targets in place:
    the next khsStep follows the last accepted points on both sides."""
    sc = scenes.sphere_scene(motion=True, frames=3)
    out = []
    for lib in (gpu_lib, oracle_lib):
        s = kn.HairSolver(lib)
        try:
            scenes.load_into(s, sc, animation=False)
            s.update_roots(sc.root_points_at(1))
            bad = sc.root_points_at(2).copy()
            bad[sc.offsets[0]:sc.offsets[1]] = bad[sc.offsets[0]]
            with pytest.raises(RuntimeError):
                s.update_roots(bad)
            s.step(sc.frame_dt)
            out.append(s.state()[0])
        finally:
            s.close()
    assert np.abs(out[0] - out[1]).max() <= 1e-6
