"""The oracle's root targets (its restatement of Solver::compute_root_targets,
src/solver.cpp:416-447, exported as khsxComputeRootTargets), which the GPU
library's device root-target pass is compared against.

* At the rest pose the targets are the internal nodes themselves: the
  positions equal the built nodes and the rotation vectors vanish (the
  frames walked from the rest tangents are the reference frames).
* A rigid rotation R of the source points rotates the positions, and each
  target rotation takes the node's rest tangent to R times it.
* The reference's error order (solver.cpp:802-824): a count mismatch gives
  KHS_ERROR_INVALID_ARGUMENT, a non-finite coordinate or a degenerate
  tangent KHS_ERROR_INVALID_HAIR, and those come before a bad frame index
  or a small output array.
"""
import ctypes
import math

import numpy as np

import khs_native as kn
import scenes


def _oracle(lib, scene):
    s = kn.HairSolver(lib)
    scenes.load_into(s, scene, animation=False)
    return s


def test_rest_pose_targets_are_the_nodes(oracle_lib):
    sc = scenes.sphere_scene(strands=16, nodes=12)
    s = _oracle(oracle_lib, sc)
    try:
        pos, rot = s.compute_root_targets(sc.points)
        assert np.abs(pos - s.internal_positions()).max() <= 1e-15
        assert np.abs(rot).max() <= 1e-12
    finally:
        s.close()


def _rodrigues(w):
    a = np.linalg.norm(w)
    if a == 0.0:
        return np.eye(3)
    k = w / a
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + math.sin(a) * K + (1 - math.cos(a)) * K @ K


def test_rigid_rotation_turns_every_tangent(oracle_lib):
    """Rotating the source points by R: the positions rotate, and each
    target rotation takes the node's rest tangent (the third column of its
    reference frame) to the rotated tangent.  The twist about the tangent
    is not R's: the walk starts from the reference frame's first column as
    its hint (solver.cpp:434), as in the reference."""
    sc = scenes.sphere_scene(strands=16, nodes=12)
    s = _oracle(oracle_lib, sc)
    try:
        R = _rodrigues(0.7 * np.array([0.2, -0.5, 0.84]) / np.linalg.norm([0.2, -0.5, 0.84]))
        x = s.internal_positions()
        pos, rot = s.compute_root_targets(sc.points @ R.T)
        assert np.abs(pos - x @ R.T).max() <= 1e-14
        count = len(sc.points)
        mapping = np.zeros(count, dtype=np.uint32)
        s._check(s._library.khsCopyOriginalToInternalMap(s.handle, ctypes.c_void_p(mapping.ctypes.data), count))
        worst = 0.0
        for a, b in zip(sc.offsets[:-1], sc.offsets[1:]):
            first, last = int(mapping[a]), int(mapping[b - 1])
            for n in range(first, last + 1):
                lo, hi = (n, n + 1) if n == first else ((n - 1, n) if n == last else (n - 1, n + 1))
                t = x[hi] - x[lo]
                t /= np.linalg.norm(t)
                worst = max(worst, float(np.abs(_rodrigues(rot[n]) @ t - R @ t).max()))
        assert worst <= 1e-12, worst
    finally:
        s.close()


def test_error_order(oracle_lib):
    sc = scenes.sphere_scene(strands=8, nodes=10)
    s = _oracle(oracle_lib, sc)
    try:
        s.allocate_animation(2)
        lib, h = s._library, s.handle
        n = len(sc.points)
        nodes = s.build_stats().internal_node_count
        pos = np.zeros((nodes, 3))
        rot = np.zeros((nodes, 3))

        def codes(points, frame, capacity=nodes):
            p = np.ascontiguousarray(points, dtype=np.float64)
            ptr = ctypes.c_void_p(p.ctypes.data)
            return (lib.khsUpdateRootTargets(h, ptr, len(p)), lib.khsSetRootAnimationFrame(h, frame, ptr, len(p)),
                    lib.khsxComputeRootTargets(h, ptr, len(p), ctypes.c_void_p(pos.ctypes.data),
                                               ctypes.c_void_p(rot.ctypes.data), capacity))

        good = sc.points
        bad = good.copy()
        bad[3, 2] = np.inf
        flat = good.copy()
        flat[sc.offsets[1]:sc.offsets[2]] = good[sc.offsets[1]]
        assert codes(good, 1) == (kn.OK, kn.OK, kn.OK)
        assert codes(good[: n - 1], 1) == (kn.ERROR_INVALID_ARGUMENT,) * 3
        assert codes(bad, 1) == (kn.ERROR_INVALID_HAIR,) * 3
        assert codes(flat, 1) == (kn.ERROR_INVALID_HAIR,) * 3
        assert codes(good, 5) == (kn.OK, kn.ERROR_INVALID_ARGUMENT, kn.OK)
        # khsxComputeRootTargets checks its output capacity before computing.
        assert codes(flat, 5, nodes - 1) == (kn.ERROR_INVALID_HAIR, kn.ERROR_INVALID_HAIR, kn.ERROR_INVALID_ARGUMENT)
        assert codes(good, 1, nodes - 1)[2] == kn.ERROR_INVALID_ARGUMENT
    finally:
        s.close()
