"""The pinned output ring (khsxSetOutputRing, khsxCopyOutputFrame,
khsxMapOutputFrame): the bake loop's per-frame output without a synchronous
device-to-host copy (the reference add-on calls khsCopyOriginalPositions
after every frame, addon.py:748-757).

* Every frame the ring holds equals khsCopyOriginalPositions right after
  that frame, bit for bit, through both the copy and the mapped view.
* Frames the ring has moved past, and frames not stepped yet, are refused;
  so are reads with the ring off, and frames past the one a rollback
  restored.
* The ring does not change the solve: the final state is the same bits
  with and without it.
* Timing on the body scene: the per-frame output through the ring against
  the synchronous copy into pageable memory (printed).
"""
import ctypes
import time

import numpy as np
import pytest

import khs_native as kn
import scenes

pytestmark = pytest.mark.gpu


def _frames(lib, scene, ring, frames):
    s = kn.HairSolver(lib)
    scenes.load_into(s, scene, frames=frames + 1)
    s.set_solve_mode(kn.MODE_MIXED)
    if ring:
        s.set_output_ring(ring)
    return s


def test_output_ring_matches_synchronous_copy(gpu_lib):
    sc = scenes.sphere_scene(motion=True, frames=6)
    s = _frames(gpu_lib, sc, 3, 6)
    try:
        direct = {}
        for f in range(0, 6):
            s.step_animation_frame(f, sc.frame_dt)
            direct[f] = s.positions()
            assert np.array_equal(s.output_frame(f), direct[f]), f
            assert np.array_equal(s.map_output_frame(f), direct[f]), f
            for old in range(0, f + 1):
                held = f - old < 3
                if held:
                    assert np.array_equal(s.output_frame(old), direct[old]), (f, old)
                else:
                    out = np.zeros_like(direct[old])
                    r = s._library.khsxCopyOutputFrame(s.handle, old, ctypes.c_void_p(out.ctypes.data), len(out))
                    assert r == kn.ERROR_INVALID_ARGUMENT, (f, old, r)
        out = np.zeros_like(direct[0])
        assert s._library.khsxCopyOutputFrame(s.handle, 9, ctypes.c_void_p(out.ctypes.data), len(out)) == \
            kn.ERROR_INVALID_ARGUMENT
        assert s._library.khsxCopyOutputFrame(s.handle, 5, ctypes.c_void_p(out.ctypes.data), len(out) - 1) == \
            kn.ERROR_INVALID_ARGUMENT
        q_ring = s.state()[0]
        s.set_output_ring(0)
        assert s._library.khsxCopyOutputFrame(s.handle, 5, ctypes.c_void_p(out.ctypes.data), len(out)) == \
            kn.ERROR_INVALID_STATE
    finally:
        s.close()
    plain = _frames(gpu_lib, sc, 0, 6)
    try:
        for f in range(0, 6):
            plain.step_animation_frame(f, sc.frame_dt)
        assert np.array_equal(plain.state()[0], q_ring)
    finally:
        plain.close()


def test_output_ring_after_rollback(gpu_lib):
    """After khsxRollbackToFrame the ring drops the frames past the restored
    one (they belong to the abandoned trajectory) and holds each re-stepped
    frame once, equal to the positions after it."""
    sc = scenes.sphere_scene(motion=True, frames=6)
    s = _frames(gpu_lib, sc, 4, 6)
    try:
        s.set_rollback_ring(6)
        for f in range(0, 5):
            s.step_animation_frame(f, sc.frame_dt)
        s._check(s._library.khsxRollbackToFrame(s.handle, 2))
        out = np.zeros((int(s._library.khsGetOriginalPointCount(s.handle)), 3))
        for gone in (3, 4):
            assert s._library.khsxCopyOutputFrame(s.handle, gone, ctypes.c_void_p(out.ctypes.data), len(out)) == \
                kn.ERROR_INVALID_ARGUMENT, gone
        assert s.output_frame(2) is not None
        for f in (3, 4):
            s.step_animation_frame(f, sc.frame_dt)
            assert np.array_equal(s.output_frame(f), s.positions()), f
    finally:
        s.close()


def test_output_ring_timing_body_scene(gpu_lib):
    sc = scenes.body_scene(frames=4)
    s = _frames(gpu_lib, sc, 4, 3)
    try:
        s.step_animation_frame(0, sc.frame_dt)
        rows = []
        for f in (1, 2):
            s.step_animation_frame(f, sc.frame_dt)
            t0 = time.perf_counter()
            sync = s.positions()
            t1 = time.perf_counter()
            ring = s.output_frame(f)
            t2 = time.perf_counter()
            view = s.map_output_frame(f)
            t3 = time.perf_counter()
            assert np.array_equal(sync, ring) and np.array_equal(sync, view)
            rows.append((1e3 * (t1 - t0), 1e3 * (t2 - t1), 1e3 * (t3 - t2)))
        for f, (a, b, c) in zip((1, 2), rows):
            print(f"frame {f}: synchronous copy {a:.2f} ms, ring copy {b:.2f} ms, ring view {c:.3f} ms "
                  f"({len(sync)} points)")
    finally:
        s.close()
