"""Scenes and helpers that drive the solve down its failure-side branches.

Each follows a result code or branch of the reference's frame driver
(src/cuda_backend.cu):

* ``line_search_exhausted`` -- ``minimum_line_search_step`` above the first
  trial step, so no trial is ever taken: the block direction and its
  steepest-descent retry both fail, every adaptive attempt fails at its first
  substep, and the frame returns KHS_ERROR_NOT_CONVERGED with failure kind
  NONLINEAR_SOLVE (:666-679, :711, :713-716).
* ``infeasible_checkpoint`` -- a checkpoint whose state puts one free node on
  a collider triangle: the first evaluation of every attempt is outside the
  barrier's feasible region, giving KHS_ERROR_NOT_CONVERGED with kind
  BARRIER_INFEASIBLE (:655, :711).
* ``cancel_mid_frame`` -- khsRequestCancel from a second thread while the
  frame runs: observed once per Gauss-Newton iteration (:657), the frame
  returns KHS_ERROR_INVALID_STATE with the frame-start state restored (:714).
* ``steepest_heavy`` -- one line-search trial per direction: the block
  direction's trial often fails the Armijo test, so the steepest-descent
  retry runs (:677-678).
* ``root_jump`` -- roots jumping 3 cm per frame with no collider: the
  Gauss-Newton direction moves nodes farther than the translation trust
  radius and is scaled (:623-630).
"""
from __future__ import annotations

import dataclasses
import threading
import time

import numpy as np

import khs_native as kn
import scenes

HEADER = 24  # checkpoint header: magic u64, ABI u32, frame u32, dof u64


def line_search_exhausted():
    sc = scenes.sphere_scene(motion=True, frames=1)
    sc.desc["minimum_line_search_step"] = 2.0
    return sc


def steepest_heavy(strands: int = 40, frames: int = 2):
    sc = scenes.ellipsoid_scene(strands=strands, frames=frames)
    sc.desc["line_search_iterations"] = 1
    return sc


def root_jump(shift: float = 0.03, frames: int = 2, substeps: int = 2):
    base = scenes.sphere_scene(motion=False, frames=frames, substeps=substeps)
    pts = base.points
    return dataclasses.replace(base, name="jump", vertices=None, triangles=None, collider_at=None,
                               root_points_at=lambda f: pts + np.array([shift * f, 0.0, 0.0]))


def infeasible_scene():
    return scenes.sphere_scene(motion=False, frames=1)


def split(blob: bytes) -> tuple[np.ndarray, np.ndarray]:
    body = np.frombuffer(blob[HEADER:], dtype=np.float64)
    dof = body.size // 2
    return body[:dof].reshape(-1, 6).copy(), body[dof:].reshape(-1, 6).copy()


def join(blob: bytes, q: np.ndarray, v: np.ndarray) -> bytes:
    return blob[:HEADER] + np.ascontiguousarray(q, dtype=np.float64).tobytes() + \
        np.ascontiguousarray(v, dtype=np.float64).tobytes()


def infeasible_checkpoint(blob: bytes, scene, node: int = 2) -> bytes:
    """``blob`` with ``node`` (the first free node of strand 0) moved onto
    the centroid of the collider triangle nearest to it."""
    q, v = split(blob)
    verts = scene.collider_at(0)
    tri = scene.triangles.astype(np.int64)
    centroids = verts[tri].mean(axis=1)
    k = int(np.argmin(np.linalg.norm(centroids - q[node, :3], axis=1)))
    q[node, :3] = centroids[k]
    return join(blob, q, v)


def cancel_mid_frame(step, progress, cancel, timeout: float = 60.0) -> int:
    """Runs ``step()`` (a blocking frame) on this thread and calls
    ``cancel()`` from a second one once ``progress()`` reports a running
    Gauss-Newton iteration; returns the frame's result code."""
    done = threading.Event()

    def canceller():
        t0 = time.monotonic()
        while not done.is_set() and time.monotonic() - t0 < timeout:
            p = progress()
            if p.phase not in (kn.PHASE_IDLE, kn.PHASE_FINISHED, kn.PHASE_FAILED) and p.nonlinear_iteration >= 1:
                cancel()
                return
            time.sleep(0.0005)

    th = threading.Thread(target=canceller)
    th.start()
    try:
        return step()
    finally:
        done.set()
        th.join()
