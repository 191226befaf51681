"""Comparisons against the reference's own FP64 CUDA backend.

``tests/golden/reference_gpu.npz`` holds trajectories of the reference's
``src/cuda_backend.cu`` (compiled unchanged for sm_103a) on GB300, made by
``tests/golden/make_ref_golden.py``.  Each case was run twice: the reference
sums gradients, Hessian blocks, energies and friction impulses with double
atomics, so its two runs differ, and ``spread`` records by how much.

What the fixture shows about the reference itself:
* well-conditioned cases (the sphere scenes, the 40-strand ellipsoid) repeat
  to 1e-10 m / 1e-8 rad or better, so trajectories are compared in full;
* contact-heavy frames whose Gauss-Newton loop hits its iteration cap are
  chaotic: the 1,000-strand ellipsoid's two runs part by 0.6 mm in frame 1
  and 6.7 mm by frame 4, the body scene's by 0.9 mm in frame 5, and the
  CPU oracle perturbed by 1e-15 relative parts from itself by 1.8 cm in the
  pole scene's first frame.  No implementation, the reference included, can
  follow such a trajectory to 1e-6 m; these are compared one frame at a time
  from the reference's own state (the per-substep bar), and their counts
  where the reference repeats its own.
"""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np

import khs_native as kn
import scenes

GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_gpu.npz"
TOL = 1e-6
CHECKPOINT_MAGIC = 0x3154504348534B
ABI_VERSION = 5

SCENES = {
    "sphere_static": lambda: scenes.sphere_scene(motion=False, frames=1),
    "sphere_moving": lambda: scenes.sphere_scene(motion=True, frames=3),
    "ellipsoid40": lambda: scenes.ellipsoid_scene(strands=40, frames=2),
    "pole": lambda: scenes.pole_scene(frames=2),
    "ellipsoid1000": lambda: scenes.ellipsoid_scene(),
    "body5": lambda: scenes.body_scene(frames=5),
}

COUNTS = ("newton_iterations", "line_search_evaluations", "substeps", "contact_candidate_count",
          "active_contact_count")


def count_ok(ours: int, a: int, b: int) -> bool:
    """A count agrees with the reference: equal to its run where its two runs
    agree, else inside their range widened by its width (the reference's own
    run-to-run spread of that count)."""
    if a == b:
        return ours == a
    lo, hi = min(a, b), max(a, b)
    return lo - (hi - lo) <= ours <= hi + (hi - lo)


def load() -> dict:
    d = np.load(GOLDEN)
    return {k: d[k] for k in d.files}


def stat(g: dict, case: str, frame: int, name: str, run: str = "stats") -> float:
    fields = list(g["stat_fields"])
    return float(g[f"{case}__{run}"][frame, fields.index(name)])


def checkpoint(frame: int, q: np.ndarray, v: np.ndarray) -> bytes:
    """A checkpoint blob (the reference's layout, cuda_backend.cu:182-187)
    holding state (q, v) after animation frame ``frame``."""
    dof = q.size
    return struct.pack("<QIIQ", CHECKPOINT_MAGIC, ABI_VERSION, frame, dof) + \
        np.ascontiguousarray(q, dtype=np.float64).tobytes() + np.ascontiguousarray(v, dtype=np.float64).tobytes()


def sensitivity(oracle_lib, case: str, frames: int | None = None) -> list[tuple[float, float]]:
    """Per frame, how far the oracle's own trajectory moves (positions,
    rotations) when the root targets change by +-1e-15 relative: the
    amplification of last-bit differences that belongs to the scene."""
    import parity

    base = parity.run(oracle_lib, SCENES[case](), frames=frames)
    out = [(0.0, 0.0)] * len(base)
    for eps in (1e-15, -1e-15):
        sc = SCENES[case]()
        pts = sc.root_points_at
        sc.root_points_at = lambda f, pts=pts, eps=eps: pts(f) * (1.0 + eps)
        for k, fr in enumerate(parity.compare(parity.run(oracle_lib, sc, frames=frames), base)):
            out[k] = (max(out[k][0], fr["max_position"]), max(out[k][1], fr["max_rotation"]))
    return out


def tolerances(g: dict, case: str, sens: list[tuple[float, float]]) -> list[tuple[float, float]]:
    """Per frame (position, rotation) tolerance against the reference:
    1e-6 m / 1e-6 rad, or 4x the larger of the reference's run-to-run
    spread and the oracle's sensitivity where that is larger."""
    spread = g[f"{case}__spread"]
    return [(max(TOL, 4.0 * max(spread[k, 0], s[0])), max(TOL, 4.0 * max(spread[k, 1], s[1])))
            for k, s in enumerate(sens)]


def trajectory_deviation(g: dict, case: str, frames: list[dict]) -> list[dict]:
    """Per stepped frame: max position / rotation deviation from the
    reference's run, and each library-vs-reference count pair."""
    ref_q = g[f"{case}__q"]
    sample = g.get(f"{case}__sample")
    out = []
    for k, fr in enumerate(frames):
        q = fr["q"] if sample is None else fr["q"][sample]
        dq = np.abs(q - ref_q[k])
        entry = {"frame": k + 1, "position": float(dq[:, :3].max()), "rotation": float(dq[:, 3:].max()),
                 "result": (fr["result"], int(g[f"{case}__result"][k]))}
        for c in COUNTS:
            entry[c] = (int(getattr(fr["stats"], c)), int(stat(g, case, k, c)), int(stat(g, case, k, c, "stats_b")))
        out.append(entry)
    return out


def frame_tolerance(oracle_lib, g: dict, case: str, frame: int) -> tuple[float, float]:
    """(position, rotation) tolerance of one frame from the reference's
    state: 1e-6, or 4x the oracle's change under a +-1e-15 relative change
    of the root targets over that frame where that is larger."""
    base = step_from_reference_state(oracle_lib, g, case, frame, q_out=True)["q"]
    pos = rot = 0.0
    for eps in (1e-15, -1e-15):
        q = step_from_reference_state(oracle_lib, g, case, frame, eps=eps, q_out=True)["q"]
        dq = np.abs(q - base)
        pos, rot = max(pos, float(dq[:, :3].max())), max(rot, float(dq[:, 3:].max()))
    return max(TOL, 4.0 * pos), max(TOL, 4.0 * rot)


def step_from_reference_state(lib, g: dict, case: str, frame: int, mode: int | None = None, eps: float = 0.0,
                              q_out: bool = False) -> dict:
    """Restores the reference's state after ``frame`` (full q, v from the
    fixture) into ``lib`` and steps frame ``frame + 1`` (root targets scaled
    by 1 + ``eps``)."""
    sc = SCENES[case]()
    if eps:
        pts = sc.root_points_at
        sc.root_points_at = lambda f: pts(f) * (1.0 + eps)
    s = kn.HairSolver(lib)
    scenes.load_into(s, sc)
    if mode is not None:
        s.set_solve_mode(mode)
    s.restore_checkpoint(checkpoint(frame, g[f"{case}__q"][frame - 1], g[f"{case}__v"][frame - 1]))
    r = s._library.khsStepAnimationFrame(s.handle, frame + 1, sc.frame_dt)
    q, v = s.state()
    st = s.stats()
    s.close()
    dq = np.abs(q - g[f"{case}__q"][frame])
    return {"result": r, "position": float(dq[:, :3].max()), "rotation": float(dq[:, 3:].max()),
            "q": q if q_out else None,
            "counts": {c: (int(getattr(st, c)), int(stat(g, case, frame, c)), int(stat(g, case, frame, c, "stats_b")))
                       for c in COUNTS}}
