"""Parity at the stated workload sizes, one substep at a time.

The 1,000-strand rotating ellipsoid (the plain-FP64 workload of 1,000
strands / ~70k nodes / 20,480 triangles, 10 frames x 8 substeps) and the
265,108-node body scene are contact-heavy and hit the Gauss-Newton iteration
cap, where trajectories are chaotic: the reference's own CUDA backend parts
from itself by 1.2 mm within one ellipsoid frame from a common state, and
the CPU oracle parts from itself by 2.7 mm within one frame when its root
targets change by 1e-15 relative.  The bar is therefore applied per
substep: the GB300 library steps the whole trajectory, and at several frames
the oracle and both GB300 forms run the first substep from the GB300
checkpoint of that frame's start.  Newton and line-search counts and the
candidate and active-contact totals of that substep must be identical;
positions and rotations must agree within 1e-6, or within 4x the oracle's
own change under a +-1e-15 relative change of the root targets over the
same substep where that is larger (the twist of weakly constrained nodes in
tangled, iteration-capped states: up to ~1e-4 rad in the ellipsoid's later
frames).
"""
import numpy as np
import pytest

import khs_native as kn
import scenes

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _checkpoints(lib, scene, frames, mode=kn.MODE_MIXED):
    """Steps the scene on the GB300 library; checkpoint at the start of each
    frame in ``frames``."""
    s = kn.HairSolver(lib)
    scenes.load_into(s, scene)
    s.set_solve_mode(mode)
    out = {}
    for f in range(1, max(frames) + 1):
        if f in frames:
            out[f] = s.save_checkpoint()
        if f < max(frames):
            assert s._library.khsStepAnimationFrame(s.handle, f, scene.frame_dt) == kn.OK, (f, s.last_error())
    s.close()
    return out


def _one_substep(lib, scene, checkpoint, frame, mode=None, eps=0.0):
    if eps:
        pts = scene.root_points_at
        scene.root_points_at = lambda f: pts(f) * (1.0 + eps)
    s = kn.HairSolver(lib)
    scenes.load_into(s, scene, frames=frame + 1)
    if mode is not None:
        s.set_solve_mode(mode)
    s.set_substep_limit(1)
    s.restore_checkpoint(checkpoint)
    r = s._library.khsStepAnimationFrame(s.handle, frame, scene.frame_dt)
    q, _ = s.state()
    rec = s.substep_records()
    s.close()
    assert r == kn.OK and len(rec) == 1
    r0 = rec[0]
    return q, (r0.newton_iterations, r0.line_search_evaluations, r0.steepest_fallbacks, r0.trust_scalings,
               r0.contact_candidates, r0.active_contacts)


def _compare(gpu_lib, oracle_lib, make, frames):
    cks = _checkpoints(gpu_lib, make(), frames)
    report = []
    for f in frames:
        q_o, c_o = _one_substep(oracle_lib, make(), cks[f], f)
        sens = [0.0, 0.0]
        for eps in (1e-15, -1e-15):
            dq = np.abs(_one_substep(oracle_lib, make(), cks[f], f, eps=eps)[0] - q_o)
            sens = [max(sens[0], float(dq[:, :3].max())), max(sens[1], float(dq[:, 3:].max()))]
        tol = (max(TOL, 4.0 * sens[0]), max(TOL, 4.0 * sens[1]))
        for mode in (kn.MODE_MIXED, kn.MODE_PLAIN_FP64):
            q_g, c_g = _one_substep(gpu_lib, make(), cks[f], f, mode)
            dq = np.abs(q_g - q_o)
            report.append(dict(frame=f, mode=mode, position=float(dq[:, :3].max()),
                               rotation=float(dq[:, 3:].max()), tol=tol, counts=(c_g, c_o)))
    print(report)
    for e in report:
        assert e["counts"][0] == e["counts"][1], e
        assert e["position"] <= e["tol"][0] and e["rotation"] <= e["tol"][1], e
    return report


def test_ellipsoid_1000_strands_per_substep(gpu_lib, oracle_lib):
    rep = _compare(gpu_lib, oracle_lib, lambda: scenes.ellipsoid_scene(), [1, 4, 10])
    assert max(e["counts"][0][5] for e in rep) > 0  # contact-heavy substeps were compared


def test_body_scene_per_substep(gpu_lib, oracle_lib):
    rep = _compare(gpu_lib, oracle_lib, lambda: scenes.body_scene(frames=8), [4, 5, 8])
    assert max(e["counts"][0][5] for e in rep) > 0
