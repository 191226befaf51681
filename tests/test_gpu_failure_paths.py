"""Failure-side branches on the GB300 library, against the CPU oracle and,
where its sources are staged, the reference's own CUDA backend:

* the line search that can take no trial (NONLINEAR_SOLVE) and the start
  outside the barrier's feasible region (BARRIER_INFEASIBLE) give the
  reference's result code and the oracle's failure diagnostics field for
  field, with the frame-start state restored;
* khsRequestCancel from a second thread stops the frame with
  KHS_ERROR_INVALID_STATE and restores its start state;
* the steepest-descent retry and the trust-radius scaling: scenes that take
  them many times keep parity with the oracle (identical per-substep counts
  of Newton iterations, line-search trials, steepest retries and trust
  scalings; positions within 1e-6 m, rotations within 1e-6 rad)."""
import numpy as np
import pytest

import failure_cases as fc
import khs_native as kn
import parity
import refgpu
import scenes

pytestmark = pytest.mark.gpu

TOL = 1e-6
DIAG_FIELDS = ["kind", "frame_index", "substep", "requested_substeps", "attempted_substeps", "maximum_substeps",
               "adaptive_attempt_count", "strand_index", "element_index", "collider_triangle_index"]


def _solver(lib, scene, mode=None):
    s = kn.HairSolver(lib)
    scenes.load_into(s, scene)
    if mode is not None:
        s.set_solve_mode(mode)
    return s


def _diag(d):
    return {f: getattr(d, f) for f in DIAG_FIELDS}


@pytest.mark.parametrize("mode", [kn.MODE_PLAIN_FP64, kn.MODE_MIXED])
def test_line_search_exhausted(gpu_lib, oracle_lib, mode):
    sc = fc.line_search_exhausted()
    out = []
    for lib, m in ((gpu_lib, mode), (oracle_lib, None)):
        s = _solver(lib, sc, m)
        before = s.save_checkpoint()
        r = s._library.khsStepAnimationFrame(s.handle, 1, sc.frame_dt)
        out.append((r, _diag(s.failure_diagnostics()), s.save_checkpoint() == before))
        s.close()
    assert out[0] == out[1]
    assert out[0][0] == kn.ERROR_NOT_CONVERGED and out[0][1]["kind"] == kn.FAILURE_NONLINEAR_SOLVE and out[0][2]


@pytest.mark.parametrize("mode", [kn.MODE_PLAIN_FP64, kn.MODE_MIXED])
def test_infeasible_start(gpu_lib, oracle_lib, mode):
    sc = fc.infeasible_scene()
    out = []
    for lib, m in ((gpu_lib, mode), (oracle_lib, None)):
        s = _solver(lib, sc, m)
        bad = fc.infeasible_checkpoint(s.save_checkpoint(), sc)
        s.restore_checkpoint(bad)
        r = s._library.khsStepAnimationFrame(s.handle, 1, sc.frame_dt)
        out.append((r, _diag(s.failure_diagnostics()), s.save_checkpoint() == bad))
        s.close()
    assert out[0] == out[1]
    assert out[0][0] == kn.ERROR_NOT_CONVERGED and out[0][1]["kind"] == kn.FAILURE_BARRIER_INFEASIBLE and out[0][2]


@pytest.mark.parametrize("mode", [kn.MODE_PLAIN_FP64, kn.MODE_MIXED])
def test_cancel_from_another_thread(gpu_lib, mode):
    sc = scenes.ellipsoid_scene(strands=1000, frames=1)
    s = _solver(gpu_lib, sc, mode)
    before = s.save_checkpoint()
    r = fc.cancel_mid_frame(lambda: s._library.khsStepAnimationFrame(s.handle, 1, sc.frame_dt), s.progress, s.cancel)
    assert r == kn.ERROR_INVALID_STATE
    assert s.progress().cancelled == 1
    assert s.failure_diagnostics().kind == kn.FAILURE_NONE
    assert s.save_checkpoint() == before
    assert s._library.khsStepAnimationFrame(s.handle, 1, sc.frame_dt) == kn.OK
    again = s.save_checkpoint()
    s.close()
    t = _solver(gpu_lib, sc, mode)
    assert t._library.khsStepAnimationFrame(t.handle, 1, sc.frame_dt) == kn.OK
    assert t.save_checkpoint() == again
    t.close()


def _record_counts(frames):
    return [[(r.newton_iterations, r.line_search_evaluations, r.steepest_fallbacks, r.trust_scalings,
              r.contact_candidates, r.active_contacts) for r in fr["records"]] for fr in frames]


def _perturbed(make, eps):
    sc = make()
    base = sc.root_points_at
    sc.root_points_at = lambda f: base(f) * (1.0 + eps)
    return sc


# (scene, branch counter, substep limit): the steepest-descent scene takes a
# single line-search trial per direction and its state becomes sensitive
# after a few substeps, so its first four substeps are compared.
FALLBACK_SCENES = [(lambda: fc.steepest_heavy(frames=1), "steepest_fallbacks", 4),
                   (fc.root_jump, "trust_scalings", 0)]


@pytest.mark.parametrize("case", range(len(FALLBACK_SCENES)))
@pytest.mark.parametrize("mode", [kn.MODE_PLAIN_FP64, kn.MODE_MIXED])
def test_fallback_branches_keep_parity(gpu_lib, oracle_lib, case, mode):
    """Identical per-substep counts; positions and rotations within
    max(1e-6, 4 x the oracle's own change under a 1e-15 relative change of
    the root targets): steepest-descent steps with a single trial amplify
    last-bit differences (5e-6 m / 5e-4 rad after four substeps)."""
    make, field, limit = FALLBACK_SCENES[case]
    gpu = parity.run(gpu_lib, make(), mode=mode, substep_limit=limit)
    ora = parity.run(oracle_lib, make(), substep_limit=limit)
    own = [parity.compare(parity.run(oracle_lib, _perturbed(make, eps), substep_limit=limit), ora)
           for eps in (1e-15, -1e-15)]
    assert _record_counts(gpu) == _record_counts(ora)
    assert sum(getattr(r, field) for fr in gpu for r in fr["records"]) > 0
    for k, fr in enumerate(parity.compare(gpu, ora)):
        pos_tol = max(TOL, 4.0 * max(o[k]["max_position"] for o in own))
        rot_tol = max(TOL, 4.0 * max(o[k]["max_rotation"] for o in own))
        assert fr["result"] == (kn.OK, kn.OK), (k, fr)
        assert fr["max_position"] <= pos_tol and fr["max_rotation"] <= rot_tol, (k, fr, pos_tol, rot_tol)


# ---- the reference's own CUDA backend ---------------------------------------

@pytest.fixture(scope="module")
def ref_lib():
    if not refgpu.available():
        pytest.skip("the reference CUDA sources are not staged in oracle/_ref/src")
    return refgpu.RefLibrary()


def test_reference_failure_codes(ref_lib, oracle_lib):
    """The reference backend gives the same result codes and failure kinds
    on the same two failing frames."""
    sc = fc.line_search_exhausted()
    s = refgpu.RefSolver(ref_lib, oracle_lib, sc)
    before = s.save_checkpoint()
    assert s.step_animation_frame(1, sc.frame_dt) == kn.ERROR_NOT_CONVERGED
    d = s.failure()
    assert (d.kind, d.substep, d.attempted_substeps, d.adaptive_attempt_count) == (kn.FAILURE_NONLINEAR_SOLVE, 1, 32, 4)
    assert s.save_checkpoint() == before
    s.close()
    sc = fc.infeasible_scene()
    s = refgpu.RefSolver(ref_lib, oracle_lib, sc)
    bad = fc.infeasible_checkpoint(s.save_checkpoint(), sc)
    s.restore_checkpoint(bad)
    assert s.step_animation_frame(1, sc.frame_dt) == kn.ERROR_NOT_CONVERGED
    assert s.failure().kind == kn.FAILURE_BARRIER_INFEASIBLE
    assert s.save_checkpoint() == bad
    s.close()


def test_reference_cancel(ref_lib, oracle_lib):
    sc = scenes.ellipsoid_scene(strands=1000, frames=1)
    s = refgpu.RefSolver(ref_lib, oracle_lib, sc)
    before = s.save_checkpoint()
    r = fc.cancel_mid_frame(lambda: s.step_animation_frame(1, sc.frame_dt), s.progress, s.cancel)
    assert r == kn.ERROR_INVALID_STATE
    assert s.save_checkpoint() == before
    s.close()


def test_reference_trust_radius_branch(ref_lib, gpu_lib, oracle_lib):
    """The reference backend, the oracle and the GB300 library on the scene
    whose directions are scaled to the trust radius: same result codes,
    Newton and line-search counts; states within max(1e-6, 4 x the oracle's
    own change under a 1e-15 relative change of the root targets).  (The
    steepest-descent scene is compared only over its first substeps, which
    the reference backend cannot stop after.)"""
    ref = refgpu.run(ref_lib, oracle_lib, fc.root_jump())
    ora = parity.run(oracle_lib, fc.root_jump())
    gpu = parity.run(gpu_lib, fc.root_jump(), mode=kn.MODE_MIXED)
    own = parity.compare(parity.run(oracle_lib, _perturbed(fc.root_jump, 1e-15)), ora)
    for k, (a, b, c) in enumerate(zip(ref, ora, gpu)):
        assert a["result"] == b["result"] == c["result"] == kn.OK, k
        for f in ("newton_iterations", "line_search_evaluations"):
            assert getattr(a["stats"], f) == getattr(b["stats"], f) == getattr(c["stats"], f), (k, f)
        pos_tol = max(TOL, 4.0 * own[k]["max_position"])
        rot_tol = max(TOL, 4.0 * own[k]["max_rotation"])
        for other in (b, c):
            dq = np.abs(a["q"] - other["q"])
            assert dq[:, :3].max() <= pos_tol and dq[:, 3:].max() <= rot_tol, (k, dq[:, :3].max(), dq[:, 3:].max())
