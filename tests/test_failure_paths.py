"""Failure-side branches of the frame driver on the CPU oracle, with the
reference's result codes and failure diagnostics (src/cuda_backend.cu:655,
657, 677-679, 711-716); the same cases run on the GB300 library in
test_gpu_failure_paths.py."""
import numpy as np

import failure_cases as fc
import khs_native as kn
import scenes


def _solver(lib, scene):
    s = kn.HairSolver(lib)
    scenes.load_into(s, scene)
    return s


def test_line_search_exhausted_reports_nonlinear_solve(oracle_lib):
    sc = fc.line_search_exhausted()
    s = _solver(oracle_lib, sc)
    before = s.save_checkpoint()
    r = s._library.khsStepAnimationFrame(s.handle, 1, sc.frame_dt)
    assert r == kn.ERROR_NOT_CONVERGED
    assert "line search" in s.last_error()
    d = s.failure_diagnostics()
    assert (d.kind, d.frame_index, d.substep) == (kn.FAILURE_NONLINEAR_SOLVE, 1, 1)
    assert (d.requested_substeps, d.attempted_substeps, d.maximum_substeps, d.adaptive_attempt_count) == (4, 32, 32, 4)
    assert s.save_checkpoint() == before  # the frame-start state is restored
    s.close()


def test_infeasible_start_reports_barrier_infeasible(oracle_lib):
    sc = fc.infeasible_scene()
    s = _solver(oracle_lib, sc)
    bad = fc.infeasible_checkpoint(s.save_checkpoint(), sc)
    s.restore_checkpoint(bad)
    r = s._library.khsStepAnimationFrame(s.handle, 1, sc.frame_dt)
    assert r == kn.ERROR_NOT_CONVERGED
    assert "barrier" in s.last_error()
    d = s.failure_diagnostics()
    assert (d.kind, d.frame_index, d.substep, d.adaptive_attempt_count) == (kn.FAILURE_BARRIER_INFEASIBLE, 1, 1, 4)
    assert s.save_checkpoint() == bad
    s.close()


def test_cancel_from_another_thread(oracle_lib):
    sc = scenes.ellipsoid_scene(strands=200, frames=1)
    s = _solver(oracle_lib, sc)
    before = s.save_checkpoint()
    r = fc.cancel_mid_frame(lambda: s._library.khsStepAnimationFrame(s.handle, 1, sc.frame_dt), s.progress, s.cancel)
    assert r == kn.ERROR_INVALID_STATE
    assert s.progress().cancelled == 1
    assert s.failure_diagnostics().kind == kn.FAILURE_NONE  # a cancel is not a failure (cuda_backend.cu:711)
    assert s.save_checkpoint() == before
    # The frame can be stepped again and gives the uncancelled result.
    assert s._library.khsStepAnimationFrame(s.handle, 1, sc.frame_dt) == kn.OK
    again = s.state()
    s.close()
    t = _solver(oracle_lib, sc)
    assert t._library.khsStepAnimationFrame(t.handle, 1, sc.frame_dt) == kn.OK
    q, v = t.state()
    assert np.array_equal(q, again[0]) and np.array_equal(v, again[1])
    t.close()


def test_branch_scenes_take_their_branches(oracle_lib):
    """The scenes used for parity of the fallback branches really take them."""
    for make, field in ((fc.steepest_heavy, "steepest_fallbacks"), (fc.root_jump, "trust_scalings")):
        sc = make()
        s = _solver(oracle_lib, sc)
        total = 0
        for f in range(1, sc.frames):
            assert s._library.khsStepAnimationFrame(s.handle, f, sc.frame_dt) == kn.OK, s.last_error()
            total += sum(getattr(r, field) for r in s.substep_records())
        assert total > 0, field
        s.close()
