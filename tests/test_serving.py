"""Serving loop host logic on CPU with the oracle library: requests are
admitted by slot and byte budget (never exceeding either), every request
completes, and each result equals the same request run alone."""
import numpy as np

import khs_native as kn
import scenes
import serving


def _stream(n, seed=9):
    reqs = []
    for i in range(n):
        sc = scenes.sphere_scene(seed=seed + i, strands=6 + 2 * i, nodes=8, frames=2, motion=True)
        reqs.append(serving.Request(rid=i, scene=sc, arrival=0.01 * i, frames=2))
    return reqs


def test_admission_respects_budget_and_results_match_solo(oracle_lib):
    oracle_lib.lib.khsOracleSetThreads(1)
    reqs = _stream(5)
    sizes = [serving.estimate_bytes(r.scene, 0) for r in reqs]
    budget = max(sizes) + min(sizes)  # at most two requests fit at once
    server = serving.Server(oracle_lib, budget, max_slots=3, mode=kn.MODE_PLAIN_FP64, ring_slots=0)
    mixed = server.run(reqs)
    assert server.peak_bytes <= budget and server.peak_slots <= 3
    assert all(r.status == kn.OK for r in mixed), [r.error for r in mixed]
    for req, res in zip(reqs, mixed):
        solo = serving.run_request(oracle_lib, req, kn.MODE_PLAIN_FP64, 0)
        assert np.array_equal(solo.q, res.q)
        assert len(res.frame_ms) == req.frames
    s = serving.summary(mixed, server.makespan)
    assert s["completed"] == len(reqs) and s["p99_frame_ms"] >= s["p50_frame_ms"] > 0


def test_request_over_budget_is_rejected(oracle_lib):
    reqs = _stream(2)
    server = serving.Server(oracle_lib, serving.estimate_bytes(reqs[0].scene, 0), max_slots=2,
                            mode=kn.MODE_PLAIN_FP64, ring_slots=0)
    res = server.run(reqs)
    assert res[0].status == kn.OK
    assert res[1].status == kn.ERROR_INVALID_ARGUMENT and "budget" in res[1].error


def _fake_runner(actual, hold_s):
    """A request runner that reports ``actual`` resident bytes once built
    and then occupies its slot for ``hold_s`` seconds."""
    import time

    def run(lib, req, mode, ring_slots, on_resident=None):
        if on_resident is not None:
            on_resident(actual)
        time.sleep(hold_s)
        return serving.Result(rid=req.rid, frame_ms=[1.0], substeps=[8], nodes=10, resident=actual)
    return run


def test_admission_uses_the_solvers_reported_bytes():
    """A request reserves its estimate while it builds and then holds only
    the bytes its solver reports, so a second request that did not fit next
    to the first one's estimate is admitted while the first still runs."""
    reqs = [serving.Request(rid=i, scene=None, arrival=0.0, frames=1) for i in range(2)]
    estimate = lambda scene, ring: 6  # noqa: E731
    server = serving.Server(None, budget_bytes=10, max_slots=4, estimate=estimate, runner=_fake_runner(3, 0.3))
    res = server.run(reqs)
    assert all(r.status == kn.OK for r in res)
    assert server.peak_slots == 2  # 3 reported + 6 reserved fit in 10
    assert server.peak_bytes <= 10
    # With the estimate held for the whole run the two never overlap.
    server = serving.Server(None, budget_bytes=10, max_slots=4, estimate=estimate, runner=_fake_runner(6, 0.1))
    server.run(reqs)
    assert server.peak_slots == 1


def test_reported_bytes_above_the_estimate_hold_back_admission():
    reqs = [serving.Request(rid=i, scene=None, arrival=0.0, frames=1) for i in range(3)]
    server = serving.Server(None, budget_bytes=10, max_slots=4, estimate=lambda scene, ring: 4,
                            runner=_fake_runner(7, 0.2))
    res = server.run(reqs)
    assert all(r.status == kn.OK for r in res)
    assert len(res) == 3 and server.peak_slots <= 2


def test_rejected_request_reports_the_solver_result(oracle_lib):
    """A request whose hair starts inside the closed collider is rejected by
    khsBuild with KHS_ERROR_INITIAL_INTERSECTION, and the serving loop
    reports that code (not a generic internal error); the other requests of
    the stream complete."""
    import numpy as np

    good = scenes.sphere_scene(seed=3, strands=6, nodes=8, frames=2, motion=True)
    bad = scenes.sphere_scene(seed=3, strands=6, nodes=8, frames=2, motion=True)
    bad.points = np.asarray(bad.points) * 0.5  # every hair point inside the unit-radius sphere collider
    bad.root_points_at = lambda f: bad.points
    reqs = [serving.Request(rid=0, scene=good, arrival=0.0, frames=1), serving.Request(rid=1, scene=bad, arrival=0.0, frames=1)]
    server = serving.Server(oracle_lib, 10 ** 12, max_slots=2, mode=kn.MODE_PLAIN_FP64, ring_slots=0)
    res = server.run(reqs)
    assert res[0].status == kn.OK
    assert res[1].status == kn.ERROR_INITIAL_INTERSECTION, (res[1].status, res[1].error)
    assert serving.summary(res, server.makespan)["failed_by_result"] == {str(kn.ERROR_INITIAL_INTERSECTION): 1}
