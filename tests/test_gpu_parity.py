"""Parity of the GB300 plain FP64 solve with the CPU FP64 oracle.

Same seeded scenes through both libraries; per frame:
* node positions within 1e-6 m and rotation vectors within 1e-6 rad
  (the tolerance stated for FP64 trajectories; the two differ only by the
  rounding of transcendental functions and of reduction order),
* identical Gauss-Newton / line-search / substep counts and identical
  candidate and active-contact totals,
* integer contact work bit-exact: at the GPU's own state the oracle's
  broad + narrow phase gives the same per-element candidate count, closest
  triangle, active flag and gap bits as the GPU's last evaluation, and on
  identical perturbed states both libraries classify every element
  identically.
"""
import numpy as np
import pytest

import parity
import scenes
import khs_native as kn

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _check(report, rotation_tol=None):
    for k, fr in enumerate(report):
        assert fr["result"][0] == fr["result"][1], (k, fr)
        assert fr["max_position"] <= TOL, (k, fr)
        assert fr["max_rotation"] <= (rotation_tol[k] if rotation_tol else TOL), (k, fr)
        assert fr["newton"][0] == fr["newton"][1], (k, fr)
        assert fr["line_search"][0] == fr["line_search"][1], (k, fr)
        assert fr["substeps"][0] == fr["substeps"][1], (k, fr)
        assert fr["candidates"][0] == fr["candidates"][1], (k, fr)
        assert fr["active"][0] == fr["active"][1], (k, fr)
        if "own_state_mismatch" in fr:
            assert all(v == 0 for v in fr["own_state_mismatch"].values()), (k, fr)


def test_sphere_static_single_frame(gpu_lib, oracle_lib):
    sc = scenes.sphere_scene(motion=False, frames=1)
    _check(parity.compare(parity.run(gpu_lib, sc, probe=oracle_lib), parity.run(oracle_lib, sc)))


def test_sphere_moving(gpu_lib, oracle_lib):
    sc = scenes.sphere_scene(motion=True, frames=3)
    rep = parity.compare(parity.run(gpu_lib, sc, probe=oracle_lib), parity.run(oracle_lib, sc))
    print(rep)
    _check(rep)


def _perturbed(scene, eps):
    base = scene.root_points_at
    scene.root_points_at = lambda f: base(f) * (1.0 + eps)
    return scene


def test_ellipsoid_contact(gpu_lib, oracle_lib):
    """Contact-heavy frames that exhaust the 24-iteration Newton budget: the
    weakly constrained twist of some nodes makes the rotation iterate
    sensitive at the 1e-6 rad level to last-bit changes of the inputs.  The
    oracle's own sensitivity is measured by rerunning it with the root
    targets scaled by (1 + 1e-15); rotations must agree within
    max(1e-6 rad, 4 x that sensitivity), positions within 1e-6 m."""
    sc = scenes.ellipsoid_scene(strands=40, frames=2)
    ref = parity.run(oracle_lib, sc)
    rep = parity.compare(parity.run(gpu_lib, sc, probe=oracle_lib), ref)
    own = parity.compare(parity.run(oracle_lib, _perturbed(scenes.ellipsoid_scene(strands=40, frames=2), 1e-15)), ref)
    rot_tol = [max(TOL, 4.0 * fr["max_rotation"]) for fr in own]
    print(rep, rot_tol)
    _check(rep, rot_tol)


def test_contact_query_bitexact_on_identical_states(gpu_lib, oracle_lib):
    """Both libraries classify the same perturbed states identically."""
    sc = scenes.ellipsoid_scene(strands=200, frames=1)
    solvers = []
    for lib in (gpu_lib, oracle_lib):
        s = kn.HairSolver(lib)
        scenes.load_into(s, sc)
        solvers.append(s)
    q0, _ = solvers[1].state()
    rng = np.random.default_rng(7)
    axes = np.array([0.09, 0.11, 0.12])
    for trial in range(4):
        q = q0.copy()
        # Pull nodes towards the surface so many elements fall inside the
        # barrier band, some inside the minimum gap.
        x = q[:, :3]
        r = np.linalg.norm(x / axes, axis=1, keepdims=True)
        target = 1.0 + rng.uniform(-0.002, 0.01, size=r.shape)
        q[:, :3] = x / r * target * np.where(rng.uniform(size=r.shape) < 0.5, 1.0, r / target)
        a = solvers[0].query_contacts(q)
        b = solvers[1].query_contacts(q)
        mism = parity.records_equal(a, b)
        assert all(v == 0 for v in mism.values()), (trial, mism)
        assert a["active"].sum() > 0 and a["candidate_count"].sum() > 0
    for s in solvers:
        s.close()


# ---- mixed form -----------------------------------------------------------

def test_mixed_sphere_moving(gpu_lib, oracle_lib):
    sc = scenes.sphere_scene(motion=True, frames=3)
    rep = parity.compare(parity.run(gpu_lib, sc, mode=kn.MODE_MIXED, probe=oracle_lib), parity.run(oracle_lib, sc))
    print(rep)
    _check(rep)


def test_mixed_ellipsoid_contact(gpu_lib, oracle_lib):
    sc = scenes.ellipsoid_scene(strands=40, frames=2)
    ref = parity.run(oracle_lib, sc)
    rep = parity.compare(parity.run(gpu_lib, sc, mode=kn.MODE_MIXED, probe=oracle_lib), ref)
    own = parity.compare(parity.run(oracle_lib, _perturbed(scenes.ellipsoid_scene(strands=40, frames=2), 1e-15)), ref)
    rot_tol = [max(TOL, 4.0 * fr["max_rotation"]) for fr in own]
    print(rep, rot_tol)
    _check(rep, rot_tol)


def test_mixed_pole_dense_leaves(gpu_lib, oracle_lib):
    """Elements next to the pole of a UV sphere, where 360 sliver triangles
    meet, reach hundreds of BVH leaves: more than the 32 an element caches,
    so the mixed form keeps their leaf lists in the leaf pool and the
    warp-cooperative passes take them 32 at a time.  The mixed form must
    reproduce the plain form's trajectory bit for bit, and at its own state
    the oracle's per-element contact classification."""
    mixed = parity.run(gpu_lib, scenes.pole_scene(frames=2), mode=kn.MODE_MIXED, probe=oracle_lib)
    plain = parity.run(gpu_lib, scenes.pole_scene(frames=2), mode=kn.MODE_PLAIN_FP64)
    assert max(int(fr["contacts"]["candidate_count"].max()) for fr in mixed) > 32 * 8
    assert len(mixed) == len(plain) == 2
    for k, (fm, fp) in enumerate(zip(mixed, plain)):
        assert fm["result"] == fp["result"] == kn.OK, (k, fm["error"], fp["error"])
        assert np.array_equal(fm["q"], fp["q"]) and np.array_equal(fm["v"], fp["v"]), k
        assert all(v == 0 for v in parity.records_equal(fm["contacts"], fp["contacts"]).values()), k
        assert all(v == 0 for v in parity.records_equal(fm["contacts"], fm["probe_contacts"]).values()), k


def test_mixed_contact_query_bitexact(gpu_lib, oracle_lib):
    """The FP32 broadphase + FP32-filtered narrow phase classifies every
    element exactly like the FP64 oracle (candidate counts, closest
    triangle, active flag, gap bits)."""
    sc = scenes.ellipsoid_scene(strands=200, frames=1)
    g = kn.HairSolver(gpu_lib)
    scenes.load_into(g, sc)
    g.set_solve_mode(kn.MODE_MIXED)
    o = kn.HairSolver(oracle_lib)
    scenes.load_into(o, sc)
    q0, _ = o.state()
    rng = np.random.default_rng(11)
    axes = np.array([0.09, 0.11, 0.12])
    for trial in range(4):
        q = q0.copy()
        x = q[:, :3]
        r = np.linalg.norm(x / axes, axis=1, keepdims=True)
        target = 1.0 + rng.uniform(-0.002, 0.01, size=r.shape)
        q[:, :3] = x / r * target * np.where(rng.uniform(size=r.shape) < 0.5, 1.0, r / target)
        mism = parity.records_equal(g.query_contacts(q), o.query_contacts(q))
        assert all(v == 0 for v in mism.values()), (trial, mism)
    g.close()
    o.close()


# ---- float-float factorisation with FP64 refinement -------------------------

def test_mixed_ff_sphere_moving(gpu_lib, oracle_lib):
    """Float-float block factorisation + FP64 refinement on the Gauss-Newton
    residual: the moving-sphere frames stay within 1e-6 m / 1e-6 rad of the
    FP64 oracle with identical Newton, line-search and substep counts; every
    direction took at least one refinement sweep and none fell back to the
    FP64 factorisation."""
    sc = scenes.sphere_scene(motion=True, frames=3)
    out = parity.run(gpu_lib, sc, mode=kn.MODE_MIXED_FF, probe=oracle_lib)
    rep = parity.compare(out, parity.run(oracle_lib, sc))
    print(rep)
    _check(rep)
    sweeps = sum(r.refinement_sweeps for fr in out for r in fr["records"])
    newton = sum(r.newton_iterations for fr in out for r in fr["records"])
    assert sum(r.fp64_fallbacks for fr in out for r in fr["records"]) == 0
    assert sweeps >= newton > 0


def test_block_solve_layouts_bit_identical(gpu_lib):
    """Every block-solve launch shape (5 strands of 6 lanes, 2 of 12 or 1 of
    18 lanes per warp, the longest strands on 18 lanes or on a pair of warps
    and the rest five per warp, any number of blocks per SM) gives bit-identical
    trajectories, so the one-time launch tuning cannot change a result."""
    sc = scenes.ellipsoid_scene(strands=200, frames=2)
    finals = []
    for spw, bps, nlong in ((5, 1, 0), (2, 1, 0), (2, 3, 0), (5, 4, 0), (1, 1, 0), (5, 2, 17), (1, 1, 17), (1, 2, 40)):
        s = kn.HairSolver(gpu_lib)
        scenes.load_into(s, sc)
        s.set_block_solve_schedule(spw, bps, nlong)
        for f in range(1, sc.frames):
            assert s._library.khsStepAnimationFrame(s.handle, f, sc.frame_dt) == kn.OK, s.last_error()
        finals.append(s.state())
        s.close()
    for q, v in finals[1:]:
        assert np.array_equal(q, finals[0][0]) and np.array_equal(v, finals[0][1])


def test_block_solve_tiers_bit_identical(gpu_lib):
    """The tiered shapes (the longest strands on four warps each, then one
    and two per warp, the rest five per warp; odd pair counts, every strand
    on four warps, 1-3 blocks per SM) give the same trajectory bit for bit
    as the five-per-warp layout, and the tuned shape does too."""
    sc = scenes.ellipsoid_scene(strands=200, frames=2)
    shapes = [None, "tuned", (10, 20, 41, 2), (37, 0, 0, 3), (1, 1, 1, 1), (200, 0, 0, 2), (0, 60, 60, 2), (25, 25, 150, 3)]
    finals = []
    for shape in shapes:
        s = kn.HairSolver(gpu_lib)
        scenes.load_into(s, sc)
        if shape is None:
            s.set_block_solve_schedule(5, 1, 0)
        elif shape != "tuned":
            s.set_block_solve_tiers(*shape)
        for f in range(1, sc.frames):
            assert s._library.khsStepAnimationFrame(s.handle, f, sc.frame_dt) == kn.OK, s.last_error()
        finals.append(s.state())
        s.close()
    for shape, (q, v) in zip(shapes[1:], finals[1:]):
        assert np.array_equal(q, finals[0][0]) and np.array_equal(v, finals[0][1]), shape
    s = kn.HairSolver(gpu_lib)
    scenes.load_into(s, sc)
    assert s._library.khsxSetBlockSolveTiers(s.handle, 150, 40, 20, 2) == kn.ERROR_INVALID_ARGUMENT  # > strands
    assert s._library.khsxSetBlockSolveTiers(s.handle, 1, 1, 1, 0) == kn.ERROR_INVALID_ARGUMENT
    s.close()
