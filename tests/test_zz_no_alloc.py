"""khsxQueryContactsNoAlloc against khsxQueryContacts.

The no-allocation entry point runs the same broad + narrow phase through a
file-scope device scratch array.  Two calls in a row on different states must
give records bit-identical to the allocating entry point, in both solve
modes, and must leave the solver's own contact records unchanged; solvers
whose state and records do not fit the scratch are rejected.  This file is
collected last so that it also runs after every other GPU test has used the
library in the same process.
"""
import numpy as np
import pytest

import parity
import scenes
import khs_native as kn

pytestmark = pytest.mark.gpu


def _surface_states(q0, count, seed):
    """States with nodes pulled towards the ellipsoid surface, so that many
    elements fall inside the barrier band and some inside the minimum gap."""
    rng = np.random.default_rng(seed)
    axes = np.array([0.09, 0.11, 0.12])
    out = []
    for _ in range(count):
        q = q0.copy()
        x = q[:, :3]
        r = np.linalg.norm(x / axes, axis=1, keepdims=True)
        target = 1.0 + rng.uniform(-0.002, 0.01, size=r.shape)
        q[:, :3] = x / r * target * np.where(rng.uniform(size=r.shape) < 0.5, 1.0, r / target)
        out.append(q)
    return out


def _bit_equal(a, b):
    mism = parity.records_equal(a, b)
    assert all(v == 0 for v in mism.values()), mism
    assert np.array_equal(a["gap"].view(np.uint64), b["gap"].view(np.uint64))
    assert np.array_equal(a["reserved"], b["reserved"])


@pytest.mark.parametrize("mode", [kn.MODE_PLAIN_FP64, kn.MODE_MIXED])
def test_no_alloc_query_matches_allocating_query(gpu_lib, mode):
    sc = scenes.ellipsoid_scene(strands=200, frames=1)
    s = kn.HairSolver(gpu_lib)
    scenes.load_into(s, sc)
    s.set_solve_mode(mode)
    q0, _ = s.state()
    count = s.build_stats().element_count
    for q in _surface_states(q0, 2, seed=11 + mode):
        expected = s.query_contacts(q)
        own = s.contact_records()
        got = np.zeros(count, dtype=kn.CONTACT_DTYPE)
        assert s.query_contacts_no_alloc(q, got) == kn.OK
        _bit_equal(got, expected)
        assert expected["active"].sum() > 0 and expected["candidate_count"].sum() > 0
        _bit_equal(s.contact_records(), own)
    s.close()


def test_no_alloc_query_after_stepping(gpu_lib):
    """After frames of a moving collider (the query uses the collider as the
    last substep left it), two calls in a row match the allocating query."""
    sc = scenes.sphere_scene(motion=True, frames=3)
    s = kn.HairSolver(gpu_lib)
    scenes.load_into(s, sc)
    s.set_solve_mode(kn.MODE_MIXED)
    count = s.build_stats().element_count
    for f in (1, 2):
        assert s._library.khsStepAnimationFrame(s.handle, f, sc.frame_dt) == kn.OK
        q, _ = s.state()
        for q_call in (q, q * (1.0 + 1e-9)):
            got = np.zeros(count, dtype=kn.CONTACT_DTYPE)
            assert s.query_contacts_no_alloc(q_call, got) == kn.OK
            _bit_equal(got, s.query_contacts(q_call))
    s.close()


def test_no_alloc_query_rejects_bad_sizes(gpu_lib):
    sc = scenes.ellipsoid_scene(strands=200, frames=1)
    s = kn.HairSolver(gpu_lib)
    scenes.load_into(s, sc, animation=False)
    q, _ = s.state()
    count = s.build_stats().element_count
    short = np.zeros(count - 1, dtype=kn.CONTACT_DTYPE)
    assert s.query_contacts_no_alloc(q, short) == kn.ERROR_INVALID_ARGUMENT
    full = np.zeros(count, dtype=kn.CONTACT_DTYPE)
    assert s.query_contacts_no_alloc(q[:-1], full) == kn.ERROR_INVALID_ARGUMENT
    s.close()

    big = scenes.ellipsoid_scene(strands=2000, frames=1)
    s = kn.HairSolver(gpu_lib)
    scenes.load_into(s, big, animation=False)
    st = s.build_stats()
    required = -(-48 * st.internal_node_count // 256) * 256 + 24 * st.element_count
    assert required > kn.NO_ALLOC_SCRATCH_BYTES
    q, _ = s.state()
    out = np.zeros(st.element_count, dtype=kn.CONTACT_DTYPE)
    assert s.query_contacts_no_alloc(q, out) == kn.ERROR_INVALID_ARGUMENT
    s.close()
