"""Generates tests/golden/oracle_trajectories.npz: per-frame node states
(q: positions and rotation vectors of every internal node), step counters
and per-element contact records of the CPU FP64 oracle on two seeded scenes:

* sphere_moving -- scenes.sphere_scene(motion=True, frames=3): 64 strands x
  32 nodes on a rotating, drifting 0.1 m sphere (icosphere L3), 4 substeps;
* ellipsoid40   -- scenes.ellipsoid_scene(strands=40, frames=2): helical
  strands on a rotating ellipsoid (icosphere L5), 8 substeps.

The oracle is pinned on the reference's own test invariants
(tests/test_oracle_reference_invariants.py); these fixtures freeze its
trajectories so later changes to either library are checked against the
same numbers.  Run:  python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path[:0] = [str(REPO / "kami-hair-solver_gb300"), str(REPO / "tests")]

import conftest  # noqa: E402
import khs_native as kn  # noqa: E402
import scenes  # noqa: E402

CASES = {
    "sphere_moving": lambda: scenes.sphere_scene(motion=True, frames=3),
    "ellipsoid40": lambda: scenes.ellipsoid_scene(strands=40, frames=2),
}


def trajectory(lib, scene):
    s = kn.HairSolver(lib)
    scenes.load_into(s, scene)
    out = {"q": [], "stats": [], "contacts": []}
    for f in range(1, scene.frames):
        r = s._library.khsStepAnimationFrame(s.handle, f, scene.frame_dt)
        assert r == kn.OK, s.last_error()
        st = s.stats()
        out["q"].append(s.state()[0])
        out["stats"].append([st.substeps, st.newton_iterations, st.line_search_evaluations,
                             st.contact_candidate_count, st.active_contact_count])
        out["contacts"].append(s.contact_records())
    s.close()
    return out


def main():
    lib = kn.Library(conftest.build_oracle())
    arrays = {}
    for name, make in CASES.items():
        t = trajectory(lib, make())
        arrays[f"{name}_q"] = np.stack(t["q"])
        arrays[f"{name}_stats"] = np.asarray(t["stats"], dtype=np.uint64)
        c = np.stack(t["contacts"])
        for field in ("candidate_count", "closest_triangle", "active"):
            arrays[f"{name}_{field}"] = c[field]
        arrays[f"{name}_gap"] = c["gap"]
    np.savez_compressed(HERE / "oracle_trajectories.npz", **arrays)
    print({k: v.shape for k, v in arrays.items()})


if __name__ == "__main__":
    main()
