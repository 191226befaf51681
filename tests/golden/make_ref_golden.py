"""Generates tests/golden/reference_gpu.npz: trajectories of the reference's
own FP64 CUDA backend (src/cuda_backend.cu compiled unchanged for sm_103a,
driven through oracle/ref_bridge.cpp) on the seeded scenes of the tests.

Runs on a machine with a CUDA device and the reference sources staged in
oracle/_ref/src (``make -C oracle stage-ref REFERENCE=<checkout>`` where the
reference is checked out; the staged folder travels with the working tree).

    python tests/golden/make_ref_golden.py [out.npz]

Per case and stepped frame it records the result code, the step statistics
(counts and norms), the reference's wall time per frame, and the node state
(q: positions and rotation vectors).  The reference sums gradient, Hessian,
energies and friction with double atomics, so two runs of it differ in the
last bits; every case is therefore run twice and the per-frame maximum
position and rotation difference between the two runs is stored as the
reference's own run-to-run spread.  Small cases keep q and v of every node;
the 1,000-strand ellipsoid and the 265k-node body scene keep q of a fixed
sample of nodes (every 37th / 97th) to keep the fixture small.
"""
from __future__ import annotations

import subprocess
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path[:0] = [str(REPO / "kami-hair-solver_gb300"), str(REPO / "tests"), str(REPO / "oracle")]

import khs_native as kn  # noqa: E402
import refgpu  # noqa: E402
import scenes  # noqa: E402

STAT_FIELDS = ["substeps", "converged_substeps", "newton_iterations", "linear_solves", "line_search_evaluations",
               "contact_candidate_count", "active_contact_count", "initial_residual_norm", "final_residual_norm",
               "relative_residual_norm", "increment_norm", "minimum_gap", "accepted_step_length", "ccd_step_limit",
               "kinetic_energy", "elastic_energy", "contact_energy"]

CASES = {
    "sphere_static": (lambda: scenes.sphere_scene(motion=False, frames=1), None),
    "sphere_moving": (lambda: scenes.sphere_scene(motion=True, frames=3), None),
    "ellipsoid40": (lambda: scenes.ellipsoid_scene(strands=40, frames=2), None),
    "pole": (lambda: scenes.pole_scene(frames=2), None),
    "ellipsoid1000": (lambda: scenes.ellipsoid_scene(), 37),
    "body5": (lambda: scenes.body_scene(frames=5), 97),
}


def stats_row(st) -> np.ndarray:
    return np.array([float(getattr(st, f)) for f in STAT_FIELDS])


def run_case(ref, oracle, make, every):
    runs = []
    for rep in range(2):
        sc = make()
        s = refgpu.RefSolver(ref, oracle, sc)
        frames = []
        for f in range(1, sc.frames):
            t0 = time.perf_counter()
            r = s.step_animation_frame(f, sc.frame_dt)
            wall = time.perf_counter() - t0
            q, v = s.state()
            frames.append(dict(result=r, stats=stats_row(s.stats()), q=q, v=v, wall=wall))
            print(f"  run {rep} frame {f}: result {r} newton {int(s.stats().newton_iterations)} "
                  f"substeps {int(s.stats().substeps)} {wall * 1e3:.0f} ms", flush=True)
            if r != kn.OK:
                break
        s.close()
        runs.append(frames)
    a, b = runs
    out = {}
    n = len(a)
    out["result"] = np.array([fr["result"] for fr in a], dtype=np.int32)
    out["stats"] = np.stack([fr["stats"] for fr in a])
    out["wall_s"] = np.array([[fa["wall"], fb["wall"]] for fa, fb in zip(a, b)])
    spread = []
    for fa, fb in zip(a, b):
        d = np.abs(fa["q"] - fb["q"])
        spread.append([d[:, :3].max(), d[:, 3:].max()])
    out["spread"] = np.array(spread)
    out["stats_b"] = np.stack([fr["stats"] for fr in b])
    if every is None:
        out["q"] = np.stack([fr["q"] for fr in a])
        out["v"] = np.stack([fr["v"] for fr in a])
    else:
        idx = np.arange(0, a[0]["q"].shape[0], every, dtype=np.int64)
        out["sample"] = idx
        out["q"] = np.stack([fr["q"][idx] for fr in a])
    assert len(b) == n
    return out


def main(out_path: Path) -> None:
    ref = refgpu.RefLibrary()
    subprocess.run(["make", "-s", "-C", str(REPO / "oracle")], check=True)
    oracle = kn.Library(REPO / "oracle" / "_build" / "libkhs_oracle.so")
    data = {"stat_fields": np.array(STAT_FIELDS)}
    only = set(sys.argv[2:])
    for name, (make, every) in CASES.items():
        if only and name not in only:
            continue
        print(name, flush=True)
        for k, val in run_case(ref, oracle, make, every).items():
            data[f"{name}__{k}"] = val
    np.savez_compressed(out_path, **data)
    print("wrote", out_path)


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else HERE / "reference_gpu.npz")
