"""Mixed-precision report on the 1,000-strand rotating ellipsoid (1,000
helical strands of 20-120 nodes, ~70k nodes, a 20,480-triangle ellipsoid
rotating at 2 rad/s, 10 frames x 8 substeps).

The float-float mode (``KHSX_MODE_MIXED_FF``: the block-tridiagonal
factorisation in float-float with FP64 refinement of the Gauss-Newton
residual, at most 3 sweeps, FP64 fallback) and the mixed form
(``KHSX_MODE_MIXED``: FP32 filters, FP64 solve, bit-identical to plain FP64)
are compared with the CPU FP64 oracle:

* per frame, over the whole trajectory: the largest node position and
  rotation-vector difference, and the relative difference of the total
  energy (kinetic + elastic + contact of the frame's last iterate).  The
  reference's own CUDA backend differs from itself by its run-to-run spread
  (from ``tests/golden/reference_gpu.npz``), listed beside them: these
  contact-heavy, iteration-capped frames amplify last-bit differences;
* per substep from a common state: from the mixed form's checkpoint at the
  start of every frame, the oracle and both GB300 forms run one substep;
  largest position and rotation difference and energy relative difference
  of that substep, and whether the Newton and line-search counts agree;
* the refinement sweeps of the float-float mode: solves (one per Gauss-
  Newton iteration), sweeps, FP64 fallbacks, and a histogram over substeps
  of the sweeps beyond one per solve.

Needs a CUDA device (runs the GB300 library and the oracle on the host):

    python tests/mixed_precision_report.py out.json
"""
from __future__ import annotations

import json
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
sys.path[:0] = [str(REPO / "kami-hair-solver_gb300"), str(HERE)]

import khs_native as kn  # noqa: E402
import scenes  # noqa: E402


def _energy(st) -> float:
    return float(st.kinetic_energy + st.elastic_energy + st.contact_energy)


def trajectory(lib, make, mode=None) -> dict:
    """Steps every frame; per frame q, total energy and substep records."""
    sc = make()
    s = kn.HairSolver(lib)
    scenes.load_into(s, sc)
    if mode is not None:
        s.set_solve_mode(mode)
    out = {"q": [], "energy": [], "records": [], "checkpoints": [], "seconds": []}
    for f in range(1, sc.frames):
        out["checkpoints"].append(s.save_checkpoint())
        t0 = time.perf_counter()
        r = s._library.khsStepAnimationFrame(s.handle, f, sc.frame_dt)
        out["seconds"].append(time.perf_counter() - t0)
        assert r == kn.OK, (f, s.last_error())
        out["q"].append(s.state()[0])
        out["energy"].append(_energy(s.stats()))
        out["records"].append([(r.newton_iterations, r.line_search_evaluations, r.refinement_sweeps, r.fp64_fallbacks)
                               for r in s.substep_records()])
    s.close()
    return out


def one_substep(lib, make, checkpoint, frame, mode=None):
    sc = make()
    s = kn.HairSolver(lib)
    scenes.load_into(s, sc, frames=frame + 1)
    if mode is not None:
        s.set_solve_mode(mode)
    s.set_substep_limit(1)
    s.restore_checkpoint(checkpoint)
    r = s._library.khsStepAnimationFrame(s.handle, frame, sc.frame_dt)
    assert r == kn.OK, (frame, s.last_error())
    q = s.state()[0]
    e = _energy(s.stats())
    rec = s.substep_records()[0]
    s.close()
    return q, e, (rec.newton_iterations, rec.line_search_evaluations)


def _dev(a, b):
    d = np.abs(a - b)
    return float(d[:, :3].max()), float(d[:, 3:].max())


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def main(out_path: Path) -> None:
    import khs_build

    gpu = kn.Library(khs_build.build())
    subprocess.run(["make", "-s", "-C", str(REPO / "oracle")], check=True)
    oracle = kn.Library(REPO / "oracle" / "_build" / "libkhs_oracle.so")
    make = scenes.ellipsoid_scene
    t0 = time.perf_counter()
    ff = trajectory(gpu, make, kn.MODE_MIXED_FF)
    mixed = trajectory(gpu, make, kn.MODE_MIXED)
    orc = trajectory(oracle, make)
    print(f"trajectories in {time.perf_counter() - t0:.0f} s", flush=True)
    spread = None
    fixture = HERE / "golden" / "reference_gpu.npz"
    if fixture.exists():
        spread = np.load(fixture)["ellipsoid1000__spread"]
    frames = []
    for i in range(len(orc["q"])):
        f = i + 1
        row = {"frame": f,
               "ff_position_m": _dev(ff["q"][i], orc["q"][i])[0], "ff_rotation_rad": _dev(ff["q"][i], orc["q"][i])[1],
               "ff_energy_rel": _rel(ff["energy"][i], orc["energy"][i]),
               "mixed_position_m": _dev(mixed["q"][i], orc["q"][i])[0],
               "mixed_rotation_rad": _dev(mixed["q"][i], orc["q"][i])[1],
               "mixed_energy_rel": _rel(mixed["energy"][i], orc["energy"][i]),
               "substeps": len(orc["records"][i]),
               "newton_oracle": sum(r[0] for r in orc["records"][i]),
               "newton_ff": sum(r[0] for r in ff["records"][i])}
        if spread is not None and i < len(spread):
            row["reference_self_position_m"] = float(spread[i][0])
            row["reference_self_rotation_rad"] = float(spread[i][1])
        # One substep from the mixed form's state at this frame's start.
        ck = mixed["checkpoints"][i]
        q_o, e_o, c_o = one_substep(oracle, make, ck, f)
        for name, mode in (("ff", kn.MODE_MIXED_FF), ("mixed", kn.MODE_MIXED)):
            q_g, e_g, c_g = one_substep(gpu, make, ck, f, mode)
            p, r = _dev(q_g, q_o)
            row[f"substep_{name}_position_m"] = p
            row[f"substep_{name}_rotation_rad"] = r
            row[f"substep_{name}_energy_rel"] = _rel(e_g, e_o)
            row[f"substep_{name}_same_counts"] = c_g == c_o
        frames.append(row)
        print(json.dumps(row), flush=True)
    recs = [r for fr in ff["records"] for r in fr]
    solves = sum(r[0] for r in recs)
    sweeps = sum(r[2] for r in recs)
    extra = [r[2] - r[0] for r in recs]
    hist = {str(k): int(sum(1 for x in extra if x == k)) for k in sorted(set(extra))}
    report = {
        "workload": "1,000 helical strands (20-120 nodes, 69k nodes), 20,480-triangle ellipsoid rotating at 2 rad/s, "
                    "frames 1-9, 8 base substeps",
        "frames": frames,
        "refinement": {"substeps": len(recs), "solves": solves, "sweeps": sweeps,
                       "fp64_fallbacks": int(sum(r[3] for r in recs)),
                       "extra_sweeps_per_substep_histogram": hist, "max_sweeps_per_solve": 3},
        "seconds": {"ff": float(sum(ff["seconds"])), "mixed": float(sum(mixed["seconds"])),
                    "oracle": float(sum(orc["seconds"]))},
    }
    out_path.write_text(json.dumps(report, indent=1) + "\n")
    print(json.dumps(report["refinement"]), json.dumps(report["seconds"]))
    print("wrote", out_path)


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path("mixed_precision_report.json"))
