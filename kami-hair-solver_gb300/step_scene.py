"""Steps one of the seeded scenes through the C ABI and prints one JSON line
per frame (result, substeps, Gauss-Newton iterations, contacts, device
milliseconds).  A small command line for trying the library and for
profiling one kernel of a known workload (for example under ncu with a
kernel filter):

    python kami-hair-solver_gb300/step_scene.py --scene body --frames 1
    python kami-hair-solver_gb300/step_scene.py --scene ellipsoid --frames 3 --mode plain

Scenes: ``sphere`` (64 strands x 32 nodes on a moving sphere), ``ellipsoid``
(1,000 helical strands on a rotating 20,480-triangle ellipsoid), ``body``
(6,757 strands / 265,108 nodes on a swaying 449,940-triangle head and
torso).
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent))

import khs_build  # noqa: E402
import khs_native as kn  # noqa: E402
import scenes  # noqa: E402

SCENES = {
    "sphere": lambda frames: scenes.sphere_scene(motion=True, frames=frames + 1),
    "ellipsoid": lambda frames: scenes.ellipsoid_scene(frames=frames + 1),
    "body": lambda frames: scenes.body_scene(frames=frames + 1),
}
MODES = {"plain": kn.MODE_PLAIN_FP64, "mixed": kn.MODE_MIXED, "mixed-ff": kn.MODE_MIXED_FF}


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--scene", choices=sorted(SCENES), default="body")
    ap.add_argument("--frames", type=int, default=1)
    ap.add_argument("--mode", choices=sorted(MODES), default="mixed")
    args = ap.parse_args()
    lib = kn.Library(khs_build.build())
    sc = SCENES[args.scene](args.frames)
    s = kn.HairSolver(lib)
    scenes.load_into(s, sc)
    s.set_solve_mode(MODES[args.mode])
    status = 0
    for f in range(1, args.frames + 1):
        r = s._library.khsStepAnimationFrame(s.handle, f, sc.frame_dt)
        st = s.stats()
        print(json.dumps({"frame": f, "result": int(r), "substeps": int(st.substeps),
                          "newton_iterations": int(st.newton_iterations),
                          "active_contacts": int(st.active_contact_count),
                          "device_ms": float(s.gpu_stats().last_frame_milliseconds)}), flush=True)
        if r != kn.OK:
            print(s.last_error(), file=sys.stderr)
            status = 1
            break
    s.close()
    sys.exit(status)


if __name__ == "__main__":
    main()
