"""The device BVH layout that the stackless walks rely on (right-first
preorder, escape index = end of the subtree, so it always advances) on the
colliders of the test and bench scenes (tests/native/test_bvh_layout.cpp)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import scenes

REPO = Path(__file__).resolve().parents[1]


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_escape_indices_advance(tmp_path):
    exe = tmp_path / "bvh_layout"
    csrc = REPO / "kami-hair-solver_gb300" / "csrc"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{csrc}", f"-I{REPO / 'include'}",
                    str(REPO / "tests" / "native" / "test_bvh_layout.cpp"), str(csrc / "khs_model.cpp"), "-o",
                    str(exe)], check=True)
    colliders = []
    for sc in (scenes.sphere_scene(), scenes.ellipsoid_scene(strands=10, frames=1), scenes.pole_scene(frames=1),
               scenes.body_scene(frames=1)):
        colliders.append((sc.name, np.asarray(sc.vertices), np.asarray(sc.triangles)))
    v, f = scenes.icosphere(0)
    colliders.append(("single icosahedron", v, f[:1]))  # one triangle: a lone leaf
    for name, verts, tris in colliders:
        vp, tp = tmp_path / "v.bin", tmp_path / "t.bin"
        np.ascontiguousarray(verts, dtype=np.float64).tofile(vp)
        np.ascontiguousarray(tris, dtype=np.uint32).tofile(tp)
        out = subprocess.run([str(exe), str(vp), str(tp)], capture_output=True, text=True)
        print(name, out.stdout.strip())
        assert out.returncode == 0 and "PASS" in out.stdout, (name, out.stdout + out.stderr)
