"""The product's BVH-walked ray-parity inside test (khs_model.cpp, used by
khsBuild's initial-feasibility check) against the reference's all-triangle
loop (src/solver.cpp:608-632, restated by the oracle) on closed meshes, with
points placed where the parity test is most sensitive to rounding: on rays
through mesh vertices and edge midpoints, on the symmetry planes of a UV
sphere, and within 1e-9 m of vertices (tests/native/test_inside_parity.cpp).
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import scenes

REPO = Path(__file__).resolve().parents[1]
RAY = np.array([1.0, 0.0000012345, 0.0000023456])


def _points(verts, tris, rng, count):
    lo, hi = verts.min(0), verts.max(0)
    mid, half = 0.5 * (lo + hi), 0.65 * (hi - lo)
    out = [mid + half * rng.uniform(-1.0, 1.0, size=(count, 3))]
    # Near vertices, both sides of the surface.
    pick = verts[rng.integers(0, len(verts), count // 4)]
    out.append(pick + rng.normal(size=pick.shape) * 1e-9)
    # On the ray through a vertex or an edge midpoint, behind it.
    pick = verts[rng.integers(0, len(verts), count // 4)]
    out.append(pick - rng.uniform(0.01, 0.5, size=(len(pick), 1)) * (hi - lo).max() * RAY)
    e = tris[rng.integers(0, len(tris), count // 4)]
    edge_mid = 0.5 * (verts[e[:, 0]] + verts[e[:, 1]])
    out.append(edge_mid - rng.uniform(0.01, 0.5, size=(len(edge_mid), 1)) * (hi - lo).max() * RAY)
    # Exactly on the planes y = 0 and z = a vertex height.
    p = mid + half * rng.uniform(-1.0, 1.0, size=(count // 4, 3))
    p[:, 1] = 0.0
    p[:, 2] = verts[rng.integers(0, len(verts), len(p)), 2]
    out.append(p)
    return np.concatenate(out)


def _meshes():
    v, f = scenes.icosphere(4)
    yield "icosphere L4 ellipsoid", v * np.array([0.09, 0.11, 0.12]) + np.array([0.01, -0.02, 0.03]), f
    v, f = scenes.uv_ellipsoid((0.0, 0.0, 0.0), (0.08, 0.10, 0.115), 72, 40)
    yield "UV ellipsoid", v, f
    v, f = scenes.icosphere(1)
    yield "coarse icosphere, 0.5 m", v * 0.5, f


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_bvh_inside_test_matches_all_triangle_loop(tmp_path):
    exe = tmp_path / "inside_parity"
    csrc = REPO / "kami-hair-solver_gb300" / "csrc"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{csrc}", f"-I{REPO / 'oracle'}",
                    f"-I{REPO / 'include'}", str(REPO / "tests" / "native" / "test_inside_parity.cpp"),
                    str(csrc / "khs_model.cpp"), "-o", str(exe)], check=True)
    rng = np.random.default_rng(11)
    for name, verts, tris in _meshes():
        verts = np.ascontiguousarray(verts, dtype=np.float64)
        tris = np.ascontiguousarray(tris, dtype=np.uint32)
        pts = np.ascontiguousarray(_points(verts, tris, rng, 8000), dtype=np.float64)
        files = [tmp_path / f"{k}.bin" for k in ("v", "t", "p")]
        verts.tofile(files[0])
        tris.tofile(files[1])
        pts.tofile(files[2])
        out = subprocess.run([str(exe), *map(str, files)], capture_output=True, text=True)
        print(name, out.stdout)
        assert out.returncode == 0 and "PASS" in out.stdout, name + ": " + out.stdout + out.stderr
        inside = int(out.stdout.split("(")[1].split()[0])
        assert 0 < inside < len(pts), (name, inside)


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_bvh_inside_test_on_a_large_request(tmp_path):
    """The hair points of the largest serving request (20,000 strands,
    1.77M points) against its 20,480-triangle closed ellipsoid: the BVH walk
    over all points, checked against the all-triangle loop on every 500th
    point, whose time is scaled to all points (printed)."""
    exe = tmp_path / "inside_parity"
    csrc = REPO / "kami-hair-solver_gb300" / "csrc"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{csrc}", f"-I{REPO / 'oracle'}",
                    f"-I{REPO / 'include'}", str(REPO / "tests" / "native" / "test_inside_parity.cpp"),
                    str(csrc / "khs_model.cpp"), "-o", str(exe)], check=True)
    sc = scenes.ellipsoid_scene(seed=7, strands=20000, node_range=(16, 160), frames=1, level=5,
                                axes=(0.095, 0.11, 0.12))
    files = [tmp_path / f"{k}.bin" for k in ("v", "t", "p")]
    np.ascontiguousarray(sc.vertices, dtype=np.float64).tofile(files[0])
    np.ascontiguousarray(sc.triangles, dtype=np.uint32).tofile(files[1])
    np.ascontiguousarray(sc.points, dtype=np.float64).tofile(files[2])
    out = subprocess.run([str(exe), *map(str, files), "500"], capture_output=True, text=True)
    print(out.stdout)
    assert out.returncode == 0 and "PASS" in out.stdout, out.stdout + out.stderr
