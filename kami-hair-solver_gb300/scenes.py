"""Seeded synthetic scenes for the solver's workloads.

The reference's only benchmark scene is a private Blender file, so these
generators stand in for it with the shapes, sizes and value distributions of
each workload:

* ``sphere_scene``     -- 64 straight strands x 32 nodes on a 0.1 m sphere
                          (icosphere L3, 1,280 triangles); optionally moving.
* ``ellipsoid_scene``  -- strands with uniform node counts, 2 mm +-10 %
                          segments and helical curl on the upper hemisphere
                          of a rotating ellipsoid (icosphere L5, 20,480
                          triangles).
* ``body_scene``       -- 6,757 strands / 265,108 internal nodes with
                          lognormal(3.6, 0.5) counts on a head ellipsoid
                          above a torso capsule (225,184 vertices) swaying
                          3 cm at 0.5 Hz.
* ``serving_request``  -- one request of the request stream: log-uniform
                          strand count, uniform node counts, ellipsoid of
                          5k-50k triangles.

A ``Scene`` carries the curves, the collider, per-frame root points and
collider vertices, and the solver settings; ``load_into`` uploads it through
the C ABI binding.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Callable

import numpy as np


@dataclasses.dataclass
class Scene:
    name: str
    points: np.ndarray            # (P, 3) float64
    offsets: np.ndarray           # (S + 1,) uint32
    vertices: np.ndarray | None   # (V, 3) float64
    triangles: np.ndarray | None  # (T, 3) uint32
    frames: int
    fps: float
    desc: dict
    material: dict
    root_points_at: Callable[[int], np.ndarray]
    collider_at: Callable[[int], np.ndarray] | None
    seed: int = 0

    @property
    def frame_dt(self) -> float:
        return 1.0 / self.fps

    @property
    def strands(self) -> int:
        return len(self.offsets) - 1


# ---------------------------------------------------------------------------
# meshes

def icosphere(level: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere subdivided ``level`` times (10*4^L + 2 vertices)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in verts]
    f = list(faces)
    for _ in range(level):
        cache: dict[tuple[int, int], int] = {}

        def mid(a: int, b: int) -> int:
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = v[a] + v[b]
                v.append(m / np.linalg.norm(m))
                cache[key] = len(v) - 1
            return cache[key]

        nf = []
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    return np.array(v), np.array(f, dtype=np.uint32)


def uv_ellipsoid(center, axes, segments: int, rings: int) -> tuple[np.ndarray, np.ndarray]:
    """Closed, outward-oriented UV ellipsoid: segments*rings + 2 vertices."""
    theta = np.pi * (np.arange(1, rings + 1) / (rings + 1))
    phi = 2.0 * np.pi * np.arange(segments) / segments
    st, ct = np.sin(theta)[:, None], np.cos(theta)[:, None]
    ring = np.stack([st * np.cos(phi)[None, :], st * np.sin(phi)[None, :], np.broadcast_to(ct, (rings, segments))], -1)
    body = ring.reshape(-1, 3)
    v = np.concatenate([[[0.0, 0.0, 1.0]], body, [[0.0, 0.0, -1.0]]]) * np.asarray(axes) + np.asarray(center)
    return v, _uv_faces(segments, rings, closed_bottom=True)


def _uv_faces(segments: int, rings: int, closed_bottom: bool) -> np.ndarray:
    faces = []
    s = segments
    idx = lambda r, k: 1 + r * s + (k % s)
    for k in range(s):
        faces.append((0, idx(0, k), idx(0, k + 1)))
    for r in range(rings - 1):
        for k in range(s):
            a, b, c, d = idx(r, k), idx(r + 1, k), idx(r + 1, k + 1), idx(r, k + 1)
            faces.append((a, b, c))
            faces.append((a, c, d))
    if closed_bottom:
        bottom = 1 + rings * s
        for k in range(s):
            faces.append((bottom, idx(rings - 1, k + 1), idx(rings - 1, k)))
    return np.array(faces, dtype=np.uint32)


def capsule(z_bottom: float, z_top: float, radius: float, segments: int, rings: int,
            open_bottom: bool = False) -> tuple[np.ndarray, np.ndarray]:
    """Vertical capsule around the z axis (cylinder from z_bottom to z_top
    with hemispherical caps), rings spread evenly along the profile arc;
    segments*rings + 2 vertices (the bottom pole is kept but left unconnected
    when ``open_bottom``, which leaves a boundary ring)."""
    cyl = z_top - z_bottom
    arc = np.pi * radius + cyl
    s = arc * (np.arange(1, rings + 1) / (rings + 1))
    rr, zz = np.empty(rings), np.empty(rings)
    cap = 0.5 * np.pi * radius
    for k, sk in enumerate(s):
        if sk < cap:
            a = sk / radius
            rr[k], zz[k] = radius * math.sin(a), z_top + radius * math.cos(a)
        elif sk < cap + cyl:
            rr[k], zz[k] = radius, z_top - (sk - cap)
        else:
            a = (sk - cap - cyl) / radius
            rr[k], zz[k] = radius * math.cos(a), z_bottom - radius * math.sin(a)
    phi = 2.0 * np.pi * np.arange(segments) / segments
    body = np.stack([rr[:, None] * np.cos(phi)[None, :], rr[:, None] * np.sin(phi)[None, :],
                     np.broadcast_to(zz[:, None], (rings, segments))], -1).reshape(-1, 3)
    v = np.concatenate([[[0.0, 0.0, z_top + radius]], body, [[0.0, 0.0, z_bottom - radius]]])
    return v, _uv_faces(segments, rings, closed_bottom=not open_bottom)


def _rotation_z(angle: float) -> np.ndarray:
    c, s = math.cos(angle), math.sin(angle)
    return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])


# ---------------------------------------------------------------------------
# strands

def _orthonormal(n: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    a = np.where(np.abs(n[:, :1]) < 0.9, np.array([[1.0, 0.0, 0.0]]), np.array([[0.0, 1.0, 0.0]]))
    u = np.cross(n, a)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    w = np.cross(n, u)
    return u, w


def _jitter(n: np.ndarray, sigma: float, rng: np.random.Generator) -> np.ndarray:
    u, w = _orthonormal(n)
    a, b = rng.normal(0.0, sigma, size=(2, len(n)))
    d = n + u * a[:, None] + w * b[:, None]
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def _helix_strand(root, direction, count, seg, radius, pitch, phase, rng, seg_jitter=0.0):
    """Points of a helical curl around ``direction`` starting at ``root``,
    consecutive chords of length ``seg`` (+- seg_jitter relative)."""
    u, w = _orthonormal(direction[None, :])
    u, w = u[0], w[0]
    turn_len = math.hypot(2 * math.pi * radius, pitch)
    # Place points by arc length on the curve, then rescale every chord to
    # its requested length along its own direction.
    lengths = np.array([seg * (1.0 + (rng.uniform(-seg_jitter, seg_jitter) if seg_jitter else 0.0)) for _ in range(count - 1)])
    s = np.concatenate([[0.0], np.cumsum(lengths)])
    ang = 2 * math.pi * s / turn_len + phase
    axial = pitch * s / turn_len
    curve = (np.asarray(root)[None, :] + axial[:, None] * direction[None, :] +
             radius * ((np.cos(ang) - math.cos(phase))[:, None] * u[None, :] + (np.sin(ang) - math.sin(phase))[:, None] * w[None, :]))
    chords = np.diff(curve, axis=0)
    chords *= (lengths / np.linalg.norm(chords, axis=1))[:, None]
    return np.concatenate([curve[:1], curve[:1] + np.cumsum(chords, axis=0)])


def _assemble(strands: list[np.ndarray]) -> tuple[np.ndarray, np.ndarray]:
    offsets = np.zeros(len(strands) + 1, dtype=np.uint32)
    offsets[1:] = np.cumsum([len(s) for s in strands])
    return np.concatenate(strands).astype(np.float64), offsets


# ---------------------------------------------------------------------------
# workloads

HAIR_MATERIAL_SMALL = dict(density=1300.0, radius=4.0e-5, young_modulus=3.0e9, poisson_ratio=0.25,
                           barrier_distance=1.0e-3, friction=0.3)


def sphere_scene(seed: int = 1, strands: int = 64, nodes: int = 32, length: float = 0.2, frames: int = 1,
                 substeps: int = 4, motion: bool = False, angular_velocity: float = 2.0,
                 drift=(0.01, 0.0, 0.0)) -> Scene:
    """Straight strands on the outward normals of a 0.1 m sphere (icosphere
    L3) with N(0, 0.05 rad) direction jitter.  ``motion`` rotates the sphere
    (and the roots riding it) about z and drifts it, which drives the
    Gauss-Newton solve; the static form converges at iteration 0."""
    rng = np.random.default_rng(seed)
    R = 0.1
    v, f = icosphere(3)
    v = v * R
    # Roots: Fibonacci lattice over the sphere, seeded rotation.
    k = np.arange(strands) + 0.5
    zc = 1.0 - 2.0 * k / strands
    ph = np.pi * (1.0 + 5.0 ** 0.5) * k + rng.uniform(0, 2 * np.pi)
    normals = np.stack([np.sqrt(1 - zc ** 2) * np.cos(ph), np.sqrt(1 - zc ** 2) * np.sin(ph), zc], 1)
    dirs = _jitter(normals, 0.05, rng)
    roots = normals * (R + 1.0e-4)
    seg = length / (nodes - 1)
    strand_list = [roots[s][None, :] + np.arange(nodes)[:, None] * seg * dirs[s][None, :] for s in range(strands)]
    points, offsets = _assemble(strand_list)
    fps = 24.0

    def transform(frame: int):
        if not motion:
            return np.eye(3), np.zeros(3)
        t = frame / fps
        return _rotation_z(angular_velocity * t), np.asarray(drift) * t

    def roots_at(frame: int) -> np.ndarray:
        Rm, tr = transform(frame)
        return points @ Rm.T + tr

    def collider_at(frame: int) -> np.ndarray:
        Rm, tr = transform(frame)
        return v @ Rm.T + tr

    desc = dict(substeps=substeps, maximum_substeps=max(32, substeps), fixed_root_nodes=2)
    return Scene("sphere", points, offsets, v, f, frames + 1, fps, desc, dict(HAIR_MATERIAL_SMALL), roots_at,
                 collider_at, seed)


def pole_scene(seed: int = 4, strands: int = 48, nodes: int = 32, seg: float = 1.0e-3, frames: int = 2,
               substeps: int = 4, segments: int = 360, rings: int = 120) -> Scene:
    """Strands lying across the pole of a UV sphere (0.1 m, ``segments``
    x ``rings``), where ``segments`` sliver triangles meet in one vertex: a
    dense patch of the collider, so that elements near the pole reach
    hundreds of leaves.  Roots on a ring 2-6 mm from the pole, strands tilted
    70 degrees from the normal towards the pole axis, 1 mm segments.  The
    sphere turns about z (through the pole) and drifts."""
    rng = np.random.default_rng(seed)
    R = 0.1
    v, f = uv_ellipsoid((0.0, 0.0, 0.0), (R, R, R), segments, rings)
    strand_list = []
    for k in range(strands):
        rho = rng.uniform(0.002, 0.006)
        ph = 2 * np.pi * k / strands + rng.uniform(0, 0.1)
        n = np.array([rho * np.cos(ph), rho * np.sin(ph), math.sqrt(R * R - rho * rho)]) / R
        inward = -np.array([np.cos(ph), np.sin(ph), 0.0])
        inward -= n * np.dot(inward, n)
        inward /= np.linalg.norm(inward)
        tilt = math.radians(70.0 + rng.uniform(-5.0, 5.0))
        d = math.cos(tilt) * n + math.sin(tilt) * inward
        root = n * (R + 1.0e-4)
        strand_list.append(root[None, :] + np.arange(nodes)[:, None] * seg * d[None, :])
    points, offsets = _assemble(strand_list)
    fps = 24.0

    def transform(frame: int):
        t = frame / fps
        return _rotation_z(1.5 * t), np.array([0.004, -0.002, 0.0]) * t

    def roots_at(frame: int) -> np.ndarray:
        Rm, tr = transform(frame)
        return points @ Rm.T + tr

    def collider_at(frame: int) -> np.ndarray:
        Rm, tr = transform(frame)
        return v @ Rm.T + tr

    desc = dict(substeps=substeps, maximum_substeps=max(32, substeps), fixed_root_nodes=2)
    return Scene("pole", points, offsets, v, f, frames + 1, fps, desc, dict(HAIR_MATERIAL_SMALL), roots_at,
                 collider_at, seed)


def ellipsoid_scene(seed: int = 2, strands: int = 1000, node_range=(20, 120), frames: int = 10, substeps: int = 8,
                    level: int = 5, angular_velocity: float = 2.0, axes=(0.09, 0.11, 0.12)) -> Scene:
    """Helical strands (curl radius U[2,10] mm, pitch U[5,20] mm, 2 mm +-10 %
    segments) rooted on the upper hemisphere of an ellipsoid rotating about
    z; roots ride the rotation."""
    rng = np.random.default_rng(seed)
    axes = np.asarray(axes)
    v, f = icosphere(level)
    v = v * axes
    # Upper-hemisphere roots: sample directions, map to the ellipsoid.
    d = rng.normal(size=(strands * 3, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d[d[:, 2] > 0.15][:strands]
    surf = d * axes
    normal = surf / axes ** 2
    normal /= np.linalg.norm(normal, axis=1, keepdims=True)
    roots = surf + normal * 2.0e-4
    counts = rng.integers(node_range[0], node_range[1] + 1, size=strands)
    dirs = _jitter(normal, 0.05, rng)
    strand_list = []
    for s in range(strands):
        strand_list.append(_helix_strand(roots[s], dirs[s], int(counts[s]), 0.002, rng.uniform(0.002, 0.010),
                                         rng.uniform(0.005, 0.020), rng.uniform(0, 2 * np.pi), rng, seg_jitter=0.1))
    points, offsets = _assemble(strand_list)
    fps = 24.0

    def roots_at(frame: int) -> np.ndarray:
        return points @ _rotation_z(angular_velocity * frame / fps).T

    def collider_at(frame: int) -> np.ndarray:
        return v @ _rotation_z(angular_velocity * frame / fps).T

    desc = dict(substeps=substeps, maximum_substeps=max(32, substeps), fixed_root_nodes=2)
    return Scene("ellipsoid", points, offsets, v, f, frames + 1, fps, desc, dict(HAIR_MATERIAL_SMALL), roots_at,
                 collider_at, seed)


BODY_STRANDS = 6757
BODY_NODES = 265108
BODY_VERTICES = 225184


def body_scene(seed: int = 3, frames: int = 30, substeps: int = 8, maximum_substeps: int = 64,
               strands: int = BODY_STRANDS, total_nodes: int = BODY_NODES) -> Scene:
    """Full-scene stand-in: head ellipsoid (UV 360x300) above an open-bottom
    torso capsule (UV 420x279), 225,184 vertices in all, swaying with
    amplitude 3 cm at 0.5 Hz (seeded phases; the torso sway fades towards
    its bottom).  Strands: lognormal(3.6, 0.5) point counts clamped to
    [8, 200] and adjusted so the internal node count (including the
    invisible extension of strands shorter than 20 mm) is ``total_nodes``;
    2 mm segments with a gentle seeded curl, rooted on the upper part of the
    head along the jittered outward normal."""
    rng = np.random.default_rng(seed)
    head_axes = np.array([0.08, 0.10, 0.115])
    hv, hf = uv_ellipsoid((0.0, 0.0, 0.0), head_axes, 360, 300)
    tv, tf = capsule(-0.85, -0.45, 0.16, 420, 279, open_bottom=True)
    vertices = np.concatenate([hv, tv])
    triangles = np.concatenate([hf, tf + len(hv)]).astype(np.uint32)
    assert len(vertices) == BODY_VERTICES or (len(vertices) > 0)
    # Point counts per strand, then an exact fix-up of the internal total.
    counts = np.clip(np.round(np.exp(rng.normal(3.6, 0.5, size=strands))), 8, 200).astype(np.int64)
    seg = 0.002
    min_len = 0.02

    def internal(c):  # points + one invisible node when shorter than 20 mm
        return c + ((c - 1) * seg < min_len - 1e-9).astype(np.int64)

    scale = total_nodes / internal(counts).sum()
    counts = np.clip(np.round(counts * scale), 8, 200).astype(np.int64)
    diff = total_nodes - int(internal(counts).sum())
    order = rng.permutation(strands)
    k = 0
    while diff != 0:
        s = order[k % strands]
        if diff > 0 and counts[s] < 200 and counts[s] >= 11:
            counts[s] += 1
        elif diff < 0 and counts[s] > 11:
            counts[s] -= 1
        diff = total_nodes - int(internal(counts).sum())
        k += 1
    # Roots on the upper head.
    d = rng.normal(size=(strands * 3, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d[d[:, 2] > 0.1][:strands]
    surf = d * head_axes
    normal = surf / head_axes ** 2
    normal /= np.linalg.norm(normal, axis=1, keepdims=True)
    roots = surf + normal * 2.0e-4
    dirs = _jitter(normal, 0.05, rng)
    strand_list = [_helix_strand(roots[s], dirs[s], int(counts[s]), seg, rng.uniform(0.01, 0.03),
                                 rng.uniform(0.08, 0.2), rng.uniform(0, 2 * np.pi), rng) for s in range(strands)]
    points, offsets = _assemble(strand_list)
    fps = 24.0
    amp, freq = 0.03, 0.5
    phase = rng.uniform(0, 2 * np.pi, size=2)
    z = vertices[:, 2]
    weight = np.where(z > -0.3, 1.0, np.clip((z + 1.01) / 0.71, 0.0, 1.0))

    def sway(frame: int) -> np.ndarray:
        t = frame / fps
        return amp * np.array([math.sin(2 * math.pi * freq * t + phase[0]) - math.sin(phase[0]),
                               0.5 * (math.sin(2 * math.pi * freq * t + phase[1]) - math.sin(phase[1])), 0.0])

    def roots_at(frame: int) -> np.ndarray:
        return points + sway(frame)[None, :]

    def collider_at(frame: int) -> np.ndarray:
        return vertices + weight[:, None] * sway(frame)[None, :]

    desc = dict(substeps=substeps, maximum_substeps=maximum_substeps, fixed_root_nodes=2, minimum_dynamic_length=min_len)
    return Scene("body", points, offsets, vertices, triangles, frames + 1, fps, desc, {}, roots_at, collider_at, seed)


def serving_request(seed: int, strand_range=(100, 20000), node_range=(16, 160), tri_range=(5000, 50000),
                    frames: int = 10, substeps: int = 8) -> Scene:
    """One request of the serving stream: log-uniform strand count, uniform
    node counts, an ellipsoid collider of 5k-50k triangles (icosphere level
    chosen by the target count), 10 frames x 8 substeps."""
    rng = np.random.default_rng(seed)
    strands = int(round(math.exp(rng.uniform(math.log(strand_range[0]), math.log(strand_range[1])))))
    target_tris = rng.uniform(*tri_range)
    level = 4 if target_tris < 12000 else 5  # 5,120 / 20,480 triangles
    axes = (0.09 + 0.01 * rng.uniform(), 0.11, 0.12)
    sc = ellipsoid_scene(seed=seed, strands=strands, node_range=node_range, frames=frames, substeps=substeps,
                         level=level, axes=axes)
    sc.name = "request"
    return sc


# ---------------------------------------------------------------------------

def apply_settings(solver, scene: Scene) -> None:
    for k, val in scene.desc.items():
        setattr(solver.desc, k, val)
    for k, val in scene.material.items():
        setattr(solver.material, k, val)


def load_into(solver, scene: Scene, animation: bool = True, frames: int | None = None) -> None:
    """Creates, configures and builds ``solver`` (a khs_native.HairSolver)
    for ``scene``; with ``animation`` every frame is uploaded to the device
    and finalized (the khsStepAnimationFrame path)."""
    apply_settings(solver, scene)
    solver.create()
    solver.set_hair(scene.points, scene.offsets)
    if scene.triangles is not None:
        solver.set_collider(scene.vertices, scene.triangles)
    solver.build()
    if animation:
        n = scene.frames if frames is None else frames
        solver.allocate_animation(n)
        for f in range(n):
            solver.set_root_animation_frame(f, scene.root_points_at(f))
            solver.set_collider_animation_frame(f, scene.collider_at(f) if scene.collider_at else None)
        solver.finalize_animation()
