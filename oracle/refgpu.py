"""ORACLE — test infrastructure only: the reference's own FP64 CUDA backend,
driven from the tests and from the bench's baseline legs.

``oracle/_ref/libkhs_ref.so`` is the reference's ``src/cuda_backend.cu``
compiled unchanged for sm_103a plus ``oracle/ref_bridge.cpp`` (a flat C API
over ``kami::CudaBackend``).  The rod model it is initialised with comes from
the CPU oracle's builder (``khsOracleExportModel``), handed over as the
reference's ``Solver::build`` hands its own (solver.cpp:485-519); root targets
come from the oracle's ``khsxComputeRootTargets`` (solver.cpp:416-447).

``available()`` says whether the library exists or can be built here: the
reference sources must have been staged into ``oracle/_ref/src``
(``make -C oracle stage-ref REFERENCE=<checkout>``) and a CUDA device must be
present to run it.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

import khs_native as kn

REPO = Path(__file__).resolve().parents[1]
REF_DIR = REPO / "oracle" / "_ref"
REF_SO = REF_DIR / "libkhs_ref.so"
STAGED = REF_DIR / "src" / "cuda_backend.cu"

_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_INT = ctypes.c_int


def staged() -> bool:
    return STAGED.exists()


def build() -> Path:
    """Builds oracle/_ref/libkhs_ref.so from the staged sources."""
    if not staged():
        raise FileNotFoundError("the reference CUDA sources are not staged in oracle/_ref/src")
    subprocess.run(["make", "-s", "-C", str(REPO / "oracle"), "ref"], check=True)
    return REF_SO


def available() -> bool:
    return staged() or REF_SO.exists()


class RefLibrary:
    def __init__(self, path: Path | None = None):
        self.path = Path(path) if path else build()
        lib = ctypes.CDLL(str(self.path))
        lib.khsRefCreate.restype = _P
        lib.khsRefCreate.argtypes = [_P] * 11 + [ctypes.POINTER(_INT), ctypes.c_char_p, _U32]
        lib.khsRefDestroy.argtypes = [_P]
        lib.khsRefLastError.restype = ctypes.c_char_p
        lib.khsRefLastError.argtypes = [_P]
        for name, args in {
            "khsRefAllocateAnimation": [_P, _U32],
            "khsRefSetRootAnimationFrame": [_P, _U32, _P, _P, _U32],
            "khsRefSetColliderAnimationFrame": [_P, _U32, _P, _U32],
            "khsRefFinalizeAnimation": [_P],
            "khsRefStepAnimationFrame": [_P, _U32, ctypes.c_double],
            "khsRefUpdateRoots": [_P, _P, _P, _U32],
            "khsRefUpdateCollider": [_P, _P, _U32],
            "khsRefStep": [_P, ctypes.c_double],
            "khsRefSaveCheckpoint": [_P, _P, ctypes.c_uint64],
            "khsRefRestoreCheckpoint": [_P, _P, ctypes.c_uint64],
            "khsRefCopyOriginalPositions": [_P, _P, _U32],
            "khsRefStats": [_P, _P],
            "khsRefGpuStats": [_P, _P],
            "khsRefFailure": [_P, _P],
            "khsRefProgress": [_P, _P],
            "khsRefCancel": [_P],
        }.items():
            fn = getattr(lib, name)
            fn.restype = _INT
            fn.argtypes = args
        lib.khsRefCheckpointSize.restype = ctypes.c_uint64
        lib.khsRefCheckpointSize.argtypes = [_P]
        self.lib = lib


def _ptr(a):
    return a.ctypes.data_as(_P) if a is not None and a.size else None


def export_model(oracle_solver: kn.HairSolver) -> dict:
    """The oracle's built model in the backend's layout."""
    lib = oracle_solver._library
    lib.khsOracleModelSizes.argtypes = [_P, _P]
    lib.khsOracleModelSizes.restype = None
    lib.khsOracleExportModel.argtypes = [_P] * 9
    lib.khsOracleExportModel.restype = None
    sizes = np.zeros(6, dtype=np.uint32)
    lib.khsOracleModelSizes(oracle_solver.handle, _ptr(sizes))
    n, e, s, p, v, t = (int(x) for x in sizes)
    m = dict(sizes=sizes,
             node_f=np.zeros((n, 18)), node_u=np.zeros((n, 4), dtype=np.uint32),
             elem_f=np.zeros((e, 7)), elem_u=np.zeros((e, 4), dtype=np.uint32),
             strand_u=np.zeros((s, 2), dtype=np.uint32), mapping=np.zeros(p, dtype=np.uint32),
             collider=np.zeros((max(v, 1), 3)), tris=np.zeros((max(t, 1), 3), dtype=np.uint32))
    lib.khsOracleExportModel(oracle_solver.handle, *(_ptr(m[k]) for k in
                             ("node_f", "node_u", "elem_f", "elem_u", "strand_u", "mapping", "collider", "tris")))
    return m


class RefSolver:
    """One scene on the reference backend, animation frames uploaded."""

    def __init__(self, ref: RefLibrary, oracle_lib: kn.Library, scene, frames: int | None = None):
        import scenes

        self.ref = ref
        self.scene = scene
        self.frames = scene.frames if frames is None else frames
        builder = kn.HairSolver(oracle_lib)
        scenes.load_into(builder, scene, animation=False)
        m = export_model(builder)
        self.nodes = int(m["sizes"][0])
        self.mapping = m["mapping"].copy()
        result = _INT(0)
        err = ctypes.create_string_buffer(512)
        self.handle = ref.lib.khsRefCreate(ctypes.byref(builder.desc), ctypes.byref(builder.material), _ptr(m["sizes"]),
                                           *(_ptr(m[k]) for k in ("node_f", "node_u", "elem_f", "elem_u", "strand_u",
                                                                  "mapping", "collider", "tris")),
                                           ctypes.byref(result), err, 512)
        if not self.handle:
            builder.close()
            raise RuntimeError(f"reference backend: {result.value} {err.value.decode()}")
        self._check(ref.lib.khsRefAllocateAnimation(self.handle, self.frames))
        for f in range(self.frames):
            pos, rot = builder.compute_root_targets(scene.root_points_at(f))
            self._check(ref.lib.khsRefSetRootAnimationFrame(self.handle, f, _ptr(pos), _ptr(rot), self.nodes))
            if scene.collider_at is not None:
                verts = np.ascontiguousarray(scene.collider_at(f), dtype=np.float64)
                self._check(ref.lib.khsRefSetColliderAnimationFrame(self.handle, f, _ptr(verts), len(verts)))
        self._check(ref.lib.khsRefFinalizeAnimation(self.handle))
        builder.close()

    def _check(self, r: int):
        if r != kn.OK:
            raise RuntimeError(f"reference backend error {r}: {self.last_error()}")

    def last_error(self) -> str:
        return self.ref.lib.khsRefLastError(self.handle).decode("utf-8", errors="replace")

    def step_animation_frame(self, frame: int, dt: float) -> int:
        return int(self.ref.lib.khsRefStepAnimationFrame(self.handle, frame, dt))

    def stats(self) -> kn.StepStats:
        st = kn.StepStats()
        st.struct_size = ctypes.sizeof(st)
        self._check(self.ref.lib.khsRefStats(self.handle, ctypes.byref(st)))
        return st

    def gpu_stats(self) -> kn.GpuStats:
        g = kn.GpuStats()
        g.struct_size = ctypes.sizeof(g)
        self._check(self.ref.lib.khsRefGpuStats(self.handle, ctypes.byref(g)))
        return g

    def failure(self) -> kn.FailureDiagnostics:
        d = kn.FailureDiagnostics()
        d.struct_size = ctypes.sizeof(d)
        self._check(self.ref.lib.khsRefFailure(self.handle, ctypes.byref(d)))
        return d

    def save_checkpoint(self) -> bytes:
        size = int(self.ref.lib.khsRefCheckpointSize(self.handle))
        buf = (ctypes.c_ubyte * size)()
        self._check(self.ref.lib.khsRefSaveCheckpoint(self.handle, buf, size))
        return bytes(buf)

    def restore_checkpoint(self, blob: bytes):
        buf = (ctypes.c_ubyte * len(blob)).from_buffer_copy(blob)
        self._check(self.ref.lib.khsRefRestoreCheckpoint(self.handle, buf, len(blob)))

    def state(self) -> tuple[np.ndarray, np.ndarray]:
        blob = self.save_checkpoint()
        body = np.frombuffer(blob[24:], dtype=np.float64)
        dof = body.size // 2
        return body[:dof].reshape(-1, 6).copy(), body[dof:].reshape(-1, 6).copy()

    def progress(self) -> kn.Progress:
        p = kn.Progress()
        p.struct_size = ctypes.sizeof(p)
        self._check(self.ref.lib.khsRefProgress(self.handle, ctypes.byref(p)))
        return p

    def cancel(self):
        self._check(self.ref.lib.khsRefCancel(self.handle))

    def close(self):
        if self.handle:
            self.ref.lib.khsRefDestroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run(ref: RefLibrary, oracle_lib, scene, frames: int | None = None, checkpoint: bytes | None = None,
        first: int = 1):
    """Steps ``scene`` on the reference backend; per frame the result code,
    step stats and state (q, v), like tests/parity.py's ``run``."""
    s = RefSolver(ref, oracle_lib, scene, frames)
    if checkpoint is not None:
        s.restore_checkpoint(checkpoint)
    out = []
    for f in range(first, s.frames):
        r = s.step_animation_frame(f, scene.frame_dt)
        st = s.stats()
        q, v = s.state()
        out.append(dict(result=r, stats=st, q=q, v=v, error=s.last_error() if r else ""))
        if r != kn.OK:
            break
    s.close()
    return out
