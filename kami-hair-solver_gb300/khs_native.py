"""ctypes binding for the kami-hair-solver C ABI (ABI version 5).

Mirrors the reference binding ``HairSolver``
(blender_extension/kami_hair_solver/native.py:180-413): same method names,
argument meaning and error behaviour (``RuntimeError`` carrying
``khsGetLastError``).  Differences: positions come back as ``numpy`` arrays of
shape (n, 3) instead of lists of tuples, the library path defaults to the
in-tree GB300 build, and ``Library`` exposes raw result codes for tests.

The same binding loads any library that exports this ABI, which is how the
tests drive the GB300 product and the CPU oracle with identical calls.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

ABI_VERSION = 5
OK = 0
ERROR_INVALID_ARGUMENT = 1
ERROR_INVALID_STATE = 2
ERROR_INVALID_HAIR = 3
ERROR_INVALID_COLLIDER = 4
ERROR_INITIAL_INTERSECTION = 5
ERROR_NOT_CONVERGED = 6
ERROR_NUMERICAL_FAILURE = 7
ERROR_OUT_OF_MEMORY = 8
ERROR_INTERNAL = 9

PHASE_IDLE, PHASE_PREPARING, PHASE_ASSEMBLING, PHASE_LINEAR_SOLVE = 0, 1, 2, 3
PHASE_CCD, PHASE_LINE_SEARCH, PHASE_FINISHED, PHASE_FAILED = 4, 5, 6, 7

FAILURE_NONE, FAILURE_SWEEP, FAILURE_BARRIER_INFEASIBLE, FAILURE_NONLINEAR_SOLVE = 0, 1, 2, 3

MODE_PLAIN_FP64 = 0
MODE_MIXED = 1
MODE_MIXED_FF = 2

PACKAGE_DIR = Path(__file__).resolve().parent
DEFAULT_LIBRARY = PACKAGE_DIR / "_build" / "libkami_hair_solver.so"

c_u32, c_i32, c_u64, c_f64 = ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_double


class Vec3(ctypes.Structure):
    _fields_ = [("x", c_f64), ("y", c_f64), ("z", c_f64)]


class Triangle(ctypes.Structure):
    _fields_ = [("i0", c_u32), ("i1", c_u32), ("i2", c_u32)]


class SolverDesc(ctypes.Structure):
    _fields_ = [
        ("struct_size", c_u32), ("gravity", Vec3), ("substeps", c_u32), ("maximum_substeps", c_u32),
        ("newton_iterations", c_u32), ("line_search_iterations", c_u32), ("absolute_tolerance", c_f64),
        ("relative_tolerance", c_f64), ("increment_tolerance", c_f64), ("minimum_line_search_step", c_f64),
        ("minimum_gap", c_f64), ("maximum_element_length", c_f64), ("minimum_dynamic_length", c_f64),
        ("fixed_root_nodes", c_u32), ("thread_count", c_u32),
    ]


class HairMaterial(ctypes.Structure):
    _fields_ = [
        ("struct_size", c_u32), ("density", c_f64), ("radius", c_f64), ("young_modulus", c_f64),
        ("poisson_ratio", c_f64), ("shear_correction", c_f64), ("mass_damping", c_f64),
        ("contact_stiffness", c_f64), ("barrier_distance", c_f64), ("friction", c_f64),
        ("friction_smoothing", c_f64), ("collider_offset", c_f64),
    ]


class BuildStats(ctypes.Structure):
    _fields_ = [
        ("struct_size", c_u32), ("strand_count", c_u32), ("original_point_count", c_u32),
        ("internal_node_count", c_u32), ("element_count", c_u32), ("fixed_node_count", c_u32),
        ("collider_vertex_count", c_u32), ("collider_triangle_count", c_u32),
        ("excluded_collider_triangle_count", c_u32), ("collider_boundary_edge_count", c_u32),
        ("collider_nonmanifold_edge_count", c_u32), ("collider_inconsistent_edge_count", c_u32),
        ("collider_inverted_closed_component_count", c_u32), ("merged_zero_length_segment_count", c_u32),
        ("virtual_extension_strand_count", c_u32), ("virtual_extension_node_count", c_u32),
        ("virtual_extension_rest_length", c_f64), ("degree_of_freedom_count", c_u64),
        ("estimated_bytes", c_u64), ("initial_minimum_gap", c_f64),
    ]


class StepStats(ctypes.Structure):
    _fields_ = [
        ("struct_size", c_u32), ("substeps", c_u32), ("converged_substeps", c_u32),
        ("newton_iterations", c_u32), ("linear_solves", c_u32), ("line_search_evaluations", c_u32),
        ("contact_candidate_count", c_u64), ("active_contact_count", c_u64),
        ("initial_residual_norm", c_f64), ("final_residual_norm", c_f64), ("relative_residual_norm", c_f64),
        ("increment_norm", c_f64), ("objective_change", c_f64), ("minimum_gap", c_f64),
        ("accepted_step_length", c_f64), ("ccd_step_limit", c_f64), ("kinetic_energy", c_f64),
        ("elastic_energy", c_f64), ("contact_energy", c_f64), ("friction_energy", c_f64), ("phase", ctypes.c_int),
    ]


class GpuInfo(ctypes.Structure):
    _fields_ = [
        ("struct_size", c_u32), ("available", c_u32), ("device_ordinal", c_i32),
        ("compute_capability_major", c_u32), ("compute_capability_minor", c_u32),
        ("total_vram_bytes", c_u64), ("device_name", ctypes.c_char * 128),
    ]


class GpuStats(ctypes.Structure):
    _fields_ = [
        ("struct_size", c_u32), ("animation_frame_count", c_u32), ("resident_bytes", c_u64),
        ("peak_temporary_bytes", c_u64), ("last_frame_milliseconds", c_f64),
        ("last_assembly_milliseconds", c_f64), ("last_collision_milliseconds", c_f64),
        ("last_optimization_milliseconds", c_f64),
    ]


class Progress(ctypes.Structure):
    _fields_ = [
        ("struct_size", c_u32), ("phase", c_u32), ("frame_index", c_u32), ("frame_count", c_u32),
        ("substep", c_u32), ("substep_count", c_u32), ("nonlinear_iteration", c_u32),
        ("nonlinear_iteration_limit", c_u32), ("cancelled", c_u32), ("frame_elapsed_seconds", c_f64),
    ]


class FailureDiagnostics(ctypes.Structure):
    _fields_ = [
        ("struct_size", c_u32), ("kind", c_u32), ("frame_index", c_u32), ("substep", c_u32),
        ("requested_substeps", c_u32), ("attempted_substeps", c_u32), ("maximum_substeps", c_u32),
        ("adaptive_attempt_count", c_u32), ("strand_index", c_u32), ("element_index", c_u32),
        ("collider_triangle_index", c_u32), ("reserved", c_u32), ("distance", c_f64),
        ("required_distance", c_f64), ("clearance", c_f64), ("collider_substep_displacement", c_f64),
        ("collider_frame_displacement", c_f64), ("hair_start", Vec3), ("hair_end", Vec3),
        ("collider_point", Vec3),
    ]


class SubstepRecord(ctypes.Structure):
    _fields_ = [
        ("struct_size", c_u32), ("substep", c_u32), ("newton_iterations", c_u32),
        ("line_search_evaluations", c_u32), ("steepest_fallbacks", c_u32), ("refinement_sweeps", c_u32),
        ("fp64_fallbacks", c_u32), ("trust_scalings", c_u32), ("contact_candidates", c_u64), ("active_contacts", c_u64), ("final_residual_norm", c_f64),
        ("minimum_gap", c_f64),
    ]


class ContactRecord(ctypes.Structure):
    _fields_ = [("candidate_count", c_u32), ("closest_triangle", c_u32), ("active", c_u32),
                ("reserved", c_u32), ("gap", c_f64)]


class KernelTiming(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 40), ("launches", c_u64), ("total_milliseconds", c_f64)]


CONTACT_DTYPE = np.dtype([("candidate_count", "<u4"), ("closest_triangle", "<u4"), ("active", "<u4"),
                          ("reserved", "<u4"), ("gap", "<f8")])

P = ctypes.POINTER
VP = ctypes.c_void_p

# (name, restype, argtypes) for every exported entry point of the v5 ABI.
ABI_FUNCTIONS = [
    ("khsGetAbiVersion", c_u32, []),
    ("khsGetGpuInfo", ctypes.c_int, [P(GpuInfo)]),
    ("khsDefaultSolverDesc", None, [P(SolverDesc)]),
    ("khsDefaultHairMaterial", None, [P(HairMaterial)]),
    ("khsCreate", VP, [P(SolverDesc)]),
    ("khsDestroy", None, [VP]),
    ("khsSetHairCurves", ctypes.c_int, [VP, VP, c_u32, VP, c_u32, P(HairMaterial)]),
    ("khsSetColliderMesh", ctypes.c_int, [VP, VP, c_u32, VP, c_u32]),
    ("khsBuild", ctypes.c_int, [VP]),
    ("khsUpdateRuntimeParameters", ctypes.c_int, [VP, P(SolverDesc), P(HairMaterial)]),
    ("khsUpdateColliderVertices", ctypes.c_int, [VP, VP, c_u32]),
    ("khsUpdateRootTargets", ctypes.c_int, [VP, VP, c_u32]),
    ("khsStep", ctypes.c_int, [VP, c_f64]),
    ("khsAllocateAnimation", ctypes.c_int, [VP, c_u32]),
    ("khsSetRootAnimationFrame", ctypes.c_int, [VP, c_u32, VP, c_u32]),
    ("khsSetColliderAnimationFrame", ctypes.c_int, [VP, c_u32, VP, c_u32]),
    ("khsFinalizeAnimation", ctypes.c_int, [VP]),
    ("khsStepAnimationFrame", ctypes.c_int, [VP, c_u32, c_f64]),
    ("khsGetAnimationCheckpointSize", c_u64, [VP]),
    ("khsSaveAnimationCheckpoint", ctypes.c_int, [VP, VP, c_u64]),
    ("khsRestoreAnimationCheckpoint", ctypes.c_int, [VP, VP, c_u64]),
    ("khsGetOriginalPointCount", c_u32, [VP]),
    ("khsGetInternalNodeCount", c_u32, [VP]),
    ("khsCopyOriginalPositions", ctypes.c_int, [VP, VP, c_u32]),
    ("khsCopyInternalPositions", ctypes.c_int, [VP, VP, c_u32]),
    ("khsCopyOriginalToInternalMap", ctypes.c_int, [VP, VP, c_u32]),
    ("khsGetBuildStats", ctypes.c_int, [VP, P(BuildStats)]),
    ("khsGetLastStepStats", ctypes.c_int, [VP, P(StepStats)]),
    ("khsGetGpuStats", ctypes.c_int, [VP, P(GpuStats)]),
    ("khsGetProgress", ctypes.c_int, [VP, P(Progress)]),
    ("khsGetFailureDiagnostics", ctypes.c_int, [VP, P(FailureDiagnostics)]),
    ("khsRequestCancel", ctypes.c_int, [VP]),
    ("khsGetLastError", ctypes.c_char_p, [VP]),
]

# Additive GB300 extensions.
EXTENSION_FUNCTIONS = [
    ("khsxSetSolveMode", ctypes.c_int, [VP, c_u32]),
    ("khsxGetSolveMode", c_u32, [VP]),
    ("khsxSetSubstepLimit", ctypes.c_int, [VP, c_u32]),
    ("khsxCopyState", ctypes.c_int, [VP, VP, VP, c_u64]),
    ("khsxGetSubstepRecordCount", c_u32, [VP]),
    ("khsxCopySubstepRecords", ctypes.c_int, [VP, P(SubstepRecord), c_u32]),
    ("khsxCopyContactRecords", ctypes.c_int, [VP, VP, c_u32]),
    ("khsxQueryContacts", ctypes.c_int, [VP, VP, c_u64, VP, c_u32]),
    ("khsxSetBlockSolveSchedule", ctypes.c_int, [VP, c_u32, c_u32, c_u32]),
    ("khsxSetBlockSolveTiers", ctypes.c_int, [VP, c_u32, c_u32, c_u32, c_u32]),
    ("khsxSetRollbackRing", ctypes.c_int, [VP, c_u32]),
    ("khsxRollbackToFrame", ctypes.c_int, [VP, c_u32]),
    ("khsxQueryContactsNoAlloc", ctypes.c_int, [VP, VP, c_u64, VP, c_u32]),
    ("khsxComputeRootTargets", ctypes.c_int, [VP, VP, c_u32, VP, VP, c_u32]),
    ("khsxSetOutputRing", ctypes.c_int, [VP, c_u32]),
    ("khsxCopyOutputFrame", ctypes.c_int, [VP, c_u32, VP, c_u32]),
    ("khsxMapOutputFrame", ctypes.c_int, [VP, c_u32, P(VP)]),
    ("khsxSetProfiling", ctypes.c_int, [VP, c_u32]),
    ("khsxGetKernelTimings", c_u32, [VP, VP, c_u32]),
    ("khsxResetKernelTimings", ctypes.c_int, [VP]),
    ("khsxGetKernelLaunchCount", c_u64, [VP]),
    ("khsxMeasurePipePeaks", ctypes.c_int, [P(c_f64), P(c_f64)]),
]

# Entry points the CPU oracle does not provide (device-only measurement).
DEVICE_ONLY = {"khsxSetProfiling", "khsxGetKernelTimings", "khsxResetKernelTimings", "khsxGetKernelLaunchCount",
               "khsxMeasurePipePeaks", "khsxQueryContactsNoAlloc", "khsxSetBlockSolveSchedule", "khsxSetBlockSolveTiers",
               "khsxSetRollbackRing", "khsxRollbackToFrame", "khsxSetOutputRing", "khsxCopyOutputFrame",
               "khsxMapOutputFrame"}

# Size of the file-scope device scratch behind khsxQueryContactsNoAlloc
# (KHSX_NO_ALLOC_SCRATCH_BYTES in the C header).
NO_ALLOC_SCRATCH_BYTES = 8 * 1024 * 1024


def _vec3_buffer(values) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(values, dtype=np.float64).reshape((-1, 3)))


def _ptr(array: np.ndarray | None):
    return None if array is None else ctypes.c_void_p(array.ctypes.data)


class KhsError(RuntimeError):
    """A failed C-ABI call: ``code`` is its KhsResult."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = int(code)


class Library:
    """Loaded ABI library with typed entry points (raw result codes)."""

    def __init__(self, path: str | Path | None = None, extensions: bool = True):
        self.path = Path(path) if path else DEFAULT_LIBRARY
        if not self.path.exists():
            raise FileNotFoundError(f"solver library not built: {self.path}")
        # RTLD_LOCAL keeps two libraries exporting the same symbols apart.
        self.lib = ctypes.CDLL(str(self.path), mode=os.RTLD_LOCAL)
        for name, restype, argtypes in ABI_FUNCTIONS + (EXTENSION_FUNCTIONS if extensions else []):
            if name in DEVICE_ONLY and not hasattr(self.lib, name):
                continue
            fn = getattr(self.lib, name)
            fn.restype = restype
            fn.argtypes = argtypes
        if self.lib.khsGetAbiVersion() != ABI_VERSION:
            raise RuntimeError("solver library ABI version mismatch")

    def __getattr__(self, name):
        return getattr(self.lib, name)

    def default_desc(self) -> SolverDesc:
        d = SolverDesc()
        self.lib.khsDefaultSolverDesc(ctypes.byref(d))
        return d

    def default_material(self) -> HairMaterial:
        m = HairMaterial()
        self.lib.khsDefaultHairMaterial(ctypes.byref(m))
        return m


class HairSolver:
    """Solver handle with the reference binding's interface.

    Methods raise ``RuntimeError`` with the library's last error message when
    a call does not return ``KHS_OK`` (native.py:235-238).
    """

    def __init__(self, library_path: str | Path | Library | None = None):
        self.library = library_path if isinstance(library_path, Library) else Library(library_path)
        self._library = self.library.lib
        self._handle = None
        self.desc = self.library.default_desc()
        self.material = self.library.default_material()

    # -- lifetime ---------------------------------------------------------
    def create(self):
        if self._handle:
            self.close()
        self._handle = self._library.khsCreate(ctypes.byref(self.desc))
        if not self._handle:
            raise RuntimeError("cannot create the hair solver; check the solver description")

    def close(self):
        if self._handle:
            self._library.khsDestroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._handle

    def gpu_info(self) -> GpuInfo:
        info = GpuInfo()
        info.struct_size = ctypes.sizeof(info)
        if self._library.khsGetGpuInfo(ctypes.byref(info)) != OK:
            raise RuntimeError("no CUDA GPU available")
        return info

    def last_error(self) -> str:
        message = self._library.khsGetLastError(self._handle)
        return message.decode("utf-8", errors="replace") if message else ""

    def _check(self, result: int):
        if result != OK:
            raise KhsError(result, self.last_error() or f"hair solver error {result}")

    # -- scene input ------------------------------------------------------
    def set_hair(self, points, offsets):
        pts = _vec3_buffer(points)
        offs = np.ascontiguousarray(np.asarray(offsets, dtype=np.uint32))
        self._check(self._library.khsSetHairCurves(self._handle, _ptr(pts), len(pts), _ptr(offs), len(offs) - 1,
                                                   ctypes.byref(self.material)))

    def set_collider(self, vertices, triangles):
        if triangles is None or len(triangles) == 0:
            self._check(self._library.khsSetColliderMesh(self._handle, None, 0, None, 0))
            return
        verts = _vec3_buffer(vertices)
        tris = np.ascontiguousarray(np.asarray(triangles, dtype=np.uint32).reshape((-1, 3)))
        self._check(self._library.khsSetColliderMesh(self._handle, _ptr(verts), len(verts), _ptr(tris), len(tris)))

    def build(self) -> BuildStats:
        self._check(self._library.khsBuild(self._handle))
        return self.build_stats()

    def build_stats(self) -> BuildStats:
        stats = BuildStats()
        stats.struct_size = ctypes.sizeof(stats)
        self._check(self._library.khsGetBuildStats(self._handle, ctypes.byref(stats)))
        return stats

    def update_runtime_parameters(self):
        self._check(self._library.khsUpdateRuntimeParameters(self._handle, ctypes.byref(self.desc),
                                                             ctypes.byref(self.material)))

    def update_roots(self, points):
        pts = _vec3_buffer(points)
        self._check(self._library.khsUpdateRootTargets(self._handle, _ptr(pts), len(pts)))

    def update_collider(self, vertices):
        verts = _vec3_buffer(vertices)
        self._check(self._library.khsUpdateColliderVertices(self._handle, _ptr(verts), len(verts)))

    # -- stepping ---------------------------------------------------------
    def step(self, dt):
        self._check(self._library.khsStep(self._handle, float(dt)))
        return self.positions(), self.stats()

    def allocate_animation(self, frame_count):
        self._check(self._library.khsAllocateAnimation(self._handle, int(frame_count)))

    def set_root_animation_frame(self, frame, points):
        pts = _vec3_buffer(points)
        self._check(self._library.khsSetRootAnimationFrame(self._handle, int(frame), _ptr(pts), len(pts)))

    def set_collider_animation_frame(self, frame, vertices):
        if vertices is None or len(vertices) == 0:
            self._check(self._library.khsSetColliderAnimationFrame(self._handle, int(frame), None, 0))
            return
        verts = _vec3_buffer(vertices)
        self._check(self._library.khsSetColliderAnimationFrame(self._handle, int(frame), _ptr(verts), len(verts)))

    def finalize_animation(self):
        self._check(self._library.khsFinalizeAnimation(self._handle))

    def step_animation_frame(self, frame, dt):
        self._check(self._library.khsStepAnimationFrame(self._handle, int(frame), float(dt)))
        return self.positions(), self.stats()

    # -- checkpoints ------------------------------------------------------
    def checkpoint_size(self) -> int:
        return int(self._library.khsGetAnimationCheckpointSize(self._handle))

    def save_checkpoint(self) -> bytes:
        size = self.checkpoint_size()
        if not size:
            raise RuntimeError("the animation state cannot be saved yet")
        storage = (ctypes.c_ubyte * size)()
        self._check(self._library.khsSaveAnimationCheckpoint(self._handle, storage, size))
        return bytes(storage)

    def restore_checkpoint(self, checkpoint: bytes):
        storage = (ctypes.c_ubyte * len(checkpoint)).from_buffer_copy(checkpoint)
        self._check(self._library.khsRestoreAnimationCheckpoint(self._handle, storage, len(checkpoint)))

    # -- readback ---------------------------------------------------------
    def stats(self) -> StepStats:
        stats = StepStats()
        stats.struct_size = ctypes.sizeof(stats)
        self._check(self._library.khsGetLastStepStats(self._handle, ctypes.byref(stats)))
        return stats

    def gpu_stats(self) -> GpuStats:
        stats = GpuStats()
        stats.struct_size = ctypes.sizeof(stats)
        self._check(self._library.khsGetGpuStats(self._handle, ctypes.byref(stats)))
        return stats

    def progress(self) -> Progress:
        progress = Progress()
        progress.struct_size = ctypes.sizeof(progress)
        self._check(self._library.khsGetProgress(self._handle, ctypes.byref(progress)))
        return progress

    def failure_diagnostics(self) -> FailureDiagnostics:
        diagnostics = FailureDiagnostics()
        diagnostics.struct_size = ctypes.sizeof(diagnostics)
        self._check(self._library.khsGetFailureDiagnostics(self._handle, ctypes.byref(diagnostics)))
        return diagnostics

    def cancel(self):
        self._check(self._library.khsRequestCancel(self._handle))

    def positions(self) -> np.ndarray:
        count = int(self._library.khsGetOriginalPointCount(self._handle))
        out = np.empty((count, 3), dtype=np.float64)
        self._check(self._library.khsCopyOriginalPositions(self._handle, _ptr(out), count))
        return out

    def internal_positions(self) -> np.ndarray:
        count = int(self._library.khsGetInternalNodeCount(self._handle))
        out = np.empty((count, 3), dtype=np.float64)
        self._check(self._library.khsCopyInternalPositions(self._handle, _ptr(out), count))
        return out

    def mapping(self) -> np.ndarray:
        count = int(self._library.khsGetOriginalPointCount(self._handle))
        out = np.empty(count, dtype=np.uint32)
        self._check(self._library.khsCopyOriginalToInternalMap(self._handle, _ptr(out), count))
        return out

    # -- GB300 extensions -------------------------------------------------
    def set_solve_mode(self, mode: int):
        self._check(self._library.khsxSetSolveMode(self._handle, int(mode)))

    def set_substep_limit(self, substeps: int):
        """khsxSetSubstepLimit: end every following frame after ``substeps``
        substeps (0: whole frames)."""
        self._check(self._library.khsxSetSubstepLimit(self._handle, int(substeps)))

    def state(self) -> tuple[np.ndarray, np.ndarray]:
        n = int(self._library.khsGetInternalNodeCount(self._handle))
        q = np.empty((n, 6), dtype=np.float64)
        v = np.empty((n, 6), dtype=np.float64)
        self._check(self._library.khsxCopyState(self._handle, _ptr(q), _ptr(v), 6 * n))
        return q, v

    def substep_records(self) -> list[SubstepRecord]:
        count = int(self._library.khsxGetSubstepRecordCount(self._handle))
        records = (SubstepRecord * max(count, 1))()
        self._check(self._library.khsxCopySubstepRecords(self._handle, records, count))
        return list(records[:count])

    def set_profiling(self, on: bool):
        self._check(self._library.khsxSetProfiling(self._handle, 1 if on else 0))

    def kernel_timings(self) -> dict:
        cap = 64
        buf = (KernelTiming * cap)()
        n = int(self._library.khsxGetKernelTimings(self._handle, buf, cap))
        return {buf[k].name.decode(): (int(buf[k].launches), float(buf[k].total_milliseconds)) for k in range(min(n, cap))}

    def reset_kernel_timings(self):
        self._check(self._library.khsxResetKernelTimings(self._handle))

    def kernel_launches(self) -> int:
        return int(self._library.khsxGetKernelLaunchCount(self._handle))

    def query_contacts(self, q: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(q, dtype=np.float64)
        count = self.build_stats().element_count
        out = np.zeros(count, dtype=CONTACT_DTYPE)
        self._check(self._library.khsxQueryContacts(self._handle, _ptr(q), q.size, _ptr(out), count))
        return out

    def set_rollback_ring(self, slots: int) -> None:
        self._check(self._library.khsxSetRollbackRing(self._handle, slots))

    def rollback_to_frame(self, frame: int) -> None:
        self._check(self._library.khsxRollbackToFrame(self._handle, frame))

    def set_block_solve_schedule(self, strands_per_warp: int, blocks_per_sm: int = 1, long_strands: int = 0) -> None:
        self._check(self._library.khsxSetBlockSolveSchedule(self._handle, strands_per_warp, blocks_per_sm, long_strands))

    def set_block_solve_tiers(self, quads: int, singles: int, doubles: int, blocks_per_sm: int = 2) -> None:
        self._check(self._library.khsxSetBlockSolveTiers(self._handle, quads, singles, doubles, blocks_per_sm))

    def query_contacts_no_alloc(self, q: np.ndarray, out: np.ndarray) -> int:
        """khsxQueryContactsNoAlloc into a caller-owned CONTACT_DTYPE array;
        returns the raw result code (the entry point records no message)."""
        q = np.ascontiguousarray(q, dtype=np.float64)
        if out.dtype != CONTACT_DTYPE or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous CONTACT_DTYPE array")
        return int(self._library.khsxQueryContactsNoAlloc(self._handle, _ptr(q), q.size, _ptr(out), out.size))

    def set_output_ring(self, slots: int):
        self._check(self._library.khsxSetOutputRing(self._handle, int(slots)))

    def output_frame(self, frame: int) -> np.ndarray:
        """khsxCopyOutputFrame: (P, 3) positions of an animation frame."""
        n = int(self._library.khsGetOriginalPointCount(self._handle))
        out = np.zeros((n, 3), dtype=np.float64)
        self._check(self._library.khsxCopyOutputFrame(self._handle, int(frame), _ptr(out), n))
        return out

    def map_output_frame(self, frame: int) -> np.ndarray:
        """khsxMapOutputFrame: a read-only view of the pinned slot (valid
        until the ring moves past the frame)."""
        n = int(self._library.khsGetOriginalPointCount(self._handle))
        ptr = ctypes.c_void_p()
        self._check(self._library.khsxMapOutputFrame(self._handle, int(frame), ctypes.byref(ptr)))
        buf = (ctypes.c_double * (3 * n)).from_address(ptr.value)
        view = np.frombuffer(buf, dtype=np.float64).reshape(n, 3)
        view.flags.writeable = False
        return view

    def compute_root_targets(self, points) -> tuple[np.ndarray, np.ndarray]:
        """khsxComputeRootTargets: (positions, rotation vectors) of every
        internal node, each (N, 3), for the evaluated source points."""
        pts = _vec3_buffer(points)
        n = self.build_stats().internal_node_count
        pos = np.zeros((n, 3), dtype=np.float64)
        rot = np.zeros((n, 3), dtype=np.float64)
        self._check(self._library.khsxComputeRootTargets(self._handle, _ptr(pts), len(pts), _ptr(pos), _ptr(rot), n))
        return pos, rot

    def contact_records(self) -> np.ndarray:
        count = self.build_stats().element_count
        out = np.zeros(count, dtype=CONTACT_DTYPE)
        self._check(self._library.khsxCopyContactRecords(self._handle, _ptr(out), count))
        return out
