"""The reference's own known-answer tests, restated against the C ABI.

Each ``case_*`` function follows one test of the reference project
(tests/test_solver.cpp, tests/test_c_api.c) call for call and asserts the
same invariants with the same tolerances.  They take a ``khs_native.Library``
so the identical case runs against the CPU oracle (pinning it, CPU suite) and
against the GB300 product library (``-m gpu``).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

import khs_native as kn


def _solver(lib, desc, material=None):
    s = kn.HairSolver(lib)
    s.desc = desc
    if material is not None:
        s.material = material
    s.create()
    return s


def case_c_api_defaults(lib, require_gpu: bool):
    """tests/test_c_api.c:5-31 (the cc >= 12 check becomes cc == 10.x)."""
    desc = lib.default_desc()
    material = lib.default_material()
    assert lib.khsGetAbiVersion() == 5
    assert desc.struct_size == ctypes.sizeof(kn.SolverDesc)
    assert material.struct_size == ctypes.sizeof(kn.HairMaterial)
    assert desc.minimum_dynamic_length == 0.0
    assert desc.maximum_substeps == 32
    desc.maximum_substeps = desc.substeps - 1
    assert not lib.khsCreate(ctypes.byref(desc))
    desc.maximum_substeps = 32
    desc.minimum_dynamic_length = -1.0
    assert not lib.khsCreate(ctypes.byref(desc))
    desc.minimum_dynamic_length = 0.0
    if require_gpu:
        info = kn.GpuInfo()
        info.struct_size = ctypes.sizeof(info)
        assert lib.khsGetGpuInfo(ctypes.byref(info)) == kn.OK
        assert info.available == 1
        assert info.compute_capability_major == 10
        assert info.total_vram_bytes > 0
    handle = lib.khsCreate(ctypes.byref(desc))
    assert handle
    lib.khsDestroy(handle)


def case_rest_state_and_subdivision(lib):
    """tests/test_solver.cpp:18-60."""
    desc = lib.default_desc()
    desc.gravity = kn.Vec3(0.0, 0.0, 0.0)
    desc.substeps = 1
    desc.fixed_root_nodes = 1
    desc.maximum_element_length = 0.006
    material = lib.default_material()
    material.mass_damping = 0.0
    s = _solver(lib, desc, material)
    points = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, -0.01], [0.0, 0.0, -0.02]])
    s.set_hair(points, [0, 3])
    s.build()
    assert lib.khsGetInternalNodeCount(s.handle) == 5
    s.desc.substeps = 2
    s.desc.newton_iterations = 32
    s.material.density = 1400.0
    s.material.radius = 5.0e-5
    s.material.young_modulus = 2.0e9
    s.update_runtime_parameters()
    changed = kn.SolverDesc.from_buffer_copy(s.desc)
    changed.maximum_element_length = 0.007
    assert lib.khsUpdateRuntimeParameters(s.handle, ctypes.byref(changed), ctypes.byref(s.material)) == \
        kn.ERROR_INVALID_ARGUMENT
    out, stats = s.step(1.0 / 24.0)
    assert np.max(np.abs(out - points)) < 1.0e-10
    assert stats.phase == kn.PHASE_FINISHED
    assert stats.final_residual_norm < 1.0e-5
    s.close()


def case_minimum_dynamic_length_preserves_visible_prefix(lib):
    """tests/test_solver.cpp:62-107."""
    desc = lib.default_desc()
    desc.gravity = kn.Vec3(0.0, 0.0, 0.0)
    desc.substeps = 1
    desc.fixed_root_nodes = 1
    desc.maximum_element_length = 0.06
    desc.minimum_dynamic_length = 0.30
    material = lib.default_material()
    material.mass_damping = 0.0
    s = _solver(lib, desc, material)
    points = np.array([[0.0, 0.0, 0.0], [0.05, 0.0, 0.0], [0.10, 0.0, 0.0]])
    s.set_hair(points, [0, 3])
    b = s.build()
    assert b.original_point_count == 3
    assert b.internal_node_count == 7
    assert b.element_count == 6
    assert b.virtual_extension_strand_count == 1
    assert b.virtual_extension_node_count == 4
    assert abs(b.virtual_extension_rest_length - 0.20) < 1.0e-12
    internal = s.internal_positions()
    assert abs(internal[-1, 0] - 0.30) < 1.0e-12
    assert abs(internal[-1, 1]) < 1.0e-12 and abs(internal[-1, 2]) < 1.0e-12
    out, _ = s.step(1.0 / 24.0)
    assert np.max(np.abs(out - points)) < 1.0e-10
    s.close()


def case_virtual_extension_ignores_collider_contact(lib):
    """tests/test_solver.cpp:109-170."""
    desc = lib.default_desc()
    desc.gravity = kn.Vec3(0.0, 0.0, 0.0)
    desc.substeps = 1
    desc.fixed_root_nodes = 1
    desc.maximum_element_length = 0.05
    desc.minimum_dynamic_length = 0.30
    material = lib.default_material()
    material.mass_damping = 0.0
    points = np.array([[0.0, 0.0, 0.0], [0.05, 0.0, 0.0]])
    tri = [[0, 1, 2]]
    # Static triangle that crosses only the invisible extension.
    s = _solver(lib, desc, material)
    s.set_hair(points, [0, 2])
    s.set_collider([[0.10, -1.0, 0.0], [0.40, -1.0, 0.0], [0.25, 1.0, 0.0]], tri)
    b = s.build()
    assert b.virtual_extension_strand_count == 1
    assert math.isinf(b.initial_minimum_gap)
    _, st = s.step(1.0 / 24.0)
    assert st.contact_candidate_count == 0
    assert st.active_contact_count == 0
    s.close()
    # Moving triangle that sweeps through only the invisible extension.
    s = _solver(lib, desc, material)
    s.set_hair(points, [0, 2])
    s.set_collider([[0.10, -1.0, -0.1], [0.40, -1.0, -0.1], [0.25, 1.0, -0.1]], tri)
    s.build()
    s.update_collider([[0.10, -1.0, 0.1], [0.40, -1.0, 0.1], [0.25, 1.0, 0.1]])
    _, st = s.step(1.0 / 24.0)
    assert st.contact_candidate_count == 0
    assert st.active_contact_count == 0
    s.close()


def case_duplicate_mapping(lib):
    """tests/test_solver.cpp:172-195."""
    desc = lib.default_desc()
    desc.gravity = kn.Vec3(0.0, 0.0, 0.0)
    desc.maximum_element_length = 1.0
    desc.fixed_root_nodes = 1
    s = _solver(lib, desc)
    s.set_hair([[0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, 0.0, 0.1]], [0, 3])
    b = s.build()
    m = s.mapping()
    assert m[0] == m[1]
    assert m[2] != m[1]
    assert b.merged_zero_length_segment_count == 1
    s.close()


def case_initial_intersection_rejected(lib):
    """tests/test_solver.cpp:197-216."""
    desc = lib.default_desc()
    desc.maximum_element_length = 1.0
    desc.fixed_root_nodes = 1
    material = lib.default_material()
    material.radius = 1.0e-3
    material.barrier_distance = 2.0e-3
    s = _solver(lib, desc, material)
    s.set_hair([[-0.2, 0.0, 0.2], [-0.1, 0.0, 0.1], [0.1, 0.0, -0.1]], [0, 3])
    s.set_collider([[-1.0, -1.0, 0.0], [1.0, -1.0, 0.0], [0.0, 1.0, 0.0]], [[0, 1, 2]])
    assert lib.khsBuild(s.handle) == kn.ERROR_INITIAL_INTERSECTION
    s.close()


def case_barrier_contact_remains_feasible(lib):
    """tests/test_solver.cpp:218-251."""
    desc = lib.default_desc()
    desc.substeps = 4
    desc.fixed_root_nodes = 1
    desc.maximum_element_length = 0.02
    desc.newton_iterations = 40
    material = lib.default_material()
    material.radius = 2.0e-4
    material.young_modulus = 1.0e6
    material.contact_stiffness = 100.0
    material.barrier_distance = 2.0e-3
    material.mass_damping = 2.0
    s = _solver(lib, desc, material)
    s.set_hair([[0.0, 0.0, 0.03], [0.0, 0.0, 0.02], [0.0, 0.0, 0.01], [0.0, 0.0, 0.001]], [0, 4])
    s.set_collider([[-1.0, -1.0, 0.0], [1.0, -1.0, 0.0], [1.0, 1.0, 0.0], [-1.0, 1.0, 0.0]], [[0, 1, 2], [0, 2, 3]])
    s.build()
    for _ in range(3):
        _, st = s.step(1.0 / 60.0)
    assert st.active_contact_count > 0
    assert st.minimum_gap > desc.minimum_gap
    assert st.phase == kn.PHASE_FINISHED
    s.close()
    return st


def case_moving_collider_tunnelling_rejected(lib):
    """tests/test_solver.cpp:253-288."""
    desc = lib.default_desc()
    desc.substeps = 1
    desc.maximum_substeps = 4
    desc.fixed_root_nodes = 1
    desc.maximum_element_length = 1.0
    material = lib.default_material()
    material.radius = 1.0e-3
    s = _solver(lib, desc, material)
    s.set_hair([[-0.2, 0.0, 0.0], [-0.1, 0.0, 0.0], [0.1, 0.0, 0.0]], [0, 3])
    s.set_collider([[-1.0, -1.0, -0.1], [1.0, -1.0, -0.1], [0.0, 1.0, -0.1]], [[0, 1, 2]])
    s.build()
    s.update_collider([[-1.0, -1.0, 0.1], [1.0, -1.0, 0.1], [0.0, 1.0, 0.1]])
    assert lib.khsStep(s.handle, 1.0 / 24.0) == kn.ERROR_NOT_CONVERGED
    d = s.failure_diagnostics()
    assert d.kind == kn.FAILURE_SWEEP
    assert d.requested_substeps == 1
    assert d.attempted_substeps == 4
    assert d.maximum_substeps == 4
    assert d.adaptive_attempt_count == 3
    assert d.strand_index == 0
    assert d.collider_triangle_index == 0
    assert d.distance <= d.required_distance + 1.0e-12
    assert abs(d.collider_frame_displacement - 0.2) < 1.0e-12
    s.close()
    return d


def case_gpu_resident_animation(lib, expect_positive_frame_time: bool = True):
    """tests/test_solver.cpp:290-343."""
    desc = lib.default_desc()
    desc.gravity = kn.Vec3(0.0, 0.0, 0.0)
    desc.substeps = 1
    desc.newton_iterations = 100
    desc.fixed_root_nodes = 1
    desc.maximum_element_length = 1.0
    s = _solver(lib, desc)
    first = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, -0.1], [0.0, 0.0, -0.2]])
    second = np.array([[0.001, 0.0, 0.0], [0.001, 0.0, -0.1], [0.001, 0.0, -0.2]])
    s.set_hair(first, [0, 3])
    s.build()
    s.allocate_animation(2)
    s.set_root_animation_frame(0, first)
    s.set_root_animation_frame(1, second)
    s.set_collider_animation_frame(0, None)
    s.set_collider_animation_frame(1, None)
    s.finalize_animation()
    assert s.checkpoint_size() > 0
    ckpt = s.save_checkpoint()
    first_result, _ = s.step_animation_frame(1, 1.0 / 24.0)
    s.restore_checkpoint(ckpt)
    repeated, _ = s.step_animation_frame(1, 1.0 / 24.0)
    assert np.max(np.abs(first_result - repeated)) < 1.0e-14
    g = s.gpu_stats()
    assert g.animation_frame_count == 2
    assert g.resident_bytes > 0
    if expect_positive_frame_time:
        assert g.last_frame_milliseconds > 0.0
    assert s.progress().phase == kn.PHASE_FINISHED
    s.close()


ALL_SOLVER_CASES = [
    case_rest_state_and_subdivision,
    case_minimum_dynamic_length_preserves_visible_prefix,
    case_virtual_extension_ignores_collider_contact,
    case_duplicate_mapping,
    case_initial_intersection_rejected,
    case_barrier_contact_remains_feasible,
    case_moving_collider_tunnelling_rejected,
    case_gpu_resident_animation,
]
