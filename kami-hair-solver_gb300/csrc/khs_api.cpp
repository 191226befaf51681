// C ABI of the GB300 solver (include/kami_hair_solver.h).
//
// A KhsSolver owns the caller's scene input, the host rod model built from
// it and the device Engine.  Argument validation, result codes, error
// strings and the order of checks follow the reference's API and Solver
// layers (src/api.cpp:16-304, src/solver.cpp:121-900) so a caller sees the
// same behaviour; no exception crosses the ABI.
#include "kami_hair_solver.h"
#include "khs_engine.hpp"
#include "khs_model.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <new>
#include <string>
#include <vector>

namespace {

using khs::Vec;

bool material_ok_for_hair(const KhsHairMaterial &m)
{
    return m.density > 0.0 && m.radius > 0.0 && m.young_modulus > 0.0 && m.poisson_ratio > -1.0 && m.poisson_ratio < 0.5 &&
           m.shear_correction > 0.0 && m.contact_stiffness > 0.0 && m.barrier_distance > 0.0 && m.friction >= 0.0 &&
           m.friction_smoothing > 0.0;
}

bool material_ok_full(const KhsHairMaterial &m)
{
    return material_ok_for_hair(m) && m.mass_damping >= 0.0 && m.collider_offset >= 0.0;
}

bool finite3(const KhsVec3 &v) { return std::isfinite(v.x) && std::isfinite(v.y) && std::isfinite(v.z); }
Vec to_vec(const KhsVec3 &v) { Vec r; r.x = v.x; r.y = v.y; r.z = v.z; return r; }

}  // namespace

struct KhsSolver {
    explicit KhsSolver(const KhsSolverDesc &d) : desc(d)
    {
        step_stats.struct_size = sizeof(KhsStepStats);
        step_stats.phase = KHS_PHASE_IDLE;
        build_stats.struct_size = sizeof(KhsBuildStats);
    }

    KhsSolverDesc desc;
    KhsHairMaterial material{};
    khs::SceneInput input;
    khs::Model model;
    std::unique_ptr<khs::Engine> engine;
    bool built = false;
    uint32_t mode = KHSX_MODE_PLAIN_FP64;
    uint32_t substep_limit = 0;
    std::vector<Vec> collider_pending;
    KhsBuildStats build_stats{};
    KhsStepStats step_stats{};
    std::string error;

    void clear_built()
    {
        built = false;
        engine.reset();
        model = khs::Model{};
    }

    KhsResult set_hair(const KhsVec3 *points, uint32_t point_count, const uint32_t *offsets, uint32_t strand_count,
                       const KhsHairMaterial &m)
    {
        if (!points || !offsets || point_count < 2 || strand_count == 0 || offsets[0] != 0 ||
            offsets[strand_count] != point_count) {
            error = "hair points or strand offsets are invalid";
            return KHS_ERROR_INVALID_ARGUMENT;
        }
        for (uint32_t s = 0; s < strand_count; ++s)
            if (offsets[s + 1] <= offsets[s] || offsets[s + 1] > point_count) {
                error = "hair strand offsets are not increasing";
                return KHS_ERROR_INVALID_HAIR;
            }
        if (!material_ok_for_hair(m)) {
            error = "hair material values are out of range";
            return KHS_ERROR_INVALID_ARGUMENT;
        }
        std::vector<Vec> pts(point_count);
        for (uint32_t i = 0; i < point_count; ++i) {
            if (!finite3(points[i])) {
                error = "hair point " + std::to_string(i) + " has a non-finite coordinate";
                return KHS_ERROR_INVALID_HAIR;
            }
            pts[i] = to_vec(points[i]);
        }
        clear_built();
        input.points = std::move(pts);
        input.offsets.assign(offsets, offsets + strand_count + 1);
        input.has_hair = true;
        material = m;
        error.clear();
        return KHS_OK;
    }

    KhsResult set_collider(const KhsVec3 *vertices, uint32_t vertex_count, const KhsTriangle *tris, uint32_t tri_count)
    {
        if (tri_count == 0) {
            input.has_collider = false;
            input.collider_vertices.clear();
            input.collider_triangles.clear();
            input.excluded_triangles = 0;
            collider_pending.clear();
            built = false;
            return KHS_OK;
        }
        if (!vertices || !tris || vertex_count < 3) {
            error = "collider vertex or triangle arrays are invalid";
            return KHS_ERROR_INVALID_ARGUMENT;
        }
        std::vector<Vec> verts(vertex_count);
        for (uint32_t i = 0; i < vertex_count; ++i) verts[i] = to_vec(vertices[i]);
        std::vector<uint32_t> valid;
        uint32_t excluded = 0;
        for (uint32_t k = 0; k < tri_count; ++k) {
            const KhsTriangle &t = tris[k];
            if (t.i0 >= vertex_count || t.i1 >= vertex_count || t.i2 >= vertex_count || t.i0 == t.i1 || t.i1 == t.i2 ||
                t.i2 == t.i0 || !finite3(vertices[t.i0]) || !finite3(vertices[t.i1]) || !finite3(vertices[t.i2])) {
                ++excluded;
                continue;
            }
            const Vec a = verts[t.i0], b = verts[t.i1], c = verts[t.i2];
            const double e1x = b.x - a.x, e1y = b.y - a.y, e1z = b.z - a.z;
            const double e2x = c.x - a.x, e2y = c.y - a.y, e2z = c.z - a.z;
            const double cx = e1y * e2z - e1z * e2y, cy = e1z * e2x - e1x * e2z, cz = e1x * e2y - e1y * e2x;
            if (cx * cx + cy * cy + cz * cz <= 1.0e-24) {  // degenerate (solver.cpp:203-208)
                ++excluded;
                continue;
            }
            valid.push_back(t.i0);
            valid.push_back(t.i1);
            valid.push_back(t.i2);
        }
        if (valid.empty()) {
            error = "the collider has no valid triangle";
            return KHS_ERROR_INVALID_COLLIDER;
        }
        input.collider_vertices = std::move(verts);
        input.collider_triangles = std::move(valid);
        input.excluded_triangles = excluded;
        input.has_collider = true;
        collider_pending = input.collider_vertices;
        built = false;
        error.clear();
        return KHS_OK;
    }

    KhsResult build()
    {
        if (!input.has_hair) {
            error = "set hair curves before building";
            return KHS_ERROR_INVALID_STATE;
        }
        step_stats.phase = KHS_PHASE_PREPARING;
        engine.reset();
        built = false;
        std::string err;
        if (!khs::build_rod_model(input, desc, material, model, err)) {
            error = err;
            step_stats.phase = KHS_PHASE_FAILED;
            return KHS_ERROR_INVALID_HAIR;
        }
        std::vector<Vec> root_pos, root_rot;
        if (!khs::root_targets(model, input.points, root_pos, root_rot)) {
            error = "cannot build the initial root directions";
            step_stats.phase = KHS_PHASE_FAILED;
            return KHS_ERROR_INVALID_HAIR;
        }
        double initial_gap = std::numeric_limits<double>::infinity();
        if (input.has_collider) {
            model.collider = input.collider_vertices;
            model.tri = input.collider_triangles;
            khs::collider_topology(model);
            if (!khs::initial_feasibility(model, desc, material, initial_gap, err)) {
                error = err;
                step_stats.phase = KHS_PHASE_FAILED;
                return KHS_ERROR_INITIAL_INTERSECTION;
            }
            khs::build_device_bvh(model);
        }
        std::unique_ptr<khs::Engine> e(new khs::Engine());
        e->set_mode(mode);
        e->set_substep_limit(substep_limit);
        e->initialize(model, desc, material, root_pos, root_rot);
        engine = std::move(e);
        collider_pending = model.collider;
        built = true;
        build_stats = {};
        build_stats.struct_size = sizeof(KhsBuildStats);
        build_stats.strand_count = uint32_t(model.strands());
        build_stats.original_point_count = uint32_t(input.points.size());
        build_stats.internal_node_count = uint32_t(model.nodes());
        build_stats.element_count = uint32_t(model.elements());
        build_stats.fixed_node_count = uint32_t(std::count(model.fixed.begin(), model.fixed.end(), uint8_t(1)));
        build_stats.collider_vertex_count = uint32_t(model.collider.size());
        build_stats.collider_triangle_count = uint32_t(model.tri.size() / 3);
        build_stats.excluded_collider_triangle_count = input.excluded_triangles;
        build_stats.collider_boundary_edge_count = model.boundary_edges;
        build_stats.collider_nonmanifold_edge_count = model.nonmanifold_edges;
        build_stats.collider_inconsistent_edge_count = model.inconsistent_edges;
        build_stats.collider_inverted_closed_component_count = model.inverted_components;
        build_stats.merged_zero_length_segment_count = model.merged_segments;
        build_stats.virtual_extension_strand_count = model.extension_strands;
        build_stats.virtual_extension_node_count = model.extension_nodes;
        build_stats.virtual_extension_rest_length = model.extension_length;
        uint64_t free_dofs = 0;
        for (uint8_t f : model.fixed) if (!f) free_dofs += 6;
        build_stats.degree_of_freedom_count = free_dofs;
        build_stats.estimated_bytes = engine->gpu_stats().resident_bytes;
        build_stats.initial_minimum_gap = initial_gap;
        step_stats = {};
        step_stats.struct_size = sizeof(KhsStepStats);
        step_stats.phase = KHS_PHASE_IDLE;
        error.clear();
        return KHS_OK;
    }

    KhsResult update_runtime(const KhsSolverDesc &d, const KhsHairMaterial &m)
    {
        if (!built || !engine) {
            error = "build the solver before updating runtime parameters";
            return KHS_ERROR_INVALID_STATE;
        }
        if (d.maximum_element_length != desc.maximum_element_length ||
            d.minimum_dynamic_length != desc.minimum_dynamic_length || d.fixed_root_nodes != desc.fixed_root_nodes) {
            error = "maximum_element_length, minimum_dynamic_length and fixed_root_nodes cannot change after build";
            return KHS_ERROR_INVALID_ARGUMENT;
        }
        if (!material_ok_full(m)) {
            error = "runtime material values are out of range";
            return KHS_ERROR_INVALID_ARGUMENT;
        }
        desc = d;
        material = m;
        khs::assign_masses(model, material);
        engine->update_runtime(desc, material, model.mass, model.rotational_mass);
        error.clear();
        return KHS_OK;
    }

    KhsResult update_collider(const KhsVec3 *v, uint32_t n)
    {
        if (!built || !input.has_collider) {
            error = "no built collider";
            return KHS_ERROR_INVALID_STATE;
        }
        if (!v || n != collider_pending.size()) {
            error = "the animated collider vertex count changed";
            return KHS_ERROR_INVALID_COLLIDER;
        }
        std::vector<Vec> verts(n);
        for (uint32_t i = 0; i < n; ++i) {
            if (!finite3(v[i])) {
                error = "the animated collider has a non-finite coordinate";
                return KHS_ERROR_INVALID_COLLIDER;
            }
            verts[i] = to_vec(v[i]);
        }
        collider_pending = verts;
        engine->set_pending_collider(verts);
        return KHS_OK;
    }

    // Source points of new root targets: the solver must be built, the
    // count must match the curves, every coordinate finite
    // (solver.cpp:802-811).  The targets themselves are computed on the
    // device by the engine.
    KhsResult check_root_points(const KhsVec3 *p, uint32_t n, KhsResult bad_point, KhsResult bad_count)
    {
        if (!built || !engine || !p || n != input.points.size()) {
            error = "the root target point count does not match the source curves";
            return bad_count;
        }
        for (uint32_t i = 0; i < n; ++i)
            if (!finite3(p[i])) {
                error = "root targets have a non-finite coordinate";
                return bad_point;
            }
        return KHS_OK;
    }

    KhsResult update_roots(const KhsVec3 *p, uint32_t n)
    {
        const KhsResult r = check_root_points(p, n, KHS_ERROR_INVALID_HAIR, KHS_ERROR_INVALID_ARGUMENT);
        if (r != KHS_OK) return r;
        return from_engine(engine->set_pending_root_points(p, n));
    }

    KhsResult from_engine(KhsResult r)
    {
        if (r != KHS_OK) error = engine->last_error();
        return r;
    }

    KhsResult after_engine(KhsResult r)
    {
        step_stats = engine->stats();
        if (r != KHS_OK) error = engine->last_error();
        else error.clear();
        return r;
    }
};

namespace {

template<class F> KhsResult guarded(KhsSolver *s, F &&f)
{
    if (!s) return KHS_ERROR_INVALID_ARGUMENT;
    try {
        return f();
    } catch (const std::bad_alloc &) {
        s->error = "out of host memory";
        return KHS_ERROR_OUT_OF_MEMORY;
    } catch (const std::exception &e) {
        s->error = std::string("internal exception: ") + e.what();
        return KHS_ERROR_INTERNAL;
    } catch (...) {
        s->error = "unknown internal exception";
        return KHS_ERROR_INTERNAL;
    }
}

bool valid_desc(const KhsSolverDesc *d)
{
    return d && d->struct_size >= sizeof(KhsSolverDesc) && d->substeps > 0 && d->maximum_substeps >= d->substeps &&
           d->newton_iterations > 0 && d->line_search_iterations > 0 && d->absolute_tolerance > 0.0 &&
           d->relative_tolerance > 0.0 && d->increment_tolerance > 0.0 && d->minimum_line_search_step > 0.0 &&
           d->minimum_gap > 0.0 && d->maximum_element_length > 0.0 && d->minimum_dynamic_length >= 0.0 &&
           std::isfinite(d->minimum_dynamic_length) && d->fixed_root_nodes > 0;
}

bool valid_material(const KhsHairMaterial *m) { return m && m->struct_size >= sizeof(KhsHairMaterial) && material_ok_full(*m); }

}  // namespace

extern "C" {

KHS_API uint32_t khsGetAbiVersion(void) { return KHS_ABI_VERSION; }

KHS_API KhsResult khsGetGpuInfo(KhsGpuInfo *info)
{
    if (!info || info->struct_size < sizeof(KhsGpuInfo)) return KHS_ERROR_INVALID_ARGUMENT;
    std::string error;
    KhsGpuInfo r{};
    const bool ok = khs::query_device(r, error);
    *info = r;
    return ok ? KHS_OK : KHS_ERROR_INVALID_STATE;
}

KHS_API void khsDefaultSolverDesc(KhsSolverDesc *d)
{
    if (!d) return;
    std::memset(d, 0, sizeof(*d));
    d->struct_size = sizeof(*d);
    d->gravity = {0.0, 0.0, -9.81};
    d->substeps = 8;
    d->maximum_substeps = 32;
    d->newton_iterations = 24;
    d->line_search_iterations = 20;
    d->absolute_tolerance = 1.0e-8;
    d->relative_tolerance = 1.0e-5;
    d->increment_tolerance = 1.0e-8;
    d->minimum_line_search_step = 1.0e-9;
    d->minimum_gap = 1.0e-7;
    d->maximum_element_length = 0.01;
    d->minimum_dynamic_length = 0.0;
    d->fixed_root_nodes = 2;
    d->thread_count = 0;
}

KHS_API void khsDefaultHairMaterial(KhsHairMaterial *m)
{
    if (!m) return;
    std::memset(m, 0, sizeof(*m));
    m->struct_size = sizeof(*m);
    m->density = 1300.0;
    m->radius = 4.0e-5;
    m->young_modulus = 4.0e9;
    m->poisson_ratio = 0.38;
    m->shear_correction = 0.9;
    m->mass_damping = 8.0;
    m->contact_stiffness = 1.0e4;
    m->barrier_distance = 2.0e-4;
    m->friction = 0.35;
    m->friction_smoothing = 1.0e-6;
    m->collider_offset = 0.0;
}

KHS_API KhsSolver *khsCreate(const KhsSolverDesc *desc)
{
    if (!valid_desc(desc)) return nullptr;
    try { return new KhsSolver(*desc); } catch (...) { return nullptr; }
}

KHS_API void khsDestroy(KhsSolver *solver) { delete solver; }

KHS_API KhsResult khsSetHairCurves(KhsSolver *s, const KhsVec3 *points, uint32_t point_count, const uint32_t *offsets,
                                   uint32_t strand_count, const KhsHairMaterial *material)
{
    if (!material || material->struct_size < sizeof(KhsHairMaterial)) return KHS_ERROR_INVALID_ARGUMENT;
    return guarded(s, [&] { return s->set_hair(points, point_count, offsets, strand_count, *material); });
}

KHS_API KhsResult khsSetColliderMesh(KhsSolver *s, const KhsVec3 *vertices, uint32_t vertex_count,
                                     const KhsTriangle *triangles, uint32_t triangle_count)
{
    return guarded(s, [&] { return s->set_collider(vertices, vertex_count, triangles, triangle_count); });
}

KHS_API KhsResult khsBuild(KhsSolver *s) { return guarded(s, [&] { return s->build(); }); }

KHS_API KhsResult khsUpdateRuntimeParameters(KhsSolver *s, const KhsSolverDesc *d, const KhsHairMaterial *m)
{
    if (!valid_desc(d) || !valid_material(m)) return KHS_ERROR_INVALID_ARGUMENT;
    return guarded(s, [&] { return s->update_runtime(*d, *m); });
}

KHS_API KhsResult khsUpdateColliderVertices(KhsSolver *s, const KhsVec3 *v, uint32_t n)
{
    return guarded(s, [&] { return s->update_collider(v, n); });
}

KHS_API KhsResult khsUpdateRootTargets(KhsSolver *s, const KhsVec3 *p, uint32_t n)
{
    return guarded(s, [&] { return s->update_roots(p, n); });
}

KHS_API KhsResult khsStep(KhsSolver *s, double frame_dt)
{
    return guarded(s, [&] {
        if (!s->built || !s->engine) {
            s->error = "prepare the hair solver before stepping";
            return KHS_ERROR_INVALID_STATE;
        }
        if (!(frame_dt > 0.0) || !std::isfinite(frame_dt)) {
            s->error = "the time step must be positive and finite";
            return KHS_ERROR_INVALID_ARGUMENT;
        }
        return s->after_engine(s->engine->step(frame_dt));
    });
}

KHS_API KhsResult khsAllocateAnimation(KhsSolver *s, uint32_t frame_count)
{
    return guarded(s, [&] {
        if (!s->built || !s->engine) return KHS_ERROR_INVALID_STATE;
        const KhsResult r = s->engine->allocate_animation(frame_count);
        if (r != KHS_OK) s->error = s->engine->last_error();
        return r;
    });
}

KHS_API KhsResult khsSetRootAnimationFrame(KhsSolver *s, uint32_t frame_index, const KhsVec3 *points, uint32_t point_count)
{
    return guarded(s, [&] {
        const KhsResult c = s->check_root_points(points, point_count, KHS_ERROR_INVALID_HAIR, KHS_ERROR_INVALID_ARGUMENT);
        if (c != KHS_OK) return c;
        return s->from_engine(s->engine->set_root_animation_frame(frame_index, points, point_count));
    });
}

KHS_API KhsResult khsSetColliderAnimationFrame(KhsSolver *s, uint32_t frame_index, const KhsVec3 *vertices, uint32_t vertex_count)
{
    return guarded(s, [&] {
        if (!s->built || !s->engine) return KHS_ERROR_INVALID_STATE;
        const KhsResult r = s->engine->set_collider_animation_frame(frame_index, vertices, vertex_count);
        if (r != KHS_OK) s->error = s->engine->last_error();
        return r;
    });
}

KHS_API KhsResult khsFinalizeAnimation(KhsSolver *s)
{
    return guarded(s, [&] {
        if (!s->built || !s->engine) return KHS_ERROR_INVALID_STATE;
        const KhsResult r = s->engine->finalize_animation();
        if (r != KHS_OK) s->error = s->engine->last_error();
        return r;
    });
}

KHS_API KhsResult khsStepAnimationFrame(KhsSolver *s, uint32_t frame_index, double frame_dt)
{
    return guarded(s, [&] {
        if (!s->built || !s->engine) return KHS_ERROR_INVALID_STATE;
        return s->after_engine(s->engine->step_animation_frame(frame_index, frame_dt));
    });
}

KHS_API uint64_t khsGetAnimationCheckpointSize(const KhsSolver *s)
{
    return s && s->built && s->engine ? s->engine->checkpoint_size() : 0;
}

KHS_API KhsResult khsSaveAnimationCheckpoint(KhsSolver *s, void *data, uint64_t capacity)
{
    return guarded(s, [&] {
        if (!s->built || !s->engine) return KHS_ERROR_INVALID_STATE;
        return s->engine->save_checkpoint(data, capacity);
    });
}

KHS_API KhsResult khsRestoreAnimationCheckpoint(KhsSolver *s, const void *data, uint64_t size)
{
    return guarded(s, [&] {
        if (!s->built || !s->engine) return KHS_ERROR_INVALID_STATE;
        const KhsResult r = s->engine->restore_checkpoint(data, size);
        if (r != KHS_OK) s->error = s->engine->last_error();
        else { s->error.clear(); s->step_stats = s->engine->stats(); }
        return r;
    });
}

KHS_API uint32_t khsGetOriginalPointCount(const KhsSolver *s) { return s ? uint32_t(s->input.points.size()) : 0; }
KHS_API uint32_t khsGetInternalNodeCount(const KhsSolver *s) { return s ? uint32_t(s->model.nodes()) : 0; }

KHS_API KhsResult khsCopyOriginalPositions(const KhsSolver *s, KhsVec3 *positions, uint32_t capacity)
{
    if (!s) return KHS_ERROR_INVALID_ARGUMENT;
    if (!s->built || !s->engine || !positions || capacity < s->model.mapping.size()) return KHS_ERROR_INVALID_ARGUMENT;
    try { return s->engine->copy_original_positions(positions, capacity); } catch (...) { return KHS_ERROR_INTERNAL; }
}

KHS_API KhsResult khsCopyInternalPositions(const KhsSolver *s, KhsVec3 *positions, uint32_t capacity)
{
    if (!s) return KHS_ERROR_INVALID_ARGUMENT;
    if (!s->built || !s->engine || !positions || capacity < s->model.nodes()) return KHS_ERROR_INVALID_ARGUMENT;
    try { return s->engine->copy_internal_positions(positions, capacity); } catch (...) { return KHS_ERROR_INTERNAL; }
}

KHS_API KhsResult khsCopyOriginalToInternalMap(const KhsSolver *s, uint32_t *indices, uint32_t capacity)
{
    if (!s) return KHS_ERROR_INVALID_ARGUMENT;
    if (!s->built || !indices || capacity < s->model.mapping.size()) return KHS_ERROR_INVALID_ARGUMENT;
    std::copy(s->model.mapping.begin(), s->model.mapping.end(), indices);
    return KHS_OK;
}

KHS_API KhsResult khsGetBuildStats(const KhsSolver *s, KhsBuildStats *stats)
{
    if (!s) return KHS_ERROR_INVALID_ARGUMENT;
    if (!s->built || !stats || stats->struct_size < sizeof(KhsBuildStats)) return KHS_ERROR_INVALID_ARGUMENT;
    *stats = s->build_stats;
    return KHS_OK;
}

KHS_API KhsResult khsGetLastStepStats(const KhsSolver *s, KhsStepStats *stats)
{
    if (!s) return KHS_ERROR_INVALID_ARGUMENT;
    if (!stats || stats->struct_size < sizeof(KhsStepStats)) return KHS_ERROR_INVALID_ARGUMENT;
    *stats = s->step_stats;
    return KHS_OK;
}

KHS_API KhsResult khsGetGpuStats(const KhsSolver *s, KhsGpuStats *stats)
{
    if (!s) return KHS_ERROR_INVALID_ARGUMENT;
    if (!s->engine || !stats || stats->struct_size < sizeof(KhsGpuStats)) return KHS_ERROR_INVALID_ARGUMENT;
    *stats = s->engine->gpu_stats();
    return KHS_OK;
}

KHS_API KhsResult khsGetProgress(const KhsSolver *s, KhsProgress *progress)
{
    if (!s) return KHS_ERROR_INVALID_ARGUMENT;
    if (!s->engine || !progress || progress->struct_size < sizeof(KhsProgress)) return KHS_ERROR_INVALID_ARGUMENT;
    *progress = s->engine->progress();
    return KHS_OK;
}

KHS_API KhsResult khsGetFailureDiagnostics(const KhsSolver *s, KhsFailureDiagnostics *diagnostics)
{
    if (!s) return KHS_ERROR_INVALID_ARGUMENT;
    if (!s->engine || !diagnostics || diagnostics->struct_size < sizeof(KhsFailureDiagnostics))
        return KHS_ERROR_INVALID_ARGUMENT;
    *diagnostics = s->engine->failure_diagnostics();
    return KHS_OK;
}

KHS_API KhsResult khsRequestCancel(KhsSolver *s)
{
    return guarded(s, [&] {
        if (!s->engine) return KHS_ERROR_INVALID_STATE;
        s->engine->request_cancel();
        return KHS_OK;
    });
}

KHS_API const char *khsGetLastError(const KhsSolver *s)
{
    static const char *none = "no hair solver";
    return s ? s->error.c_str() : none;
}

// ---- extensions ----------------------------------------------------------

KHS_API KhsResult khsxSetSolveMode(KhsSolver *s, uint32_t mode)
{
    if (!s || mode > KHSX_MODE_MIXED_FF) return KHS_ERROR_INVALID_ARGUMENT;
    s->mode = mode;
    if (s->engine) s->engine->set_mode(mode);
    return KHS_OK;
}

KHS_API uint32_t khsxGetSolveMode(const KhsSolver *s) { return s ? s->mode : 0; }

KHS_API KhsResult khsxSetSubstepLimit(KhsSolver *s, uint32_t substeps)
{
    if (!s) return KHS_ERROR_INVALID_ARGUMENT;
    s->substep_limit = substeps;
    if (s->engine) s->engine->set_substep_limit(substeps);
    return KHS_OK;
}

KHS_API KhsResult khsxSetRollbackRing(KhsSolver *s, uint32_t slots)
{
    return guarded(s, [&] {
        if (!s->built || !s->engine) return KHS_ERROR_INVALID_STATE;
        const KhsResult r = s->engine->set_rollback_ring(slots);
        if (r != KHS_OK) s->error = s->engine->last_error();
        return r;
    });
}

KHS_API KhsResult khsxRollbackToFrame(KhsSolver *s, uint32_t frame)
{
    return guarded(s, [&] {
        if (!s->built || !s->engine) return KHS_ERROR_INVALID_STATE;
        const KhsResult r = s->engine->rollback_to_frame(frame);
        if (r != KHS_OK) s->error = s->engine->last_error();
        return r;
    });
}

KHS_API KhsResult khsxSetOutputRing(KhsSolver *s, uint32_t slots)
{
    return guarded(s, [&] {
        if (!s->built || !s->engine) return KHS_ERROR_INVALID_STATE;
        return s->from_engine(s->engine->set_output_ring(slots));
    });
}

KHS_API KhsResult khsxCopyOutputFrame(KhsSolver *s, uint32_t frame, KhsVec3 *positions, uint32_t capacity)
{
    return guarded(s, [&] {
        if (!s->built || !s->engine) return KHS_ERROR_INVALID_STATE;
        if (!positions) return KHS_ERROR_INVALID_ARGUMENT;
        return s->from_engine(s->engine->output_frame(frame, positions, capacity, nullptr));
    });
}

KHS_API KhsResult khsxMapOutputFrame(KhsSolver *s, uint32_t frame, const KhsVec3 **positions)
{
    return guarded(s, [&] {
        if (!s->built || !s->engine) return KHS_ERROR_INVALID_STATE;
        if (!positions) return KHS_ERROR_INVALID_ARGUMENT;
        *positions = nullptr;
        return s->from_engine(s->engine->output_frame(frame, nullptr, 0, positions));
    });
}

KHS_API KhsResult khsxSetBlockSolveSchedule(KhsSolver *s, uint32_t strands_per_warp, uint32_t blocks_per_sm,
                                            uint32_t long_strands)
{
    return guarded(s, [&] {
        if (!s->built || !s->engine) return KHS_ERROR_INVALID_STATE;
        return s->engine->set_block_solve_schedule(strands_per_warp, blocks_per_sm, long_strands);
    });
}

KHS_API KhsResult khsxSetBlockSolveTiers(KhsSolver *s, uint32_t quads, uint32_t singles, uint32_t doubles,
                                         uint32_t blocks_per_sm)
{
    return guarded(s, [&] {
        if (!s->built || !s->engine) return KHS_ERROR_INVALID_STATE;
        return s->engine->set_block_solve_tiers(quads, singles, doubles, blocks_per_sm);
    });
}

KHS_API KhsResult khsxCopyState(const KhsSolver *s, double *q, double *v, uint64_t dof_capacity)
{
    if (!s || !s->built || !s->engine) return KHS_ERROR_INVALID_ARGUMENT;
    try { return s->engine->copy_state(q, v, dof_capacity); } catch (...) { return KHS_ERROR_INTERNAL; }
}

KHS_API uint32_t khsxGetSubstepRecordCount(const KhsSolver *s)
{
    return s && s->engine ? uint32_t(s->engine->substep_records().size()) : 0;
}

KHS_API KhsResult khsxCopySubstepRecords(const KhsSolver *s, KhsxSubstepRecord *records, uint32_t capacity)
{
    if (!s || !s->engine) return KHS_ERROR_INVALID_ARGUMENT;
    const auto &r = s->engine->substep_records();
    if (!records || capacity < r.size()) return r.empty() ? KHS_OK : KHS_ERROR_INVALID_ARGUMENT;
    std::copy(r.begin(), r.end(), records);
    return KHS_OK;
}

KHS_API KhsResult khsxCopyContactRecords(const KhsSolver *s, KhsxContactRecord *records, uint32_t capacity)
{
    if (!s || !s->built || !s->engine) return KHS_ERROR_INVALID_ARGUMENT;
    try { return s->engine->copy_contact_records(records, capacity); } catch (...) { return KHS_ERROR_INTERNAL; }
}

KHS_API KhsResult khsxQueryContacts(KhsSolver *s, const double *q, uint64_t dof_count, KhsxContactRecord *records,
                                    uint32_t capacity)
{
    return guarded(s, [&] {
        if (!s->built || !s->engine) return KHS_ERROR_INVALID_STATE;
        return s->engine->query_contacts(q, dof_count, records, capacity);
    });
}

KHS_API KhsResult khsxQueryContactsNoAlloc(KhsSolver *s, const double *q, uint64_t dof_count,
                                           KhsxContactRecord *records, uint32_t capacity)
{
    if (!s) return KHS_ERROR_INVALID_ARGUMENT;
    if (!s->built || !s->engine) return KHS_ERROR_INVALID_STATE;
    return s->engine->query_contacts_no_alloc(q, dof_count, records, capacity);
}

KHS_API KhsResult khsxComputeRootTargets(KhsSolver *s, const KhsVec3 *points, uint32_t point_count, KhsVec3 *positions,
                                         KhsVec3 *rotations, uint32_t node_capacity)
{
    return guarded(s, [&] {
        const KhsResult c = s->check_root_points(points, point_count, KHS_ERROR_INVALID_HAIR, KHS_ERROR_INVALID_ARGUMENT);
        if (c != KHS_OK) return c;
        if (!positions || !rotations || node_capacity < s->model.nodes()) {
            s->error = "the root target output arrays are smaller than the internal node count";
            return KHS_ERROR_INVALID_ARGUMENT;
        }
        return s->from_engine(s->engine->root_targets_to_host(points, point_count, positions, rotations));
    });
}

KHS_API KhsResult khsxSetProfiling(KhsSolver *s, uint32_t enable)
{
    return guarded(s, [&] {
        if (!s->engine) return KHS_ERROR_INVALID_STATE;
        s->engine->set_profiling(enable != 0);
        return KHS_OK;
    });
}

KHS_API uint32_t khsxGetKernelTimings(const KhsSolver *s, KhsxKernelTiming *timings, uint32_t capacity)
{
    if (!s || !s->engine) return 0;
    try {
        const auto t = s->engine->kernel_timings();
        for (uint32_t k = 0; k < capacity && k < t.size(); ++k) {
            std::memset(&timings[k], 0, sizeof(KhsxKernelTiming));
            std::strncpy(timings[k].name, t[k].name, sizeof(timings[k].name) - 1);
            timings[k].launches = t[k].launches;
            timings[k].total_milliseconds = t[k].milliseconds;
        }
        return uint32_t(t.size());
    } catch (...) {
        return 0;
    }
}

KHS_API KhsResult khsxResetKernelTimings(KhsSolver *s)
{
    return guarded(s, [&] {
        if (!s->engine) return KHS_ERROR_INVALID_STATE;
        s->engine->reset_kernel_timings();
        return KHS_OK;
    });
}

KHS_API uint64_t khsxGetKernelLaunchCount(const KhsSolver *s) { return s && s->engine ? s->engine->kernel_launches() : 0; }

KHS_API KhsResult khsxMeasurePipePeaks(double *fp64_tflops, double *fp32_tflops)
{
    if (!fp64_tflops || !fp32_tflops) return KHS_ERROR_INVALID_ARGUMENT;
    try {
        std::string error;
        return khs::measure_pipe_peaks(*fp64_tflops, *fp32_tflops, error) ? KHS_OK : KHS_ERROR_INVALID_STATE;
    } catch (...) {
        return KHS_ERROR_INTERNAL;
    }
}

}  // extern "C"
