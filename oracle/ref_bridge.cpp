// ORACLE — test infrastructure only: a flat C API over the reference's own
// FP64 CUDA backend (kami::CudaBackend, reference src/cuda_backend.hpp:42-88),
// so tests can step the unmodified reference solver on a GB300 and compare it
// with the CPU oracle and the product library.
//
// The reference's host layer (src/solver.cpp, src/api.cpp) needs Eigen, which
// is not available, so the model it would build is taken from the CPU
// oracle's builder (khsOracleExportModel), whose output restates
// solver.cpp:227-447, and handed to the backend exactly as
// Solver::build() does (solver.cpp:485-519).  Root targets come from the
// oracle's khsxComputeRootTargets (solver.cpp:416-447).  Everything after
// initialize() is the reference's own code: run_frame, optimize_substep and
// every kernel of cuda_backend.cu, compiled unchanged for sm_103a.
//
// Built by `make -C oracle ref` into oracle/_ref/libkhs_ref.so from the
// staged reference sources (`make -C oracle stage-ref REFERENCE=<path>`).
// Nothing in the product links or loads this library.
#include "cuda_backend.hpp"

#include <cstring>
#include <exception>
#include <memory>
#include <string>
#include <vector>

namespace {

struct RefSolver {
    std::unique_ptr<kami::CudaBackend> backend;
    std::string error;
};

template<class F> int guarded(RefSolver *s, F &&f)
{
    if (!s || !s->backend) return KHS_ERROR_INVALID_STATE;
    try {
        const KhsResult r = f();
        if (r != KHS_OK) s->error = s->backend->last_error();
        return int(r);
    } catch (const std::exception &e) {
        s->error = e.what();
        return KHS_ERROR_INTERNAL;
    } catch (...) {
        s->error = "unknown exception";
        return KHS_ERROR_INTERNAL;
    }
}

std::vector<KhsVec3> vec3s(const KhsVec3 *p, uint32_t n) { return std::vector<KhsVec3>(p, p + n); }

}  // namespace

extern "C" {

__attribute__((visibility("default"))) void *khsRefCreate(
    const KhsSolverDesc *desc, const KhsHairMaterial *material, const uint32_t *sizes, const double *node_f,
    const uint32_t *node_u, const double *elem_f, const uint32_t *elem_u, const uint32_t *strand_u,
    const uint32_t *mapping, const double *collider, const uint32_t *tris, int *result, char *error,
    uint32_t error_capacity)
{
    auto report = [&](int r, const std::string &msg) -> void * {
        if (result) *result = r;
        if (error && error_capacity) {
            std::strncpy(error, msg.c_str(), error_capacity - 1);
            error[error_capacity - 1] = 0;
        }
        return nullptr;
    };
    if (!desc || !material || !sizes) return report(KHS_ERROR_INVALID_ARGUMENT, "null argument");
    try {
        const uint32_t N = sizes[0], E = sizes[1], S = sizes[2], P = sizes[3], V = sizes[4], T = sizes[5];
        std::vector<kami::CudaNodeInit> nodes(N);
        for (uint32_t i = 0; i < N; ++i) {
            const double *f = node_f + 18 * size_t(i);
            const uint32_t *u = node_u + 4 * size_t(i);
            kami::CudaNodeInit &n = nodes[i];
            n.position = {f[0], f[1], f[2]};
            n.rotation = {f[3], f[4], f[5]};
            for (int row = 0; row < 3; ++row) n.reference[row] = {f[6 + 3 * row], f[7 + 3 * row], f[8 + 3 * row]};
            n.mass = f[15];
            n.rotational_mass = f[16];
            n.binding_t = f[17];
            n.strand = u[0];
            n.binding_left = u[1];
            n.binding_right = u[2];
            n.fixed = u[3] != 0;
        }
        std::vector<kami::CudaElementInit> elements(E);
        for (uint32_t e = 0; e < E; ++e) {
            const double *f = elem_f + 7 * size_t(e);
            const uint32_t *u = elem_u + 4 * size_t(e);
            elements[e] = {u[0], u[1], u[2], u[3], f[0], {f[1], f[2], f[3]}, {f[4], f[5], f[6]}};
        }
        std::vector<std::vector<uint32_t>> strand_nodes(S);
        for (uint32_t s = 0; s < S; ++s)
            for (uint32_t k = 0; k < strand_u[2 * s + 1]; ++k) strand_nodes[s].push_back(strand_u[2 * s] + k);
        std::vector<uint32_t> map(mapping, mapping + P);
        std::vector<KhsVec3> verts(V);
        for (uint32_t v = 0; v < V; ++v) verts[v] = {collider[3 * v], collider[3 * v + 1], collider[3 * v + 2]};
        std::vector<kami::CudaTriangleInit> triangles(T);
        for (uint32_t t = 0; t < T; ++t) triangles[t] = {tris[3 * t], tris[3 * t + 1], tris[3 * t + 2]};

        auto s = std::make_unique<RefSolver>();
        s->backend = kami::make_cuda_backend();
        if (!s->backend) return report(KHS_ERROR_INVALID_STATE, "the reference CUDA backend could not be created");
        const KhsResult r = s->backend->initialize(*desc, *material, nodes, elements, strand_nodes, map, verts, triangles);
        if (r != KHS_OK) return report(r, s->backend->last_error());
        if (result) *result = KHS_OK;
        return s.release();
    } catch (const std::exception &e) {
        return report(KHS_ERROR_INTERNAL, e.what());
    }
}

__attribute__((visibility("default"))) void khsRefDestroy(void *h) { delete static_cast<RefSolver *>(h); }

__attribute__((visibility("default"))) const char *khsRefLastError(void *h)
{
    return h ? static_cast<RefSolver *>(h)->error.c_str() : "";
}

__attribute__((visibility("default"))) int khsRefAllocateAnimation(void *h, uint32_t frames)
{
    auto *s = static_cast<RefSolver *>(h);
    return guarded(s, [&] { return s->backend->allocate_animation(frames); });
}

__attribute__((visibility("default"))) int khsRefSetRootAnimationFrame(void *h, uint32_t frame, const KhsVec3 *pos,
                                                                       const KhsVec3 *rot, uint32_t n)
{
    auto *s = static_cast<RefSolver *>(h);
    return guarded(s, [&] { return s->backend->set_root_animation_frame(frame, vec3s(pos, n), vec3s(rot, n)); });
}

__attribute__((visibility("default"))) int khsRefSetColliderAnimationFrame(void *h, uint32_t frame, const KhsVec3 *v,
                                                                           uint32_t n)
{
    auto *s = static_cast<RefSolver *>(h);
    return guarded(s, [&] { return s->backend->set_collider_animation_frame(frame, v, n); });
}

__attribute__((visibility("default"))) int khsRefFinalizeAnimation(void *h)
{
    auto *s = static_cast<RefSolver *>(h);
    return guarded(s, [&] { return s->backend->finalize_animation(); });
}

__attribute__((visibility("default"))) int khsRefStepAnimationFrame(void *h, uint32_t frame, double dt)
{
    auto *s = static_cast<RefSolver *>(h);
    return guarded(s, [&] { return s->backend->step_animation_frame(frame, dt); });
}

__attribute__((visibility("default"))) int khsRefUpdateRoots(void *h, const KhsVec3 *pos, const KhsVec3 *rot,
                                                             uint32_t n)
{
    auto *s = static_cast<RefSolver *>(h);
    return guarded(s, [&] { return s->backend->update_roots(vec3s(pos, n), vec3s(rot, n)); });
}

__attribute__((visibility("default"))) int khsRefUpdateCollider(void *h, const KhsVec3 *v, uint32_t n)
{
    auto *s = static_cast<RefSolver *>(h);
    return guarded(s, [&] { return s->backend->update_collider(v, n); });
}

__attribute__((visibility("default"))) int khsRefStep(void *h, double dt)
{
    auto *s = static_cast<RefSolver *>(h);
    return guarded(s, [&] { return s->backend->step(dt); });
}

__attribute__((visibility("default"))) uint64_t khsRefCheckpointSize(void *h)
{
    auto *s = static_cast<RefSolver *>(h);
    return s && s->backend ? s->backend->animation_checkpoint_size() : 0;
}

__attribute__((visibility("default"))) int khsRefSaveCheckpoint(void *h, void *data, uint64_t capacity)
{
    auto *s = static_cast<RefSolver *>(h);
    return guarded(s, [&] { return s->backend->save_animation_checkpoint(data, capacity); });
}

__attribute__((visibility("default"))) int khsRefRestoreCheckpoint(void *h, const void *data, uint64_t size)
{
    auto *s = static_cast<RefSolver *>(h);
    return guarded(s, [&] { return s->backend->restore_animation_checkpoint(data, size); });
}

__attribute__((visibility("default"))) int khsRefCopyOriginalPositions(void *h, KhsVec3 *out, uint32_t capacity)
{
    auto *s = static_cast<RefSolver *>(h);
    return guarded(s, [&] { return s->backend->copy_original_positions(out, capacity); });
}

__attribute__((visibility("default"))) int khsRefStats(void *h, KhsStepStats *out)
{
    auto *s = static_cast<RefSolver *>(h);
    if (!out || out->struct_size < sizeof(KhsStepStats)) return KHS_ERROR_INVALID_ARGUMENT;
    return guarded(s, [&] { *out = s->backend->stats(); return KHS_OK; });
}

__attribute__((visibility("default"))) int khsRefGpuStats(void *h, KhsGpuStats *out)
{
    auto *s = static_cast<RefSolver *>(h);
    if (!out || out->struct_size < sizeof(KhsGpuStats)) return KHS_ERROR_INVALID_ARGUMENT;
    return guarded(s, [&] { *out = s->backend->gpu_stats(); return KHS_OK; });
}

__attribute__((visibility("default"))) int khsRefFailure(void *h, KhsFailureDiagnostics *out)
{
    auto *s = static_cast<RefSolver *>(h);
    if (!out || out->struct_size < sizeof(KhsFailureDiagnostics)) return KHS_ERROR_INVALID_ARGUMENT;
    return guarded(s, [&] { *out = s->backend->failure_diagnostics(); return KHS_OK; });
}

__attribute__((visibility("default"))) int khsRefProgress(void *h, KhsProgress *out)
{
    auto *s = static_cast<RefSolver *>(h);
    if (!out || out->struct_size < sizeof(KhsProgress)) return KHS_ERROR_INVALID_ARGUMENT;
    return guarded(s, [&] { *out = s->backend->progress(); return KHS_OK; });
}

__attribute__((visibility("default"))) int khsRefCancel(void *h)
{
    auto *s = static_cast<RefSolver *>(h);
    return guarded(s, [&] { s->backend->request_cancel(); return KHS_OK; });
}

}  // extern "C"
