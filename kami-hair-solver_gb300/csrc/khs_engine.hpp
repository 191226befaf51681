// GB300 device engine: owns every device-resident array of one solver and
// runs frames of adaptive substeps.  Host control flow follows the
// reference's run_frame / optimize_substep (src/cuda_backend.cu:604-723);
// every stage is a hand-written sm_103a kernel (khs_engine.cu) and the
// cuBLAS level-1 calls of the reference are replaced by deterministic
// fixed-order block reductions.
#pragma once

#include "khs_model.hpp"
#include "kami_hair_solver.h"

#include <atomic>
#include <chrono>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

namespace khs {

struct EvalStats {
    double objective = 0, elastic = 0, contact = 0, kinetic = 0, minimum_gap = 0, grad_norm2 = 0;
    uint64_t candidates = 0, active = 0;
    int feasible = 1;
};

struct KernelTiming {
    const char *name;
    uint64_t launches;
    double milliseconds;
};

class Engine {
public:
    Engine();
    ~Engine();
    Engine(const Engine &) = delete;
    Engine &operator=(const Engine &) = delete;

    // Uploads the built model.  Throws std::runtime_error on CUDA errors.
    void initialize(const Model &model, const KhsSolverDesc &desc, const KhsHairMaterial &material,
                    const std::vector<Vec> &root_pos, const std::vector<Vec> &root_rot);
    void update_runtime(const KhsSolverDesc &desc, const KhsHairMaterial &material, const std::vector<double> &mass,
                        const std::vector<double> &rotational_mass);
    // Root targets of every node (positions and rotation vectors) for the
    // evaluated source points, computed on the device (solver.cpp:416-447):
    // into the pending targets of the next step, into an animation frame, or
    // back to the host.  The points must be finite; a degenerate tangent
    // gives KHS_ERROR_INVALID_HAIR and changes nothing.
    KhsResult set_pending_root_points(const KhsVec3 *points, uint32_t count);
    KhsResult root_targets_to_host(const KhsVec3 *points, uint32_t count, KhsVec3 *positions, KhsVec3 *rotations);
    void set_pending_collider(const std::vector<Vec> &vertices);

    KhsResult allocate_animation(uint32_t frames);
    KhsResult set_root_animation_frame(uint32_t frame, const KhsVec3 *points, uint32_t count);
    KhsResult set_collider_animation_frame(uint32_t frame, const KhsVec3 *vertices, uint32_t count);
    KhsResult finalize_animation();

    KhsResult step(double frame_dt);
    KhsResult step_animation_frame(uint32_t frame, double frame_dt);

    uint64_t checkpoint_size() const;
    KhsResult save_checkpoint(void *data, uint64_t capacity);
    KhsResult restore_checkpoint(const void *data, uint64_t size);
    // Device-resident rollback ring of the last `slots` animation frames
    // (q and v), filled after every successful animation frame.
    KhsResult set_rollback_ring(uint32_t slots);
    KhsResult rollback_to_frame(uint32_t frame);
    // Pinned output ring of the last `slots` animation frames' original-point
    // positions, copied from the device on a second stream after every frame
    // (0 turns it off).  output_frame waits for the frame's copy, then copies
    // it to `out` (capacity >= the point count) and/or returns a view of the
    // pinned slot, valid until `slots` more frames are stepped.
    KhsResult set_output_ring(uint32_t slots);
    KhsResult output_frame(uint32_t frame, KhsVec3 *out, uint32_t capacity, const KhsVec3 **view);

    KhsResult copy_original_positions(KhsVec3 *out, uint32_t capacity) const;
    KhsResult copy_internal_positions(KhsVec3 *out, uint32_t capacity) const;
    KhsResult copy_state(double *q, double *v, uint64_t capacity) const;
    KhsResult copy_contact_records(KhsxContactRecord *out, uint32_t capacity) const;
    // Contact classification of every element at the given positions
    // (6 * N values) against the current collider.
    KhsResult query_contacts(const double *q, uint64_t dof, KhsxContactRecord *out, uint32_t capacity);
    // The same query through a file-scope device scratch array: allocates
    // nothing, leaves the solver's contact records alone, never throws.
    KhsResult query_contacts_no_alloc(const double *q, uint64_t dof, KhsxContactRecord *out, uint32_t capacity);

    void set_mode(uint32_t mode) { mode_ = mode; }
    // Ends every frame after its first `substeps` substeps (0: whole frames).
    void set_substep_limit(uint32_t substeps) { substep_limit_ = substeps; }
    // Block-solve launch shape: 5, 2 or 1 strands per warp and blocks of four
    // warps per SM (long_strands > 0 with 5: the longest strands one per
    // warp first); 0 strands per warp restores the one-time tuning.
    KhsResult set_block_solve_schedule(uint32_t strands_per_warp, uint32_t blocks_per_sm, uint32_t long_strands);
    KhsResult set_block_solve_tiers(uint32_t quads, uint32_t singles, uint32_t doubles, uint32_t blocks_per_sm);
    uint32_t mode() const { return mode_; }

    KhsStepStats stats() const { return step_stats_; }
    KhsGpuStats gpu_stats() const { return gpu_stats_; }
    KhsProgress progress() const;
    KhsFailureDiagnostics failure_diagnostics() const { return failure_; }
    const std::vector<KhsxSubstepRecord> &substep_records() const { return records_; }
    void request_cancel() { cancel_.store(true); }
    const std::string &last_error() const { return error_; }

    // Number of kernels this engine has launched (for launch accounting).
    uint64_t kernel_launches() const;
    // Per-kernel CUDA-event timing on the engine's stream.
    void set_profiling(bool on);
    std::vector<KernelTiming> kernel_timings() const;
    void reset_kernel_timings();

private:
    struct Impl;
    std::unique_ptr<Impl> d_;

    KhsResult fail(KhsResult r, const std::string &message);
    KhsResult run_root_pass(const KhsVec3 *points, uint32_t count);
    void push_output(uint32_t frame);
    void drop_outputs_after(uint32_t frame);
    void clear_failure();
    void set_failure_context(uint32_t kind, uint32_t frame, uint32_t sub, uint32_t attempted, uint32_t maximum,
                             uint32_t attempts);
    KhsResult run_frame(double frame_dt, const double *root_a, const double *rot_a, const double *root_b,
                        const double *rot_b, const double *collider_a, const double *collider_b, uint32_t frame,
                        uint32_t frame_count);
    KhsResult optimize_substep(double dt, KhsxSubstepRecord &rec);
    EvalStats evaluate(bool gradient, double dt, double alpha_for_trial, const double *alpha_dev = nullptr);
    bool make_direction(KhsxSubstepRecord &rec, double grad_norm2);
    void tune_block_solve();
    void launch_block_solve();
    void launch_ccd_bound();
    void push_ring(uint32_t frame);
    // Both return whether the trust radius scaled the direction.
    bool make_steepest();
    bool limit_direction(double max_translation);

    KhsSolverDesc desc_{};
    KhsHairMaterial material_{};
    uint32_t mode_ = 0, substep_limit_ = 0;
    bool initialized_ = false, animation_ready_ = false;
    uint32_t animation_frames_ = 0, current_frame_ = 0;
    std::vector<bool> root_frame_set_, collider_frame_set_;
    double trust_radius_ = 0.0, max_rest_length_ = 0.0, last_dt_ = 0.0;
    bool rebuild_cache_ = true;  // mixed form: recollect contact leaves at the next evaluation
    KhsStepStats step_stats_{};
    KhsGpuStats gpu_stats_{};
    KhsFailureDiagnostics failure_{};
    std::vector<KhsxSubstepRecord> records_;
    std::string error_;
    std::atomic<bool> cancel_{false};
    std::atomic<uint32_t> progress_phase_{KHS_PHASE_IDLE}, progress_frame_{0}, progress_frame_count_{0},
        progress_substep_{0}, progress_substep_count_{0}, progress_iteration_{0};
    std::chrono::steady_clock::time_point frame_clock_ = std::chrono::steady_clock::now();
};

bool query_device(KhsGpuInfo &info, std::string &error);
bool measure_pipe_peaks(double &fp64_tflops, double &fp32_tflops, std::string &error);

}  // namespace khs
