/*
 * kami_hair_solver.h — C ABI of the GB300-native Cosserat hair solver.
 *
 * This header is a drop-in replacement for the reference library's public
 * header (include/kami_hair_solver.h, ABI version 5).  Every type below has
 * the same field order, field types and therefore the same size/offsets as the
 * reference ABI, so a caller compiled against the reference header (the
 * Blender ctypes binding, C/C++ hosts) can load this library unchanged.  The
 * layout equality is asserted by tests/test_abi_layout.py against an
 * independent ctypes mirror of the reference structs.
 *
 * Each function carries the reference declaration it replaces
 * (kami_hair_solver.h:<line>) and the reference implementation whose
 * argument meaning and error behaviour it follows (api.cpp:<line>).
 *
 * Additive GB300 extensions (not present in the reference) are declared at
 * the end with the khsx prefix; they never change a v5 struct.
 */
#ifndef KAMI_HAIR_SOLVER_H
#define KAMI_HAIR_SOLVER_H

#include <stddef.h>
#include <stdint.h>

#if defined(_WIN32)
#  if defined(KHS_BUILD_DLL)
#    define KHS_API __declspec(dllexport)
#  else
#    define KHS_API __declspec(dllimport)
#  endif
#else
#  define KHS_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* kami_hair_solver.h:21 */
#define KHS_ABI_VERSION 5u

/* Opaque solver handle (kami_hair_solver.h:23). */
typedef struct KhsSolver KhsSolver;

/* World-space point, metres, FP64 (kami_hair_solver.h:25-29). */
typedef struct KhsVec3 {
    double x;
    double y;
    double z;
} KhsVec3;

/* Collider triangle as three vertex indices (kami_hair_solver.h:31-35). */
typedef struct KhsTriangle {
    uint32_t i0;
    uint32_t i1;
    uint32_t i2;
} KhsTriangle;

/* Result codes (kami_hair_solver.h:37-48). */
typedef enum KhsResult {
    KHS_OK = 0,
    KHS_ERROR_INVALID_ARGUMENT = 1,
    KHS_ERROR_INVALID_STATE = 2,
    KHS_ERROR_INVALID_HAIR = 3,
    KHS_ERROR_INVALID_COLLIDER = 4,
    KHS_ERROR_INITIAL_INTERSECTION = 5,
    KHS_ERROR_NOT_CONVERGED = 6,
    KHS_ERROR_NUMERICAL_FAILURE = 7,
    KHS_ERROR_OUT_OF_MEMORY = 8,
    KHS_ERROR_INTERNAL = 9
} KhsResult;

/* Phase reported by progress/step stats (kami_hair_solver.h:50-59). */
typedef enum KhsProgressPhase {
    KHS_PHASE_IDLE = 0,
    KHS_PHASE_PREPARING = 1,
    KHS_PHASE_ASSEMBLING = 2,
    KHS_PHASE_LINEAR_SOLVE = 3,
    KHS_PHASE_CCD = 4,
    KHS_PHASE_LINE_SEARCH = 5,
    KHS_PHASE_FINISHED = 6,
    KHS_PHASE_FAILED = 7
} KhsProgressPhase;

/* Solver configuration (kami_hair_solver.h:61-78). */
typedef struct KhsSolverDesc {
    uint32_t struct_size;
    KhsVec3 gravity;
    uint32_t substeps;
    uint32_t maximum_substeps;
    uint32_t newton_iterations;
    uint32_t line_search_iterations;
    double absolute_tolerance;
    double relative_tolerance;
    double increment_tolerance;
    double minimum_line_search_step;
    double minimum_gap;
    double maximum_element_length;
    /* 0 disables it.  Strands whose rest length is shorter are extended along
       the tip tangent by invisible nodes up to this rest length. */
    double minimum_dynamic_length;
    uint32_t fixed_root_nodes;
    uint32_t thread_count;
} KhsSolverDesc;

/* Rod material and contact parameters (kami_hair_solver.h:80-93). */
typedef struct KhsHairMaterial {
    uint32_t struct_size;
    double density;
    double radius;
    double young_modulus;
    double poisson_ratio;
    double shear_correction;
    double mass_damping;
    double contact_stiffness;
    double barrier_distance;
    double friction;
    double friction_smoothing;
    double collider_offset;
} KhsHairMaterial;

/* Build-time counters (kami_hair_solver.h:95-116). */
typedef struct KhsBuildStats {
    uint32_t struct_size;
    uint32_t strand_count;
    uint32_t original_point_count;
    uint32_t internal_node_count;
    uint32_t element_count;
    uint32_t fixed_node_count;
    uint32_t collider_vertex_count;
    uint32_t collider_triangle_count;
    uint32_t excluded_collider_triangle_count;
    uint32_t collider_boundary_edge_count;
    uint32_t collider_nonmanifold_edge_count;
    uint32_t collider_inconsistent_edge_count;
    uint32_t collider_inverted_closed_component_count;
    uint32_t merged_zero_length_segment_count;
    uint32_t virtual_extension_strand_count;
    uint32_t virtual_extension_node_count;
    double virtual_extension_rest_length;
    uint64_t degree_of_freedom_count;
    uint64_t estimated_bytes;
    double initial_minimum_gap;
} KhsBuildStats;

/* Per-frame solve counters (kami_hair_solver.h:118-140). */
typedef struct KhsStepStats {
    uint32_t struct_size;
    uint32_t substeps;
    uint32_t converged_substeps;
    uint32_t newton_iterations;
    uint32_t linear_solves;
    uint32_t line_search_evaluations;
    uint64_t contact_candidate_count;
    uint64_t active_contact_count;
    double initial_residual_norm;
    double final_residual_norm;
    double relative_residual_norm;
    double increment_norm;
    double objective_change;
    double minimum_gap;
    double accepted_step_length;
    double ccd_step_limit;
    double kinetic_energy;
    double elastic_energy;
    double contact_energy;
    double friction_energy;
    KhsProgressPhase phase;
} KhsStepStats;

/* Device description (kami_hair_solver.h:142-150). */
typedef struct KhsGpuInfo {
    uint32_t struct_size;
    uint32_t available;
    int32_t device_ordinal;
    uint32_t compute_capability_major;
    uint32_t compute_capability_minor;
    uint64_t total_vram_bytes;
    char device_name[128];
} KhsGpuInfo;

/* Device residency and timing (kami_hair_solver.h:152-161). */
typedef struct KhsGpuStats {
    uint32_t struct_size;
    uint32_t animation_frame_count;
    uint64_t resident_bytes;
    uint64_t peak_temporary_bytes;
    double last_frame_milliseconds;
    double last_assembly_milliseconds;
    double last_collision_milliseconds;
    double last_optimization_milliseconds;
} KhsGpuStats;

/* Cross-thread progress snapshot (kami_hair_solver.h:163-174). */
typedef struct KhsProgress {
    uint32_t struct_size;
    uint32_t phase;
    uint32_t frame_index;
    uint32_t frame_count;
    uint32_t substep;
    uint32_t substep_count;
    uint32_t nonlinear_iteration;
    uint32_t nonlinear_iteration_limit;
    uint32_t cancelled;
    double frame_elapsed_seconds;
} KhsProgress;

/* kami_hair_solver.h:176-181 */
typedef enum KhsFailureKind {
    KHS_FAILURE_NONE = 0,
    KHS_FAILURE_MOVING_COLLIDER_SWEEP = 1,
    KHS_FAILURE_BARRIER_INFEASIBLE = 2,
    KHS_FAILURE_NONLINEAR_SOLVE = 3
} KhsFailureKind;

/* kami_hair_solver.h:183-204 */
typedef struct KhsFailureDiagnostics {
    uint32_t struct_size;
    uint32_t kind;
    uint32_t frame_index;
    uint32_t substep;
    uint32_t requested_substeps;
    uint32_t attempted_substeps;
    uint32_t maximum_substeps;
    uint32_t adaptive_attempt_count;
    uint32_t strand_index;
    uint32_t element_index;
    uint32_t collider_triangle_index;
    uint32_t reserved;
    double distance;
    double required_distance;
    double clearance;
    double collider_substep_displacement;
    double collider_frame_displacement;
    KhsVec3 hair_start;
    KhsVec3 hair_end;
    KhsVec3 collider_point;
} KhsFailureDiagnostics;

/* ---- Version, device, defaults, lifetime --------------------------------- */

/* Replaces kami_hair_solver.h:206 (api.cpp:64). */
KHS_API uint32_t khsGetAbiVersion(void);
/* Replaces kami_hair_solver.h:207 (api.cpp:66-77).  INVALID_STATE without a GPU. */
KHS_API KhsResult khsGetGpuInfo(KhsGpuInfo *info);
/* Replaces kami_hair_solver.h:208 (api.cpp:79-98). */
KHS_API void khsDefaultSolverDesc(KhsSolverDesc *desc);
/* Replaces kami_hair_solver.h:209 (api.cpp:100-116). */
KHS_API void khsDefaultHairMaterial(KhsHairMaterial *material);
/* Replaces kami_hair_solver.h:210 (api.cpp:118-123).  NULL on an invalid desc. */
KHS_API KhsSolver *khsCreate(const KhsSolverDesc *desc);
/* Replaces kami_hair_solver.h:211 (api.cpp:125). */
KHS_API void khsDestroy(KhsSolver *solver);

/* ---- Scene input --------------------------------------------------------- */

/* Replaces kami_hair_solver.h:214-219 (api.cpp:127-135).
   offsets has strand_count + 1 entries, offsets[0] == 0 and the last one is
   point_count.  Inputs are copied before return. */
KHS_API KhsResult khsSetHairCurves(KhsSolver *solver,
                                   const KhsVec3 *points,
                                   uint32_t point_count,
                                   const uint32_t *offsets,
                                   uint32_t strand_count,
                                   const KhsHairMaterial *material);

/* Replaces kami_hair_solver.h:222-226 (api.cpp:137-144).  Zero triangles
   removes the collider; degenerate triangles are excluded at build. */
KHS_API KhsResult khsSetColliderMesh(KhsSolver *solver,
                                     const KhsVec3 *vertices,
                                     uint32_t vertex_count,
                                     const KhsTriangle *triangles,
                                     uint32_t triangle_count);

/* Replaces kami_hair_solver.h:228 (api.cpp:146-149).  Builds the internal rod
   model on the host and uploads it to device-resident SoA arrays. */
KHS_API KhsResult khsBuild(KhsSolver *solver);

/* Replaces kami_hair_solver.h:235-237 (api.cpp:151-158).  Updates numerical
   and material parameters while keeping the state; maximum_element_length,
   minimum_dynamic_length and fixed_root_nodes may not change. */
KHS_API KhsResult khsUpdateRuntimeParameters(KhsSolver *solver,
                                              const KhsSolverDesc *desc,
                                              const KhsHairMaterial *material);

/* Replaces kami_hair_solver.h:240-242 (api.cpp:160-166).  Collider vertices
   that the next khsStep interpolates towards. */
KHS_API KhsResult khsUpdateColliderVertices(KhsSolver *solver,
                                            const KhsVec3 *vertices,
                                            uint32_t vertex_count);

/* Replaces kami_hair_solver.h:245-247 (api.cpp:168-174).  Evaluated source
   curve points that drive the fixed roots of the next khsStep. */
KHS_API KhsResult khsUpdateRootTargets(KhsSolver *solver,
                                       const KhsVec3 *points,
                                       uint32_t point_count);

/* Replaces kami_hair_solver.h:249 (api.cpp:176-179).  One frame of adaptive
   substeps towards the pending root/collider targets. */
KHS_API KhsResult khsStep(KhsSolver *solver, double frame_dt);

/* ---- Device-resident animation ------------------------------------------ */

/* Replaces kami_hair_solver.h:252 (api.cpp:181-184). */
KHS_API KhsResult khsAllocateAnimation(KhsSolver *solver, uint32_t frame_count);
/* Replaces kami_hair_solver.h:253-256 (api.cpp:186-192). */
KHS_API KhsResult khsSetRootAnimationFrame(KhsSolver *solver,
                                           uint32_t frame_index,
                                           const KhsVec3 *points,
                                           uint32_t point_count);
/* Replaces kami_hair_solver.h:257-260 (api.cpp:194-200). */
KHS_API KhsResult khsSetColliderAnimationFrame(KhsSolver *solver,
                                               uint32_t frame_index,
                                               const KhsVec3 *vertices,
                                               uint32_t vertex_count);
/* Replaces kami_hair_solver.h:261 (api.cpp:202-205). */
KHS_API KhsResult khsFinalizeAnimation(KhsSolver *solver);
/* Replaces kami_hair_solver.h:262-264 (api.cpp:207-212).  THE hot entry:
   frame 0 is a no-op, frames must be stepped in increasing order. */
KHS_API KhsResult khsStepAnimationFrame(KhsSolver *solver,
                                        uint32_t frame_index,
                                        double frame_dt);

/* ---- Checkpoints ---------------------------------------------------------- */

/* Replaces kami_hair_solver.h:270 (api.cpp:214-217).  The blob is a 24-byte
   header followed by q[6N] and v[6N] in FP64, per-node interleaved. */
KHS_API uint64_t khsGetAnimationCheckpointSize(const KhsSolver *solver);
/* Replaces kami_hair_solver.h:271-273 (api.cpp:219-224). */
KHS_API KhsResult khsSaveAnimationCheckpoint(KhsSolver *solver,
                                              void *data,
                                              uint64_t capacity);
/* Replaces kami_hair_solver.h:274-276 (api.cpp:226-231). */
KHS_API KhsResult khsRestoreAnimationCheckpoint(KhsSolver *solver,
                                                 const void *data,
                                                 uint64_t size);

/* ---- Readback ------------------------------------------------------------- */

/* Replaces kami_hair_solver.h:278 (api.cpp:233-236). */
KHS_API uint32_t khsGetOriginalPointCount(const KhsSolver *solver);
/* Replaces kami_hair_solver.h:279 (api.cpp:238-241). */
KHS_API uint32_t khsGetInternalNodeCount(const KhsSolver *solver);
/* Replaces kami_hair_solver.h:280-282 (api.cpp:243-248). */
KHS_API KhsResult khsCopyOriginalPositions(const KhsSolver *solver,
                                           KhsVec3 *positions,
                                           uint32_t capacity);
/* Replaces kami_hair_solver.h:283-285 (api.cpp:250-255). */
KHS_API KhsResult khsCopyInternalPositions(const KhsSolver *solver,
                                           KhsVec3 *positions,
                                           uint32_t capacity);
/* Replaces kami_hair_solver.h:286-288 (api.cpp:257-262). */
KHS_API KhsResult khsCopyOriginalToInternalMap(const KhsSolver *solver,
                                               uint32_t *indices,
                                               uint32_t capacity);
/* Replaces kami_hair_solver.h:289-290 (api.cpp:264-268). */
KHS_API KhsResult khsGetBuildStats(const KhsSolver *solver,
                                   KhsBuildStats *stats);
/* Replaces kami_hair_solver.h:291-292 (api.cpp:270-274). */
KHS_API KhsResult khsGetLastStepStats(const KhsSolver *solver,
                                      KhsStepStats *stats);
/* Replaces kami_hair_solver.h:293 (api.cpp:276-280). */
KHS_API KhsResult khsGetGpuStats(const KhsSolver *solver, KhsGpuStats *stats);
/* Replaces kami_hair_solver.h:294 (api.cpp:282-286).  Safe to call from
   another thread while a step runs. */
KHS_API KhsResult khsGetProgress(const KhsSolver *solver, KhsProgress *progress);
/* Replaces kami_hair_solver.h:295-296 (api.cpp:288-293). */
KHS_API KhsResult khsGetFailureDiagnostics(const KhsSolver *solver,
                                            KhsFailureDiagnostics *diagnostics);
/* Replaces kami_hair_solver.h:297 (api.cpp:295-298).  Cooperative; observed
   once per Gauss-Newton iteration.  Safe from another thread. */
KHS_API KhsResult khsRequestCancel(KhsSolver *solver);
/* Replaces kami_hair_solver.h:298 (api.cpp:300-304).  Valid until the next
   mutating call on the same solver. */
KHS_API const char *khsGetLastError(const KhsSolver *solver);

/* ======================================================================== */
/* GB300 extensions (additive; no counterpart in the reference ABI).         */
/* ======================================================================== */

/* Solve forms selectable per solver. */
typedef enum KhsxSolveMode {
    /* Plain FP64 form: the reference method decision for decision, each
       stage a hand-written sm_103a kernel, FP64 throughout. */
    KHSX_MODE_PLAIN_FP64 = 0,
    /* Mixed form: FP32 broadphase (outward-rounded FP32 BVH boxes, exact
       FP64 re-test at the leaves), FP32-filtered narrow phase with a
       converged FP64 pass over the survivors, FP32 CCD / sweep skip tests
       with exact FP64 decisions, exact early termination of the CCD
       advancement.  State, gradient, Gauss-Newton blocks and their
       factorisation, energies, barrier distances and CCD steps stay FP64,
       so its results equal the plain form's bit for bit.  (A plain FP32
       block factorisation does not converge under FP64 refinement for these
       rods: tests/test_fp32_factorization_study.py.) */
    KHSX_MODE_MIXED = 1,
    /* Mixed form with a float-float (two FP32 words, about 48 bits)
       block-tridiagonal factorisation and FP64 iterative refinement on the
       Gauss-Newton residual: sweeps repeat (at most 3) while a strand's
       relative correction exceeds 1e-4; a float-float pivot failure falls
       back to the FP64 factorisation (KhsxSubstepRecord.fp64_fallbacks).
       Directions differ from the plain form's by rounding only. */
    KHSX_MODE_MIXED_FF = 2
} KhsxSolveMode;

/* Selects the solve form.  May be called before or after khsBuild. */
KHS_API KhsResult khsxSetSolveMode(KhsSolver *solver, uint32_t mode);
KHS_API uint32_t khsxGetSolveMode(const KhsSolver *solver);

/* Launch shape of the FP64 block-tridiagonal solve.  By default it is tuned
   once per solver by timing each shape on the first system; this pins it:
   strands_per_warp 5 (6 lanes per strand), 2 (12 lanes per strand, half
   the instructions on each strand's sequential chain) or 1 (18 lanes),
   blocks_per_sm 1-8; long_strands > 0 first gives that many longest
   strands one warp of 18 lanes each (with strands_per_warp 5) or a pair of
   warps each (with strands_per_warp 1: one warp runs the pivot steps on the
   diagonal blocks, the other applies them to the coupling blocks and the
   right-hand side), the rest five per warp.  strands_per_warp 0 restores
   the tuning.  Every shape gives bit-identical directions.
   Requires a built solver. */
KHS_API KhsResult khsxSetBlockSolveSchedule(KhsSolver *solver, uint32_t strands_per_warp, uint32_t blocks_per_sm,
                                            uint32_t long_strands);

/* Tiered launch shape of the FP64 block-tridiagonal solve (the tuner also
   considers it): the `quads` longest strands each on four warps of one
   block (one warp runs the pivot steps on the diagonal blocks, three apply
   them to two columns each of the coupling blocks and the right-hand side
   and form the next Schur complement), the next `singles` strands one per
   warp (18 lanes), the next `doubles` two per warp (12 lanes each), the rest
   five per warp; blocks_per_sm 1-8; quads + singles + doubles must not
   exceed the strand count.  Every shape gives bit-identical directions.
   No counterpart in the reference (its solve is one thread per strand,
   src/cuda_backend.cu:866-881).  Requires a built solver. */
KHS_API KhsResult khsxSetBlockSolveTiers(KhsSolver *solver, uint32_t quads, uint32_t singles, uint32_t doubles,
                                         uint32_t blocks_per_sm);

/* Device-resident rollback ring: the rod state (q and v) after each of the
   last `slots` successful animation frames stays in device memory (2 x 48
   bytes per internal node per slot), so a serving loop can rewind a bake
   without a host round trip.  slots 0 frees the ring.  Setting a ring also
   stores the current frame.  Requires a built solver. */
KHS_API KhsResult khsxSetRollbackRing(KhsSolver *solver, uint32_t slots);

/* Restores q and v of `frame` from the ring (KHS_ERROR_INVALID_ARGUMENT if
   the ring no longer holds it) and makes it the current animation frame;
   later frames are dropped from the ring.  The next khsStepAnimationFrame
   call steps frame + 1. */
KHS_API KhsResult khsxRollbackToFrame(KhsSolver *solver, uint32_t frame);

/* Output ring for baking (replaces the reference add-on's per-frame
   synchronous khsCopyOriginalPositions, addon.py:748-757; the per-frame
   checkpoint it also takes is covered by khsxSetRollbackRing).  After each
   successful khsStepAnimationFrame (frame 0 included) the original points'
   positions are gathered on the device and copied to pinned host memory on
   a second stream, overlapping the next frame; the last `slots` frames are
   kept (24 bytes per point per slot, on the device and pinned on the host).
   slots 0 frees the ring.  Requires a built solver. */
KHS_API KhsResult khsxSetOutputRing(KhsSolver *solver, uint32_t slots);

/* Waits for `frame`'s copy and writes its positions (capacity >= the
   original point count).  KHS_ERROR_INVALID_STATE with the ring off,
   KHS_ERROR_INVALID_ARGUMENT if the ring does not hold the frame. */
KHS_API KhsResult khsxCopyOutputFrame(KhsSolver *solver, uint32_t frame, KhsVec3 *positions,
                                      uint32_t capacity);

/* As khsxCopyOutputFrame, but returns a pointer to the pinned slot itself
   (no host copy), valid until `slots` more frames are stepped or the ring
   is changed. */
KHS_API KhsResult khsxMapOutputFrame(KhsSolver *solver, uint32_t frame, const KhsVec3 **positions);

/* Copies the full generalised state: q and v are 6 * internal_node_count
   FP64 values each, per-node interleaved (x, y, z, rx, ry, rz).  Either
   pointer may be NULL. */
KHS_API KhsResult khsxCopyState(const KhsSolver *solver, double *q, double *v,
                                uint64_t dof_capacity);

/* Per-substep Gauss-Newton record of the last frame (for diagnostics and the
   refinement histogram of the mixed form). */
typedef struct KhsxSubstepRecord {
    uint32_t struct_size;
    uint32_t substep;
    uint32_t newton_iterations;
    uint32_t line_search_evaluations;
    uint32_t steepest_fallbacks;
    uint32_t refinement_sweeps;    /* KHSX_MODE_MIXED_FF: FP64 refinement sweeps */
    uint32_t fp64_fallbacks;       /* KHSX_MODE_MIXED_FF: directions re-solved in FP64 */
    uint32_t trust_scalings;       /* directions scaled down to the translation trust radius */
    uint64_t contact_candidates;
    uint64_t active_contacts;
    double final_residual_norm;
    double minimum_gap;
} KhsxSubstepRecord;

/* Ends every following frame after its first `substeps` substeps (0, the
   default, runs whole frames).  A frame cut short returns KHS_OK with the
   state after those substeps.  For sampled comparisons and timing of
   partial frames against another implementation from one checkpoint; a
   bake never sets it.  May be called before or after khsBuild. */
KHS_API KhsResult khsxSetSubstepLimit(KhsSolver *solver, uint32_t substeps);

/* Number of substep records of the last frame (last adaptive attempt). */
KHS_API uint32_t khsxGetSubstepRecordCount(const KhsSolver *solver);
KHS_API KhsResult khsxCopySubstepRecords(const KhsSolver *solver,
                                         KhsxSubstepRecord *records,
                                         uint32_t capacity);

/* Per-element broadphase/narrowphase result of the most recent
   gradient evaluation (the state the last accepted iterate was assembled
   at).  closest_triangle is UINT32_MAX when the element had no candidate;
   active is 1 when 0 < gap - minimum_gap and gap < barrier_distance. */
typedef struct KhsxContactRecord {
    uint32_t candidate_count;
    uint32_t closest_triangle;
    uint32_t active;
    uint32_t reserved;
    double gap;
} KhsxContactRecord;

/* capacity must be >= the element count (KhsBuildStats.element_count). */
KHS_API KhsResult khsxCopyContactRecords(const KhsSolver *solver,
                                         KhsxContactRecord *records,
                                         uint32_t capacity);

/* Broad + narrow phase of every element at the caller's state q (6 values
   per internal node, as khsxCopyState returns) against the collider as
   the last substep left it.  Does not change q or v; the records (as in
   khsxCopyContactRecords) replace those khsxCopyContactRecords returns.  This is the integer contact work of one
   evaluation, exposed so it can be compared bit for bit. */
KHS_API KhsResult khsxQueryContacts(KhsSolver *solver, const double *q,
                                    uint64_t dof_count,
                                    KhsxContactRecord *records,
                                    uint32_t capacity);

/* khsxQueryContacts for callers that cannot allocate memory while they run:
   a render or audio thread with a fixed memory budget, a plug-in whose host
   owns the device memory pool, or a process whose caching allocator already
   holds the free device memory.  No counterpart in the reference.

   Same arguments and results as khsxQueryContacts (q and v unchanged),
   but the call allocates nothing (no cudaMalloc, cudaFree, host heap or
   library allocation): the caller's state and the records pass through one
   file-scope device array of KHSX_NO_ALLOC_SCRATCH_BYTES per device, and
   the solver's own contact records are left unchanged.
   - Size limit: 48 bytes per internal node (rounded up to 256) plus 24
     bytes per element must fit in KHSX_NO_ALLOC_SCRATCH_BYTES (about 100k
     elements of 1000-strand scenes); larger solvers get
     KHS_ERROR_INVALID_ARGUMENT.
   - The first call on a device does set-up (it looks up the array's device
     address and may load the device code); make it before any stream
     capture.
   - The array is shared by every solver on the device: calls that overlap
     in time on one device race; serialise them.
   - Errors are returned only (KHS_ERROR_INTERNAL for a CUDA failure); the
     message of khsGetLastError is not updated. */
#define KHSX_NO_ALLOC_SCRATCH_BYTES (8u * 1024u * 1024u)
KHS_API KhsResult khsxQueryContactsNoAlloc(KhsSolver *solver, const double *q,
                                           uint64_t dof_count,
                                           KhsxContactRecord *records,
                                           uint32_t capacity);

/* Root targets of every internal node for evaluated source points: the
   positions and rotation vectors khsUpdateRootTargets and
   khsSetRootAnimationFrame hand to the solver (replaces the host pass
   Solver::compute_root_targets, src/solver.cpp:416-447, which those entry
   points run per call in the reference).  All three entry points compute
   them on the device.  point_count must equal the curves' point count and
   node_capacity at least the internal node count; positions and rotations
   receive node_capacity >= N entries.  Errors: KHS_ERROR_INVALID_ARGUMENT
   (unbuilt solver, count or capacity), KHS_ERROR_INVALID_HAIR (a non-finite
   coordinate or a degenerate tangent). */
KHS_API KhsResult khsxComputeRootTargets(KhsSolver *solver, const KhsVec3 *points,
                                         uint32_t point_count, KhsVec3 *positions,
                                         KhsVec3 *rotations, uint32_t node_capacity);

/* ---- measurement ------------------------------------------------------- */

/* With profiling on, every kernel launch of the solver is bracketed by CUDA
   events on the solver's stream and the device time is accumulated per
   kernel.  Off by default. */
KHS_API KhsResult khsxSetProfiling(KhsSolver *solver, uint32_t enable);

typedef struct KhsxKernelTiming {
    char name[40];
    uint64_t launches;
    double total_milliseconds;
} KhsxKernelTiming;

/* Writes up to capacity entries, returns the number of kernels timed since
   profiling was enabled (or since the last reset). */
KHS_API uint32_t khsxGetKernelTimings(const KhsSolver *solver, KhsxKernelTiming *timings, uint32_t capacity);
KHS_API KhsResult khsxResetKernelTimings(KhsSolver *solver);

/* Kernels launched by this solver since it was built. */
KHS_API uint64_t khsxGetKernelLaunchCount(const KhsSolver *solver);

/* Measures the FP64 and FP32 FMA-pipe throughput of device 0 with a
   dependent-chain-free FMA kernel (TFLOP/s, 2 flops per FMA). */
KHS_API KhsResult khsxMeasurePipePeaks(double *fp64_tflops, double *fp32_tflops);

#ifdef __cplusplus
}
#endif

#endif /* KAMI_HAIR_SOLVER_H */
