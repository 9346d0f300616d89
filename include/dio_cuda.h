/*
 * dio_cuda.h -- C ABI of the GB300 (sm_103a) rigid-body pipeline.
 *
 * This is the drop-in boundary for Diomedes' per-step physics path.  Every
 * entry point below replaces one method of the reference's Vulkan compute
 * objects or of its host-side contact preparation; the comment on each names
 * the reference interface (file:line in nathenjacobe/diomedes) it stands in
 * for.  All record layouts are byte-identical to the reference's #[repr(C)]
 * structs so a Rust `-sys` crate can pass its existing Vec<GpuBody>,
 * Vec<GpuAvbdContact>, ... slices straight through.
 *
 * Conventions
 *   - Every call returns an int status (DIO_OK on success).  Capacity
 *     overflow is reported as DIO_ERR_CAPACITY instead of the reference's
 *     assert!/silent drop.
 *   - Calls are stream-ordered on the context's CUDA stream.  A context is
 *     owned by one host thread at a time.
 *   - Host pointers are plain host memory (pinned or pageable); the library
 *     copies in and out.  Sizes are element counts, not bytes.
 *   - Body indices in pairs, contacts and constraints are indices into the
 *     body array of the same call (or of the uploaded world).
 */
#ifndef DIO_CUDA_H
#define DIO_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum DioStatus {
    DIO_OK = 0,
    DIO_ERR_INVALID = 1,   /* null pointer, out-of-range index, bad option   */
    DIO_ERR_CAPACITY = 2,  /* more bodies/pairs/contacts than the context has */
    DIO_ERR_TIMEOUT = 3,   /* a bounded device wait gave up                  */
    DIO_ERR_CUDA = 4,      /* a CUDA runtime call failed                     */
    DIO_ERR_NONFINITE = 5, /* NaN/Inf detected in solver state               */
    DIO_ERR_STATE = 6      /* call order (e.g. read before submit)           */
};

/* ------------------------------------------------------------ constants */
/* shape tags: engine/gpu_physics/narrowphase/src/support.rs:5-7 (0..2).
 * BOX and HULL are extensions (per-axis half extents; convex vertex hull). */
#define DIO_SHAPE_SPHERE 0u
#define DIO_SHAPE_CUBE 1u
#define DIO_SHAPE_TETRAHEDRON 2u
#define DIO_SHAPE_BOX 3u
#define DIO_SHAPE_HULL 4u

/* contact `b` for rows against the container box:
 * engine/gpu_physics/avbd/src/lib.rs:75 */
#define DIO_CONTAINER 0xFFFFFFFFu

/* constraint kinds: engine/gpu_physics/avbd/src/lib.rs:76-79 */
#define DIO_CONSTRAINT_SPRING 0u
#define DIO_CONSTRAINT_ROD 1u
#define DIO_CONSTRAINT_BALL_SOCKET 2u
#define DIO_CONSTRAINT_ROPE 3u

/* narrow-phase output slots per candidate pair:
 * engine/gpu_physics/narrowphase/src/lib.rs:31 */
#define DIO_CONTACTS_PER_PAIR 4u

/* ---------------------------------------------------------------- records */
/* GpuShape, engine/src/render/compute.rs:28-34 (80 bytes).
 * sphere: radius in corners[0][0]; cube: half extent in corners[0][0..3];
 * tetrahedron: the four corners; box: half extents corners[0][0..3];
 * hull: pad[0] = first vertex in the hull-vertex pool, pad[1] = count. */
typedef struct DioShape {
    uint32_t tag;
    uint32_t pad[3];
    float corners[4][4];
} DioShape;

/* GpuBody, engine/src/render/compute.rs:78-82 (112 bytes) */
typedef struct DioGpuBody {
    float position[4];
    float orientation[4]; /* quaternion x, y, z, w */
    DioShape shape;
} DioGpuBody;

/* GpuPair, engine/src/render/compute.rs:97-100 */
typedef struct DioPair {
    uint32_t a;
    uint32_t b;
} DioPair;

/* GpuContactOut, engine/src/render/compute.rs:123-133 (80 bytes) */
typedef struct DioContactOut {
    uint32_t valid;
    uint32_t a;
    uint32_t b;
    uint32_t pad;
    float normal[4];
    float depth;
    float pad2[3];
    float point_a[4];
    float point_b[4];
} DioContactOut;

/* The part of a body that a frame loop changes and reads back every frame
 * (64 bytes; extension): its pose and velocities.  Shapes, masses, joints and
 * containers stay on the device from dio_world_upload, so a frame moves 64 B
 * per body each way instead of the GpuBody + GpuAvbdBodyState records'
 * 192 B of AvbdSolver::sync_bodies_from_gpu and the uploads of
 * demos/avbd_box/src/main.rs:232-257.  Positions are FP32: an FP64 world
 * (DIO_PREC_SPLIT / DIO_PREC_F64) takes and returns them rounded. */
typedef struct DioBodyMotion {
    float position[3];
    float orientation[4]; /* quaternion x, y, z, w */
    float velocity[3];
    float angular_velocity[3];
    float prev_velocity[3];
} DioBodyMotion;

/* GpuAvbdBodyState, engine/src/render/gpu_physics.rs:18-26 (80 bytes) */
typedef struct DioBodyState {
    float vel[4];
    float ang[4];
    float prev_vel[4];
    float inv_moment[4];
    float inv_mass;
    float friction;
    float pad[2];
} DioBodyState;

/* GpuAvbdContact, engine/src/render/gpu_physics.rs:31-44 (144 bytes) */
typedef struct DioContact {
    uint32_t a;
    uint32_t b; /* DIO_CONTAINER for container rows */
    float friction;
    float pad;
    float normal[4];
    float tangent1[4];
    float tangent2[4];
    float r_a[4];
    float r_b[4];
    float c0[4];
    float penalty[4];
    float lambda[4];
} DioContact;

/* GpuAvbdConstraint, engine/src/render/gpu_physics.rs:49-56 (48 bytes).
 * anchor_a.w = rest length (spring, rod) / max length (rope) / 0 (ball);
 * anchor_b.w = stiffness. */
typedef struct DioConstraint {
    uint32_t a;
    uint32_t b;
    uint32_t kind;
    uint32_t pad;
    float anchor_a[4];
    float anchor_b[4];
} DioConstraint;

/* AvbdRunOptions, engine/src/render/gpu_physics.rs:76-83 */
typedef struct DioRunOptions {
    float dt;
    float gravity[3];
    float alpha;
    float beta_lin;
    float penalty_max;
    uint32_t iterations;
} DioRunOptions;

/* AvbdOptions, engine/src/physics/gpu.rs:127-155 (usize iterations -> u32) */
typedef struct DioAvbdOptions {
    float dt;
    float gravity[3];
    uint32_t iterations;
    float alpha;
    float beta_lin;
    float margin;
    float penalty_min;
    float penalty_max;
    float gamma;
    float friction;
} DioAvbdOptions;

/* AvbdContainer, engine/src/physics/gpu.rs:118-123: a static box whose
 * interior is free space (its floor is the ground plane). */
typedef struct DioContainer {
    float center[3];
    float half_extent;
    float rotation[4]; /* x, y, z, w */
} DioContainer;

/* AvbdGpuResult, engine/src/render/gpu_physics.rs:86-94.  Caller-owned
 * arrays; any pointer may be NULL to skip that field. */
typedef struct DioAvbdResult {
    float* positions;          /* n * 3 */
    float* orientations;       /* n * 4 (x, y, z, w) */
    float* velocities;         /* n * 3 */
    float* angular_velocities; /* n * 3 */
    float* prev_velocities;    /* n * 3 */
    float* lambda;             /* m * 3 */
    float* penalty;            /* m * 3 */
} DioAvbdResult;

/* Context capacities.  The reference fixes (1024 bodies, 16384 pairs /
 * contacts) at engine/src/render/renderer.rs:81,141. */
typedef struct DioCapacity {
    uint32_t max_bodies;
    uint32_t max_pairs;
    uint32_t max_contacts;
    uint32_t max_joints;
    uint32_t max_scenes;
    uint32_t max_hull_vertices;
} DioCapacity;

/* Solver schedule and precision (extensions; no reference counterpart). */
enum DioSolverMode {
    DIO_SOLVER_JACOBI = 0,  /* reference schedule: ping-pong snapshot */
    DIO_SOLVER_COLORED = 1  /* graph-coloured Gauss-Seidel sweeps     */
};
enum DioPrecision {
    DIO_PREC_F32 = 0,   /* everything in FP32 (reference arithmetic)        */
    DIO_PREC_SPLIT = 1, /* FP64 poses/inertial/lambda, FP32 Hessian + LDL    */
    DIO_PREC_F64 = 2    /* everything in FP64 (the all-FP64 GPU oracle run) */
};

/* number of primal kernel variants selectable by DioConfig.primal_variant */
#define DIO_PRIMAL_VARIANTS 11

typedef struct DioConfig {
    uint32_t solver_mode;       /* DioSolverMode                          */
    uint32_t precision;         /* DioPrecision (fixed at world upload)   */
    uint32_t contacts_per_pair; /* 4 (reference) or 8 (extended manifold) */
    uint32_t use_graph;         /* replay each step as a CUDA graph       */
    uint32_t primal_variant;    /* primal kernel variant, 0 .. DIO_PRIMAL_VARIANTS-1
                                   (launch shape, body tiles; every variant
                                   computes the same bits; autotuned)     */
    uint32_t block_size;        /* threads per CTA of the scene-chunk
                                   solve: 0 (512) or 640 (autotuned)      */
    uint32_t batched_solver;    /* DioSolveLaunch: DIO_SOLVE_AUTO (0) runs
                                   a world step's whole solve (init, the
                                   iterations, recover) as one launch, a
                                   CTA per chunk of whole scenes with the
                                   poses in shared memory, when every
                                   scene fits a chunk (2048 bodies, 1024
                                   with FP64 poses) and no joint crosses
                                   scenes; DIO_SOLVE_PER_PHASE (1) always
                                   launches init / primal / dual / recover
                                   kernels.  Both give identical results. */
    uint32_t profile;           /* time primal / dual launches with events */
    uint32_t broad_phase;       /* 0: LBVH (default), 1: dense sweep        */
    uint32_t bvh_rebuild_period; /* LBVH topology rebuilt every N steps and
                                    refitted in between (0: every 4)     */
    uint32_t contact_lag;       /* 1: the demos' frame pipelining -- pair
                                   rows of step t come from the narrow phase
                                   of step t-1 (its witness points, this
                                   step's transforms; demos/avbd_box/src/
                                   main.rs:203-207,244-249); container rows
                                   are current.  0 (default): no lag      */
    uint32_t debug_flags;       /* testing only, 0 in normal use:
                                   DIO_DEBUG_EPA_NO_FIRST_WAIT makes the
                                   EPA's first bounded wait for its hull
                                   copies give up at once (the step then
                                   returns DIO_ERR_TIMEOUT; the second
                                   wait, always at its full budget, still
                                   lets the copies land)                  */
} DioConfig;
#define DIO_DEBUG_EPA_NO_FIRST_WAIT 1u
typedef enum DioSolveLaunch { DIO_SOLVE_AUTO = 0, DIO_SOLVE_PER_PHASE = 1 } DioSolveLaunch;

/* World description for the fused device-resident step (extension of the
 * demos' per-frame loop, demos/avbd_box/src/main.rs:189-273). */
typedef struct DioWorldDesc {
    uint32_t n_bodies;
    uint32_t n_constraints;
    uint32_t n_scenes;            /* 0 or 1: one scene                      */
    uint32_t n_hull_vertices;
    const DioGpuBody* bodies;     /* pose + shape                            */
    const DioBodyState* state;    /* velocities, inverse mass/moment         */
    const DioConstraint* constraints;
    const uint32_t* scene_offsets; /* n_scenes + 1 body offsets, or NULL   */
    const DioContainer* containers; /* one per scene, or NULL (no container) */
    const float* hull_vertices;   /* n_hull_vertices * 4 (x, y, z, pad)      */
    const double* positions_f64;  /* optional n * 3 FP64 positions           */
    const double* orientations_f64; /* optional n * 4 FP64 orientations      */
} DioWorldDesc;

typedef struct DioStepStats {
    uint32_t pairs;
    uint32_t contacts;
    uint32_t colors;
    uint32_t error_flags;
    uint64_t steps;
    uint64_t kernel_launches; /* kernels of this library launched so far   */
    uint32_t primal_launches; /* primal launches timed (DioConfig.profile) */
    uint32_t dual_launches;   /* dual launches timed                       */
    double primal_ms;         /* summed primal kernel time (CUDA events)   */
    double dual_ms;           /* summed dual kernel time                   */
    double broad_ms;          /* summed broad-phase time (AABB .. pairs)   */
    double narrow_ms;         /* summed narrow-phase time                  */
    double rows_ms;           /* summed row build + warm start + CSR time  */
    double solve_ms;          /* summed init .. recover time               */
    uint32_t chunk_launches;  /* scene-chunk solve launches timed          */
    uint32_t pad;
    double chunk_ms;          /* summed scene-chunk solve kernel time      */
} DioStepStats;

typedef struct DioCtx DioCtx;

/* ------------------------------------------------------------- lifecycle */
/* NarrowPhaseCompute::new + AvbdCompute::new,
 * engine/src/render/compute.rs:176, engine/src/render/gpu_physics.rs:224 */
int dio_ctx_create(const DioCapacity* capacity, DioCtx** out);
/* NarrowPhaseCompute::destroy + AvbdCompute::destroy,
 * engine/src/render/compute.rs:707, engine/src/render/gpu_physics.rs:652 */
int dio_ctx_destroy(DioCtx* ctx);
/* Human-readable text for a status code (static storage). */
const char* dio_status_string(int status);
/* Last error message recorded on the context (static until next call). */
const char* dio_ctx_last_error(const DioCtx* ctx);
/* Solver schedule / precision / tuning knobs (extension). */
int dio_ctx_configure(DioCtx* ctx, const DioConfig* config);
int dio_ctx_get_config(const DioCtx* ctx, DioConfig* out);
/* Run work on a caller's cudaStream_t (NULL = the context's own stream). */
int dio_ctx_set_stream(DioCtx* ctx, void* cuda_stream);
/* Block until all work on the context's stream has finished. */
int dio_ctx_synchronize(DioCtx* ctx);  /* also reports deferred device error flags */

/* ----------------------------------------------- broad + narrow phase */
/* NarrowPhaseCompute::submit_broad, engine/src/render/compute.rs:490-567:
 * per-body support AABB, then overlap pairs (a < b).  The pair list is
 * sorted by (a, b); the reference's atomic-append order is arbitrary. */
int dio_broad_submit(DioCtx* ctx, const DioGpuBody* bodies, uint32_t n);
/* NarrowPhaseCompute::read_pair_count, engine/src/render/compute.rs:570-579.
 * Returns DIO_ERR_CAPACITY (and the true count) when pairs overflowed. */
int dio_broad_pair_count(DioCtx* ctx, uint32_t* count);
/* NarrowPhaseCompute::read_pairs, engine/src/render/compute.rs:583-597 */
int dio_read_pairs(DioCtx* ctx, DioPair* out, uint32_t cap, uint32_t* n);
/* NarrowPhaseCompute::submit, engine/src/render/compute.rs:404-484:
 * upload bodies + explicit pairs and run the narrow phase. */
int dio_narrow_submit_pairs(DioCtx* ctx, const DioGpuBody* bodies, uint32_t n,
                            const DioPair* pairs, uint32_t n_pairs);
/* NarrowPhaseCompute::submit_narrow, engine/src/render/compute.rs:601-671:
 * narrow phase over the pairs the last dio_broad_submit produced. */
int dio_narrow_submit(DioCtx* ctx, uint32_t pair_count);
/* NarrowPhaseCompute::read, engine/src/render/compute.rs:675-693: the raw
 * slots, DIO_CONTACTS_PER_PAIR per pair (unused slots have valid == 0). */
int dio_narrow_read(DioCtx* ctx, DioContactOut* out, uint32_t cap, uint32_t* n);
/* Hull vertex pool for DIO_SHAPE_HULL bodies (extension). */
int dio_set_hull_vertices(DioCtx* ctx, const float* xyzw, uint32_t count);

/* ------------------------------------------------ contact preparation */
/* AvbdSolver::raw_contact + prepare_contacts + finalize_contacts,
 * engine/src/physics/gpu.rs:188-311, run on the device: decode the valid
 * narrow-phase slots, build rows (normal = -n, tangents, body-frame lever
 * arms, c0 = margin - depth), append container rows for dynamic bodies,
 * warm-start (lambda, penalty) from `prev` by (a, b) key, decay, and build
 * the per-body CSR.  `prev` are the previous step's rows carrying the
 * solved lambda/penalty (AvbdSolver::contacts after sync_bodies_from_gpu). */
int dio_prepare_contacts(DioCtx* ctx, const DioGpuBody* bodies,
                         const DioBodyState* state, uint32_t n,
                         const DioContactOut* slots, uint32_t n_slots,
                         const DioContact* prev, uint32_t n_prev,
                         const DioContainer* container,
                         const DioAvbdOptions* options, DioContact* out,
                         uint32_t cap, uint32_t* m, uint32_t* offsets,
                         uint32_t* indices, uint32_t index_cap);

/* ---------------------------------------------------------- AVBD solve */
/* AvbdCompute::submit, engine/src/render/gpu_physics.rs:439-561:
 * init, (primal, dual) x iterations, recover.  positions are n * 3 floats,
 * orientations n * 4 (x, y, z, w); offsets n + 1; indices offsets[n]. */
int dio_avbd_submit(DioCtx* ctx, const DioBodyState* state,
                    const float* positions, const float* orientations,
                    uint32_t n, const DioContact* contacts, uint32_t m,
                    const DioConstraint* constraints, uint32_t n_constraints,
                    const uint32_t* offsets, const uint32_t* indices,
                    const DioRunOptions* options);
/* AvbdCompute::read, engine/src/render/gpu_physics.rs:565-622 */
int dio_avbd_read(DioCtx* ctx, const DioAvbdResult* out);

/* No counterpart in the reference.  The AVBD solve of dio_avbd_submit for
 * callers that may not allocate device memory (a host that owns its device
 * memory through another allocator, or a real-time loop that must not
 * allocate once running).  Needs no context; every pointer is DEVICE
 * memory the caller owns: state (n), positions (n * 3), orientations
 * (n * 4), contacts (m; lambda and penalty are updated in place),
 * constraints, offsets (n + 1) and indices (offsets[n]).  Results go to
 * out_positions (n * 3), out_orientations (n * 4) and out_state (n; may
 * alias state).  Scratch lives in a fixed device array of the library
 * (about 3 MB per GPU, held until exit): at most 4096 bodies, 16384
 * contacts and 4096 joints, else DIO_ERR_CAPACITY.  Joints are scanned per
 * body as in the reference.  Calls share that array, so calls that overlap
 * on the GPU race.  The first call on each device looks up the array's
 * address with that device current and caches it for the current CUDA
 * context (a new context, e.g. after cudaDeviceReset, is looked up again);
 * make that first call before any stream capture.  Synchronous: it waits on
 * `cuda_stream` (NULL = default stream) once to validate the indices
 * (DIO_ERR_INVALID for a contact, CSR or joint index out of range) and once
 * at the end; a non-finite pose or velocity after the solve returns
 * DIO_ERR_NONFINITE, as dio_avbd_read does. */
int dio_avbd_solve_noalloc(const DioBodyState* state, const float* positions,
                           const float* orientations, uint32_t n,
                           DioContact* contacts, uint32_t m,
                           const DioConstraint* constraints,
                           uint32_t n_constraints, const uint32_t* offsets,
                           const uint32_t* indices,
                           const DioRunOptions* options, float* out_positions,
                           float* out_orientations, DioBodyState* out_state,
                           void* cuda_stream);

/* ------------------------------------------- fused device-resident step */
/* Upload a world (one or many packed scenes).  Replaces the per-frame
 * uploads of demos/avbd_box/src/main.rs:232-271. */
int dio_world_upload(DioCtx* ctx, const DioWorldDesc* desc);
/* One or more full steps of every scene: broad -> narrow -> rows + warm
 * start -> solve, all on the device (demos' frame loop without the
 * one-frame contact lag).  Scenes are packed into the same launches; a
 * one-scene world per context is the plain one-scene-per-launch path. */
int dio_step(DioCtx* ctx, const DioAvbdOptions* options, uint32_t steps);
/* dio_step without the closing synchronisation (the async submit of the
 * reference's frame loop, engine/src/render/gpu_physics.rs:435-561): the
 * steps are enqueued on the context's stream and the call returns; device
 * error flags are reported by the next synchronising call
 * (dio_ctx_synchronize, dio_step, dio_world_download, dio_world_stats). */
int dio_step_async(DioCtx* ctx, const DioAvbdOptions* options, uint32_t steps);
/* dio_world_download enqueued without waiting (the double-buffered read of
 * engine/src/render/compute.rs:160-165,423-425): the copies into the
 * caller's buffers (page-locked for a truly asynchronous copy) complete in
 * stream order; wait with dio_ctx_synchronize or an event on the stream. */
int dio_world_download_async(DioCtx* ctx, DioGpuBody* bodies, DioBodyState* state);
/* Per-frame pose/state upload of the demos (demos/avbd_box/src/main.rs:232-
 * 257): replace every body's pose (position, orientation) and state
 * (velocities, inverse mass/moment) from host arrays, keeping shapes, joints
 * and the warm-start rows.  Either pointer may be NULL. */
int dio_world_set_state(DioCtx* ctx, const DioGpuBody* bodies, const DioBodyState* state);
/* AvbdSolver::sync_bodies_from_gpu, engine/src/physics/gpu.rs:212-237:
 * read the world's poses (FP32) and state back. Either pointer may be NULL. */
int dio_world_download(DioCtx* ctx, DioGpuBody* bodies, DioBodyState* state);
/* The demos' per-frame loop (demos/avbd_box/src/main.rs:232-257: upload the
 * poses, step, read them back) over a batch held as `count` worlds, one per
 * context: for each step and world in order, dio_world_set_state(bodies[g],
 * states[g]), dio_step_async(1) and dio_world_download_async(bodies[g],
 * states[g]).  Contexts on separate streams overlap one world's host copies
 * with another world's steps; page-locked host arrays keep the copies
 * asynchronous.  Every context is synchronised before the call returns (device
 * error flags included); the first failure is returned and recorded on the
 * context it came from.  No argument may be NULL; count == 0 is a no-op. */
int dio_worlds_step_host(DioCtx* const* ctxs, uint32_t count, DioGpuBody* const* bodies,
                         DioBodyState* const* states, const DioAvbdOptions* options, uint32_t steps);
/* Extension: replace every body's pose and velocities from `motion` (n
 * records), keeping shapes, masses, joints and the warm-start rows; enqueued
 * on the context's stream (a page-locked array keeps the copy asynchronous;
 * leave it unchanged until the stream has passed the copy). */
int dio_world_set_motion(DioCtx* ctx, const DioBodyMotion* motion);
/* Extension: read every body's pose and velocities into `motion` (n
 * records); the _async form returns once the copy is enqueued. */
int dio_world_download_motion(DioCtx* ctx, DioBodyMotion* motion);
int dio_world_download_motion_async(DioCtx* ctx, DioBodyMotion* motion);
/* Extension: dio_worlds_step_host with motion records: per step and world,
 * dio_world_set_motion, dio_step_async(1), dio_world_download_motion_async,
 * every world's copy queued before the next world's step; every context is
 * synchronised before the call returns.  No argument may be NULL; count == 0
 * is a no-op. */
int dio_worlds_step_motion_host(DioCtx* const* ctxs, uint32_t count, DioBodyMotion* const* motions,
                                const DioAvbdOptions* options, uint32_t steps);
/* FP64 poses (exact in DIO_PREC_SPLIT / DIO_PREC_F64 worlds). */
int dio_world_download_f64(DioCtx* ctx, double* positions, double* orientations);
/* The last step's contact rows with their solved lambda / penalty. */
int dio_world_contacts(DioCtx* ctx, DioContact* out, uint32_t cap, uint32_t* m);
/* Per-body colour of the last coloured step (DIO_SOLVER_COLORED). */
int dio_world_colors(DioCtx* ctx, uint32_t* out, uint32_t cap, uint32_t* n);
/* Counters of the last step (synchronises the stream when profiling). */
int dio_world_stats(DioCtx* ctx, DioStepStats* out);
/* Reset the kernel timers and launch counter of the world (extension). */
int dio_world_reset_timers(DioCtx* ctx);
/* Headless transform export: every body's transform written, in body order
 * and stream-ordered on the context's stream (no synchronisation), into a
 * DEVICE buffer the caller owns -- e.g. a renderer's instance buffer.
 * Replaces the per-instance host copy of demos/avbd_box/src/main.rs:276-280
 * and the model matrices of engine/src/render/renderer.rs:251-255.
 *   DIO_XFORM_POSE  32 B: float4 position (w = 0), float4 quaternion xyzw
 *   DIO_XFORM_MAT4  64 B: column-major 4x4 model matrix = translation *
 *                   rotation * scale (Mat4::from_scale_rotation_translation)
 * `scales` (device, one float per body, uniform scale) may be NULL (1).
 * `out` and `stride_bytes` must be multiples of 16, stride >= the record. */
enum { DIO_XFORM_POSE = 0, DIO_XFORM_MAT4 = 1 };
int dio_world_export_transforms(DioCtx* ctx, uint32_t format, const float* scales, void* out,
                                size_t stride_bytes);
/* Checkpoint (extension; no reference counterpart -- the reference's state
 * round trip is sync_bodies_from_gpu, engine/src/physics/gpu.rs:212-237,
 * which drops the warm-start rows and the FP64 poses).  Serialises the world
 * into a versioned byte image: bodies and shapes, state, joints, scene table
 * with containers, hull vertices, the poses / velocities in the world's own
 * precision and the last step's rows with their lambda / penalty (the next
 * warm start's source).  With buffer == NULL only *size is set; a capacity
 * below the image size returns DIO_ERR_CAPACITY. */
int dio_world_checkpoint(DioCtx* ctx, void* buffer, size_t capacity, size_t* size);
/* Resume a checkpoint into this context (same precision, enough capacity):
 * the world is uploaded from the image and its dynamic state and warm-start
 * rows restored, so stepping continues bit for bit as the checkpointed world
 * would have.  A damaged or foreign image returns DIO_ERR_INVALID. */
int dio_world_resume(DioCtx* ctx, const void* buffer, size_t size);
/* Autotuner (extension): times the solve launch (one scene-chunk launch
 * against init / primal / dual / recover per phase), the primal launch-shape
 * variants (when the per-phase launches win) and the LBVH rebuild period on
 * the uploaded world (trial_steps timed steps per
 * candidate, starting from a device snapshot that is restored afterwards,
 * so the world's state is unchanged), applies the fastest configuration and
 * returns it in `best`.  With `cache_path` set, a tuned configuration for
 * the same device and world shape is reused from / appended to that text
 * file.  Every candidate computes bit-identical results. */
int dio_autotune(DioCtx* ctx, const DioAvbdOptions* options,
                 uint32_t trial_steps, const char* cache_path, DioConfig* best);

#ifdef __cplusplus
}
#endif

#endif /* DIO_CUDA_H */
