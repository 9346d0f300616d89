// engine.cuh -- device buffer layout and per-phase launch entry points.
//
// HBM layout (structure of arrays, one slot per body / pair / row, sized by
// the context capacities):
//   bodies   pos[2], rot[2]       ping-pong pose buffers (Jacobi parity)
//            init_pos, init_rot   pose at step start       (avbd_init)
//            inert_pos, inert_rot inertial target           (avbd_init)
//            vel, ang, prev_vel   velocities
//            inv                  inverse moment xyz, inverse mass in w
//            shape                DioShape (80 B, the reference GpuShape)
//            scene                scene index of the body
//   pairs    DioPair list sorted by (a, b), count in counters
//   slots    narrow-phase output, `per_pair` slots per pair
//   rows     RowStatic (80 B at FP32) + RowDual (penalty, lambda) + (a, b)
//   CSR      row_off[n+1], row_idx[2m] (row), row_oth[2m] (other body | B flag)
//   joints   DioConstraint records + per-body joint CSR
// Pose arrays use P (float or double), everything else R.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

#include "../../include/dio_cuda.h"
#include "dio_math.cuh"

namespace dio {

constexpr uint32_t kContainer = 0xFFFFFFFFu;
constexpr uint32_t kIsB = 0x80000000u;  // row_oth flag: this body is `b`

// error_flags bits (device counters)
enum : uint32_t {
    kErrPairOverflow = 1u << 0,
    kErrRowOverflow = 1u << 1,
    kErrEpaFaces = 1u << 2,
    kErrEpaHorizon = 1u << 3,
    kErrTimeout = 1u << 4,
    kErrNonFinite = 1u << 5,
    kErrIndexOverflow = 1u << 6,
    kErrColorOverflow = 1u << 7,
    kErrBadIndex = 1u << 8,
};

struct Counters {
    uint32_t pairs;           // candidate pairs found (may exceed capacity)
    uint32_t rows;            // total contact rows
    uint32_t pair_rows;       // rows from narrow-phase slots
    uint32_t container_rows;  // rows against containers
    uint32_t gjk_work;        // pairs routed to GJK
    uint32_t epa_work;        // pairs routed to EPA
    uint32_t error_flags;
    uint32_t colors;
    uint32_t color_remaining;
    uint32_t scene_cursor;
    uint32_t prev_rows;       // rows of the previous step (warm-start source)
    uint32_t prev_pair_rows;  // of which from narrow-phase slots
    uint32_t long_count;      // CSR segments too long for the in-thread sort
    uint32_t dyn_changed;     // a state update turned a body static or dynamic
    uint32_t prev_pairs;      // pairs of the previous step (contact-lag rows)
    uint32_t traverse_pairs;  // pairs appended by the global trees' count pass
};

// Static part of one contact row (80 B at R = float):
//   n.xyz normal, n.w friction; t1.xyz, t1.w = c0.z; t2.xyz;
//   ra.xyz r_a (body frame), ra.w = c0.x; rb.xyz r_b, rb.w = c0.y
template <class R>
struct RowStatic {
    A4<R> n, t1, t2, ra, rb;
};
template <class P, class R>
struct RowDual {
    A4<R> penalty;  // xyz
    A4<P> lambda;   // xyz
};

// Narrow-phase slot; at R = float its bytes are exactly DioContactOut.
template <class R>
struct Slot {
    uint32_t valid, a, b, pad;
    A4<R> normal;
    R depth, pad2[3];
    A4<R> pa, pb;
};

// One scene of a packed world.
struct SceneDesc {
    uint32_t body_lo, body_hi;
    uint32_t has_container, pad;
    float center[3], half_extent;
    float rotation[4];
};

// One joint seen from one of its bodies (built once per upload from the
// joint list and the per-body joint CSR, joint order kept per body).
struct JView {
    float4 self_anchor;   // xyz; w = rest length / max length
    float4 other_anchor;  // xyz; w = stiffness
    uint32_t other;       // the other body
    uint32_t kind;        // constraint kind | kIsB when this body is `b`
    uint32_t pad[2];
};

template <class P, class R>
struct DevWorld {
    uint32_t n;  // bodies
    const uint32_t* dyn_list;  // dynamic bodies, ordered by work signature
    uint32_t n_dyn;
    const JView* jview;        // per-body joint views (joint CSR order)
    // poses
    A4<P>* pos[2];
    A4<P>* rot[2];
    A4<P>* init_pos;
    A4<P>* init_rot;
    A4<P>* inert_pos;
    A4<P>* inert_rot;
    A4<P>* vel;
    A4<P>* ang;
    A4<P>* prev_vel;
    A4<R>* inv;  // inv_moment xyz, inv_mass w
    A4<R>* mdt2;  // per step: m/dt^2 in x, I/dt^2 in y..w (dynamic bodies)
    R* friction;
    DioShape* shape;
    uint32_t* scene;
    A4<P>* origin;  // per-scene detection origin (split precision rebase)
    const A4<R>* walls;  // per scene, 6 container walls: outward normal xyz, plane offset w
    const A4<R>* hull;  // hull vertex pool
    // broad phase
    A4<R>* aabb_min;
    A4<R>* aabb_max;
    DioPair* pairs;
    uint32_t max_pairs;
    // narrow phase
    Slot<R>* slots;
    uint32_t per_pair;
    uint32_t* gjk_list;
    A4<R>* simplex;   // 8 x A4 per EPA entry (4 points, 4 witnesses)
    uint32_t* epa_list;
    uint32_t epa_wait_polls;  // budget of the EPA's first wait for its hull copies
    // rows
    RowStatic<R>* rs;
    RowDual<P, R>* rd;
    uint2* ab;
    uint32_t max_rows;
    uint32_t* row_off;
    uint32_t* row_idx;
    uint32_t* row_oth;
    uint32_t max_incid;
    // joints
    const DioConstraint* joints;
    uint32_t n_joints;
    const uint32_t* joint_off;
    const uint32_t* joint_idx;
    // colouring
    uint32_t* color;
    uint32_t* color_order;  // bodies sorted by colour
    uint32_t* color_off;    // colour -> first index in color_order
    // scenes
    const SceneDesc* scenes;
    uint32_t n_scenes;
    Counters* ctr;
};

// Solver parameters shared by init / primal / dual / recover
// (AvbdPush, engine/src/render/gpu_physics.rs:61-71).
template <class R>
struct SolveParams {
    R dt;
    R gx, gy, gz;
    R alpha;
    R beta_lin;
    R penalty_max;
    uint32_t iterations;
};

template <class R>
struct PrepParams {
    R dt;
    R margin;
    R penalty_min;
    R penalty_max;
    R alpha_gamma;  // alpha * gamma, rounded in R
    R gamma;
    R friction;
};

inline int grid_for(uint64_t n, int block, int max_blocks = 1 << 20) {
    uint64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > (uint64_t)max_blocks) g = max_blocks;
    return (int)g;
}

// ---- programmatic dependent launch ----
// A kernel launched with programmatic stream serialisation may start while
// its predecessor drains; griddepcontrol.wait (first thing in the kernel)
// blocks until the predecessor has completed and its writes are visible, and
// launch_dependents lets the successor's CTAs be scheduled early.  Launched
// without the attribute, both instructions have no effect.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Warp-aggregated append (ballot/popc compaction): the lanes that reach the
// call together take consecutive slots from *cursor with one atomic, in lane
// order.  Works on shared or global cursors.
__device__ __forceinline__ uint32_t warp_append(uint32_t* cursor) {
    uint32_t lane, lt;
    asm("mov.u32 %0, %%laneid;" : "=r"(lane));
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    const uint32_t m = __activemask();
    const uint32_t leader = (uint32_t)(__ffs(m) - 1);
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(cursor, (uint32_t)__popc(m));
    base = __shfl_sync(m, base, (int)leader);
    return base + (uint32_t)__popc(m & lt);
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(bool pdl, void (*kern)(KArgs...), int grid, int block, size_t smem, cudaStream_t s,
                            Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

}  // namespace dio
