// engine_impl.cuh -- one engine instance: device buffers and the step
// pipeline, templated on pose precision P and arithmetic precision R.
// Included by exactly one translation unit per precision.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <vector>

#include "engine_base.h"
#include "k_avbd.cuh"
#include "k_broad.cuh"
#include "k_chunk.cuh"
#include "k_color.cuh"
#include "k_lbvh.cuh"
#include "k_narrow_kernels.cuh"
#include "k_rows.cuh"
#include "k_scan.cuh"

namespace dio {

#define DIO_CK(expr)                                                            \
    do {                                                                        \
        cudaError_t e_ = (expr);                                                \
        if (e_ != cudaSuccess) {                                                \
            err = std::string(#expr) + ": " + cudaGetErrorString(e_);           \
            return DIO_ERR_CUDA;                                                \
        }                                                                       \
    } while (0)

#define DIO_TRY(expr)            \
    do {                         \
        int rc_ = (expr);        \
        if (rc_ != DIO_OK) return rc_; \
    } while (0)

// small kernels used by the pipeline ------------------------------------
static __global__ void k_set_u32(uint32_t* dst, uint32_t v) { *dst = v; }
static __global__ void k_copy_u32(uint32_t* dst, const uint32_t* src) { *dst = *src; }
static __global__ void k_sum_rows(Counters* c, const uint32_t* pair_rows, const uint32_t* cont_rows, uint32_t max_rows) {
    pdl_enter();
    c->pair_rows = *pair_rows;
    c->container_rows = *cont_rows;
    uint64_t t = (uint64_t)*pair_rows + *cont_rows;
    c->rows = t > max_rows ? max_rows : (uint32_t)t;
    if (t > max_rows) c->error_flags |= kErrRowOverflow;
}
static __global__ void k_pairs_total(Counters* c, const uint32_t* total, uint32_t max_pairs) {
    pdl_enter();
    c->pairs = *total;
    if (*total > max_pairs) c->error_flags |= kErrPairOverflow;
}

template <class P, class R>
__global__ void k_unpack_bodies(DevWorld<P, R> w, const DioGpuBody* bodies, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const DioGpuBody b = bodies[i];
        w.pos[0][i] = A4<P>{P(b.position[0]), P(b.position[1]), P(b.position[2]), P(0)};
        w.rot[0][i] = A4<P>{P(b.orientation[0]), P(b.orientation[1]), P(b.orientation[2]), P(b.orientation[3])};
        w.shape[i] = b.shape;
        w.scene[i] = 0;
    }
}

template <class P, class R>
__global__ void k_set_pose(DevWorld<P, R> w, const DioGpuBody* bodies, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = *reinterpret_cast<const float4*>(bodies[i].position);
        const float4 q = *reinterpret_cast<const float4*>(bodies[i].orientation);
        w.pos[0][i] = A4<P>{P(p.x), P(p.y), P(p.z), P(0)};
        w.rot[0][i] = A4<P>{P(q.x), P(q.y), P(q.z), P(q.w)};
    }
}

template <class P, class R>
__global__ void k_unpack_pose3(DevWorld<P, R> w, const float* pos3, const float* quat4, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        w.pos[0][i] = A4<P>{P(pos3[3 * i]), P(pos3[3 * i + 1]), P(pos3[3 * i + 2]), P(0)};
        w.rot[0][i] = A4<P>{P(quat4[4 * i]), P(quat4[4 * i + 1]), P(quat4[4 * i + 2]), P(quat4[4 * i + 3])};
        w.scene[i] = 0;
    }
}

template <class P, class R>
__global__ void k_unpack_pose_f64(DevWorld<P, R> w, const double* pos3, const double* quat4, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (pos3) w.pos[0][i] = A4<P>{P(pos3[3 * i]), P(pos3[3 * i + 1]), P(pos3[3 * i + 2]), P(0)};
        if (quat4)
            w.rot[0][i] = A4<P>{P(quat4[4 * i]), P(quat4[4 * i + 1]), P(quat4[4 * i + 2]), P(quat4[4 * i + 3])};
    }
}

// DioBodyMotion records in / out (pose and velocities)
template <class P, class R>
__global__ void k_unpack_motion(DevWorld<P, R> w, const DioBodyMotion* m, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const DioBodyMotion r = m[i];
        w.pos[0][i] = A4<P>{P(r.position[0]), P(r.position[1]), P(r.position[2]), P(0)};
        w.rot[0][i] = A4<P>{P(r.orientation[0]), P(r.orientation[1]), P(r.orientation[2]), P(r.orientation[3])};
        w.vel[i] = A4<P>{P(r.velocity[0]), P(r.velocity[1]), P(r.velocity[2]), P(0)};
        w.ang[i] = A4<P>{P(r.angular_velocity[0]), P(r.angular_velocity[1]), P(r.angular_velocity[2]), P(0)};
        w.prev_vel[i] = A4<P>{P(r.prev_velocity[0]), P(r.prev_velocity[1]), P(r.prev_velocity[2]), P(0)};
    }
}
template <class P, class R>
__global__ void k_pack_motion(DevWorld<P, R> w, DioBodyMotion* m, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const A4<P> p = w.pos[0][i], q = w.rot[0][i], v = w.vel[i], a = w.ang[i], pv = w.prev_vel[i];
        DioBodyMotion r;
        r.position[0] = float(p.x), r.position[1] = float(p.y), r.position[2] = float(p.z);
        r.orientation[0] = float(q.x), r.orientation[1] = float(q.y), r.orientation[2] = float(q.z);
        r.orientation[3] = float(q.w);
        r.velocity[0] = float(v.x), r.velocity[1] = float(v.y), r.velocity[2] = float(v.z);
        r.angular_velocity[0] = float(a.x), r.angular_velocity[1] = float(a.y), r.angular_velocity[2] = float(a.z);
        r.prev_velocity[0] = float(pv.x), r.prev_velocity[1] = float(pv.y), r.prev_velocity[2] = float(pv.z);
        m[i] = r;
    }
}

template <class P, class R>
__global__ void k_unpack_state(DevWorld<P, R> w, const DioBodyState* st, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const DioBodyState s = st[i];
        w.vel[i] = A4<P>{P(s.vel[0]), P(s.vel[1]), P(s.vel[2]), P(0)};
        w.ang[i] = A4<P>{P(s.ang[0]), P(s.ang[1]), P(s.ang[2]), P(0)};
        w.prev_vel[i] = A4<P>{P(s.prev_vel[0]), P(s.prev_vel[1]), P(s.prev_vel[2]), P(0)};
        w.inv[i] = A4<R>{R(s.inv_moment[0]), R(s.inv_moment[1]), R(s.inv_moment[2]), R(s.inv_mass)};
        w.friction[i] = R(s.friction);
    }
}

template <class P, class R>
__global__ void k_unpack_contacts(RowStatic<R>* rs, RowDual<P, R>* rd, uint2* ab, const DioContact* c, uint32_t m,
                                  uint32_t n, uint32_t* err) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        const DioContact x = c[r];
        RowStatic<R> s;
        s.n = A4<R>{R(x.normal[0]), R(x.normal[1]), R(x.normal[2]), R(x.friction)};
        s.t1 = A4<R>{R(x.tangent1[0]), R(x.tangent1[1]), R(x.tangent1[2]), R(x.c0[2])};
        s.t2 = A4<R>{R(x.tangent2[0]), R(x.tangent2[1]), R(x.tangent2[2]), R(0)};
        s.ra = A4<R>{R(x.r_a[0]), R(x.r_a[1]), R(x.r_a[2]), R(x.c0[0])};
        s.rb = A4<R>{R(x.r_b[0]), R(x.r_b[1]), R(x.r_b[2]), R(x.c0[1])};
        rs[r] = s;
        RowDual<P, R> d;
        d.penalty = A4<R>{R(x.penalty[0]), R(x.penalty[1]), R(x.penalty[2]), R(0)};
        d.lambda = A4<P>{P(x.lambda[0]), P(x.lambda[1]), P(x.lambda[2]), P(0)};
        rd[r] = d;
        ab[r] = make_uint2(x.a, x.b);
        if (x.a >= n || (x.b != kContainer && x.b >= n)) atomicOr(err, kErrBadIndex);
    }
}

template <class P, class R>
__global__ void k_pack_contacts(const RowStatic<R>* rs, const RowDual<P, R>* rd, const uint2* ab, DioContact* out,
                                const uint32_t* m_dev) {
    uint32_t m = *m_dev;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        const RowStatic<R> s = rs[r];
        const RowDual<P, R> d = rd[r];
        DioContact x;
        x.a = ab[r].x;
        x.b = ab[r].y;
        x.friction = float(s.n.w);
        x.pad = 0.f;
        auto put = [](float* f, A4<R> v) {
            f[0] = float(v.x);
            f[1] = float(v.y);
            f[2] = float(v.z);
            f[3] = 0.f;
        };
        put(x.normal, s.n);
        put(x.tangent1, s.t1);
        put(x.tangent2, s.t2);
        put(x.r_a, s.ra);
        put(x.r_b, s.rb);
        x.c0[0] = float(s.ra.w);
        x.c0[1] = float(s.rb.w);
        x.c0[2] = float(s.t1.w);
        x.c0[3] = 0.f;
        put(x.penalty, d.penalty);
        x.lambda[0] = float(d.lambda.x);
        x.lambda[1] = float(d.lambda.y);
        x.lambda[2] = float(d.lambda.z);
        x.lambda[3] = 0.f;
        out[r] = x;
    }
}

// Given the reference CSR (offsets, indices), derive the other-body array.
static __global__ void k_csr_other(const uint32_t* off, const uint32_t* idx, const uint2* ab, uint32_t* oth, uint32_t n,
                            uint32_t m, uint32_t* err) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        for (uint32_t j = off[i]; j < off[i + 1]; ++j) {
            uint32_t r = idx[j];
            if (r >= m) {
                atomicOr(err, kErrBadIndex);
                oth[j] = kContainer;
                continue;
            }
            uint2 v = ab[r];
            if (v.y == kContainer)
                oth[j] = kContainer;
            else if (v.x == i)
                oth[j] = v.y;
            else
                oth[j] = v.x | kIsB;
        }
    }
}

// Per-body transform records for a renderer (dio_world_export_transforms).
// The matrix is the standard unit-quaternion rotation (columns
// (1-2(y^2+z^2), 2(xy+wz), 2(xz-wy)), ...) scaled per body and translated,
// the same construction as Mat4::from_scale_rotation_translation.
template <class P, class R>
__global__ void k_export_xform(const A4<P>* pos, const A4<P>* rot, uint32_t n, uint32_t format, const float* scales,
                               char* out, size_t stride) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const A4<P> p = pos[i], q = rot[i];
        const float px = float(p.x), py = float(p.y), pz = float(p.z);
        const float x = float(q.x), y = float(q.y), z = float(q.z), w = float(q.w);
        float4* o = reinterpret_cast<float4*>(out + (size_t)i * stride);
        if (format == DIO_XFORM_POSE) {
            o[0] = make_float4(px, py, pz, 0.f);
            o[1] = make_float4(x, y, z, w);
            continue;
        }
        const float s = scales ? scales[i] : 1.f;
        const float x2 = x + x, y2 = y + y, z2 = z + z;
        const float xx = x * x2, xy = x * y2, xz = x * z2;
        const float yy = y * y2, yz = y * z2, zz = z * z2;
        const float wx = w * x2, wy = w * y2, wz = w * z2;
        o[0] = make_float4((1.f - (yy + zz)) * s, (xy + wz) * s, (xz - wy) * s, 0.f);
        o[1] = make_float4((xy - wz) * s, (1.f - (xx + zz)) * s, (yz + wx) * s, 0.f);
        o[2] = make_float4((xz + wy) * s, (yz - wx) * s, (1.f - (xx + yy)) * s, 0.f);
        o[3] = make_float4(px, py, pz, 1.f);
    }
}

template <class P, class R>
__global__ void k_pack_result(DevWorld<P, R> w, uint32_t n, int buf, float* pos3, float* quat4, float* vel,
                              float* ang, float* prev) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        A4<P> p = w.pos[buf][i], q = w.rot[buf][i], v = w.vel[i], a = w.ang[i], pv = w.prev_vel[i];
        pos3[3 * i] = float(p.x);
        pos3[3 * i + 1] = float(p.y);
        pos3[3 * i + 2] = float(p.z);
        quat4[4 * i] = float(q.x);
        quat4[4 * i + 1] = float(q.y);
        quat4[4 * i + 2] = float(q.z);
        quat4[4 * i + 3] = float(q.w);
        vel[3 * i] = float(v.x);
        vel[3 * i + 1] = float(v.y);
        vel[3 * i + 2] = float(v.z);
        ang[3 * i] = float(a.x);
        ang[3 * i + 1] = float(a.y);
        ang[3 * i + 2] = float(a.z);
        prev[3 * i] = float(pv.x);
        prev[3 * i + 1] = float(pv.y);
        prev[3 * i + 2] = float(pv.z);
    }
}

template <class P, class R>
__global__ void k_pack_dual(const RowDual<P, R>* rd, uint32_t m, float* lambda, float* penalty) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        RowDual<P, R> d = rd[r];
        lambda[3 * r] = float(d.lambda.x);
        lambda[3 * r + 1] = float(d.lambda.y);
        lambda[3 * r + 2] = float(d.lambda.z);
        penalty[3 * r] = float(d.penalty.x);
        penalty[3 * r + 1] = float(d.penalty.y);
        penalty[3 * r + 2] = float(d.penalty.z);
    }
}

template <class P, class R>
__global__ void k_pack_world(DevWorld<P, R> w, DioGpuBody* bodies, DioBodyState* st, double* p64, double* q64) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        A4<P> p = w.pos[0][i], q = w.rot[0][i];
        if (bodies) {
            DioGpuBody b;
            b.position[0] = float(p.x);
            b.position[1] = float(p.y);
            b.position[2] = float(p.z);
            b.position[3] = 0.f;
            b.orientation[0] = float(q.x);
            b.orientation[1] = float(q.y);
            b.orientation[2] = float(q.z);
            b.orientation[3] = float(q.w);
            b.shape = w.shape[i];
            bodies[i] = b;
        }
        if (st) {
            DioBodyState s;
            A4<P> v = w.vel[i], a = w.ang[i], pv = w.prev_vel[i];
            A4<R> inv = w.inv[i];
            s.vel[0] = float(v.x), s.vel[1] = float(v.y), s.vel[2] = float(v.z), s.vel[3] = 0.f;
            s.ang[0] = float(a.x), s.ang[1] = float(a.y), s.ang[2] = float(a.z), s.ang[3] = 0.f;
            s.prev_vel[0] = float(pv.x), s.prev_vel[1] = float(pv.y), s.prev_vel[2] = float(pv.z);
            s.prev_vel[3] = 0.f;
            s.inv_moment[0] = float(inv.x), s.inv_moment[1] = float(inv.y), s.inv_moment[2] = float(inv.z);
            s.inv_moment[3] = 0.f;
            s.inv_mass = float(inv.w);
            s.friction = float(w.friction[i]);
            s.pad[0] = s.pad[1] = 0.f;
            st[i] = s;
        }
        if (p64) {
            p64[3 * i] = double(p.x);
            p64[3 * i + 1] = double(p.y);
            p64[3 * i + 2] = double(p.z);
        }
        if (q64) {
            q64[4 * i] = double(q.x);
            q64[4 * i + 1] = double(q.y);
            q64[4 * i + 2] = double(q.z);
            q64[4 * i + 3] = double(q.w);
        }
    }
}

template <class P, class R>
__global__ void k_dyn_flags(DevWorld<P, R> w, uint32_t n, uint32_t* flags, uint32_t* keep) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t f = w.inv[i].w != R(0) ? 1u : 0u;
        flags[i] = f;
        keep[i] = f;
    }
}

// did the set of dynamic bodies change since the list was built?
template <class P, class R>
__global__ void k_dyn_changed(DevWorld<P, R> w, uint32_t n, const uint32_t* keep, uint32_t* changed) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if ((w.inv[i].w != R(0) ? 1u : 0u) != keep[i]) *changed = 1u;
}

static __global__ void k_dyn_fill(const uint32_t* flags, const uint32_t* pos, uint32_t n, uint32_t* list) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (flags[i]) list[pos[i]] = i;
}

// Work signature of a dynamic body for the primal's thread order: ball-socket
// incidences (three rows each) first, then distance joints, then the shape.
// Bodies with one signature run the same code path, so sorting the list by
// it keeps warps convergent; the Jacobi primal does not depend on the order.
// With `scene_chunk` set the key leads with the body's solve chunk, so each
// chunk's dynamic bodies form one signature-ordered run of the list.
template <class P, class R>
__global__ void k_dyn_keys(DevWorld<P, R> w, const uint32_t* list, uint32_t nd, const uint32_t* scene_chunk,
                           uint32_t* keys) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nd; t += gridDim.x * blockDim.x) {
        const uint32_t i = list[t];
        uint32_t nb = 0, nl = 0;
        if (w.n_joints)
            for (uint32_t k = w.joint_off[i]; k < w.joint_off[i + 1]; ++k) {
                if ((w.jview[k].kind & ~kIsB) == DIO_CONSTRAINT_BALL_SOCKET)
                    ++nb;
                else
                    ++nl;
            }
        nb = nb > 3u ? 3u : nb;
        nl = nl > 3u ? 3u : nl;
        const uint32_t tag = w.shape[i].tag > 7u ? 7u : w.shape[i].tag;
        const uint32_t chunk = scene_chunk ? scene_chunk[w.scene[i]] : 0u;
        keys[t] = (chunk << 7) | ((3u - nb) << 5) | ((3u - nl) << 3) | tag;
    }
}

// [first, last) of each solve chunk's run in the chunk-ordered dynamic-body
// list (runs start zeroed: a chunk without dynamic bodies keeps (0, 0))
template <class P, class R>
__global__ void k_chunk_dyn_runs(DevWorld<P, R> w, const uint32_t* list, uint32_t nd, const uint32_t* scene_chunk,
                                 uint2* runs) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nd; t += gridDim.x * blockDim.x) {
        const uint32_t c = scene_chunk[w.scene[list[t]]];
        if (t == 0 || scene_chunk[w.scene[list[t - 1]]] != c) runs[c].x = t;
        if (t + 1 == nd || scene_chunk[w.scene[list[t + 1]]] != c) runs[c].y = t + 1;
    }
}

// one JView per (body, joint) incidence in the body's joint-CSR order
static __global__ void k_build_jview(const DioConstraint* joints, const uint32_t* joff, const uint32_t* jidx,
                                     uint32_t n, JView* out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        for (uint32_t k = joff[i]; k < joff[i + 1]; ++k) {
            const DioConstraint j = joints[jidx[k]];
            const bool is_a = j.a == i;
            JView v;
            const float* sa = is_a ? j.anchor_a : j.anchor_b;
            const float* oa = is_a ? j.anchor_b : j.anchor_a;
            v.self_anchor = make_float4(sa[0], sa[1], sa[2], j.anchor_a[3]);
            v.other_anchor = make_float4(oa[0], oa[1], oa[2], j.anchor_b[3]);
            v.other = is_a ? j.b : j.a;
            v.kind = j.kind | (is_a ? 0u : kIsB);
            v.pad[0] = v.pad[1] = 0u;
            out[k] = v;
        }
    }
}

// joint incidences (body, joint id) for the per-body joint CSR
static __global__ void k_joint_inc(const DioConstraint* j, uint32_t nj, uint32_t n, uint32_t* body, uint32_t* id,
                            uint32_t* err) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nj; k += gridDim.x * blockDim.x) {
        uint32_t a = j[k].a, b = j[k].b;
        if (a >= n || b >= n) {
            atomicOr(err, kErrBadIndex);
            a = n;
            b = n;
        }
        body[2 * k] = a;
        id[2 * k] = k;
        body[2 * k + 1] = (b == a) ? n : b;
        id[2 * k + 1] = k;
    }
}

static __global__ void k_count_lt(const uint32_t* body, uint32_t total, uint32_t n, uint32_t* counts) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < total; j += gridDim.x * blockDim.x)
        if (body[j] < n) atomicAdd(&counts[body[j]], 1u);
}

static __global__ void k_scene_of(uint32_t* scene, const SceneDesc* sc, uint32_t ns) {
    uint32_t s = blockIdx.x;
    if (s >= ns) return;
    for (uint32_t i = sc[s].body_lo + threadIdx.x; i < sc[s].body_hi; i += blockDim.x) scene[i] = s;
}

static inline uint32_t bits_for(uint32_t v) {
    uint32_t b = 1;
    while (b < 32 && (1ull << b) <= v) ++b;
    return b;
}

template <class P, class R>
class Engine final : public EngineBase {
   public:
    Engine(const DioCapacity& cap, cudaStream_t s, const DioConfig& cfg) : cap_(cap), stream_(s), cfg_(cfg) {}
    ~Engine() override {
        drop_graphs();
        collect_spans();
        if (snap_) cudaFree(snap_);
        for (auto e : ev_free_) cudaEventDestroy(e);
        release();
    }

    int init() {
        const uint32_t N = std::max(1u, cap_.max_bodies);
        const uint32_t PP = std::max(1u, cap_.max_pairs);
        const uint32_t M = std::max(1u, cap_.max_contacts);
        const uint32_t J = std::max(1u, cap_.max_joints);
        const uint32_t S = std::max(1u, cap_.max_scenes);
        const uint32_t H = std::max(1u, cap_.max_hull_vertices);
        per_cap_ = cfg_.contacts_per_pair == 8 ? 8 : 4;
        for (int b = 0; b < 2; ++b) {
            DIO_TRY(alloc(&w_.pos[b], N));
            DIO_TRY(alloc(&w_.rot[b], N));
        }
        DIO_TRY(alloc(&w_.init_pos, N));
        DIO_TRY(alloc(&w_.init_rot, N));
        DIO_TRY(alloc(&w_.inert_pos, N));
        DIO_TRY(alloc(&w_.inert_rot, N));
        DIO_TRY(alloc(&w_.vel, N));
        DIO_TRY(alloc(&w_.ang, N));
        DIO_TRY(alloc(&w_.prev_vel, N));
        DIO_TRY(alloc(&w_.inv, N));
        DIO_TRY(alloc(&w_.mdt2, N));
        DIO_TRY(alloc(&w_.friction, N));
        DIO_TRY(alloc(&w_.shape, N));
        DIO_TRY(alloc(&w_.scene, N));
        DIO_TRY(alloc(&origin_, S));
        DIO_TRY(alloc(&walls_, 6ull * S));
        w_.walls = walls_;
        DIO_TRY(alloc(&w_.aabb_min, N));
        DIO_TRY(alloc(&w_.aabb_max, N));
        DIO_TRY(alloc(&w_.color, N));
        DIO_TRY(alloc(&w_.color_order, N));
        DIO_TRY(alloc(&w_.color_off, 1025));
        DIO_TRY(alloc(&w_.pairs, PP));
        DIO_TRY(alloc(&w_.slots, (size_t)PP * per_cap_));
        slots_[0] = w_.slots;  // slots_[1]: allocated when contact_lag is first used
        DIO_TRY(alloc(&w_.gjk_list, PP));
        DIO_TRY(alloc(&w_.epa_list, PP));
        DIO_TRY(alloc(&w_.simplex, (size_t)PP * 8));
        // LBVH
        DIO_TRY(alloc(&lb_bounds_, 6ull * S));
        DIO_TRY(alloc(&lb_keys_, N));
        DIO_TRY(alloc(&lb_keys_s_, N));
        DIO_TRY(alloc(&lb_vals_, N));
        DIO_TRY(alloc(&lb_leaf_, N));
        DIO_TRY(alloc(&lb_children_, N));
        DIO_TRY(alloc(&lb_parent_, 2ull * N));
        DIO_TRY(alloc(&lb_visits_, N));
        DIO_TRY(alloc(&lb_leaf_min_, N));
        DIO_TRY(alloc(&lb_leaf_max_, N));
        DIO_TRY(alloc(&lb_node_min_, N));
        DIO_TRY(alloc(&lb_node_max_, N));
        DIO_TRY(alloc(&lb_pb_, PP));
        DIO_TRY(alloc(&lb_gscratch_, PP));
        DIO_TRY(alloc(&lb_long_, N));
        DIO_TRY(alloc(&lb_long_count_, 1));
        for (int b = 0; b < 2; ++b) {
            DIO_TRY(alloc(&rs_[b], M));
            DIO_TRY(alloc(&rd_[b], M));
            DIO_TRY(alloc(&ab_[b], M));
            DIO_TRY(alloc(&keys_s_[b], M));
            DIO_TRY(alloc(&ids_s_[b], M));
        }
        DIO_TRY(alloc(&keys_raw_, M));
        DIO_TRY(alloc(&ids_raw_, M));
        const size_t INC = std::max<size_t>(2ull * M, 2ull * J);
        DIO_TRY(alloc(&inc_body_, INC));
        DIO_TRY(alloc(&inc_row_, INC));
        DIO_TRY(alloc(&inc_body_s_, INC));
        DIO_TRY(alloc(&inc_row_s_, INC));
        DIO_TRY(alloc(&w_.row_off, (size_t)N + 1));
        DIO_TRY(alloc(&w_.row_idx, 2ull * M));
        DIO_TRY(alloc(&w_.row_oth, 2ull * M));
        DIO_TRY(alloc(&joints_, J));
        DIO_TRY(alloc(&joint_off_, (size_t)N + 1));
        DIO_TRY(alloc(&joint_idx_, 2ull * J));
        DIO_TRY(alloc(&jview_, 2ull * J));
        DIO_TRY(alloc(&dyn_list_, N));
        DIO_TRY(alloc(&dyn_tmp_, N));
        DIO_TRY(alloc(&dyn_keep_, N));
        DIO_TRY(alloc(&color_hist_, kMaxColors + 2));
        const size_t CNT = std::max<size_t>(std::max<size_t>(N, (size_t)PP * per_cap_), 2ull * M) + 2;
        DIO_TRY(alloc(&counts_, CNT));
        DIO_TRY(alloc(&offsets_, CNT));
        DIO_TRY(alloc(&counts2_, (size_t)N + 2));
        DIO_TRY(alloc(&offsets2_, (size_t)N + 2));
        DIO_TRY(alloc(&scenes_, S));
        DIO_TRY(alloc(&chunks_, S));
        DIO_TRY(alloc(&solve_chunks_, S));
        DIO_TRY(alloc(&chunk_dyn_, S));
        DIO_TRY(alloc(&scene_chunk_, S));
        DIO_TRY(alloc(&chunk_n_, S));
        DIO_TRY(alloc(&chunk_ovf_, S));
        DIO_TRY(alloc(&chunk_tot_, S));
        // pair scratch of the shared-memory trees: scratch_k_ slots per body
        scratch_k_ = (uint32_t)std::min<uint64_t>(8, std::max<uint64_t>(2, 2 * ((uint64_t)PP + N - 1) / N));
        DIO_TRY(alloc(&tree_scratch_, (size_t)N * scratch_k_));
        DIO_TRY(alloc(&hull_, H));
        DIO_TRY(alloc(&ctr_, 1));
        DIO_CK(cudaMallocHost(&hctr_, sizeof(Counters)));
        // prefix sums and radix sorts: up to CNT scanned counts, and sorts of
        // row keys (M), incidences (INC) and per-body keys (N)
        DIO_CK(ss_.init((uint32_t)std::max<size_t>(std::max<size_t>(M, N), INC),
                        (uint32_t)std::max<size_t>(CNT, (size_t)kMaxColors + 2), &ctr_->error_flags, stream_));
        ss_.counter = &launches_;  // the scans and sorts count as the step's kernels
        // API staging (device + pinned host)
        stage_bytes_ = (size_t)N * (sizeof(DioGpuBody) + sizeof(DioBodyState) + 64 + 16) + (size_t)M * sizeof(DioContact) +
                       (size_t)J * sizeof(DioConstraint) + ((size_t)N + 1) * 4 + 2ull * M * 4 +
                       (size_t)PP * per_cap_ * sizeof(DioContactOut) + (size_t)PP * sizeof(DioPair) +
                       (size_t)M * 24 + 4096;
        DIO_CK(cudaMalloc(&dstage_, stage_bytes_));
        DIO_CK(cudaMallocHost(&hstage_, stage_bytes_));
        DIO_CK(cudaMemsetAsync(ctr_, 0, sizeof(Counters), stream_));
        DIO_CK(cudaMemsetAsync(joint_off_, 0, ((size_t)N + 1) * 4, stream_));
        w_.origin = nullptr;
        w_.hull = hull_;
        w_.max_pairs = PP;
        w_.per_pair = per_cap_;
        w_.epa_wait_polls = (cfg_.debug_flags & DIO_DEBUG_EPA_NO_FIRST_WAIT) ? 0u : kEpaWaitPolls;
        w_.max_rows = M;
        w_.max_incid = 2 * M;
        w_.joints = joints_;
        w_.joint_off = joint_off_;
        w_.joint_idx = joint_idx_;
        w_.n_joints = 0;
        w_.scenes = scenes_;
        w_.n_scenes = 0;
        w_.ctr = ctr_;
        w_.n = 0;
        set_rows(0);
        int dev = 0;
        DIO_CK(cudaGetDevice(&dev));
        DIO_CK(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev));
        DIO_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&dual_ctas_per_sm_, k_dual<P, R>, 256, 0));
        dual_ctas_per_sm_ = std::max(1, dual_ctas_per_sm_);
        const int tree_bytes = (int)scene_tree_bytes<R>(scene_tree_cap<R>());
        DIO_CK(cudaFuncSetAttribute(k_scene_tree<R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, tree_bytes));
        DIO_CK(cudaFuncSetAttribute(k_scene_tree<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, tree_bytes));
        DIO_CK(cudaFuncSetAttribute(k_chunk_build<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)chunk_build_bytes<R>()));
        DIO_CK(cudaFuncSetAttribute(k_primal_warp<P, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)primal_warp_smem<R>()));
        DIO_CK(cudaFuncSetAttribute(k_primal_color_warp<P, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)primal_warp_smem<R>()));
        DIO_CK(cudaFuncSetAttribute(k_solve_chunks<P, R, kChunkThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)chunk_smem_bytes<P>(solve_chunk_cap<P>())));
        DIO_CK(cudaFuncSetAttribute(k_solve_chunks<P, R, kChunkThreadsWide>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)chunk_smem_bytes<P>(solve_chunk_cap<P>())));
        DIO_CK(cudaFuncSetAttribute(k_solve_chunks_colored<P, R, kChunkThreads>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)chunk_colored_smem_bytes<P>(solve_chunk_cap<P>())));
        DIO_CK(cudaFuncSetAttribute(k_solve_chunks_colored<P, R, kChunkThreadsWide>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)chunk_colored_smem_bytes<P>(solve_chunk_cap<P>())));
        return DIO_OK;
    }
    // largest scene, and the chunks of consecutive scenes (each of at most
    // scene_tree_cap bodies, packed up to that many) for k_scene_tree
    // Consecutive scenes packed into chunks of at most `cap` bodies (scenes
    // larger than cap are left out), largest chunks first: CTAs start in
    // chunk order, so the last wave holds the short ones.  Returns the
    // bodies of the largest chunk.
    uint32_t pack_chunks(uint32_t cap, std::vector<uint2>& out) const {
        out.clear();
        uint32_t open_bodies = 0, largest = 0;
        bool open = false;
        auto close = [&](uint32_t end) {
            if (!open) return;
            out.back().y = end;
            largest = std::max(largest, open_bodies);
            open = false;
        };
        for (uint32_t s = 0; s < (uint32_t)scenes_host_.size(); ++s) {
            const uint32_t sz = scenes_host_[s].body_hi - scenes_host_[s].body_lo;
            if (sz > cap) {
                close(s);
                continue;
            }
            if (open && open_bodies + sz > cap) close(s);
            if (!open) {
                out.push_back(make_uint2(s, s));
                open_bodies = 0;
                open = true;
            }
            open_bodies += sz;
        }
        close((uint32_t)scenes_host_.size());
        auto bodies_of = [&](const uint2& c) { return scenes_host_[c.y - 1].body_hi - scenes_host_[c.x].body_lo; };
        std::stable_sort(out.begin(), out.end(),
                         [&](const uint2& a, const uint2& b) { return bodies_of(a) > bodies_of(b); });
        return largest;
    }
    // Chunks of the scene-chunk solve.  It runs one CTA per chunk and one CTA
    // per SM, so it takes about (waves) x (largest chunk): for k = 1, 2, ...
    // waves the smallest chunk size that packs every scene into at most k x
    // SMs chunks (greedy over consecutive scenes) is found by bisection, and
    // the k with the smallest k x size wins.  Returns the largest chunk's
    // bodies (0: some scene exceeds solve_chunk_cap).
    uint32_t pack_solve_chunks() {
        const uint32_t cap = solve_chunk_cap<P>();
        uint32_t largest = 0;
        for (const SceneDesc& sd : scenes_host_) largest = std::max(largest, sd.body_hi - sd.body_lo);
        solve_chunks_host_.clear();
        if (scenes_host_.empty() || largest == 0 || largest > cap) return 0;
        auto count_at = [&](uint32_t m) {
            uint64_t count = 0, open = 0;
            for (const SceneDesc& sd : scenes_host_) {
                const uint32_t sz = sd.body_hi - sd.body_lo;
                if (!count || open + sz > m) {
                    ++count;
                    open = 0;
                }
                open += sz;
            }
            return count;
        };
        const uint64_t sm = (uint64_t)std::max(1, sms_);
        uint64_t best_cost = ~0ull;
        uint32_t best_m = cap;
        for (uint64_t k = 1; k <= 64; ++k) {
            if (count_at(cap) > k * sm) continue;
            uint32_t lo = largest, hi = cap;  // the smallest size with at most k x SMs chunks
            while (lo < hi) {
                const uint32_t mid = lo + (hi - lo) / 2;
                if (count_at(mid) <= k * sm)
                    hi = mid;
                else
                    lo = mid + 1;
            }
            if (k * lo < best_cost) {
                best_cost = k * lo;
                best_m = lo;
            }
            if (lo == largest || k * sm >= scenes_host_.size()) break;  // more waves cannot help
        }
        return pack_chunks(best_m, solve_chunks_host_);
    }
    // largest scene; the chunks of the broad phase's shared-memory trees
    // (scene_tree_cap<R> bodies) and of the scene-chunk solve
    // (solve_chunk_cap<P> bodies)
    int note_scene_sizes() {
        scene_max_ = 0;
        for (const SceneDesc& sd : scenes_host_) scene_max_ = std::max(scene_max_, sd.body_hi - sd.body_lo);
        chunk_max_ = pack_chunks(scene_tree_cap<R>(), chunks_host_);
        solve_chunk_max_ = pack_solve_chunks();
        // solve chunk of every scene (when every scene has one)
        chunked_scenes_ = !solve_chunks_host_.empty() && scene_max_ <= solve_chunk_cap<P>();
        if (chunked_scenes_) {
            std::vector<uint32_t> sch(scenes_host_.size(), 0u);
            for (uint32_t c = 0; c < (uint32_t)solve_chunks_host_.size(); ++c)
                for (uint32_t sc = solve_chunks_host_[c].x; sc < solve_chunks_host_[c].y; ++sc) sch[sc] = c;
            DIO_CK(cudaMemcpyAsync(scene_chunk_, sch.data(), sch.size() * 4, cudaMemcpyHostToDevice, stream_));
            DIO_CK(cudaStreamSynchronize(stream_));  // sch is a host temporary
        }
        if (!chunks_host_.empty())
            DIO_CK(cudaMemcpyAsync(chunks_, chunks_host_.data(), chunks_host_.size() * sizeof(uint2),
                                   cudaMemcpyHostToDevice, stream_));
        if (!solve_chunks_host_.empty())
            DIO_CK(cudaMemcpyAsync(solve_chunks_, solve_chunks_host_.data(),
                                   solve_chunks_host_.size() * sizeof(uint2), cudaMemcpyHostToDevice, stream_));
        return DIO_OK;
    }

    void set_stream(cudaStream_t s) override { stream_ = s; }
    void set_config(const DioConfig& c) override {
        drop_graphs();
        uint32_t per = cfg_.contacts_per_pair;
        cfg_ = c;
        if (c.contacts_per_pair != 4 && c.contacts_per_pair != 8) cfg_.contacts_per_pair = per;
        if (cfg_.contacts_per_pair > per_cap_) cfg_.contacts_per_pair = per_cap_;
        // lagged rows need the previous step's slots in this layout
        if (cfg_.contacts_per_pair != per || !cfg_.contact_lag) lag_primed_ = false;
        w_.epa_wait_polls = (cfg_.debug_flags & DIO_DEBUG_EPA_NO_FIRST_WAIT) ? 0u : kEpaWaitPolls;
    }

    // ------------------------------------------------ reference-mirror API
    int broad_submit(const DioGpuBody* bodies, uint32_t n) override {
        if (n > cap_.max_bodies) return cap_err("too many bodies for the compute buffers");
        api_bodies_ = n;
        if (n == 0) {
            DIO_CK(cudaMemsetAsync(ctr_, 0, sizeof(Counters), stream_));
            return DIO_OK;
        }
        DIO_TRY(upload_bodies(bodies, n, n_hull_));
        DIO_TRY(single_scene(n, nullptr));
        DIO_CK(cudaMemsetAsync(ctr_, 0, sizeof(Counters), stream_));
        rebuild_now_ = true;
        lbvh_valid_ = false;
        return run_broad(0, n);
    }
    int pair_count(uint32_t* count) override {
        if (!count) return inval("null count");
        DIO_TRY(pull_counters());
        *count = hctr_->pairs;
        if (hctr_->pairs > cap_.max_pairs) return cap_err("broad phase found more pairs than max_pairs");
        return DIO_OK;
    }
    int read_pairs(DioPair* out, uint32_t cap, uint32_t* n) override {
        DIO_TRY(pull_counters());
        uint32_t c = std::min(hctr_->pairs, cap_.max_pairs);
        if (n) *n = c;
        uint32_t k = std::min(c, cap);
        if (k && out) {
            DIO_CK(cudaMemcpyAsync(out, w_.pairs, (size_t)k * sizeof(DioPair), cudaMemcpyDeviceToHost, stream_));
            DIO_CK(cudaStreamSynchronize(stream_));
        }
        return c > cap ? cap_err("output buffer smaller than the pair count") : DIO_OK;
    }
    int narrow_submit_pairs(const DioGpuBody* bodies, uint32_t n, const DioPair* pairs, uint32_t np) override {
        if (n > cap_.max_bodies) return cap_err("too many bodies for the compute buffers");
        if (np > cap_.max_pairs) return cap_err("too many pairs for the compute buffers");
        last_np_ = np;
        if (np == 0) return DIO_OK;
        DIO_TRY(upload_bodies(bodies, n, n_hull_));
        api_bodies_ = n;
        DIO_TRY(single_scene(n, nullptr));
        DIO_CK(cudaMemcpyAsync(w_.pairs, pairs, (size_t)np * sizeof(DioPair), cudaMemcpyHostToDevice, stream_));
        DIO_CK(cudaMemsetAsync(ctr_, 0, sizeof(Counters), stream_));
        return run_narrow(np, nullptr);
    }
    int narrow_submit(uint32_t np) override {
        if (np > cap_.max_pairs) return cap_err("too many pairs for the compute buffers");
        last_np_ = np;
        if (np == 0) return DIO_OK;
        DIO_CK(cudaMemsetAsync(&ctr_->gjk_work, 0, 2 * sizeof(uint32_t), stream_));
        return run_narrow(np, nullptr);
    }
    int narrow_read(DioContactOut* out, uint32_t cap, uint32_t* n) override {
        uint32_t slots = last_np_ * cfg_.contacts_per_pair;
        if (n) *n = slots;
        if (slots > cap) return cap_err("output buffer smaller than the slot count");
        if (slots == 0) return DIO_OK;
        if (sizeof(R) == 4 && cfg_.contacts_per_pair == w_.per_pair) {
            DIO_CK(cudaMemcpyAsync(out, w_.slots, (size_t)slots * sizeof(DioContactOut), cudaMemcpyDeviceToHost,
                                   stream_));
        } else {
            return inval("narrow_read needs an FP32 engine");
        }
        DIO_CK(cudaStreamSynchronize(stream_));
        DIO_TRY(check_flags());
        return DIO_OK;
    }
    int set_hull(const float* xyzw, uint32_t count) override {
        if (count > cap_.max_hull_vertices) return cap_err("too many hull vertices");
        if (count == 0) {
            n_hull_ = 0;
            return DIO_OK;
        }
        std::vector<A4<R>> tmp(count);
        for (uint32_t i = 0; i < count; ++i)
            tmp[i] = A4<R>{R(xyzw[4 * i]), R(xyzw[4 * i + 1]), R(xyzw[4 * i + 2]), R(0)};
        DIO_CK(cudaMemcpyAsync(hull_, tmp.data(), count * sizeof(A4<R>), cudaMemcpyHostToDevice, stream_));
        DIO_CK(cudaStreamSynchronize(stream_));
        n_hull_ = count;
        return DIO_OK;
    }

    int prepare_contacts(const DioGpuBody* bodies, const DioBodyState* state, uint32_t n, const DioContactOut* slots,
                         uint32_t n_slots, const DioContact* prev, uint32_t n_prev, const DioContainer* container,
                         const DioAvbdOptions* options, DioContact* out, uint32_t cap, uint32_t* m, uint32_t* offsets,
                         uint32_t* indices, uint32_t index_cap) override {
        if (!options || (n && (!bodies || !state))) return inval("null argument");
        if (n > cap_.max_bodies) return cap_err("too many bodies");
        if ((uint64_t)n_slots > (uint64_t)cap_.max_pairs * per_cap_) return cap_err("too many slots");
        if (n_prev > cap_.max_contacts) return cap_err("too many previous contacts");
        if constexpr (sizeof(R) != 4) {
            return inval("prepare_contacts needs an FP32 engine");
        } else {
            DIO_TRY(upload_bodies(bodies, n, n_hull_));
            DIO_TRY(upload_state(state, n));
            DIO_TRY(single_scene(n, container));
            DIO_CK(cudaMemsetAsync(ctr_, 0, sizeof(Counters), stream_));
            // previous rows into the "previous" buffer, then their sorted keys
            int pb = 1 - cur_;
            if (n_prev) {
                DioContact* dprev = reinterpret_cast<DioContact*>(dstage_);
                DIO_CK(cudaMemcpyAsync(dprev, prev, (size_t)n_prev * sizeof(DioContact), cudaMemcpyHostToDevice, stream_));
                k_unpack_contacts<P, R><<<grid_for(n_prev, 256), 256, 0, stream_>>>(rs_[pb], rd_[pb], ab_[pb], dprev,
                                                                                    n_prev, 0xFFFFFFFFu, &ctr_->error_flags);
                DIO_TRY(sort_keys(ab_[pb], n_prev, keys_s_[pb], ids_s_[pb]));
            }
            n_prev_rows_ = n_prev;
            // slots -> device (FP32 slots are DioContactOut bytes)
            if (n_slots)
                DIO_CK(cudaMemcpyAsync(w_.slots, slots, (size_t)n_slots * sizeof(DioContactOut), cudaMemcpyHostToDevice,
                                       stream_));
            DIO_TRY(build_rows(opts_prep(*options), n_slots, 1, nullptr, n));
            DIO_TRY(pull_counters());
            uint32_t M = hctr_->rows;
            *m = M;
            DIO_TRY(finish_rows(opts_prep(*options), M, n));
            uint32_t ninc = 0;
            DIO_CK(cudaMemcpyAsync(&ninc, w_.row_off + n, 4, cudaMemcpyDeviceToHost, stream_));
            DIO_CK(cudaStreamSynchronize(stream_));
            DIO_TRY(check_flags());
            if (M > cap || ninc > index_cap) return cap_err("output buffers smaller than the rows / CSR");
            DioContact* dout = reinterpret_cast<DioContact*>(dstage_);
            k_pack_contacts<P, R><<<grid_for(M, 256), 256, 0, stream_>>>(w_.rs, w_.rd, w_.ab, dout, &ctr_->rows);
            if (M) DIO_CK(cudaMemcpyAsync(out, dout, (size_t)M * sizeof(DioContact), cudaMemcpyDeviceToHost, stream_));
            DIO_CK(cudaMemcpyAsync(offsets, w_.row_off, ((size_t)n + 1) * 4, cudaMemcpyDeviceToHost, stream_));
            if (ninc) DIO_CK(cudaMemcpyAsync(indices, w_.row_idx, (size_t)ninc * 4, cudaMemcpyDeviceToHost, stream_));
            DIO_CK(cudaStreamSynchronize(stream_));
            cur_ = 1 - cur_;
            set_rows(cur_);
            return DIO_OK;
        }
    }

    int avbd_submit(const DioBodyState* state, const float* positions, const float* orientations, uint32_t n,
                    const DioContact* contacts, uint32_t m, const DioConstraint* constraints, uint32_t nj,
                    const uint32_t* offsets, const uint32_t* indices, const DioRunOptions* options) override {
        if (!options) return inval("null options");
        if (n > cap_.max_bodies) return cap_err("too many bodies for the AVBD buffers");
        if (m > cap_.max_contacts) return cap_err("too many contacts for the AVBD buffers");
        if (nj > cap_.max_joints) return cap_err("too many constraints for the AVBD buffers");
        api_n_ = n;
        api_m_ = m;
        api_iters_ = options->iterations;
        if (n == 0) return DIO_OK;
        if (!state || !positions || !orientations || !offsets || (m && !contacts) || (nj && !constraints))
            return inval("null argument");
        uint32_t ninc = offsets[n];
        if (ninc > 2ull * cap_.max_contacts) return cap_err("too many CSR indices");
        if (ninc && !indices) return inval("null indices");
        w_.n_joints = 0;  // this call's joints are uploaded below
        DIO_TRY(upload_state(state, n));
        // poses
        char* st = reinterpret_cast<char*>(dstage_);
        float* dpos = reinterpret_cast<float*>(st);
        float* dq = dpos + 3 * (size_t)n;
        DIO_CK(cudaMemcpyAsync(dpos, positions, (size_t)n * 12, cudaMemcpyHostToDevice, stream_));
        DIO_CK(cudaMemcpyAsync(dq, orientations, (size_t)n * 16, cudaMemcpyHostToDevice, stream_));
        k_unpack_pose3<P, R><<<grid_for(n, 256), 256, 0, stream_>>>(w_, dpos, dq, n);
        DIO_CK(cudaMemsetAsync(ctr_, 0, sizeof(Counters), stream_));
        // rows
        w_.n = n;
        if (m) {
            DioContact* dc = reinterpret_cast<DioContact*>(st + align256((size_t)n * 28));
            DIO_CK(cudaMemcpyAsync(dc, contacts, (size_t)m * sizeof(DioContact), cudaMemcpyHostToDevice, stream_));
            k_unpack_contacts<P, R><<<grid_for(m, 256), 256, 0, stream_>>>(w_.rs, w_.rd, w_.ab, dc, m, n,
                                                                           &ctr_->error_flags);
        }
        DIO_CK(cudaMemcpyAsync(w_.row_off, offsets, ((size_t)n + 1) * 4, cudaMemcpyHostToDevice, stream_));
        if (ninc) DIO_CK(cudaMemcpyAsync(w_.row_idx, indices, (size_t)ninc * 4, cudaMemcpyHostToDevice, stream_));
        k_csr_other<<<grid_for(n, 128), 128, 0, stream_>>>(w_.row_off, w_.row_idx, w_.ab, w_.row_oth, n, m,
                                                          &ctr_->error_flags);
        DIO_TRY(upload_joints(constraints, nj, n));
        k_set_u32<<<1, 1, 0, stream_>>>(&ctr_->rows, m);
        SolveParams<R> o = solve_params(options->dt, options->gravity, options->alpha, options->beta_lin,
                                        options->penalty_max, options->iterations);
        DIO_TRY(solve(o, n, m));
        return DIO_OK;
    }

    int avbd_read(const DioAvbdResult* out) override {
        if (!out) return inval("null result");
        uint32_t n = api_n_, m = api_m_;
        if (n == 0) return DIO_OK;
        uint32_t fp_read = (api_iters_ == 0 ? 0u : api_iters_ - 1u) % 2u;
        int buf = 1 - (int)fp_read;
        size_t nb = (size_t)n * 4 * (3 + 4 + 3 + 3 + 3);
        size_t mb = (size_t)m * 4 * 6;
        float* d = reinterpret_cast<float*>(dstage_);
        float *dp = d, *dqq = dp + 3 * (size_t)n, *dv = dqq + 4 * (size_t)n, *da = dv + 3 * (size_t)n,
              *dpv = da + 3 * (size_t)n, *dl = dpv + 3 * (size_t)n, *dk = dl + 3 * (size_t)m;
        k_pack_result<P, R><<<grid_for(n, 256), 256, 0, stream_>>>(w_, n, buf, dp, dqq, dv, da, dpv);
        if (m) k_pack_dual<P, R><<<grid_for(m, 256), 256, 0, stream_>>>(w_.rd, m, dl, dk);
        DIO_CK(cudaMemcpyAsync(hstage_, d, nb + mb, cudaMemcpyDeviceToHost, stream_));
        DIO_CK(cudaStreamSynchronize(stream_));
        DIO_TRY(check_flags());
        const float* h = reinterpret_cast<const float*>(hstage_);
        const float *hp = h, *hq = hp + 3 * (size_t)n, *hv = hq + 4 * (size_t)n, *ha = hv + 3 * (size_t)n,
                    *hpv = ha + 3 * (size_t)n, *hl = hpv + 3 * (size_t)n, *hk = hl + 3 * (size_t)m;
        if (out->positions) std::memcpy(out->positions, hp, (size_t)n * 12);
        if (out->orientations) std::memcpy(out->orientations, hq, (size_t)n * 16);
        if (out->velocities) std::memcpy(out->velocities, hv, (size_t)n * 12);
        if (out->angular_velocities) std::memcpy(out->angular_velocities, ha, (size_t)n * 12);
        if (out->prev_velocities) std::memcpy(out->prev_velocities, hpv, (size_t)n * 12);
        if (out->lambda && m) std::memcpy(out->lambda, hl, (size_t)m * 12);
        if (out->penalty && m) std::memcpy(out->penalty, hk, (size_t)m * 12);
        return DIO_OK;
    }

    // ------------------------------------------------------------- world
    int world_upload(const DioWorldDesc* d) override {
        if (!d) return inval("null world");
        uint32_t n = d->n_bodies;
        if (n > cap_.max_bodies) return cap_err("too many bodies");
        if (d->n_constraints > cap_.max_joints) return cap_err("too many constraints");
        uint32_t ns = d->n_scenes == 0 ? 1 : d->n_scenes;
        if (ns > cap_.max_scenes) return cap_err("too many scenes");
        if (d->n_hull_vertices > cap_.max_hull_vertices) return cap_err("too many hull vertices");
        if (n && (!d->bodies || !d->state)) return inval("null bodies/state");
        if (d->n_hull_vertices && !d->hull_vertices) return inval("null hull vertices");
        if (n && !hull_ranges_ok(d->bodies, n, d->n_hull_vertices))
            return inval("hull vertex range beyond the hull-vertex pool");
        drop_graphs();
        lbvh_valid_ = false;
        w_.n_joints = 0;  // the world's joints are uploaded below
        DIO_TRY(upload_bodies(d->bodies, n, d->n_hull_vertices));
        if (d->positions_f64 || d->orientations_f64) {
            double* dp = reinterpret_cast<double*>(dstage_);
            double* dq = dp + 3 * (size_t)n;
            if (d->positions_f64)
                DIO_CK(cudaMemcpyAsync(dp, d->positions_f64, (size_t)n * 24, cudaMemcpyHostToDevice, stream_));
            if (d->orientations_f64)
                DIO_CK(cudaMemcpyAsync(dq, d->orientations_f64, (size_t)n * 32, cudaMemcpyHostToDevice, stream_));
            k_unpack_pose_f64<P, R><<<grid_for(n, 256), 256, 0, stream_>>>(
                w_, d->positions_f64 ? dp : nullptr, d->orientations_f64 ? dq : nullptr, n);
        }
        DIO_TRY(upload_state(d->state, n));
        // scenes
        std::vector<SceneDesc> sc(ns);
        std::vector<A4<P>> org(ns);
        for (uint32_t s = 0; s < ns; ++s) {
            SceneDesc& x = sc[s];
            std::memset(&x, 0, sizeof x);
            x.body_lo = (d->scene_offsets && d->n_scenes) ? d->scene_offsets[s] : 0;
            x.body_hi = (d->scene_offsets && d->n_scenes) ? d->scene_offsets[s + 1] : n;
            if (x.body_hi < x.body_lo || x.body_hi > n) return inval("bad scene offsets");
            x.rotation[3] = 1.f;
            org[s] = A4<P>{P(0), P(0), P(0), P(0)};
            if (d->containers) {
                const DioContainer& c = d->containers[s];
                x.has_container = 1;
                std::memcpy(x.center, c.center, 12);
                x.half_extent = c.half_extent;
                std::memcpy(x.rotation, c.rotation, 16);
                if (cfg_.precision == DIO_PREC_SPLIT) org[s] = A4<P>{P(c.center[0]), P(c.center[1]), P(c.center[2]), P(0)};
            }
        }
        scenes_host_ = sc;
        DIO_TRY(note_scene_sizes());
        DIO_CK(cudaMemcpyAsync(scenes_, sc.data(), ns * sizeof(SceneDesc), cudaMemcpyHostToDevice, stream_));
        DIO_CK(cudaMemcpyAsync(origin_, org.data(), ns * sizeof(A4<P>), cudaMemcpyHostToDevice, stream_));
        w_.origin = cfg_.precision == DIO_PREC_SPLIT ? origin_ : nullptr;
        k_scene_walls<P, R><<<grid_for(6ull * ns, 128), 128, 0, stream_>>>(w_, scenes_, ns, walls_);
        w_.n_scenes = ns;
        k_scene_of<<<ns, 128, 0, stream_>>>(w_.scene, scenes_, ns);
        n_hull_ = d->n_hull_vertices;
        if (d->n_hull_vertices) {
            std::vector<A4<R>> hv(d->n_hull_vertices);
            for (uint32_t i = 0; i < d->n_hull_vertices; ++i)
                hv[i] = A4<R>{R(d->hull_vertices[4 * i]), R(d->hull_vertices[4 * i + 1]),
                              R(d->hull_vertices[4 * i + 2]), R(0)};
            DIO_CK(cudaMemcpyAsync(hull_, hv.data(), hv.size() * sizeof(A4<R>), cudaMemcpyHostToDevice, stream_));
            DIO_CK(cudaStreamSynchronize(stream_));
        }
        w_.n = n;
        DIO_CK(cudaMemsetAsync(ctr_, 0, sizeof(Counters), stream_));
        DIO_TRY(upload_joints(d->constraints, d->n_constraints, n));
        // the scene-chunk solve needs every scene in a chunk and every joint
        // inside one scene (a chunk's shared memory holds its own bodies only)
        chunk_world_ = n && chunked_scenes_ &&
                       joints_within_scenes(d->constraints, d->n_constraints);
        n_prev_rows_ = 0;
        steps_ = 0;
        lag_primed_ = false;
        world_ready_ = true;
        DIO_CK(cudaStreamSynchronize(stream_));
        return check_flags();
    }

    int step(const DioAvbdOptions* options, uint32_t steps) override {
        DIO_TRY(step_async(options, steps));
        // one synchronisation per call: device-side error flags
        return check_flags();
    }
    int step_async(const DioAvbdOptions* options, uint32_t steps) override {
        if (!options) return inval("null options");
        if (!world_ready_) return state_err("no world uploaded");
        if (cfg_.contact_lag) {
            if (!slots_[1]) DIO_TRY(alloc(&slots_[1], (size_t)cap_.max_pairs * per_cap_));
            if (!lag_primed_) {
                // first lagged step: no previous detection (the roll at the
                // step's start turns this count into the previous one)
                k_set_u32<<<1, 1, 0, stream_>>>(&ctr_->pairs, 0u);
                lag_primed_ = true;
            }
        } else {
            lag_primed_ = false;
        }
        for (uint32_t k = 0; k < steps; ++k) {
            if (cfg_.solver_mode == DIO_SOLVER_COLORED && !use_chunk_solve())
                DIO_TRY(step_once_colored(*options));
            else if (cfg_.use_graph)
                DIO_TRY(step_graph(*options));
            else
                DIO_TRY(step_once_dev(*options));
        }
        return DIO_OK;
    }
    int sync_check() override { return check_flags(); }

    int set_state(const DioGpuBody* bodies, const DioBodyState* state) override {
        DIO_TRY(set_state_begin(bodies, state));
        return set_state_end();
    }
    int set_state_begin(const DioGpuBody* bodies, const DioBodyState* state) override {
        if (!world_ready_) return state_err("no world uploaded");
        if (state_pending_) return state_err("set_state_begin twice without set_state_end");
        uint32_t n = w_.n;
        if (bodies) {
            DioGpuBody* db = reinterpret_cast<DioGpuBody*>(dstage_);
            DIO_CK(cudaMemcpyAsync(db, bodies, (size_t)n * sizeof(DioGpuBody), cudaMemcpyHostToDevice, stream_));
            k_set_pose<P, R><<<grid_for(n, 256), 256, 0, stream_>>>(w_, db, n);
            ++launches_;
        }
        if (state && n) {
            DioBodyState* ds = reinterpret_cast<DioBodyState*>(reinterpret_cast<char*>(dstage_) +
                                                               align256((size_t)n * sizeof(DioGpuBody)));
            DIO_CK(cudaMemcpyAsync(ds, state, (size_t)n * sizeof(DioBodyState), cudaMemcpyHostToDevice, stream_));
            k_unpack_state<P, R><<<grid_for(n, 256), 256, 0, stream_>>>(w_, ds, n);
            ++launches_;
            if (dyn_list_n_ == n) {
                // the list is kept unless a body turned static or dynamic
                DIO_CK(cudaMemsetAsync(&ctr_->dyn_changed, 0, 4, stream_));
                k_dyn_changed<P, R><<<grid_for(n, 256), 256, 0, stream_>>>(w_, n, dyn_keep_, &ctr_->dyn_changed);
                DIO_CK(cudaMemcpyAsync(&hctr_->dyn_changed, &ctr_->dyn_changed, 4, cudaMemcpyDeviceToHost, stream_));
                state_pending_ = 1;
            } else {
                state_pending_ = 2;
            }
        }
        return DIO_OK;
    }
    int set_state_end() override {
        int pending = state_pending_;
        state_pending_ = 0;
        if (pending == 1) {
            DIO_CK(cudaStreamSynchronize(stream_));
            if (!hctr_->dyn_changed) return DIO_OK;
        }
        if (pending) return build_dyn_list(w_.n);
        return DIO_OK;
    }

    int set_motion(const DioBodyMotion* motion) override {
        if (!world_ready_) return state_err("no world uploaded");
        if (!motion) return inval("null motion records");
        const uint32_t n = w_.n;
        if (!n) return DIO_OK;
        DioBodyMotion* dm = reinterpret_cast<DioBodyMotion*>(dstage_);
        DIO_CK(cudaMemcpyAsync(dm, motion, (size_t)n * sizeof(DioBodyMotion), cudaMemcpyHostToDevice, stream_));
        k_unpack_motion<P, R><<<grid_for(n, 256), 256, 0, stream_>>>(w_, dm, n);
        ++launches_;
        return DIO_OK;
    }
    int download_motion_async(DioBodyMotion* motion) override {
        if (!world_ready_) return state_err("no world uploaded");
        if (!motion) return inval("null motion records");
        const uint32_t n = w_.n;
        if (!n) return DIO_OK;
        // staged behind the upload's half of the staging buffer, so a
        // read-back and the next frame's upload never share bytes
        DioBodyMotion* dm = reinterpret_cast<DioBodyMotion*>(reinterpret_cast<char*>(dstage_) +
                                                             align256((size_t)n * sizeof(DioBodyMotion)));
        k_pack_motion<P, R><<<grid_for(n, 256), 256, 0, stream_>>>(w_, dm, n);
        ++launches_;
        DIO_CK(cudaMemcpyAsync(motion, dm, (size_t)n * sizeof(DioBodyMotion), cudaMemcpyDeviceToHost, stream_));
        return DIO_OK;
    }

    int download(DioGpuBody* bodies, DioBodyState* state) override {
        DIO_TRY(download_async(bodies, state));
        DIO_CK(cudaStreamSynchronize(stream_));
        return DIO_OK;
    }
    int download_async(DioGpuBody* bodies, DioBodyState* state) override {
        if (!world_ready_) return state_err("no world uploaded");
        uint32_t n = w_.n;
        if (!n) return DIO_OK;
        DioGpuBody* db = reinterpret_cast<DioGpuBody*>(dstage_);
        DioBodyState* ds = reinterpret_cast<DioBodyState*>(reinterpret_cast<char*>(dstage_) +
                                                           align256((size_t)n * sizeof(DioGpuBody)));
        k_pack_world<P, R><<<grid_for(n, 256), 256, 0, stream_>>>(w_, bodies ? db : nullptr, state ? ds : nullptr,
                                                                  nullptr, nullptr);
        if (bodies) DIO_CK(cudaMemcpyAsync(bodies, db, (size_t)n * sizeof(DioGpuBody), cudaMemcpyDeviceToHost, stream_));
        if (state) DIO_CK(cudaMemcpyAsync(state, ds, (size_t)n * sizeof(DioBodyState), cudaMemcpyDeviceToHost, stream_));
        return DIO_OK;
    }

    int download_f64(double* positions, double* orientations) override {
        if (!world_ready_) return state_err("no world uploaded");
        uint32_t n = w_.n;
        if (!n) return DIO_OK;
        double* dp = reinterpret_cast<double*>(dstage_);
        double* dq = dp + 3 * (size_t)n;
        k_pack_world<P, R><<<grid_for(n, 256), 256, 0, stream_>>>(w_, nullptr, nullptr, dp, dq);
        if (positions) DIO_CK(cudaMemcpyAsync(positions, dp, (size_t)n * 24, cudaMemcpyDeviceToHost, stream_));
        if (orientations) DIO_CK(cudaMemcpyAsync(orientations, dq, (size_t)n * 32, cudaMemcpyDeviceToHost, stream_));
        DIO_CK(cudaStreamSynchronize(stream_));
        return DIO_OK;
    }

    int contacts(DioContact* out, uint32_t cap, uint32_t* m) override {
        // rows of the last step live in the "previous" buffer after the swap
        int pb = 1 - cur_;
        DIO_TRY(pull_counters());
        uint32_t M = steps_ ? hctr_->rows : 0;
        if (m) *m = M;
        if (M > cap) return cap_err("output buffer smaller than the row count");
        if (!M) return DIO_OK;
        DioContact* dout = reinterpret_cast<DioContact*>(dstage_);
        uint32_t* dm = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(dstage_) + align256((size_t)M * sizeof(DioContact)));
        k_set_u32<<<1, 1, 0, stream_>>>(dm, M);
        k_pack_contacts<P, R><<<grid_for(M, 256), 256, 0, stream_>>>(rs_[pb], rd_[pb], ab_[pb], dout, dm);
        DIO_CK(cudaMemcpyAsync(out, dout, (size_t)M * sizeof(DioContact), cudaMemcpyDeviceToHost, stream_));
        DIO_CK(cudaStreamSynchronize(stream_));
        return DIO_OK;
    }

    int colors(uint32_t* out, uint32_t cap, uint32_t* n) override {
        uint32_t N = w_.n;
        if (n) *n = N;
        if (N > cap) return cap_err("output buffer smaller than the body count");
        if (N) {
            DIO_CK(cudaMemcpyAsync(out, w_.color, (size_t)N * 4, cudaMemcpyDeviceToHost, stream_));
            DIO_CK(cudaStreamSynchronize(stream_));
        }
        return DIO_OK;
    }

    int stats(DioStepStats* out) override {
        if (!out) return inval("null stats");
        DIO_TRY(pull_counters());
        out->pairs = hctr_->pairs;
        out->contacts = hctr_->rows;
        out->colors = hctr_->colors;
        out->error_flags = hctr_->error_flags;
        out->steps = steps_;
        collect_spans();
        out->kernel_launches = launches_;
        out->primal_launches = primal_n_;
        out->dual_launches = dual_n_;
        out->primal_ms = primal_ms_;
        out->dual_ms = dual_ms_;
        out->broad_ms = phase_ms_[0];
        out->narrow_ms = phase_ms_[1];
        out->rows_ms = phase_ms_[2];
        out->solve_ms = phase_ms_[3];
        out->chunk_launches = solve_chunk_n_;
        out->chunk_ms = solve_chunk_ms_;
        return DIO_OK;
    }

   private:
    // ------------------------------------------------------------ helpers
    template <class T>
    int alloc(T** p, size_t count) {
        DIO_CK(cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(1, count) * sizeof(T)));
        allocs_.push_back(*p);
        return DIO_OK;
    }
    void release() {
        for (void* p : allocs_) cudaFree(p);
        allocs_.clear();
        ss_.release();
        if (dstage_) cudaFree(dstage_);
        if (hstage_) cudaFreeHost(hstage_);
        if (hctr_) cudaFreeHost(hctr_);
        dstage_ = nullptr;
        hstage_ = nullptr;
        hctr_ = nullptr;
    }
    static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
    int inval(const char* m) {
        err = m;
        return DIO_ERR_INVALID;
    }
    int cap_err(const char* m) {
        err = m;
        return DIO_ERR_CAPACITY;
    }
    int state_err(const char* m) {
        err = m;
        return DIO_ERR_STATE;
    }
    void set_rows(int b) {
        w_.rs = rs_[b];
        w_.rd = rd_[b];
        w_.ab = ab_[b];
    }
    int pull_counters() {
        DIO_CK(cudaMemcpyAsync(hctr_, ctr_, sizeof(Counters), cudaMemcpyDeviceToHost, stream_));
        DIO_CK(cudaStreamSynchronize(stream_));
        return DIO_OK;
    }
    int check_flags() {
        DIO_TRY(pull_counters());
        uint32_t f = hctr_->error_flags;
        if (!f) return DIO_OK;
        DIO_CK(cudaMemsetAsync(&ctr_->error_flags, 0, 4, stream_));
        if (f & kErrBadIndex) return inval("body / row index out of range");
        if (f & kErrPairOverflow) return cap_err("device capacity exceeded: more candidate pairs than max_pairs");
        if (f & kErrRowOverflow) return cap_err("device capacity exceeded: more contact rows than max_contacts");
        if (f & kErrIndexOverflow)
            return cap_err("device capacity exceeded: a traversal stack, a tree's pair scratch or a per-body "
                           "segment sort ran out of room");
        if (f & (kErrEpaFaces | kErrEpaHorizon)) return cap_err("EPA polytope exceeded its shared-memory capacity");
        if (f & kErrColorOverflow) return cap_err("colouring needed more than 256 colours or did not converge");
        if (f & kErrTimeout) {
            err = "device wait timed out";
            return DIO_ERR_TIMEOUT;
        }
        if (f & kErrNonFinite) {
            err = "non-finite solver state";
            return DIO_ERR_NONFINITE;
        }
        return DIO_OK;
    }
    // a hull body's vertex range [first, first + count) must lie in the
    // hull-vertex pool: the support queries and the EPA's bulk copies read it
    static bool hull_ranges_ok(const DioGpuBody* bodies, uint32_t n, uint32_t n_hull) {
        for (uint32_t i = 0; i < n; ++i) {
            const DioShape& sh = bodies[i].shape;
            if (sh.tag == DIO_SHAPE_HULL && (uint64_t)sh.pad[0] + sh.pad[1] > n_hull) return false;
        }
        return true;
    }
    int upload_bodies(const DioGpuBody* bodies, uint32_t n, uint32_t n_hull) {
        if (!n) return DIO_OK;
        if (!bodies) return inval("null bodies");
        if (!hull_ranges_ok(bodies, n, n_hull)) return inval("hull vertex range beyond the hull-vertex pool");
        DioGpuBody* db = reinterpret_cast<DioGpuBody*>(dstage_);
        DIO_CK(cudaMemcpyAsync(db, bodies, (size_t)n * sizeof(DioGpuBody), cudaMemcpyHostToDevice, stream_));
        k_unpack_bodies<P, R><<<grid_for(n, 256), 256, 0, stream_>>>(w_, db, n);
        w_.n = n;
        return DIO_OK;
    }
    int upload_state(const DioBodyState* state, uint32_t n) {
        if (!n) return DIO_OK;
        if (!state) return inval("null state");
        DioBodyState* ds = reinterpret_cast<DioBodyState*>(reinterpret_cast<char*>(dstage_) +
                                                           align256((size_t)n * sizeof(DioGpuBody)));
        DIO_CK(cudaMemcpyAsync(ds, state, (size_t)n * sizeof(DioBodyState), cudaMemcpyHostToDevice, stream_));
        k_unpack_state<P, R><<<grid_for(n, 256), 256, 0, stream_>>>(w_, ds, n);
        return build_dyn_list(n);
    }
    // compacted list of dynamic bodies (inverse mass != 0), index order
    int build_dyn_list(uint32_t n) {
        dyn_list_n_ = n;
        k_dyn_flags<P, R><<<grid_for(n, 256), 256, 0, stream_>>>(w_, n, counts2_, dyn_keep_);
        DIO_CK(cudaMemsetAsync(counts2_ + n, 0, 4, stream_));
        DIO_CK(ss_.scan(counts2_, offsets2_, n + 1, false, stream_));
        k_dyn_fill<<<grid_for(n, 256), 256, 0, stream_>>>(counts2_, offsets2_, n, dyn_list_);
        uint32_t nd = 0;
        DIO_CK(cudaMemcpyAsync(&nd, offsets2_ + n, 4, cudaMemcpyDeviceToHost, stream_));
        DIO_CK(cudaStreamSynchronize(stream_));
        if (w_.n_dyn != nd) drop_graphs();  // launch shapes depend on it
        w_.n_dyn = nd;
        w_.dyn_list = dyn_list_;
        return order_dyn_list();
    }
    // stable sort of the dynamic-body list by work signature (k_dyn_keys);
    // index order is kept inside a signature
    int order_dyn_list() {
        const uint32_t nd = w_.n_dyn;
        const uint32_t nc = (uint32_t)solve_chunks_host_.size();
        if (nc) DIO_CK(cudaMemsetAsync(chunk_dyn_, 0, nc * sizeof(uint2), stream_));
        if (!nd) return DIO_OK;
        // in chunk order when every scene has a solve chunk (the scene-chunk
        // solve walks its chunk's run), else by signature alone
        const uint32_t* sch = chunked_scenes_ ? scene_chunk_ : nullptr;
        k_dyn_keys<P, R><<<grid_for(nd, 256), 256, 0, stream_>>>(w_, dyn_list_, nd, sch, counts2_);
        const uint32_t end_bit = 7u + (sch ? bits_for(nc) : 0u);
        DIO_CK(ss_.sort_pairs(counts2_, offsets2_, dyn_list_, dyn_tmp_, nd, 0u, end_bit, false, stream_));
        DIO_CK(cudaMemcpyAsync(dyn_list_, dyn_tmp_, (size_t)nd * 4, cudaMemcpyDeviceToDevice, stream_));
        if (sch) k_chunk_dyn_runs<P, R><<<grid_for(nd, 256), 256, 0, stream_>>>(w_, dyn_list_, nd, sch, chunk_dyn_);
        return DIO_OK;
    }
    int single_scene(uint32_t n, const DioContainer* c) {
        SceneDesc x;
        std::memset(&x, 0, sizeof x);
        x.body_lo = 0;
        x.body_hi = n;
        x.rotation[3] = 1.f;
        if (c) {
            x.has_container = 1;
            std::memcpy(x.center, c->center, 12);
            x.half_extent = c->half_extent;
            std::memcpy(x.rotation, c->rotation, 16);
        }
        DIO_CK(cudaMemcpyAsync(scenes_, &x, sizeof x, cudaMemcpyHostToDevice, stream_));
        DIO_CK(cudaMemsetAsync(w_.scene, 0, (size_t)std::max(n, 1u) * 4, stream_));
        w_.n_scenes = 1;
        w_.origin = nullptr;
        k_scene_walls<P, R><<<1, 32, 0, stream_>>>(w_, scenes_, 1u, walls_);
        w_.n = n;
        // the API path is single-scene FP32; keep host scene table in sync
        scenes_host_.assign(1, x);
        DIO_TRY(note_scene_sizes());
        DIO_CK(cudaStreamSynchronize(stream_));
        return DIO_OK;
    }
    // every joint's two bodies in one scene of the uploaded world
    bool joints_within_scenes(const DioConstraint* cons, uint32_t nj) const {
        auto scene_of = [&](uint32_t b) -> int64_t {
            auto it = std::upper_bound(scenes_host_.begin(), scenes_host_.end(), b,
                                       [](uint32_t v, const SceneDesc& sd) { return v < sd.body_hi; });
            if (it == scenes_host_.end() || b < it->body_lo) return -1;
            return it - scenes_host_.begin();
        };
        for (uint32_t k = 0; k < nj; ++k) {
            const int64_t sa = scene_of(cons[k].a);
            if (sa < 0 || sa != scene_of(cons[k].b)) return false;
        }
        return true;
    }
    // the whole solve of a world step as one launch (k_solve_chunks)
    bool use_chunk_solve() const { return chunk_world_ && cfg_.batched_solver == DIO_SOLVE_AUTO; }
    bool chunk_solve_possible() const override { return chunk_world_; }
    int solve_chunks(const SolveParams<R>& o) {
        const uint32_t cap = solve_chunk_max_;  // shared memory sized to the largest chunk
        cudaEvent_t e0 = span_begin();
        const int grid = (int)solve_chunks_host_.size();
        const bool wide = cfg_.block_size == (uint32_t)kChunkThreadsWide;
        if (cfg_.solver_mode == DIO_SOLVER_COLORED) {
            // the coloured Gauss-Seidel schedule, colouring included
            const size_t cs = chunk_colored_smem_bytes<P>(cap);
            if (wide)
                DIO_CK(launch_k(pdl(), k_solve_chunks_colored<P, R, kChunkThreadsWide>, grid, kChunkThreadsWide, cs,
                                stream_, w_, (const uint2*)solve_chunks_, (const uint2*)chunk_dyn_, scenes_, cap, o));
            else
                DIO_CK(launch_k(pdl(), k_solve_chunks_colored<P, R, kChunkThreads>, grid, kChunkThreads, cs,
                                stream_, w_, (const uint2*)solve_chunks_, (const uint2*)chunk_dyn_, scenes_, cap, o));
            span_end(e0, 6);
            ++launches_;
            return DIO_OK;
        }
        const size_t smem = chunk_smem_bytes<P>(cap);
        if (wide)
            DIO_CK(launch_k(pdl(), k_solve_chunks<P, R, kChunkThreadsWide>, grid, kChunkThreadsWide, smem, stream_, w_,
                            (const uint2*)solve_chunks_, (const uint2*)chunk_dyn_, scenes_, cap, o));
        else
            DIO_CK(launch_k(pdl(), k_solve_chunks<P, R, kChunkThreads>, grid, kChunkThreads, smem, stream_, w_,
                            (const uint2*)solve_chunks_, (const uint2*)chunk_dyn_, scenes_, cap, o));
        span_end(e0, 6);
        ++launches_;
        return DIO_OK;
    }
    int upload_joints(const DioConstraint* cons, uint32_t nj, uint32_t n) {
        w_.n_joints = nj;
        if (!nj) {
            DIO_CK(cudaMemsetAsync(joint_off_, 0, ((size_t)n + 1) * 4, stream_));
            return order_dyn_list();
        }
        DIO_CK(cudaMemcpyAsync(joints_, cons, (size_t)nj * sizeof(DioConstraint), cudaMemcpyHostToDevice, stream_));
        uint32_t total = 2 * nj;
        k_joint_inc<<<grid_for(nj, 256), 256, 0, stream_>>>(joints_, nj, n, inc_body_, inc_row_, &ctr_->error_flags);
        DIO_CK(ss_.sort_pairs(inc_body_, inc_body_s_, inc_row_, inc_row_s_, total, 0u, bits_for(n + 1), false,
                              stream_));
        DIO_CK(cudaMemsetAsync(counts2_, 0, ((size_t)n + 1) * 4, stream_));
        k_count_lt<<<grid_for(total, 256), 256, 0, stream_>>>(inc_body_s_, total, n, counts2_);
        DIO_CK(ss_.scan(counts2_, joint_off_, n + 1, false, stream_));
        DIO_CK(cudaMemcpyAsync(joint_idx_, inc_row_s_, (size_t)total * 4, cudaMemcpyDeviceToDevice, stream_));
        k_build_jview<<<grid_for(n, 128), 128, 0, stream_>>>(joints_, joint_off_, joint_idx_, n, jview_);
        w_.jview = jview_;
        return order_dyn_list();
    }
    int sort_keys(const uint2* ab, uint32_t m, unsigned long long* keys_out, uint32_t* ids_out) {
        if (!m) return DIO_OK;
        return sort_keys_n(ab, m, keys_out, ids_out);
    }
    int sort_keys_n(const uint2* ab, uint32_t m, unsigned long long* keys_out, uint32_t* ids_out);

    static PrepParams<R> opts_prep(const DioAvbdOptions& o) {
        PrepParams<R> p;
        p.dt = R(o.dt);
        p.margin = R(o.margin);
        p.penalty_min = R(o.penalty_min);
        p.penalty_max = R(o.penalty_max);
        p.alpha_gamma = R(o.alpha) * R(o.gamma);
        p.gamma = R(o.gamma);
        p.friction = R(o.friction);
        return p;
    }
    static SolveParams<R> solve_params(float dt, const float* g, float alpha, float beta, float kmax, uint32_t it) {
        SolveParams<R> o;
        o.dt = R(dt);
        o.gx = R(g[0]);
        o.gy = R(g[1]);
        o.gz = R(g[2]);
        o.alpha = R(alpha);
        o.beta_lin = R(beta);
        o.penalty_max = R(kmax);
        o.iterations = it;
        return o;
    }

    int run_broad(uint32_t lo, uint32_t hi) {
        uint32_t n = hi - lo;
        int g = grid_for(n, 128);
        DIO_CK(launch_k(pdl(), k_aabb<P, R>, g, 128, 0, stream_, w_, lo, hi));
        ++launches_;
        if (cfg_.broad_phase == 0 && lo == 0) return run_lbvh(n);
        constexpr int kB = 128;
        int gd = grid_for(n, kB);
        k_dense<P, R, kB><<<gd, kB, 0, stream_>>>(w_, lo, hi, counts_, offsets_, false);
        DIO_CK(cudaMemsetAsync(counts_ + n, 0, 4, stream_));
        DIO_CK(ss_.scan(counts_, offsets_, n + 1, false, stream_));
        k_dense<P, R, kB><<<gd, kB, 0, stream_>>>(w_, lo, hi, counts_, offsets_, true);
        k_pairs_total<<<1, 1, 0, stream_>>>(ctr_, offsets_ + n, w_.max_pairs);
        launches_ += 3;
        return DIO_OK;
    }

    // LBVH over every scene of bodies [0, n); AABBs already computed
    int run_lbvh(uint32_t n) {
        uint32_t ns = std::max(1u, w_.n_scenes);
        int g = grid_for(n, 256);
        if (!rebuild_now_) return run_lbvh_refit(n, g);
        const uint32_t sbits = ns > 1 ? bits_for(ns - 1) : 0;
        const uint32_t abits = std::min(10u, (32u - sbits) / 3u);
        if (!chunks_host_.empty() && scene_max_ <= scene_tree_cap<R>()) {
            // every scene has a shared-memory tree: one CTA per chunk builds
            // its trees (bounds, keys, sort, nodes) in one launch
            DIO_CK(launch_k(pdl(), k_chunk_build<R>, (int)chunks_host_.size(), kSceneTreeThreads,
                            chunk_build_bytes<R>(), stream_, (const A4<R>*)w_.aabb_min, (const A4<R>*)w_.aabb_max,
                            (const SceneDesc*)scenes_, (const uint32_t*)w_.scene, (const uint2*)chunks_, n,
                            std::max(2u, chunk_max_), sbits, abits, lb_keys_s_, lb_leaf_, lb_children_, lb_parent_,
                            &ctr_->error_flags));
            ++launches_;
            return run_lbvh_refit(n, g);
        }
        DIO_CK(launch_k(pdl(), k_bounds_init, grid_for(ns, 128), 128, 0, stream_, lb_bounds_, ns));
        DIO_CK(launch_k(pdl(), k_scene_bounds<R>, g, 256, 0, stream_, (const A4<R>*)w_.aabb_min,
                        (const A4<R>*)w_.aabb_max, (const uint32_t*)w_.scene, n, lb_bounds_));
        DIO_CK(launch_k(pdl(), k_morton<R>, g, 256, 0, stream_, (const A4<R>*)w_.aabb_min, (const A4<R>*)w_.aabb_max,
                        (const uint32_t*)w_.scene, n, (const uint32_t*)lb_bounds_, sbits, abits, lb_keys_, lb_vals_));
        DIO_CK(ss_.sort_pairs(lb_keys_, lb_keys_s_, lb_vals_, lb_leaf_, n, 0u, sbits + 3u * abits, pdl(), stream_));
        DIO_CK(launch_k(pdl(), k_karras, g, 256, 0, stream_, (const uint32_t*)lb_keys_s_, (const SceneDesc*)scenes_,
                        (const uint32_t*)w_.scene, n, lb_children_, lb_parent_));
        launches_ += 4;
        return run_lbvh_refit(n, g);
    }

    // Refit the current tree to this step's AABBs and traverse it.  Any
    // valid tree over the scene's leaves yields the exact overlap set, so
    // the topology is rebuilt only every bvh_rebuild_period steps.
    // Scenes of at most scene_tree_cap bodies are refitted and traversed by
    // k_scene_tree (one CTA per chunk of scenes, trees in shared memory),
    // larger ones by the global k_refit / k_traverse.
    int run_lbvh_refit(uint32_t n, int g) {
        const uint32_t cap = scene_tree_cap<R>();
        const uint32_t nchunks = (uint32_t)chunks_host_.size();
        const uint32_t tcap = std::max(2u, chunk_max_);
        const size_t tbytes = scene_tree_bytes<R>(tcap);
        const bool global_path = scene_max_ > cap;
        const uint32_t tcap_skip = cap;
        TreeArgs ta;
        ta.leaf_body = lb_leaf_;
        ta.scenes = scenes_;
        ta.scene_of_pos = w_.scene;
        ta.chunks = chunks_;
        ta.n = n;
        ta.cap_bodies = tcap;
        ta.children = lb_children_;
        ta.parent = lb_parent_;
        ta.counts = counts_;
        ta.offsets = offsets_;
        ta.pb = lb_pb_;
        ta.cap = w_.max_pairs;
        ta.scratch = tree_scratch_;
        ta.scratch_k = scratch_k_;
        ta.chunk_n = chunk_n_;
        ta.chunk_ovf = chunk_ovf_;
        ta.chunk_tot = chunk_tot_;
        ta.err = &ctr_->error_flags;
        // every scene in a shared-memory tree: the write pass also forms the
        // offsets, sorts the partner lists and emits the pairs
        ta.fused = (nchunks && !global_path) ? 1u : 0u;
        ta.nchunks = nchunks;
        ta.pairs = w_.pairs;
        ta.ctr = ctr_;
        auto scene_tree = [&](bool write) -> cudaError_t {
            if (!nchunks) return cudaSuccess;
            ++launches_;
            if (write)
                return launch_k(pdl(), k_scene_tree<R, true>, (int)nchunks, kSceneTreeThreads, tbytes, stream_,
                                (const A4<R>*)w_.aabb_min, (const A4<R>*)w_.aabb_max, lb_leaf_min_, lb_leaf_max_,
                                lb_node_min_, lb_node_max_, ta);
            return launch_k(pdl(), k_scene_tree<R, false>, (int)nchunks, kSceneTreeThreads, tbytes, stream_,
                            (const A4<R>*)w_.aabb_min, (const A4<R>*)w_.aabb_max, lb_leaf_min_, lb_leaf_max_,
                            lb_node_min_, lb_node_max_, ta);
        };
        int gt = grid_for(n, 128);
        DIO_CK(scene_tree(false));
        if (ta.fused) {
            DIO_CK(scene_tree(true));
            return DIO_OK;
        }
        if (global_path) {
            DIO_CK(cudaMemsetAsync(lb_visits_, 0, (size_t)n * 4, stream_));
            if (!world_step_) DIO_CK(cudaMemsetAsync(&ctr_->traverse_pairs, 0, 4, stream_));  // else k_roll_counters
            k_refit<R><<<g, 256, 0, stream_>>>(w_.aabb_min, w_.aabb_max, lb_leaf_, scenes_, w_.scene, n,
                                               lb_children_, lb_parent_, lb_leaf_min_, lb_leaf_max_, lb_node_min_,
                                               lb_node_max_, lb_visits_, tcap_skip, counts_);
            // a walk per leaf fills the SMs from about 512 leaves per SM; fewer
            // leaves split each walk over four threads
            const uint32_t split = (uint64_t)n < (uint64_t)sms_ * 512u ? kWalkSplit : 1u;
            k_traverse_count<R><<<grid_for((uint64_t)n * split, 128), 128, 0, stream_>>>(
                lb_leaf_, scenes_, w_.scene, n, lb_children_, lb_leaf_min_, lb_leaf_max_, lb_node_min_, lb_node_max_,
                counts_, lb_gscratch_, w_.max_pairs, &ctr_->traverse_pairs, &ctr_->error_flags, tcap_skip, split);
            launches_ += 2;
        }
        if (!world_step_) DIO_CK(cudaMemsetAsync(counts_ + n, 0, 4, stream_));  // else k_roll_counters
        DIO_CK(ss_.scan(counts_, offsets_, n + 1, pdl(), stream_));
        DIO_CK(scene_tree(true));
        if (global_path) {
            // the scratch pairs to their offsets (counts_ taken down to zero),
            // or, when the scratch overflowed, the full write traversal
            DIO_CK(launch_k(pdl(), k_place_scratch, sms_ * 4, 256, 0, stream_, (const uint2*)lb_gscratch_,
                            (const uint32_t*)&ctr_->traverse_pairs, w_.max_pairs, (const uint32_t*)offsets_, counts_,
                            lb_pb_, w_.max_pairs));
            DIO_CK(launch_k(pdl(), k_traverse<R>, gt, 128, 0, stream_, (const uint32_t*)lb_leaf_,
                            (const SceneDesc*)scenes_, (const uint32_t*)w_.scene, n, (const uint2*)lb_children_,
                            (const A4<R>*)lb_leaf_min_, (const A4<R>*)lb_leaf_max_, (const A4<R>*)lb_node_min_,
                            (const A4<R>*)lb_node_max_, (const uint32_t*)offsets_, lb_pb_, w_.max_pairs,
                            (const uint32_t*)&ctr_->traverse_pairs, w_.max_pairs, &ctr_->error_flags, tcap_skip));
            launches_ += 2;
        }
        DIO_CK(launch_k(pdl(), k_pairs_total, 1, 1, 0, stream_, ctr_,
                        (const uint32_t*)(offsets_ + n), w_.max_pairs));
        if (!world_step_) DIO_CK(cudaMemsetAsync(lb_long_count_, 0, 4, stream_));  // else k_roll_counters
        DIO_CK(launch_k(pdl(), k_sort_segments, g, 256, 0, stream_, (const uint32_t*)offsets_, n, w_.max_pairs, lb_pb_,
                        lb_long_, lb_long_count_));
        DIO_CK(launch_k(pdl(), k_sort_long, sms_, 512, 0, stream_, (const uint32_t*)offsets_, lb_pb_,
                        (const uint32_t*)lb_long_, (const uint32_t*)lb_long_count_, &ctr_->error_flags));
        DIO_CK(launch_k(pdl(), k_pairs_from_segments, g, 256, 0, stream_, (const uint32_t*)offsets_, n,
                        (const uint32_t*)lb_pb_, w_.pairs, w_.max_pairs));
        launches_ += 4;
        return DIO_OK;
    }

    // narrow phase over np pairs (np_dev: device count, else np)
    int run_narrow(uint32_t np, const uint32_t* np_dev) {
        uint32_t per = cfg_.contacts_per_pair;
        w_.per_pair = per;
        int g = np_dev ? sms_ * 8 : grid_for(np, 128);
        DIO_CK(launch_k(pdl(), k_narrow_main<P, R>, g, 128, 0, stream_, w_, np_dev, np));
        DIO_CK(launch_k(pdl(), k_gjk<P, R>, sms_ * 4, 128, 0, stream_, w_));
        DIO_CK(launch_k(pdl(), k_epa<P, R>, sms_ * 4, 32 * epa_warps<R>(), 0, stream_, w_));
        launches_ += 3;
        return DIO_OK;
    }

    // Rows from `groups` groups of `per` slots (+ container rows for bodies).
    // src: the narrow slots the pair rows come from (w_.slots, or the
    // previous step's with contact_lag)
    int build_rows(const PrepParams<R>& o, uint32_t groups, uint32_t per, const uint32_t* groups_dev, uint32_t n,
                   const Slot<R>* src = nullptr) {
        uint32_t G = groups;
        if (!src) src = w_.slots;
        if (G) {
            // grid-stride over the live groups (a device count: fixed grids)
            DIO_CK(launch_k(pdl(), k_slot_count<R>, std::min(grid_for(G, 256), sms_ * 8), 256, 0, stream_, src, per,
                            groups_dev, G, counts_));
            // offsets of the live groups, the total at offsets_[G]
            DIO_CK(ss_.scan(counts_, offsets_, G, pdl(), stream_, groups_dev, offsets_ + G));
            DIO_CK(launch_k(pdl(), k_slot_rows<P, R>, std::min(grid_for(G, 128), sms_ * 16), 128, 0, stream_, w_, src,
                            per, groups_dev, G, (const uint32_t*)offsets_, o));
        } else {
            DIO_CK(cudaMemsetAsync(offsets_, 0, 4, stream_));
        }
        const uint32_t* pair_rows = offsets_ + G;
        if (n) {
            DIO_CK(launch_k(pdl() && G, k_cont_count<P, R>, grid_for(n, 128), 128, 0, stream_, w_, 0u, n, o, counts2_));
            DIO_CK(ss_.scan(counts2_, offsets2_, n + 1, pdl(), stream_));
            // clears counts2_ for the CSR count of finish_rows_world
            DIO_CK(launch_k(pdl(), k_cont_rows<P, R>, grid_for(n, 128), 128, 0, stream_, w_, 0u, n, o,
                            (const uint32_t*)offsets2_, pair_rows, counts2_));
        } else {
            DIO_CK(cudaMemsetAsync(offsets2_, 0, 4, stream_));
        }
        DIO_CK(launch_k(pdl() && n, k_sum_rows, 1, 1, 0, stream_, ctr_, pair_rows, (const uint32_t*)(offsets2_ + n),
                        w_.max_rows));
        launches_ += 5;
        return DIO_OK;
    }

    // warm start + decay + CSR for M rows (host-known count)
    int finish_rows(const PrepParams<R>& o, uint32_t M, uint32_t n) {
        int pb = 1 - cur_;
        if (M) {
            k_row_keys<<<grid_for(M, 256), 256, 0, stream_>>>(w_.ab, &ctr_->rows, M, keys_raw_, ids_raw_, inc_body_,
                                                              inc_row_, n);
            DIO_CK(ss_.sort_pairs(keys_raw_, keys_s_[cur_], ids_raw_, ids_s_[cur_], M, 0u, 64u, false, stream_));
            k_warm<P, R><<<grid_for(M, 256), 256, 0, stream_>>>(w_, &ctr_->rows, keys_s_[cur_], ids_s_[cur_],
                                                                keys_s_[pb], ids_s_[pb], n_prev_rows_, rd_[pb], o);
            DIO_CK(ss_.sort_pairs(inc_body_, inc_body_s_, inc_row_, inc_row_s_, 2 * M, 0u, bits_for(n + 1), false,
                                  stream_));
        }
        DIO_CK(cudaMemsetAsync(counts2_, 0, ((size_t)n + 1) * 4, stream_));
        if (M) k_inc_count<<<grid_for(2 * M, 256), 256, 0, stream_>>>(inc_body_s_, &ctr_->rows, n, counts2_);
        DIO_CK(ss_.scan(counts2_, w_.row_off, n + 1, false, stream_));
        if (M) k_csr_fill<P, R><<<grid_for(2 * M, 256), 256, 0, stream_>>>(w_, inc_body_s_, inc_row_s_, &ctr_->rows);
        launches_ += M ? 4 : 0;
        return DIO_OK;
    }

    // m_dev: device row count (fixed grid, device-bounded loops) or null (host m)
    int solve(const SolveParams<R>& o, uint32_t n, uint32_t m, const uint32_t* m_dev = nullptr) {
        if (n == 0) return DIO_OK;
        int gb = grid_for(n, 256);
        // device-counted rows: one resident wave, rows strided over it
        int gm = m_dev ? std::min(grid_for(cap_.max_contacts, 256), sms_ * dual_ctas_per_sm_)
                       : grid_for(std::max(m, 1u), 256);
        if (m_dev) m = cap_.max_contacts;
        DIO_CK(launch_k(pdl(), k_init<P, R>, gb, 256, 0, stream_, w_, 0u, n, o));
        launches_ += 2;
        // programmatic dependent launch between the solve's kernels, unless
        // event timers sit between them
        const bool pdl = !cfg_.profile;
        for (uint32_t k = 0; k < o.iterations; ++k) {
            int par = (int)(k % 2);
            cudaEvent_t e0 = span_begin();
            launch_primal<P, R>((int)cfg_.primal_variant, pdl, w_, par, 1 - par, o, stream_);
            span_end(e0, 0);
            ++launches_;
            if (m) {
                cudaEvent_t e1 = span_begin();
                DIO_CK(launch_k(pdl, k_dual<P, R>, gm, 256, 0, stream_, w_, 0u, m, m_dev, 1 - par, o));
                span_end(e1, 1);
                ++launches_;
            }
        }
        uint32_t fp = (o.iterations - 1u) % 2u;
        int rb = fp == 0 ? 1 : 0;
        uint32_t fp_read = (o.iterations == 0 ? 0u : o.iterations - 1u) % 2u;
        int final_buf = 1 - (int)fp_read;
        DIO_CK(launch_k(pdl, k_recover<P, R>, gb, 256, 0, stream_, w_, 0u, n, rb, final_buf, o));
        DIO_CK(cudaGetLastError());
        return DIO_OK;
    }

    // kernel timing with CUDA events on the launching stream (profile on)
    cudaEvent_t take_event() {
        if (ev_free_.empty()) {
            cudaEvent_t e = nullptr;
            cudaEventCreate(&e);
            return e;
        }
        cudaEvent_t e = ev_free_.back();
        ev_free_.pop_back();
        return e;
    }
    // inside a capture an event record must be external to become a graph node
    void record(cudaEvent_t e) {
        if (capturing_)
            cudaEventRecordWithFlags(e, stream_, cudaEventRecordExternal);
        else
            cudaEventRecord(e, stream_);
    }
    cudaEvent_t span_begin() {
        if (!cfg_.profile) return nullptr;
        cudaEvent_t e = take_event();
        record(e);
        return e;
    }
    void span_end(cudaEvent_t e0, int kind) {
        if (!e0) return;
        cudaEvent_t e1 = take_event();
        record(e1);
        if (capturing_)
            cap_spans_.push_back({e0, e1, kind});  // placeholders, rebound per replay
        else
            spans_.push_back({e0, e1, kind});
    }
    void collect_spans() {
        if (spans_.empty()) return;
        cudaStreamSynchronize(stream_);
        for (auto& s : spans_) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, s.a, s.b);
            if (s.kind == 0) {
                primal_ms_ += ms;
                ++primal_n_;
            } else if (s.kind == 1) {
                dual_ms_ += ms;
                ++dual_n_;
            } else if (s.kind == 6) {
                solve_chunk_ms_ += ms;
                ++solve_chunk_n_;
            } else {
                phase_ms_[s.kind - 2] += ms;
            }
            ev_free_.push_back(s.a);
            ev_free_.push_back(s.b);
        }
        spans_.clear();
    }

   public:
    int snapshot() override {
        if (!world_ready_) return state_err("no world uploaded");
        const size_t nb = (size_t)std::max(1u, cap_.max_bodies), nr = (size_t)std::max(1u, cap_.max_contacts);
        if (!snap_) {
            snap_bytes_ = nb * sizeof(A4<P>) * 5 + nr * (sizeof(RowStatic<R>) + sizeof(RowDual<P, R>) + sizeof(uint2)) * 2 +
                          sizeof(Counters) + 4096;
            DIO_CK(cudaMalloc(&snap_, snap_bytes_));
        }
        DIO_TRY(snap_copy(true));
        snap_cur_ = cur_;
        snap_steps_ = steps_;
        snap_valid_ = lbvh_valid_;
        return DIO_OK;
    }
    int restore() override {
        if (!snap_) return state_err("no snapshot");
        DIO_TRY(snap_copy(false));
        cur_ = snap_cur_;
        set_rows(cur_);
        steps_ = snap_steps_;
        lbvh_valid_ = snap_valid_;
        return DIO_OK;
    }
    int export_transforms(uint32_t format, const float* scales, void* out, size_t stride) override {
        if (!world_ready_) return state_err("no world uploaded");
        if (format != DIO_XFORM_POSE && format != DIO_XFORM_MAT4) return inval("unknown transform format");
        const size_t rec = format == DIO_XFORM_POSE ? 32 : 64;
        if (!out || stride < rec || stride % 16 || reinterpret_cast<uintptr_t>(out) % 16)
            return inval("output must be 16-byte aligned with a stride of at least one record");
        if (!w_.n) return DIO_OK;
        k_export_xform<P, R><<<grid_for(w_.n, 256), 256, 0, stream_>>>(w_.pos[0], w_.rot[0], w_.n, format, scales,
                                                                     static_cast<char*>(out), stride);
        DIO_CK(cudaGetLastError());
        return DIO_OK;
    }

    // ------------------------------------------------------- checkpoint
    // Image: header, then 16-byte aligned sections in kCkptSections order.
    struct CkptHeader {
        char magic[8];
        uint32_t version, precision, p_bytes, r_bytes;
        uint32_t n, n_joints, n_scenes, n_hull;
        uint32_t rows, pair_rows, has_container, per_pair, lag_pairs, pad;
        uint64_t steps, total_bytes;
    };
    enum { kCkBodies, kCkState, kCkJoints, kCkScenes, kCkHull, kCkPos, kCkRot, kCkVel, kCkAng, kCkPrevVel,
           kCkRowStatic, kCkRowDual, kCkRowAb, kCkSlots, kCkptSections };
    static size_t ckpt_layout(const CkptHeader& h, size_t off[kCkptSections]) {
        const size_t a4 = (size_t)h.n * sizeof(A4<P>);
        const size_t sz[kCkptSections] = {(size_t)h.n * sizeof(DioGpuBody),     (size_t)h.n * sizeof(DioBodyState),
                                          (size_t)h.n_joints * sizeof(DioConstraint),
                                          (size_t)h.n_scenes * sizeof(SceneDesc), (size_t)h.n_hull * 16,
                                          a4, a4, a4, a4, a4,
                                          (size_t)h.rows * sizeof(RowStatic<R>),
                                          (size_t)h.rows * sizeof(RowDual<P, R>), (size_t)h.rows * sizeof(uint2),
                                          (size_t)h.lag_pairs * h.per_pair * sizeof(Slot<R>)};
        size_t o = (sizeof(CkptHeader) + 15) & ~size_t(15);
        for (int k = 0; k < kCkptSections; ++k) {
            off[k] = o;
            o += (sz[k] + 15) & ~size_t(15);
        }
        return o;
    }
    static constexpr char kCkptMagic[8] = {'D', 'I', 'O', 'C', 'K', 'P', 'T', '1'};

   public:
    int checkpoint(void* out, size_t cap, size_t* size) override {
        if (!world_ready_) return state_err("no world uploaded");
        DIO_TRY(pull_counters());
        CkptHeader h;
        std::memset(&h, 0, sizeof h);
        std::memcpy(h.magic, kCkptMagic, 8);
        h.version = 1;
        h.precision = cfg_.precision;
        h.p_bytes = sizeof(P);
        h.r_bytes = sizeof(R);
        h.n = w_.n;
        h.n_joints = w_.n_joints;
        h.n_scenes = (uint32_t)scenes_host_.size();
        h.n_hull = n_hull_;
        h.rows = steps_ ? std::min(hctr_->rows, cap_.max_contacts) : 0u;
        h.pair_rows = std::min(steps_ ? hctr_->pair_rows : 0u, h.rows);
        h.has_container = !scenes_host_.empty() && scenes_host_[0].has_container;
        h.per_pair = cfg_.contacts_per_pair;
        // a contact-lag world's next rows come from the last step's slots
        const bool lagged = cfg_.contact_lag && slots_[1] && lag_primed_ && steps_;
        h.lag_pairs = lagged ? std::min(hctr_->pairs, cap_.max_pairs) : 0u;
        h.steps = steps_;
        size_t off[kCkptSections];
        h.total_bytes = ckpt_layout(h, off);
        *size = h.total_bytes;
        if (!out) return DIO_OK;
        if (cap < h.total_bytes) return cap_err("checkpoint buffer smaller than the image");
        char* b = static_cast<char*>(out);
        std::memset(b, 0, h.total_bytes);
        std::memcpy(b, &h, sizeof h);
        DIO_TRY(download(reinterpret_cast<DioGpuBody*>(b + off[kCkBodies]),
                         reinterpret_cast<DioBodyState*>(b + off[kCkState])));
        if (h.n_joints)
            DIO_CK(cudaMemcpyAsync(b + off[kCkJoints], joints_, (size_t)h.n_joints * sizeof(DioConstraint),
                                   cudaMemcpyDeviceToHost, stream_));
        if (h.n_scenes) std::memcpy(b + off[kCkScenes], scenes_host_.data(), h.n_scenes * sizeof(SceneDesc));
        std::vector<A4<R>> hv(h.n_hull);
        if (h.n_hull)
            DIO_CK(cudaMemcpyAsync(hv.data(), hull_, hv.size() * sizeof(A4<R>), cudaMemcpyDeviceToHost, stream_));
        const size_t a4 = (size_t)h.n * sizeof(A4<P>);
        A4<P>* src[5] = {w_.pos[0], w_.rot[0], w_.vel, w_.ang, w_.prev_vel};
        for (int k = 0; k < 5; ++k)
            if (a4) DIO_CK(cudaMemcpyAsync(b + off[kCkPos + k], src[k], a4, cudaMemcpyDeviceToHost, stream_));
        const int pb = 1 - cur_;  // the last step's rows
        if (h.rows) {
            DIO_CK(cudaMemcpyAsync(b + off[kCkRowStatic], rs_[pb], (size_t)h.rows * sizeof(RowStatic<R>),
                                   cudaMemcpyDeviceToHost, stream_));
            DIO_CK(cudaMemcpyAsync(b + off[kCkRowDual], rd_[pb], (size_t)h.rows * sizeof(RowDual<P, R>),
                                   cudaMemcpyDeviceToHost, stream_));
            DIO_CK(cudaMemcpyAsync(b + off[kCkRowAb], ab_[pb], (size_t)h.rows * sizeof(uint2), cudaMemcpyDeviceToHost,
                                   stream_));
        }
        if (h.lag_pairs)
            DIO_CK(cudaMemcpyAsync(b + off[kCkSlots], slots_[pb], (size_t)h.lag_pairs * h.per_pair * sizeof(Slot<R>),
                                   cudaMemcpyDeviceToHost, stream_));
        DIO_CK(cudaStreamSynchronize(stream_));
        float* hf = reinterpret_cast<float*>(b + off[kCkHull]);
        for (uint32_t i = 0; i < h.n_hull; ++i) {
            hf[4 * i] = float(hv[i].x);
            hf[4 * i + 1] = float(hv[i].y);
            hf[4 * i + 2] = float(hv[i].z);
            hf[4 * i + 3] = 0.f;
        }
        return DIO_OK;
    }
    int resume(const void* in, size_t size) override {
        CkptHeader h;
        if (size < sizeof h) return inval("checkpoint image too small");
        std::memcpy(&h, in, sizeof h);
        if (std::memcmp(h.magic, kCkptMagic, 8) || h.version != 1) return inval("not a checkpoint image");
        if (h.precision != cfg_.precision || h.p_bytes != sizeof(P) || h.r_bytes != sizeof(R))
            return inval("checkpoint precision differs from the context's");
        size_t off[kCkptSections];
        if (ckpt_layout(h, off) != h.total_bytes || size < h.total_bytes) return inval("truncated checkpoint image");
        if (h.rows > cap_.max_contacts) return cap_err("checkpoint rows exceed the context's contact capacity");
        if (h.pair_rows > h.rows || !h.n_scenes) return inval("inconsistent checkpoint header");
        if (h.lag_pairs && (h.lag_pairs > cap_.max_pairs || h.per_pair != cfg_.contacts_per_pair || !cfg_.contact_lag))
            return inval("a contact-lag checkpoint needs a contact-lag context with the same slots per pair");
        const char* b = static_cast<const char*>(in);
        std::vector<SceneDesc> sd(h.n_scenes);
        std::memcpy(sd.data(), b + off[kCkScenes], h.n_scenes * sizeof(SceneDesc));
        std::vector<uint32_t> offs(h.n_scenes + 1);
        std::vector<DioContainer> conts(h.n_scenes);
        for (uint32_t s = 0; s < h.n_scenes; ++s) {
            if (sd[s].body_lo != (s ? sd[s - 1].body_hi : 0u) || sd[s].body_hi < sd[s].body_lo)
                return inval("checkpoint scene table is not a partition of the bodies");
            offs[s] = sd[s].body_lo;
            std::memcpy(conts[s].center, sd[s].center, 12);
            conts[s].half_extent = sd[s].half_extent;
            std::memcpy(conts[s].rotation, sd[s].rotation, 16);
        }
        offs[h.n_scenes] = sd[h.n_scenes - 1].body_hi;
        if (offs[h.n_scenes] != h.n) return inval("checkpoint scene table is not a partition of the bodies");
        DioWorldDesc d;
        std::memset(&d, 0, sizeof d);
        d.n_bodies = h.n;
        d.n_constraints = h.n_joints;
        d.n_scenes = h.n_scenes;
        d.n_hull_vertices = h.n_hull;
        d.bodies = reinterpret_cast<const DioGpuBody*>(b + off[kCkBodies]);
        d.state = reinterpret_cast<const DioBodyState*>(b + off[kCkState]);
        d.constraints = h.n_joints ? reinterpret_cast<const DioConstraint*>(b + off[kCkJoints]) : nullptr;
        d.scene_offsets = offs.data();
        d.containers = h.has_container ? conts.data() : nullptr;
        d.hull_vertices = h.n_hull ? reinterpret_cast<const float*>(b + off[kCkHull]) : nullptr;
        DIO_TRY(world_upload(&d));
        // the dynamic state in this world's precision, over the FP32 poses
        const size_t a4 = (size_t)h.n * sizeof(A4<P>);
        A4<P>* dst[5] = {w_.pos[0], w_.rot[0], w_.vel, w_.ang, w_.prev_vel};
        for (int k = 0; k < 5; ++k)
            if (a4) DIO_CK(cudaMemcpyAsync(dst[k], b + off[kCkPos + k], a4, cudaMemcpyHostToDevice, stream_));
        // the last step's rows: the next step's warm-start source
        const int pb = 1 - cur_;
        if (h.rows) {
            DIO_CK(cudaMemcpyAsync(rs_[pb], b + off[kCkRowStatic], (size_t)h.rows * sizeof(RowStatic<R>),
                                   cudaMemcpyHostToDevice, stream_));
            DIO_CK(cudaMemcpyAsync(rd_[pb], b + off[kCkRowDual], (size_t)h.rows * sizeof(RowDual<P, R>),
                                   cudaMemcpyHostToDevice, stream_));
            DIO_CK(cudaMemcpyAsync(ab_[pb], b + off[kCkRowAb], (size_t)h.rows * sizeof(uint2), cudaMemcpyHostToDevice,
                                   stream_));
        }
        k_set_u32<<<1, 1, 0, stream_>>>(&ctr_->rows, h.rows);
        k_set_u32<<<1, 1, 0, stream_>>>(&ctr_->pair_rows, h.pair_rows);
        if (h.lag_pairs) {
            if (!slots_[1]) DIO_TRY(alloc(&slots_[1], (size_t)cap_.max_pairs * per_cap_));
            DIO_CK(cudaMemcpyAsync(slots_[pb], b + off[kCkSlots], (size_t)h.lag_pairs * h.per_pair * sizeof(Slot<R>),
                                   cudaMemcpyHostToDevice, stream_));
            k_set_u32<<<1, 1, 0, stream_>>>(&ctr_->pairs, h.lag_pairs);
            lag_primed_ = true;
        }
        n_prev_rows_ = h.rows;
        steps_ = h.steps;
        DIO_CK(cudaStreamSynchronize(stream_));
        return check_flags();
    }

    int world_sizes(uint32_t* n, uint32_t* n_dyn, uint32_t* n_joints, uint32_t* n_scenes) override {
        *n = w_.n;
        *n_dyn = w_.n_dyn;
        *n_joints = w_.n_joints;
        *n_scenes = w_.n_scenes;
        return DIO_OK;
    }

   private:
    int snap_copy(bool save) {
        char* p = static_cast<char*>(snap_);
        const size_t nb = (size_t)std::max(1u, cap_.max_bodies), nr = (size_t)std::max(1u, cap_.max_contacts);
        auto cp = [&](void* dev, size_t bytes) -> cudaError_t {
            cudaError_t e = save ? cudaMemcpyAsync(p, dev, bytes, cudaMemcpyDeviceToDevice, stream_)
                                 : cudaMemcpyAsync(dev, p, bytes, cudaMemcpyDeviceToDevice, stream_);
            p += (bytes + 255) & ~size_t(255);
            return e;
        };
        const size_t a4 = nb * sizeof(A4<P>);
        DIO_CK(cp(w_.pos[0], a4));
        DIO_CK(cp(w_.rot[0], a4));
        DIO_CK(cp(w_.vel, a4));
        DIO_CK(cp(w_.ang, a4));
        DIO_CK(cp(w_.prev_vel, a4));
        for (int b = 0; b < 2; ++b) {
            DIO_CK(cp(rs_[b], nr * sizeof(RowStatic<R>)));
            DIO_CK(cp(rd_[b], nr * sizeof(RowDual<P, R>)));
            DIO_CK(cp(ab_[b], nr * sizeof(uint2)));
        }
        DIO_CK(cp(ctr_, sizeof(Counters)));
        DIO_CK(cudaStreamSynchronize(stream_));
        return DIO_OK;
    }
    void* snap_ = nullptr;
    size_t snap_bytes_ = 0;
    int snap_cur_ = 0;
    uint64_t snap_steps_ = 0;
    bool snap_valid_ = false;

   public:
    int reset_timers() override {
        collect_spans();
        primal_ms_ = dual_ms_ = solve_chunk_ms_ = 0.0;
        primal_n_ = dual_n_ = solve_chunk_n_ = 0;
        for (double& x : phase_ms_) x = 0.0;
        launches_ = 0;
        return DIO_OK;
    }

   private:

    // One step with every count kept on the device: no host synchronisation,
    // fixed launch shapes, so the whole step can be captured in a graph.
    // the world step's narrow slots: one buffer, or with contact_lag this
    // step's (written by the narrow phase) and the previous step's (read by
    // the pair rows), alternating with the row buffers
    void set_slots() { w_.slots = cfg_.contact_lag && slots_[1] ? slots_[cur_] : slots_[0]; }
    int build_world_rows(const PrepParams<R>& pp, uint32_t n) {
        if (cfg_.contact_lag && slots_[1])
            return build_rows(pp, cap_.max_pairs, cfg_.contacts_per_pair, &ctr_->prev_pairs, n, slots_[1 - cur_]);
        return build_rows(pp, cap_.max_pairs, cfg_.contacts_per_pair, &ctr_->pairs, n);
    }
    int step_body_dev(const DioAvbdOptions& opt) {
        struct WorldStep {  // the flag holds for this step's launches only
            bool& f;
            explicit WorldStep(bool& f) : f(f) { f = true; }
            ~WorldStep() { f = false; }
        } scope(world_step_);
        uint32_t n = w_.n;
        PrepParams<R> pp = opts_prep(opt);
        set_rows(cur_);
        set_slots();
        // zeroes the LBVH pair-count scan's closing entry and the long-segment
        // count of the pair sort (counts_ is written again later in the step)
        k_roll_counters<<<1, 1, 0, stream_>>>(ctr_, n && cfg_.broad_phase == 0 ? counts_ + n : nullptr,
                                              lb_long_count_);
        ++launches_;
        cudaEvent_t e = span_begin();
        if (n) DIO_TRY(run_broad(0, n));
        span_end(e, 2);
        e = span_begin();
        DIO_TRY(run_narrow(cap_.max_pairs, &ctr_->pairs));
        span_end(e, 3);
        e = span_begin();
        DIO_TRY(build_world_rows(pp, n));
        DIO_TRY(finish_rows_world(pp, n));
        span_end(e, 4);
        SolveParams<R> so = solve_params(opt.dt, opt.gravity, opt.alpha, opt.beta_lin, opt.penalty_max, opt.iterations);
        e = span_begin();
        if (use_chunk_solve())
            DIO_TRY(solve_chunks(so));
        else
            DIO_TRY(solve(so, n, 0, &ctr_->rows));
        span_end(e, 5);
        return DIO_OK;
    }

    // Coloured Gauss-Seidel step: same detection and rows, then a colouring
    // and per-colour primal sweeps in place (host-driven colour loop).
    int step_once_colored(const DioAvbdOptions& opt) {
        plan_rebuild();
        uint32_t n = w_.n;
        PrepParams<R> pp = opts_prep(opt);
        set_rows(cur_);
        set_slots();
        k_roll_counters<<<1, 1, 0, stream_>>>(ctr_, nullptr, nullptr);
        cudaEvent_t e = span_begin();
        if (n) DIO_TRY(run_broad(0, n));
        span_end(e, 2);
        e = span_begin();
        DIO_TRY(run_narrow(cap_.max_pairs, &ctr_->pairs));
        span_end(e, 3);
        e = span_begin();
        DIO_TRY(build_world_rows(pp, n));
        DIO_TRY(finish_rows_world(pp, n));
        span_end(e, 4);
        DIO_TRY(color_world(n));
        SolveParams<R> so = solve_params(opt.dt, opt.gravity, opt.alpha, opt.beta_lin, opt.penalty_max, opt.iterations);
        e = span_begin();
        if (n) {
            const int gb = grid_for(n, 256);
            const int gf = std::min(grid_for(cap_.max_contacts, 256), sms_ * 8);
            k_init<P, R><<<gb, 256, 0, stream_>>>(w_, 0, n, so);
            for (uint32_t it = 0; it < so.iterations; ++it) {
                for (uint32_t c = 0; c < ncolors_; ++c) {
                    uint32_t c0 = color_off_h_[c], c1 = color_off_h_[c + 1];
                    if (c1 <= c0) continue;
                    cudaEvent_t e0 = span_begin();
                    if (cfg_.primal_variant == 10)  // warp per body
                        k_primal_color_warp<P, R><<<grid_for(c1 - c0, kPrimalWarpWarps), kPrimalWarpWarps * 32,
                                                    primal_warp_smem<R>(), stream_>>>(w_, c0, c1, so);
                    else
                        k_primal_color<P, R><<<grid_for(c1 - c0, 128), 128, 0, stream_>>>(w_, c0, c1, so);
                    span_end(e0, 0);
                    ++launches_;
                }
                cudaEvent_t e1 = span_begin();
                k_dual<P, R><<<gf, 256, 0, stream_>>>(w_, 0, cap_.max_contacts, &ctr_->rows, 0, so);
                span_end(e1, 1);
                ++launches_;
            }
            k_recover<P, R><<<gb, 256, 0, stream_>>>(w_, 0, n, 0, 0, so);
            launches_ += 2;
        }
        span_end(e, 5);
        DIO_CK(cudaGetLastError());
        cur_ = 1 - cur_;
        set_rows(cur_);
        ++steps_;
        return DIO_OK;
    }

    // Jones-Plassmann rounds until every dynamic body has a colour, then
    // the per-colour body lists (colour counts read back to the host).
    int color_world(uint32_t n) {
        if (!n) {
            ncolors_ = 0;
            return DIO_OK;
        }
        const int g = grid_for(std::max(1u, w_.n_dyn), 256);
        k_color_init<P, R><<<grid_for(n, 256), 256, 0, stream_>>>(w_);
        k_set_u32<<<1, 1, 0, stream_>>>(&ctr_->color_remaining, w_.n_dyn);
        k_set_u32<<<1, 1, 0, stream_>>>(&ctr_->colors, 0);
        uint32_t remaining = w_.n_dyn, rounds = 0;
        while (remaining) {
            for (int r = 0; r < 4; ++r) {
                k_color_select<P, R><<<g, 256, 0, stream_>>>(w_, counts_);
                k_color_assign<P, R><<<g, 256, 0, stream_>>>(w_, counts_);
                launches_ += 2;
            }
            rounds += 4;
            DIO_CK(cudaMemcpyAsync(&remaining, &ctr_->color_remaining, 4, cudaMemcpyDeviceToHost, stream_));
            DIO_CK(cudaStreamSynchronize(stream_));
            if (rounds > 4096) return cap_err("colouring did not converge");
        }
        DIO_CK(cudaMemsetAsync(color_hist_, 0, (kMaxColors + 1) * 4, stream_));
        k_color_hist<P, R><<<g, 256, 0, stream_>>>(w_, color_hist_);
        DIO_CK(ss_.scan(color_hist_, w_.color_off, kMaxColors + 1, false, stream_));
        DIO_CK(cudaMemsetAsync(color_hist_, 0, (kMaxColors + 1) * 4, stream_));
        k_color_fill<P, R><<<g, 256, 0, stream_>>>(w_, color_hist_);
        launches_ += 3;
        DIO_CK(cudaMemcpyAsync(&ncolors_, &ctr_->colors, 4, cudaMemcpyDeviceToHost, stream_));
        DIO_CK(cudaMemcpyAsync(color_off_h_, w_.color_off, (kMaxColors + 1) * 4, cudaMemcpyDeviceToHost, stream_));
        DIO_CK(cudaStreamSynchronize(stream_));
        return DIO_OK;
    }

    // decide whether this step rebuilds the LBVH topology or refits it
    void plan_rebuild() {
        uint32_t period = cfg_.bvh_rebuild_period ? cfg_.bvh_rebuild_period : 4;
        rebuild_now_ = !lbvh_valid_ || period <= 1 || (steps_ % period) == 0;
        lbvh_valid_ = true;
    }

    int step_once_dev(const DioAvbdOptions& opt) {
        plan_rebuild();
        DIO_TRY(step_body_dev(opt));
        cur_ = 1 - cur_;
        set_rows(cur_);
        ++steps_;
        return DIO_OK;
    }

    // warm start + decay + dynamic-body CSR, all bounded by device counts
    int finish_rows_world(const PrepParams<R>& o, uint32_t n) {
        int pb = 1 - cur_;
        const int gf = std::min(grid_for(cap_.max_contacts, 256), sms_ * 8);
        DIO_CK(launch_k(pdl(), k_warm_sections<P, R>, gf, 256, 0, stream_, w_, (const uint2*)ab_[pb],
                        (const RowDual<P, R>*)rd_[pb], o));
        // counts2_ was cleared by k_cont_rows (build_rows, bodies [0, n))
        if (!n) DIO_CK(cudaMemsetAsync(counts2_, 0, 4, stream_));
        DIO_CK(launch_k(pdl() && n, k_csr_count_dyn<P, R>, gf, 256, 0, stream_, w_, counts2_));
        DIO_CK(ss_.scan(counts2_, w_.row_off, n + 1, pdl(), stream_));
        // takes the counts back to zero
        DIO_CK(launch_k(pdl(), k_csr_scatter_dyn<P, R>, gf, 256, 0, stream_, w_, counts2_));
        int gn = grid_for(n, 256);
        DIO_CK(launch_k(pdl(), k_sort_segments, gn, 256, 0, stream_, (const uint32_t*)w_.row_off, n, w_.max_incid,
                        w_.row_idx, lb_long_, &ctr_->long_count));
        DIO_CK(launch_k(pdl(), k_sort_long, sms_, 512, 0, stream_, (const uint32_t*)w_.row_off, w_.row_idx,
                        (const uint32_t*)lb_long_, (const uint32_t*)&ctr_->long_count, &ctr_->error_flags));
        DIO_CK(launch_k(pdl(), k_csr_other_dyn<P, R>, gn, 256, 0, stream_, w_));
        launches_ += 6;
        return DIO_OK;
    }

    // ---- CUDA graph of one step, one per row-buffer parity ------------
    struct GraphSlot {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        DioAvbdOptions opt{};
        std::vector<std::pair<cudaGraphNode_t, cudaGraphNode_t>> span_nodes;
        std::vector<int> span_kinds;
    };
    GraphSlot graphs_[4];  // (row-buffer parity, LBVH rebuild or refit)
    bool rebuild_now_ = true;
    bool lbvh_valid_ = false;

    void drop_graphs() {
        for (auto& g : graphs_) {
            if (g.exec) cudaGraphExecDestroy(g.exec);
            if (g.graph) cudaGraphDestroy(g.graph);
            g = GraphSlot();
        }
    }

    int capture(GraphSlot& g, const DioAvbdOptions& opt) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        if (g.graph) cudaGraphDestroy(g.graph);
        g = GraphSlot();
        cap_spans_.clear();
        DIO_CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        capturing_ = true;
        const uint64_t l0 = launches_;
        int rc = step_body_dev(opt);
        launches_per_step_ = launches_ - l0;  // counted at replay, not capture
        launches_ = l0;
        capturing_ = false;
        cudaGraph_t graph = nullptr;
        cudaError_t ce = cudaStreamEndCapture(stream_, &graph);
        if (rc != DIO_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        DIO_CK(ce);
        // map the captured event-record nodes back to their spans
        size_t count = 0;
        DIO_CK(cudaGraphGetNodes(graph, nullptr, &count));
        std::vector<cudaGraphNode_t> nodes(count);
        DIO_CK(cudaGraphGetNodes(graph, nodes.data(), &count));
        std::vector<std::pair<cudaEvent_t, cudaGraphNode_t>> ev_nodes;
        for (auto nd : nodes) {
            cudaGraphNodeType t;
            DIO_CK(cudaGraphNodeGetType(nd, &t));
            if (t == cudaGraphNodeTypeEventRecord) {
                cudaEvent_t ev;
                DIO_CK(cudaGraphEventRecordNodeGetEvent(nd, &ev));
                ev_nodes.push_back({ev, nd});
            }
        }
        auto find = [&](cudaEvent_t ev) -> cudaGraphNode_t {
            for (auto& p : ev_nodes)
                if (p.first == ev) return p.second;
            return nullptr;
        };
        for (auto& s : cap_spans_) {
            g.span_nodes.push_back({find(s.a), find(s.b)});
            g.span_kinds.push_back(s.kind);
        }
        DIO_CK(cudaGraphInstantiate(&g.exec, graph, 0));
        g.graph = graph;  // its node handles address the exec's event nodes
        g.opt = opt;
        // the placeholder events now belong to the graph's nodes only
        for (auto& s : cap_spans_) {
            ev_free_.push_back(s.a);
            ev_free_.push_back(s.b);
        }
        cap_spans_.clear();
        return DIO_OK;
    }

    int step_graph(const DioAvbdOptions& opt) {
        plan_rebuild();
        GraphSlot& g = graphs_[cur_ * 2 + (rebuild_now_ ? 1 : 0)];
        if (!g.exec || std::memcmp(&g.opt, &opt, sizeof opt) != 0) DIO_TRY(capture(g, opt));
        for (size_t k = 0; k < g.span_nodes.size(); ++k) {
            if (!g.span_nodes[k].first || !g.span_nodes[k].second) continue;
            cudaEvent_t e0 = take_event(), e1 = take_event();
            DIO_CK(cudaGraphExecEventRecordNodeSetEvent(g.exec, g.span_nodes[k].first, e0));
            DIO_CK(cudaGraphExecEventRecordNodeSetEvent(g.exec, g.span_nodes[k].second, e1));
            spans_.push_back({e0, e1, g.span_kinds[k]});
        }
        DIO_CK(cudaGraphLaunch(g.exec, stream_));
        launches_ += launches_per_step_;
        cur_ = 1 - cur_;
        set_rows(cur_);
        ++steps_;
        return DIO_OK;
    }
    uint64_t launches_per_step_ = 0;

    DioCapacity cap_;
    cudaStream_t stream_;
    DioConfig cfg_;
    DevWorld<P, R> w_{};
    std::vector<void*> allocs_;
    uint32_t per_cap_ = 4;
    int sms_ = 152;
    RowStatic<R>* rs_[2] = {};
    RowDual<P, R>* rd_[2] = {};
    uint2* ab_[2] = {};
    unsigned long long* keys_s_[2] = {};
    uint32_t* ids_s_[2] = {};
    unsigned long long* keys_raw_ = nullptr;
    uint32_t* ids_raw_ = nullptr;
    uint32_t *inc_body_ = nullptr, *inc_row_ = nullptr, *inc_body_s_ = nullptr, *inc_row_s_ = nullptr;
    DioConstraint* joints_ = nullptr;
    uint32_t *joint_off_ = nullptr, *joint_idx_ = nullptr;
    JView* jview_ = nullptr;
    uint32_t* dyn_list_ = nullptr;
    uint32_t* dyn_tmp_ = nullptr;
    uint32_t* dyn_keep_ = nullptr;  // dynamic flags the list was built from
    uint32_t dyn_list_n_ = 0xFFFFFFFFu;
    uint32_t* color_hist_ = nullptr;
    uint32_t ncolors_ = 0;
    uint32_t color_off_h_[kMaxColors + 1] = {};
    uint32_t *counts_ = nullptr, *offsets_ = nullptr, *counts2_ = nullptr, *offsets2_ = nullptr;
    SceneDesc* scenes_ = nullptr;
    std::vector<SceneDesc> scenes_host_;
    bool chunk_world_ = false;  // every scene in a solve chunk, joints inside scenes
    uint32_t scene_max_ = 0;  // bodies in the largest scene
    uint32_t chunk_max_ = 0;  // bodies in the largest scene chunk
    std::vector<uint2> chunks_host_;
    std::vector<uint2> solve_chunks_host_;  // chunks of the scene-chunk solve
    uint2* solve_chunks_ = nullptr;
    uint2* chunk_dyn_ = nullptr;        // each solve chunk's run of the dynamic-body list
    uint32_t* scene_chunk_ = nullptr;   // solve chunk of every scene
    bool chunked_scenes_ = false;       // every scene has a solve chunk
    uint32_t solve_chunk_max_ = 0;      // bodies of the largest solve chunk
    uint2* chunks_ = nullptr;
    Slot<R>* slots_[2] = {nullptr, nullptr};
    // inside step_body_dev: its scratch zeroing is done by k_roll_counters and
    // consecutive kernels of ours are chained by programmatic launch
    bool world_step_ = false;
    bool pdl() const { return world_step_ && !cfg_.profile; }
    int state_pending_ = 0;    // set_state_begin left: 1 the dynamic-set check, 2 a list rebuild
    bool lag_primed_ = false;  // the previous step's slots are this mode's
    uint32_t* chunk_n_ = nullptr;
    uint32_t* chunk_ovf_ = nullptr;
    uint32_t* chunk_tot_ = nullptr;
    uint2* tree_scratch_ = nullptr;
    uint32_t scratch_k_ = 2;
    A4<P>* origin_ = nullptr;
    A4<R>* walls_ = nullptr;
    A4<R>* hull_ = nullptr;
    Counters* ctr_ = nullptr;
    Counters* hctr_ = nullptr;
    ScanSort ss_;  // prefix sums and radix sorts
    void* dstage_ = nullptr;
    void* hstage_ = nullptr;
    size_t stage_bytes_ = 0;
    int cur_ = 0;
    uint32_t n_prev_rows_ = 0;
    uint32_t n_hull_ = 0;  // hull vertices of the uploaded world
    int dual_ctas_per_sm_ = 4;
    uint32_t api_bodies_ = 0, api_n_ = 0, api_m_ = 0, api_iters_ = 0, last_np_ = 0;
    uint64_t steps_ = 0;
    bool world_ready_ = false;
    struct Span {
        cudaEvent_t a, b;
        int kind;
    };
    std::vector<Span> spans_;
    bool capturing_ = false;
    std::vector<Span> cap_spans_;
    std::vector<cudaEvent_t> ev_free_;
    // LBVH buffers
    uint32_t* lb_bounds_ = nullptr;
    uint32_t *lb_keys_ = nullptr, *lb_keys_s_ = nullptr;
    uint32_t *lb_vals_ = nullptr, *lb_leaf_ = nullptr, *lb_parent_ = nullptr, *lb_visits_ = nullptr;
    uint2* lb_children_ = nullptr;
    A4<R>*lb_leaf_min_ = nullptr, *lb_leaf_max_ = nullptr, *lb_node_min_ = nullptr, *lb_node_max_ = nullptr;
    uint32_t *lb_pb_ = nullptr, *lb_long_ = nullptr, *lb_long_count_ = nullptr;
    uint2* lb_gscratch_ = nullptr;  // pairs of the global trees' count pass
    double primal_ms_ = 0.0, dual_ms_ = 0.0;
    double phase_ms_[4] = {0.0, 0.0, 0.0, 0.0};  // broad, narrow, rows, solve
    uint32_t primal_n_ = 0, dual_n_ = 0, solve_chunk_n_ = 0;
    double solve_chunk_ms_ = 0.0;
    uint64_t launches_ = 0;
};

static __global__ void k_keys_only(const uint2* ab, uint32_t m, unsigned long long* keys, uint32_t* ids) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        keys[r] = row_key(ab[r]);
        ids[r] = r;
    }
}

template <class P, class R>
int Engine<P, R>::sort_keys_n(const uint2* ab, uint32_t m, unsigned long long* keys_out, uint32_t* ids_out) {
    k_keys_only<<<grid_for(m, 256), 256, 0, stream_>>>(ab, m, keys_raw_, ids_raw_);
    DIO_CK(ss_.sort_pairs(keys_raw_, keys_out, ids_raw_, ids_out, m, 0u, 64u, false, stream_));
    return DIO_OK;
}

template <class P, class R>
EngineBase* make_engine_t(const DioCapacity& cap, cudaStream_t s, const DioConfig& cfg) {
    auto* e = new Engine<P, R>(cap, s, cfg);
    int rc = e->init();
    if (rc != DIO_OK) {
        std::string msg = e->err;
        delete e;
        return nullptr;
    }
    return e;
}

}  // namespace dio
