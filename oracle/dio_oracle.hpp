// dio_oracle.hpp -- CPU oracle for the Diomedes per-step rigid-body path.
//
// TEST INFRASTRUCTURE ONLY.  This header is a plain C++ restatement of the
// reference's algorithm (nathenjacobe/diomedes) that the tests compare the
// CUDA implementation with and that the bench times as the CPU baseline.  Nothing in the shipped
// library includes or links it.
//
// Parity status: the reference is Rust compiled to SPIR-V (rust-gpu) and
// cannot be built here (no Rust toolchain, un-vendored git dependencies), so
// this restatement is pinned by the reference's own unit-test known answers
// (cuboid.rs:403-422, shape.rs:53-95, physics/gpu.rs:420-433,
// constraints.rs:158-186, render/gpu_physics.rs:701-721) plus analytic
// cases; the AVBD / GJK / EPA / broad-phase / warm-start arithmetic is
// "parity unpinned" beyond those (no golden trajectories exist upstream).
//
// Template parameters
//   P  pose precision: positions, orientations, velocities, lambda
//   R  arithmetic precision: shapes, contact rows, Hessian, LDL, narrow phase
//   <float, float>   reference arithmetic (glam f32)
//   <double, double> the all-FP64 oracle of the same step
//   <double, float>  the split-precision mode
//
// Float op order follows the reference expression by expression (left to
// right, no contraction: compile with -ffp-contract=off).  glam 0.33.3
// (Vec3/Quat/Mat3) is a third-party dependency absent from the reference
// tree; its operations are restated from its published scalar forms:
// Hamilton product with glam's term order, conjugate inverse of a unit
// quaternion, q * v as (w w - b.b) v + 2 (v.b) b + 2 w (b x v), normalise as
// v * (1/|v|).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <utility>
#include <type_traits>
#include <vector>

namespace dio_oracle {

// ------------------------------------------------------------------ math
template <class R>
struct V3 {
    R x, y, z;
};
template <class R>
struct Qt {
    R x, y, z, w;
};

template <class R>
inline V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R>
inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R>
inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R>
inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R>
inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R>
inline V3<R> mulv(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R>
inline V3<R> divs(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R>
inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R>
inline V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R>
inline R length_sq(V3<R> a) { return dot(a, a); }
template <class R>
inline R length(V3<R> a) { return std::sqrt(dot(a, a)); }
template <class R>
inline V3<R> normalize(V3<R> a) { return a * (R(1) / length(a)); }
template <class R>
inline V3<R> normalize_or_zero(V3<R> a) {
    R rcp = R(1) / length(a);
    if (std::isfinite(rcp) && rcp > R(0)) return a * rcp;
    return {R(0), R(0), R(0)};
}
template <class T, class R>
inline V3<T> cast3(V3<R> a) { return {T(a.x), T(a.y), T(a.z)}; }
template <class T, class R>
inline Qt<T> castq(Qt<R> q) { return {T(q.x), T(q.y), T(q.z), T(q.w)}; }

// Hamilton product a * b.
template <class R>
inline Qt<R> qmul(Qt<R> a, Qt<R> b) {
    return {a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
            a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
            a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w,
            a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
}
// Inverse of a unit quaternion (the conjugate).
template <class R>
inline Qt<R> conj(Qt<R> q) { return {-q.x, -q.y, -q.z, q.w}; }
// q * v for unit q (glam 0.33.3 Quat::mul_vec3, the published scalar form
// that the shader build and glam's scalar path evaluate): with b = q.xyz,
//   v (w w - b.b) + b (2 (v.b)) + (b x v) (2 w)
// -- every product rounded, sums left to right.  DIO_ORACLE_ROTATE_TQ
// selects the algebraically equal v + w t + b x t, t = 2 (b x v), which the
// tests build separately to measure how far the rotation's rounding alone
// moves a step.
template <class R>
inline V3<R> rotate(Qt<R> q, V3<R> v) {
    V3<R> b{q.x, q.y, q.z};
#ifdef DIO_ORACLE_ROTATE_TQ
    V3<R> t = cross(b, v) * R(2);
    return v + t * q.w + cross(b, t);
#else
    const R b2 = dot(b, b);
    return v * (q.w * q.w - b2) + b * (dot(v, b) * R(2)) + cross(b, v) * (q.w * R(2));
#endif
}
template <class R>
inline Qt<R> qnormalize(Qt<R> q) {
    R len = std::sqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    R inv = R(1) / len;
    return {q.x * inv, q.y * inv, q.z * inv, q.w * inv};
}
// quat_step, engine/gpu_physics/avbd/src/lib.rs:91-94:
// normalize(q + (delta, 0) * q * 0.5)
template <class R>
inline Qt<R> quat_step(Qt<R> q, V3<R> d) {
    Qt<R> p{d.x, d.y, d.z, R(0)};
    Qt<R> s = qmul(p, q);
    s = {s.x * R(0.5), s.y * R(0.5), s.z * R(0.5), s.w * R(0.5)};
    return qnormalize(Qt<R>{q.x + s.x, q.y + s.y, q.z + s.z, q.w + s.w});
}
// quat_step of the split mode: the increment (d, 0) * q / 2 is formed in R
// from the rounded quaternion and added to the P quaternion; 1/|q| is seeded
// in R (correctly rounded sqrt and division) and refined by one Newton step
// in P (relative error ~1e-14; the quaternion is renormalised every step),
// or taken in P when |u|^2 lies outside [1e-30, 1e30].
template <class P, class R>
inline Qt<P> quat_step_split(Qt<P> q, V3<R> d) {
    Qt<R> s = qmul(Qt<R>{d.x, d.y, d.z, R(0)}, castq<R>(q));
    s = {s.x * R(0.5), s.y * R(0.5), s.z * R(0.5), s.w * R(0.5)};
    const Qt<P> u{q.x + P(s.x), q.y + P(s.y), q.z + P(s.z), q.w + P(s.w)};
    const P n = u.x * u.x + u.y * u.y + u.z * u.z + u.w * u.w;
    // an R seed only where n and its root stay well inside R's range; a
    // quaternion blown up by a huge increment (|u|^2 beyond R) is normalised
    // in P (an R seed would overflow to a zero quaternion, then NaN)
    P r;
    if (n > P(1.0e-30) && n < P(1.0e30)) {
        r = P(R(1) / std::sqrt(R(n)));
        r = r * (P(1.5) - P(0.5) * n * r * r);
    } else {
        r = P(1) / std::sqrt(n);
    }
    return {u.x * r, u.y * r, u.z * r, u.w * r};
}
// ang_diff, engine/gpu_physics/avbd/src/lib.rs:96-99: 2 * vec(to * from^-1)
template <class R>
inline V3<R> ang_diff(Qt<R> to, Qt<R> from) {
    Qt<R> rel = qmul(to, conj(from));
    return {R(2) * rel.x, R(2) * rel.y, R(2) * rel.z};
}

// ---------------------------------------------------------------- shapes
enum : uint32_t { SPHERE = 0, CUBE = 1, TETRAHEDRON = 2, BOX = 3, HULL = 4 };
constexpr uint32_t CONTAINER = 0xFFFFFFFFu;
enum : uint32_t { SPRING = 0, ROD = 1, BALL_SOCKET = 2, ROPE = 3 };

template <class R>
struct Shape {
    uint32_t tag = SPHERE;
    uint32_t hull_first = 0, hull_count = 0;
    V3<R> c[4] = {};  // corners[i].xyz
};

// support, engine/gpu_physics/narrowphase/src/support.rs:21-61 (and the
// identical broadphase/src/lib.rs:79-114).  Tetrahedron / hull ties keep the
// FIRST maximal corner (strict >).  BOX shares the cube's sign select; HULL
// is the same first-max rule over its vertex list.
template <class R>
inline V3<R> support(const Shape<R>& s, V3<R> d, const V3<R>* hull) {
    switch (s.tag) {
        case SPHERE:
            return normalize_or_zero(d) * s.c[0].x;
        case CUBE:
        case BOX:
            return {d.x >= R(0) ? s.c[0].x : -s.c[0].x, d.y >= R(0) ? s.c[0].y : -s.c[0].y,
                    d.z >= R(0) ? s.c[0].z : -s.c[0].z};
        case TETRAHEDRON: {
            V3<R> best = s.c[0];
            R best_dot = dot(best, d);
            for (int i = 1; i < 4; ++i) {
                R dd = dot(s.c[i], d);
                if (dd > best_dot) {
                    best_dot = dd;
                    best = s.c[i];
                }
            }
            return best;
        }
        case HULL: {
            if (s.hull_count == 0 || hull == nullptr) return {R(0), R(0), R(0)};
            V3<R> best = hull[s.hull_first];
            R best_dot = dot(best, d);
            for (uint32_t i = 1; i < s.hull_count; ++i) {
                V3<R> v = hull[s.hull_first + i];
                R dd = dot(v, d);
                if (dd > best_dot) {
                    best_dot = dd;
                    best = v;
                }
            }
            return best;
        }
        default:
            return {R(0), R(0), R(0)};
    }
}

template <class R>
struct NBody {  // GpuBody as the kernels see it
    V3<R> pos;
    Qt<R> rot;
    Shape<R> shape;
};

template <class R>
inline V3<R> world_support(const NBody<R>& b, V3<R> d, const V3<R>* hull) {
    V3<R> local = rotate(conj(b.rot), d);
    return rotate(b.rot, support(b.shape, local, hull)) + b.pos;
}

// ------------------------------------------------------------ broad phase
// aabb, engine/gpu_physics/broadphase/src/lib.rs:121-151
template <class R>
inline void aabb(const NBody<R>& b, const V3<R>* hull, V3<R>& mn, V3<R>& mx) {
    const V3<R> X{R(1), R(0), R(0)}, Y{R(0), R(1), R(0)}, Z{R(0), R(0), R(1)};
    mn = b.pos;
    mx = b.pos;
    V3<R> sx = world_support(b, X, hull);
    V3<R> snx = world_support(b, -X, hull);
    V3<R> sy = world_support(b, Y, hull);
    V3<R> sny = world_support(b, -Y, hull);
    V3<R> sz = world_support(b, Z, hull);
    V3<R> snz = world_support(b, -Z, hull);
    if (sx.x > mx.x) mx.x = sx.x;
    if (snx.x < mn.x) mn.x = snx.x;
    if (sy.y > mx.y) mx.y = sy.y;
    if (sny.y < mn.y) mn.y = sny.y;
    if (sz.z > mx.z) mx.z = sz.z;
    if (snz.z < mn.z) mn.z = snz.z;
}

template <class R>
inline bool overlap(const V3<R>& mna, const V3<R>& mxa, const V3<R>& mnb, const V3<R>& mxb) {
    // broad_sweep_dense closed-interval test, broadphase/src/lib.rs:195-200
    return mna.x <= mxb.x && mnb.x <= mxa.x && mna.y <= mxb.y && mnb.y <= mxa.y &&
           mna.z <= mxb.z && mnb.z <= mxa.z;
}

// broad_sweep_dense, broadphase/src/lib.rs:171-216, restated sequentially:
// every i < j whose AABBs overlap, in (i, j) lexicographic order, for bodies
// [lo, hi).  The reference appends in arbitrary atomic order; this
// canonical order is the set sorted by (a, b).
template <class R>
inline void broad_dense(const std::vector<V3<R>>& mn, const std::vector<V3<R>>& mx,
                        uint32_t lo, uint32_t hi, std::vector<std::pair<uint32_t, uint32_t>>& out) {
    for (uint32_t i = lo; i < hi; ++i)
        for (uint32_t j = i + 1; j < hi; ++j)
            if (overlap(mn[i], mx[i], mn[j], mx[j])) out.push_back({i, j});
}

// Same pair set by sort-and-sweep (a faster CPU broad phase used by the CPU
// baseline) along the axis on which the scene's boxes spread widest (a wall
// standing in the y-z plane would make a sweep on x quadratic); the
// closed-interval test is identical, so the set is identical to broad_dense
// for any axis, and sorting restores the canonical order.
template <class R>
inline R axis_of(const V3<R>& v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
template <class R>
inline void broad_sap(const std::vector<V3<R>>& mn, const std::vector<V3<R>>& mx, uint32_t lo,
                      uint32_t hi, std::vector<std::pair<uint32_t, uint32_t>>& out) {
    if (hi <= lo) return;
    int ax = 0;
    R best = R(-1);
    for (int k = 0; k < 3; ++k) {
        R a = axis_of(mn[lo], k), b = a;
        for (uint32_t i = lo + 1; i < hi; ++i) {
            const R v = axis_of(mn[i], k);
            a = v < a ? v : a;
            b = v > b ? v : b;
        }
        if (b - a > best) {
            best = b - a;
            ax = k;
        }
    }
    std::vector<uint32_t> order;
    for (uint32_t i = lo; i < hi; ++i) order.push_back(i);
    std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        const R ka = axis_of(mn[a], ax), kb = axis_of(mn[b], ax);
        return ka < kb || (ka == kb && a < b);
    });
    size_t start = out.size();
    for (size_t s = 0; s < order.size(); ++s) {
        uint32_t i = order[s];
        const R end = axis_of(mx[i], ax);
        for (size_t t = s + 1; t < order.size(); ++t) {
            uint32_t j = order[t];
            if (!(axis_of(mn[j], ax) <= end)) break;
            if (overlap(mn[i], mx[i], mn[j], mx[j])) out.push_back({std::min(i, j), std::max(i, j)});
        }
    }
    std::sort(out.begin() + start, out.end());
}

// ------------------------------------------------------------ narrow phase
template <class R>
struct Slot {  // GpuContactOut, compute.rs:123-133
    uint32_t valid = 0, a = 0, b = 0;
    V3<R> normal{};
    R depth = 0;
    V3<R> point_a{}, point_b{};
};

template <class R>
struct Manifold {
    V3<R> normal{};
    R depth = 0;
    V3<R> pa[8], pb[8];
    uint32_t count = 0;
};

template <class R>
inline void axes_of(const NBody<R>& b, V3<R> ax[3]) {
    ax[0] = rotate(b.rot, V3<R>{R(1), R(0), R(0)});
    ax[1] = rotate(b.rot, V3<R>{R(0), R(1), R(0)});
    ax[2] = rotate(b.rot, V3<R>{R(0), R(0), R(1)});
}

// Projected radius of a box along `axis`.  CUBE follows cuboid.rs:37-40
// (half * (|.| + |.| + |.|) with half = corners[0].x); BOX (extension)
// weights each axis by its own half extent.
template <class R>
inline R box_radius(const NBody<R>& b, const V3<R> ax[3], V3<R> axis, bool per_axis) {
    if (!per_axis) {
        R half = b.shape.c[0].x;
        return half * (std::fabs(dot(axis, ax[0])) + std::fabs(dot(axis, ax[1])) +
                       std::fabs(dot(axis, ax[2])));
    }
    V3<R> h = b.shape.tag == BOX ? b.shape.c[0] : V3<R>{b.shape.c[0].x, b.shape.c[0].x, b.shape.c[0].x};
    return h.x * std::fabs(dot(axis, ax[0])) + h.y * std::fabs(dot(axis, ax[1])) +
           h.z * std::fabs(dot(axis, ax[2]));
}
template <class R>
inline R half_along(const NBody<R>& b, uint32_t i, bool per_axis) {
    if (!per_axis || b.shape.tag != BOX) return b.shape.c[0].x;
    return i == 0 ? b.shape.c[0].x : (i == 1 ? b.shape.c[0].y : b.shape.c[0].z);
}

template <class R>
struct SatBest {
    R overlap;
    V3<R> normal;
    uint32_t kind, index;
};

// test_axis, engine/gpu_physics/narrowphase/src/cuboid.rs:19-52
template <class R>
inline bool test_axis(V3<R> raw, uint32_t kind, uint32_t index, const NBody<R>& a, const V3<R> aax[3],
                      const NBody<R>& b, const V3<R> bax[3], V3<R> delta, bool per_axis,
                      SatBest<R>& best) {
    if (length_sq(raw) <= R(1.0e-8)) return true;
    V3<R> axis = normalize(raw);
    R ra = box_radius(a, aax, axis, per_axis);
    R rb = box_radius(b, bax, axis, per_axis);
    R ov = ra + rb - std::fabs(dot(delta, axis));
    if (ov < R(0)) return false;
    if (ov < best.overlap) {
        best.overlap = ov;
        best.normal = dot(delta, axis) >= R(0) ? axis : -axis;
        best.kind = kind;
        best.index = index;
    }
    return true;
}

// sat, cuboid.rs:54-167: 3 face axes of a, 3 of b, then 9 edge crosses.
template <class R>
inline bool sat(const NBody<R>& a, const NBody<R>& b, bool per_axis, SatBest<R>& best) {
    V3<R> aax[3], bax[3];
    axes_of(a, aax);
    axes_of(b, bax);
    V3<R> delta = b.pos - a.pos;
    best.overlap = std::numeric_limits<R>::max();
    best.normal = {R(1), R(0), R(0)};
    best.kind = 0;
    best.index = 0;
    for (uint32_t i = 0; i < 3; ++i)
        if (!test_axis(aax[i], 0, i, a, aax, b, bax, delta, per_axis, best)) return false;
    for (uint32_t i = 0; i < 3; ++i)
        if (!test_axis(bax[i], 1, i, a, aax, b, bax, delta, per_axis, best)) return false;
    for (uint32_t i = 0; i < 3; ++i)
        for (uint32_t j = 0; j < 3; ++j)
            if (!test_axis(cross(aax[i], bax[j]), 2, i * 3 + j, a, aax, b, bax, delta, per_axis, best))
                return false;
    return true;
}

// face_frame, cuboid.rs:169-196 (per-axis extents for BOX)
template <class R>
inline void face_frame(const NBody<R>& body, uint32_t axis_index, V3<R> outward, bool per_axis,
                       V3<R> verts[4], V3<R>& center, V3<R>& u, V3<R>& v, R& eu, R& ev) {
    V3<R> ax[3];
    axes_of(body, ax);
    V3<R> axis = ax[axis_index];
    V3<R> fn = axis * (dot(axis, outward) >= R(0) ? R(1) : R(-1));
    R hn = half_along(body, axis_index, per_axis);
    center = body.pos + fn * hn;
    uint32_t ui, vi;
    if (axis_index == 0) {
        ui = 1;
        vi = 2;
    } else if (axis_index == 1) {
        ui = 0;
        vi = 2;
    } else {
        ui = 0;
        vi = 1;
    }
    u = ax[ui];
    v = ax[vi];
    eu = half_along(body, ui, per_axis);
    ev = half_along(body, vi, per_axis);
    verts[0] = center + u * eu + v * ev;
    verts[1] = center - u * eu + v * ev;
    verts[2] = center - u * eu - v * ev;
    verts[3] = center + u * eu - v * ev;
}

// incident_axis, cuboid.rs:198-214
template <class R>
inline uint32_t incident_axis(const NBody<R>& body, V3<R> n) {
    V3<R> ax[3];
    axes_of(body, ax);
    uint32_t best_axis = 0;
    R best_dot = std::fabs(dot(ax[0], n));
    for (uint32_t i = 1; i < 3; ++i) {
        R d = std::fabs(dot(ax[i], n));
        if (d > best_dot) {
            best_dot = d;
            best_axis = i;
        }
    }
    return best_axis;
}

// clip_plane, cuboid.rs:216-250 (Sutherland-Hodgman, at most 8 points)
template <class R>
inline uint32_t clip_plane(const V3<R> in[8], uint32_t n_in, V3<R> normal, R offset, V3<R> out[8]) {
    if (n_in == 0) return 0;
    uint32_t count = 0;
    V3<R> prev = in[n_in - 1];
    R prev_d = dot(normal, prev) - offset;
    for (uint32_t i = 0; i < n_in; ++i) {
        V3<R> cur = in[i];
        R cur_d = dot(normal, cur) - offset;
        bool prev_in = prev_d <= R(1.0e-5);
        bool cur_in = cur_d <= R(1.0e-5);
        if (prev_in != cur_in) {
            R den = prev_d - cur_d;
            if (std::fabs(den) > R(1.0e-8) && count < 8) {
                R t = prev_d / den;
                t = t < R(0) ? R(0) : (t > R(1) ? R(1) : t);
                out[count++] = prev + (cur - prev) * t;
            }
        }
        if (cur_in && count < 8) out[count++] = cur;
        prev = cur;
        prev_d = cur_d;
    }
    return count;
}

// centered_contact, cuboid.rs:252-272
template <class R>
inline Manifold<R> centered_contact(const NBody<R>& a, const NBody<R>& b, V3<R> normal, R depth,
                                    bool per_axis) {
    V3<R> aax[3], bax[3];
    axes_of(a, aax);
    axes_of(b, bax);
    R ra = box_radius(a, aax, normal, per_axis);
    R rb = box_radius(b, bax, normal, per_axis);
    Manifold<R> m;
    m.normal = normal;
    m.depth = depth;
    for (int i = 0; i < 8; ++i) m.pa[i] = m.pb[i] = V3<R>{R(0), R(0), R(0)};
    m.pa[0] = a.pos + normal * ra;
    m.pb[0] = b.pos - normal * rb;
    m.count = 1;
    return m;
}

// collide_manifold, cuboid.rs:276-377.  max_contacts = 4 is the reference;
// 8 keeps every clipped point (extended manifold).
template <class R>
inline bool collide_manifold(const NBody<R>& a, const NBody<R>& b, uint32_t max_contacts,
                             Manifold<R>& out) {
    bool a_box = a.shape.tag == CUBE || a.shape.tag == BOX;
    bool b_box = b.shape.tag == CUBE || b.shape.tag == BOX;
    if (!a_box || !b_box) return false;
    bool per_axis = !(a.shape.tag == CUBE && b.shape.tag == CUBE);
    SatBest<R> best;
    if (!sat(a, b, per_axis, best)) return false;
    V3<R> normal = best.normal;
    R depth = best.overlap;
    if (best.kind == 2) {
        out = centered_contact(a, b, normal, depth, per_axis);
        return true;
    }
    bool ref_is_a = best.kind == 0;
    V3<R> rn = ref_is_a ? normal : -normal;
    const NBody<R>& refb = ref_is_a ? a : b;
    const NBody<R>& incb = ref_is_a ? b : a;
    uint32_t inc_axis = incident_axis(incb, rn);
    V3<R> ref_face[4], center, u, v;
    R eu, ev;
    face_frame(refb, best.index, rn, per_axis, ref_face, center, u, v, eu, ev);
    V3<R> pa[8], pb[8], inc_face[4], c2, u2, v2;
    R eu2, ev2;
    face_frame(incb, inc_axis, -rn, per_axis, inc_face, c2, u2, v2, eu2, ev2);
    for (int i = 0; i < 8; ++i) pa[i] = pb[i] = V3<R>{R(0), R(0), R(0)};
    for (int i = 0; i < 4; ++i) pa[i] = inc_face[i];
    uint32_t count = 4;
    count = clip_plane(pa, count, u, dot(u, center) + eu, pb);
    count = clip_plane(pb, count, -u, dot(-u, center) + eu, pa);
    count = clip_plane(pa, count, v, dot(v, center) + ev, pb);
    count = clip_plane(pb, count, -v, dot(-v, center) + ev, pa);
    if (count == 0) {
        out = centered_contact(a, b, normal, depth, per_axis);
        return true;
    }
    R ref_plane = dot(rn, center);
    Manifold<R> m;
    for (int i = 0; i < 8; ++i) m.pa[i] = m.pb[i] = V3<R>{R(0), R(0), R(0)};
    uint32_t cc = 0;
    for (uint32_t i = 0; i < count; ++i) {
        if (cc >= max_contacts) break;
        V3<R> ip = pa[i];
        R pd = ref_plane - dot(rn, ip);
        if (pd < R(-1.0e-5)) continue;
        V3<R> rp = ip + rn * (pd > R(0) ? pd : R(0));
        if (ref_is_a) {
            m.pa[cc] = rp;
            m.pb[cc] = ip;
        } else {
            m.pa[cc] = ip;
            m.pb[cc] = rp;
        }
        ++cc;
    }
    if (cc == 0) {
        out = centered_contact(a, b, normal, depth, per_axis);
        return true;
    }
    m.normal = normal;
    m.depth = depth;
    m.count = cc;
    out = m;
    return true;
}

// ----------------------------------------------------------------- GJK
template <class R>
struct Simplex {  // gjk.rs:14-63
    V3<R> p[4], w[4];
    uint32_t len = 0;
    void push_front(V3<R> point, V3<R> wit) {
        for (uint32_t i = len; i > 0; --i) {
            p[i] = p[i - 1];
            w[i] = w[i - 1];
        }
        p[0] = point;
        w[0] = wit;
        len = std::min<uint32_t>(len + 1, 4);
    }
    void remove(uint32_t index) {
        for (uint32_t i = index; i + 1 < len; ++i) {
            p[i] = p[i + 1];
            w[i] = w[i + 1];
        }
        len -= 1;
    }
    void swap(uint32_t i, uint32_t j) {
        std::swap(p[i], p[j]);
        std::swap(w[i], w[j]);
    }
};

// world_support_witness, gjk.rs:67-73
template <class R>
inline void support_witness(const NBody<R>& a, const NBody<R>& b, V3<R> d, const V3<R>* hull,
                            V3<R>& point, V3<R>& wit) {
    V3<R> al = rotate(conj(a.rot), d);
    V3<R> ap = rotate(a.rot, support(a.shape, al, hull)) + a.pos;
    V3<R> bl = rotate(conj(b.rot), -d);
    V3<R> bp = rotate(b.rot, support(b.shape, bl, hull)) + b.pos;
    point = ap - bp;
    wit = ap;
}

template <class R>
inline bool same_dir(V3<R> a, V3<R> b) { return dot(a, b) > R(0); }
template <class R>
inline V3<R> triple(V3<R> a, V3<R> b, V3<R> c) { return cross(cross(a, b), c); }
// any_perpendicular, gjk.rs:214-223
template <class R>
inline V3<R> any_perpendicular(V3<R> v) {
    V3<R> axis;
    if (std::fabs(v.x) <= std::fabs(v.y) && std::fabs(v.x) <= std::fabs(v.z))
        axis = {R(1), R(0), R(0)};
    else if (std::fabs(v.y) <= std::fabs(v.z))
        axis = {R(0), R(1), R(0)};
    else
        axis = {R(0), R(0), R(1)};
    return normalize_or_zero(cross(axis, v));
}

// contains_origin, gjk.rs:112-201
template <class R>
inline bool contains_origin(Simplex<R>& s, V3<R>& d) {
    if (s.len == 4) {
        V3<R> a = s.p[0], b = s.p[1], c = s.p[2], dd = s.p[3];
        V3<R> ao = -a, ab = b - a, ac = c - a, ad = dd - a;
        V3<R> abc = cross(ab, ac), acd = cross(ac, ad), adb = cross(ad, ab);
        if (same_dir(abc, ao))
            s.remove(3);
        else if (same_dir(acd, ao))
            s.remove(1);
        else if (same_dir(adb, ao))
            s.remove(2);
        else
            return true;
    }
    switch (s.len) {
        case 1:
            d = -s.p[0];
            return false;
        case 2: {
            V3<R> a = s.p[0], b = s.p[1];
            V3<R> ab = b - a, ao = -a;
            if (same_dir(ab, ao)) {
                V3<R> t = triple(ab, ao, ab);
                if (length_sq(t) < R(1e-12)) t = any_perpendicular(ab);
                d = t;
            } else {
                s.remove(1);
                d = ao;
            }
            return false;
        }
        case 3: {
            V3<R> a = s.p[0], b = s.p[1], c = s.p[2];
            V3<R> ab = b - a, ac = c - a, ao = -a;
            V3<R> abc = cross(ab, ac);
            if (same_dir(cross(abc, ac), ao)) {
                if (same_dir(ac, ao)) {
                    s.remove(1);
                    d = triple(ac, ao, ac);
                } else if (same_dir(ab, ao)) {
                    s.remove(2);
                    d = triple(ab, ao, ab);
                } else {
                    s.len = 1;
                    d = ao;
                }
            } else if (same_dir(cross(ab, abc), ao)) {
                if (same_dir(ab, ao)) {
                    s.remove(2);
                    d = triple(ab, ao, ab);
                } else {
                    s.len = 1;
                    d = ao;
                }
            } else {
                if (dot(abc, ao) > R(0)) {
                    d = abc;
                } else {
                    s.swap(1, 2);
                    d = -abc;
                }
            }
            return false;
        }
        default:
            return false;
    }
}

// gjk, gjk.rs:77-109 (64 iterations)
template <class R>
inline bool gjk(const NBody<R>& a, const NBody<R>& b, const V3<R>* hull, Simplex<R>& out) {
    V3<R> d = a.pos - b.pos;
    if (d.x == R(0) && d.y == R(0) && d.z == R(0)) d = {R(1), R(0), R(0)};
    Simplex<R> s;
    V3<R> pt, wt;
    support_witness(a, b, d, hull, pt, wt);
    s.push_front(pt, wt);
    d = -s.p[0];
    for (int it = 0; it < 64; ++it) {
        support_witness(a, b, d, hull, pt, wt);
        if (dot(pt, d) < R(0)) return false;
        s.push_front(pt, wt);
        if (contains_origin(s, d)) {
            out = s;
            return true;
        }
        if (length_sq(d) < R(1e-12)) d = any_perpendicular(s.p[0]);
    }
    return false;
}

// ----------------------------------------------------------------- EPA
template <class R>
struct Face {
    uint32_t a = 0, b = 0, c = 0;
    V3<R> normal{};
    R distance = 0;
};

constexpr uint32_t EPA_MAX_VERTICES = 256;
constexpr uint32_t EPA_MAX_FACES = 512;

template <class R>
struct Polytope {  // epa.rs:33-86
    V3<R> v[EPA_MAX_VERTICES];
    V3<R> w[EPA_MAX_VERTICES];
    Face<R> f[EPA_MAX_FACES];
    uint32_t nv = 0, nf = 0;
    Polytope() {
        for (auto& x : v) x = V3<R>{R(0), R(0), R(0)};
        for (auto& x : w) x = V3<R>{R(0), R(0), R(0)};
    }
    void add_face(uint32_t a, uint32_t b, uint32_t c) {
        if (nf >= EPA_MAX_FACES) return;
        V3<R> va = v[a];
        V3<R> n = cross(v[b] - va, v[c] - va);
        if (length_sq(n) < R(1e-12)) return;
        n = normalize(n);
        Face<R> face;
        face.a = a;
        face.b = b;
        face.c = c;
        face.normal = n;
        face.distance = dot(n, va);
        if (face.distance < R(0)) {
            face.a = c;
            face.c = a;
            face.normal = -face.normal;
            face.distance = -face.distance;
        }
        f[nf++] = face;
    }
};

template <class R>
struct Penetration {
    V3<R> normal;
    R depth;
    V3<R> pa, pb;
};

// face_contact, epa.rs:193-240
template <class R>
inline Penetration<R> face_contact(const Face<R>& face, const Polytope<R>& poly) {
    V3<R> va = poly.v[face.a], vb = poly.v[face.b], vc = poly.v[face.c];
    V3<R> closest = face.normal * face.distance;
    V3<R> v0 = vb - va, v1 = vc - va, v2 = closest - va;
    R d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0), d21 = dot(v2, v1);
    R denom = d00 * d11 - d01 * d01;
    R w1, w2, w3;
    if (std::fabs(denom) > R(1e-12)) {
        w2 = (d11 * d20 - d01 * d21) / denom;
        w3 = (d00 * d21 - d01 * d20) / denom;
        w1 = R(1) - w2 - w3;
    } else {
        w1 = R(1);
        w2 = R(0);
        w3 = R(0);
    }
    auto clamp01 = [](R x) { return x < R(0) ? R(0) : (x > R(1) ? R(1) : x); };
    w1 = clamp01(w1);
    w2 = clamp01(w2);
    w3 = clamp01(w3);
    R sum = w1 + w2 + w3;
    if (sum > R(1e-12)) {
        w1 = w1 / sum;
        w2 = w2 / sum;
        w3 = w3 / sum;
    } else {
        w1 = R(1);
        w2 = R(0);
        w3 = R(0);
    }
    V3<R> wa = poly.w[face.a], wb = poly.w[face.b], wc = poly.w[face.c];
    V3<R> pa = wa * w1 + wb * w2 + wc * w3;
    V3<R> mk = va * w1 + vb * w2 + vc * w3;
    return {face.normal, face.distance, pa, pa - mk};
}

template <class R>
inline bool edge_in_face(uint32_t a, uint32_t b, const Face<R>& f) {
    return (f.a == a && f.b == b) || (f.b == a && f.c == b) || (f.c == a && f.a == b) ||
           (f.a == b && f.b == a) || (f.b == b && f.c == a) || (f.c == b && f.a == a);
}

// epa, epa.rs:89-189.  `overflow` reports a horizon larger than the
// reference's fixed array (a case the reference would index out of bounds).
template <class R>
inline bool epa(const NBody<R>& a, const NBody<R>& b, const Simplex<R>& s, const V3<R>* hull,
                Penetration<R>& out, bool* overflow = nullptr) {
    static thread_local Polytope<R> poly_storage;
    Polytope<R>& poly = poly_storage;
    poly = Polytope<R>();
    for (uint32_t i = 0; i < s.len; ++i) {
        poly.v[i] = s.p[i];
        poly.w[i] = s.w[i];
    }
    poly.nv = s.len;
    poly.add_face(0, 1, 2);
    poly.add_face(0, 3, 1);
    poly.add_face(0, 2, 3);
    poly.add_face(1, 3, 2);
    static thread_local std::vector<uint32_t> visible;
    static thread_local std::vector<std::pair<uint32_t, uint32_t>> horizon;
    for (int it = 0; it < 64; ++it) {
        // no face of nonzero area (a flat or collapsed simplex): no contact.
        // The reference would take its zero default face here and emit a
        // zero normal at zero depth (epa.rs:44-66,102-123), whose tangents
        // are NaN -- a deliberate difference.
        if (poly.nf == 0) return false;
        uint32_t mi = 0;
        R md = poly.f[0].distance;
        for (uint32_t i = 1; i < poly.nf; ++i)
            if (poly.f[i].distance < md) {
                md = poly.f[i].distance;
                mi = i;
            }
        Face<R> mf = poly.f[mi];
        V3<R> sp, sw;
        support_witness(a, b, mf.normal, hull, sp, sw);
        R sd = dot(mf.normal, sp);
        if (sd - mf.distance < R(1e-4)) {
            out = face_contact(poly.f[mi], poly);
            return true;
        }
        uint32_t ni = poly.nv;
        if (ni >= EPA_MAX_VERTICES) {
            out = face_contact(poly.f[mi], poly);
            return true;
        }
        poly.v[ni] = sp;
        poly.w[ni] = sw;
        poly.nv += 1;
        visible.assign(poly.nf, 0);
        for (uint32_t i = 0; i < poly.nf; ++i) {
            const Face<R>& f = poly.f[i];
            visible[i] = dot(f.normal, sp - poly.v[f.a]) > R(0) ? 1u : 0u;
        }
        horizon.clear();
        for (uint32_t i = 0; i < poly.nf; ++i) {
            if (!visible[i]) continue;
            const Face<R> f = poly.f[i];
            uint32_t e[3][2] = {{f.a, f.b}, {f.b, f.c}, {f.c, f.a}};
            for (int k = 0; k < 3; ++k) {
                bool shared = false;
                for (uint32_t j = 0; j < poly.nf; ++j) {
                    if (j == i) continue;
                    if (visible[j] && edge_in_face(e[k][0], e[k][1], poly.f[j])) {
                        shared = true;
                        break;
                    }
                }
                if (!shared) horizon.push_back({e[k][0], e[k][1]});
            }
        }
        if (horizon.size() > EPA_MAX_FACES && overflow) *overflow = true;
        uint32_t wr = 0;
        for (uint32_t i = 0; i < poly.nf; ++i)
            if (!visible[i]) poly.f[wr++] = poly.f[i];
        poly.nf = wr;
        for (auto& h : horizon) poly.add_face(ni, h.first, h.second);
    }
    return false;
}

// narrowphase_main, engine/gpu_physics/narrowphase/src/lib.rs:89-158, for
// one pair: fills `slots[0..per_pair)` (all cleared first, as the host
// zero-fill at compute.rs:625-626 does).  Returns the number written.
template <class R>
inline uint32_t narrow_pair(const NBody<R>& a, const NBody<R>& b, uint32_t ia, uint32_t ib,
                            const V3<R>* hull, uint32_t per_pair, Slot<R>* slots,
                            bool* overflow = nullptr) {
    for (uint32_t k = 0; k < per_pair; ++k) slots[k] = Slot<R>();
    auto write = [&](uint32_t k, V3<R> n, R depth, V3<R> pa, V3<R> pb) {
        slots[k].valid = 1;
        slots[k].a = ia;
        slots[k].b = ib;
        slots[k].normal = n;
        slots[k].depth = depth;
        slots[k].point_a = pa;
        slots[k].point_b = pb;
    };
    bool a_box = a.shape.tag == CUBE || a.shape.tag == BOX;
    bool b_box = b.shape.tag == CUBE || b.shape.tag == BOX;
    if (a_box && b_box) {
        Manifold<R> m;
        if (collide_manifold(a, b, per_pair, m)) {
            for (uint32_t k = 0; k < m.count; ++k) write(k, m.normal, m.depth, m.pa[k], m.pb[k]);
            return m.count;
        }
        return 0;
    }
    if (a.shape.tag == SPHERE && b.shape.tag == SPHERE) {
        V3<R> delta = b.pos - a.pos;
        R dist = length(delta);
        R radius = a.shape.c[0].x + b.shape.c[0].x;
        if (dist >= radius || dist <= R(1.1920928955078125e-7)) return 0;
        V3<R> n = divs(delta, dist);
        write(0, n, radius - dist, a.pos + n * a.shape.c[0].x, b.pos - n * b.shape.c[0].x);
        return 1;
    }
    Simplex<R> s;
    if (gjk(a, b, hull, s)) {
        Penetration<R> pen;
        if (epa(a, b, s, hull, pen, overflow)) {
            write(0, pen.normal, pen.depth, pen.pa, pen.pb);
            return 1;
        }
    }
    return 0;
}

// ---------------------------------------------------------- contact rows
template <class P, class R>
struct Row {  // AvbdContact, engine/src/physics/gpu.rs:103-115
    uint32_t a = 0, b = 0;
    R friction = 0;
    V3<R> n{}, t1{}, t2{}, ra{}, rb{}, c0{}, penalty{};
    V3<P> lambda{};
};

template <class R>
struct Options {  // AvbdOptions, engine/src/physics/gpu.rs:127-155
    R dt = R(1) / R(60);
    V3<R> gravity{R(0), R(-10), R(0)};
    uint32_t iterations = 10;
    R alpha = R(0.99), beta_lin = R(10000), margin = R(0.01), penalty_min = R(1),
      penalty_max = R(1e10), gamma = R(0.999), friction = R(0.8);
};

// tangents, engine/src/physics/gpu.rs:406-414
template <class R>
inline void tangents(V3<R> n, V3<R>& t1, V3<R>& t2) {
    V3<R> c = std::fabs(n.x) > R(0.9) ? cross(n, V3<R>{R(0), R(1), R(0)}) : cross(n, V3<R>{R(1), R(0), R(0)});
    t1 = normalize(c);
    t2 = cross(n, t1);
}

// raw_contact, engine/src/physics/gpu.rs:239-264
template <class P, class R>
inline Row<P, R> raw_contact(uint32_t a, uint32_t b, const NBody<R>& ba, const NBody<R>& bb, V3<R> normal,
                             R depth, V3<R> pa, V3<R> pb, const Options<R>& o) {
    Row<P, R> r;
    tangents(normal, r.t1, r.t2);
    r.a = a;
    r.b = b;
    r.n = -normal;
    r.ra = rotate(conj(ba.rot), pa - ba.pos);
    r.rb = rotate(conj(bb.rot), pb - bb.pos);
    r.c0 = {o.margin - depth, R(0), R(0)};
    r.penalty = {o.penalty_min, o.penalty_min, o.penalty_min};
    r.lambda = {P(0), P(0), P(0)};
    r.friction = o.friction;
    return r;
}

template <class R>
struct Container {  // AvbdContainer, engine/src/physics/gpu.rs:118-123
    V3<R> center{};
    Qt<R> rotation{R(0), R(0), R(0), R(1)};
    R half_extent = 0;
};

// cube_support_face, engine/src/physics/gpu.rs:314-350 (per-axis for BOX)
template <class R>
inline void cube_support_face(const NBody<R>& body, V3<R> outward, V3<R> pts[4]) {
    V3<R> ax[3];
    axes_of(body, ax);
    uint32_t ai = 0;
    R best = std::fabs(dot(ax[0], outward));
    for (uint32_t i = 1; i < 3; ++i) {
        R al = std::fabs(dot(ax[i], outward));
        if (al > best) {
            ai = i;
            best = al;
        }
    }
    bool per_axis = body.shape.tag == BOX;
    V3<R> fa = ax[ai];
    V3<R> fn = fa * (dot(fa, outward) >= R(0) ? R(1) : R(-1));
    R hn = half_along(body, ai, per_axis);
    V3<R> center = body.pos + fn * hn;
    uint32_t ui = ai == 0 ? 1 : 0, vi = ai == 2 ? 1 : 2;
    V3<R> u = ax[ui], v = ax[vi];
    R eu = half_along(body, ui, per_axis), ev = half_along(body, vi, per_axis);
    pts[0] = center + u * eu + v * ev;
    pts[1] = center - u * eu + v * ev;
    pts[2] = center - u * eu - v * ev;
    pts[3] = center + u * eu - v * ev;
}

// container_contacts, engine/src/physics/gpu.rs:352-404
template <class P, class R>
inline void container_contacts(const Container<R>& c, const NBody<R>& body, V3<R> vel, uint32_t index,
                               const V3<R>* hull, const Options<R>& o, std::vector<Row<P, R>>& out) {
    const V3<R> axes[6] = {{R(1), R(0), R(0)}, {R(1), R(0), R(0)}, {R(0), R(1), R(0)},
                           {R(0), R(1), R(0)}, {R(0), R(0), R(1)}, {R(0), R(0), R(1)}};
    const R signs[6] = {R(1), R(-1), R(1), R(-1), R(1), R(-1)};
    for (int k = 0; k < 6; ++k) {
        V3<R> outward = rotate(c.rotation, axes[k] * signs[k]);
        R plane = dot(c.center, outward) + c.half_extent;
        V3<R> pts[4];
        uint32_t np;
        if (body.shape.tag == CUBE || body.shape.tag == BOX) {
            cube_support_face(body, outward, pts);
            np = 4;
        } else {
            V3<R> local = rotate(conj(body.rot), outward);
            pts[0] = rotate(body.rot, support(body.shape, local, hull)) + body.pos;
            np = 1;
        }
        V3<R> normal = -outward;
        V3<R> t1, t2;
        tangents(normal, t1, t2);
        for (uint32_t p = 0; p < np; ++p) {
            V3<R> cp = pts[p];
            R cur = dot(cp, outward) - plane;
            V3<R> pred = cp + vel * o.dt;
            R pd = dot(pred, outward) - plane;
            R depth = std::fmax(cur, pd);
            if (depth > R(0)) {
                Row<P, R> r;
                r.a = index;
                r.b = CONTAINER;
                r.n = normal;
                r.t1 = t1;
                r.t2 = t2;
                r.ra = rotate(conj(body.rot), cp - body.pos);
                r.rb = {R(0), R(0), R(0)};
                r.c0 = {o.margin - depth, R(0), R(0)};
                r.penalty = {o.penalty_min, o.penalty_min, o.penalty_min};
                r.lambda = {P(0), P(0), P(0)};
                r.friction = o.friction;
                out.push_back(r);
            }
        }
    }
}

// finalize_contacts, engine/src/physics/gpu.rs:266-311: warm start from the
// previous rows by (a, b) key (HashMap insert keeps the LAST previous row per
// key; remove hands it to the FIRST new row with that key only), decay, and
// the per-body CSR (a, then b unless CONTAINER, in row order).
template <class P, class R>
inline void finalize_contacts(const std::vector<Row<P, R>>& prev, std::vector<Row<P, R>>& rows,
                              uint32_t n, const Options<R>& o, std::vector<uint32_t>& offsets,
                              std::vector<uint32_t>& indices) {
    std::map<std::pair<uint32_t, uint32_t>, size_t> warm;
    for (size_t i = 0; i < prev.size(); ++i) warm[{prev[i].a, prev[i].b}] = i;
    R ag = o.alpha * o.gamma;
    for (auto& r : rows) {
        auto it = warm.find({r.a, r.b});
        if (it != warm.end()) {
            r.lambda = prev[it->second].lambda;
            r.penalty = prev[it->second].penalty;
            warm.erase(it);
        }
        r.lambda = r.lambda * P(ag);
        V3<R> k = r.penalty * o.gamma;
        auto cl = [&](R x) { return std::fmin(std::fmax(x, o.penalty_min), o.penalty_max); };
        r.penalty = {cl(k.x), cl(k.y), cl(k.z)};
    }
    offsets.assign(n + 1, 0);
    for (auto& r : rows) {
        offsets[r.a + 1] += 1;
        if (r.b != CONTAINER) offsets[r.b + 1] += 1;
    }
    for (uint32_t i = 0; i < n; ++i) offsets[i + 1] += offsets[i];
    indices.assign(offsets[n], 0);
    std::vector<uint32_t> cursor(offsets.begin(), offsets.end());
    for (size_t i = 0; i < rows.size(); ++i) {
        indices[cursor[rows[i].a]++] = uint32_t(i);
        if (rows[i].b != CONTAINER) indices[cursor[rows[i].b]++] = uint32_t(i);
    }
}

// ------------------------------------------------------------------- AVBD
template <class P, class R>
struct BodyState {  // GpuAvbdBodyState, render/gpu_physics.rs:18-26
    V3<P> vel{}, ang{}, prev_vel{};
    V3<R> inv_moment{};
    R inv_mass = 0, friction = 0;
};

template <class R>
struct Joint {  // GpuAvbdConstraint, avbd/src/lib.rs:50-59
    uint32_t a = 0, b = 0, kind = 0;
    V3<R> anchor_a{}, anchor_b{};
    R aw = 0;  // rest / max length
    R bw = 0;  // stiffness
};

template <class R>
struct RunOptions {  // AvbdRunOptions, render/gpu_physics.rs:76-83
    R dt = R(1) / R(60);
    V3<R> gravity{R(0), R(-10), R(0)};
    R alpha = R(0.99), beta_lin = R(10000), penalty_max = R(1e10);
    uint32_t iterations = 10;
};

// solve6, engine/gpu_physics/avbd/src/lib.rs:107-180: unpivoted LDL^T of the
// symmetric 6x6 block given by its lower triangle H[i][j], i >= j.
template <class R>
inline void solve6(const R H[6][6], const R b[6], R x[6]) {
    R a11 = H[0][0], a21 = H[1][0], a31 = H[2][0], a22 = H[1][1], a32 = H[2][1], a33 = H[2][2];
    R a41 = H[3][0], a51 = H[4][0], a61 = H[5][0], a42 = H[3][1], a52 = H[4][1], a62 = H[5][1];
    R a43 = H[3][2], a53 = H[4][2], a63 = H[5][2];
    R a44 = H[3][3], a54 = H[4][3], a64 = H[5][3], a55 = H[4][4], a65 = H[5][4], a66 = H[5][5];
    R l21 = a21 / a11, l31 = a31 / a11, l41 = a41 / a11, l51 = a51 / a11, l61 = a61 / a11;
    R d1 = a11;
    R d2 = a22 - l21 * l21 * d1;
    R l32 = (a32 - l21 * l31 * d1) / d2;
    R l42 = (a42 - l21 * l41 * d1) / d2;
    R l52 = (a52 - l21 * l51 * d1) / d2;
    R l62 = (a62 - l21 * l61 * d1) / d2;
    R d3 = a33 - (l31 * l31 * d1 + l32 * l32 * d2);
    R l43 = (a43 - l31 * l41 * d1 - l32 * l42 * d2) / d3;
    R l53 = (a53 - l31 * l51 * d1 - l32 * l52 * d2) / d3;
    R l63 = (a63 - l31 * l61 * d1 - l32 * l62 * d2) / d3;
    R d4 = a44 - (l41 * l41 * d1 + l42 * l42 * d2 + l43 * l43 * d3);
    R l54 = (a54 - l41 * l51 * d1 - l42 * l52 * d2 - l43 * l53 * d3) / d4;
    R l64 = (a64 - l41 * l61 * d1 - l42 * l62 * d2 - l43 * l63 * d3) / d4;
    R d5 = a55 - (l51 * l51 * d1 + l52 * l52 * d2 + l53 * l53 * d3 + l54 * l54 * d4);
    R l65 = (a65 - l51 * l61 * d1 - l52 * l62 * d2 - l53 * l63 * d3 - l54 * l64 * d4) / d5;
    R d6 = a66 - (l61 * l61 * d1 + l62 * l62 * d2 + l63 * l63 * d3 + l64 * l64 * d4 + l65 * l65 * d5);
    R y1 = b[0];
    R y2 = b[1] - l21 * y1;
    R y3 = b[2] - l31 * y1 - l32 * y2;
    R y4 = b[3] - l41 * y1 - l42 * y2 - l43 * y3;
    R y5 = b[4] - l51 * y1 - l52 * y2 - l53 * y3 - l54 * y4;
    R y6 = b[5] - l61 * y1 - l62 * y2 - l63 * y3 - l64 * y4 - l65 * y5;
    R z1 = y1 / d1, z2 = y2 / d2, z3 = y3 / d3, z4 = y4 / d4, z5 = y5 / d5, z6 = y6 / d6;
    x[5] = z6;
    x[4] = z5 - l65 * x[5];
    x[3] = z4 - l54 * x[4] - l64 * x[5];
    x[2] = z3 - l43 * x[3] - l53 * x[4] - l63 * x[5];
    x[1] = z2 - l32 * x[2] - l42 * x[3] - l52 * x[4] - l62 * x[5];
    x[0] = z1 - l21 * x[1] - l31 * x[2] - l41 * x[3] - l51 * x[4] - l61 * x[5];
}

// One row (J_lin, J_ang) with stiffness k and force f stamped into the
// block: H += J J^T k (lower triangle), g += J f.  add_constraint_row,
// avbd/src/lib.rs:182-198, and the contact stamping at :400-416.
template <class R>
inline void stamp(R H[6][6], R g[6], V3<R> jl, V3<R> ja, R k, R f) {
    const R J[6] = {jl.x, jl.y, jl.z, ja.x, ja.y, ja.z};
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j <= i; ++j) H[i][j] = H[i][j] + J[i] * J[j] * k;
    for (int i = 0; i < 6; ++i) g[i] = g[i] + J[i] * f;
}

// Device-buffer image of one AVBD solve (AvbdCompute's buffers).
template <class P, class R>
struct AvbdBuffers {
    uint32_t n = 0;
    std::vector<BodyState<P, R>> state;
    std::vector<V3<P>> pos[2];
    std::vector<Qt<P>> rot[2];
    std::vector<V3<P>> init_lin, inert_lin;
    std::vector<Qt<P>> init_ang, inert_ang;
};

template <class P, class R>
struct Avbd {
    // avbd_init, avbd/src/lib.rs:202-254
    static void init(AvbdBuffers<P, R>& B, uint32_t i, const RunOptions<R>& o) {
        const auto& st = B.state[i];
        V3<P> pos = B.pos[0][i];
        Qt<P> rot = B.rot[0][i];
        P dt = P(o.dt);
        V3<P> g = cast3<P>(o.gravity);
        B.init_lin[i] = pos;
        B.init_ang[i] = rot;
        V3<P> ip = pos + st.vel * dt;
        if (st.inv_mass > R(0)) ip = ip + g * (dt * dt);
        B.inert_lin[i] = ip;
        B.inert_ang[i] = quat_step(rot, st.ang * dt);
        if (st.inv_mass > R(0)) {
            // adaptive gravity weight, clamped to [0, 1]: formed in R in the
            // split mode (it only scales the warm-start offset)
            using F = std::conditional_t<std::is_same<P, R>::value, P, R>;
            const F dtf = F(o.dt);
            const V3<F> gf = cast3<F>(o.gravity);
            V3<F> accel = divs(cast3<F>(st.vel - st.prev_vel), dtf);
            F gm = length(gf);
            F w = F(0);
            if (gm > F(0)) {
                w = dot(accel, divs(gf, gm)) / gm;
                w = w < F(0) ? F(0) : (w > F(1) ? F(1) : w);
            }
            B.pos[0][i] = pos + st.vel * dt + g * (P(w) * dt * dt);
            B.rot[0][i] = B.inert_ang[i];  // the same quat_step(rot, ang dt)
        } else {
            B.pos[0][i] = pos;
            B.rot[0][i] = rot;
        }
    }

    // avbd_primal, avbd/src/lib.rs:258-551.  `rd`/`wr` select the snapshot
    // and output buffers (Jacobi: rd = parity, wr = 1 - parity; coloured
    // Gauss-Seidel: rd = wr = 0).  `jidx` is an optional per-body joint CSR
    // (joint order preserved); without it all joints are scanned.
    static void primal(AvbdBuffers<P, R>& B, uint32_t i, int rd, int wr, const std::vector<Row<P, R>>& rows,
                       const std::vector<uint32_t>& off, const std::vector<uint32_t>& idx,
                       const std::vector<Joint<R>>& joints, const std::vector<uint32_t>* joff,
                       const std::vector<uint32_t>* jidx, const RunOptions<R>& o) {
        const auto& st = B.state[i];
        if (st.inv_mass == R(0)) return;
        V3<P> sp = B.pos[rd][i];
        Qt<P> sq = B.rot[rd][i];
        Qt<R> sqr = castq<R>(sq);
        R dt = o.dt;
        R mass = R(1) / st.inv_mass;
        V3<R> moment{R(1) / st.inv_moment.x, R(1) / st.inv_moment.y, R(1) / st.inv_moment.z};
        R dt2 = dt * dt;
        V3<R> m_dt2{mass / dt2, mass / dt2, mass / dt2};
        V3<R> i_dt2 = divs(moment, dt2);
        R H[6][6] = {};
        R g[6] = {};
        H[0][0] = m_dt2.x;
        H[1][1] = m_dt2.y;
        H[2][2] = m_dt2.z;
        H[3][3] = i_dt2.x;
        H[4][4] = i_dt2.y;
        H[5][5] = i_dt2.z;
        V3<R> rl = mulv(m_dt2, cast3<R>(sp - B.inert_lin[i]));
        V3<R> ra = mulv(i_dt2, ang_diff(castq<R>(sq), castq<R>(B.inert_ang[i])));
        g[0] = rl.x;
        g[1] = rl.y;
        g[2] = rl.z;
        g[3] = ra.x;
        g[4] = ra.y;
        g[5] = ra.z;
        V3<R> dq_self_lin = cast3<R>(sp - B.init_lin[i]);
        V3<R> dq_self_ang = ang_diff(castq<R>(sq), castq<R>(B.init_ang[i]));
        R k_alpha = R(1) - o.alpha;
        for (uint32_t j = off[i]; j < off[i + 1]; ++j) {
            const Row<P, R>& c = rows[idx[j]];
            bool is_a = c.a == i;
            uint32_t other = is_a ? c.b : c.a;
            V3<R> r0 = is_a ? c.n : -c.n;
            V3<R> r1 = is_a ? c.t1 : -c.t1;
            V3<R> r2 = is_a ? c.t2 : -c.t2;
            V3<R> rw = rotate(sqr, is_a ? c.ra : c.rb);
            V3<R> dol{}, doa{}, rot_other{};
            if (other != CONTAINER) {
                V3<P> op = B.pos[rd][other];
                Qt<P> oq = B.rot[rd][other];
                dol = cast3<R>(op - B.init_lin[other]);
                doa = ang_diff(castq<R>(oq), castq<R>(B.init_ang[other]));
                rot_other = rotate(castq<R>(oq), is_a ? c.rb : c.ra);
            }
            V3<R> j0 = cross(rw, r0), j1 = cross(rw, r1), j2 = cross(rw, r2);
            R c0 = c.c0.x * k_alpha, c1 = c.c0.y * k_alpha, c2 = c.c0.z * k_alpha;
            c0 = c0 + (dot(r0, dq_self_lin) + dot(j0, dq_self_ang) - dot(r0, dol) - dot(cross(rot_other, r0), doa));
            c1 = c1 + (dot(r1, dq_self_lin) + dot(j1, dq_self_ang) - dot(r1, dol) - dot(cross(rot_other, r1), doa));
            c2 = c2 + (dot(r2, dq_self_lin) + dot(j2, dq_self_ang) - dot(r2, dol) - dot(cross(rot_other, r2), doa));
            // the forces only feed the R Hessian: in the split mode they are
            // formed in R from the P lambda (the dual accumulates lambda in P)
            using F = std::conditional_t<std::is_same<P, R>::value, P, R>;
            F f0p = F(c.penalty.x * c0) + F(c.lambda.x);
            f0p = std::fmin(f0p, F(0));  // f32::min: NaN-ignoring
            F f1r = F(c.penalty.y * c1) + F(c.lambda.y);
            F f2r = F(c.penalty.z * c2) + F(c.lambda.z);
            F bounds = std::fabs(f0p) * F(c.friction);
            F tm = std::sqrt(f1r * f1r + f2r * f2r);
            F f1 = f1r, f2 = f2r;
            if (tm > bounds && tm > F(0)) {
                F s = bounds / tm;
                f1 = f1r * s;
                f2 = f2r * s;
            }
            stamp(H, g, r0, j0, c.penalty.x, R(f0p));
            stamp(H, g, r1, j1, c.penalty.y, R(f1));
            stamp(H, g, r2, j2, c.penalty.z, R(f2));
        }
        auto joint_row = [&](const Joint<R>& jt) {
            bool is_a = jt.a == i;
            V3<P> pa = is_a ? sp : B.pos[rd][jt.a];
            V3<P> pb = !is_a ? sp : B.pos[rd][jt.b];
            Qt<P> qa = is_a ? sq : B.rot[rd][jt.a];
            Qt<P> qb = !is_a ? sq : B.rot[rd][jt.b];
            V3<R> self_anchor = is_a ? jt.anchor_a : jt.anchor_b;
            R sign = is_a ? R(1) : R(-1);
            V3<R> delta;
            if constexpr (std::is_same<P, R>::value) {
                V3<P> wpa = pa + rotate(qa, jt.anchor_a);
                V3<P> wpb = pb + rotate(qb, jt.anchor_b);
                delta = wpa - wpb;
            } else {
                // split mode: the position difference in P, the anchor
                // offsets (small body-frame vectors) rotated and differenced in R
                delta = cast3<R>(pa - pb) +
                        (rotate(castq<R>(qa), jt.anchor_a) - rotate(castq<R>(qb), jt.anchor_b));
            }
            V3<R> r_self = rotate(sqr, self_anchor);
            R stiff = jt.bw;
            if (jt.kind == BALL_SOCKET) {
                V3<R> jx = V3<R>{R(1), R(0), R(0)} * sign;
                V3<R> jy = V3<R>{R(0), R(1), R(0)} * sign;
                V3<R> jz = V3<R>{R(0), R(0), R(1)} * sign;
                stamp(H, g, jx, cross(r_self, jx), stiff, delta.x * stiff);
                stamp(H, g, jy, cross(r_self, jy), stiff, delta.y * stiff);
                stamp(H, g, jz, cross(r_self, jz), stiff, delta.z * stiff);
            } else {
                R len = length(delta);
                bool active = len > R(1.0e-6) && (jt.kind != ROPE || len > jt.aw);
                if (active) {
                    V3<R> nn = divs(delta, len);
                    V3<R> jl = nn * sign;
                    V3<R> ja = cross(r_self, jl);
                    R force = stiff * (len - jt.aw);
                    stamp(H, g, jl, ja, stiff, force);
                }
            }
        };
        if (jidx) {
            for (uint32_t k = (*joff)[i]; k < (*joff)[i + 1]; ++k) joint_row(joints[(*jidx)[k]]);
        } else {
            for (const auto& jt : joints)
                if (jt.a == i || jt.b == i) joint_row(jt);
        }
        R rhs[6] = {-g[0], -g[1], -g[2], -g[3], -g[4], -g[5]};
        R dx[6];
        solve6(H, rhs, dx);
        B.pos[wr][i] = sp + cast3<P>(V3<R>{dx[0], dx[1], dx[2]});
        if constexpr (std::is_same<P, R>::value)
            B.rot[wr][i] = quat_step(sq, V3<P>{dx[3], dx[4], dx[5]});
        else
            B.rot[wr][i] = quat_step_split<P, R>(sq, V3<R>{dx[3], dx[4], dx[5]});
    }

    // avbd_dual, avbd/src/lib.rs:565-663; `rd` is the buffer holding the new
    // state (Jacobi: 1 - parity).
    static void dual(AvbdBuffers<P, R>& B, Row<P, R>& c, int rd, const RunOptions<R>& o) {
        V3<P> pa = B.pos[rd][c.a];
        Qt<P> qa = B.rot[rd][c.a];
        V3<R> dal = cast3<R>(pa - B.init_lin[c.a]);
        V3<R> daa = ang_diff(castq<R>(qa), castq<R>(B.init_ang[c.a]));
        V3<R> dbl{}, dba{}, rbw{};
        if (c.b != CONTAINER) {
            V3<P> pb = B.pos[rd][c.b];
            Qt<P> qb = B.rot[rd][c.b];
            dbl = cast3<R>(pb - B.init_lin[c.b]);
            dba = ang_diff(castq<R>(qb), castq<R>(B.init_ang[c.b]));
            rbw = rotate(castq<R>(qb), c.rb);
        }
        V3<R> raw = rotate(castq<R>(qa), c.ra);
        V3<R> r0 = c.n, r1 = c.t1, r2 = c.t2;
        R k_alpha = R(1) - o.alpha;
        R c0 = c.c0.x * k_alpha, c1 = c.c0.y * k_alpha, c2 = c.c0.z * k_alpha;
        c0 = c0 + (dot(r0, dal) + dot(cross(raw, r0), daa) - dot(r0, dbl) - dot(cross(rbw, r0), dba));
        c1 = c1 + (dot(r1, dal) + dot(cross(raw, r1), daa) - dot(r1, dbl) - dot(cross(rbw, r1), dba));
        c2 = c2 + (dot(r2, dal) + dot(cross(raw, r2), daa) - dot(r2, dbl) - dot(cross(rbw, r2), dba));
        P f0 = std::fmin(P(c.penalty.x * c0) + c.lambda.x, P(0));
        P f1r = P(c.penalty.y * c1) + c.lambda.y;
        P f2r = P(c.penalty.z * c2) + c.lambda.z;
        P bounds = std::fabs(f0) * P(c.friction);
        P tm, f1 = f1r, f2 = f2r;
        if constexpr (std::is_same<P, R>::value) {
            tm = std::sqrt(f1r * f1r + f2r * f2r);
            if (tm > bounds && tm > P(0)) {
                P s = bounds / tm;
                f1 = f1r * s;
                f2 = f2r * s;
            }
        } else {
            // split mode: the cone magnitude and its scale factor in R, applied
            // to the P forces (lambda still accumulates in P)
            const R f1q = R(f1r), f2q = R(f2r);
            const R tmr = std::sqrt(f1q * f1q + f2q * f2q);
            tm = P(tmr);
            if (tm > bounds && tm > P(0)) {
                const R sr = R(bounds) / tmr;
                f1 = f1r * P(sr);
                f2 = f2r * P(sr);
            }
        }
        c.lambda = {f0, f1, f2};
        if (f0 < P(0)) c.penalty.x = std::fmin(c.penalty.x + o.beta_lin * std::fabs(c0), o.penalty_max);
        if (tm <= bounds) {
            c.penalty.y = std::fmin(c.penalty.y + o.beta_lin * std::fabs(c1), o.penalty_max);
            c.penalty.z = std::fmin(c.penalty.z + o.beta_lin * std::fabs(c2), o.penalty_max);
        }
    }

    // avbd_recover, avbd/src/lib.rs:667-699
    static void recover(AvbdBuffers<P, R>& B, uint32_t i, int rd, const RunOptions<R>& o) {
        auto& st = B.state[i];
        if (st.inv_mass == R(0)) return;
        V3<P> pos = B.pos[rd][i];
        Qt<P> rot = B.rot[rd][i];
        P dt = P(o.dt);
        st.prev_vel = st.vel;
        Qt<P> rel = qmul(rot, conj(B.init_ang[i]));
        if constexpr (std::is_same<P, R>::value) {
            st.vel = divs(pos - B.init_lin[i], dt);
            st.ang = divs(V3<P>{P(2) * rel.x, P(2) * rel.y, P(2) * rel.z}, dt);
        } else {  // split mode: one division, then products (within an ulp of P)
            const P inv_dt = P(1) / dt;
            st.vel = (pos - B.init_lin[i]) * inv_dt;
            st.ang = V3<P>{P(2) * rel.x, P(2) * rel.y, P(2) * rel.z} * inv_dt;
        }
    }
};

// Jones-Plassmann colouring of the dynamic-body graph (edges: contact rows
// between two dynamic bodies, joints between two dynamic bodies).  Priority
// is a hash of the body index; ties break by index.  Each round, every
// uncoloured vertex whose (priority, index) beats all uncoloured neighbours
// takes the smallest colour unused by its coloured neighbours.  Static
// bodies get colour 0xFFFFFFFF.  No reference counterpart (the reference
// primal is Jacobi, avbd/src/lib.rs:6-9).
inline uint32_t color_hash(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

template <class P, class R>
inline uint32_t color_bodies(uint32_t n, const std::vector<BodyState<P, R>>& st, const std::vector<Row<P, R>>& rows,
                             const std::vector<Joint<R>>& joints, std::vector<uint32_t>& color) {
    std::vector<std::vector<uint32_t>> adj(n);
    auto dyn = [&](uint32_t i) { return i < n && st[i].inv_mass != R(0); };
    for (auto& r : rows)
        if (r.b != CONTAINER && r.a != r.b && dyn(r.a) && dyn(r.b)) {
            adj[r.a].push_back(r.b);
            adj[r.b].push_back(r.a);
        }
    for (auto& j : joints)
        if (j.a != j.b && dyn(j.a) && dyn(j.b)) {
            adj[j.a].push_back(j.b);
            adj[j.b].push_back(j.a);
        }
    const uint32_t NONE = 0xFFFFFFFFu;
    color.assign(n, NONE);
    auto beats = [&](uint32_t v, uint32_t u) {
        uint32_t pv = color_hash(v), pu = color_hash(u);
        return pv > pu || (pv == pu && v > u);
    };
    uint32_t remaining = 0, ncolors = 0;
    for (uint32_t i = 0; i < n; ++i) remaining += dyn(i) ? 1 : 0;
    std::vector<uint32_t> sel;
    while (remaining) {
        sel.clear();
        for (uint32_t v = 0; v < n; ++v) {
            if (!dyn(v) || color[v] != NONE) continue;
            bool best = true;
            for (uint32_t u : adj[v])
                if (color[u] == NONE && u != v && !beats(v, u)) {
                    best = false;
                    break;
                }
            if (best) sel.push_back(v);
        }
        for (uint32_t v : sel) {
            std::vector<bool> used;
            for (uint32_t u : adj[v])
                if (color[u] != NONE) {
                    if (used.size() <= color[u]) used.resize(color[u] + 1, false);
                    used[color[u]] = true;
                }
            uint32_t c = 0;
            while (c < used.size() && used[c]) ++c;
            color[v] = c;
            ncolors = std::max(ncolors, c + 1);
        }
        remaining -= uint32_t(sel.size());
    }
    return ncolors;
}

// AvbdCompute::submit + read, render/gpu_physics.rs:439-622: the schedule is
// init; k = 0..I-1: primal(parity k%2), dual(k%2); recover(final parity);
// both parities are seeded with the un-warm-started pose (:479-482).
// `colors`/`ncolors` switch to the coloured Gauss-Seidel schedule.
template <class P, class R>
struct AvbdResult {
    std::vector<V3<P>> pos;
    std::vector<Qt<P>> rot;
};

template <class P, class R>
inline void avbd_run(AvbdBuffers<P, R>& B, std::vector<Row<P, R>>& rows, const std::vector<uint32_t>& off,
                     const std::vector<uint32_t>& idx, const std::vector<Joint<R>>& joints,
                     const std::vector<uint32_t>* joff, const std::vector<uint32_t>* jidx,
                     const RunOptions<R>& o, const std::vector<uint32_t>* colors, uint32_t ncolors,
                     AvbdResult<P, R>& out, int threads = 1) {
    uint32_t n = B.n;
    if (n == 0) {
        out.pos.clear();
        out.rot.clear();
        return;
    }
    B.pos[1] = B.pos[0];
    B.rot[1] = B.rot[0];
    B.init_lin.resize(n);
    B.init_ang.resize(n);
    B.inert_lin.resize(n);
    B.inert_ang.resize(n);
    (void)threads;
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
    for (int64_t i = 0; i < int64_t(n); ++i) Avbd<P, R>::init(B, uint32_t(i), o);
    uint32_t iters = o.iterations;
    int final_buf;
    if (!colors) {
        for (uint32_t k = 0; k < iters; ++k) {
            int par = int(k % 2);
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads) if (threads > 1)
            for (int64_t i = 0; i < int64_t(n); ++i)
                Avbd<P, R>::primal(B, uint32_t(i), par, 1 - par, rows, off, idx, joints, joff, jidx, o);
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
            for (int64_t c = 0; c < int64_t(rows.size()); ++c) Avbd<P, R>::dual(B, rows[c], 1 - par, o);
        }
        uint32_t fp = (iters - 1u) % 2u;  // u32 wrap when iterations == 0
        int rb = fp == 0 ? 1 : 0;
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
        for (int64_t i = 0; i < int64_t(n); ++i) Avbd<P, R>::recover(B, uint32_t(i), rb, o);
        uint32_t fp_read = (iters == 0 ? 0u : iters - 1u) % 2u;
        final_buf = 1 - int(fp_read);
    } else {
        std::vector<std::vector<uint32_t>> by_color(ncolors);
        for (uint32_t i = 0; i < n; ++i)
            if ((*colors)[i] < ncolors) by_color[(*colors)[i]].push_back(i);
        for (uint32_t k = 0; k < iters; ++k) {
            for (uint32_t c = 0; c < ncolors; ++c) {
                const auto& list = by_color[c];
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads) if (threads > 1)
                for (int64_t t = 0; t < int64_t(list.size()); ++t)
                    Avbd<P, R>::primal(B, list[t], 0, 0, rows, off, idx, joints, joff, jidx, o);
            }
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
            for (int64_t c = 0; c < int64_t(rows.size()); ++c) Avbd<P, R>::dual(B, rows[c], 0, o);
        }
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
        for (int64_t i = 0; i < int64_t(n); ++i) Avbd<P, R>::recover(B, uint32_t(i), 0, o);
        final_buf = 0;
    }
    out.pos = B.pos[final_buf];
    out.rot = B.rot[final_buf];
}

// ------------------------------------------------------------- world step
// The per-frame sequence of demos/avbd_box/src/main.rs:189-273 defined
// without the one-frame contact lag: detect on S_t, build rows, warm start,
// solve, sync into S_{t+1}.  Scenes are independent body ranges; a packed
// multi-scene world is the union of its scenes (pair rows of every scene in
// scene order, then container rows of every dynamic body in index order).
template <class P, class R>
struct World {
    std::vector<V3<P>> pos;
    std::vector<Qt<P>> rot;
    std::vector<Shape<R>> shape;
    std::vector<BodyState<P, R>> state;
    std::vector<Joint<R>> joints;
    std::vector<uint32_t> scene_off;  // n_scenes + 1
    std::vector<Container<R>> containers;
    std::vector<uint8_t> has_container;
    std::vector<V3<R>> hull;
    std::vector<Row<P, R>> rows;  // last step's rows (warm start source)
    std::vector<uint32_t> colors;
    uint32_t ncolors = 0;
    uint32_t per_pair = 4;
    bool colored = false;
    // the demos' frame pipelining (demos/avbd_box/src/main.rs:203-207,244-249):
    // the narrow phase read at frame t was submitted at frame t-1, and
    // raw_contact (engine/src/physics/gpu.rs:239-264) applies its witness
    // points to the current transforms
    bool lag = false;
    std::vector<Slot<R>> prev_slots;
    bool split_rebase = false;  // detect in scene-local R coordinates
    bool use_sap = true;
    int threads = 1;
    uint64_t last_pairs = 0;
    bool epa_overflow = false;

    uint32_t n() const { return uint32_t(pos.size()); }

    V3<P> origin(uint32_t s) const {
        if (!split_rebase || !has_container[s]) return {P(0), P(0), P(0)};
        return cast3<P>(containers[s].center);
    }

    void step(const Options<R>& o) {
        uint32_t N = n();
        uint32_t S = uint32_t(scene_off.size()) - 1;
        std::vector<NBody<R>> nb(N);
        std::vector<uint32_t> scene_of(N);
        for (uint32_t s = 0; s < S; ++s) {
            V3<P> org = origin(s);
            for (uint32_t i = scene_off[s]; i < scene_off[s + 1]; ++i) {
                nb[i].pos = cast3<R>(pos[i] - org);
                nb[i].rot = castq<R>(rot[i]);
                nb[i].shape = shape[i];
                scene_of[i] = s;
            }
        }
        const V3<R>* hp = hull.empty() ? nullptr : hull.data();
        std::vector<V3<R>> mn(N), mx(N);
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
        for (int64_t i = 0; i < int64_t(N); ++i) aabb(nb[i], hp, mn[i], mx[i]);
        std::vector<std::pair<uint32_t, uint32_t>> pairs;
        for (uint32_t s = 0; s < S; ++s) {
            if (use_sap)
                broad_sap(mn, mx, scene_off[s], scene_off[s + 1], pairs);
            else
                broad_dense(mn, mx, scene_off[s], scene_off[s + 1], pairs);
        }
        last_pairs = pairs.size();
        std::vector<Slot<R>> slots(pairs.size() * per_pair);
        bool ovf = false;
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads) if (threads > 1) reduction(|| : ovf)
        for (int64_t p = 0; p < int64_t(pairs.size()); ++p) {
            bool o2 = false;
            narrow_pair(nb[pairs[p].first], nb[pairs[p].second], pairs[p].first, pairs[p].second, hp, per_pair,
                        &slots[p * per_pair], &o2);
            ovf = ovf || o2;
        }
        epa_overflow = ovf;
        std::vector<Row<P, R>> nrows;
        if (lag) prev_slots.swap(slots);  // rows from the previous step's detection
        for (auto& sl : slots)
            if (sl.valid)
                nrows.push_back(raw_contact<P, R>(sl.a, sl.b, nb[sl.a], nb[sl.b], sl.normal, sl.depth, sl.point_a,
                                                  sl.point_b, o));
        for (uint32_t i = 0; i < N; ++i) {
            uint32_t s = scene_of[i];
            if (state[i].inv_mass == R(0) || !has_container[s]) continue;
            Container<R> c = containers[s];
            c.center = cast3<R>(cast3<P>(c.center) - origin(s));
            container_contacts<P, R>(c, nb[i], cast3<R>(state[i].vel), i, hp, o, nrows);
        }
        std::vector<uint32_t> off, idx;
        finalize_contacts(rows, nrows, N, o, off, idx);
        rows.swap(nrows);
        // per-body joint CSR (joint order preserved)
        std::vector<uint32_t> joff(N + 1, 0), jidx;
        for (auto& j : joints) {
            joff[j.a + 1] += 1;
            if (j.b != j.a) joff[j.b + 1] += 1;
        }
        for (uint32_t i = 0; i < N; ++i) joff[i + 1] += joff[i];
        jidx.assign(joff[N], 0);
        {
            std::vector<uint32_t> cur(joff.begin(), joff.end());
            for (uint32_t k = 0; k < joints.size(); ++k) {
                jidx[cur[joints[k].a]++] = k;
                if (joints[k].b != joints[k].a) jidx[cur[joints[k].b]++] = k;
            }
        }
        RunOptions<R> ro;
        ro.dt = o.dt;
        ro.gravity = o.gravity;
        ro.alpha = o.alpha;
        ro.beta_lin = o.beta_lin;
        ro.penalty_max = o.penalty_max;
        ro.iterations = o.iterations;
        AvbdBuffers<P, R> B;
        B.n = N;
        B.state = state;
        B.pos[0] = pos;
        B.rot[0] = rot;
        if (colored) ncolors = color_bodies(N, state, rows, joints, colors);
        AvbdResult<P, R> res;
        avbd_run(B, rows, off, idx, joints, &joff, &jidx, ro, colored ? &colors : nullptr, ncolors, res,
                 threads);
        // sync_bodies_from_gpu, engine/src/physics/gpu.rs:212-237
        for (uint32_t i = 0; i < N; ++i) {
            if (state[i].inv_mass == R(0)) continue;
            pos[i] = res.pos[i];
            rot[i] = res.rot[i];
            state[i].vel = B.state[i].vel;
            state[i].ang = B.state[i].ang;
            state[i].prev_vel = B.state[i].prev_vel;
        }
    }
};

}  // namespace dio_oracle
