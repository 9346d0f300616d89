// dio_math.cuh -- vector / quaternion arithmetic for the sm_103a kernels.
//
// The reference kernels use glam 0.33.3 f32 types (Vec3, Quat, Mat3) inside
// rust-gpu shaders (engine/gpu_physics/*/src/*.rs).  These helpers restate the
// operations the reference calls -- Hamilton product, conjugate inverse of a
// unit quaternion, rotation q * v in glam's mul_vec3 form, normalisation as
// v * (1/|v|) -- with a fixed left-to-right evaluation order.  The library is compiled with
// --fmad=false, so every expression rounds exactly as written and pair sets,
// manifold counts and solver states are reproducible bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define DIO_HD __host__ __device__ __forceinline__

namespace dio {

template <class R>
struct V3 {
    R x, y, z;
};
template <class R>
struct Q4 {
    R x, y, z, w;
};

// 16-byte (float) / 32-byte (double) aligned 4-vectors for vector loads.
template <class R>
struct alignas(4 * sizeof(R)) A4 {
    R x, y, z, w;
};

template <class R>
DIO_HD V3<R> mk3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R>
DIO_HD V3<R> add(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R>
DIO_HD V3<R> sub(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R>
DIO_HD V3<R> neg(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R>
DIO_HD V3<R> scale(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R>
DIO_HD V3<R> mulv(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R>
DIO_HD V3<R> divs(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R>
DIO_HD R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R>
DIO_HD V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R>
DIO_HD R length_sq(V3<R> a) { return dot(a, a); }
DIO_HD float dsqrt(float x) { return sqrtf(x); }
DIO_HD double dsqrt(double x) { return sqrt(x); }
DIO_HD float dabs(float x) { return fabsf(x); }
DIO_HD double dabs(double x) { return fabs(x); }
template <class R>
DIO_HD R length(V3<R> a) { return dsqrt(dot(a, a)); }
template <class R>
DIO_HD V3<R> normalize(V3<R> a) { return scale(a, R(1) / length(a)); }
template <class R>
DIO_HD bool finite_(R x) { return isfinite(x); }
template <class R>
DIO_HD V3<R> normalize_or_zero(V3<R> a) {
    R rcp = R(1) / length(a);
    if (finite_(rcp) && rcp > R(0)) return scale(a, rcp);
    return {R(0), R(0), R(0)};
}
template <class T, class R>
DIO_HD V3<T> cast3(V3<R> a) { return {T(a.x), T(a.y), T(a.z)}; }
template <class T, class R>
DIO_HD Q4<T> castq(Q4<R> q) { return {T(q.x), T(q.y), T(q.z), T(q.w)}; }
template <class R>
DIO_HD V3<R> xyz(A4<R> a) { return {a.x, a.y, a.z}; }
template <class R>
DIO_HD Q4<R> quat(A4<R> a) { return {a.x, a.y, a.z, a.w}; }
template <class R>
DIO_HD A4<R> pack(V3<R> v, R w = R(0)) { return {v.x, v.y, v.z, w}; }
template <class R>
DIO_HD A4<R> packq(Q4<R> q) { return {q.x, q.y, q.z, q.w}; }

// Hamilton product a * b.
template <class R>
DIO_HD Q4<R> qmul(Q4<R> a, Q4<R> b) {
    return {a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
            a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
            a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w,
            a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
}
template <class R>
DIO_HD Q4<R> conj(Q4<R> q) { return {-q.x, -q.y, -q.z, q.w}; }
// q * v for unit q, in the form glam 0.33's Quat::mul_vec3 evaluates it
// (its scalar path, also what the rust-gpu shaders compile): with b = q.xyz,
//   v (w w - b.b) + b (2 (v.b)) + (b x v) (2 w),
// each product rounded, sums left to right.
template <class R>
DIO_HD V3<R> rotate(Q4<R> q, V3<R> v) {
    const V3<R> b{q.x, q.y, q.z};
    const R b2 = dot(b, b);
    const V3<R> r = add(scale(v, q.w * q.w - b2), scale(b, dot(v, b) * R(2)));
    return add(r, scale(cross(b, v), q.w * R(2)));
}
template <class R>
DIO_HD Q4<R> qnormalize(Q4<R> q) {
    R len = dsqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    R inv = R(1) / len;
    return {q.x * inv, q.y * inv, q.z * inv, q.w * inv};
}
// quat_step, engine/gpu_physics/avbd/src/lib.rs:91-94
template <class R>
DIO_HD Q4<R> quat_step(Q4<R> q, V3<R> d) {
    Q4<R> p{d.x, d.y, d.z, R(0)};
    Q4<R> s = qmul(p, q);
    s = {s.x * R(0.5), s.y * R(0.5), s.z * R(0.5), s.w * R(0.5)};
    return qnormalize(Q4<R>{q.x + s.x, q.y + s.y, q.z + s.z, q.w + s.w});
}
// quat_step of the split mode: the increment (d, 0) * q / 2 is formed in R
// from the rounded quaternion and added to the P quaternion; 1/|q| is seeded
// in R (correctly rounded sqrt and division) and refined by one Newton step
// in P (relative error ~1e-14; the quaternion is renormalised every step),
// or taken in P when |u|^2 lies outside [1e-30, 1e30].
template <class P, class R>
DIO_HD Q4<P> quat_step_split(Q4<P> q, V3<R> d) {
    Q4<R> s = qmul(Q4<R>{d.x, d.y, d.z, R(0)}, castq<R>(q));
    s = {s.x * R(0.5), s.y * R(0.5), s.z * R(0.5), s.w * R(0.5)};
    const Q4<P> u{q.x + P(s.x), q.y + P(s.y), q.z + P(s.z), q.w + P(s.w)};
    const P n = u.x * u.x + u.y * u.y + u.z * u.z + u.w * u.w;
    // an R seed only where n and its root stay well inside R's range; a
    // quaternion blown up by a huge increment (|u|^2 beyond R) is normalised
    // in P (an R seed would overflow to a zero quaternion, then NaN)
    P r;
    if (n > P(1.0e-30) && n < P(1.0e30)) {
        r = P(R(1) / dsqrt(R(n)));
        r = r * (P(1.5) - P(0.5) * n * r * r);
    } else {
        r = P(1) / dsqrt(n);
    }
    return {u.x * r, u.y * r, u.z * r, u.w * r};
}
// ang_diff, engine/gpu_physics/avbd/src/lib.rs:96-99
template <class R>
DIO_HD V3<R> ang_diff(Q4<R> to, Q4<R> from) {
    Q4<R> rel = qmul(to, conj(from));
    return {R(2) * rel.x, R(2) * rel.y, R(2) * rel.z};
}

template <class R>
DIO_HD R dmin(R a, R b) { return a < b ? a : b; }
template <class R>
DIO_HD R dmax(R a, R b) { return a > b ? a : b; }

// glam's f32::min / f32::max return the non-NaN operand; restate that.
DIO_HD float fmin_(float a, float b) { return fminf(a, b); }
DIO_HD double fmin_(double a, double b) { return fmin(a, b); }
DIO_HD float fmax_(float a, float b) { return fmaxf(a, b); }
DIO_HD double fmax_(double a, double b) { return fmax(a, b); }

}  // namespace dio
