// k_narrow.cuh -- narrow phase on sm_103a.
//
// Restates engine/gpu_physics/narrowphase/src/{lib,support,cuboid,gjk,epa}.rs.
// Work split (the reference runs one thread per pair for everything):
//   k_narrow_main  one thread per pair: clears the pair's slots, runs the box
//                  SAT manifold or the analytic sphere test in-thread, and
//                  queues every other pair for GJK.
//   k_gjk          one thread per queued pair: GJK with witness tracking;
//                  intersecting pairs queue their final simplex for EPA.
//   k_epa          one warp per queued pair: the expanding polytope lives in
//                  shared memory; face search, visibility, horizon extraction
//                  and face compaction are lane-parallel with ballot/scan,
//                  preserving the reference's sequential face order exactly.
#pragma once

#include "engine.cuh"

namespace dio {

template <class R>
struct ShapeR {
    uint32_t tag, hf, hc;
    V3<R> c[4];
};

template <class R>
__device__ __forceinline__ ShapeR<R> load_shape(const DioShape* s) {
    ShapeR<R> o;
    const uint4 h = *reinterpret_cast<const uint4*>(s);
    o.tag = h.x;
    o.hf = h.y;
    o.hc = h.z;
    const float4* c = reinterpret_cast<const float4*>(s->corners);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float4 v = c[i];
        o.c[i] = {R(v.x), R(v.y), R(v.z)};
    }
    return o;
}

template <class R>
struct NB {
    V3<R> pos;
    Q4<R> rot;
    ShapeR<R> shape;
};

// support, support.rs:21-61 (first max wins ties); BOX shares the cube's sign
// select, HULL scans its vertex list with the same first-max rule.
template <class R>
__device__ __forceinline__ V3<R> support(const ShapeR<R>& s, V3<R> d, const A4<R>* hull) {
    switch (s.tag) {
        case DIO_SHAPE_SPHERE:
            return scale(normalize_or_zero(d), s.c[0].x);
        case DIO_SHAPE_CUBE:
        case DIO_SHAPE_BOX:
            return {d.x >= R(0) ? s.c[0].x : -s.c[0].x, d.y >= R(0) ? s.c[0].y : -s.c[0].y,
                    d.z >= R(0) ? s.c[0].z : -s.c[0].z};
        case DIO_SHAPE_TETRAHEDRON: {
            V3<R> best = s.c[0];
            R bd = dot(best, d);
#pragma unroll
            for (int i = 1; i < 4; ++i) {
                R dd = dot(s.c[i], d);
                if (dd > bd) {
                    bd = dd;
                    best = s.c[i];
                }
            }
            return best;
        }
        case DIO_SHAPE_HULL: {
            if (s.hc == 0 || hull == nullptr) return {R(0), R(0), R(0)};
            V3<R> best = xyz(hull[s.hf]);
            R bd = dot(best, d);
            for (uint32_t i = 1; i < s.hc; ++i) {
                V3<R> v = xyz(hull[s.hf + i]);
                R dd = dot(v, d);
                if (dd > bd) {
                    bd = dd;
                    best = v;
                }
            }
            return best;
        }
        default:
            return {R(0), R(0), R(0)};
    }
}

// support() of a hull with the 32 lanes of a warp over its vertices (every
// lane calls it with the same arguments and gets the same vertex): each
// lane keeps its first maximum over vertices lane, lane + 32, ..., then the
// warp keeps the largest value, ties to the lower index -- the first
// maximum in vertex order, as the serial scan finds it (NaN products never
// win a strict comparison there, and a NaN first product keeps vertex 0).
template <class R>
__device__ __forceinline__ V3<R> support_warp(const ShapeR<R>& s, V3<R> d, const A4<R>* hull, uint32_t lane) {
    if (s.tag != DIO_SHAPE_HULL || s.hc == 0 || hull == nullptr) return support(s, d, hull);
    const V3<R> v0 = xyz(hull[s.hf]);
    if (isnan(dot(v0, d))) return v0;
    R bv = R(0);
    uint32_t bi = 0xFFFFFFFFu;
    for (uint32_t i = lane; i < s.hc; i += 32) {
        const R dd = dot(xyz(hull[s.hf + i]), d);
        if (!isnan(dd) && (bi == 0xFFFFFFFFu || dd > bv)) {
            bv = dd;
            bi = i;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const R ov = __shfl_xor_sync(0xFFFFFFFFu, bv, off);
        const uint32_t oi = __shfl_xor_sync(0xFFFFFFFFu, bi, off);
        if (oi != 0xFFFFFFFFu && (bi == 0xFFFFFFFFu || ov > bv || (ov == bv && oi < bi))) {
            bv = ov;
            bi = oi;
        }
    }
    return xyz(hull[s.hf + bi]);
}

template <class R>
__device__ __forceinline__ void support_witness(const NB<R>& a, const NB<R>& b, V3<R> d, const A4<R>* hull,
                                                V3<R>& point, V3<R>& wit) {
    V3<R> al = rotate(conj(a.rot), d);
    V3<R> ap = add(rotate(a.rot, support(a.shape, al, hull)), a.pos);
    V3<R> bl = rotate(conj(b.rot), neg(d));
    V3<R> bp = add(rotate(b.rot, support(b.shape, bl, hull)), b.pos);
    point = sub(ap, bp);
    wit = ap;
}
// the same with the warp's lanes over hull vertices (all 32 lanes call it)
template <class R>
__device__ __forceinline__ void support_witness_warp(const NB<R>& a, const NB<R>& b, V3<R> d, const A4<R>* hull,
                                                     V3<R>& point, V3<R>& wit, uint32_t lane) {
    V3<R> al = rotate(conj(a.rot), d);
    V3<R> ap = add(rotate(a.rot, support_warp(a.shape, al, hull, lane)), a.pos);
    V3<R> bl = rotate(conj(b.rot), neg(d));
    V3<R> bp = add(rotate(b.rot, support_warp(b.shape, bl, hull, lane)), b.pos);
    point = sub(ap, bp);
    wit = ap;
}

// ---------------------------------------------------------------- SAT
template <class R>
__device__ __forceinline__ void axes_of(Q4<R> q, V3<R> ax[3]) {
    ax[0] = rotate(q, V3<R>{R(1), R(0), R(0)});
    ax[1] = rotate(q, V3<R>{R(0), R(1), R(0)});
    ax[2] = rotate(q, V3<R>{R(0), R(0), R(1)});
}

template <class R>
__device__ __forceinline__ V3<R> box_half(const ShapeR<R>& s) {
    if (s.tag == DIO_SHAPE_BOX) return s.c[0];
    return {s.c[0].x, s.c[0].x, s.c[0].x};
}

// projected radius: cuboid.rs:37-40 for CUBE pairs, per-axis for BOX
template <class R>
__device__ __forceinline__ R box_radius(V3<R> h, const V3<R> ax[3], V3<R> axis, bool per_axis) {
    if (!per_axis) return h.x * (dabs(dot(axis, ax[0])) + dabs(dot(axis, ax[1])) + dabs(dot(axis, ax[2])));
    return h.x * dabs(dot(axis, ax[0])) + h.y * dabs(dot(axis, ax[1])) + h.z * dabs(dot(axis, ax[2]));
}

template <class R>
__device__ __forceinline__ R comp(V3<R> v, uint32_t i) {
    return i == 0 ? v.x : (i == 1 ? v.y : v.z);
}

template <class R>
struct Manifold {
    V3<R> normal;
    R depth;
    V3<R> pa[8], pb[8];
    uint32_t count;
};

// test_axis, cuboid.rs:19-52
template <class R>
__device__ __forceinline__ bool test_axis(V3<R> raw, uint32_t kind, uint32_t index, V3<R> ha, const V3<R> aax[3],
                                          V3<R> hb, const V3<R> bax[3], V3<R> delta, bool per_axis, R& best_ov,
                                          V3<R>& best_n, uint32_t& best_kind, uint32_t& best_idx) {
    if (length_sq(raw) <= R(1.0e-8)) return true;
    V3<R> axis = normalize(raw);
    R ra = box_radius(ha, aax, axis, per_axis);
    R rb = box_radius(hb, bax, axis, per_axis);
    R ov = ra + rb - dabs(dot(delta, axis));
    if (ov < R(0)) return false;
    if (ov < best_ov) {
        best_ov = ov;
        best_n = dot(delta, axis) >= R(0) ? axis : neg(axis);
        best_kind = kind;
        best_idx = index;
    }
    return true;
}

template <class R>
__device__ __forceinline__ void face_frame(V3<R> pos, const V3<R> ax[3], V3<R> h, uint32_t ai, V3<R> outward,
                                           V3<R>* verts, V3<R>& center, V3<R>& u, V3<R>& v, R& eu, R& ev) {
    V3<R> axis = ax[ai];
    V3<R> fn = scale(axis, dot(axis, outward) >= R(0) ? R(1) : R(-1));
    center = add(pos, scale(fn, comp(h, ai)));
    uint32_t ui = ai == 0 ? 1u : 0u;
    uint32_t vi = ai == 2 ? 1u : 2u;
    u = ax[ui];
    v = ax[vi];
    eu = comp(h, ui);
    ev = comp(h, vi);
    if (verts) {
        verts[0] = add(add(center, scale(u, eu)), scale(v, ev));
        verts[1] = add(sub(center, scale(u, eu)), scale(v, ev));
        verts[2] = sub(sub(center, scale(u, eu)), scale(v, ev));
        verts[3] = sub(add(center, scale(u, eu)), scale(v, ev));
    }
}

// clip_plane, cuboid.rs:216-250
template <class R>
__device__ __forceinline__ uint32_t clip_plane(const V3<R>* in, uint32_t n_in, V3<R> normal, R offset, V3<R>* out) {
    if (n_in == 0) return 0;
    uint32_t count = 0;
    V3<R> prev = in[n_in - 1];
    R prev_d = dot(normal, prev) - offset;
    for (uint32_t i = 0; i < n_in; ++i) {
        V3<R> cur = in[i];
        R cur_d = dot(normal, cur) - offset;
        bool pin = prev_d <= R(1.0e-5);
        bool cin = cur_d <= R(1.0e-5);
        if (pin != cin) {
            R den = prev_d - cur_d;
            if (dabs(den) > R(1.0e-8) && count < 8) {
                R t = prev_d / den;
                t = t < R(0) ? R(0) : (t > R(1) ? R(1) : t);
                out[count++] = add(prev, scale(sub(cur, prev), t));
            }
        }
        if (cin && count < 8) out[count++] = cur;
        prev = cur;
        prev_d = cur_d;
    }
    return count;
}

template <class R>
__device__ __forceinline__ void centered_contact(const NB<R>& a, const V3<R> aax[3], V3<R> ha, const NB<R>& b,
                                                 const V3<R> bax[3], V3<R> hb, V3<R> normal, R depth, bool per_axis,
                                                 Manifold<R>& m) {
    R ra = box_radius(ha, aax, normal, per_axis);
    R rb = box_radius(hb, bax, normal, per_axis);
    m.normal = normal;
    m.depth = depth;
    m.pa[0] = add(a.pos, scale(normal, ra));
    m.pb[0] = sub(b.pos, scale(normal, rb));
    m.count = 1;
}

// collide_manifold, cuboid.rs:276-377 (max_contacts 4 = reference, 8 = all)
template <class R>
__device__ bool collide_manifold(const NB<R>& a, const NB<R>& b, uint32_t max_contacts, Manifold<R>& m) {
    bool per_axis = !(a.shape.tag == DIO_SHAPE_CUBE && b.shape.tag == DIO_SHAPE_CUBE);
    V3<R> aax[3], bax[3];
    axes_of(a.rot, aax);
    axes_of(b.rot, bax);
    V3<R> ha = box_half(a.shape), hb = box_half(b.shape);
    V3<R> delta = sub(b.pos, a.pos);
    R best_ov = 3.402823466e+38f;
    if (sizeof(R) == 8) best_ov = R(1.7976931348623157e308);
    V3<R> best_n{R(1), R(0), R(0)};
    uint32_t best_kind = 0, best_idx = 0;
    for (uint32_t i = 0; i < 3; ++i)
        if (!test_axis(aax[i], 0, i, ha, aax, hb, bax, delta, per_axis, best_ov, best_n, best_kind, best_idx))
            return false;
    for (uint32_t i = 0; i < 3; ++i)
        if (!test_axis(bax[i], 1, i, ha, aax, hb, bax, delta, per_axis, best_ov, best_n, best_kind, best_idx))
            return false;
    for (uint32_t i = 0; i < 3; ++i)
        for (uint32_t j = 0; j < 3; ++j)
            if (!test_axis(cross(aax[i], bax[j]), 2, i * 3 + j, ha, aax, hb, bax, delta, per_axis, best_ov, best_n,
                           best_kind, best_idx))
                return false;
    V3<R> normal = best_n;
    R depth = best_ov;
    if (best_kind == 2) {
        centered_contact(a, aax, ha, b, bax, hb, normal, depth, per_axis, m);
        return true;
    }
    bool ref_a = best_kind == 0;
    V3<R> rn = ref_a ? normal : neg(normal);
    // incident_axis, cuboid.rs:198-214
    const V3<R>* iax = ref_a ? bax : aax;
    uint32_t inc_axis = 0;
    R bdot = dabs(dot(iax[0], rn));
    for (uint32_t i = 1; i < 3; ++i) {
        R d = dabs(dot(iax[i], rn));
        if (d > bdot) {
            bdot = d;
            inc_axis = i;
        }
    }
    V3<R> center, u, v, c2, u2, v2;
    R eu, ev, eu2, ev2;
    face_frame(ref_a ? a.pos : b.pos, ref_a ? aax : bax, ref_a ? ha : hb, best_idx, rn, (V3<R>*)nullptr, center, u,
               v, eu, ev);
    V3<R> pa[8], pb[8];
    face_frame(ref_a ? b.pos : a.pos, iax, ref_a ? hb : ha, inc_axis, neg(rn), pa, c2, u2, v2, eu2, ev2);
    uint32_t count = 4;
    count = clip_plane(pa, count, u, dot(u, center) + eu, pb);
    count = clip_plane(pb, count, neg(u), dot(neg(u), center) + eu, pa);
    count = clip_plane(pa, count, v, dot(v, center) + ev, pb);
    count = clip_plane(pb, count, neg(v), dot(neg(v), center) + ev, pa);
    if (count == 0) {
        centered_contact(a, aax, ha, b, bax, hb, normal, depth, per_axis, m);
        return true;
    }
    R ref_plane = dot(rn, center);
    uint32_t cc = 0;
    for (uint32_t i = 0; i < count; ++i) {
        if (cc >= max_contacts) break;
        V3<R> ip = pa[i];
        R pd = ref_plane - dot(rn, ip);
        if (pd < R(-1.0e-5)) continue;
        V3<R> rp = add(ip, scale(rn, pd > R(0) ? pd : R(0)));
        m.pa[cc] = ref_a ? rp : ip;
        m.pb[cc] = ref_a ? ip : rp;
        ++cc;
    }
    if (cc == 0) {
        centered_contact(a, aax, ha, b, bax, hb, normal, depth, per_axis, m);
        return true;
    }
    m.normal = normal;
    m.depth = depth;
    m.count = cc;
    return true;
}

// ---------------------------------------------------------------- GJK
template <class R>
struct Simplex {
    V3<R> p[4], w[4];
    uint32_t len;
    __device__ void push_front(V3<R> pt, V3<R> wt) {
#pragma unroll
        for (int i = 3; i > 0; --i)
            if (i <= (int)len) {
                p[i] = p[i - 1];
                w[i] = w[i - 1];
            }
        p[0] = pt;
        w[0] = wt;
        len = len + 1 < 4 ? len + 1 : 4;
    }
    __device__ void remove(uint32_t index) {
#pragma unroll
        for (uint32_t i = 0; i < 3; ++i)
            if (i >= index && i + 1 < len) {
                p[i] = p[i + 1];
                w[i] = w[i + 1];
            }
        len -= 1;
    }
    __device__ void swap12() {
        V3<R> t = p[1];
        p[1] = p[2];
        p[2] = t;
        t = w[1];
        w[1] = w[2];
        w[2] = t;
    }
};

template <class R>
__device__ __forceinline__ bool same_dir(V3<R> a, V3<R> b) { return dot(a, b) > R(0); }
template <class R>
__device__ __forceinline__ V3<R> triple(V3<R> a, V3<R> b, V3<R> c) { return cross(cross(a, b), c); }
template <class R>
__device__ __forceinline__ V3<R> any_perpendicular(V3<R> v) {
    V3<R> axis;
    if (dabs(v.x) <= dabs(v.y) && dabs(v.x) <= dabs(v.z))
        axis = {R(1), R(0), R(0)};
    else if (dabs(v.y) <= dabs(v.z))
        axis = {R(0), R(1), R(0)};
    else
        axis = {R(0), R(0), R(1)};
    return normalize_or_zero(cross(axis, v));
}

// contains_origin, gjk.rs:112-201
template <class R>
__device__ bool contains_origin(Simplex<R>& s, V3<R>& d) {
    if (s.len == 4) {
        V3<R> a = s.p[0];
        V3<R> ao = neg(a), ab = sub(s.p[1], a), ac = sub(s.p[2], a), ad = sub(s.p[3], a);
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
    if (s.len == 1) {
        d = neg(s.p[0]);
        return false;
    }
    if (s.len == 2) {
        V3<R> a = s.p[0];
        V3<R> ab = sub(s.p[1], a), ao = neg(a);
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
    if (s.len == 3) {
        V3<R> a = s.p[0];
        V3<R> ab = sub(s.p[1], a), ac = sub(s.p[2], a), ao = neg(a);
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
                s.swap12();
                d = neg(abc);
            }
        }
        return false;
    }
    return false;
}

// gjk, gjk.rs:77-109
template <class R>
__device__ bool gjk(const NB<R>& a, const NB<R>& b, const A4<R>* hull, Simplex<R>& s) {
    V3<R> d = sub(a.pos, b.pos);
    if (d.x == R(0) && d.y == R(0) && d.z == R(0)) d = {R(1), R(0), R(0)};
    s.len = 0;
    V3<R> pt, wt;
    support_witness(a, b, d, hull, pt, wt);
    s.push_front(pt, wt);
    d = neg(s.p[0]);
    for (int it = 0; it < 64; ++it) {
        support_witness(a, b, d, hull, pt, wt);
        if (dot(pt, d) < R(0)) return false;
        s.push_front(pt, wt);
        if (contains_origin(s, d)) return true;
        if (length_sq(d) < R(1e-12)) d = any_perpendicular(s.p[0]);
    }
    return false;
}

// ---------------------------------------------------------------- EPA
constexpr int kEpaV = 68;   // 4 simplex points + one per iteration (64)
constexpr int kEpaF = 256;  // face capacity (reference: 512; overflow flagged)
constexpr int kEpaH = 256;  // horizon capacity (reference: 512; overflow flagged)
template <class R>
__host__ __device__ constexpr int epa_warps() { return sizeof(R) == 8 ? 2 : 4; }  // FP64 polytopes are twice the size

template <class R>
struct EpaSmem {
    A4<R> v[kEpaV];
    A4<R> w[kEpaV];
    A4<R> fnd[kEpaF];      // face normal xyz, distance w
    uint32_t fabc[kEpaF];  // a | b << 8 | c << 16
    uint32_t hor[kEpaH];   // a | b << 8
};

__device__ __forceinline__ uint32_t fa_(uint32_t f) { return f & 0xFF; }
__device__ __forceinline__ uint32_t fb_(uint32_t f) { return (f >> 8) & 0xFF; }
__device__ __forceinline__ uint32_t fc_(uint32_t f) { return (f >> 16) & 0xFF; }

__device__ __forceinline__ bool edge_in_face(uint32_t a, uint32_t b, uint32_t f) {
    uint32_t x = fa_(f), y = fb_(f), z = fc_(f);
    return (x == a && y == b) || (y == a && z == b) || (z == a && x == b) || (x == b && y == a) ||
           (y == b && z == a) || (z == b && x == a);
}

// add_face arithmetic, epa.rs:58-85.  Returns false for a degenerate face.
template <class R>
__device__ __forceinline__ bool make_face(const EpaSmem<R>& S, uint32_t a, uint32_t b, uint32_t c, A4<R>& nd,
                                          uint32_t& abc) {
    V3<R> va = xyz(S.v[a]);
    V3<R> n = cross(sub(xyz(S.v[b]), va), sub(xyz(S.v[c]), va));
    if (length_sq(n) < R(1e-12)) return false;
    n = normalize(n);
    R dist = dot(n, va);
    if (dist < R(0)) {
        uint32_t t = a;
        a = c;
        c = t;
        n = neg(n);
        dist = -dist;
    }
    nd = pack(n, dist);
    abc = a | (b << 8) | (c << 16);
    return true;
}

// face_contact, epa.rs:193-240
template <class R>
__device__ void face_contact(const EpaSmem<R>& S, A4<R> nd, uint32_t abc, V3<R>& normal, R& depth, V3<R>& pa,
                             V3<R>& pb) {
    uint32_t ia = fa_(abc), ib = fb_(abc), ic = fc_(abc);
    V3<R> va = xyz(S.v[ia]), vb = xyz(S.v[ib]), vc = xyz(S.v[ic]);
    V3<R> n = xyz(nd);
    R dist = nd.w;
    V3<R> closest = scale(n, dist);
    V3<R> v0 = sub(vb, va), v1 = sub(vc, va), v2 = sub(closest, va);
    R d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0), d21 = dot(v2, v1);
    R denom = d00 * d11 - d01 * d01;
    R w1, w2, w3;
    if (dabs(denom) > R(1e-12)) {
        w2 = (d11 * d20 - d01 * d21) / denom;
        w3 = (d00 * d21 - d01 * d20) / denom;
        w1 = R(1) - w2 - w3;
    } else {
        w1 = R(1);
        w2 = R(0);
        w3 = R(0);
    }
    w1 = w1 < R(0) ? R(0) : (w1 > R(1) ? R(1) : w1);
    w2 = w2 < R(0) ? R(0) : (w2 > R(1) ? R(1) : w2);
    w3 = w3 < R(0) ? R(0) : (w3 > R(1) ? R(1) : w3);
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
    V3<R> wa = xyz(S.w[ia]), wb = xyz(S.w[ib]), wc = xyz(S.w[ic]);
    pa = add(add(scale(wa, w1), scale(wb, w2)), scale(wc, w3));
    V3<R> mk = add(add(scale(va, w1), scale(vb, w2)), scale(vc, w3));
    pb = sub(pa, mk);
    normal = n;
    depth = dist;
}

// Warp-cooperative epa, epa.rs:89-189.  All lanes of the warp call it with
// the same arguments; returns true (uniformly) on convergence.
template <class R>
__device__ bool epa_warp(EpaSmem<R>& S, const NB<R>& a, const NB<R>& b, const A4<R>* simplex, const A4<R>* hull,
                         uint32_t* err, V3<R>& normal, R& depth, V3<R>& pa, V3<R>& pb) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    if (lane < 4) {
        S.v[lane] = simplex[lane];
        S.w[lane] = simplex[4 + lane];
    }
    if (lane == 0) {
        S.fnd[0] = A4<R>{R(0), R(0), R(0), R(0)};
        S.fabc[0] = 0;
    }
    __syncwarp();
    uint32_t nf = 0;
    uint32_t nv = 4;
    {
        // the four initial faces, epa.rs:97-100, added in order
        const uint32_t init[4] = {0u | (1u << 8) | (2u << 16), 0u | (3u << 8) | (1u << 16),
                                  0u | (2u << 8) | (3u << 16), 1u | (3u << 8) | (2u << 16)};
        A4<R> nd;
        uint32_t abc;
        bool ok = false;
        if (lane < 4) ok = make_face(S, fa_(init[lane]), fb_(init[lane]), fc_(init[lane]), nd, abc);
        uint32_t okm = __ballot_sync(0xFFFFFFFFu, ok);
        __syncwarp();
        if (ok) {
            uint32_t pos = __popc(okm & lt_mask);
            S.fnd[pos] = nd;
            S.fabc[pos] = abc;
        }
        nf = __popc(okm);
        __syncwarp();
    }
    for (int it = 0; it < 64; ++it) {
        // no face of nonzero area (a flat or collapsed simplex): no contact,
        // where the reference would emit its zero default face (a zero normal
        // at zero depth, whose tangents are NaN)
        if (nf == 0) return false;  // warp-uniform
        // closest face: first minimum in index order (strict <)
        uint32_t mi = 0;
        {
            R d0 = S.fnd[0].w;
            if (nf > 0 && !isnan(d0)) {
                R bv = R(0);
                uint32_t bi = 0xFFFFFFFFu;
                for (uint32_t i = lane; i < nf; i += 32) {
                    R d = S.fnd[i].w;
                    if (isnan(d)) continue;
                    if (bi == 0xFFFFFFFFu || d < bv) {
                        bv = d;
                        bi = i;
                    }
                }
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    R ov = __shfl_xor_sync(0xFFFFFFFFu, bv, off);
                    uint32_t oi = __shfl_xor_sync(0xFFFFFFFFu, bi, off);
                    bool take = oi != 0xFFFFFFFFu && (bi == 0xFFFFFFFFu || ov < bv || (ov == bv && oi < bi));
                    if (take) {
                        bv = ov;
                        bi = oi;
                    }
                }
                mi = bi;
            }
        }
        A4<R> mnd = S.fnd[mi];
        uint32_t mabc = S.fabc[mi];
        V3<R> sp, sw;
        support_witness_warp(a, b, xyz(mnd), hull, sp, sw, lane);
        R sd = dot(xyz(mnd), sp);
        if (sd - mnd.w < R(1e-4)) {
            face_contact(S, mnd, mabc, normal, depth, pa, pb);
            return true;
        }
        uint32_t ni = nv;
        if (ni >= 256u) {
            face_contact(S, mnd, mabc, normal, depth, pa, pb);
            return true;
        }
        if (lane == 0) {
            S.v[ni] = pack(sp);
            S.w[ni] = pack(sw);
        }
        nv += 1;
        __syncwarp();
        // visibility masks (one 32-bit ballot per chunk of faces)
        uint32_t vm[kEpaF / 32];
#pragma unroll
        for (int c = 0; c < kEpaF / 32; ++c) {
            vm[c] = 0u;
            if (c * 32 >= (int)nf) continue;  // warp-uniform
            uint32_t i = c * 32 + lane;
            bool vis = false;
            if (i < nf) {
                A4<R> f = S.fnd[i];
                vis = dot(xyz(f), sub(sp, xyz(S.v[fa_(S.fabc[i])]))) > R(0);
            }
            vm[c] = __ballot_sync(0xFFFFFFFFu, vis);
        }
        // horizon: edges of visible faces not shared with another visible face
        uint32_t hc = 0;
        for (int c = 0; c < kEpaF / 32; ++c) {
            if (c * 32 >= (int)nf) break;
            uint32_t i = c * 32 + lane;
            uint32_t my[3];
            uint32_t k = 0;
            if ((vm[c] >> lane) & 1u) {
                uint32_t f = S.fabc[i];
                uint32_t e[3][2] = {{fa_(f), fb_(f)}, {fb_(f), fc_(f)}, {fc_(f), fa_(f)}};
                for (int ee = 0; ee < 3; ++ee) {
                    bool shared = false;
                    for (int cc = 0; cc < kEpaF / 32 && !shared; ++cc) {
                        uint32_t m = vm[cc];
                        while (m) {
                            uint32_t bit = __ffs(m) - 1;
                            m &= m - 1;
                            uint32_t j = cc * 32 + bit;
                            if (j == i) continue;
                            if (edge_in_face(e[ee][0], e[ee][1], S.fabc[j])) {
                                shared = true;
                                break;
                            }
                        }
                    }
                    if (!shared) my[k++] = e[ee][0] | (e[ee][1] << 8);
                }
            }
            // order-preserving append (inclusive warp scan of k)
            uint32_t incl = k;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, off);
                if (lane >= (uint32_t)off) incl += t;
            }
            uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
            uint32_t base = hc + incl - k;
            for (uint32_t t = 0; t < k; ++t)
                if (base + t < (uint32_t)kEpaH) S.hor[base + t] = my[t];
            hc += total;
        }
        if (hc > (uint32_t)kEpaH) {
            if (lane == 0) atomicOr(err, kErrEpaHorizon);
            hc = kEpaH;
        }
        __syncwarp();
        // compact the kept (invisible) faces in place, preserving order
        uint32_t wr = 0;
        for (int c = 0; c < kEpaF / 32; ++c) {
            if (c * 32 >= (int)nf) break;
            uint32_t i = c * 32 + lane;
            bool keep = i < nf && !((vm[c] >> lane) & 1u);
            A4<R> f;
            uint32_t fabc = 0;
            if (keep) {
                f = S.fnd[i];
                fabc = S.fabc[i];
            }
            uint32_t km = __ballot_sync(0xFFFFFFFFu, keep);
            __syncwarp();
            if (keep) {
                uint32_t pos = wr + __popc(km & lt_mask);
                S.fnd[pos] = f;
                S.fabc[pos] = fabc;
            }
            wr += __popc(km);
            __syncwarp();
        }
        nf = wr;
        // stitch the horizon to the new vertex (degenerate faces dropped)
        for (uint32_t c = 0; c * 32 < hc; ++c) {
            uint32_t h = c * 32 + lane;
            A4<R> nd;
            uint32_t abc = 0;
            bool ok = false;
            if (h < hc) {
                uint32_t e = S.hor[h];
                ok = make_face(S, ni, e & 0xFF, (e >> 8) & 0xFF, nd, abc);
            }
            uint32_t okm = __ballot_sync(0xFFFFFFFFu, ok);
            uint32_t pos = nf + __popc(okm & lt_mask);
            if (ok && pos < (uint32_t)kEpaF) {
                S.fnd[pos] = nd;
                S.fabc[pos] = abc;
            }
            uint32_t add_n = __popc(okm);
            if (nf + add_n > (uint32_t)kEpaF) {
                if (lane == 0) atomicOr(err, kErrEpaFaces);
                nf = kEpaF;
            } else {
                nf += add_n;
            }
            __syncwarp();
        }
    }
    return false;
}

}  // namespace dio
