// k_avbd.cuh -- AVBD init / primal / dual / recover on sm_103a.
//
// Restates engine/gpu_physics/avbd/src/lib.rs:202-699.  Differences in
// structure (not in arithmetic):
//   * SoA poses (16-byte vector loads) instead of AoS Vec4 buffers.
//   * Contacts are read through a per-body CSR that also carries the other
//     body and the a/b side, so the row's (a, b) never has to be fetched.
//   * Joints are read through a per-body joint CSR in joint order instead of
//     the reference's scan over every joint for every body (O(N J)); the
//     accumulation order per body is unchanged.
//   * P (pose precision) may be double: inertial targets, poses and lambda
//     accumulate in FP64 while the 6x6 Hessian, LDL^T and rows stay in R.
//   * The final pose is also left in buffer 0, so a device-resident world
//     starts every step from buffer 0.
#pragma once

#include <type_traits>

#include "div_rn.cuh"
#include "engine.cuh"

namespace dio {

template <class R>
struct Block6 {
    R h[21];  // lower triangle, row-major: (0,0) (1,0) (1,1) (2,0) ...
    R g[6];
};

__device__ __forceinline__ constexpr int tri(int i, int j) { return i * (i + 1) / 2 + j; }

// H += J J^T k, g += J f (add_constraint_row, avbd/src/lib.rs:182-198)
template <class R>
__device__ __forceinline__ void stamp(Block6<R>& B, V3<R> jl, V3<R> ja, R k, R f) {
    const R J[6] = {jl.x, jl.y, jl.z, ja.x, ja.y, ja.z};
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j) B.h[tri(i, j)] = B.h[tri(i, j)] + J[i] * J[j] * k;
#pragma unroll
    for (int i = 0; i < 6; ++i) B.g[i] = B.g[i] + J[i] * f;
}

// stamp() for a row whose Jacobian entries outside MASK are exact zeros
// (a ball-socket axis row: J = (s e_k, r x s e_k)).  The H terms with a zero
// factor are +-0 when J and k are finite, and adding +-0 leaves an H entry
// unchanged because a round-to-nearest sum that starts at +0 (or at the
// positive diagonal) is never -0; so skipping them is exact.  g takes all
// six terms (its start values can be -0).  Callers check finiteness first.
template <int MASK, class R>
__device__ __forceinline__ void stamp_masked(Block6<R>& B, V3<R> jl, V3<R> ja, R k, R f) {
    const R J[6] = {jl.x, jl.y, jl.z, ja.x, ja.y, ja.z};
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j)
            if (((MASK >> i) & 1) && ((MASK >> j) & 1)) B.h[tri(i, j)] = B.h[tri(i, j)] + J[i] * J[j] * k;
#pragma unroll
    for (int i = 0; i < 6; ++i) B.g[i] = B.g[i] + J[i] * f;
}
constexpr int kMaskAxisX = (1 << 0) | (1 << 4) | (1 << 5);  // J = (s, 0, 0, 0, s r.z, -s r.y)
constexpr int kMaskAxisY = (1 << 1) | (1 << 3) | (1 << 5);  // J = (0, s, 0, -s r.z, 0, s r.x)
constexpr int kMaskAxisZ = (1 << 2) | (1 << 3) | (1 << 4);  // J = (0, 0, s, s r.y, -s r.x, 0)

// solve6, avbd/src/lib.rs:107-180 (unpivoted LDL^T); solves H x = -g.  Each
// quotient by a pivot is the IEEE quotient (div_rn.cuh: one reciprocal per
// pivot, a correction step per quotient).
template <class R>
__device__ __forceinline__ void solve6(const Block6<R>& B, R x[6]) {
    const R* H = B.h;
    R a11 = H[tri(0, 0)], a21 = H[tri(1, 0)], a31 = H[tri(2, 0)], a22 = H[tri(1, 1)], a32 = H[tri(2, 1)],
      a33 = H[tri(2, 2)];
    R a41 = H[tri(3, 0)], a51 = H[tri(4, 0)], a61 = H[tri(5, 0)], a42 = H[tri(3, 1)], a52 = H[tri(4, 1)],
      a62 = H[tri(5, 1)];
    R a43 = H[tri(3, 2)], a53 = H[tri(4, 2)], a63 = H[tri(5, 2)];
    R a44 = H[tri(3, 3)], a54 = H[tri(4, 3)], a64 = H[tri(5, 3)], a55 = H[tri(4, 4)], a65 = H[tri(5, 4)],
      a66 = H[tri(5, 5)];
    const Divisor<R> p1(a11);
    R l21 = p1.div(a21), l31 = p1.div(a31), l41 = p1.div(a41), l51 = p1.div(a51), l61 = p1.div(a61);
    R d1 = a11;
    R d2 = a22 - l21 * l21 * d1;
    const Divisor<R> p2(d2);
    R l32 = p2.div(a32 - l21 * l31 * d1);
    R l42 = p2.div(a42 - l21 * l41 * d1);
    R l52 = p2.div(a52 - l21 * l51 * d1);
    R l62 = p2.div(a62 - l21 * l61 * d1);
    R d3 = a33 - (l31 * l31 * d1 + l32 * l32 * d2);
    const Divisor<R> p3(d3);
    R l43 = p3.div(a43 - l31 * l41 * d1 - l32 * l42 * d2);
    R l53 = p3.div(a53 - l31 * l51 * d1 - l32 * l52 * d2);
    R l63 = p3.div(a63 - l31 * l61 * d1 - l32 * l62 * d2);
    R d4 = a44 - (l41 * l41 * d1 + l42 * l42 * d2 + l43 * l43 * d3);
    const Divisor<R> p4(d4);
    R l54 = p4.div(a54 - l41 * l51 * d1 - l42 * l52 * d2 - l43 * l53 * d3);
    R l64 = p4.div(a64 - l41 * l61 * d1 - l42 * l62 * d2 - l43 * l63 * d3);
    R d5 = a55 - (l51 * l51 * d1 + l52 * l52 * d2 + l53 * l53 * d3 + l54 * l54 * d4);
    const Divisor<R> p5(d5);
    R l65 = p5.div(a65 - l51 * l61 * d1 - l52 * l62 * d2 - l53 * l63 * d3 - l54 * l64 * d4);
    R d6 = a66 - (l61 * l61 * d1 + l62 * l62 * d2 + l63 * l63 * d3 + l64 * l64 * d4 + l65 * l65 * d5);
    R b0 = -B.g[0], b1 = -B.g[1], b2 = -B.g[2], b3 = -B.g[3], b4 = -B.g[4], b5 = -B.g[5];
    R y1 = b0;
    R y2 = b1 - l21 * y1;
    R y3 = b2 - l31 * y1 - l32 * y2;
    R y4 = b3 - l41 * y1 - l42 * y2 - l43 * y3;
    R y5 = b4 - l51 * y1 - l52 * y2 - l53 * y3 - l54 * y4;
    R y6 = b5 - l61 * y1 - l62 * y2 - l63 * y3 - l64 * y4 - l65 * y5;
    R z1 = p1.div(y1), z2 = p2.div(y2), z3 = p3.div(y3), z4 = p4.div(y4), z5 = p5.div(y5), z6 = y6 / d6;
    x[5] = z6;
    x[4] = z5 - l65 * x[5];
    x[3] = z4 - l54 * x[4] - l64 * x[5];
    x[2] = z3 - l43 * x[3] - l53 * x[4] - l63 * x[5];
    x[1] = z2 - l32 * x[2] - l42 * x[3] - l52 * x[4] - l62 * x[5];
    x[0] = z1 - l21 * x[1] - l31 * x[2] - l41 * x[3] - l51 * x[4] - l61 * x[5];
}

// avbd_init, avbd/src/lib.rs:202-254 (+ seeding buffer 1 with the
// un-warm-started pose, render/gpu_physics.rs:479-482)
template <class P, class R>
__device__ __forceinline__ void init_body(const DevWorld<P, R>& w, uint32_t i, const SolveParams<R>& o) {
    A4<P> p4 = w.pos[0][i];
    A4<P> q4 = w.rot[0][i];
    R inv_mass = w.inv[i].w;
    // buffer 1 holds the un-warm-started pose for bodies the primal never
    // writes (static ones); a dynamic body's copy is overwritten by the first
    // primal before anything reads it, unless there is no iteration at all
    if (inv_mass == R(0) || o.iterations == 0) {
        w.pos[1][i] = p4;
        w.rot[1][i] = q4;
    }
    V3<P> pos = xyz(p4);
    Q4<P> rot = quat(q4);
    V3<P> vel = xyz(w.vel[i]);
    V3<P> ang = xyz(w.ang[i]);
    P dt = P(o.dt);
    V3<P> g{P(o.gx), P(o.gy), P(o.gz)};
    w.init_pos[i] = pack(pos);
    w.init_rot[i] = q4;
    V3<P> ip = add(pos, scale(vel, dt));
    if (inv_mass > R(0)) ip = add(ip, scale(g, dt * dt));
    w.inert_pos[i] = pack(ip);
    Q4<P> irot = quat_step(rot, scale(ang, dt));
    w.inert_rot[i] = packq(irot);
    if (w.mdt2 && inv_mass != R(0)) {
        // the primal's diagonal, constant over the step (avbd/src/lib.rs:293-296)
        const A4<R> inv = w.inv[i];
        const R mass = R(1) / inv.w;
        const V3<R> moment{R(1) / inv.x, R(1) / inv.y, R(1) / inv.z};
        const R dt2 = o.dt * o.dt;
        const V3<R> idt2 = divs(moment, dt2);
        w.mdt2[i] = A4<R>{mass / dt2, idt2.x, idt2.y, idt2.z};
    }
    if (inv_mass > R(0)) {
        // adaptive gravity weight, clamped to [0, 1]: formed in R in the split
        // mode (it only scales the warm-start offset)
        using Fq = std::conditional_t<std::is_same<P, R>::value, P, R>;
        const Fq dtf = Fq(o.dt);
        const V3<Fq> gf{Fq(o.gx), Fq(o.gy), Fq(o.gz)};
        V3<Fq> accel = divs(cast3<Fq>(sub(vel, xyz(w.prev_vel[i]))), dtf);
        Fq gm = length(gf);
        Fq wgt = Fq(0);
        if (gm > Fq(0)) {
            wgt = dot(accel, divs(gf, gm)) / gm;
            wgt = wgt < Fq(0) ? Fq(0) : (wgt > Fq(1) ? Fq(1) : wgt);
        }
        w.pos[0][i] = pack(add(add(pos, scale(vel, dt)), scale(g, P(wgt) * dt * dt)));
        w.rot[0][i] = packq(irot);  // the same quat_step(rot, ang dt)
    }
}

template <class P, class R>
__global__ void __launch_bounds__(256) k_init(DevWorld<P, R> w, uint32_t lo, uint32_t hi, SolveParams<R> o) {
    pdl_enter();
    for (uint32_t i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += gridDim.x * blockDim.x)
        init_body(w, i, o);
}

// Where the primal reads another body's snapshot / step-start pose: global
// memory, or a shared-memory tile of consecutive bodies with a global
// fallback.  Both return the same values.
// `store` writes a body's new pose (the primal's output buffer).
template <class P, class R>
struct GlobalFetch {
    const DevWorld<P, R>& w;
    int rd;
    __device__ __forceinline__ A4<P> pos(uint32_t j) const { return w.pos[rd][j]; }
    __device__ __forceinline__ A4<P> rot(uint32_t j) const { return w.rot[rd][j]; }
    __device__ __forceinline__ A4<P> ipos(uint32_t j) const { return w.init_pos[j]; }
    __device__ __forceinline__ A4<P> irot(uint32_t j) const { return w.init_rot[j]; }
    __device__ __forceinline__ void store(uint32_t i, A4<P> p, A4<P> q) const {
        w.pos[1 - rd][i] = p;
        w.rot[1 - rd][i] = q;
    }
};

template <class P, class R, int T>
struct TileFetch {
    const DevWorld<P, R>& w;
    int rd;
    uint32_t lo;
    const A4<P>* sp;
    const A4<P>* sq;
    const A4<P>* si;
    const A4<P>* sr;
    __device__ __forceinline__ A4<P> pos(uint32_t j) const { return j - lo < (uint32_t)T ? sp[j - lo] : w.pos[rd][j]; }
    __device__ __forceinline__ A4<P> rot(uint32_t j) const { return j - lo < (uint32_t)T ? sq[j - lo] : w.rot[rd][j]; }
    __device__ __forceinline__ A4<P> ipos(uint32_t j) const { return j - lo < (uint32_t)T ? si[j - lo] : w.init_pos[j]; }
    __device__ __forceinline__ A4<P> irot(uint32_t j) const { return j - lo < (uint32_t)T ? sr[j - lo] : w.init_rot[j]; }
    __device__ __forceinline__ void store(uint32_t i, A4<P> p, A4<P> q) const {
        w.pos[1 - rd][i] = p;
        w.rot[1 - rd][i] = q;
    }
};

// Poses of one scene chunk held in shared memory: bodies [lo, lo + count)
// at index j - lo.  Every body a chunk's rows and joints touch lies in the
// chunk (rows and joints never cross scenes).
template <class P>
struct SmemFetch {
    const A4<P>* sp;  // snapshot (read) buffer
    const A4<P>* sq;
    const A4<P>* si;  // step-start pose
    const A4<P>* sr;
    A4<P>* wp;        // the primal's output buffer
    A4<P>* wq;
    uint32_t lo;
    __device__ __forceinline__ A4<P> pos(uint32_t j) const { return sp[j - lo]; }
    __device__ __forceinline__ A4<P> rot(uint32_t j) const { return sq[j - lo]; }
    __device__ __forceinline__ A4<P> ipos(uint32_t j) const { return si[j - lo]; }
    __device__ __forceinline__ A4<P> irot(uint32_t j) const { return sr[j - lo]; }
    __device__ __forceinline__ void store(uint32_t i, A4<P> p, A4<P> q) const {
        wp[i - lo] = p;
        wq[i - lo] = q;
    }
};

// Clamped row forces shared by avbd_primal and avbd_dual (avbd/src/lib.rs:
// 380-406, 606-631): normal f0 <= 0, friction (f1, f2) scaled back onto the
// cone |f_t| <= mu |f0|; `tm` (unclamped friction magnitude) and `bounds`
// feed the dual's penalty rule.
template <class P, class R>
__device__ __forceinline__ void row_forces(const RowDual<P, R>& du, R mu, R c0, R c1, R c2, P& f0, P& f1, P& f2,
                                           P& tm, P& bounds) {
    f0 = fmin_(P(du.penalty.x * c0) + du.lambda.x, P(0));
    const P f1r = P(du.penalty.y * c1) + du.lambda.y;
    const P f2r = P(du.penalty.z * c2) + du.lambda.z;
    bounds = dabs(f0) * P(mu);
    f1 = f1r;
    f2 = f2r;
    if constexpr (std::is_same<P, R>::value) {
        tm = dsqrt(f1r * f1r + f2r * f2r);
        if (tm > bounds && tm > P(0)) {
            const P s = bounds / tm;
            f1 = f1r * s;
            f2 = f2r * s;
        }
    } else {
        // split mode: the cone magnitude and its scale factor in R, applied to
        // the P forces (lambda still accumulates in P)
        const R f1q = R(f1r), f2q = R(f2r);
        const R tmr = dsqrt(f1q * f1q + f2q * f2q);
        tm = P(tmr);
        if (tm > bounds && tm > P(0)) {
            const R sr = R(bounds) / tmr;
            f1 = f1r * P(sr);
            f2 = f2r * P(sr);
        }
    }
}

// One contact row seen from body i (avbd/src/lib.rs:321-418): its three
// stamps (normal, tangent 1, tangent 2) as Jacobian rows (jl, ja), stiffness
// k and force f.
template <class P, class R, class F>
__device__ __forceinline__ void primal_row_terms(const RowStatic<R>& rs, const RowDual<P, R>& du, uint32_t oth,
                                                 const F& fetch, Q4<R> sqr, V3<R> dqsl, V3<R> dqsa, R k_alpha,
                                                 V3<R> jl[3], V3<R> ja[3], R k[3], R f[3]) {
    const bool container = oth == kContainer;
    const bool is_a = container || !(oth & kIsB);
    const uint32_t other = oth & ~kIsB;
    V3<R> n = xyz(rs.n), t1 = xyz(rs.t1), t2 = xyz(rs.t2);
    V3<R> r0 = is_a ? n : neg(n);
    V3<R> r1 = is_a ? t1 : neg(t1);
    V3<R> r2 = is_a ? t2 : neg(t2);
    V3<R> rw = rotate(sqr, is_a ? xyz(rs.ra) : xyz(rs.rb));
    V3<R> dol{R(0), R(0), R(0)}, doa{R(0), R(0), R(0)}, rot_other{R(0), R(0), R(0)};
    if (!container) {
        A4<P> op = fetch.pos(other);
        A4<P> oq = fetch.rot(other);
        dol = cast3<R>(sub(xyz(op), xyz(fetch.ipos(other))));
        doa = ang_diff(castq<R>(quat(oq)), castq<R>(quat(fetch.irot(other))));
        rot_other = rotate(castq<R>(quat(oq)), is_a ? xyz(rs.rb) : xyz(rs.ra));
    }
    V3<R> j0 = cross(rw, r0), j1 = cross(rw, r1), j2 = cross(rw, r2);
    R c0 = rs.ra.w * k_alpha, c1 = rs.rb.w * k_alpha, c2 = rs.t1.w * k_alpha;
    c0 = c0 + (dot(r0, dqsl) + dot(j0, dqsa) - dot(r0, dol) - dot(cross(rot_other, r0), doa));
    c1 = c1 + (dot(r1, dqsl) + dot(j1, dqsa) - dot(r1, dol) - dot(cross(rot_other, r1), doa));
    c2 = c2 + (dot(r2, dqsl) + dot(j2, dqsa) - dot(r2, dol) - dot(cross(rot_other, r2), doa));
    // the forces only feed the R Hessian: in the split mode they are formed
    // in R from the P lambda (the dual accumulates lambda in P)
    using Fq = std::conditional_t<std::is_same<P, R>::value, P, R>;
    const RowDual<Fq, R> dv{du.penalty, A4<Fq>{Fq(du.lambda.x), Fq(du.lambda.y), Fq(du.lambda.z), Fq(0)}};
    Fq f0, f1, f2, tm, bounds;
    row_forces(dv, rs.n.w, c0, c1, c2, f0, f1, f2, tm, bounds);
    jl[0] = r0;
    jl[1] = r1;
    jl[2] = r2;
    ja[0] = j0;
    ja[1] = j1;
    ja[2] = j2;
    k[0] = du.penalty.x;
    k[1] = du.penalty.y;
    k[2] = du.penalty.z;
    f[0] = R(f0);
    f[1] = R(f1);
    f[2] = R(f2);
}
template <class P, class R, class F>
__device__ __forceinline__ void primal_row_core(const RowStatic<R>& rs, const RowDual<P, R>& du, uint32_t oth,
                                                const F& fetch, Q4<R> sqr, V3<R> dqsl, V3<R> dqsa, R k_alpha,
                                                Block6<R>& B) {
    V3<R> jl[3], ja[3];
    R k[3], f[3];
    primal_row_terms<P, R>(rs, du, oth, fetch, sqr, dqsl, dqsa, k_alpha, jl, ja, k, f);
#pragma unroll
    for (int s = 0; s < 3; ++s) stamp(B, jl[s], ja[s], k[s], f[s]);
}
template <class P, class R, class F>
__device__ __forceinline__ void primal_row_f(const DevWorld<P, R>& w, uint32_t r, uint32_t oth, const F& fetch,
                                             Q4<R> sqr, V3<R> dqsl, V3<R> dqsa, R k_alpha, Block6<R>& B) {
    primal_row_core<P, R>(w.rs[r], w.rd[r], oth, fetch, sqr, dqsl, dqsa, k_alpha, B);
}
// The rows of a body read from the world's current row duals.
struct RowsFromWorld {
    template <class P, class R, class F>
    __device__ __forceinline__ void operator()(const DevWorld<P, R>& w, uint32_t i, uint32_t r, uint32_t oth,
                                               const F& fetch, Q4<R> sqr, V3<R> dqsl, V3<R> dqsa, R k_alpha,
                                               Block6<R>& B) const {
        primal_row_f(w, r, oth, fetch, sqr, dqsl, dqsa, k_alpha, B);
    }
};

template <class P, class R>
__device__ __forceinline__ void primal_row(const DevWorld<P, R>& w, uint32_t r, uint32_t oth, int rd, Q4<R> sqr,
                                           V3<R> dqsl, V3<R> dqsa, R k_alpha, Block6<R>& B) {
    primal_row_f(w, r, oth, GlobalFetch<P, R>{w, rd}, sqr, dqsl, dqsa, k_alpha, B);
}

// One joint seen from body i (avbd/src/lib.rs:425-537).
template <class P, class R>
__device__ __forceinline__ void primal_joint(const DevWorld<P, R>& w, const DioConstraint& jt, uint32_t i, int rd,
                                             V3<P> sp, Q4<P> sq, Q4<R> sqr, Block6<R>& B) {
    const bool is_a = jt.a == i;
    V3<R> anc_a{R(jt.anchor_a[0]), R(jt.anchor_a[1]), R(jt.anchor_a[2])};
    V3<R> anc_b{R(jt.anchor_b[0]), R(jt.anchor_b[1]), R(jt.anchor_b[2])};
    V3<P> pa = is_a ? sp : xyz(w.pos[rd][jt.a]);
    V3<P> pb = !is_a ? sp : xyz(w.pos[rd][jt.b]);
    Q4<P> qa = is_a ? sq : quat(w.rot[rd][jt.a]);
    Q4<P> qb = !is_a ? sq : quat(w.rot[rd][jt.b]);
    V3<P> wpa = add(pa, rotate(qa, cast3<P>(anc_a)));
    V3<P> wpb = add(pb, rotate(qb, cast3<P>(anc_b)));
    V3<R> self_anchor = is_a ? anc_a : anc_b;
    R sign = is_a ? R(1) : R(-1);
    V3<R> delta = cast3<R>(sub(wpa, wpb));
    V3<R> r_self = rotate(sqr, self_anchor);
    R stiff = R(jt.anchor_b[3]);
    if (jt.kind == DIO_CONSTRAINT_BALL_SOCKET) {
        V3<R> jx = scale(V3<R>{R(1), R(0), R(0)}, sign);
        V3<R> jy = scale(V3<R>{R(0), R(1), R(0)}, sign);
        V3<R> jz = scale(V3<R>{R(0), R(0), R(1)}, sign);
        stamp(B, jx, cross(r_self, jx), stiff, delta.x * stiff);
        stamp(B, jy, cross(r_self, jy), stiff, delta.y * stiff);
        stamp(B, jz, cross(r_self, jz), stiff, delta.z * stiff);
    } else {
        R len = length(delta);
        R target = R(jt.anchor_a[3]);
        bool active = len > R(1.0e-6) && (jt.kind != DIO_CONSTRAINT_ROPE || len > target);
        if (active) {
            const Divisor<R> dl(len);  // the IEEE quotients (div_rn.cuh)
            const V3<R> nn{dl.div(delta.x), dl.div(delta.y), dl.div(delta.z)};
            V3<R> jl = scale(nn, sign);
            V3<R> ja = cross(r_self, jl);
            stamp(B, jl, ja, stiff, stiff * (len - target));
        }
    }
}

// The same joint row from a JView: p_a - p_b is formed exactly as the
// reference forms it (joint a's anchor point minus joint b's).  `op4`/`oq4`
// are the other body's snapshot pose, loaded by the caller.
template <class P, class R>
__device__ __forceinline__ void primal_jview_p(const JView& jv, A4<P> op4, A4<P> oq4, V3<P> sp, Q4<P> sq,
                                               Q4<R> sqr, Block6<R>& B) {
    const bool is_a = !(jv.kind & kIsB);
    const uint32_t kind = jv.kind & ~kIsB;
    const V3<R> anc_s{R(jv.self_anchor.x), R(jv.self_anchor.y), R(jv.self_anchor.z)};
    const V3<R> anc_o{R(jv.other_anchor.x), R(jv.other_anchor.y), R(jv.other_anchor.z)};
    const V3<R> r_self = rotate(sqr, anc_s);
    V3<R> delta;  // joint a's anchor point minus joint b's
    if constexpr (std::is_same<P, R>::value) {
        const V3<P> p_self = add(sp, r_self);
        const V3<P> p_other = add(xyz(op4), rotate(quat(oq4), anc_o));
        delta = is_a ? sub(p_self, p_other) : sub(p_other, p_self);
    } else {
        // split mode: the position difference in P, the anchor offsets (small
        // body-frame vectors) rotated and differenced in R
        const V3<R> r_other = rotate(castq<R>(quat(oq4)), anc_o);
        delta = is_a ? add(cast3<R>(sub(sp, xyz(op4))), sub(r_self, r_other))
                     : add(cast3<R>(sub(xyz(op4), sp)), sub(r_other, r_self));
    }
    const R sign = is_a ? R(1) : R(-1);
    const R stiff = R(jv.other_anchor.w);
    if (kind == DIO_CONSTRAINT_BALL_SOCKET) {
        V3<R> jx = scale(V3<R>{R(1), R(0), R(0)}, sign);
        V3<R> jy = scale(V3<R>{R(0), R(1), R(0)}, sign);
        V3<R> jz = scale(V3<R>{R(0), R(0), R(1)}, sign);
        if (finite_(stiff * (dabs(r_self.x) + dabs(r_self.y) + dabs(r_self.z)))) {
            stamp_masked<kMaskAxisX>(B, jx, cross(r_self, jx), stiff, delta.x * stiff);
            stamp_masked<kMaskAxisY>(B, jy, cross(r_self, jy), stiff, delta.y * stiff);
            stamp_masked<kMaskAxisZ>(B, jz, cross(r_self, jz), stiff, delta.z * stiff);
        } else {
            stamp(B, jx, cross(r_self, jx), stiff, delta.x * stiff);
            stamp(B, jy, cross(r_self, jy), stiff, delta.y * stiff);
            stamp(B, jz, cross(r_self, jz), stiff, delta.z * stiff);
        }
    } else {
        R len = length(delta);
        R target = R(jv.self_anchor.w);
        bool active = len > R(1.0e-6) && (kind != DIO_CONSTRAINT_ROPE || len > target);
        if (active) {
            const Divisor<R> dl(len);  // the IEEE quotients (div_rn.cuh)
            const V3<R> nn{dl.div(delta.x), dl.div(delta.y), dl.div(delta.z)};
            V3<R> jl = scale(nn, sign);
            V3<R> ja = cross(r_self, jl);
            stamp(B, jl, ja, stiff, stiff * (len - target));
        }
    }
}

template <class P, class R, class F>
__device__ __forceinline__ void primal_jview_f(const JView& jv, const F& fetch, V3<P> sp, Q4<P> sq, Q4<R> sqr,
                                               Block6<R>& B) {
    primal_jview_p<P, R>(jv, fetch.pos(jv.other), fetch.rot(jv.other), sp, sq, sqr, B);
}

// The inertial start of body i's 6x6 system: diagonal M/dt^2, I/dt^2 and
// the gradient toward the inertial pose.
template <class P, class R>
__device__ __forceinline__ void primal_inertia(const DevWorld<P, R>& w, uint32_t i, const A4<R>& inv, V3<P> sp,
                                               Q4<R> sqr, const SolveParams<R>& o, Block6<R>& B) {
    R mdt2;
    V3<R> idt2;
    if (w.mdt2) {
        const A4<R> d = w.mdt2[i];  // stored by init: the same divisions, once per step
        mdt2 = d.x;
        idt2 = V3<R>{d.y, d.z, d.w};
    } else {
        const R mass = R(1) / inv.w;
        const V3<R> moment{R(1) / inv.x, R(1) / inv.y, R(1) / inv.z};
        const R dt2 = o.dt * o.dt;
        mdt2 = mass / dt2;
        idt2 = divs(moment, dt2);
    }
#pragma unroll
    for (int k = 0; k < 21; ++k) B.h[k] = R(0);
    B.h[tri(0, 0)] = mdt2;
    B.h[tri(1, 1)] = mdt2;
    B.h[tri(2, 2)] = mdt2;
    B.h[tri(3, 3)] = idt2.x;
    B.h[tri(4, 4)] = idt2.y;
    B.h[tri(5, 5)] = idt2.z;
    const V3<R> rl = mulv(V3<R>{mdt2, mdt2, mdt2}, cast3<R>(sub(sp, xyz(w.inert_pos[i]))));
    const V3<R> ra = mulv(idt2, ang_diff(sqr, castq<R>(quat(w.inert_rot[i]))));
    B.g[0] = rl.x;
    B.g[1] = rl.y;
    B.g[2] = rl.z;
    B.g[3] = ra.x;
    B.g[4] = ra.y;
    B.g[5] = ra.z;
}

// Joint rows, the 6x6 solve and the pose update of body i (the tail of
// avbd_primal)
template <class P, class R, class F>
__device__ __forceinline__ void primal_finish(const DevWorld<P, R>& w, uint32_t i, uint32_t k0, uint32_t k1,
                                              const F& fetch, V3<P> sp, Q4<P> sq, Q4<R> sqr, Block6<R>& B) {
    for (uint32_t k = k0; k < k1; ++k) {
        const JView jv = w.jview[k];
        primal_jview_f<P, R>(jv, fetch, sp, sq, sqr, B);
    }
    R dx[6];
    solve6(B, dx);
    const A4<P> np = pack(add(sp, cast3<P>(V3<R>{dx[0], dx[1], dx[2]})));
    if constexpr (std::is_same<P, R>::value)
        fetch.store(i, np, packq(quat_step(sq, V3<P>{dx[3], dx[4], dx[5]})));
    else
        fetch.store(i, np, packq(quat_step_split<P, R>(sq, V3<R>{dx[3], dx[4], dx[5]})));
}

// avbd_primal for one body: reads the snapshot through `fetch` and stores
// the new pose through it.  [k0, k1) is the body's joint-view range.
template <class P, class R, class F, class Rows = RowsFromWorld>
__device__ __forceinline__ void primal_body_f(const DevWorld<P, R>& w, uint32_t i, uint32_t k0, uint32_t k1,
                                              const SolveParams<R>& o, const F& fetch, const Rows& rows = Rows()) {
    const A4<R> inv = w.inv[i];
    if (inv.w == R(0)) return;
    const V3<P> sp = xyz(fetch.pos(i));
    const Q4<P> sq = quat(fetch.rot(i));
    const Q4<R> sqr = castq<R>(sq);
    Block6<R> B;
    primal_inertia(w, i, inv, sp, sqr, o, B);
    const uint32_t j0 = w.row_off[i], j1 = w.row_off[i + 1];
    if (j0 < j1) {
        // displacement since the step start: read only by contact rows
        const V3<R> dqsl = cast3<R>(sub(sp, xyz(fetch.ipos(i))));
        const V3<R> dqsa = ang_diff(sqr, castq<R>(quat(fetch.irot(i))));
        const R k_alpha = R(1) - o.alpha;
        for (uint32_t j = j0; j < j1; ++j) rows(w, i, w.row_idx[j], w.row_oth[j], fetch, sqr, dqsl, dqsa, k_alpha, B);
    }
    primal_finish(w, i, k0, k1, fetch, sp, sq, sqr, B);
}

template <class P, class R>
__device__ __forceinline__ void primal_body(const DevWorld<P, R>& w, uint32_t i, int rd, const SolveParams<R>& o) {
    const uint32_t k0 = w.n_joints ? w.joint_off[i] : 0u, k1 = w.n_joints ? w.joint_off[i + 1] : 0u;
    primal_body_f(w, i, k0, k1, o, GlobalFetch<P, R>{w, rd});
}

// Tile variant: the CTA's T consecutive bodies stage their snapshot and
// step-start poses in shared memory; neighbours inside the tile (chain links,
// nearby boxes) are read from there.  Jacobi only (buffer rd is read-only
// during the launch).
template <class P, class R, int T, int MINB>
__global__ void __launch_bounds__(T, MINB) k_primal_tile(DevWorld<P, R> w, int rd, int wr, SolveParams<R> o) {
    __shared__ A4<P> s_pos[T], s_rot[T], s_ipos[T], s_irot[T];
    pdl_enter();
    const uint32_t lo = blockIdx.x * T;
    const uint32_t i = lo + threadIdx.x;
    if (i < w.n) {
        s_pos[threadIdx.x] = w.pos[rd][i];
        s_rot[threadIdx.x] = w.rot[rd][i];
        s_ipos[threadIdx.x] = w.init_pos[i];
        s_irot[threadIdx.x] = w.init_rot[i];
    }
    __syncthreads();
    if (i < w.n) {
        const uint32_t k0 = w.n_joints ? w.joint_off[i] : 0u, k1 = w.n_joints ? w.joint_off[i + 1] : 0u;
        primal_body_f(w, i, k0, k1, o, TileFetch<P, R, T>{w, rd, lo, s_pos, s_rot, s_ipos, s_irot});
    }
}

// One thread per dynamic body (static bodies are never solved,
// avbd/src/lib.rs:280-282, so they are left out of the launch).
// BLOCK threads per CTA, at least MINB CTAs per SM (a register bound); the
// variants are chosen per world by the autotuner.
template <class P, class R, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) k_primal(DevWorld<P, R> w, int rd, int wr, SolveParams<R> o) {
    pdl_enter();
    for (uint32_t t = blockIdx.x * BLOCK + threadIdx.x; t < w.n_dyn; t += gridDim.x * BLOCK)
        primal_body(w, w.dyn_list[t], rd, o);
}

// Warp per dynamic body, for worlds whose bodies carry many contact rows
// (a thread per body walks its rows one dependent gather after another):
// lane l forms the three stamps of the body's incidence j0 + 32 q + l and
// writes their 27 products each (21 Hessian terms, 6 gradient terms, the
// products exactly as stamp() forms them) to shared memory; lane e < 27 then
// adds entry e of the 6x6 system over the incidences and stamps in the
// serial order -- the same sums, term for term, as primal_body_f.  Lane 0
// adds the joint rows and solves.
constexpr int kPrimalWarpWarps = 4;
template <class R>
__host__ __device__ constexpr size_t primal_warp_smem() {
    return (size_t)kPrimalWarpWarps * 32 * 3 * 28 * sizeof(R);
}
// One body's primal by the calling warp (all 32 lanes, the same i);
// prod: the warp's [32][3][28] product staging in shared memory.
template <class P, class R, class F>
__device__ __forceinline__ void primal_warp_body(const DevWorld<P, R>& w, uint32_t i, const SolveParams<R>& o,
                                                 const F& fetch, R* prod, uint32_t lane) {
    const A4<R> inv = w.inv[i];
    if (inv.w == R(0)) return;  // warp-uniform
    const V3<P> sp = xyz(fetch.pos(i));
    const Q4<P> sq = quat(fetch.rot(i));
    const Q4<R> sqr = castq<R>(sq);
    Block6<R> B;
    primal_inertia(w, i, inv, sp, sqr, o, B);
    // lane e holds entry e: h[0..20], then g[0..5]
    R acc = R(0);
#pragma unroll
    for (int e = 0; e < 21; ++e)
        if (lane == (uint32_t)e) acc = B.h[e];
#pragma unroll
    for (int e = 0; e < 6; ++e)
        if (lane == (uint32_t)(21 + e)) acc = B.g[e];
    const uint32_t j0 = w.row_off[i], j1 = w.row_off[i + 1];
    if (j0 < j1) {
        const V3<R> dqsl = cast3<R>(sub(sp, xyz(fetch.ipos(i))));
        const V3<R> dqsa = ang_diff(sqr, castq<R>(quat(fetch.irot(i))));
        const R k_alpha = R(1) - o.alpha;
        for (uint32_t base = j0; base < j1; base += 32u) {
            const uint32_t cnt = min(32u, j1 - base);
            if (lane < cnt) {
                const uint32_t j = base + lane;
                const uint32_t r = w.row_idx[j];
                V3<R> jl[3], ja[3];
                R k[3], f[3];
                primal_row_terms<P, R>(w.rs[r], w.rd[r], w.row_oth[j], fetch, sqr, dqsl, dqsa, k_alpha, jl, ja, k,
                                       f);
                R* mine = prod + lane * (3 * 28);
#pragma unroll
                for (int s = 0; s < 3; ++s) {
                    const R J[6] = {jl[s].x, jl[s].y, jl[s].z, ja[s].x, ja[s].y, ja[s].z};
#pragma unroll
                    for (int a = 0; a < 6; ++a)
#pragma unroll
                        for (int b = 0; b <= a; ++b) mine[s * 28 + tri(a, b)] = J[a] * J[b] * k[s];
#pragma unroll
                    for (int a = 0; a < 6; ++a) mine[s * 28 + 21 + a] = J[a] * f[s];
                }
            }
            __syncwarp();
            if (lane < 27u)
                for (uint32_t q = 0; q < cnt; ++q) {
                    const R* pq = prod + q * (3 * 28) + lane;
                    acc = acc + pq[0];
                    acc = acc + pq[28];
                    acc = acc + pq[56];
                }
            __syncwarp();
        }
    }
#pragma unroll
    for (int e = 0; e < 21; ++e) B.h[e] = __shfl_sync(0xFFFFFFFFu, acc, e);
#pragma unroll
    for (int e = 0; e < 6; ++e) B.g[e] = __shfl_sync(0xFFFFFFFFu, acc, 21 + e);
    if (lane == 0u) {
        const uint32_t k0 = w.n_joints ? w.joint_off[i] : 0u, k1 = w.n_joints ? w.joint_off[i + 1] : 0u;
        primal_finish(w, i, k0, k1, fetch, sp, sq, sqr, B);
    }
}

template <class P, class R>
__global__ void __launch_bounds__(kPrimalWarpWarps * 32) k_primal_warp(DevWorld<P, R> w, int rd, int wr,
                                                                        SolveParams<R> o) {
    pdl_enter();
    extern __shared__ __align__(16) unsigned char primal_warp_smem_raw[];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    R* prod = reinterpret_cast<R*>(primal_warp_smem_raw) + (size_t)warp * 32 * 3 * 28;  // [32][3][28]
    const GlobalFetch<P, R> fetch{w, rd};
    const uint32_t nwarps = gridDim.x * kPrimalWarpWarps;
    for (uint32_t t = blockIdx.x * kPrimalWarpWarps + warp; t < w.n_dyn; t += nwarps)
        primal_warp_body(w, w.dyn_list[t], o, fetch, prod, lane);
}

// variants: 0-5 k_primal over the dynamic-body list with {threads per CTA,
// min CTAs per SM}; 6-9 k_primal_tile over body tiles; 10 k_primal_warp
constexpr int kPrimalVariants = DIO_PRIMAL_VARIANTS;
constexpr int kPrimalShape[kPrimalVariants][2] = {{128, 4}, {128, 5}, {128, 6}, {256, 2}, {256, 3},
                                                  {64, 10}, {128, 5}, {128, 6}, {256, 3}, {64, 10},
                                                  {kPrimalWarpWarps * 32, 1}};

template <class P, class R>
inline void launch_primal(int variant, bool pdl, const DevWorld<P, R>& w, int rd, int wr, const SolveParams<R>& o,
                          cudaStream_t s) {
    const uint32_t nd = w.n_dyn > 0 ? w.n_dyn : 1;
    auto grid = [&](int block) { return grid_for(nd, block); };
    switch (variant) {
        case 0:
            launch_k(pdl, k_primal<P, R, 128, 4>, grid(128), 128, 0, s, w, rd, wr, o);
            break;
        case 2:
            launch_k(pdl, k_primal<P, R, 128, 6>, grid(128), 128, 0, s, w, rd, wr, o);
            break;
        case 3:
            launch_k(pdl, k_primal<P, R, 256, 2>, grid(256), 256, 0, s, w, rd, wr, o);
            break;
        case 4:
            launch_k(pdl, k_primal<P, R, 256, 3>, grid(256), 256, 0, s, w, rd, wr, o);
            break;
        case 5:
            launch_k(pdl, k_primal<P, R, 64, 10>, grid(64), 64, 0, s, w, rd, wr, o);
            break;
        case 6:
            launch_k(pdl, k_primal_tile<P, R, 128, 5>, grid_for(w.n, 128), 128, 0, s, w, rd, wr, o);
            break;
        case 7:
            launch_k(pdl, k_primal_tile<P, R, 128, 6>, grid_for(w.n, 128), 128, 0, s, w, rd, wr, o);
            break;
        case 8:
            launch_k(pdl, k_primal_tile<P, R, 256, 3>, grid_for(w.n, 256), 256, 0, s, w, rd, wr, o);
            break;
        case 9:
            launch_k(pdl, k_primal_tile<P, R, 64, 10>, grid_for(w.n, 64), 64, 0, s, w, rd, wr, o);
            break;
        case 10:
            launch_k(pdl, k_primal_warp<P, R>, grid_for(nd, kPrimalWarpWarps), kPrimalWarpWarps * 32,
                     primal_warp_smem<R>(), s, w, rd, wr, o);
            break;
        default:
            launch_k(pdl, k_primal<P, R, 128, 5>, grid(128), 128, 0, s, w, rd, wr, o);
            break;
    }
}

// Buffer 0 read and written in place (the coloured Gauss-Seidel sweeps).
template <class P, class R>
struct InPlaceFetch {
    const DevWorld<P, R>& w;
    __device__ __forceinline__ A4<P> pos(uint32_t j) const { return w.pos[0][j]; }
    __device__ __forceinline__ A4<P> rot(uint32_t j) const { return w.rot[0][j]; }
    __device__ __forceinline__ A4<P> ipos(uint32_t j) const { return w.init_pos[j]; }
    __device__ __forceinline__ A4<P> irot(uint32_t j) const { return w.init_rot[j]; }
    __device__ __forceinline__ void store(uint32_t i, A4<P> p, A4<P> q) const {
        w.pos[0][i] = p;
        w.rot[0][i] = q;
    }
};

// Coloured Gauss-Seidel sweep: bodies color_order[c0 .. c1) in place.
template <class P, class R>
__global__ void __launch_bounds__(128) k_primal_color(DevWorld<P, R> w, uint32_t c0, uint32_t c1, SolveParams<R> o) {
    for (uint32_t t = c0 + blockIdx.x * blockDim.x + threadIdx.x; t < c1; t += gridDim.x * blockDim.x) {
        const uint32_t i = w.color_order[t];
        const uint32_t k0 = w.n_joints ? w.joint_off[i] : 0u, k1 = w.n_joints ? w.joint_off[i + 1] : 0u;
        primal_body_f(w, i, k0, k1, o, InPlaceFetch<P, R>{w});
    }
}

// The same sweep with a warp per body (primal variant 10)
template <class P, class R>
__global__ void __launch_bounds__(kPrimalWarpWarps * 32)
    k_primal_color_warp(DevWorld<P, R> w, uint32_t c0, uint32_t c1, SolveParams<R> o) {
    extern __shared__ __align__(16) unsigned char primal_warp_smem_raw[];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    R* prod = reinterpret_cast<R*>(primal_warp_smem_raw) + (size_t)warp * 32 * 3 * 28;
    const InPlaceFetch<P, R> fetch{w};
    for (uint32_t t = c0 + blockIdx.x * kPrimalWarpWarps + warp; t < c1; t += gridDim.x * kPrimalWarpWarps)
        primal_warp_body(w, w.color_order[t], o, fetch, prod, lane);
}

// avbd_dual, avbd/src/lib.rs:565-663: the row's dual update from its bodies' new poses (a, and b unless the
// row is against a container) and step-start poses.
template <class P, class R>
__device__ __forceinline__ RowDual<P, R> dual_update(const RowStatic<R>& rs, RowDual<P, R> du, A4<P> pa4, A4<P> qa4,
                                                     A4<P> ia_p, A4<P> ia_q, bool has_b, A4<P> pb4, A4<P> qb4,
                                                     A4<P> ib_p, A4<P> ib_q, const SolveParams<R>& o) {
    V3<R> dal = cast3<R>(sub(xyz(pa4), xyz(ia_p)));
    V3<R> daa = ang_diff(castq<R>(quat(qa4)), castq<R>(quat(ia_q)));
    V3<R> dbl{R(0), R(0), R(0)}, dba{R(0), R(0), R(0)}, rbw{R(0), R(0), R(0)};
    if (has_b) {
        dbl = cast3<R>(sub(xyz(pb4), xyz(ib_p)));
        dba = ang_diff(castq<R>(quat(qb4)), castq<R>(quat(ib_q)));
        rbw = rotate(castq<R>(quat(qb4)), xyz(rs.rb));
    }
    V3<R> raw = rotate(castq<R>(quat(qa4)), xyz(rs.ra));
    V3<R> r0 = xyz(rs.n), r1 = xyz(rs.t1), r2 = xyz(rs.t2);
    const R k_alpha = R(1) - o.alpha;
    R c0 = rs.ra.w * k_alpha, c1 = rs.rb.w * k_alpha, c2 = rs.t1.w * k_alpha;
    c0 = c0 + (dot(r0, dal) + dot(cross(raw, r0), daa) - dot(r0, dbl) - dot(cross(rbw, r0), dba));
    c1 = c1 + (dot(r1, dal) + dot(cross(raw, r1), daa) - dot(r1, dbl) - dot(cross(rbw, r1), dba));
    c2 = c2 + (dot(r2, dal) + dot(cross(raw, r2), daa) - dot(r2, dbl) - dot(cross(rbw, r2), dba));
    P f0, f1, f2, tm, bounds;
    row_forces(du, rs.n.w, c0, c1, c2, f0, f1, f2, tm, bounds);
    du.lambda.x = f0;
    du.lambda.y = f1;
    du.lambda.z = f2;
    if (f0 < P(0)) du.penalty.x = fmin_(du.penalty.x + o.beta_lin * dabs(c0), o.penalty_max);
    if (tm <= bounds) {
        du.penalty.y = fmin_(du.penalty.y + o.beta_lin * dabs(c1), o.penalty_max);
        du.penalty.z = fmin_(du.penalty.z + o.beta_lin * dabs(c2), o.penalty_max);
    }
    return du;
}
// avbd_dual, avbd/src/lib.rs:565-663, for row c of `rd`: new duals into
// `out`; `fetch` reads the new state.
template <class P, class R, class F>
__device__ __forceinline__ void dual_row_io(const DevWorld<P, R>& w, uint32_t c, const F& fetch,
                                            const RowDual<P, R>* rd, RowDual<P, R>* out, const SolveParams<R>& o) {
    const uint2 ab = w.ab[c];
    const bool has_b = ab.y != kContainer;
    const uint32_t b = has_b ? ab.y : ab.x;
    out[c] = dual_update<P, R>(w.rs[c], rd[c], fetch.pos(ab.x), fetch.rot(ab.x), fetch.ipos(ab.x),
                               fetch.irot(ab.x), has_b, fetch.pos(b), fetch.rot(b), fetch.ipos(b), fetch.irot(b), o);
}
template <class P, class R, class F>
__device__ __forceinline__ void dual_row_f(const DevWorld<P, R>& w, uint32_t c, const F& fetch,
                                           const SolveParams<R>& o) {
    dual_row_io(w, c, fetch, w.rd, w.rd, o);
}
template <class P, class R>
__device__ __forceinline__ void dual_row(const DevWorld<P, R>& w, uint32_t c, int rd, const SolveParams<R>& o) {
    dual_row_f(w, c, GlobalFetch<P, R>{w, rd}, o);
}

template <class P, class R>
__global__ void __launch_bounds__(256) k_dual(DevWorld<P, R> w, uint32_t lo, uint32_t hi, const uint32_t* dyn_hi,
                                              int rd, SolveParams<R> o) {
    pdl_enter();
    uint32_t end = dyn_hi ? *dyn_hi : hi;
    for (uint32_t c = lo + blockIdx.x * blockDim.x + threadIdx.x; c < end; c += gridDim.x * blockDim.x)
        dual_row(w, c, rd, o);
}

// avbd_recover, avbd/src/lib.rs:667-699; also leaves the final pose in
// buffer 0 when it lives in buffer 1.
template <class P, class R, class F>
__device__ __forceinline__ void recover_body_f(const DevWorld<P, R>& w, uint32_t i, const F& fetch,
                                               const SolveParams<R>& o) {
    if (w.inv[i].w == R(0)) return;
    A4<P> p4 = fetch.pos(i);
    A4<P> q4 = fetch.rot(i);
    P dt = P(o.dt);
    A4<P> v = w.vel[i];
    w.prev_vel[i] = v;
    const Q4<P> rel = qmul(quat(q4), conj(quat(fetch.irot(i))));
    V3<P> nv, na;
    if constexpr (std::is_same<P, R>::value) {
        nv = divs(sub(xyz(p4), xyz(fetch.ipos(i))), dt);
        na = divs(V3<P>{P(2) * rel.x, P(2) * rel.y, P(2) * rel.z}, dt);
    } else {  // split mode: one division, then products (within an ulp of P)
        const P inv_dt = P(1) / dt;
        nv = scale(sub(xyz(p4), xyz(fetch.ipos(i))), inv_dt);
        na = scale(V3<P>{P(2) * rel.x, P(2) * rel.y, P(2) * rel.z}, inv_dt);
    }
    w.vel[i] = pack(nv);
    w.ang[i] = pack(na);
    // a non-finite pose or velocity is reported (DIO_ERR_NONFINITE), as the
    // reference demos' constraint tracing reports it (demos/constraints/src/main.rs:24-60)
    if (w.ctr && !(finite_(nv.x) && finite_(nv.y) && finite_(nv.z) && finite_(na.x) && finite_(na.y) &&
                   finite_(na.z) && finite_(q4.w)))
        atomicOr(&w.ctr->error_flags, kErrNonFinite);
}
template <class P, class R>
__device__ __forceinline__ void recover_body(const DevWorld<P, R>& w, uint32_t i, int rb, const SolveParams<R>& o) {
    recover_body_f(w, i, GlobalFetch<P, R>{w, rb}, o);
}

template <class P, class R>
__global__ void __launch_bounds__(256) k_recover(DevWorld<P, R> w, uint32_t lo, uint32_t hi, int rb, int final_buf,
                                                 SolveParams<R> o) {
    pdl_enter();
    for (uint32_t i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += gridDim.x * blockDim.x) {
        recover_body(w, i, rb, o);
        if (final_buf != 0) {
            w.pos[0][i] = w.pos[final_buf][i];
            w.rot[0][i] = w.rot[final_buf][i];
        }
    }
}

}  // namespace dio
