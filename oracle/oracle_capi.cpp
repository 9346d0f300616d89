// oracle_capi.cpp -- extern "C" surface of the CPU oracle (TEST INFRASTRUCTURE).
//
// Exposes the restated reference algorithm (dio_oracle.hpp) with the same
// record layouts as include/dio_cuda.h so tests can feed identical bytes to
// the oracle and to the CUDA library.  Only tests, the smoke check and the
// CPU-baseline leg of bench.py load this library.
#include <cstdio>
#include <cstring>
#include <memory>

#include "../include/dio_cuda.h"
#include "dio_oracle.hpp"

using namespace dio_oracle;

namespace {

template <class R>
Shape<R> to_shape(const DioShape& s) {
    Shape<R> o;
    o.tag = s.tag;
    o.hull_first = s.pad[0];
    o.hull_count = s.pad[1];
    for (int i = 0; i < 4; ++i) o.c[i] = {R(s.corners[i][0]), R(s.corners[i][1]), R(s.corners[i][2])};
    return o;
}

template <class R>
NBody<R> to_nbody(const DioGpuBody& b) {
    NBody<R> o;
    o.pos = {R(b.position[0]), R(b.position[1]), R(b.position[2])};
    o.rot = {R(b.orientation[0]), R(b.orientation[1]), R(b.orientation[2]), R(b.orientation[3])};
    o.shape = to_shape<R>(b.shape);
    return o;
}

template <class R>
std::vector<V3<R>> to_hull(const float* h, uint32_t n) {
    std::vector<V3<R>> o(n);
    for (uint32_t i = 0; i < n; ++i) o[i] = {R(h[4 * i]), R(h[4 * i + 1]), R(h[4 * i + 2])};
    return o;
}

template <class R>
Options<R> to_options(const DioAvbdOptions& o) {
    Options<R> r;
    r.dt = R(o.dt);
    r.gravity = {R(o.gravity[0]), R(o.gravity[1]), R(o.gravity[2])};
    r.iterations = o.iterations;
    r.alpha = R(o.alpha);
    r.beta_lin = R(o.beta_lin);
    r.margin = R(o.margin);
    r.penalty_min = R(o.penalty_min);
    r.penalty_max = R(o.penalty_max);
    r.gamma = R(o.gamma);
    r.friction = R(o.friction);
    return r;
}

template <class P, class R>
Row<P, R> to_row(const DioContact& c) {
    Row<P, R> r;
    r.a = c.a;
    r.b = c.b;
    r.friction = R(c.friction);
    auto v = [](const float* f) { return V3<R>{R(f[0]), R(f[1]), R(f[2])}; };
    r.n = v(c.normal);
    r.t1 = v(c.tangent1);
    r.t2 = v(c.tangent2);
    r.ra = v(c.r_a);
    r.rb = v(c.r_b);
    r.c0 = v(c.c0);
    r.penalty = v(c.penalty);
    r.lambda = {P(c.lambda[0]), P(c.lambda[1]), P(c.lambda[2])};
    return r;
}

template <class P, class R>
DioContact from_row(const Row<P, R>& r) {
    DioContact c;
    std::memset(&c, 0, sizeof c);
    c.a = r.a;
    c.b = r.b;
    c.friction = float(r.friction);
    auto put = [](float* f, V3<R> v) {
        f[0] = float(v.x);
        f[1] = float(v.y);
        f[2] = float(v.z);
        f[3] = 0.f;
    };
    put(c.normal, r.n);
    put(c.tangent1, r.t1);
    put(c.tangent2, r.t2);
    put(c.r_a, r.ra);
    put(c.r_b, r.rb);
    put(c.c0, r.c0);
    put(c.penalty, r.penalty);
    c.lambda[0] = float(r.lambda.x);
    c.lambda[1] = float(r.lambda.y);
    c.lambda[2] = float(r.lambda.z);
    return c;
}

template <class P, class R>
BodyState<P, R> to_state(const DioBodyState& s) {
    BodyState<P, R> o;
    o.vel = {P(s.vel[0]), P(s.vel[1]), P(s.vel[2])};
    o.ang = {P(s.ang[0]), P(s.ang[1]), P(s.ang[2])};
    o.prev_vel = {P(s.prev_vel[0]), P(s.prev_vel[1]), P(s.prev_vel[2])};
    o.inv_moment = {R(s.inv_moment[0]), R(s.inv_moment[1]), R(s.inv_moment[2])};
    o.inv_mass = R(s.inv_mass);
    o.friction = R(s.friction);
    return o;
}

template <class R>
Joint<R> to_joint(const DioConstraint& c) {
    Joint<R> j;
    j.a = c.a;
    j.b = c.b;
    j.kind = c.kind;
    j.anchor_a = {R(c.anchor_a[0]), R(c.anchor_a[1]), R(c.anchor_a[2])};
    j.aw = R(c.anchor_a[3]);
    j.anchor_b = {R(c.anchor_b[0]), R(c.anchor_b[1]), R(c.anchor_b[2])};
    j.bw = R(c.anchor_b[3]);
    return j;
}

template <class R>
Container<R> to_container(const DioContainer& c) {
    Container<R> o;
    o.center = {R(c.center[0]), R(c.center[1]), R(c.center[2])};
    o.rotation = {R(c.rotation[0]), R(c.rotation[1]), R(c.rotation[2]), R(c.rotation[3])};
    o.half_extent = R(c.half_extent);
    return o;
}

// ------------------------------------------------------------------ world
struct WorldBase {
    virtual ~WorldBase() = default;
    virtual void step(const DioAvbdOptions& o, uint32_t steps) = 0;
    virtual void download(DioGpuBody* b, DioBodyState* s) = 0;
    virtual void download_f64(double* p, double* q) = 0;
    virtual uint32_t contacts(DioContact* out, uint32_t cap) = 0;
    virtual uint32_t colors(uint32_t* out, uint32_t cap) = 0;
    virtual void stats(DioStepStats* s) = 0;
    virtual void set_lag(bool on) = 0;
    uint64_t steps_done = 0;
};

template <class P, class R>
struct WorldT : WorldBase {
    World<P, R> w;
    // switching the lag on starts from no previous detection
    void set_lag(bool on) override {
        if (on && !w.lag) w.prev_slots.clear();
        w.lag = on;
    }
    std::vector<DioShape> raw_shapes;
    void step(const DioAvbdOptions& o, uint32_t steps) override {
        Options<R> opt = to_options<R>(o);
        for (uint32_t k = 0; k < steps; ++k) w.step(opt);
        steps_done += steps;
    }
    void download(DioGpuBody* b, DioBodyState* s) override {
        for (uint32_t i = 0; i < w.n(); ++i) {
            if (b) {
                b[i].position[0] = float(w.pos[i].x);
                b[i].position[1] = float(w.pos[i].y);
                b[i].position[2] = float(w.pos[i].z);
                b[i].position[3] = 0.f;
                b[i].orientation[0] = float(w.rot[i].x);
                b[i].orientation[1] = float(w.rot[i].y);
                b[i].orientation[2] = float(w.rot[i].z);
                b[i].orientation[3] = float(w.rot[i].w);
                b[i].shape = raw_shapes[i];
            }
            if (s) {
                const auto& st = w.state[i];
                auto put = [](float* f, V3<P> v) {
                    f[0] = float(v.x);
                    f[1] = float(v.y);
                    f[2] = float(v.z);
                    f[3] = 0.f;
                };
                put(s[i].vel, st.vel);
                put(s[i].ang, st.ang);
                put(s[i].prev_vel, st.prev_vel);
                s[i].inv_moment[0] = float(st.inv_moment.x);
                s[i].inv_moment[1] = float(st.inv_moment.y);
                s[i].inv_moment[2] = float(st.inv_moment.z);
                s[i].inv_moment[3] = 0.f;
                s[i].inv_mass = float(st.inv_mass);
                s[i].friction = float(st.friction);
                s[i].pad[0] = s[i].pad[1] = 0.f;
            }
        }
    }
    void download_f64(double* p, double* q) override {
        for (uint32_t i = 0; i < w.n(); ++i) {
            if (p) {
                p[3 * i] = double(w.pos[i].x);
                p[3 * i + 1] = double(w.pos[i].y);
                p[3 * i + 2] = double(w.pos[i].z);
            }
            if (q) {
                q[4 * i] = double(w.rot[i].x);
                q[4 * i + 1] = double(w.rot[i].y);
                q[4 * i + 2] = double(w.rot[i].z);
                q[4 * i + 3] = double(w.rot[i].w);
            }
        }
    }
    uint32_t contacts(DioContact* out, uint32_t cap) override {
        uint32_t m = uint32_t(w.rows.size());
        for (uint32_t i = 0; i < m && i < cap && out; ++i) out[i] = from_row(w.rows[i]);
        return m;
    }
    uint32_t colors(uint32_t* out, uint32_t cap) override {
        uint32_t n = uint32_t(w.colors.size());
        for (uint32_t i = 0; i < n && i < cap && out; ++i) out[i] = w.colors[i];
        return n;
    }
    void stats(DioStepStats* s) override {
        s->pairs = uint32_t(w.last_pairs);
        s->contacts = uint32_t(w.rows.size());
        s->colors = w.ncolors;
        s->error_flags = w.epa_overflow ? 1u : 0u;
        s->steps = steps_done;
    }
};

template <class P, class R>
WorldBase* make_world(const DioWorldDesc& d, const DioConfig& cfg, int threads) {
    auto* W = new WorldT<P, R>();
    auto& w = W->w;
    uint32_t n = d.n_bodies;
    w.pos.resize(n);
    w.rot.resize(n);
    w.shape.resize(n);
    w.state.resize(n);
    W->raw_shapes.resize(n);
    for (uint32_t i = 0; i < n; ++i) {
        const DioGpuBody& b = d.bodies[i];
        if (d.positions_f64)
            w.pos[i] = {P(d.positions_f64[3 * i]), P(d.positions_f64[3 * i + 1]), P(d.positions_f64[3 * i + 2])};
        else
            w.pos[i] = {P(b.position[0]), P(b.position[1]), P(b.position[2])};
        if (d.orientations_f64)
            w.rot[i] = {P(d.orientations_f64[4 * i]), P(d.orientations_f64[4 * i + 1]),
                        P(d.orientations_f64[4 * i + 2]), P(d.orientations_f64[4 * i + 3])};
        else
            w.rot[i] = {P(b.orientation[0]), P(b.orientation[1]), P(b.orientation[2]), P(b.orientation[3])};
        w.shape[i] = to_shape<R>(b.shape);
        W->raw_shapes[i] = b.shape;
        w.state[i] = to_state<P, R>(d.state[i]);
    }
    for (uint32_t k = 0; k < d.n_constraints; ++k) w.joints.push_back(to_joint<R>(d.constraints[k]));
    uint32_t S = d.n_scenes == 0 ? 1 : d.n_scenes;
    w.scene_off.assign(S + 1, 0);
    if (d.scene_offsets && d.n_scenes > 0)
        for (uint32_t s = 0; s <= S; ++s) w.scene_off[s] = d.scene_offsets[s];
    else
        w.scene_off[1] = n;
    w.containers.resize(S);
    w.has_container.assign(S, 0);
    if (d.containers)
        for (uint32_t s = 0; s < S; ++s) {
            w.containers[s] = to_container<R>(d.containers[s]);
            w.has_container[s] = 1;
        }
    w.hull = to_hull<R>(d.hull_vertices, d.n_hull_vertices);
    w.per_pair = cfg.contacts_per_pair == 8 ? 8 : 4;
    w.colored = cfg.solver_mode == DIO_SOLVER_COLORED;
    w.lag = cfg.contact_lag != 0;
    w.split_rebase = cfg.precision == DIO_PREC_SPLIT;
    w.threads = threads < 1 ? 1 : threads;
    return W;
}

}  // namespace

extern "C" {

int oracle_abi_version() { return 1; }

int oracle_support(const DioShape* shape, const float* dir, const float* hull, uint32_t nh, float* out) {
    auto h = to_hull<float>(hull, nh);
    V3<float> r = support(to_shape<float>(*shape), V3<float>{dir[0], dir[1], dir[2]}, h.empty() ? nullptr : h.data());
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
    return 0;
}

int oracle_aabb(const DioGpuBody* bodies, uint32_t n, const float* hull, uint32_t nh, float* out) {
    auto h = to_hull<float>(hull, nh);
    for (uint32_t i = 0; i < n; ++i) {
        V3<float> mn, mx;
        aabb(to_nbody<float>(bodies[i]), h.empty() ? nullptr : h.data(), mn, mx);
        float* o = out + 8 * i;
        o[0] = mn.x;
        o[1] = mn.y;
        o[2] = mn.z;
        o[3] = 0.f;
        o[4] = mx.x;
        o[5] = mx.y;
        o[6] = mx.z;
        o[7] = 0.f;
    }
    return 0;
}

// Dense (or sort-and-sweep) pair set of bodies [0, n) sorted by (a, b).
// *count receives the full count even when it exceeds cap.
int oracle_broad(const DioGpuBody* bodies, uint32_t n, const float* hull, uint32_t nh, uint32_t use_sap,
                 DioPair* out, uint32_t cap, uint32_t* count) {
    auto h = to_hull<float>(hull, nh);
    std::vector<V3<float>> mn(n), mx(n);
    for (uint32_t i = 0; i < n; ++i) aabb(to_nbody<float>(bodies[i]), h.empty() ? nullptr : h.data(), mn[i], mx[i]);
    std::vector<std::pair<uint32_t, uint32_t>> pairs;
    if (use_sap)
        broad_sap(mn, mx, 0, n, pairs);
    else
        broad_dense(mn, mx, 0, n, pairs);
    *count = uint32_t(pairs.size());
    for (uint32_t i = 0; i < pairs.size() && i < cap; ++i) out[i] = DioPair{pairs[i].first, pairs[i].second};
    return pairs.size() > cap ? DIO_ERR_CAPACITY : 0;
}

int oracle_narrow(const DioGpuBody* bodies, uint32_t n, const DioPair* pairs, uint32_t np, const float* hull,
                  uint32_t nh, uint32_t per_pair, DioContactOut* out) {
    (void)n;
    auto h = to_hull<float>(hull, nh);
    std::vector<Slot<float>> slots(per_pair);
    for (uint32_t p = 0; p < np; ++p) {
        NBody<float> a = to_nbody<float>(bodies[pairs[p].a]);
        NBody<float> b = to_nbody<float>(bodies[pairs[p].b]);
        narrow_pair(a, b, pairs[p].a, pairs[p].b, h.empty() ? nullptr : h.data(), per_pair, slots.data());
        for (uint32_t k = 0; k < per_pair; ++k) {
            DioContactOut& o = out[p * per_pair + k];
            std::memset(&o, 0, sizeof o);
            const Slot<float>& s = slots[k];
            o.valid = s.valid;
            o.a = s.a;
            o.b = s.b;
            o.normal[0] = s.normal.x;
            o.normal[1] = s.normal.y;
            o.normal[2] = s.normal.z;
            o.depth = s.depth;
            o.point_a[0] = s.point_a.x;
            o.point_a[1] = s.point_a.y;
            o.point_a[2] = s.point_a.z;
            o.point_b[0] = s.point_b.x;
            o.point_b[1] = s.point_b.y;
            o.point_b[2] = s.point_b.z;
        }
    }
    return 0;
}

// Mirror of dio_prepare_contacts: decode + raw_contact + container rows +
// finalize_contacts (warm start, decay, CSR).
int oracle_prepare_contacts(const DioGpuBody* bodies, const DioBodyState* state, uint32_t n,
                            const DioContactOut* slots, uint32_t n_slots, const DioContact* prev, uint32_t n_prev,
                            const DioContainer* container, const DioAvbdOptions* options, const float* hull,
                            uint32_t nh, DioContact* out, uint32_t cap, uint32_t* m, uint32_t* offsets,
                            uint32_t* indices, uint32_t index_cap, uint32_t* n_indices) {
    Options<float> o = to_options<float>(*options);
    auto h = to_hull<float>(hull, nh);
    std::vector<NBody<float>> nb(n);
    for (uint32_t i = 0; i < n; ++i) nb[i] = to_nbody<float>(bodies[i]);
    std::vector<Row<float, float>> rows, prow;
    for (uint32_t s = 0; s < n_slots; ++s) {
        const DioContactOut& c = slots[s];
        if (!c.valid) continue;
        if (c.a >= n || c.b >= n) return DIO_ERR_INVALID;
        rows.push_back(raw_contact<float, float>(c.a, c.b, nb[c.a], nb[c.b], {c.normal[0], c.normal[1], c.normal[2]},
                                                 c.depth, {c.point_a[0], c.point_a[1], c.point_a[2]},
                                                 {c.point_b[0], c.point_b[1], c.point_b[2]}, o));
    }
    if (container) {
        Container<float> ct = to_container<float>(*container);
        for (uint32_t i = 0; i < n; ++i)
            if (state[i].inv_mass != 0.f)
                container_contacts<float, float>(ct, nb[i], {state[i].vel[0], state[i].vel[1], state[i].vel[2]}, i,
                                                 h.empty() ? nullptr : h.data(), o, rows);
    }
    for (uint32_t i = 0; i < n_prev; ++i) prow.push_back(to_row<float, float>(prev[i]));
    std::vector<uint32_t> off, idx;
    finalize_contacts(prow, rows, n, o, off, idx);
    *m = uint32_t(rows.size());
    *n_indices = uint32_t(idx.size());
    if (rows.size() > cap || idx.size() > index_cap) return DIO_ERR_CAPACITY;
    for (size_t i = 0; i < rows.size(); ++i) out[i] = from_row(rows[i]);
    for (uint32_t i = 0; i <= n; ++i) offsets[i] = off[i];
    for (size_t i = 0; i < idx.size(); ++i) indices[i] = idx[i];
    return 0;
}

}  // extern "C"

namespace {
template <class P, class R>
int avbd_run_t(const DioBodyState* state, const float* pos, const float* quat, uint32_t n, const DioContact* contacts,
               uint32_t m, const DioConstraint* cons, uint32_t nj, const uint32_t* offsets, const uint32_t* indices,
               const DioRunOptions* ro, uint32_t use_joint_csr, float* out_pos, float* out_rot, float* out_vel,
               float* out_ang, float* out_prev, float* out_lambda, float* out_penalty) {
    AvbdBuffers<P, R> B;
    B.n = n;
    B.state.resize(n);
    B.pos[0].resize(n);
    B.rot[0].resize(n);
    for (uint32_t i = 0; i < n; ++i) {
        B.state[i] = to_state<P, R>(state[i]);
        B.pos[0][i] = {P(pos[3 * i]), P(pos[3 * i + 1]), P(pos[3 * i + 2])};
        B.rot[0][i] = {P(quat[4 * i]), P(quat[4 * i + 1]), P(quat[4 * i + 2]), P(quat[4 * i + 3])};
    }
    std::vector<Row<P, R>> rows(m);
    for (uint32_t i = 0; i < m; ++i) rows[i] = to_row<P, R>(contacts[i]);
    std::vector<Joint<R>> joints(nj);
    for (uint32_t i = 0; i < nj; ++i) joints[i] = to_joint<R>(cons[i]);
    std::vector<uint32_t> off(offsets, offsets + n + 1), idx(indices, indices + (n ? offsets[n] : 0));
    RunOptions<R> o;
    o.dt = R(ro->dt);
    o.gravity = {R(ro->gravity[0]), R(ro->gravity[1]), R(ro->gravity[2])};
    o.alpha = R(ro->alpha);
    o.beta_lin = R(ro->beta_lin);
    o.penalty_max = R(ro->penalty_max);
    o.iterations = ro->iterations;
    std::vector<uint32_t> joff(n + 1, 0), jidx;
    if (use_joint_csr) {
        for (auto& j : joints) {
            joff[j.a + 1] += 1;
            if (j.b != j.a) joff[j.b + 1] += 1;
        }
        for (uint32_t i = 0; i < n; ++i) joff[i + 1] += joff[i];
        jidx.assign(joff[n], 0);
        std::vector<uint32_t> cur(joff.begin(), joff.end());
        for (uint32_t k = 0; k < nj; ++k) {
            jidx[cur[joints[k].a]++] = k;
            if (joints[k].b != joints[k].a) jidx[cur[joints[k].b]++] = k;
        }
    }
    AvbdResult<P, R> res;
    avbd_run(B, rows, off, idx, joints, use_joint_csr ? &joff : nullptr, use_joint_csr ? &jidx : nullptr, o, nullptr,
             0, res, 1);
    for (uint32_t i = 0; i < n; ++i) {
        if (out_pos) {
            out_pos[3 * i] = float(res.pos[i].x);
            out_pos[3 * i + 1] = float(res.pos[i].y);
            out_pos[3 * i + 2] = float(res.pos[i].z);
        }
        if (out_rot) {
            out_rot[4 * i] = float(res.rot[i].x);
            out_rot[4 * i + 1] = float(res.rot[i].y);
            out_rot[4 * i + 2] = float(res.rot[i].z);
            out_rot[4 * i + 3] = float(res.rot[i].w);
        }
        auto put = [&](float* dst, V3<P> v) {
            if (!dst) return;
            dst[3 * i] = float(v.x);
            dst[3 * i + 1] = float(v.y);
            dst[3 * i + 2] = float(v.z);
        };
        put(out_vel, B.state[i].vel);
        put(out_ang, B.state[i].ang);
        put(out_prev, B.state[i].prev_vel);
    }
    for (uint32_t c = 0; c < m; ++c) {
        if (out_lambda) {
            out_lambda[3 * c] = float(rows[c].lambda.x);
            out_lambda[3 * c + 1] = float(rows[c].lambda.y);
            out_lambda[3 * c + 2] = float(rows[c].lambda.z);
        }
        if (out_penalty) {
            out_penalty[3 * c] = float(rows[c].penalty.x);
            out_penalty[3 * c + 1] = float(rows[c].penalty.y);
            out_penalty[3 * c + 2] = float(rows[c].penalty.z);
        }
    }
    return 0;
}
}  // namespace

extern "C" {

// Mirror of AvbdCompute::run (submit + read).  precision: 0 f32, 2 f64.
int oracle_avbd_run(uint32_t precision, const DioBodyState* state, const float* pos, const float* quat, uint32_t n,
                    const DioContact* contacts, uint32_t m, const DioConstraint* cons, uint32_t nj,
                    const uint32_t* offsets, const uint32_t* indices, const DioRunOptions* ro, uint32_t use_joint_csr,
                    float* out_pos, float* out_rot, float* out_vel, float* out_ang, float* out_prev,
                    float* out_lambda, float* out_penalty) {
    if (precision == DIO_PREC_F64)
        return avbd_run_t<double, double>(state, pos, quat, n, contacts, m, cons, nj, offsets, indices, ro,
                                          use_joint_csr, out_pos, out_rot, out_vel, out_ang, out_prev, out_lambda,
                                          out_penalty);
    if (precision == DIO_PREC_SPLIT)
        return avbd_run_t<double, float>(state, pos, quat, n, contacts, m, cons, nj, offsets, indices, ro,
                                         use_joint_csr, out_pos, out_rot, out_vel, out_ang, out_prev, out_lambda,
                                         out_penalty);
    return avbd_run_t<float, float>(state, pos, quat, n, contacts, m, cons, nj, offsets, indices, ro, use_joint_csr,
                                    out_pos, out_rot, out_vel, out_ang, out_prev, out_lambda, out_penalty);
}

uint32_t oracle_color_hash(uint32_t x) { return color_hash(x); }

void* oracle_world_create(const DioWorldDesc* desc, const DioConfig* cfg, int threads) {
    DioConfig c{};
    if (cfg) c = *cfg;
    if (c.contacts_per_pair == 0) c.contacts_per_pair = 4;
    if (c.precision == DIO_PREC_F64) return make_world<double, double>(*desc, c, threads);
    if (c.precision == DIO_PREC_SPLIT) return make_world<double, float>(*desc, c, threads);
    return make_world<float, float>(*desc, c, threads);
}
void oracle_world_destroy(void* h) { delete static_cast<WorldBase*>(h); }
int oracle_world_set_lag(void* h, int on) {
    static_cast<WorldBase*>(h)->set_lag(on != 0);
    return 0;
}
int oracle_world_step(void* h, const DioAvbdOptions* o, uint32_t steps) {
    static_cast<WorldBase*>(h)->step(*o, steps);
    return 0;
}
int oracle_world_download(void* h, DioGpuBody* b, DioBodyState* s) {
    static_cast<WorldBase*>(h)->download(b, s);
    return 0;
}
int oracle_world_download_f64(void* h, double* p, double* q) {
    static_cast<WorldBase*>(h)->download_f64(p, q);
    return 0;
}
int oracle_world_contacts(void* h, DioContact* out, uint32_t cap, uint32_t* m) {
    *m = static_cast<WorldBase*>(h)->contacts(out, cap);
    return *m > cap ? DIO_ERR_CAPACITY : 0;
}
int oracle_world_colors(void* h, uint32_t* out, uint32_t cap, uint32_t* n) {
    *n = static_cast<WorldBase*>(h)->colors(out, cap);
    return 0;
}
int oracle_world_stats(void* h, DioStepStats* s) {
    static_cast<WorldBase*>(h)->stats(s);
    return 0;
}

}  // extern "C"
