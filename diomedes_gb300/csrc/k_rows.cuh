// k_rows.cuh -- contact rows on the device.
//
// The reference builds rows on the host each frame: AvbdSolver::raw_contact
// (engine/src/physics/gpu.rs:239-264), container_contacts (:352-404),
// finalize_contacts (:266-311: warm start by (a, b), decay, CSR).  Here each
// piece is a kernel over slots / bodies / rows:
//   k_slot_count + scan  -> k_slot_rows      rows from valid narrow slots
//   k_cont_count + scan  -> k_cont_rows      container (wall / floor) rows
//   k_row_keys                               64-bit (a, b) keys + incidences
//   (radix sorts of keys / incidences)
//   k_warm                                   warm start + decay
//   k_csr_fill                               CSR idx / other-body arrays
#pragma once

#include "k_narrow.cuh"

namespace dio {

// Detection-space body: pose rebased to the scene origin and rounded to R.
template <class P, class R>
__device__ __forceinline__ NB<R> load_nb(const DevWorld<P, R>& w, uint32_t i) {
    NB<R> b;
    V3<P> org{P(0), P(0), P(0)};
    if (w.origin) org = xyz(w.origin[w.scene[i]]);
    b.pos = cast3<R>(sub(xyz(w.pos[0][i]), org));
    b.rot = castq<R>(quat(w.rot[0][i]));
    b.shape = load_shape<R>(&w.shape[i]);
    return b;
}

// tangents, engine/src/physics/gpu.rs:406-414
template <class R>
__device__ __forceinline__ void tangents(V3<R> n, V3<R>& t1, V3<R>& t2) {
    V3<R> c = dabs(n.x) > R(0.9) ? cross(n, V3<R>{R(0), R(1), R(0)}) : cross(n, V3<R>{R(1), R(0), R(0)});
    t1 = normalize(c);
    t2 = cross(n, t1);
}

template <class P, class R>
__device__ __forceinline__ void write_row(const DevWorld<P, R>& w, uint32_t r, uint32_t a, uint32_t b, V3<R> n,
                                          V3<R> t1, V3<R> t2, V3<R> ra, V3<R> rb, V3<R> c0, R friction, R kmin) {
    RowStatic<R> rs;
    rs.n = pack(n, friction);
    rs.t1 = pack(t1, c0.z);
    rs.t2 = pack(t2, R(0));
    rs.ra = pack(ra, c0.x);
    rs.rb = pack(rb, c0.y);
    w.rs[r] = rs;
    RowDual<P, R> du;
    du.penalty = A4<R>{kmin, kmin, kmin, R(0)};
    du.lambda = A4<P>{P(0), P(0), P(0), P(0)};
    w.rd[r] = du;
    w.ab[r] = make_uint2(a, b);
}

// Valid slots of each live group of `per` slots (the first min(*n_groups_dev,
// n_groups) groups); the scan that follows stops at the same count.
template <class R>
__global__ void k_slot_count(const Slot<R>* slots, uint32_t per, const uint32_t* n_groups_dev, uint32_t n_groups,
                             uint32_t* counts) {
    pdl_enter();
    const uint32_t ng = n_groups_dev ? min(*n_groups_dev, n_groups) : n_groups;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < ng; p += gridDim.x * blockDim.x) {
        uint32_t c = 0;
        for (uint32_t k = 0; k < per; ++k) c += slots[p * per + k].valid ? 1u : 0u;
        counts[p] = c;
    }
}

// raw_contact for every valid slot, rows at `offsets[group]` in slot order.
template <class P, class R>
__global__ void k_slot_rows(DevWorld<P, R> w, const Slot<R>* slots, uint32_t per, const uint32_t* n_groups_dev,
                            uint32_t n_groups, const uint32_t* offsets, PrepParams<R> o) {
    pdl_enter();
    const uint32_t ng = n_groups_dev ? min(*n_groups_dev, n_groups) : n_groups;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < ng; p += gridDim.x * blockDim.x) {
        uint32_t r = offsets[p];
        // a group without valid slots (a box overlap without contact) is
        // skipped unread; the last live group ends at the total, offsets[n_groups]
        const uint32_t r_end = p + 1 < ng ? offsets[p + 1] : offsets[n_groups];
        if (r_end == r) continue;
        for (uint32_t k = 0; k < per; ++k) {
            const Slot<R> s = slots[p * per + k];
            if (!s.valid) continue;
            if (s.a >= w.n || s.b >= w.n) {
                atomicOr(&w.ctr->error_flags, kErrBadIndex);
                continue;
            }
            if (r >= w.max_rows) {
                atomicOr(&w.ctr->error_flags, kErrRowOverflow);
                return;
            }
            NB<R> A = load_nb(w, s.a), B = load_nb(w, s.b);
            V3<R> nrm = xyz(s.normal);
            V3<R> t1, t2;
            tangents(nrm, t1, t2);
            V3<R> ra = rotate(conj(A.rot), sub(xyz(s.pa), A.pos));
            V3<R> rb = rotate(conj(B.rot), sub(xyz(s.pb), B.pos));
            write_row(w, r, s.a, s.b, neg(nrm), t1, t2, ra, rb, V3<R>{o.margin - s.depth, R(0), R(0)}, o.friction,
                      o.penalty_min);
            ++r;
        }
    }
}

// cube_support_face, engine/src/physics/gpu.rs:314-350 (per-axis for BOX)
template <class R>
__device__ __forceinline__ void support_face(const NB<R>& b, V3<R> outward, V3<R> pts[4]) {
    V3<R> ax[3];
    axes_of(b.rot, ax);
    uint32_t ai = 0;
    R best = dabs(dot(ax[0], outward));
    for (uint32_t i = 1; i < 3; ++i) {
        R al = dabs(dot(ax[i], outward));
        if (al > best) {
            ai = i;
            best = al;
        }
    }
    V3<R> h = box_half(b.shape);
    V3<R> center, u, v;
    R eu, ev;
    face_frame(b.pos, ax, h, ai, outward, pts, center, u, v, eu, ev);
}

// container_contacts for one body (engine/src/physics/gpu.rs:352-404):
// counts (write == false) or writes rows starting at `r`.
template <class P, class R>
__device__ __forceinline__ uint32_t container_rows(const DevWorld<P, R>& w, uint32_t i, const SceneDesc& sc,
                                                   const PrepParams<R>& o, bool write_out, uint32_t r) {
    const A4<R>* walls = w.walls + 6 * (size_t)w.scene[i];
    V3<R> vel = cast3<R>(xyz(w.vel[i]));
    // Quick reject: every support point lies within an L1 bounding radius of
    // the body centre, so when the centre plus that radius plus this step's
    // travel is (with rounding slack) inside a wall, that wall has no row
    // with depth > 0 -- the same empty set the full test produces.  The
    // bound needs only the shape's tag and first corner and the position, so
    // the orientation and the rest of the shape are read only for a body
    // that can reach a wall.
    const uint32_t tag = reinterpret_cast<const uint4*>(&w.shape[i])->x;
    const float4 c0 = reinterpret_cast<const float4*>(w.shape[i].corners)[0];
    V3<P> org{P(0), P(0), P(0)};
    if (w.origin) org = xyz(w.origin[w.scene[i]]);
    const V3<R> pos = cast3<R>(sub(xyz(w.pos[0][i]), org));  // as load_nb forms it
    const bool boxy = tag == DIO_SHAPE_CUBE || tag == DIO_SHAPE_BOX;
    R rbound = R(-1);
    if (boxy) {
        rbound = dabs(R(c0.x)) + dabs(R(c0.y)) + dabs(R(c0.z));
    } else if (tag == DIO_SHAPE_SPHERE) {
        rbound = dabs(R(c0.x));
    } else if (tag == DIO_SHAPE_TETRAHEDRON) {
        const ShapeR<R> sh = load_shape<R>(&w.shape[i]);
        rbound = R(0);
        for (int k = 0; k < 4; ++k)
            rbound = fmax_(rbound, dabs(sh.c[k].x) + dabs(sh.c[k].y) + dabs(sh.c[k].z));
    }
    const R travel = rbound >= R(0) ? length(vel) * o.dt : R(0);
    uint32_t reach = 0x3Fu;  // walls a support point may reach this step
    if (rbound >= R(0)) {
        reach = 0;
        for (int k = 0; k < 6; ++k) {
            const A4<R> wall = walls[k];
            const R d = dot(pos, xyz(wall));
            const R slack = R(1e-4) * (R(1) + dabs(wall.w) + dabs(d));
            if (!(d + rbound + travel + slack < wall.w)) reach |= 1u << k;
        }
    }
    if (!reach) return 0;
    NB<R> b = load_nb(w, i);
    uint32_t count = 0;
#pragma unroll 1
    for (int k = 0; k < 6; ++k) {
        if (!((reach >> k) & 1u)) continue;
        const A4<R> wall = walls[k];
        const V3<R> outward = xyz(wall);
        const R plane = wall.w;
        V3<R> pts[4];
        uint32_t np;
        if (boxy) {
            support_face(b, outward, pts);
            np = 4;
        } else {
            V3<R> local = rotate(conj(b.rot), outward);
            pts[0] = add(rotate(b.rot, support(b.shape, local, w.hull)), b.pos);
            np = 1;
        }
        V3<R> normal = neg(outward);
        V3<R> t1, t2;
        if (write_out) tangents(normal, t1, t2);
        for (uint32_t p = 0; p < np; ++p) {
            V3<R> cp = pts[p];
            R cur = dot(cp, outward) - plane;
            V3<R> pred = add(cp, scale(vel, o.dt));
            R pd = dot(pred, outward) - plane;
            R depth = fmax_(cur, pd);
            if (depth > R(0)) {
                if (write_out) {
                    if (r + count < w.max_rows) {
                        V3<R> ra = rotate(conj(b.rot), sub(cp, b.pos));
                        write_row(w, r + count, i, kContainer, normal, t1, t2, ra, V3<R>{R(0), R(0), R(0)},
                                  V3<R>{o.margin - depth, R(0), R(0)}, o.friction, o.penalty_min);
                    } else {
                        atomicOr(&w.ctr->error_flags, kErrRowOverflow);
                    }
                }
                ++count;
            }
        }
    }
    return count;
}

// The six walls of each scene's container (container_collide,
// engine/src/physics/gpu.rs): outward normal = rotation * (+-axis), plane
// offset = centre . outward + half extent; centre rebased to the scene's
// detection origin.  Computed once per upload.
template <class P, class R>
__global__ void k_scene_walls(DevWorld<P, R> w, const SceneDesc* scenes, uint32_t ns, A4<R>* walls) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < 6 * ns; t += gridDim.x * blockDim.x) {
        const uint32_t s = t / 6, k = t % 6;
        const SceneDesc sc = scenes[s];
        V3<P> org{P(0), P(0), P(0)};
        if (w.origin) org = xyz(w.origin[s]);
        const V3<R> center = cast3<R>(sub(V3<P>{P(sc.center[0]), P(sc.center[1]), P(sc.center[2])}, org));
        const Q4<R> crot{R(sc.rotation[0]), R(sc.rotation[1]), R(sc.rotation[2]), R(sc.rotation[3])};
        const R half = R(sc.half_extent);
        const V3<R> axis = k < 2 ? V3<R>{R(1), R(0), R(0)} : (k < 4 ? V3<R>{R(0), R(1), R(0)} : V3<R>{R(0), R(0), R(1)});
        const R sign = (k & 1) ? R(-1) : R(1);
        const V3<R> outward = rotate(crot, scale(axis, sign));
        walls[t] = A4<R>{outward.x, outward.y, outward.z, dot(center, outward) + half};
    }
}

// counts[hi - lo] is set to 0 for the exclusive scan over hi - lo + 1 entries
template <class P, class R>
__global__ void k_cont_count(DevWorld<P, R> w, uint32_t lo, uint32_t hi, PrepParams<R> o, uint32_t* counts) {
    pdl_enter();
    if (blockIdx.x == 0 && threadIdx.x == 0) counts[hi - lo] = 0u;
    for (uint32_t i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += gridDim.x * blockDim.x) {
        uint32_t c = 0;
        const SceneDesc sc = w.scenes[w.scene[i]];
        if (w.inv[i].w != R(0) && sc.has_container) c = container_rows(w, i, sc, o, false, 0);
        counts[i - lo] = c;
    }
}

// zero (may be null): hi - lo + 1 per-body counters cleared on the way, for
// the dynamic-body CSR count that follows
template <class P, class R>
__global__ void k_cont_rows(DevWorld<P, R> w, uint32_t lo, uint32_t hi, PrepParams<R> o, const uint32_t* offsets,
                            const uint32_t* base_dev, uint32_t* zero) {
    pdl_enter();
    uint32_t base = *base_dev;
    if (zero && blockIdx.x == 0 && threadIdx.x == 0) zero[hi - lo] = 0u;
    for (uint32_t i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += gridDim.x * blockDim.x) {
        if (zero) zero[i - lo] = 0u;
        const uint32_t r = offsets[i - lo];
        if (offsets[i - lo + 1] == r) continue;  // no rows: nothing to recompute
        const SceneDesc sc = w.scenes[w.scene[i]];
        if (w.inv[i].w != R(0) && sc.has_container) container_rows(w, i, sc, o, true, base + r);
    }
}

__device__ __forceinline__ unsigned long long row_key(uint2 ab) {
    return ((unsigned long long)ab.x << 32) | (unsigned long long)ab.y;
}

// Keys + row ids for the warm-start sorts, and the (body, row) incidences of
// the CSR (two per row; b == CONTAINER becomes the sentinel body `n`).
static __global__ void k_row_keys(const uint2* ab, const uint32_t* m_dev, uint32_t cap, unsigned long long* keys,
                           uint32_t* ids, uint32_t* inc_body, uint32_t* inc_row, uint32_t n_sentinel) {
    uint32_t m = *m_dev;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < cap; r += gridDim.x * blockDim.x) {
        if (r < m) {
            uint2 v = ab[r];
            if (keys) {
                keys[r] = row_key(v);
                ids[r] = r;
            }
            if (inc_body) {
                inc_body[2 * r] = v.x;
                inc_row[2 * r] = r;
                inc_body[2 * r + 1] = v.y == kContainer ? n_sentinel : v.y;
                inc_row[2 * r + 1] = r;
            }
        } else {
            if (keys) {
                keys[r] = ~0ull;
                ids[r] = r;
            }
            if (inc_body) {
                inc_body[2 * r] = n_sentinel;
                inc_row[2 * r] = r;
                inc_body[2 * r + 1] = n_sentinel;
                inc_row[2 * r + 1] = r;
            }
        }
    }
}

// Warm start + decay (finalize_contacts, gpu.rs:266-283).  new_keys/new_ids
// are the new rows' keys stably sorted; prev_keys/prev_ids the previous
// rows'.  The first new row of each key takes (lambda, penalty) of the LAST
// previous row with that key; every row then decays.
template <class P, class R>
__global__ void k_warm(DevWorld<P, R> w, const uint32_t* m_dev, const unsigned long long* new_keys,
                       const uint32_t* new_ids, const unsigned long long* prev_keys, const uint32_t* prev_ids,
                       uint32_t n_prev, const RowDual<P, R>* prev_dual, PrepParams<R> o) {
    uint32_t m = *m_dev;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < m; t += gridDim.x * blockDim.x) {
        unsigned long long key = new_keys[t];
        uint32_t r = new_ids[t];
        RowDual<P, R> du = w.rd[r];
        bool first = t == 0 || new_keys[t - 1] != key;
        if (first && n_prev > 0) {
            // upper bound of key in prev_keys -> last occurrence is ub - 1
            uint32_t lo = 0, hi = n_prev;
            while (lo < hi) {
                uint32_t mid = (lo + hi) >> 1;
                if (prev_keys[mid] <= key)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            if (lo > 0 && prev_keys[lo - 1] == key) {
                const RowDual<P, R> pd = prev_dual[prev_ids[lo - 1]];
                du.lambda = pd.lambda;
                du.penalty = pd.penalty;
            }
        }
        P ag = P(o.alpha_gamma);
        du.lambda.x = du.lambda.x * ag;
        du.lambda.y = du.lambda.y * ag;
        du.lambda.z = du.lambda.z * ag;
        R kx = du.penalty.x * o.gamma, ky = du.penalty.y * o.gamma, kz = du.penalty.z * o.gamma;
        du.penalty.x = fmin_(fmax_(kx, o.penalty_min), o.penalty_max);
        du.penalty.y = fmin_(fmax_(ky, o.penalty_min), o.penalty_max);
        du.penalty.z = fmin_(fmax_(kz, o.penalty_min), o.penalty_max);
        w.rd[r] = du;
    }
}

// Per-body counts of the sorted incidences -> offsets are the exclusive
// scan; the fill keeps the sorted (row-ascending) order per body.
static __global__ void k_inc_count(const uint32_t* inc_body_sorted, const uint32_t* m_dev, uint32_t n, uint32_t* counts) {
    uint32_t total = 2 * *m_dev;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < total; j += gridDim.x * blockDim.x) {
        uint32_t b = inc_body_sorted[j];
        if (b < n) atomicAdd(&counts[b], 1u);
    }
}

template <class P, class R>
__global__ void k_csr_fill(DevWorld<P, R> w, const uint32_t* inc_body_sorted, const uint32_t* inc_row_sorted,
                           const uint32_t* m_dev) {
    uint32_t total = 2 * *m_dev;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < total; j += gridDim.x * blockDim.x) {
        uint32_t b = inc_body_sorted[j];
        if (b >= w.n) continue;  // container sentinels sort last
        uint32_t r = inc_row_sorted[j];
        uint2 ab = w.ab[r];
        uint32_t oth;
        if (ab.y == kContainer)
            oth = kContainer;
        else if (ab.x == b)
            oth = ab.y;
        else
            oth = ab.x | kIsB;
        if (j < w.max_incid) {
            w.row_idx[j] = r;
            w.row_oth[j] = oth;
        }
    }
}

// ---- device-driven variants for the resident world (no host-known counts)
//
// The world's rows are in canonical order: pair rows follow the pair list,
// which is sorted by (a, b), and container rows follow the body index, so
// each section of the row list is sorted by key with equal keys adjacent.
// The warm start therefore needs no sort: a row is the first of its key when
// its predecessor in the section has another key, and the last previous row
// with that key is found by binary search in the previous step's section.

__device__ __forceinline__ bool key_less(uint2 a, uint2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); }
__device__ __forceinline__ bool key_eq(uint2 a, uint2 b) { return a.x == b.x && a.y == b.y; }

// roll the per-step counters: the finished step's row counts become the
// warm-start source, the per-step counts restart at zero (and up to two
// scratch words the step's scans and sorts expect zeroed, if given)
static __global__ void k_roll_counters(Counters* c, uint32_t* zero0, uint32_t* zero1) {
    if (zero0) *zero0 = 0u;
    if (zero1) *zero1 = 0u;
    c->prev_rows = c->rows;
    c->prev_pair_rows = c->pair_rows;
    c->prev_pairs = c->pairs;
    c->pairs = 0;
    c->rows = 0;
    c->pair_rows = 0;
    c->container_rows = 0;
    c->gjk_work = 0;
    c->epa_work = 0;
    c->long_count = 0;
    c->colors = 0;
    c->traverse_pairs = 0;
}

template <class P, class R>
__global__ void k_warm_sections(DevWorld<P, R> w, const uint2* prev_ab, const RowDual<P, R>* prev_dual,
                                PrepParams<R> o) {
    pdl_enter();
    const uint32_t m = w.ctr->rows, pair_rows = w.ctr->pair_rows;
    const uint32_t prev_m = w.ctr->prev_rows, prev_pair = w.ctr->prev_pair_rows;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        const uint2 key = w.ab[r];
        const bool cont = key.y == kContainer;
        const uint32_t sec_lo = cont ? pair_rows : 0;
        RowDual<P, R> du = w.rd[r];
        bool first = r == sec_lo || !key_eq(w.ab[r - 1], key);
        if (first) {
            uint32_t lo = cont ? prev_pair : 0, hi = cont ? prev_m : prev_pair;
            const uint32_t base = lo;
            while (lo < hi) {  // upper bound of key
                uint32_t mid = (lo + hi) >> 1;
                if (!key_less(key, prev_ab[mid]))
                    lo = mid + 1;
                else
                    hi = mid;
            }
            if (lo > base && key_eq(prev_ab[lo - 1], key)) {
                const RowDual<P, R> pd = prev_dual[lo - 1];
                du.lambda = pd.lambda;
                du.penalty = pd.penalty;
            }
        }
        P ag = P(o.alpha_gamma);
        du.lambda.x = du.lambda.x * ag;
        du.lambda.y = du.lambda.y * ag;
        du.lambda.z = du.lambda.z * ag;
        R kx = du.penalty.x * o.gamma, ky = du.penalty.y * o.gamma, kz = du.penalty.z * o.gamma;
        du.penalty.x = fmin_(fmax_(kx, o.penalty_min), o.penalty_max);
        du.penalty.y = fmin_(fmax_(ky, o.penalty_min), o.penalty_max);
        du.penalty.z = fmin_(fmax_(kz, o.penalty_min), o.penalty_max);
        w.rd[r] = du;
    }
}

// CSR of the dynamic bodies only (the primal never visits a static body):
// counts, then an atomic scatter (each body's count taken down to zero),
// then each segment sorted by row index,
// which restores the reference's fill order (finalize_contacts, gpu.rs:
// 286-310) without a sort over all incidences.
template <class P, class R>
__global__ void k_csr_count_dyn(DevWorld<P, R> w, uint32_t* counts) {
    pdl_enter();
    const uint32_t m = w.ctr->rows;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        uint2 ab = w.ab[r];
        if (w.inv[ab.x].w != R(0)) atomicAdd(&counts[ab.x], 1u);
        if (ab.y != kContainer && w.inv[ab.y].w != R(0)) atomicAdd(&counts[ab.y], 1u);
    }
}

// remaining: each body's incidence count (k_csr_count_dyn), consumed here
template <class P, class R>
__global__ void k_csr_scatter_dyn(DevWorld<P, R> w, uint32_t* remaining) {
    pdl_enter();
    const uint32_t m = w.ctr->rows;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        uint2 ab = w.ab[r];
        if (w.inv[ab.x].w != R(0)) {
            uint32_t j = w.row_off[ab.x] + atomicSub(&remaining[ab.x], 1u) - 1u;
            if (j < w.max_incid) w.row_idx[j] = r;
        }
        if (ab.y != kContainer && w.inv[ab.y].w != R(0)) {
            uint32_t j = w.row_off[ab.y] + atomicSub(&remaining[ab.y], 1u) - 1u;
            if (j < w.max_incid) w.row_idx[j] = r;
        }
    }
}

template <class P, class R>
__global__ void k_csr_other_dyn(DevWorld<P, R> w) {
    pdl_enter();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        uint32_t j0 = w.row_off[i], j1 = min(w.row_off[i + 1], w.max_incid);
        for (uint32_t j = j0; j < j1; ++j) {
            uint2 v = w.ab[w.row_idx[j]];
            w.row_oth[j] = v.y == kContainer ? kContainer : (v.x == i ? v.y : (v.x | kIsB));
        }
    }
}

}  // namespace dio
