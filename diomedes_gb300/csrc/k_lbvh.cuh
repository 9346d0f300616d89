// k_lbvh.cuh -- LBVH broad phase (replaces broad_sweep_dense,
// engine/gpu_physics/broadphase/src/lib.rs:171-216, at scale).
//
// Per step, for every scene at once:
//   k_scene_bounds   centroid bounds per scene (ordered-int atomics)
//   k_morton         30-bit Morton code of each AABB centre within its scene's
//                    bounds; key = scene << 32 | code (scenes stay contiguous)
//   radix sort       (key, body) pairs (k_scan.cuh)
//   k_karras         binary radix tree per scene (Karras 2012), internal node
//                    k of a scene covers a key range; children are leaves or
//                    internal nodes of the same scene
//   k_chunk_build    the four steps above in one launch when every scene fits
//                    the shared-memory trees: one CTA per chunk of scenes
//   k_refit          bottom-up AABB union (second arrival at a node continues)
//   k_traverse       stack traversal per leaf; a pair (i, j) is reported only
//                    by its smaller body i, so each overlap is found once;
//                    count pass, scan, write pass
//   k_sort_segments  each body's partners sorted ascending, giving the pair
//                    list in (a, b) order, the same set and order as the
//                    dense sweep
// The overlap test is the reference's closed-interval test on the same
// support AABBs, and tree boxes are exact unions, so the pair set equals the
// dense sweep's bit for bit.
#pragma once

#include "k_broad.cuh"

namespace dio {

__device__ __forceinline__ uint32_t f2ord(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}
__device__ __forceinline__ uint64_t d2ord(double f) {
    uint64_t u = (uint64_t)__double_as_longlong(f);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}

// AABB centre, rounded to FP32 (the Morton grid only needs to be monotone
// in the centre)
template <class R>
__device__ __forceinline__ void aabb_centre(const A4<R>& a, const A4<R>& b, float c[3]) {
    c[0] = float(a.x * R(0.5) + b.x * R(0.5));
    c[1] = float(a.y * R(0.5) + b.y * R(0.5));
    c[2] = float(a.z * R(0.5) + b.z * R(0.5));
}

// per-scene centroid bounds: 6 ordered uints (min xyz, max xyz)
template <class R>
__global__ void k_scene_bounds(const A4<R>* mn, const A4<R>* mx, const uint32_t* scene, uint32_t n, uint32_t* bounds) {
    pdl_enter();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float c[3];
        aabb_centre(mn[i], mx[i], c);
        uint32_t ox = f2ord(c[0]);
        uint32_t oy = f2ord(c[1]);
        uint32_t oz = f2ord(c[2]);
        const uint32_t s = scene[i];
        // lanes of one scene reduce first; their leader issues the atomics
        const uint32_t grp = __match_any_sync(__activemask(), s);
        const uint32_t nx = __reduce_min_sync(grp, ox), ny = __reduce_min_sync(grp, oy),
                       nz = __reduce_min_sync(grp, oz);
        const uint32_t xx = __reduce_max_sync(grp, ox), xy = __reduce_max_sync(grp, oy),
                       xz = __reduce_max_sync(grp, oz);
        if ((threadIdx.x & 31) == (uint32_t)(__ffs(grp) - 1)) {
            uint32_t* bs = bounds + 6 * s;
            atomicMin(&bs[0], nx);
            atomicMin(&bs[1], ny);
            atomicMin(&bs[2], nz);
            atomicMax(&bs[3], xx);
            atomicMax(&bs[4], xy);
            atomicMax(&bs[5], xz);
        }
    }
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// 32-bit key: scene index in the top `scene_bits`, then a Morton code with
// `axis_bits` per axis (10 for one scene, 7 for up to 2048 scenes); the key
// only has to keep scenes contiguous and order bodies spatially within one
// Morton code of centre c within the scene bounds bs (6 ordered uints)
__device__ __forceinline__ uint32_t morton_code(const float c[3], const uint32_t* bs, uint32_t axis_bits) {
    const float cells = float(1u << axis_bits);
    const uint32_t top = (1u << axis_bits) - 1u;
    uint32_t q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float lo = ord2f(bs[k]), hi = ord2f(bs[3 + k]);
        float ext = hi - lo;
        float t = ext > 0.f ? (c[k] - lo) / ext : 0.f;
        t = fminf(fmaxf(t, 0.f), 1.f);
        q[k] = min((uint32_t)(t * cells), top);
    }
    return (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
}

template <class R>
__global__ void k_morton(const A4<R>* mn, const A4<R>* mx, const uint32_t* scene, uint32_t n, const uint32_t* bounds,
                         uint32_t scene_bits, uint32_t axis_bits, uint32_t* keys, uint32_t* vals) {
    pdl_enter();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float c[3];
        aabb_centre(mn[i], mx[i], c);
        const uint32_t s = scene[i];
        const uint32_t code = morton_code(c, bounds + 6 * s, axis_bits);
        keys[i] = scene_bits ? ((s << (3 * axis_bits)) | code) : code;
        vals[i] = i;
    }
}

// Karras prefix length of sorted positions a, b of a scene's sorted keys
// seg[0, n); duplicates tie-break on the index.  Only XORs and equality of
// keys of one scene enter, so any key offset common to the scene cancels.
__device__ __forceinline__ int kdelta(const uint32_t* seg, int n, int a, int b) {
    if (b < 0 || b >= n) return -1;
    uint32_t ka = seg[a], kb = seg[b];
    if (ka == kb) return 32 + __clz((uint32_t)(a ^ b));
    return __clz(ka ^ kb);
}

constexpr uint32_t kLeafFlag = 0x80000000u;

// L1-bypassing loads (data produced by other CTAs of the same launch)
template <class R>
__device__ __forceinline__ A4<R> ldcg4(const A4<R>* p);
template <>
__device__ __forceinline__ A4<float> ldcg4(const A4<float>* p) {
    float4 v = __ldcg(reinterpret_cast<const float4*>(p));
    return {v.x, v.y, v.z, v.w};
}
template <>
__device__ __forceinline__ A4<double> ldcg4(const A4<double>* p) {
    const double2* q = reinterpret_cast<const double2*>(p);
    double2 a = __ldcg(q), b = __ldcg(q + 1);
    return {a.x, a.y, b.x, b.y};
}

// a 32-bit tag in (and out of) the unused w slot of a box corner, as bits
__device__ __forceinline__ uint32_t tag_of(const A4<float>& a) { return __float_as_uint(a.w); }
__device__ __forceinline__ uint32_t tag_of(const A4<double>& a) { return (uint32_t)__double_as_longlong(a.w); }
template <class R>
__device__ __forceinline__ R tag_bits(uint32_t v);
template <>
__device__ __forceinline__ float tag_bits<float>(uint32_t v) { return __uint_as_float(v); }
template <>
__device__ __forceinline__ double tag_bits<double>(uint32_t v) { return __longlong_as_double((long long)v); }

// Internal node k of a scene whose sorted keys are seg[0, ns) and whose
// slots start at global slot lo: node k lives at slot lo + k; child codes
// are global slots, leaves flagged with kLeafFlag (leaf = sorted position);
// parents of internal slots in [0, n), of leaves in [n, 2n)
__device__ __forceinline__ void karras_node(const uint32_t* seg, uint32_t lo, int ns, int k, uint32_t n,
                                            uint2* children, uint32_t* parent) {
    int d = (kdelta(seg, ns, k, k + 1) - kdelta(seg, ns, k, k - 1)) >= 0 ? 1 : -1;
    int dmin = kdelta(seg, ns, k, k - d);
    int lmax = 2;
    while (kdelta(seg, ns, k, k + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (kdelta(seg, ns, k, k + (l + t) * d) > dmin) l += t;
    int j = k + l * d;
    int dnode = kdelta(seg, ns, k, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (kdelta(seg, ns, k, k + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int gamma = k + s * d + min(d, 0);
    uint32_t left = (min(k, j) == gamma) ? ((lo + gamma) | kLeafFlag) : (lo + gamma);
    uint32_t right = (max(k, j) == gamma + 1) ? ((lo + gamma + 1) | kLeafFlag) : (lo + gamma + 1);
    children[lo + k] = make_uint2(left, right);
    parent[(left & kLeafFlag) ? n + (left & ~kLeafFlag) : left] = lo + k;
    parent[(right & kLeafFlag) ? n + (right & ~kLeafFlag) : right] = lo + k;
}

// binary radix tree per scene (Karras 2012) over the globally sorted keys
static __global__ void k_karras(const uint32_t* keys, const SceneDesc* scenes, const uint32_t* scene_of_pos,
                                uint32_t n, uint2* children, uint32_t* parent) {
    pdl_enter();
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const SceneDesc sc = scenes[scene_of_pos[p]];
        const uint32_t lo = sc.body_lo;
        const int ns = (int)(sc.body_hi - sc.body_lo);
        const int k = (int)(p - lo);
        if (k >= ns - 1) continue;  // ns - 1 internal nodes
        karras_node(keys + lo, lo, ns, k, n, children, parent);
    }
}

// leaf boxes in sorted order, then bottom-up unions; a node's max corner
// carries in w its highest leaf position (as bits).  counts: the per-body
// pair counters of the count pass, cleared here.
template <class R>
__global__ void k_refit(const A4<R>* mn, const A4<R>* mx, const uint32_t* leaf_body, const SceneDesc* scenes,
                        const uint32_t* scene_of_pos, uint32_t n, const uint2* children, const uint32_t* parent,
                        A4<R>* leaf_min, A4<R>* leaf_max, A4<R>* node_min, A4<R>* node_max, uint32_t* visits,
                        uint32_t skip_max, uint32_t* counts) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const SceneDesc sc = scenes[scene_of_pos[p]];
        if (sc.body_hi - sc.body_lo <= skip_max) continue;  // k_scene_tree's scene
        uint32_t b = leaf_body[p];
        counts[b] = 0u;
        leaf_min[p] = mn[b];
        leaf_max[p] = mx[b];
        if (sc.body_hi - sc.body_lo < 2) continue;
        __threadfence();
        uint32_t node = parent[n + p];
        while (true) {
            if (atomicAdd(&visits[node], 1u) == 0) break;  // first arrival stops
            __threadfence();
            uint2 c = children[node];
            const A4<R>* lmn = (c.x & kLeafFlag) ? leaf_min : node_min;
            const A4<R>* lmx = (c.x & kLeafFlag) ? leaf_max : node_max;
            const A4<R>* rmn = (c.y & kLeafFlag) ? leaf_min : node_min;
            const A4<R>* rmx = (c.y & kLeafFlag) ? leaf_max : node_max;
            uint32_t li = c.x & ~kLeafFlag, ri = c.y & ~kLeafFlag;
            // boxes written by other CTAs in this launch: read through L2
            A4<R> a0 = ldcg4(&lmn[li]), a1 = ldcg4(&lmx[li]), b0 = ldcg4(&rmn[ri]), b1 = ldcg4(&rmx[ri]);
            const uint32_t hi = max((c.x & kLeafFlag) ? li : tag_of(a1), (c.y & kLeafFlag) ? ri : tag_of(b1));
            node_min[node] = A4<R>{fmin_(a0.x, b0.x), fmin_(a0.y, b0.y), fmin_(a0.z, b0.z), R(0)};
            node_max[node] = A4<R>{fmax_(a1.x, b1.x), fmax_(a1.y, b1.y), fmax_(a1.z, b1.z), tag_bits<R>(hi)};
            __threadfence();
            if (node == sc.body_lo) break;  // scene root
            node = parent[node];
        }
    }
}

constexpr int kStack = 64;

// Count pass of the global trees (scenes beyond the shared-memory trees):
// the leaf at position p visits only the subtrees holding positions above
// p (a node's highest leaf position is its max corner's w), so each
// overlapping pair is found once, by its lower position; it is counted for
// body a = min(i, j) and appended as (a, b) to the pair scratch through a
// warp-aggregated cursor, from which the write pass places it without
// walking the trees again.  With split = kWalkSplit each leaf's walk is
// split over 4 threads, one per subtree two levels below the root (a leaf at
// that depth is tested directly), so a scene of a few thousand bodies still
// fills the SMs with walks; with split = 1 a thread walks from the root.
constexpr uint32_t kWalkSplit = 4;
template <class R>
__global__ void __launch_bounds__(128)
    k_traverse_count(const uint32_t* leaf_body, const SceneDesc* scenes, const uint32_t* scene_of_pos, uint32_t n,
                     const uint2* children, const A4<R>* leaf_min, const A4<R>* leaf_max, const A4<R>* node_min,
                     const A4<R>* node_max, uint32_t* counts, uint2* scratch, uint32_t scratch_cap,
                     uint32_t* scratch_n, uint32_t* err, uint32_t skip_max, uint32_t split) {
    const uint64_t total = (uint64_t)n * split;
    for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total;
         u += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t p = (uint32_t)(u / split), part = (uint32_t)(u % split);
        const SceneDesc sc = scenes[scene_of_pos[p]];
        if (sc.body_hi - sc.body_lo <= skip_max) continue;  // k_scene_tree's scene
        if (sc.body_hi - sc.body_lo < 2) continue;
        // the root (split 1), or its children, each replaced by its own
        // children when internal
        uint32_t items[kWalkSplit];
        uint32_t ni = 0;
        if (split == 1u) {
            items[ni++] = sc.body_lo;
        } else {
            const uint2 rc = children[sc.body_lo];
            const uint32_t top[2] = {rc.x, rc.y};
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                if (top[k] & kLeafFlag) {
                    items[ni++] = top[k];
                } else {
                    const uint2 gc = children[top[k]];
                    items[ni++] = gc.x;
                    items[ni++] = gc.y;
                }
            }
        }
        if (part >= ni) continue;
        const uint32_t i = leaf_body[p];
        const A4<R> qmn = leaf_min[p], qmx = leaf_max[p];
        auto emit = [&](uint32_t idx) {
            const uint32_t j = leaf_body[idx];
            const uint32_t a = min(i, j), b = max(i, j);
            atomicAdd(&counts[a], 1u);
            const uint32_t slot = warp_append(scratch_n);
            if (slot < scratch_cap) scratch[slot] = make_uint2(a, b);
        };
        const uint32_t first = items[part];
        const uint32_t fidx = first & ~kLeafFlag;
        if (first & kLeafFlag) {
            if (fidx > p && overlap(qmn, qmx, leaf_min[fidx], leaf_max[fidx])) emit(fidx);
            continue;
        }
        {
            const A4<R> fmx = node_max[fidx];
            if (!(tag_of(fmx) > p && overlap(qmn, qmx, node_min[fidx], fmx))) continue;
        }
        uint32_t stack[kStack];
        int sp = 0;
        uint32_t node = fidx;
        while (true) {
            const uint2 c = children[node];
            const uint32_t ch[2] = {c.x, c.y};
            uint32_t push = 0;
            uint32_t next[2];
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const uint32_t x = ch[k];
                const uint32_t idx = x & ~kLeafFlag;
                if (x & kLeafFlag) {
                    if (idx > p && overlap(qmn, qmx, leaf_min[idx], leaf_max[idx])) emit(idx);
                } else {
                    const A4<R> bmx = node_max[idx];
                    if (tag_of(bmx) > p && overlap(qmn, qmx, node_min[idx], bmx)) next[push++] = idx;
                }
            }
            if (push == 0) {
                if (sp == 0) break;
                node = stack[--sp];
            } else {
                node = next[0];
                if (push == 2) {
                    if (sp < kStack)
                        stack[sp++] = next[1];
                    else
                        atomicOr(err, kErrIndexOverflow);
                }
            }
        }
    }
}

// Write pass of the global trees from the count pass's scratch: pair (a, b)
// goes to offsets[a] + (a's remaining count, taken down by one; the
// segment is sorted afterwards).  Nothing when the scratch overflowed: the
// full write traversal (k_traverse) runs instead.
static __global__ void k_place_scratch(const uint2* scratch, const uint32_t* scratch_n, uint32_t scratch_cap,
                                       const uint32_t* offsets, uint32_t* remaining, uint32_t* pb, uint32_t cap) {
    pdl_enter();
    const uint32_t m = *scratch_n;
    if (m > scratch_cap) return;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
        const uint2 ab = scratch[k];
        const uint32_t pos = offsets[ab.x] + atomicSub(&remaining[ab.x], 1u) - 1u;
        if (pos < cap) pb[pos] = ab.y;
    }
}

// Full write traversal of the global trees, only when the count pass's
// scratch overflowed: per body i the partners j > i land unsorted in
// pb[offsets[i] ...]
template <class R>
__global__ void __launch_bounds__(128) k_traverse(const uint32_t* leaf_body, const SceneDesc* scenes,
                                                  const uint32_t* scene_of_pos, uint32_t n, const uint2* children,
                                                  const A4<R>* leaf_min, const A4<R>* leaf_max,
                                                  const A4<R>* node_min, const A4<R>* node_max,
                                                  const uint32_t* offsets, uint32_t* pb, uint32_t cap,
                                                  const uint32_t* scratch_n, uint32_t scratch_cap, uint32_t* err,
                                                  uint32_t skip_max) {
    pdl_enter();
    if (*scratch_n <= scratch_cap) return;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const SceneDesc sc = scenes[scene_of_pos[p]];
        if (sc.body_hi - sc.body_lo <= skip_max) continue;  // k_scene_tree's scene
        if (sc.body_hi - sc.body_lo < 2) continue;
        const uint32_t i = leaf_body[p];
        uint32_t out = offsets[i];
        const A4<R> qmn = leaf_min[p], qmx = leaf_max[p];
        uint32_t stack[kStack];
        int sp = 0;
        uint32_t node = sc.body_lo;  // root
        while (true) {
            uint2 c = children[node];
            uint32_t ch[2] = {c.x, c.y};
            uint32_t push = 0;
            uint32_t next[2];
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                uint32_t x = ch[k];
                uint32_t idx = x & ~kLeafFlag;
                if (x & kLeafFlag) {
                    if (overlap(qmn, qmx, leaf_min[idx], leaf_max[idx])) {
                        uint32_t j = leaf_body[idx];
                        if (j > i) {
                            if (out < cap) pb[out] = j;
                            ++out;
                        }
                    }
                } else if (overlap(qmn, qmx, node_min[idx], node_max[idx])) {
                    next[push++] = idx;
                }
            }
            if (push == 0) {
                if (sp == 0) break;
                node = stack[--sp];
            } else {
                node = next[0];
                if (push == 2) {
                    if (sp < kStack)
                        stack[sp++] = next[1];
                    else
                        atomicOr(err, kErrIndexOverflow);
                }
            }
        }
    }
}

// ---- one CTA per chunk of scenes, trees in shared memory ----
// Consecutive scenes of at most scene_tree_cap<R>() bodies are packed into
// chunks of at most that many bodies (a chunk's bodies and sorted positions
// are both the index range [lo, hi)).  One CTA stages its chunk's trees (leaf
// and node boxes, children, parents) in shared memory.
//   count pass  refit with shared-memory atomics (also each node's highest
//               leaf position), then traverse: the leaf at position p visits
//               only subtrees holding positions > p, so each overlapping pair
//               is found once, by its lower position; it is counted for body
//               a = min(i, j) and appended as (a, b) to the chunk's scratch
//               region (scratch_k slots per body of the chunk).  The w slots
//               of the box corners carry what a traversal step needs next: a
//               leaf's min corner its body; a node's min corner its two
//               children (chunk positions and leaf flags, 12 bits each) and
//               its max corner its highest leaf position.  A step therefore
//               loads only the two children's boxes, and the stack holds
//               children words
//   write pass  places the scratch pairs at the scanned per-body offsets; a
//               chunk whose scratch overflowed is traversed again and written
//               directly (body i's partners j > i)
// Per-body partner sets equal those of the global kernels (same trees, same
// test); the order inside a body's segment does not matter because each
// segment is sorted afterwards.
template <class R>
__host__ __device__ constexpr uint32_t scene_tree_cap() { return sizeof(R) == 4 ? 2048u : 1024u; }
template <class R>
__host__ __device__ constexpr size_t scene_tree_bytes(uint32_t cap) {
    // leaf min/max, node min/max, children, leaf parent, node parent, visit
    // flag (then per-body count), leaf's scene root
    return (size_t)cap * (4 * sizeof(A4<R>) + sizeof(uint2) + 4 * sizeof(uint32_t)) + 16;
}
// a node's children (chunk positions with leaf flags) as one 24-bit word
constexpr uint32_t kCwIndex = 0x7FFu, kCwLeaf = 0x800u;
static_assert(scene_tree_cap<float>() <= kCwIndex + 1 && scene_tree_cap<double>() <= kCwIndex + 1,
              "chunk positions must fit a children word");
__device__ __forceinline__ uint32_t children_word(uint2 c) {
    const uint32_t l = (c.x & ~kLeafFlag) | ((c.x & kLeafFlag) ? kCwLeaf : 0u);
    const uint32_t r = (c.y & ~kLeafFlag) | ((c.y & kLeafFlag) ? kCwLeaf : 0u);
    return l | (r << 12);
}
constexpr int kSceneTreeThreads = 1024;
constexpr uint32_t kNoRoot = 0xFFFFFFFFu;

struct TreeArgs {
    const uint32_t* leaf_body;
    const SceneDesc* scenes;
    const uint32_t* scene_of_pos;
    const uint2* chunks;
    uint32_t n;
    uint32_t cap_bodies;
    const uint2* children;
    const uint32_t* parent;
    uint32_t* counts;
    uint32_t* offsets;
    uint32_t* pb;
    uint32_t cap;
    uint2* scratch;
    uint32_t scratch_k;
    uint32_t* chunk_n;
    uint32_t* chunk_ovf;
    uint32_t* chunk_tot;  // pairs found per chunk (count pass)
    uint32_t* err;
    // write pass of a world whose scenes all have shared-memory trees: it
    // also forms the offsets, sorts each body's partners and emits the pairs
    uint32_t fused;
    uint32_t nchunks;
    DioPair* pairs;
    Counters* ctr;
};

// Count-pass traversal from the leaf at chunk position p: pairs with leaves at
// higher positions, counted for the lower body and appended (warp-aggregated) to the chunk's
// scratch.  Both children's boxes (and their tags) are loaded before either
// is tested, so the loads of one step overlap.
template <class R>
__device__ __forceinline__ void tree_count_leaf(uint32_t p, uint32_t root, const A4<R>* lmn, const A4<R>* lmx,
                                                const A4<R>* nmn, const A4<R>* nmx, uint32_t* vis,
                                                uint32_t* s_cursor, uint2* dst, uint32_t region, uint32_t lo,
                                                uint32_t* err) {
    const A4<R> qmn = lmn[p], qmx = lmx[p];
    const uint32_t i = tag_of(qmn);
    uint32_t stack[kStack];  // children words of the nodes still to visit
    int sp = 0;
    uint32_t cw = tag_of(nmn[root]);
    while (true) {
        uint32_t idx[2], leaf[2];
        A4<R> bmn[2], bmx[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const uint32_t c = k ? cw >> 12 : cw;
            idx[k] = c & kCwIndex;
            leaf[k] = c & kCwLeaf;
            bmn[k] = (leaf[k] ? lmn : nmn)[idx[k]];
            bmx[k] = (leaf[k] ? lmx : nmx)[idx[k]];
        }
        uint32_t w0 = 0, w1 = 0, push = 0;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            // highest leaf position below: the leaf itself, or the node's tag
            if (!((leaf[k] ? idx[k] : tag_of(bmx[k])) > p && overlap(qmn, qmx, bmn[k], bmx[k]))) continue;
            if (leaf[k]) {
                const uint32_t j = tag_of(bmn[k]);
                const uint32_t a = min(i, j), b = max(i, j);
                atomicAdd(&vis[a - lo], 1u);
                const uint32_t slot = warp_append(s_cursor);
                if (slot < region) dst[slot] = make_uint2(a, b);
            } else {
                if (push == 0)
                    w0 = tag_of(bmn[k]);
                else
                    w1 = tag_of(bmn[k]);
                ++push;
            }
        }
        if (push == 0) {
            if (sp == 0) break;
            cw = stack[--sp];
        } else {
            cw = w0;
            if (push == 2) {
                if (sp < kStack)
                    stack[sp++] = w1;
                else
                    atomicOr(err, kErrIndexOverflow);
            }
        }
    }
}

// Write-pass fallback for a chunk whose scratch overflowed: the whole tree
// from the leaf at position p, body i's partners j > i written directly at
// its scanned offset.
template <class R>
__device__ __forceinline__ void tree_write_leaf(uint32_t p, uint32_t root, const A4<R>* lmn, const A4<R>* lmx,
                                                const A4<R>* nmn, const A4<R>* nmx, const uint2* ch,
                                                const TreeArgs& t) {
    const A4<R> qmn = lmn[p], qmx = lmx[p];
    const uint32_t i = tag_of(qmn);
    uint32_t out = t.offsets[i];
    uint32_t stack[kStack];
    int sp = 0;
    uint32_t node = root;
    while (true) {
        const uint2 c = ch[node];
        const uint32_t cc[2] = {c.x, c.y};
        uint32_t n0 = 0, n1 = 0, push = 0;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const uint32_t idx = cc[k] & ~kLeafFlag;
            if (cc[k] & kLeafFlag) {
                if (overlap(qmn, qmx, lmn[idx], lmx[idx])) {
                    const uint32_t j = tag_of(lmn[idx]);
                    if (j > i) {
                        if (out < t.cap) t.pb[out] = j;
                        ++out;
                    }
                }
            } else if (overlap(qmn, qmx, nmn[idx], nmx[idx])) {
                if (push == 0)
                    n0 = idx;
                else
                    n1 = idx;
                ++push;
            }
        }
        if (push == 0) {
            if (sp == 0) break;
            node = stack[--sp];
        } else {
            node = n0;
            if (push == 2) {
                if (sp < kStack)
                    stack[sp++] = n1;
                else
                    atomicOr(t.err, kErrIndexOverflow);
            }
        }
    }
}

static_assert(scene_tree_cap<float>() <= 2u * kSceneTreeThreads && scene_tree_cap<double>() <= 2u * kSceneTreeThreads,
              "the fused offsets scan takes two bodies a thread");
// Fused write pass, part 1: the chunk's pair offsets.  base = pairs of the
// chunks whose bodies come first (chunks are contiguous body ranges),
// then a CTA-wide exclusive sum of the per-body counts: offsets[lo + p],
// the scan's prefix in excl[p], the count in cnt[p].  CTA 0 also stores the
// world's pair count (and the overflow flag), as k_pairs_total does.
__device__ __forceinline__ void fused_offsets(const TreeArgs& t, uint32_t lo, uint32_t nb, uint32_t* excl,
                                             uint32_t* cnt, uint32_t* s_red) {
    const uint32_t tid = threadIdx.x, nt = blockDim.x, lane = tid & 31u, warp = tid >> 5;
    unsigned long long before = 0, grand = 0;
    for (uint32_t c = tid; c < t.nchunks; c += nt) {
        const uint32_t tot = t.chunk_tot[c];
        grand += tot;
        if (t.scenes[t.chunks[c].x].body_lo < lo) before += tot;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        before += __shfl_xor_sync(0xFFFFFFFFu, before, o);
        grand += __shfl_xor_sync(0xFFFFFFFFu, grand, o);
    }
    unsigned long long* s_sum = reinterpret_cast<unsigned long long*>(s_red);  // 2 x 32 u64 (128 words)
    if (lane == 0) {
        s_sum[warp] = before;
        s_sum[32 + warp] = grand;
    }
    __syncthreads();
    before = grand = 0;
    for (uint32_t w = 0; w < nt / 32u; ++w) {
        before += s_sum[w];
        grand += s_sum[32 + w];
    }
    __syncthreads();
    if (blockIdx.x == 0 && tid == 0) {
        t.ctr->pairs = grand > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)grand;
        if (grand > t.cap) atomicOr(&t.ctr->error_flags, kErrPairOverflow);
    }
    // per-body counts, two consecutive bodies a thread
    const uint32_t p0 = 2u * tid;
    const uint32_t c0 = p0 < nb ? t.counts[lo + p0] : 0u, c1 = p0 + 1u < nb ? t.counts[lo + p0 + 1u] : 0u;
    uint32_t x = c0 + c1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31u) s_red[warp] = x;
    __syncthreads();
    uint32_t wofs = 0;
    for (uint32_t w = 0; w < warp; ++w) wofs += s_red[w];
    const uint32_t e0 = wofs + x - (c0 + c1);
    const uint32_t b32 = (uint32_t)before;
    if (p0 < nb) {
        excl[p0] = e0;
        cnt[p0] = c0;
        t.offsets[lo + p0] = b32 + e0;
    }
    if (p0 + 1u < nb) {
        excl[p0 + 1u] = e0 + c0;
        cnt[p0 + 1u] = c1;
        t.offsets[lo + p0 + 1u] = b32 + e0 + c0;
    }
    __syncthreads();
}

// Fused write pass, part 2: each body's partners (placed at its offsets in
// pb) sorted ascending -- up to 32 in registers by the body's thread, longer
// lists by the whole CTA (bitonic in `scratch`, the shared tree space) --
// then the pairs (body, partner) in (a, b) order.
__device__ __forceinline__ void fused_emit(const TreeArgs& t, uint32_t lo, uint32_t nb, const uint32_t* cnt,
                                          uint32_t* long_list, uint32_t* s_nlong, uint32_t* scratch,
                                          uint32_t scratch_words) {
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    if (tid == 0) *s_nlong = 0u;
    __syncthreads();
    for (uint32_t p = tid; p < nb; p += nt) {
        const uint32_t a = t.offsets[lo + p], len = cnt[p];
        if (len <= 1u || a + len > t.cap) continue;  // overflow is reported by the pair count
        if (len > 32u) {
            long_list[atomicAdd(s_nlong, 1u)] = p;
            continue;
        }
        uint32_t v[32];
        for (uint32_t k = 0; k < len; ++k) v[k] = t.pb[a + k];
        for (uint32_t k = 1; k < len; ++k) {
            const uint32_t x = v[k];
            int m = (int)k - 1;
            while (m >= 0 && v[m] > x) {
                v[m + 1] = v[m];
                --m;
            }
            v[m + 1] = x;
        }
        for (uint32_t k = 0; k < len; ++k) t.pb[a + k] = v[k];
    }
    __syncthreads();
    const uint32_t nlong = *s_nlong;
    for (uint32_t q = 0; q < nlong; ++q) {
        const uint32_t p = long_list[q];
        const uint32_t a = t.offsets[lo + p], len = cnt[p];
        uint32_t p2 = 1;
        while (p2 < len) p2 <<= 1;
        if (p2 > scratch_words) {  // cannot happen: a list is shorter than the chunk
            if (tid == 0) atomicOr(t.err, kErrIndexOverflow);
            continue;
        }
        for (uint32_t k = tid; k < p2; k += nt) scratch[k] = k < len ? t.pb[a + k] : 0xFFFFFFFFu;
        __syncthreads();
        for (uint32_t size = 2; size <= p2; size <<= 1) {
            for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
                for (uint32_t u = tid; u < p2 / 2u; u += nt) {
                    const uint32_t i = 2u * u - (u & (stride - 1u)), j = i + stride;
                    const uint32_t x = scratch[i], y = scratch[j];
                    if ((x > y) == ((i & size) == 0u)) {
                        scratch[i] = y;
                        scratch[j] = x;
                    }
                }
                __syncthreads();
            }
        }
        for (uint32_t k = tid; k < len; k += nt) t.pb[a + k] = scratch[k];
        __syncthreads();
    }
    for (uint32_t p = tid; p < nb; p += nt) {
        const uint32_t a = t.offsets[lo + p], len = cnt[p];
        for (uint32_t k = a; k < a + len && k < t.cap; ++k) t.pairs[k] = DioPair{lo + p, t.pb[k]};
    }
}

template <class R, bool WRITE>
__global__ void __launch_bounds__(kSceneTreeThreads)
    k_scene_tree(const A4<R>* aabb_min, const A4<R>* aabb_max, A4<R>* g_leaf_min, A4<R>* g_leaf_max,
                 A4<R>* g_node_min, A4<R>* g_node_max, TreeArgs t) {
    pdl_enter();
    extern __shared__ __align__(16) unsigned char tree_smem[];
    const uint32_t cidx = blockIdx.x;
    const uint2 chunk = t.chunks[cidx];  // scenes [x, y)
    const uint32_t lo = t.scenes[chunk.x].body_lo;
    const uint32_t nb = t.scenes[chunk.y - 1].body_hi - lo;
    const uint32_t cb = t.cap_bodies;
    if (nb > cb) {  // the host packs chunks within the cap
        if (threadIdx.x == 0) atomicOr(t.err, kErrIndexOverflow);
        return;
    }
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    uint32_t* s_cursor = reinterpret_cast<uint32_t*>(tree_smem);
    A4<R>* lmn = reinterpret_cast<A4<R>*>(tree_smem + 16);
    A4<R>* lmx = lmn + cb;
    A4<R>* nmn = lmx + cb;
    A4<R>* nmx = nmn + cb;
    uint2* ch = reinterpret_cast<uint2*>(nmx + cb);
    uint32_t* lpar = reinterpret_cast<uint32_t*>(ch + cb);
    uint32_t* npar = lpar + cb;
    uint32_t* vis = npar + cb;  // visit flags, then per-body pair counts
    uint32_t* lroot = vis + cb;
    // fused write pass: per-body prefix in lpar, count in npar (both unused
    // by the write pass), the long list in lroot once the trees are walked
    __shared__ uint32_t s_red[128];
    __shared__ uint32_t s_nlong;
    const bool fused = WRITE && t.fused;
    if (fused) fused_offsets(t, lo, nb, lpar, npar, s_red);
    if (WRITE && !t.chunk_ovf[cidx]) {
        // place the scratch pairs: body a's segment starts at offsets[a]
        for (uint32_t p = tid; p < nb; p += nt) vis[p] = 0u;
        __syncthreads();
        const uint32_t np = t.chunk_n[cidx];
        const uint2* src = t.scratch + (size_t)lo * t.scratch_k;
        for (uint32_t k = tid; k < np; k += nt) {
            const uint2 ab = src[k];
            const uint32_t pos = t.offsets[ab.x] + atomicAdd(&vis[ab.x - lo], 1u);
            if (pos < t.cap) t.pb[pos] = ab.y;
        }
        if (fused) {
            __syncthreads();
            fused_emit(t, lo, nb, npar, lroot, &s_nlong, reinterpret_cast<uint32_t*>(lmn),
                       (uint32_t)(cb * 2u * sizeof(A4<R>) / 4u));
        }
        return;
    }
    // slot p is leaf p of its scene and, except for a scene's last slot,
    // internal node (p - scene start) of that scene
    for (uint32_t p = tid; p < nb; p += nt) {
        const SceneDesc sc = t.scenes[t.scene_of_pos[lo + p]];
        const uint32_t root = sc.body_lo - lo, ns = sc.body_hi - sc.body_lo;
        const uint32_t b = t.leaf_body[lo + p];
        lroot[p] = ns >= 2 ? root : kNoRoot;
        if (WRITE) {
            lmn[p] = g_leaf_min[lo + p];
            lmx[p] = g_leaf_max[lo + p];
        } else {
            A4<R> a = aabb_min[b];
            const A4<R> c = aabb_max[b];
            a.w = tag_bits<R>(b);
            lmn[p] = a;
            lmx[p] = c;
            g_leaf_min[lo + p] = a;
            g_leaf_max[lo + p] = c;
            lpar[p] = ns >= 2 ? t.parent[t.n + lo + p] - lo : 0u;
        }
        if (lo + p + 1 < sc.body_hi) {  // internal node
            const uint2 c = t.children[lo + p];
            ch[p] = make_uint2((c.x & kLeafFlag) ? (((c.x & ~kLeafFlag) - lo) | kLeafFlag) : c.x - lo,
                               (c.y & kLeafFlag) ? (((c.y & ~kLeafFlag) - lo) | kLeafFlag) : c.y - lo);
            if (WRITE) {
                nmn[p] = g_node_min[lo + p];
                nmx[p] = g_node_max[lo + p];
            } else {
                npar[p] = p == root ? p : t.parent[lo + p] - lo;
                vis[p] = 0u;
            }
        }
    }
    if (!WRITE && tid == 0) *s_cursor = 0u;
    __syncthreads();
    if (!WRITE) {
        // bottom-up unions and highest leaf positions: the second arrival at
        // a node computes it
        for (uint32_t p = tid; p < nb; p += nt) {
            const uint32_t root = lroot[p];
            if (root == kNoRoot) continue;
            uint32_t node = lpar[p];
            for (uint32_t depth = 0; depth < nb; ++depth) {  // a path has < nb nodes
                __threadfence_block();
                if (atomicAdd(&vis[node], 1u) == 0) break;
                __threadfence_block();
                const uint2 c = ch[node];
                const uint32_t li = c.x & ~kLeafFlag, ri = c.y & ~kLeafFlag;
                const bool ll = c.x & kLeafFlag, rl = c.y & kLeafFlag;
                const A4<R> a0 = ll ? lmn[li] : nmn[li], a1 = ll ? lmx[li] : nmx[li];
                const A4<R> b0 = rl ? lmn[ri] : nmn[ri], b1 = rl ? lmx[ri] : nmx[ri];
                const uint32_t hi = max(ll ? li : tag_of(a1), rl ? ri : tag_of(b1));
                nmn[node] = A4<R>{fmin_(a0.x, b0.x), fmin_(a0.y, b0.y), fmin_(a0.z, b0.z),
                                  tag_bits<R>(children_word(c))};
                nmx[node] = A4<R>{fmax_(a1.x, b1.x), fmax_(a1.y, b1.y), fmax_(a1.z, b1.z), tag_bits<R>(hi)};
                if (node == root) break;
                node = npar[node];
            }
        }
        __syncthreads();
        for (uint32_t p = tid; p < nb; p += nt) {
            vis[p] = 0u;  // per-body pair counts from here on
            if (lroot[p] != kNoRoot && lo + p + 1 < t.scenes[t.scene_of_pos[lo + p]].body_hi) {
                g_node_min[lo + p] = nmn[p];
                g_node_max[lo + p] = nmx[p];
            }
        }
        __syncthreads();
    }
    const uint32_t region = nb * t.scratch_k;
    uint2* dst = t.scratch + (size_t)lo * t.scratch_k;
    for (uint32_t p = tid; p < nb; p += nt) {
        const uint32_t root = lroot[p];
        if (root == kNoRoot) continue;
        if (WRITE)
            tree_write_leaf<R>(p, root, lmn, lmx, nmn, nmx, ch, t);
        else
            tree_count_leaf<R>(p, root, lmn, lmx, nmn, nmx, vis, s_cursor, dst, region, lo, t.err);
    }
    if (!WRITE) {
        __syncthreads();
        for (uint32_t p = tid; p < nb; p += nt) t.counts[lo + p] = vis[p];
        if (tid == 0) {
            const uint32_t total = *s_cursor;
            t.chunk_n[cidx] = min(total, region);
            t.chunk_ovf[cidx] = total > region ? 1u : 0u;
            t.chunk_tot[cidx] = total;
        }
    }
    if (fused) {
        __syncthreads();
        fused_emit(t, lo, nb, npar, lroot, &s_nlong, reinterpret_cast<uint32_t*>(lmn),
                   (uint32_t)(cb * 2u * sizeof(A4<R>) / 4u));
    }
}

// ---- tree build of one chunk of scenes in one CTA ----
// The same trees as k_scene_bounds + k_morton + the global key sort +
// k_karras, for a world whose scenes all fit the shared-memory trees: per
// scene centroid bounds (shared-memory atomics), Morton keys, a sort of the
// chunk's keys in shared memory, and the Karras nodes from the sorted keys.
// The chunk's sorted order equals its slice of the global sort: scenes are
// consecutive body ranges and the scene index is the key's top field, so
// keys of the chunk sort among themselves.  Inside the CTA a key carries
// (scene - first scene of the chunk) in that field; the composite word
// (key << 32 | chunk position) is unique, so a bitonic network gives the
// stable order.
template <class R>
__host__ __device__ constexpr uint32_t chunk_build_pow2() { return scene_tree_cap<R>(); }
template <class R>
__host__ __device__ constexpr size_t chunk_build_bytes() {
    // sort words, then 6 bound words per scene (at most one scene per body),
    // reused for the sorted keys
    return (size_t)chunk_build_pow2<R>() * 8 + (size_t)scene_tree_cap<R>() * 24;
}
static_assert((scene_tree_cap<float>() & (scene_tree_cap<float>() - 1)) == 0 &&
                  (scene_tree_cap<double>() & (scene_tree_cap<double>() - 1)) == 0,
              "the chunk sort pads to a power of two no larger than the tree cap");

template <class R>
__global__ void __launch_bounds__(kSceneTreeThreads)
    k_chunk_build(const A4<R>* aabb_min, const A4<R>* aabb_max, const SceneDesc* scenes, const uint32_t* scene_of,
                  const uint2* chunks, uint32_t n, uint32_t cap_bodies, uint32_t scene_bits, uint32_t axis_bits,
                  uint32_t* keys_sorted, uint32_t* leaf_body, uint2* children, uint32_t* parent, uint32_t* err) {
    pdl_enter();
    extern __shared__ __align__(16) unsigned char build_smem[];
    const uint2 chunk = chunks[blockIdx.x];  // scenes [x, y)
    const uint32_t lo = scenes[chunk.x].body_lo;
    const uint32_t nb = scenes[chunk.y - 1].body_hi - lo;
    const uint32_t nsc = chunk.y - chunk.x;
    if (nb > cap_bodies || cap_bodies > chunk_build_pow2<R>()) {  // the host packs chunks within the cap
        if (threadIdx.x == 0) atomicOr(err, kErrIndexOverflow);
        return;
    }
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    unsigned long long* s_sort = reinterpret_cast<unsigned long long*>(build_smem);
    uint32_t* s_bounds = reinterpret_cast<uint32_t*>(s_sort + chunk_build_pow2<R>());
    for (uint32_t i = tid; i < nsc; i += nt) {
        s_bounds[6 * i + 0] = s_bounds[6 * i + 1] = s_bounds[6 * i + 2] = 0xFFFFFFFFu;
        s_bounds[6 * i + 3] = s_bounds[6 * i + 4] = s_bounds[6 * i + 5] = 0u;
    }
    __syncthreads();
    for (uint32_t p = tid; p < nb; p += nt) {
        float c[3];
        aabb_centre(aabb_min[lo + p], aabb_max[lo + p], c);
        const uint32_t ox = f2ord(c[0]), oy = f2ord(c[1]), oz = f2ord(c[2]);
        const uint32_t ls = scene_of[lo + p] - chunk.x;
        // lanes of one scene reduce first; their leader issues the atomics
        const uint32_t grp = __match_any_sync(__activemask(), ls);
        const uint32_t nx = __reduce_min_sync(grp, ox), ny = __reduce_min_sync(grp, oy),
                       nz = __reduce_min_sync(grp, oz);
        const uint32_t xx = __reduce_max_sync(grp, ox), xy = __reduce_max_sync(grp, oy),
                       xz = __reduce_max_sync(grp, oz);
        if ((tid & 31u) == (uint32_t)(__ffs(grp) - 1)) {
            uint32_t* bs = s_bounds + 6 * ls;
            atomicMin(&bs[0], nx);
            atomicMin(&bs[1], ny);
            atomicMin(&bs[2], nz);
            atomicMax(&bs[3], xx);
            atomicMax(&bs[4], xy);
            atomicMax(&bs[5], xz);
        }
    }
    __syncthreads();
    uint32_t p2 = 1;
    while (p2 < nb) p2 <<= 1;
    for (uint32_t p = tid; p < p2; p += nt) {
        unsigned long long word = ~0ull;  // padding sorts last
        if (p < nb) {
            float c[3];
            aabb_centre(aabb_min[lo + p], aabb_max[lo + p], c);
            const uint32_t ls = scene_of[lo + p] - chunk.x;
            const uint32_t code = morton_code(c, s_bounds + 6 * ls, axis_bits);
            const uint32_t key = scene_bits ? ((ls << (3 * axis_bits)) | code) : code;
            word = ((unsigned long long)key << 32) | p;
        }
        s_sort[p] = word;
    }
    __syncthreads();
    for (uint32_t size = 2; size <= p2; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t t = tid; t < p2 / 2; t += nt) {
                const uint32_t i = 2 * t - (t & (stride - 1)), j = i + stride;
                const unsigned long long a = s_sort[i], b = s_sort[j];
                if ((a > b) == ((i & size) == 0)) {
                    s_sort[i] = b;
                    s_sort[j] = a;
                }
            }
            __syncthreads();
        }
    }
    // sorted keys of the chunk (the bounds are no longer needed)
    uint32_t* s_key = s_bounds;
    const uint32_t key_base = scene_bits ? (chunk.x << (3 * axis_bits)) : 0u;
    for (uint32_t p = tid; p < nb; p += nt) {
        const unsigned long long word = s_sort[p];
        const uint32_t key = (uint32_t)(word >> 32);
        s_key[p] = key;
        keys_sorted[lo + p] = key + key_base;
        leaf_body[lo + p] = lo + (uint32_t)word;
    }
    __syncthreads();
    for (uint32_t p = tid; p < nb; p += nt) {
        const SceneDesc sc = scenes[scene_of[lo + p]];
        const int ns = (int)(sc.body_hi - sc.body_lo);
        const int k = (int)(lo + p - sc.body_lo);
        if (k >= ns - 1) continue;  // ns - 1 internal nodes
        karras_node(s_key + (sc.body_lo - lo), sc.body_lo, ns, k, n, children, parent);
    }
}

// sort each body's partner list ascending; short lists in-thread, long
// lists (> 32) by one CTA in shared memory (bitonic, up to 4096 entries)
static __global__ void k_bounds_init(uint32_t* b, uint32_t ns) {
    pdl_enter();
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        b[6 * s + 0] = b[6 * s + 1] = b[6 * s + 2] = 0xFFFFFFFFu;
        b[6 * s + 3] = b[6 * s + 4] = b[6 * s + 5] = 0u;
    }
}

static __global__ void k_sort_segments(const uint32_t* offsets, uint32_t n, uint32_t cap, uint32_t* pb, uint32_t* long_list,
                                uint32_t* long_count) {
    pdl_enter();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t a = offsets[i], b = offsets[i + 1];
        uint32_t len = b - a;
        if (len <= 1 || b > cap) continue;  // overflow is reported by the pair count
        if (len > 32) {
            long_list[warp_append(long_count)] = i;
            continue;
        }
        uint32_t v[32];
        for (uint32_t k = 0; k < len; ++k) v[k] = pb[a + k];
        for (uint32_t k = 1; k < len; ++k) {
            uint32_t x = v[k];
            int m = (int)k - 1;
            while (m >= 0 && v[m] > x) {
                v[m + 1] = v[m];
                --m;
            }
            v[m + 1] = x;
        }
        for (uint32_t k = 0; k < len; ++k) pb[a + k] = v[k];
    }
}

constexpr int kLongSort = 4096;

static __global__ void __launch_bounds__(512) k_sort_long(const uint32_t* offsets, uint32_t* pb, const uint32_t* long_list,
                                                   const uint32_t* long_count, uint32_t* err) {
    pdl_enter();
    __shared__ uint32_t s[kLongSort];
    uint32_t cnt = *long_count;
    for (uint32_t q = blockIdx.x; q < cnt; q += gridDim.x) {
        uint32_t i = long_list[q];
        uint32_t a = offsets[i], len = offsets[i + 1] - a;
        if (len > (uint32_t)kLongSort) {
            if (threadIdx.x == 0) atomicOr(err, kErrIndexOverflow);
            continue;
        }
        uint32_t p2 = 1;
        while (p2 < len) p2 <<= 1;
        for (uint32_t k = threadIdx.x; k < p2; k += blockDim.x) s[k] = k < len ? pb[a + k] : 0xFFFFFFFFu;
        __syncthreads();
        for (uint32_t size = 2; size <= p2; size <<= 1) {
            for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
                for (uint32_t t = threadIdx.x; t < p2; t += blockDim.x) {
                    uint32_t u = t ^ stride;
                    if (u > t) {
                        bool up = (t & size) == 0;
                        uint32_t x = s[t], y = s[u];
                        if ((x > y) == up) {
                            s[t] = y;
                            s[u] = x;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (uint32_t k = threadIdx.x; k < len; k += blockDim.x) pb[a + k] = s[k];
        __syncthreads();
    }
}

static __global__ void k_pairs_from_segments(const uint32_t* offsets, uint32_t n, const uint32_t* pb, DioPair* pairs,
                                      uint32_t cap) {
    pdl_enter();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (uint32_t k = offsets[i]; k < offsets[i + 1] && k < cap; ++k) pairs[k] = DioPair{i, pb[k]};
}

}  // namespace dio
