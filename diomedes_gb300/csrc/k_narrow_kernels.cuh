// k_narrow_kernels.cuh -- narrowphase_main (narrowphase/src/lib.rs:89-158)
// split into three stages: per-pair SAT / sphere, per-pair GJK, per-warp EPA.
#pragma once

#include "k_rows.cuh"

namespace dio {

template <class R>
__device__ __forceinline__ void put_slot(Slot<R>* s, uint32_t a, uint32_t b, V3<R> n, R depth, V3<R> pa, V3<R> pb) {
    Slot<R> o;
    o.valid = 1;
    o.a = a;
    o.b = b;
    o.pad = 0;
    o.normal = pack(n);
    o.depth = depth;
    o.pad2[0] = o.pad2[1] = o.pad2[2] = R(0);
    o.pa = pack(pa);
    o.pb = pack(pb);
    *s = o;
}

template <class R>
__device__ __forceinline__ void clear_slot(Slot<R>* s) {
    Slot<R> o;
    o.valid = 0;
    o.a = o.b = o.pad = 0;
    o.normal = A4<R>{R(0), R(0), R(0), R(0)};
    o.depth = R(0);
    o.pad2[0] = o.pad2[1] = o.pad2[2] = R(0);
    o.pa = o.normal;
    o.pb = o.normal;
    *s = o;
}

// Stage 1: one thread per pair.  `np_dev` (device pair count) bounds the
// work when non-null, so the launch does not depend on a host read.
template <class P, class R>
__global__ void __launch_bounds__(128) k_narrow_main(DevWorld<P, R> w, const uint32_t* np_dev, uint32_t np_cap) {
    pdl_enter();
    uint32_t np = np_dev ? min(*np_dev, np_cap) : np_cap;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        Slot<R>* slots = w.slots + (size_t)p * w.per_pair;
        for (uint32_t k = 0; k < w.per_pair; ++k) clear_slot(&slots[k]);
        DioPair pr = w.pairs[p];
        if (pr.a >= w.n || pr.b >= w.n) {
            atomicOr(&w.ctr->error_flags, kErrBadIndex);
            continue;
        }
        NB<R> a = load_nb(w, pr.a);
        NB<R> b = load_nb(w, pr.b);
        bool a_box = a.shape.tag == DIO_SHAPE_CUBE || a.shape.tag == DIO_SHAPE_BOX;
        bool b_box = b.shape.tag == DIO_SHAPE_CUBE || b.shape.tag == DIO_SHAPE_BOX;
        if (a_box && b_box) {
            Manifold<R> m;
            if (collide_manifold(a, b, w.per_pair, m))
                for (uint32_t k = 0; k < m.count; ++k) put_slot(&slots[k], pr.a, pr.b, m.normal, m.depth, m.pa[k], m.pb[k]);
        } else if (a.shape.tag == DIO_SHAPE_SPHERE && b.shape.tag == DIO_SHAPE_SPHERE) {
            V3<R> delta = sub(b.pos, a.pos);
            R dist = length(delta);
            R radius = a.shape.c[0].x + b.shape.c[0].x;
            if (!(dist >= radius || dist <= R(1.1920928955078125e-7))) {
                V3<R> n = divs(delta, dist);
                put_slot(&slots[0], pr.a, pr.b, n, radius - dist, add(a.pos, scale(n, a.shape.c[0].x)),
                         sub(b.pos, scale(n, b.shape.c[0].x)));
            }
        } else {
            const uint32_t e = warp_append(&w.ctr->gjk_work);
            w.gjk_list[e] = p;
        }
    }
}

// Stage 2: GJK, one thread per queued pair; intersecting pairs queue their
// simplex (4 points then 4 witnesses) for EPA.
template <class P, class R>
__global__ void __launch_bounds__(128) k_gjk(DevWorld<P, R> w) {
    pdl_enter();
    uint32_t nw = w.ctr->gjk_work;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < nw; e += gridDim.x * blockDim.x) {
        uint32_t p = w.gjk_list[e];
        DioPair pr = w.pairs[p];
        NB<R> a = load_nb(w, pr.a);
        NB<R> b = load_nb(w, pr.b);
        Simplex<R> s;
        if (gjk(a, b, w.hull, s)) {
            const uint32_t q = warp_append(&w.ctr->epa_work);
            w.epa_list[q] = p;
            A4<R>* dst = w.simplex + (size_t)q * 8;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                dst[k] = pack(s.p[k]);
                dst[4 + k] = pack(s.w[k]);
            }
        }
    }
}

// ---- bulk (TMA) copies global -> shared with mbarrier completion ----
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded, warp-uniform wait: every lane polls until all lanes have seen the
// phase complete, at most `tries` rounds; the result is the same in all lanes
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* bar, uint32_t parity, uint32_t tries) {
    bool done = false;
    for (uint32_t k = 0; k < tries; ++k) {
        if (!done) done = mbar_try_wait(bar, parity);
        if (__all_sync(0xFFFFFFFFu, done)) return true;
    }
    return __all_sync(0xFFFFFFFFu, done);
}

constexpr uint32_t kHullStage = 64;  // vertices per hull staged in shared memory
constexpr uint32_t kEpaWaitPolls = 1u << 20;  // rounds of the bounded waits for the hull copies

// Stage 3: EPA, one warp per queued pair, polytope in shared memory.  Hull
// vertex lists (both bodies, up to 64 vertices each) are staged into the
// warp's shared memory with bulk TMA copies, so the support queries of the
// expansion read shared memory.
template <class P, class R>
__global__ void __launch_bounds__(32 * epa_warps<R>(), 4) k_epa(DevWorld<P, R> w) {
    pdl_enter();
    constexpr int kEpaWarps = epa_warps<R>();
    __shared__ EpaSmem<R> smem[kEpaWarps];
    __shared__ A4<R> hull_s[kEpaWarps][2 * kHullStage];
    __shared__ uint64_t mbar[kEpaWarps];
    const uint32_t warp = threadIdx.x >> 5;
    const uint32_t lane = threadIdx.x & 31;
    EpaSmem<R>& S = smem[warp];
    if (lane == 0) mbar_init(&mbar[warp], 1);
    __syncwarp();
    uint32_t parity = 0;
    uint32_t nw = w.ctr->epa_work;
    for (uint32_t q = blockIdx.x * kEpaWarps + warp; q < nw; q += gridDim.x * kEpaWarps) {
        uint32_t p = w.epa_list[q];
        DioPair pr = w.pairs[p];
        NB<R> a = load_nb(w, pr.a);
        NB<R> b = load_nb(w, pr.b);
        const A4<R>* hull = w.hull;
        const bool ha = a.shape.tag == DIO_SHAPE_HULL, hb = b.shape.tag == DIO_SHAPE_HULL;
        const bool fits = (!ha || (a.shape.hc > 0 && a.shape.hc <= kHullStage)) &&
                          (!hb || (b.shape.hc > 0 && b.shape.hc <= kHullStage));
        if ((ha || hb) && fits && w.hull) {
            if (lane == 0) {
                // order the previous pair's shared-memory reads before the async writes
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                const uint32_t bytes = (ha ? a.shape.hc : 0u) * (uint32_t)sizeof(A4<R>) +
                                       (hb ? b.shape.hc : 0u) * (uint32_t)sizeof(A4<R>);
                mbar_expect_tx(&mbar[warp], bytes);
                if (ha) bulk_g2s(&hull_s[warp][0], w.hull + a.shape.hf, a.shape.hc * sizeof(A4<R>), &mbar[warp]);
                if (hb)
                    bulk_g2s(&hull_s[warp][kHullStage], w.hull + b.shape.hf, b.shape.hc * sizeof(A4<R>),
                             &mbar[warp]);
            }
            bool done = mbar_wait_warp(&mbar[warp], parity, w.epa_wait_polls);
            if (!done) {
                if (lane == 0) atomicOr(&w.ctr->error_flags, kErrTimeout);
                done = mbar_wait_warp(&mbar[warp], parity, kEpaWaitPolls);  // let the copies land
                if (!done) {
                    // the copies still have not landed: take no further pair
                    // (the step already reports DIO_ERR_TIMEOUT) and keep
                    // this warp, and so its CTA's shared memory, resident
                    // for one last, longer bounded wait before exiting
                    mbar_wait_warp(&mbar[warp], parity, 16u * kEpaWaitPolls);
                    return;  // warp-uniform
                }
            }
            parity ^= 1u;
            hull = &hull_s[warp][0];
            if (ha) a.shape.hf = 0;
            if (hb) b.shape.hf = kHullStage;
        }
        V3<R> n, pa, pb;
        R depth;
        bool ok = epa_warp(S, a, b, w.simplex + (size_t)q * 8, hull, &w.ctr->error_flags, n, depth, pa, pb);
        if (ok && lane == 0) put_slot(&w.slots[(size_t)p * w.per_pair], pr.a, pr.b, n, depth, pa, pb);
        __syncwarp();
    }
}

}  // namespace dio
