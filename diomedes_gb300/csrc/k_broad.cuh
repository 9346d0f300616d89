// k_broad.cuh -- broad phase on sm_103a.
//
// Restates engine/gpu_physics/broadphase/src/lib.rs:116-216 (support AABB,
// closed-interval overlap).  The reference appends overlapping (i, j) pairs
// through an atomic counter, so its order is arbitrary; here the pair list is
// produced in (a, b) order: a count pass, an exclusive scan and a write pass
// that visits j in ascending order.  Pairs never cross scene boundaries.
#pragma once

#include "k_narrow.cuh"
#include "k_rows.cuh"

namespace dio {

// aabb, broadphase/src/lib.rs:121-151
template <class R>
__device__ __forceinline__ void body_aabb(const NB<R>& b, const A4<R>* hull, V3<R>& mn, V3<R>& mx) {
    auto ws = [&](V3<R> d) {
        V3<R> local = rotate(conj(b.rot), d);
        return add(rotate(b.rot, support(b.shape, local, hull)), b.pos);
    };
    const V3<R> X{R(1), R(0), R(0)}, Y{R(0), R(1), R(0)}, Z{R(0), R(0), R(1)};
    mn = b.pos;
    mx = b.pos;
    V3<R> sx = ws(X), snx = ws(neg(X)), sy = ws(Y), sny = ws(neg(Y)), sz = ws(Z), snz = ws(neg(Z));
    if (sx.x > mx.x) mx.x = sx.x;
    if (snx.x < mn.x) mn.x = snx.x;
    if (sy.y > mx.y) mx.y = sy.y;
    if (sny.y < mn.y) mn.y = sny.y;
    if (sz.z > mx.z) mx.z = sz.z;
    if (snz.z < mn.z) mn.z = snz.z;
}

template <class P, class R>
__global__ void k_aabb(DevWorld<P, R> w, uint32_t lo, uint32_t hi) {
    pdl_enter();
    for (uint32_t i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += gridDim.x * blockDim.x) {
        NB<R> b = load_nb(w, i);
        V3<R> mn, mx;
        body_aabb(b, w.hull, mn, mx);
        w.aabb_min[i] = pack(mn);
        w.aabb_max[i] = pack(mx);
    }
}

template <class R>
__device__ __forceinline__ bool overlap(const A4<R>& mna, const A4<R>& mxa, const A4<R>& mnb, const A4<R>& mxb) {
    return mna.x <= mxb.x && mnb.x <= mxa.x && mna.y <= mxb.y && mnb.y <= mxa.y && mna.z <= mxb.z &&
           mnb.z <= mxa.z;
}

// Dense sweep, broad_sweep_dense (broadphase/src/lib.rs:171-216): body i
// tests j in (i, scene_hi).  The CTA stages tiles of candidate AABBs in
// shared memory; with write == false it only counts.
template <class P, class R, int kBlock>
__global__ void __launch_bounds__(kBlock) k_dense(DevWorld<P, R> w, uint32_t lo, uint32_t hi, uint32_t* counts,
                                                  const uint32_t* offsets, bool write_out) {
    __shared__ A4<R> smn[kBlock];
    __shared__ A4<R> smx[kBlock];
    const uint32_t i = lo + blockIdx.x * kBlock + threadIdx.x;
    const bool live = i < hi;
    uint32_t s_hi = 0;
    A4<R> mni{}, mxi{};
    if (live) {
        s_hi = w.scenes[w.scene[i]].body_hi;
        mni = w.aabb_min[i];
        mxi = w.aabb_max[i];
    }
    // tiles cover j from the block's first body + 1 to the block's largest scene end
    uint32_t blk_first = lo + blockIdx.x * kBlock;
    uint32_t tile_end = s_hi;
    for (int off = 16; off > 0; off >>= 1) tile_end = max(tile_end, __shfl_xor_sync(0xFFFFFFFFu, tile_end, off));
    __shared__ uint32_t warp_max[kBlock / 32];
    if ((threadIdx.x & 31) == 0) warp_max[threadIdx.x >> 5] = tile_end;
    __syncthreads();
    tile_end = 0;
    for (int k = 0; k < kBlock / 32; ++k) tile_end = max(tile_end, warp_max[k]);
    uint32_t cnt = 0;
    uint32_t out = (live && write_out) ? offsets[i - lo] : 0;
    for (uint32_t t0 = blk_first + 1; t0 < tile_end; t0 += kBlock) {
        __syncthreads();
        uint32_t j = t0 + threadIdx.x;
        if (j < tile_end) {
            smn[threadIdx.x] = w.aabb_min[j];
            smx[threadIdx.x] = w.aabb_max[j];
        }
        __syncthreads();
        if (live) {
            uint32_t jend = min(tile_end - t0, (uint32_t)kBlock);
            for (uint32_t k = 0; k < jend; ++k) {
                uint32_t jj = t0 + k;
                if (jj <= i || jj >= s_hi) continue;
                if (overlap(mni, mxi, smn[k], smx[k])) {
                    if (write_out) {
                        if (out < w.max_pairs) w.pairs[out] = DioPair{i, jj};
                        ++out;
                    } else {
                        ++cnt;
                    }
                }
            }
        }
    }
    if (live && !write_out) counts[i - lo] = cnt;
}

}  // namespace dio
