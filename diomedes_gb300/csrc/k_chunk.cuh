// k_chunk.cuh -- the whole AVBD solve of a step in one launch: one CTA per
// chunk of consecutive scenes, poses resident in shared memory.
//
// The reference dispatches init, then (primal, dual) x iterations, then
// recover as separate compute passes over every body and contact
// (engine/src/render/gpu_physics.rs:541-550), so every iteration re-reads
// every pose and row.  Scenes never couple -- rows and joints stay inside a
// scene -- so a chunk of whole scenes can run its whole schedule alone: its
// snapshot / new poses (both Jacobi parities) and step-start poses live in
// shared memory, the phases are separated by __syncthreads, and only the
// rows, joint views and per-body constants stream from L1 / L2 / HBM.  Each phase
// evaluates exactly the expressions of the per-phase kernels (the same
// device functions, reading shared instead of global memory), so the result
// is bit-identical to init, 10 x (primal, dual), recover launched one by one.
//
// Shared memory per body: pos[2], rot[2], init pos, init rot = 6 x A4<P>
// (96 B at FP32, 192 B at FP64 poses); a chunk holds at most
// solve_chunk_cap<P>() bodies (2048 / 1024), one CTA per SM.  The host packs
// scenes into chunks so that the chunks fill whole waves of the GPU's SMs.
// (Measured and dropped: 64 B per body with the step-start poses read from
// global memory, which let one wave of 152 chunks of up to 3391 bodies hold
// the bench batch, ran the solve 0.48 -> 0.59 ms: the step-start reads of
// contact rows and the smaller L1 cost more than the wave saved.  Also
// measured and dropped: forming each row's dual inside the next iteration's
// primal -- bit-identical, one barrier per iteration instead of two, duals
// of pair rows formed by both endpoints, a second dual buffer -- which ran
// 0.48 -> 0.59 ms (640 threads) and 0.50 -> 0.54 ms (512): the extra work
// and spills in the primal cost more than the barrier saved.)
#pragma once

#include "k_avbd.cuh"
#include "k_color.cuh"

namespace dio {

// threads per CTA: 512 (128 registers, no spill) or 640 (96 registers)
constexpr int kChunkThreads = 512;
constexpr int kChunkThreadsWide = 640;

template <class P>
__host__ __device__ constexpr size_t chunk_smem_bytes(uint32_t cap) {
    return (size_t)6 * cap * sizeof(A4<P>);
}
// bodies of a chunk: its poses fill at most 192 KB of shared memory
template <class P>
__host__ __device__ constexpr uint32_t solve_chunk_cap() {
    return sizeof(P) == 4 ? 2048u : 1024u;
}
static_assert(chunk_smem_bytes<float>(solve_chunk_cap<float>()) <= 200u * 1024u &&
                  chunk_smem_bytes<double>(solve_chunk_cap<double>()) <= 200u * 1024u,
              "scene-chunk poses must fit a CTA's shared memory");

// First index r in [s0, s1) with ab[r].x >= key (ab sorted by .x there), or
// s1; one warp, 32-way search (every lane must call it).
__device__ __forceinline__ uint32_t warp_lower_bound(const uint2* ab, uint32_t s0, uint32_t s1, uint32_t key) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t lo = s0, hi = s1;  // the answer lies in [lo, hi]
    while (hi - lo > 32) {
        const uint32_t step = (hi - lo + 31) / 32;
        const uint32_t probe = lo + lane * step;
        const bool less = probe < hi && ab[probe].x < key;
        const uint32_t k = __popc(__ballot_sync(0xFFFFFFFFu, less));  // probes below key form a prefix
        const uint32_t nlo = k ? lo + (k - 1) * step + 1 : lo;
        const uint32_t nhi = min(hi, lo + k * step);
        lo = nlo;
        hi = nhi;
    }
    const uint32_t probe = lo + lane;
    const bool less = probe < hi && ab[probe].x < key;
    return lo + __popc(__ballot_sync(0xFFFFFFFFu, less));
}

// One CTA per chunk (chunks[c] = scene range [x, y), bodies contiguous;
// dyn_runs[c] = the chunk's run of the dynamic-body list, ordered by work
// signature so a warp's bodies take the same code path).
// `cap` is the shared-memory capacity in bodies (the largest chunk).  Rows of the chunk: its
// pair rows are one range of the pair-row section (pairs sorted by body a,
// scenes contiguous) and its container rows one range of the container
// section (dynamic bodies in index order).
template <class P, class R, int T>
__global__ void __launch_bounds__(T, 1)
    k_solve_chunks(DevWorld<P, R> w, const uint2* chunks, const uint2* dyn_runs, const SceneDesc* scenes, uint32_t cap,
                   SolveParams<R> o) {
    extern __shared__ __align__(16) unsigned char chunk_smem[];
    __shared__ uint32_t s_rows[4];
    pdl_enter();
    // layout: pos parity 0, pos parity 1, rot parity 0, rot parity 1, step
    // start pos, step start rot (parity b at s_pos + b * cap)
    A4<P>* const s_pos = reinterpret_cast<A4<P>*>(chunk_smem);
    A4<P>* const s_rot = s_pos + 2 * cap;
    A4<P>* const s_ipos = s_pos + 4 * cap;
    A4<P>* const s_irot = s_pos + 5 * cap;
    const uint2 ch = chunks[blockIdx.x];
    const uint2 dr = dyn_runs[blockIdx.x];  // the chunk's dynamic bodies: w.dyn_list[dr.x, dr.y)
    const uint32_t lo = scenes[ch.x].body_lo, hi = scenes[ch.y - 1].body_hi;
    const uint32_t tid = threadIdx.x, nt = blockDim.x;

    // the chunk's row ranges, one warp per bound
    const uint32_t warp = tid >> 5;
    if (warp < 4) {
        const uint32_t m = w.ctr->rows;
        const uint32_t split = min(w.ctr->pair_rows, m);
        const uint32_t s0 = warp < 2 ? 0u : split, s1 = warp < 2 ? split : m;
        const uint32_t r = warp_lower_bound(w.ab, s0, s1, (warp & 1) ? hi : lo);
        if ((tid & 31) == 0) s_rows[warp] = r;
    }
    // avbd_init for the chunk's bodies (global state as the per-phase kernel
    // leaves it), then the poses of both parities and the step start into
    // shared memory: the same thread writes and reads a body's records
    for (uint32_t i = lo + tid; i < hi; i += nt) {
        init_body(w, i, o);
        s_pos[i - lo] = w.pos[0][i];
        s_rot[i - lo] = w.rot[0][i];
        s_pos[cap + i - lo] = w.pos[1][i];
        s_rot[cap + i - lo] = w.rot[1][i];
        s_ipos[i - lo] = w.init_pos[i];
        s_irot[i - lo] = w.init_rot[i];
    }
    __syncthreads();
    const uint32_t p0 = s_rows[0], p1 = s_rows[1], c0 = s_rows[2], c1 = s_rows[3];
    const uint32_t np = p1 - p0, nrows = np + (c1 - c0);
    for (uint32_t k = 0; k < o.iterations; ++k) {
        const uint32_t rd = (k & 1u) * cap, wr = cap - rd;
        const SmemFetch<P> f{s_pos + rd, s_rot + rd, s_ipos, s_irot, s_pos + wr, s_rot + wr, lo};
        for (uint32_t t = dr.x + tid; t < dr.y; t += nt) {
            const uint32_t i = w.dyn_list[t];
            const uint32_t k0 = w.n_joints ? w.joint_off[i] : 0u, k1 = w.n_joints ? w.joint_off[i + 1] : 0u;
            primal_body_f(w, i, k0, k1, o, f);
        }
        __syncthreads();
        const SmemFetch<P> fd{s_pos + wr, s_rot + wr, s_ipos, s_irot, nullptr, nullptr, lo};
        for (uint32_t t = tid; t < nrows; t += nt) dual_row_f(w, t < np ? p0 + t : c0 + (t - np), fd, o);
        __syncthreads();
    }
    // avbd_recover from the final parity, and the final pose into buffer 0
    const uint32_t fp = (o.iterations - 1u) % 2u;
    const uint32_t rb = fp == 0 ? 1u : 0u;
    const uint32_t fp_read = (o.iterations == 0 ? 0u : o.iterations - 1u) % 2u;
    const uint32_t final_buf = 1u - fp_read;
    const SmemFetch<P> fr{s_pos + rb * cap, s_rot + rb * cap, s_ipos, s_irot, nullptr, nullptr, lo};
    for (uint32_t i = lo + tid; i < hi; i += nt) {
        recover_body_f(w, i, fr, o);
        w.pos[0][i] = s_pos[final_buf * cap + i - lo];
        w.rot[0][i] = s_rot[final_buf * cap + i - lo];
    }
}

// ---------------------------------------------------------------------
// The coloured Gauss-Seidel schedule as one launch per step: each chunk
// colours its own dynamic bodies (the Jones-Plassmann rounds of k_color.cuh
// -- priority hash(index), ties by index, smallest colour free among the
// coloured neighbours -- with the colours in shared memory and a barrier
// between a round's selection and its assignment), sorts them by colour,
// then runs init, per iteration one in-place primal sweep per colour
// (barrier after each) and the dual, and recover.  One pose buffer (the
// sweeps are in place): 4 x A4<P> per body plus colour, order and selection
// arrays.  The colouring of a disconnected graph is the union of its
// components' colourings, so per-chunk rounds give the colours of the
// whole-world rounds; results equal the host-driven coloured step bit for
// bit.

template <class P>
__host__ __device__ constexpr size_t chunk_colored_smem_bytes(uint32_t cap) {
    return (size_t)4 * cap * sizeof(A4<P>) + (size_t)cap * (4 + 4 + 4) + (size_t)2 * (kMaxColors + 1) * 4;
}

constexpr uint32_t kChunkColorRounds = 4096;  // Jones-Plassmann rounds before giving up

template <class P, class R, int T>
__global__ void __launch_bounds__(T, 1)
    k_solve_chunks_colored(DevWorld<P, R> w, const uint2* chunks, const uint2* dyn_runs, const SceneDesc* scenes,
                           uint32_t cap, SolveParams<R> o) {
    extern __shared__ __align__(16) unsigned char chunk_smem[];
    __shared__ uint32_t s_rows[4];
    __shared__ uint32_t s_colored, s_ncolors;
    pdl_enter();
    A4<P>* const s_pos = reinterpret_cast<A4<P>*>(chunk_smem);
    A4<P>* const s_rot = s_pos + cap;
    A4<P>* const s_ipos = s_pos + 2 * cap;
    A4<P>* const s_irot = s_pos + 3 * cap;
    uint32_t* const s_color = reinterpret_cast<uint32_t*>(s_pos + 4 * cap);
    uint32_t* const s_order = s_color + cap;
    uint32_t* const s_sel = s_order + cap;
    uint32_t* const s_cstart = s_sel + cap;          // kMaxColors + 1
    uint32_t* const s_cursor = s_cstart + kMaxColors + 1;
    const uint2 ch = chunks[blockIdx.x];
    const uint2 dr = dyn_runs[blockIdx.x];
    const uint32_t lo = scenes[ch.x].body_lo, hi = scenes[ch.y - 1].body_hi;
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    const uint32_t warp = tid >> 5;
    if (warp < 4) {
        const uint32_t m = w.ctr->rows;
        const uint32_t split = min(w.ctr->pair_rows, m);
        const uint32_t s0 = warp < 2 ? 0u : split, s1 = warp < 2 ? split : m;
        const uint32_t r = warp_lower_bound(w.ab, s0, s1, (warp & 1) ? hi : lo);
        if ((tid & 31) == 0) s_rows[warp] = r;
    }
    if (tid == 0) {
        s_colored = 0;
        s_ncolors = 0;
    }
    for (uint32_t c = tid; c <= kMaxColors; c += nt) {
        s_cstart[c] = 0;
        s_cursor[c] = 0;
    }
    // init (the in-place schedule reads and writes buffer 0) and colours reset
    for (uint32_t i = lo + tid; i < hi; i += nt) {
        init_body(w, i, o);
        s_pos[i - lo] = w.pos[0][i];
        s_rot[i - lo] = w.rot[0][i];
        s_ipos[i - lo] = w.init_pos[i];
        s_irot[i - lo] = w.init_rot[i];
        s_color[i - lo] = kNoColor;
    }
    __syncthreads();
    // Jones-Plassmann rounds over the chunk's dynamic bodies
    const uint32_t ndyn = dr.y - dr.x;
    uint32_t rounds = 0;
    while (s_colored < ndyn) {
        if (++rounds > kChunkColorRounds) {
            if (tid == 0) atomicOr(&w.ctr->error_flags, kErrColorOverflow);
            break;
        }
        for (uint32_t t = dr.x + tid; t < dr.y; t += nt) {
            const uint32_t v = w.dyn_list[t];
            bool sel = false;
            if (s_color[v - lo] == kNoColor) {
                sel = true;
                for_each_neighbour(w, v, [&](uint32_t u) {
                    if (sel && s_color[u - lo] == kNoColor && !color_beats(v, u)) sel = false;
                });
            }
            s_sel[v - lo] = sel ? 1u : 0u;
        }
        __syncthreads();
        for (uint32_t t = dr.x + tid; t < dr.y; t += nt) {
            const uint32_t v = w.dyn_list[t];
            if (!s_sel[v - lo]) continue;
            unsigned long long used[kMaxColors / 64] = {0ull, 0ull, 0ull, 0ull};
            for_each_neighbour(w, v, [&](uint32_t u) {
                const uint32_t c = s_color[u - lo];
                if (c < kMaxColors) used[c >> 6] |= 1ull << (c & 63);
            });
            uint32_t c = kMaxColors;
            for (uint32_t q = 0; q < kMaxColors / 64; ++q)
                if (~used[q]) {
                    c = q * 64 + (__ffsll(~used[q]) - 1);
                    break;
                }
            if (c >= kMaxColors) {
                atomicOr(&w.ctr->error_flags, kErrColorOverflow);
                c = kMaxColors - 1;
            }
            s_color[v - lo] = c;
            atomicAdd(&s_colored, 1u);
            atomicMax(&s_ncolors, c + 1);
        }
        __syncthreads();
    }
    const uint32_t ncolors = s_ncolors;
    // colours out, and the chunk's dynamic bodies sorted by colour
    for (uint32_t i = lo + tid; i < hi; i += nt) w.color[i] = s_color[i - lo];
    if (tid == 0) atomicMax(&w.ctr->colors, ncolors);
    for (uint32_t t = dr.x + tid; t < dr.y; t += nt) {
        const uint32_t c = s_color[w.dyn_list[t] - lo];
        if (c < kMaxColors) atomicAdd(&s_cstart[c + 1], 1u);
    }
    __syncthreads();
    if (tid == 0)
        for (uint32_t c = 0; c < ncolors; ++c) s_cstart[c + 1] += s_cstart[c];
    __syncthreads();
    for (uint32_t t = dr.x + tid; t < dr.y; t += nt) {
        const uint32_t v = w.dyn_list[t];
        const uint32_t c = s_color[v - lo];
        if (c < kMaxColors) s_order[s_cstart[c] + atomicAdd(&s_cursor[c], 1u)] = v;
    }
    __syncthreads();
    const uint32_t p0 = s_rows[0], p1 = s_rows[1], c0 = s_rows[2], c1 = s_rows[3];
    const uint32_t np = p1 - p0, nrows = np + (c1 - c0);
    const SmemFetch<P> f{s_pos, s_rot, s_ipos, s_irot, s_pos, s_rot, lo};  // in place
    for (uint32_t k = 0; k < o.iterations; ++k) {
        for (uint32_t c = 0; c < ncolors; ++c) {
            for (uint32_t t = s_cstart[c] + tid; t < s_cstart[c + 1]; t += nt) {
                const uint32_t i = s_order[t];
                const uint32_t k0 = w.n_joints ? w.joint_off[i] : 0u, k1 = w.n_joints ? w.joint_off[i + 1] : 0u;
                primal_body_f(w, i, k0, k1, o, f);
            }
            __syncthreads();
        }
        for (uint32_t t = tid; t < nrows; t += nt) dual_row_f(w, t < np ? p0 + t : c0 + (t - np), f, o);
        __syncthreads();
    }
    for (uint32_t i = lo + tid; i < hi; i += nt) {
        recover_body_f(w, i, f, o);
        w.pos[0][i] = s_pos[i - lo];
        w.rot[0][i] = s_rot[i - lo];
    }
}

}  // namespace dio
