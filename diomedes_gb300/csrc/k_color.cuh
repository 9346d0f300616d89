// k_color.cuh -- deterministic graph colouring of the dynamic bodies and
// per-colour body lists for the Gauss-Seidel primal sweep.
//
// No reference counterpart: the reference primal is a Jacobi sweep
// (engine/gpu_physics/avbd/src/lib.rs:6-9).  Jones-Plassmann rounds over the
// body graph whose edges are contact rows and joints between two dynamic
// bodies: priority = hash(index), ties broken by index; every uncoloured
// body that beats all its uncoloured neighbours takes the smallest colour
// no coloured neighbour holds.  Selected bodies form an independent set, so
// a round's result does not depend on thread order.
#pragma once

#include "engine.cuh"

namespace dio {

constexpr uint32_t kNoColor = 0xFFFFFFFFu;
constexpr uint32_t kMaxColors = 256;

__device__ __forceinline__ uint32_t color_hash(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

__device__ __forceinline__ bool color_beats(uint32_t v, uint32_t u) {
    uint32_t pv = color_hash(v), pu = color_hash(u);
    return pv > pu || (pv == pu && v > u);
}

// visit every dynamic neighbour of body i (rows, then joints)
template <class P, class R, class F>
__device__ __forceinline__ void for_each_neighbour(const DevWorld<P, R>& w, uint32_t i, F&& f) {
    for (uint32_t j = w.row_off[i]; j < w.row_off[i + 1]; ++j) {
        uint32_t oth = w.row_oth[j];
        if (oth == kContainer) continue;
        uint32_t u = oth & ~kIsB;
        if (u != i && w.inv[u].w != R(0)) f(u);
    }
    if (w.n_joints)
        for (uint32_t k = w.joint_off[i]; k < w.joint_off[i + 1]; ++k) {
            uint32_t u = w.jview[k].other;
            if (u != i && w.inv[u].w != R(0)) f(u);
        }
}

template <class P, class R>
__global__ void k_color_init(DevWorld<P, R> w) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x)
        w.color[i] = kNoColor;
}

// selection: sel[i] = 1 when i is uncoloured and beats every uncoloured neighbour
template <class P, class R>
__global__ void k_color_select(DevWorld<P, R> w, uint32_t* sel) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < w.n_dyn; t += gridDim.x * blockDim.x) {
        uint32_t v = w.dyn_list[t];
        bool s = false;
        if (w.color[v] == kNoColor) {
            s = true;
            for_each_neighbour(w, v, [&](uint32_t u) {
                if (s && w.color[u] == kNoColor && !color_beats(v, u)) s = false;
            });
        }
        sel[v] = s ? 1u : 0u;
    }
}

// assignment: a selected body takes the smallest colour unused by its
// (previously) coloured neighbours; no neighbour of a selected body is
// selected, so writing in place is race-free
template <class P, class R>
__global__ void k_color_assign(DevWorld<P, R> w, const uint32_t* sel) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < w.n_dyn; t += gridDim.x * blockDim.x) {
        uint32_t v = w.dyn_list[t];
        if (!sel[v]) continue;
        unsigned long long used[kMaxColors / 64] = {0ull, 0ull, 0ull, 0ull};
        for_each_neighbour(w, v, [&](uint32_t u) {
            uint32_t c = w.color[u];
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
        w.color[v] = c;
        atomicSub(&w.ctr->color_remaining, 1u);
        atomicMax(&w.ctr->colors, c + 1);
    }
}

// counting sort of the dynamic bodies by colour (order inside a colour is
// irrelevant: its bodies are independent)
template <class P, class R>
__global__ void k_color_hist(DevWorld<P, R> w, uint32_t* hist) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < w.n_dyn; t += gridDim.x * blockDim.x) {
        uint32_t c = w.color[w.dyn_list[t]];
        if (c < kMaxColors) atomicAdd(&hist[c], 1u);
    }
}

template <class P, class R>
__global__ void k_color_fill(DevWorld<P, R> w, uint32_t* cursor) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < w.n_dyn; t += gridDim.x * blockDim.x) {
        uint32_t v = w.dyn_list[t];
        uint32_t c = w.color[v];
        if (c < kMaxColors) w.color_order[w.color_off[c] + atomicAdd(&cursor[c], 1u)] = v;
    }
}

}  // namespace dio
