// noalloc.cu -- dio_avbd_solve_noalloc: the AVBD solve without allocation.
//
// Who needs it: callers that cannot call cudaMalloc at the point where they
// step the solver -- a host that hands this library device memory owned by
// another allocator (a game engine's or framework's pool), or a real-time
// loop that is forbidden to allocate once it runs.  They pass device
// pointers for every input and output; the solver's scratch (ping-pong
// poses, step-start and inertial targets, unpacked rows, the CSR other-body
// array) lives in one file-scope device array below, which every GPU that
// loads this library holds until the process exits.
//
// Limits: at most kNaMaxBodies bodies, kNaMaxContacts contact rows and
// kNaMaxJoints joints per call (the reference renderer's own capacities are
// 1024 bodies and 16384 contacts).  Every call shares the one array and it
// keeps the last call's contents, so calls that overlap on the GPU (two
// streams, two host threads) race; serialise them.  The first call on each
// device looks up the array's device address (cudaGetSymbolAddress) with
// that device current; make that first call before any stream capture.  The
// address is cached per device together with the id of the CUDA context it
// belongs to, and looked up again when the current context is a different
// one (after cudaDeviceReset, say), so a stale address is never used.
// The call is synchronous: it waits on the caller's stream twice (once to
// validate the caller's indices before any kernel dereferences them, once at
// the end to read the device error flags).
#include <cuda.h>  // driver types only: the two entry points are fetched at run time
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/dio_cuda.h"
#include "k_avbd.cuh"

namespace {

using namespace dio;

constexpr uint32_t kNaMaxBodies = 4096;
constexpr uint32_t kNaMaxContacts = 16384;
constexpr uint32_t kNaMaxJoints = 4096;
constexpr int kNaMaxDevices = 64;

// scratch layout (byte offsets into the array)
constexpr size_t kB4 = sizeof(A4<float>) * kNaMaxBodies;  // one per-body A4 array
constexpr size_t kOffPose = 0;                            // pos[2], rot[2], init x2, inert x2, vel, ang, prev, inv
constexpr size_t kNumBodyA4 = 12;
constexpr size_t kOffFric = kOffPose + kNumBodyA4 * kB4;
constexpr size_t kOffRs = kOffFric + sizeof(float) * kNaMaxBodies;
constexpr size_t kOffRd = kOffRs + sizeof(RowStatic<float>) * kNaMaxContacts;
constexpr size_t kOffAb = kOffRd + sizeof(RowDual<float, float>) * kNaMaxContacts;
constexpr size_t kOffOth = kOffAb + sizeof(uint2) * kNaMaxContacts;
constexpr size_t kOffCtr = kOffOth + sizeof(uint32_t) * 2 * kNaMaxContacts;
constexpr size_t kNaScratchBytes = (kOffCtr + sizeof(Counters) + 255) & ~size_t(255);

static __device__ __align__(256) unsigned char dio_noalloc_scratch[kNaScratchBytes];

// per device: the array's address and the id of the context it belongs to
struct ScratchEntry {
    unsigned long long ctx = 0;
    void* ptr = nullptr;
};
ScratchEntry g_scratch[kNaMaxDevices];
std::mutex g_mu;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// id of the calling thread's current context (cuCtxGetCurrent + cuCtxGetId,
// fetched from the driver through the runtime, so the library does not link
// the driver library); false when there is none yet or the driver lacks them
bool current_context_id(unsigned long long* id) {
    static std::once_flag once;
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
    });
    if (!get_current || !get_id) return false;
    CUcontext c = nullptr;
    if (get_current(&c) != CUDA_SUCCESS || !c) return false;
    return get_id(c, id) == CUDA_SUCCESS;
}

// The device address of the scratch array for the current device and
// context.  Host code cannot use the array's name as a device address; the
// address comes from cudaGetSymbolAddress with the device current.
int scratch_ptr(unsigned char** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return DIO_ERR_CUDA;
    unsigned long long ctx = 0;
    const bool known = current_context_id(&ctx);
    std::lock_guard<std::mutex> lk(g_mu);
    ScratchEntry& e = g_scratch[dev];
    if (known && e.ptr && e.ctx == ctx) {
        *out = static_cast<unsigned char*>(e.ptr);
        return DIO_OK;
    }
    // first call on this device, a different context, or no context current
    // yet: look the address up (which makes the device's context current)
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, dio_noalloc_scratch) != cudaSuccess || !p) return DIO_ERR_CUDA;
    unsigned long long now = 0;
    if (current_context_id(&now))
        e = ScratchEntry{now, p};
    else
        e = ScratchEntry{};  // without a context id nothing is cached: every call asks again
    *out = static_cast<unsigned char*>(p);
    return DIO_OK;
}

__global__ void k_na_unpack(DevWorld<float, float> w, const DioBodyState* st, const float* pos3, const float* quat4,
                            uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const DioBodyState s = st[i];
        w.vel[i] = A4<float>{s.vel[0], s.vel[1], s.vel[2], 0.f};
        w.ang[i] = A4<float>{s.ang[0], s.ang[1], s.ang[2], 0.f};
        w.prev_vel[i] = A4<float>{s.prev_vel[0], s.prev_vel[1], s.prev_vel[2], 0.f};
        w.inv[i] = A4<float>{s.inv_moment[0], s.inv_moment[1], s.inv_moment[2], s.inv_mass};
        w.friction[i] = s.friction;
        w.pos[0][i] = A4<float>{pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2], 0.f};
        w.rot[0][i] = A4<float>{quat4[4 * i], quat4[4 * i + 1], quat4[4 * i + 2], quat4[4 * i + 3]};
    }
}

__global__ void k_na_rows(DevWorld<float, float> w, const DioContact* c, uint32_t m, uint32_t n) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        const DioContact x = c[r];
        RowStatic<float> s;
        s.n = A4<float>{x.normal[0], x.normal[1], x.normal[2], x.friction};
        s.t1 = A4<float>{x.tangent1[0], x.tangent1[1], x.tangent1[2], x.c0[2]};
        s.t2 = A4<float>{x.tangent2[0], x.tangent2[1], x.tangent2[2], 0.f};
        s.ra = A4<float>{x.r_a[0], x.r_a[1], x.r_a[2], x.c0[0]};
        s.rb = A4<float>{x.r_b[0], x.r_b[1], x.r_b[2], x.c0[1]};
        w.rs[r] = s;
        RowDual<float, float> d;
        d.penalty = A4<float>{x.penalty[0], x.penalty[1], x.penalty[2], 0.f};
        d.lambda = A4<float>{x.lambda[0], x.lambda[1], x.lambda[2], 0.f};
        w.rd[r] = d;
        w.ab[r] = make_uint2(x.a, x.b);
        if (x.a >= n || (x.b != kContainer && x.b >= n)) atomicOr(&w.ctr->error_flags, kErrBadIndex);
    }
}

// other-body array of the caller's CSR, bounded by the scratch capacity
__global__ void k_na_other(DevWorld<float, float> w, uint32_t n, uint32_t m, const DioConstraint* joints, uint32_t nj) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t j0 = w.row_off[i], j1 = w.row_off[i + 1];
        if (j1 < j0 || j1 > 2 * m) {
            atomicOr(&w.ctr->error_flags, kErrBadIndex);
            continue;
        }
        for (uint32_t j = j0; j < j1; ++j) {
            uint32_t r = w.row_idx[j];
            if (r >= m) {
                atomicOr(&w.ctr->error_flags, kErrBadIndex);
                w.row_oth[j] = kContainer;
                continue;
            }
            uint2 v = w.ab[r];
            w.row_oth[j] = v.y == kContainer ? kContainer : (v.x == i ? v.y : (v.x | kIsB));
        }
    }
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nj; k += gridDim.x * blockDim.x)
        if (joints[k].a >= n || joints[k].b >= n) atomicOr(&w.ctr->error_flags, kErrBadIndex);
}

// avbd_primal with the reference's scan over every joint (avbd/src/lib.rs:
// 422-539) instead of a joint CSR, which would need sorting scratch.
__global__ void __launch_bounds__(128) k_na_primal(DevWorld<float, float> w, uint32_t n, int rd, int wr,
                                                   SolveParams<float> o) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const A4<float> inv = w.inv[i];
        if (inv.w == 0.f) continue;
        const V3<float> sp = xyz(w.pos[rd][i]);
        const Q4<float> sq = quat(w.rot[rd][i]);
        const float mass = 1.f / inv.w;
        const V3<float> moment{1.f / inv.x, 1.f / inv.y, 1.f / inv.z};
        const float dt2 = o.dt * o.dt;
        const float mdt2 = mass / dt2;
        const V3<float> idt2 = divs(moment, dt2);
        Block6<float> B;
#pragma unroll
        for (int k = 0; k < 21; ++k) B.h[k] = 0.f;
        B.h[tri(0, 0)] = mdt2;
        B.h[tri(1, 1)] = mdt2;
        B.h[tri(2, 2)] = mdt2;
        B.h[tri(3, 3)] = idt2.x;
        B.h[tri(4, 4)] = idt2.y;
        B.h[tri(5, 5)] = idt2.z;
        const V3<float> rl = mulv(V3<float>{mdt2, mdt2, mdt2}, sub(sp, xyz(w.inert_pos[i])));
        const V3<float> ra = mulv(idt2, ang_diff(sq, quat(w.inert_rot[i])));
        B.g[0] = rl.x;
        B.g[1] = rl.y;
        B.g[2] = rl.z;
        B.g[3] = ra.x;
        B.g[4] = ra.y;
        B.g[5] = ra.z;
        const V3<float> dqsl = sub(sp, xyz(w.init_pos[i]));
        const V3<float> dqsa = ang_diff(sq, quat(w.init_rot[i]));
        const float k_alpha = 1.f - o.alpha;
        for (uint32_t j = w.row_off[i]; j < w.row_off[i + 1]; ++j)
            primal_row(w, w.row_idx[j], w.row_oth[j], rd, sq, dqsl, dqsa, k_alpha, B);
        for (uint32_t k = 0; k < w.n_joints; ++k) {
            const DioConstraint jt = w.joints[k];
            if (jt.a == i || jt.b == i) primal_joint(w, jt, i, rd, sp, sq, sq, B);
        }
        float dx[6];
        solve6(B, dx);
        w.pos[wr][i] = pack(add(sp, V3<float>{dx[0], dx[1], dx[2]}));
        w.rot[wr][i] = packq(quat_step(sq, V3<float>{dx[3], dx[4], dx[5]}));
    }
}

__global__ void k_na_pack(DevWorld<float, float> w, uint32_t n, int buf, const DioBodyState* st_in, float* pos3,
                          float* quat4, DioBodyState* st_out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        A4<float> p = w.pos[buf][i], q = w.rot[buf][i];
        pos3[3 * i] = p.x;
        pos3[3 * i + 1] = p.y;
        pos3[3 * i + 2] = p.z;
        quat4[4 * i] = q.x;
        quat4[4 * i + 1] = q.y;
        quat4[4 * i + 2] = q.z;
        quat4[4 * i + 3] = q.w;
        DioBodyState s = st_in[i];
        A4<float> v = w.vel[i], a = w.ang[i], pv = w.prev_vel[i];
        s.vel[0] = v.x, s.vel[1] = v.y, s.vel[2] = v.z;
        s.ang[0] = a.x, s.ang[1] = a.y, s.ang[2] = a.z;
        s.prev_vel[0] = pv.x, s.prev_vel[1] = pv.y, s.prev_vel[2] = pv.z;
        st_out[i] = s;
    }
}

__global__ void k_na_dual_out(DevWorld<float, float> w, DioContact* c, uint32_t m) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        RowDual<float, float> d = w.rd[r];
        c[r].lambda[0] = d.lambda.x;
        c[r].lambda[1] = d.lambda.y;
        c[r].lambda[2] = d.lambda.z;
        c[r].penalty[0] = d.penalty.x;
        c[r].penalty[1] = d.penalty.y;
        c[r].penalty[2] = d.penalty.z;
    }
}

}  // namespace

extern "C" int dio_avbd_solve_noalloc(const DioBodyState* state, const float* positions, const float* orientations,
                                      uint32_t n, DioContact* contacts, uint32_t m, const DioConstraint* constraints,
                                      uint32_t n_constraints, const uint32_t* offsets, const uint32_t* indices,
                                      const DioRunOptions* options, float* out_positions, float* out_orientations,
                                      DioBodyState* out_state, void* cuda_stream) {
    if (!options) return DIO_ERR_INVALID;
    if (n > kNaMaxBodies || m > kNaMaxContacts || n_constraints > kNaMaxJoints) return DIO_ERR_CAPACITY;
    if (n == 0) return DIO_OK;
    if (!state || !positions || !orientations || !offsets || !out_positions || !out_orientations || !out_state ||
        (m && (!contacts || !indices)) || (n_constraints && !constraints))
        return DIO_ERR_INVALID;
    unsigned char* base = nullptr;
    int rc = scratch_ptr(&base);
    if (rc != DIO_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);

    DevWorld<float, float> w{};
    auto a4 = [&](size_t k) { return reinterpret_cast<A4<float>*>(base + kOffPose + k * kB4); };
    w.n = n;
    w.pos[0] = a4(0);
    w.pos[1] = a4(1);
    w.rot[0] = a4(2);
    w.rot[1] = a4(3);
    w.init_pos = a4(4);
    w.init_rot = a4(5);
    w.inert_pos = a4(6);
    w.inert_rot = a4(7);
    w.vel = a4(8);
    w.ang = a4(9);
    w.prev_vel = a4(10);
    w.inv = a4(11);
    w.friction = reinterpret_cast<float*>(base + kOffFric);
    w.rs = reinterpret_cast<RowStatic<float>*>(base + kOffRs);
    w.rd = reinterpret_cast<RowDual<float, float>*>(base + kOffRd);
    w.ab = reinterpret_cast<uint2*>(base + kOffAb);
    w.row_oth = reinterpret_cast<uint32_t*>(base + kOffOth);
    w.row_off = const_cast<uint32_t*>(offsets);
    w.row_idx = const_cast<uint32_t*>(indices);
    w.joints = constraints;
    w.n_joints = n_constraints;
    w.ctr = reinterpret_cast<Counters*>(base + kOffCtr);

    // the counters must start at zero; everything else is written before use
    if (cudaMemsetAsync(w.ctr, 0, sizeof(Counters), s) != cudaSuccess) return DIO_ERR_CUDA;
    const int gb = grid_for(n, 256);
    k_na_unpack<<<gb, 256, 0, s>>>(w, state, positions, orientations, n);
    if (m) k_na_rows<<<grid_for(m, 256), 256, 0, s>>>(w, contacts, m, n);
    k_na_other<<<gb, 256, 0, s>>>(w, n, m, constraints, n_constraints);
    // validate every index before any kernel dereferences one
    uint32_t flags = 0;
    if (cudaMemcpyAsync(&flags, &w.ctr->error_flags, sizeof flags, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return DIO_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return DIO_ERR_CUDA;
    if (flags & kErrBadIndex) return DIO_ERR_INVALID;
    SolveParams<float> o;
    o.dt = options->dt;
    o.gx = options->gravity[0];
    o.gy = options->gravity[1];
    o.gz = options->gravity[2];
    o.alpha = options->alpha;
    o.beta_lin = options->beta_lin;
    o.penalty_max = options->penalty_max;
    o.iterations = options->iterations;
    k_init<float, float><<<gb, 256, 0, s>>>(w, 0, n, o);
    for (uint32_t k = 0; k < o.iterations; ++k) {
        int par = (int)(k % 2);
        k_na_primal<<<grid_for(n, 128), 128, 0, s>>>(w, n, par, 1 - par, o);
        if (m) k_dual<float, float><<<grid_for(m, 256), 256, 0, s>>>(w, 0, m, nullptr, 1 - par, o);
    }
    uint32_t fp = (o.iterations - 1u) % 2u;
    int rb = fp == 0 ? 1 : 0;
    uint32_t fp_read = (o.iterations == 0 ? 0u : o.iterations - 1u) % 2u;
    int final_buf = 1 - (int)fp_read;
    k_recover<float, float><<<gb, 256, 0, s>>>(w, 0, n, rb, final_buf, o);
    k_na_pack<<<gb, 256, 0, s>>>(w, n, final_buf, state, out_positions, out_orientations, out_state);
    if (m) k_na_dual_out<<<grid_for(m, 256), 256, 0, s>>>(w, contacts, m);
    // recover flags a non-finite pose or velocity, as the context-based solve
    // reports it (dio_avbd_read)
    if (cudaMemcpyAsync(&flags, &w.ctr->error_flags, sizeof flags, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return DIO_ERR_CUDA;
    if (cudaGetLastError() != cudaSuccess) return DIO_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return DIO_ERR_CUDA;
    if (flags & kErrNonFinite) return DIO_ERR_NONFINITE;
    return DIO_OK;
}
