// Test harness for diomedes_gb300/csrc/div_rn.cuh, compiled by
// tests/test_gpu_division.py (nvcc, sm_103a) into a scratch directory.
//   div_sweep  every a significand in [1, 2) against the b significands
//              first + k * stride (k < count): Divisor<float>(b).div(a) vs the
//              IEEE division a / b, counting bit mismatches on the device
//   div_pairs  Divisor<float>(b[i]).div(a[i]) for host arrays (random and
//              special pairs; the test compares with numpy's float32 division)
#include <cuda_runtime.h>
#include <stdint.h>

#include "div_rn.cuh"

namespace {

__global__ void k_sweep(uint32_t first, uint32_t count, uint32_t stride, unsigned long long* bad, uint32_t* witness) {
    if (blockIdx.x >= count) return;
    const uint32_t jb = first + blockIdx.x * stride;
    if (jb >= (1u << 23)) return;
    const float b = __uint_as_float(0x3F800000u | jb);
    const dio::Divisor<float> d(b);
    unsigned long long nbad = 0;
    for (uint32_t i = threadIdx.x; i < (1u << 23); i += blockDim.x) {
        const float a = __uint_as_float(0x3F800000u | i);
        const float q = d.div(a), e = a / b;
        if (__float_as_uint(q) != __float_as_uint(e)) {
            ++nbad;
            if (atomicCAS(&witness[0], 0u, 1u) == 0u) {
                witness[1] = __float_as_uint(a);
                witness[2] = __float_as_uint(b);
            }
        }
    }
    if (nbad) atomicAdd(bad, nbad);
}

__global__ void k_pairs(const float* a, const float* b, uint32_t n, float* out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = dio::Divisor<float>(b[i]).div(a[i]);
}

}  // namespace

extern "C" {

// bad: mismatch count; witness[0..2]: found flag, first mismatching a and b bits
int div_sweep(uint32_t first, uint32_t count, uint32_t stride, unsigned long long* bad, uint32_t* witness) {
    unsigned long long* d_bad = nullptr;
    uint32_t* d_w = nullptr;
    if (cudaMalloc(&d_bad, sizeof *d_bad) != cudaSuccess) return 1;
    if (cudaMalloc(&d_w, 3 * sizeof *d_w) != cudaSuccess) return 1;
    cudaMemset(d_bad, 0, sizeof *d_bad);
    cudaMemset(d_w, 0, 3 * sizeof *d_w);
    const uint32_t per_launch = 4096;  // b values per launch: each launch stays well under a second
    for (uint32_t k = 0; k < count; k += per_launch) {
        const uint32_t c = count - k < per_launch ? count - k : per_launch;
        k_sweep<<<c, 256>>>(first + k * stride, c, stride, d_bad, d_w);
    }
    int rc = cudaDeviceSynchronize() == cudaSuccess ? 0 : 2;
    cudaMemcpy(bad, d_bad, sizeof *bad, cudaMemcpyDeviceToHost);
    cudaMemcpy(witness, d_w, 3 * sizeof *d_w, cudaMemcpyDeviceToHost);
    cudaFree(d_bad);
    cudaFree(d_w);
    return rc;
}

int div_pairs(const float* a, const float* b, uint32_t n, float* out) {
    float *da = nullptr, *db = nullptr, *dq = nullptr;
    const size_t bytes = (size_t)n * sizeof(float);
    if (cudaMalloc(&da, bytes) != cudaSuccess || cudaMalloc(&db, bytes) != cudaSuccess ||
        cudaMalloc(&dq, bytes) != cudaSuccess)
        return 1;
    cudaMemcpy(da, a, bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(db, b, bytes, cudaMemcpyHostToDevice);
    k_pairs<<<256, 256>>>(da, db, n, dq);
    int rc = cudaDeviceSynchronize() == cudaSuccess ? 0 : 2;
    cudaMemcpy(out, dq, bytes, cudaMemcpyDeviceToHost);
    cudaFree(da);
    cudaFree(db);
    cudaFree(dq);
    return rc;
}
}
