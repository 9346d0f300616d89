// div_rn.cuh -- several quotients by one divisor, each bit-identical to the
// IEEE round-to-nearest division a / b.
//
// solve6's unpivoted LDL^T divides 21 times by 6 distinct pivots.  For each
// pivot b the correctly rounded reciprocal y = RN(1/b) is formed once
// (__frcp_rn); each quotient then takes Markstein's final correction step
// (P. W. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Develop. 34(1), 1990):
//     q0 = RN(a y),   r = a - b q0 (exact: one FMA),   q = RN(q0 + r y),
// which gives q = RN(a / b) when y = RN(1/b) and no intermediate leaves the
// normal range.  The step is used only when |b|, |a| and |q0| lie in
// [2^-96, 2^96] (so 1/b, q0 and the remainder r are normal and r is exact);
// a == 0 returns q0 = a * y, which carries the IEEE sign of the zero
// quotient; every other case (zero or huge pivots, subnormals, infinities,
// NaN) takes the IEEE division itself.  Within that range the computation
// scales exactly with the exponents of a and b, so it is checked against the
// IEEE division for every pair of significands a, b in [1, 2)
// (tests/test_gpu_division.py) and on random full-range pairs.
#pragma once

#include <cuda_runtime.h>

namespace dio {

template <class R>
struct Divisor {  // other types: plain division
    R b;
    __device__ __forceinline__ explicit Divisor(R b_) : b(b_) {}
    __device__ __forceinline__ R div(R a) const { return a / b; }
};

template <>
struct Divisor<float> {
    float b, y;
    bool ok;  // the pivot is in the correction step's range
    __device__ __forceinline__ explicit Divisor(float b_) : b(b_) {
#ifdef __CUDA_ARCH__
        y = __frcp_rn(b_);
#endif
        const float m = fabsf(b_);
        ok = m >= 0x1p-96f && m <= 0x1p96f;
    }
    __device__ __forceinline__ float div(float a) const {
        const float q0 = __fmul_rn(a, y);
        const float ma = fabsf(a), mq = fabsf(q0);
        const bool in_range = ma >= 0x1p-96f && ma <= 0x1p96f && mq >= 0x1p-96f && mq <= 0x1p96f;
        if (!(ok && (in_range || a == 0.f))) return a / b;
        if (a == 0.f) return q0;
        const float r = __fmaf_rn(-b, q0, a);
        return __fmaf_rn(r, y, q0);
    }
};

}  // namespace dio
