// FM demodulator arithmetic of the reference's VHS path, IEEE single
// precision with every operation rounded explicitly (no contraction), so the
// device angles and frequency differences are bit-identical to the managed
// code for the same float inputs.
#pragma once
#include <cuda_runtime.h>

namespace vhsd {

// PortedMath.VhsRustAtan2Approximation (Core/Dsp/PortedMath.cs:519-544).
__device__ __forceinline__ float vhs_atan2(float y, float x) {
    const float min_normal = 1.17549435E-38f;
    x = __fadd_rn(x, copysignf(min_normal, x));
    bool swap = fabsf(x) < fabsf(y);
    float in = swap ? __fdiv_rn(x, y) : __fdiv_rn(y, x);
    float sq = __fmul_rn(in, in);
    float p = __fadd_rn(0.05265332f, __fmul_rn(sq, -0.01172120f));
    p = __fadd_rn(-0.11643287f, __fmul_rn(sq, p));
    p = __fadd_rn(0.19354346f, __fmul_rn(sq, p));
    p = __fadd_rn(-0.33262347f, __fmul_rn(sq, p));
    p = __fadd_rn(0.99997726f, __fmul_rn(sq, p));
    float r = __fmul_rn(in, p);
    const float pi = 3.14159274f;
    float half_pi = in >= 0.0f ? pi / 2.0f : -pi / 2.0f;
    r = swap ? __fsub_rn(half_pi, r) : r;
    bool xp = x >= 0.0f, yp = y >= 0.0f;
    if (xp && yp) return r;
    if (!xp && yp) return __fadd_rn(pi, r);
    if (!xp && !yp) return __fadd_rn(-pi, r);
    return r;
}

// PortedMath.VhsRustFrequencyDifference (Core/Dsp/PortedMath.cs:546-551).
// floor(d / tau) is taken without the division where its value is certain:
// +0 for 0 < d < tau and -1 for -tau <= d < -1e-30 (the rounded quotient of a
// float d in those ranges stays inside [0, 1) resp. [-1, 0) and away from
// zero); anything else (signed zeros, NaN, tiny negatives whose quotient
// rounds to -0, |d| >= tau) takes the exact division.
__device__ __forceinline__ float vhs_freq_diff(float cur, float prev, float freq) {
    const float tau = 6.28318548f;
    float d = __fsub_rn(cur, prev);
    float q;
    if (d > 0.0f && d < tau) q = 0.0f;
    else if (d < -1.0e-30f && d >= -tau) q = -1.0f;
    else q = floorf(__fdiv_rn(d, tau));
    d = __fsub_rn(d, __fmul_rn(q, tau));
    return __fdiv_rn(__fmul_rn(d, freq), tau);
}

}  // namespace vhsd
