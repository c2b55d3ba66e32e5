// Register-level DFT butterflies and complex helpers shared by the FP32 fused
// block demodulator and the FP64 plain path.
//
// dft<R, INV>(v) computes v[k] = sum_r v[r] * exp(-/+ 2*pi*i*r*k/R) in natural
// order for R in {2, 4, 8, 16, 32}, fully unrolled on registers.  Twiddles of
// the in-register stages are the exact values cos/sin(2*pi*k/32) written out
// below; multiplications by 1 and -i are folded at compile time.
#pragma once
#include <cuda_runtime.h>

namespace vhsd {

template <typename T> struct cplx;
template <> struct cplx<float> { using type = float2; };
template <> struct cplx<double> { using type = double2; };

template <typename C>
__device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C>
__device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C>
__device__ __forceinline__ C cmul(C a, C b) {
    C r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
// a * conj(b)
template <typename C>
__device__ __forceinline__ C cmulc(C a, C b) {
    C r;
    r.x = a.x * b.x + a.y * b.y;
    r.y = a.y * b.x - a.x * b.y;
    return r;
}
template <typename C>
__device__ __forceinline__ C cconj(C a) { a.y = -a.y; return a; }
template <typename C, typename S>
__device__ __forceinline__ C cscale(C a, S s) { a.x *= s; a.y *= s; return a; }

// cos(2*pi*k/32) and sin(2*pi*k/32) for k = 0..8 (first octant is enough).
#define VHSD_C32_0 1.0
#define VHSD_C32_1 0.98078528040323044912618223613424
#define VHSD_C32_2 0.92387953251128675612818318939679
#define VHSD_C32_3 0.83146961230254523707878837761791
#define VHSD_C32_4 0.70710678118654752440084436210485
#define VHSD_C32_5 0.55557023301960222474283081394853
#define VHSD_C32_6 0.38268343236508977172845998403040
#define VHSD_C32_7 0.19509032201612826784828486847702
#define VHSD_C32_8 0.0

template <typename S>
__device__ __forceinline__ S cos32(int k) {
    // cos(2*pi*k/32) for k in [0, 32)
    k &= 31;
    int o = k & 7, q = k >> 3;
    const S t[9] = {(S)VHSD_C32_0, (S)VHSD_C32_1, (S)VHSD_C32_2, (S)VHSD_C32_3, (S)VHSD_C32_4,
                    (S)VHSD_C32_5, (S)VHSD_C32_6, (S)VHSD_C32_7, (S)VHSD_C32_8};
    // quadrant reduction: cos(q*pi/2 + a)
    S c = t[o], s = t[8 - o];
    if (q == 0) return c;
    if (q == 1) return -s;
    if (q == 2) return -c;
    return s;
}
template <typename S>
__device__ __forceinline__ S sin32(int k) { return cos32<S>(k - 8); }

// Multiply v by exp(sign * 2*pi*i*k/32), folding the trivial angles.
template <typename C, bool INV>
__device__ __forceinline__ C rot32(C v, int k) {
    using S = decltype(v.x);
    k &= 31;
    if (k == 0) return v;
    if (k == 8) {  // forward: -i ; inverse: +i
        C r;
        if (INV) { r.x = -v.y; r.y = v.x; } else { r.x = v.y; r.y = -v.x; }
        return r;
    }
    if (k == 16) { v.x = -v.x; v.y = -v.y; return v; }
    if (k == 24) {
        C r;
        if (INV) { r.x = v.y; r.y = -v.x; } else { r.x = -v.y; r.y = v.x; }
        return r;
    }
    S c = cos32<S>(k);
    S s = INV ? sin32<S>(k) : -sin32<S>(k);
    C w; w.x = c; w.y = s;
    return cmul(v, w);
}

__host__ __device__ constexpr int ilog2c(int r) { return r <= 1 ? 0 : 1 + ilog2c(r >> 1); }
__host__ __device__ constexpr int bitrev(int x, int bits) {
    int y = 0;
    for (int i = 0; i < bits; i++) { y = (y << 1) | ((x >> i) & 1); }
    return y;
}

// In-register radix-R DFT, natural order in and out (decimation in frequency
// radix-2 stages followed by a compile-time bit-reversal of register names).
template <int R, bool INV, typename C>
__device__ __forceinline__ void dft(C (&v)[R]) {
    constexpr int L = ilog2c(R);
#pragma unroll
    for (int s = 0; s < L; s++) {
        const int half = R >> (s + 1);
        const int span = half * 2;
#pragma unroll
        for (int g = 0; g < R; g += span) {
#pragma unroll
            for (int j = 0; j < half; j++) {
                C a = v[g + j], b = v[g + j + half];
                v[g + j] = cadd(a, b);
                C d = csub(a, b);
                // twiddle exp(-2 pi i j / span) = W32^(j * 32 / span)
                v[g + j + half] = rot32<C, INV>(d, j * (32 / span));
            }
        }
    }
    C t[R];
#pragma unroll
    for (int i = 0; i < R; i++) t[i] = v[bitrev(i, L)];
#pragma unroll
    for (int i = 0; i < R; i++) v[i] = t[i];
}

}  // namespace vhsd
