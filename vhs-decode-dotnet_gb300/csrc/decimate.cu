// 2:1 device decimation of an RF capture (the cuda-fast reader's opt-in
// 20-MSPS mode, src/VHSDecode.CudaFast.Native/src/cuda_fast_decimator.cu:27-64
// for the filter, :67-100 for the window).  Output i is the half-band FIR
// centred on source sample 2 i:
//
//   y[i] = c0 x[2i] + sum_{t=1..7} c_t (x[2i - (2t-1)] + x[2i + (2t-1)]),
//
// with x = 0 outside [0, source_len).  Arithmetic: the centre product is
// rounded, then each tap pair is one float add and one fused multiply-add,
// the contracted form of the reference's `value += c * (a + b)` under nvcc's
// default -fmad=true.  For int16 sources every pair sum is exact.
//
// Layout: one CTA per tile of kDecTile outputs.  Its source window (2 kDecTile
// + 32 samples from a 16-byte aligned start) is read with 16-byte loads, all of
// a thread's loads issued before any is used, converted to float once per
// sample and stored split by parity: the centre tap x[2i] sits at an even
// window position and every other tap at an odd one.  A thread then computes 4
// consecutive outputs from one 16-byte load of the even half and five of the
// odd half (lane-consecutive groups: conflict-free) and stores them as one
// 16-byte vector.  HBM-bound: 2 (int16) or 4 (float) source bytes per input
// sample, 4 bytes per output sample.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.h"

namespace vhsd {
namespace {

constexpr int kDecTile = 4096;      // outputs per CTA
constexpr int kDecThreads = 256;    // 4 groups of 4 outputs per thread
// window = source [2 o0 - 16, 2 o0 + 2 kDecTile + 16): output o0 + i is
// centred on window position 2 i + 16, its taps reach 13 either side
constexpr int kDecWin = 2 * kDecTile + 32;
constexpr int kDecHalf = kDecWin / 2;

// The filter table (cuda_fast_decimator.cu:14-24): centre, then the taps at
// offsets 1, 3, ..., 13.
__constant__ float kHalfBand[8] = {
    0.5000046374907835f,    0.3126333216205309f,    -0.09010692207961689f,  0.040107417651266825f,
    -0.017917030421899405f, 0.007100857132041433f,  -0.0022302855185240434f, 0.00041032287080936366f};

// 16 bytes of source at g (a multiple of the vector length) as floats; zeros
// outside [0, src_len).
template <typename S>
struct Vec16;
template <>
struct Vec16<int16_t> {
    static constexpr int kN = 8;
    int4 raw;
    __device__ void load(const int16_t* src, int64_t src_len, int64_t g) {
        if (g >= 0 && g + kN <= src_len) {
            raw = __ldg(reinterpret_cast<const int4*>(src + g));
        } else {
            alignas(16) int16_t h[kN];
#pragma unroll
            for (int e = 0; e < kN; e++) h[e] = (g + e >= 0 && g + e < src_len) ? src[g + e] : (int16_t)0;
            raw = *reinterpret_cast<const int4*>(h);
        }
    }
    __device__ void to_float(float* v) const {
        const int16_t* h = reinterpret_cast<const int16_t*>(&raw);
#pragma unroll
        for (int e = 0; e < kN; e++) v[e] = (float)h[e];
    }
};
template <>
struct Vec16<float> {
    static constexpr int kN = 4;
    float4 raw;
    __device__ void load(const float* src, int64_t src_len, int64_t g) {
        if (g >= 0 && g + kN <= src_len) {
            raw = __ldg(reinterpret_cast<const float4*>(src + g));
        } else {
            float h[kN];
#pragma unroll
            for (int e = 0; e < kN; e++) h[e] = (g + e >= 0 && g + e < src_len) ? src[g + e] : 0.0f;
            raw = make_float4(h[0], h[1], h[2], h[3]);
        }
    }
    __device__ void to_float(float* v) const {
        v[0] = raw.x; v[1] = raw.y; v[2] = raw.z; v[3] = raw.w;
    }
};

template <typename S>
__global__ void __launch_bounds__(kDecThreads) k_decimate_half(const S* __restrict__ src, int64_t src_len,
                                                               float* __restrict__ dst, int64_t out_len) {
    constexpr int kN = Vec16<S>::kN;                     // samples per 16-byte load
    constexpr int kVecs = kDecWin / kN;
    constexpr int kPer = (kVecs + kDecThreads - 1) / kDecThreads;
    __shared__ __align__(16) float ev[kDecHalf], od[kDecHalf];
    const int tid = threadIdx.x;
    const int64_t o0 = (int64_t)blockIdx.x * kDecTile;
    const int64_t g0 = 2 * o0 - 16;                      // a multiple of kN: 16-byte aligned
    Vec16<S> r[kPer];
#pragma unroll
    for (int k = 0; k < kPer; k++) {
        const int v = tid + k * kDecThreads;
        if (v < kVecs) r[k].load(src, src_len, g0 + (int64_t)v * kN);
    }
#pragma unroll
    for (int k = 0; k < kPer; k++) {
        const int v = tid + k * kDecThreads;
        if (v < kVecs) {
            float x[kN];
            r[k].to_float(x);
            const int h = v * (kN / 2);                  // half-window index of window position v kN
            if constexpr (kN == 8) {
                *reinterpret_cast<float4*>(ev + h) = make_float4(x[0], x[2], x[4], x[6]);
                *reinterpret_cast<float4*>(od + h) = make_float4(x[1], x[3], x[5], x[7]);
            } else {
                *reinterpret_cast<float2*>(ev + h) = make_float2(x[0], x[2]);
                *reinterpret_cast<float2*>(od + h) = make_float2(x[1], x[3]);
            }
        }
    }
    __syncthreads();
    // outputs o0 + i, i = 4 q + j: centre ev[i + 8], taps od[i + 8 - t] and od[i + 7 + t]
#pragma unroll
    for (int k = 0; k < kDecTile / 4 / kDecThreads; k++) {
        const int q = tid + k * kDecThreads;
        const int64_t o = o0 + 4 * q;
        if (o >= out_len) break;
        const float4 c4 = *reinterpret_cast<const float4*>(ev + 4 * q + 8);
        float w[20];
#pragma unroll
        for (int u = 0; u < 5; u++) {
            const float4 t4 = *reinterpret_cast<const float4*>(od + 4 * q + 4 * u);
            w[4 * u] = t4.x; w[4 * u + 1] = t4.y; w[4 * u + 2] = t4.z; w[4 * u + 3] = t4.w;
        }
        const float cen[4] = {c4.x, c4.y, c4.z, c4.w};
        float y[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            float v = __fmul_rn(kHalfBand[0], cen[j]);
#pragma unroll
            for (int t = 1; t < 8; t++) v = __fmaf_rn(kHalfBand[t], __fadd_rn(w[j + 8 - t], w[j + 7 + t]), v);
            y[j] = v;
        }
        if (o + 4 <= out_len) {
            *reinterpret_cast<float4*>(dst + o) = make_float4(y[0], y[1], y[2], y[3]);
        } else {
#pragma unroll
            for (int j = 0; j < 4; j++)
                if (o + j < out_len) dst[o + j] = y[j];
        }
    }
}

}  // namespace

cudaError_t launch_decimate_half(const int16_t* src16, const float* src32, int64_t src_len, float* dst,
                                 int64_t out_len, cudaStream_t s) {
    if (out_len <= 0) return cudaSuccess;
    if ((src16 == nullptr) == (src32 == nullptr)) return cudaErrorInvalidValue;
    const uintptr_t a = src16 ? (uintptr_t)src16 : (uintptr_t)src32;
    if ((a & 15u) != 0 || ((uintptr_t)dst & 15u) != 0) return cudaErrorInvalidValue;   // 16-byte vectors
    const int64_t grid = (out_len + kDecTile - 1) / kDecTile;
    if (grid > 0x7fffffffLL) return cudaErrorInvalidValue;
    if (src16)
        k_decimate_half<int16_t><<<(unsigned)grid, kDecThreads, 0, s>>>(src16, src_len, dst, out_len);
    else
        k_decimate_half<float><<<(unsigned)grid, kDecThreads, 0, s>>>(src32, src_len, dst, out_len);
    return cudaGetLastError();
}

}  // namespace vhsd
