// Plain FP64 block demodulator: one 32768-sample block at a time, full-length
// complex FFTs in global memory (Stockham radix-8, five passes), one kernel
// per step.  It restates the same per-block math as the fused FP32 kernel
// (Core/Dsp/RfDemodulator.cs:288-918) in binary64 and is the baseline the
// fused path is measured against.  The session replays the per-block launch
// sequence from a captured CUDA graph; the block index is read from device
// memory so one graph serves every block.
#include <cuda_runtime.h>
#include <stdint.h>

#include "fft_common.cuh"
#include "vhs_math.cuh"
#include "kernels.h"

namespace vhsd {
namespace fp64 {

constexpr int N = 32768;
constexpr int H = N / 2;

__device__ __forceinline__ double2 wN(int k, bool inv) {
    double s, c;
    sincospi(-2.0 * (double)k / (double)N, &s, &c);
    return make_double2(c, inv ? -s : s);
}

// Stockham radix-8 pass: in -> out, L = N, Ns in {1, 8, 64, 512, 4096}.
template <bool INV>
__global__ void k_pass8(const double2* __restrict__ in, double2* __restrict__ out, int Ns) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int R = 8;
    const int nbf = N / R;
    if (j >= nbf) return;
    int k = j & (Ns - 1);
    double2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = in[j + r * nbf];
    if (Ns > 1) {
#pragma unroll
        for (int r = 1; r < R; r++) {
            double2 w = wN((k * r * (N / (Ns * R))) & (N - 1), INV);
            v[r] = cmul(v[r], w);
        }
    }
    dft<R, INV>(v);
    int dst = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) out[dst + r * Ns] = v[r];
}

// a -> b -> a ... five passes; result ends in `b`.
template <bool INV>
void fft(double2* a, double2* b, cudaStream_t s) {
    int ns = 1;
    double2* src = a;
    double2* dst = b;
    for (int pidx = 0; pidx < 5; pidx++) {
        k_pass8<INV><<<(N / 8 + 255) / 256, 256, 0, s>>>(src, dst, ns);
        ns *= 8;
        double2* t = src; src = dst; dst = t;
    }
    // after 5 passes the data is in `src` (== b)
}


// int16 capture, or a float one when rf32 is set
__global__ void k_load(const int16_t* rf, const float* rf32, const int64_t* blk, double2* out) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const int64_t i = blk[0] * kStride + n;
    out[n] = make_double2(rf32 ? (double)rf32[i] : (double)rf[i], 0.0);
}

// analytic spectrum: X * RfVideo * Hilbert / N  (bins > N/2 zero)
__global__ void k_analytic_spec(const double2* X, const double* g, double2* Z) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    double m;
    if (k == 0 || k == H) m = g[k] / N;
    else if (k < H) m = 2.0 * g[k] / N;
    else m = 0.0;
    Z[k] = make_double2(X[k].x * m, X[k].y * m);
}

// demod (float polynomial atan2 of the double analytic signal) + spike flag
__global__ void k_demod(const double2* z, double* d, float fs, double diff_max, int* flag) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    double v = 0.0;
    if (n > 0) {
        float th = vhs_atan2((float)z[n].y, (float)z[n].x);
        float tp = vhs_atan2((float)z[n - 1].y, (float)z[n - 1].x);
        v = (double)vhs_freq_diff(th, tp, fs);
    }
    d[n] = v;
    if (n >= 20 && n < N - 20 && v > diff_max) atomicOr(flag, 1);
}

// diff demod (analytic first difference), only when the block has spikes
__global__ void k_diff_demod(const double2* z, double* dd, float fs, const int* flag) {
    if (!flag[0]) return;
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    double v = 0.0;
    if (n >= 1) {
        double2 a = z[n], b = z[n - 1];
        float th = vhs_atan2((float)(a.y - b.y), (float)(a.x - b.x));
        float tp;
        if (n >= 2) {
            double2 c = z[n - 2];
            tp = vhs_atan2((float)(b.y - c.y), (float)(b.x - c.x));
        } else {
            tp = vhs_atan2(0.0f, 0.0f);
        }
        v = (double)vhs_freq_diff(th, tp, fs);
    }
    dd[n] = v;
}

// ReplaceSpikes (Core/Dsp/RfDemodulator.cs:966-1001) on one warp, spike set
// taken from the demod before replacement.
__global__ void k_replace_spikes(double* d, const double* dd, double diff_max, int* flag,
                                 unsigned* mask) {
    if (!flag[0]) return;
    int lane = threadIdx.x;
    for (int base = 0; base < N; base += 32) {
        unsigned m = __ballot_sync(0xffffffffu, d[base + lane] > diff_max);
        if (lane == 0) mask[base >> 5] = m;
    }
    __syncwarp();
    for (int word = 0; word < N / 32; word++) {
        unsigned m = mask[word];
        while (m) {
            int b = __ffs(m) - 1;
            m &= m - 1;
            int i0 = word * 32 + b;
            int st = max(i0 - 8, 0), en = min(i0 + 30, N - 1);
            if (st >= en) continue;
            double mdd = -INFINITY, md = -INFINITY;
            for (int k = st + lane; k < en; k += 32) { mdd = fmax(mdd, dd[k]); md = fmax(md, d[k]); }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                mdd = fmax(mdd, __shfl_xor_sync(0xffffffffu, mdd, o));
                md = fmax(md, __shfl_xor_sync(0xffffffffu, md, o));
            }
            if (mdd < md) for (int k = st + lane; k < en; k += 32) d[k] = dd[k];
            __syncwarp();
        }
    }
    if (lane == 0) flag[0] = 0;
}

// float32 envelope filtfilt (SosFilter.ApplyForwardBackwardFloat32,
// Core/Dsp/SosFilter.cs:300-540) of raw[n] = |float(Re z[n-4])| (circular
// roll by 4), in float32 like the reference, as a parallel scan: one CTA of
// 32 warps, warp w covers samples [1024 w, 1024 w + 1024) as four rows of 256
// (8 consecutive samples per lane, lanes joined by an affine warp scan).  The
// state entering a warp's range comes from a 256-sample halo started at zero
// (the first-order filter's memory c^256 is below 1e-12); at the block edges
// the recursion starts from zero instead of the reference's padded
// steady-state start, which only touches samples the overlap-save cut drops.
struct EnvAff { float a, b; };
__device__ __forceinline__ EnvAff env_then(EnvAff first, EnvAff second) {
    return EnvAff{second.a * first.a, fmaf(second.a, first.b, second.b)};
}
__device__ __forceinline__ EnvAff env_scan(EnvAff v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        float pa = __shfl_up_sync(0xffffffffu, v.a, o), pb = __shfl_up_sync(0xffffffffu, v.b, o);
        if (lane >= o) v = env_then(EnvAff{pa, pb}, v);
    }
    return v;
}
__device__ __forceinline__ EnvAff env_scan_rev(EnvAff v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        float pa = __shfl_down_sync(0xffffffffu, v.a, o), pb = __shfl_down_sync(0xffffffffu, v.b, o);
        if (lane + o < 32) v = env_then(EnvAff{pa, pb}, v);
    }
    return v;
}

__global__ void __launch_bounds__(1024) k_envelope(const double2* z, float* work, double* env, float b0,
                                                   float b1, float a1) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n0 = warp * 1024;
    const float cc = -a1, gk = b1 - a1 * b0;
    float c8 = cc;
#pragma unroll
    for (int k = 1; k < 8; k++) c8 *= cc;
    auto raw = [&](int n) { return fabsf((float)z[(n - 4) & (N - 1)].x); };
    float yv[32];
    float carry = 0.0f;
    if (n0 >= 256) {
        float st = 0.0f;
        for (int k = 0; k < 8; k++) st = fmaf(cc, st, gk * raw(n0 - 256 + lane * 8 + k));
        EnvAff inc = env_scan(EnvAff{c8, st}, lane);
        carry = __shfl_sync(0xffffffffu, inc.b, 31);
    }
    for (int row = 0; row < 4; row++) {
        int ms = n0 + row * 256 + lane * 8;
        float ev[8], st = 0.0f;
        for (int k = 0; k < 8; k++) { ev[k] = raw(ms + k); st = fmaf(cc, st, gk * ev[k]); }
        EnvAff inc = env_scan(EnvAff{c8, st}, lane);
        float pb = __shfl_up_sync(0xffffffffu, inc.b, 1), pa = __shfl_up_sync(0xffffffffu, inc.a, 1);
        float zz = lane == 0 ? carry : fmaf(pa, carry, pb);
        for (int k = 0; k < 8; k++) { yv[row * 8 + k] = fmaf(b0, ev[k], zz); zz = fmaf(cc, zz, gk * ev[k]); }
        carry = __shfl_sync(0xffffffffu, zz, 31);
        for (int k = 0; k < 8; k++) work[ms + k] = yv[row * 8 + k];
    }
    __syncthreads();
    const int nend = n0 + 1024;
    carry = 0.0f;
    if (nend + 256 <= N) {
        float st = 0.0f;
        for (int k = 7; k >= 0; k--) st = fmaf(cc, st, gk * work[nend + lane * 8 + k]);
        EnvAff inc = env_scan_rev(EnvAff{c8, st}, lane);
        carry = __shfl_sync(0xffffffffu, inc.b, 0);
    }
    for (int row = 3; row >= 0; row--) {
        int ms = n0 + row * 256 + lane * 8;
        float st = 0.0f;
        for (int k = 7; k >= 0; k--) st = fmaf(cc, st, gk * yv[row * 8 + k]);
        EnvAff inc = env_scan_rev(EnvAff{c8, st}, lane);
        float nb = __shfl_down_sync(0xffffffffu, inc.b, 1), na = __shfl_down_sync(0xffffffffu, inc.a, 1);
        float zz = lane == 31 ? carry : fmaf(na, carry, nb);
        for (int k = 7; k >= 0; k--) {
            float y = yv[row * 8 + k];
            env[ms + k] = (double)fmaf(b0, y, zz);
            zz = fmaf(cc, zz, gk * y);
        }
        carry = __shfl_sync(0xffffffffu, zz, 0);
    }
}

// Sub-deemphasis (ApplySubDeemphasisRealCore, Core/Dsp/RfDemodulator.cs:2852-2990),
// step 1: one-sided spectrum whose inverse is the analytic signal of
// high = irfft(D Video HighPass): x2 for 0 < k < N/2, real part at 0 and N/2
// (what a c2r inverse keeps), zero above; scaled 1/N.
__global__ void k_sub_spec(const double2* D, const double2* g, double2* A) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    double2 v = make_double2(0.0, 0.0);
    if (k <= H) {
        v = cmul(D[k], g[k]);
        if (k == 0 || k == H) v = make_double2(v.x / N, 0.0);
        else v = make_double2(2.0 * v.x / N, 2.0 * v.y / N);
    }
    A[k] = v;
}

struct Aff64 { double a, b; };
__device__ __forceinline__ Aff64 aff64_then(Aff64 first, Aff64 second) {
    return Aff64{second.a * first.a, fma(second.a, first.b, second.b)};
}
__device__ __forceinline__ Aff64 aff64_scan(Aff64 v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        double pa = __shfl_up_sync(0xffffffffu, v.a, o), pb = __shfl_up_sync(0xffffffffu, v.b, o);
        if (lane >= o) v = aff64_then(Aff64{pa, pb}, v);
    }
    return v;
}
__device__ __forceinline__ Aff64 aff64_scan_rev(Aff64 v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        double pa = __shfl_down_sync(0xffffffffu, v.a, o), pb = __shfl_down_sync(0xffffffffu, v.b, o);
        if (lane + o < 32) v = aff64_then(Aff64{pa, pb}, v);
    }
    return v;
}

__device__ __forceinline__ double sub_gain64(double amp, const SubDeemph64& s) {
    amp = fmax(0.0, amp) * s.scale1;
    amp = pow(amp, s.exponent) * s.scale2;
    if (s.logistic_rate > 0.0) amp *= 1.0 / (1.0 + exp(-s.logistic_rate * (amp - s.logistic_mid)));
    return amp;
}

// Step 2: amp[n] = |a[n]| * 2 / deviation.
__global__ void k_sub_mag(const double2* a, double* amp, SubDeemph64 sub) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    amp[n] = hypot(a[n].x, a[n].y) * sub.inv_half_dev;
}

// Steps 3-4: first-order low-pass filtfilt of amp in binary64, one warp (one
// CTA) per 1024-sample range, 32 ranges per block: the range is four rows of
// 256 (8 consecutive samples per lane) joined by affine warp scans, and the
// state entering it comes from the 1024 samples before it (after it, backward)
// started at zero, where the filter's memory c^1024 is below 1e-40; at the
// block edges the recursion starts from zero instead of the padded
// steady-state start, which only moves samples the overlap-save cut drops.
// Forward: amp -> fwd.  Backward: fwd -> out.
template <bool BACKWARD>
__global__ void __launch_bounds__(32) k_sub_filt(const double* in, double* out, SubDeemph64 sub) {
    const int lane = threadIdx.x;
    const int n0 = blockIdx.x * 1024;
    const double cc = -sub.a1, gk = sub.b1 - sub.a1 * sub.b0, b0 = sub.b0;
    double c8 = cc;
#pragma unroll
    for (int k = 1; k < 8; k++) c8 *= cc;
    double carry = 0.0;
    if (!BACKWARD) {
        if (n0 >= 1024) {
            for (int hr = 0; hr < 4; hr++) {
                int ms = n0 - 1024 + hr * 256 + lane * 8;
                double ev[8], st = 0.0;
                for (int k = 0; k < 8; k++) { ev[k] = in[ms + k]; st = fma(cc, st, gk * ev[k]); }
                Aff64 inc = aff64_scan(Aff64{c8, st}, lane);
                double pb = __shfl_up_sync(0xffffffffu, inc.b, 1), pa = __shfl_up_sync(0xffffffffu, inc.a, 1);
                double z = lane == 0 ? carry : fma(pa, carry, pb);
                for (int k = 0; k < 8; k++) z = fma(cc, z, gk * ev[k]);
                carry = __shfl_sync(0xffffffffu, z, 31);
            }
        }
        for (int row = 0; row < 4; row++) {
            int ms = n0 + row * 256 + lane * 8;
            double ev[8], st = 0.0;
            for (int k = 0; k < 8; k++) { ev[k] = in[ms + k]; st = fma(cc, st, gk * ev[k]); }
            Aff64 inc = aff64_scan(Aff64{c8, st}, lane);
            double pb = __shfl_up_sync(0xffffffffu, inc.b, 1), pa = __shfl_up_sync(0xffffffffu, inc.a, 1);
            double z = lane == 0 ? carry : fma(pa, carry, pb);
            for (int k = 0; k < 8; k++) { out[ms + k] = fma(b0, ev[k], z); z = fma(cc, z, gk * ev[k]); }
            carry = __shfl_sync(0xffffffffu, z, 31);
        }
    } else {
        const int nend = n0 + 1024;
        if (nend + 1024 <= N) {
            for (int hr = 3; hr >= 0; hr--) {
                int ms = nend + hr * 256 + lane * 8;
                double ev[8], st = 0.0;
                for (int k = 7; k >= 0; k--) { ev[k] = in[ms + k]; st = fma(cc, st, gk * ev[k]); }
                Aff64 inc = aff64_scan_rev(Aff64{c8, st}, lane);
                double nb = __shfl_down_sync(0xffffffffu, inc.b, 1), na = __shfl_down_sync(0xffffffffu, inc.a, 1);
                double z = lane == 31 ? carry : fma(na, carry, nb);
                for (int k = 7; k >= 0; k--) z = fma(cc, z, gk * ev[k]);
                carry = __shfl_sync(0xffffffffu, z, 0);
            }
        }
        for (int row = 3; row >= 0; row--) {
            int ms = n0 + row * 256 + lane * 8;
            double ev[8], st = 0.0;
            for (int k = 7; k >= 0; k--) { ev[k] = in[ms + k]; st = fma(cc, st, gk * ev[k]); }
            Aff64 inc = aff64_scan_rev(Aff64{c8, st}, lane);
            double nb = __shfl_down_sync(0xffffffffu, inc.b, 1), na = __shfl_down_sync(0xffffffffu, inc.a, 1);
            double z = lane == 31 ? carry : fma(na, carry, nb);
            for (int k = 7; k >= 0; k--) { out[ms + k] = fma(b0, ev[k], z); z = fma(cc, z, gk * ev[k]); }
            carry = __shfl_sync(0xffffffffu, z, 0);
        }
    }
}

// Step 5, elementwise: video[n] -= Re a[n] (1 - map(amp[n])) + Re a[n] static_factor.
__global__ void k_sub_apply(const double2* a, const double* amp, double2* video, SubDeemph64 sub) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    double h = a[n].x;
    double g = sub_gain64(amp[n], sub);
    video[n].x -= h * (1.0 - g) + h * sub.static_factor;
}

__global__ void k_real_to_complex(const double* d, double2* out) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    out[n] = make_double2(d[n], 0.0);
}

// Hermitian spectrum D * Hfilter for bins 0..N/2 (imaginary parts of the DC and
// Nyquist bins dropped, as a c2r inverse does), mirrored above N/2, scaled 1/N.
__global__ void k_filter_spec(const double2* D, const double2* h, double2* out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    int kk = k <= H ? k : N - k;
    double2 v = cmul(D[kk], h[kk]);
    if (kk == 0 || kk == H) v.y = 0.0;
    if (k > H) v.y = -v.y;
    out[k] = make_double2(v.x / N, v.y / N);
}

__global__ void k_store(const double2* x, const int64_t* blk, double* out, int shift) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= kStride) return;
    int n = s + kCut + shift;
    out[blk[0] * kStride + s] = x[n].x;
}
__global__ void k_store_real(const double* x, const int64_t* blk, double* out) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= kStride) return;
    out[blk[0] * kStride + s] = x[s + kCut];
}
__global__ void k_next_block(int64_t* blk) { blk[0] += 1; }

}  // namespace fp64

// Work buffers: work = 4*N double2 (w0..w3), dwork = 4*N double (d, dd, env, scratch)
cudaError_t launch_demod_fp64_block(const PlainDemodParams& p, cudaStream_t s) {
    using namespace fp64;
    const int B = 256, G = (N + B - 1) / B;
    double2* w0 = p.work;
    double2* w1 = p.work + N;
    double2* w2 = p.work + 2 * N;
    double2* w3 = p.work + 3 * N;
    double* d = p.dwork;
    double* dd = p.dwork + N;
    double* env = p.dwork + 2 * N;
    float* fscr = p.fwork;
    int* flag = p.flag;
    unsigned* mask = p.mask;
    int64_t* blk = p.blk;
    k_load<<<G, B, 0, s>>>(p.rf, p.rf_f32, blk, w0);
    fft<false>(w0, w1, s);                         // X in w1
    k_analytic_spec<<<G, B, 0, s>>>(w1, p.rf_video, w2);
    fft<true>(w2, w3, s);                          // z in w3
    k_demod<<<G, B, 0, s>>>(w3, d, (float)p.fs, p.diff_max, flag);
    k_diff_demod<<<G, B, 0, s>>>(w3, dd, (float)p.fs, flag);
    k_replace_spikes<<<1, 32, 0, s>>>(d, dd, p.diff_max, flag, mask);
    k_envelope<<<1, 1024, 0, s>>>(w3, fscr, env, (float)p.env_b0, (float)p.env_b1, (float)p.env_a1);
    k_real_to_complex<<<G, B, 0, s>>>(d, w0);
    fft<false>(w0, w1, s);                         // D in w1
    k_filter_spec<<<G, B, 0, s>>>(w1, p.video, w2);
    fft<true>(w2, w3, s);                          // video in w3
    if (p.sub.high) {
        k_sub_spec<<<G, B, 0, s>>>(w1, p.sub.high, w2);
        fft<true>(w2, w0, s);                      // analytic high part in w0
        k_sub_mag<<<G, B, 0, s>>>(w0, dd, p.sub);
        k_sub_filt<false><<<N / 1024, 32, 0, s>>>(dd, d, p.sub);
        k_sub_filt<true><<<N / 1024, 32, 0, s>>>(d, dd, p.sub);
        k_sub_apply<<<G, B, 0, s>>>(w0, dd, w3, p.sub);
    }
    k_store<<<(kStride + B - 1) / B, B, 0, s>>>(w3, blk, p.video_out, 0);
    k_filter_spec<<<G, B, 0, s>>>(w1, p.sync, w2);
    fft<true>(w2, w0, s);                          // sync in w0
    k_store<<<(kStride + B - 1) / B, B, 0, s>>>(w0, blk, p.sync_out, 32);
    k_store_real<<<(kStride + B - 1) / B, B, 0, s>>>(env, blk, p.env_out);
    k_next_block<<<1, 1, 0, s>>>(blk);
    return cudaGetLastError();
}

}  // namespace vhsd
