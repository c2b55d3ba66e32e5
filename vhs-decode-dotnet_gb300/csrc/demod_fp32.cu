// Fused FP32 VHS block demodulator: one 32768-sample RF block per 2-CTA
// thread-block cluster, every intermediate spectrum kept in the two CTAs'
// shared memory and exchanged through distributed shared memory.
//
// Per block b (RF samples x[n] = rf[b*30720 + n], n < 32768, from an int16
// capture or a float one such as the 2:1 decimator's output) it computes what
// the reference's exact VHS path computes per block
// (Core/Dsp/RfDemodulator.cs:288-918, exact backend):
//   X  = rfft(x);  Y = X * RfVideo                         (stage 1)
//   z  = ifft(full(Y) * Hilbert)       analytic signal     (stage 2)
//   d  = float polynomial-atan2 FM demod of z              (stage 3)
//        + diff-demod spike repair when any d > limit      (repair path)
//   env= |Re z| rolled by 4, 700 kHz first-order filtfilt  (envelope)
//   D  = rfft(d - ire0)                                    (stage 4)
//   video = irfft(D * Video) + ire0 Video[0], sync = roll(irfft(D * VideoLowPass05), -32)
//           + ire0 VideoLowPass05[0]
//                                                          (stage 5)
//   S-VHS sub-deemphasis: a = ifft(one-sided D * Video * HighPass) (the
//   analytic signal of the high part), amp = |a| low-passed forward and
//   backward, video -= Re a * (1 - map(amp))                (stage 6)
// and writes the kept samples [1024, 31744) of video, sync and envelope to the
// stitched stream at stream index b*30720 + (n - 1024).
//
// Work split inside a cluster (rank 0 / rank 1):
//   * the 16384-point packed complex FFT of a real block is split by
//     decimation in frequency, rank 0 computing the even output bins and
//     rank 1 the odd ones; the real-FFT post-processing pairs k with M-k,
//     which have equal parity, so it stays local;
//   * inverse transforms are split by decimation in time on the input bins
//     (even bins on rank 0, odd bins on rank 1) and finished with one
//     butterfly that reads the partner CTA's half through DSMEM;
//   * the time-domain block is held as four 8192-sample chunks, chunks 0 and
//     2 on rank 0, chunks 1 and 3 on rank 1.
// Shared memory per CTA (212 KB, one CTA per SM): 16384 complex floats
// (padded against bank conflicts), a 16384-float buffer that holds the angles,
// then the demod, then (S-VHS) the kept spectrum, and in between the next
// block's RF prefetch and, during the stage-1 transform, the RfVideo table;
// plus twiddle tables.
#include <cooperative_groups.h>
#include <atomic>
#include <climits>
#include <cuda_runtime.h>
#include <stdint.h>

#include "fft_common.cuh"
#include "spikes.cuh"
#include "vhs_math.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace vhsd {
namespace fp32 {

constexpr int N = 32768;      // RF block
constexpr int M = 16384;      // packed complex length
constexpr int Q = 8192;       // half of M, chunk length
constexpr int T = 512;        // threads per CTA
constexpr int S = 30720;      // block stride
constexpr int CUT = 1024;
constexpr int BUF = M + (M >> 4);  // padded buffer length in float2

__device__ __forceinline__ int sx(int i) { return i + (i >> 4); }

struct Tw {
    float2 hi[256];  // exp(-2 pi i h*128/32768)
    float2 lo[128];  // exp(-2 pi i l/32768)
    float2 lo8[16];  // lo[8 b]: conflict-free W^(8 v) for consecutive v
};

// exp(-2 pi i k / 32768) for k in [0, 32768)
__device__ __forceinline__ float2 w32k(const Tw& t, int k) {
    return cmul(t.hi[(k >> 7) & 255], t.lo[k & 127]);
}

// One Stockham radix-R pass over `batch` transforms of length L stored
// contiguously from buf index 0.  Each thread handles J butterflies.
// Twiddles W^(k r step), r = 8a + b: W^(8a k step) is read from the tables
// (a < R/8), W^(b k step) for b < 8 is built by repeated multiplication with
// W^(k step), so a butterfly does R/8 table reads instead of R-1 and no
// strided (bank-conflicting) table pattern remains.
template <int R, int J, bool INV>
__device__ __forceinline__ void pass(float2* buf, int L, int batch, int Ns, const Tw& tw, int tid) {
    float2 v[J][R];
    int dst[J];
    bool act[J];
    const int nbf = L / R;
    const int step = 32768 / (Ns * R);
#pragma unroll
    for (int i = 0; i < J; i++) {
        int g = tid + i * T;
        act[i] = g < batch * nbf;
        dst[i] = 0;
        if (act[i]) {
            int f = g / nbf;
            int j = g - f * nbf;
            int base = f * L;
            int k = j & (Ns - 1);
#pragma unroll
            for (int r = 0; r < R; r++) v[i][r] = buf[sx(base + j + r * nbf)];
            if (Ns > 1) {
                float2 wb[8];
                wb[0] = make_float2(1.0f, 0.0f);
                wb[1] = w32k(tw, (k * step) & 32767);
                if (INV) wb[1].y = -wb[1].y;
#pragma unroll
                for (int b = 2; b < 8; b++) wb[b] = cmul(wb[b - 1], wb[1]);
#pragma unroll
                for (int a = 0; a < R / 8; a++) {
                    float2 wa = make_float2(1.0f, 0.0f);
                    if (a > 0) {
                        wa = w32k(tw, (8 * a * k * step) & 32767);
                        if (INV) wa.y = -wa.y;
                    }
#pragma unroll
                    for (int b = 0; b < 8; b++) {
                        int r = 8 * a + b;
                        if (r == 0) continue;
                        float2 w = (a == 0) ? wb[b] : (b == 0 ? wa : cmul(wa, wb[b]));
                        v[i][r] = cmul(v[i][r], w);
                    }
                }
            }
            dft<R, INV>(v[i]);
            dst[i] = base + (j - k) * R + k;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < J; i++) {
        if (act[i]) {
#pragma unroll
            for (int r = 0; r < R; r++) buf[sx(dst[i] + r * Ns)] = v[i][r];
        }
    }
    __syncthreads();
}

// Butterflies per thread of a radix-R pass over `batch` transforms of length L.
__host__ __device__ constexpr int pass_j(int L, int R, int batch) { return (batch * (L / R) + T - 1) / T; }

// The transforms are called, not inlined: each is used at two call sites, and
// one shared copy keeps the kernel's code small enough that instruction fetch
// stops stalling the warps (measured 11 % faster per block).  Each length has
// several three-pass radix plans; the kernel is compiled for the plans in
// kFftPlans (kernels.h), and the host times those once per device and launches
// the fastest (a plan selected at run time inside one kernel cost 2 %, an
// indirect call 20 %).
template <bool INV, int BATCH, int R1, int R2, int R3>
__device__ __noinline__ void fft8192p(float2* buf, const Tw& tw, int tid) {
    static_assert(R1 * R2 * R3 == Q, "radix plan");
    pass<R1, pass_j(Q, R1, BATCH), INV>(buf, Q, BATCH, 1, tw, tid);
    pass<R2, pass_j(Q, R2, BATCH), INV>(buf, Q, BATCH, R1, tw, tid);
    pass<R3, pass_j(Q, R3, BATCH), INV>(buf, Q, BATCH, R1 * R2, tw, tid);
}

template <bool INV, int R1, int R2, int R3>
__device__ __noinline__ void fft16384p(float2* buf, const Tw& tw, int tid) {
    static_assert(R1 * R2 * R3 == M, "radix plan");
    pass<R1, pass_j(M, R1, 1), INV>(buf, M, 1, 1, tw, tid);
    pass<R2, pass_j(M, R2, 1), INV>(buf, M, 1, R1, tw, tid);
    pass<R3, pass_j(M, R3, 1), INV>(buf, M, 1, R1 * R2, tw, tid);
}

// 8192-point transform(s) of plan PLAN (bits 0-1): 16x16x32, 32x16x16,
// 16x32x16 or 8x32x32.
template <bool INV, int BATCH, int PLAN>
__device__ __forceinline__ void fft8192(float2* buf, const Tw& tw, int tid) {
    constexpr int a = PLAN & 3;
    if constexpr (a == 1) fft8192p<INV, BATCH, 32, 16, 16>(buf, tw, tid);
    else if constexpr (a == 2) fft8192p<INV, BATCH, 16, 32, 16>(buf, tw, tid);
    else if constexpr (a == 3) fft8192p<INV, BATCH, 8, 32, 32>(buf, tw, tid);
    else fft8192p<INV, BATCH, 16, 16, 32>(buf, tw, tid);
}

// 16384-point transform of plan PLAN (bits 2-3): 16x32x32, 32x32x16 or 32x16x32.
template <bool INV, int PLAN>
__device__ __forceinline__ void fft16384(float2* buf, const Tw& tw, int tid) {
    constexpr int b = (PLAN >> 2) & 3;
    if constexpr (b == 1) fft16384p<INV, 32, 32, 16>(buf, tw, tid);
    else if constexpr (b == 2) fft16384p<INV, 32, 16, 32>(buf, tw, tid);
    else fft16384p<INV, 16, 32, 32>(buf, tw, tid);
}

struct Shared {
    float2 buf[BUF];
    float theta[M];          // stage 3: angle, then demod, of each local sample
    unsigned repl[N / 32];   // spike windows chosen for replacement (repair path)
    Tw tw;
    float2 nyq;              // Nyquist bin of the rank-0 half spectrum
    float2 tail_z[2][2];     // last two analytic samples of each local chunk
    float tail_theta[2];     // last angle of each local chunk
    float tail_re[2][4];     // last four Re z of each local chunk
    int flag;
    int pad_;
    long long next_blk[2];   // the cluster's next block, by iteration parity
    int next_job[2];         // batched launch: the next block's window
    int cur_job;
    FastDemodParams job;     // batched launch: the current window's parameters
};

// Half-spectrum post-processing of a real FFT computed as a packed complex
// FFT: given C[k] and C[M-k] returns X[k] = (C[k] + C*[M-k])/2
// - (i/2) W_N^k (C[k] - C*[M-k]).
__device__ __forceinline__ float2 real_post(float2 ck, float2 cmk, float2 wk) {
    float2 a = make_float2(0.5f * (ck.x + cmk.x), 0.5f * (ck.y - cmk.y));
    float2 b = make_float2(0.5f * (ck.x - cmk.x), 0.5f * (ck.y + cmk.y));
    // -i * W * b
    float2 wb = cmul(wk, b);
    return make_float2(a.x + wb.y, a.y - wb.x);
}

// Stage 1/4 post-processing: buf[0..8192) holds C at the rank's parity; write
// X * g (g = per-bin real scale supplied by `scale`) back in place.  Rank 0
// writes X[2q] at q (q < 8192) and X[16384] to nyq; rank 1 writes X[2q+1].
template <typename ScaleFn>
__device__ __forceinline__ void post_half(Shared& sh, int rank, int tid, ScaleFn scale) {
    float2* buf = sh.buf;
    if (rank == 0) {
        for (int q = tid; q < 4096; q += T) {
            int q2 = 8192 - q;
            float2 cq = buf[sx(q)];
            float2 cq2 = (q == 0) ? cq : buf[sx(q2)];
            if (q == 0) {
                // X[0] = Re C0 + Im C0, X[M] = Re C0 - Im C0 (both real)
                float x0 = cq.x + cq.y, xm = cq.x - cq.y;
                buf[sx(0)] = scale(0, make_float2(x0, 0.0f));
                sh.nyq = scale(M, make_float2(xm, 0.0f));
                // the self-paired bin 8192 (q = 4096) here, not in a ninth round
                const float2 cm = buf[sx(4096)];
                buf[sx(4096)] = scale(8192, real_post(cm, cm, w32k(sh.tw, 8192)));
            } else {
                int k = 2 * q, k2 = 2 * q2;
                float2 xk = real_post(cq, cq2, w32k(sh.tw, k));
                float2 xk2 = real_post(cq2, cq, w32k(sh.tw, k2));
                buf[sx(q)] = scale(k, xk);
                if (q2 != q) buf[sx(q2)] = scale(k2, xk2);
            }
        }
    } else {
        for (int q = tid; q < 4096; q += T) {
            int q2 = 8191 - q;
            float2 cq = buf[sx(q)], cq2 = buf[sx(q2)];
            int k = 2 * q + 1, k2 = 2 * q2 + 1;
            float2 xk = real_post(cq, cq2, w32k(sh.tw, k));
            float2 xk2 = real_post(cq2, cq, w32k(sh.tw, k2));
            buf[sx(q)] = scale(k, xk);
            buf[sx(q2)] = scale(k2, xk2);
        }
    }
    __syncthreads();
}

// Sample index n held at local position i of `rank`.
__device__ __forceinline__ int pos_to_n(int i, int rank) {
    return ((2 * (i >> 13) + rank) << 13) | (i & 8191);
}

// Affine map composition helpers for the envelope scan.
struct Aff { float a, b; };
__device__ __forceinline__ Aff aff_then(Aff first, Aff second) {
    // apply first, then second: s -> second.a*(first.a*s + first.b) + second.b
    Aff r;
    r.a = second.a * first.a;
    r.b = fmaf(second.a, first.b, second.b);
    return r;
}

__device__ __forceinline__ Aff warp_scan_incl(Aff v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        float pa = __shfl_up_sync(0xffffffffu, v.a, o);
        float pb = __shfl_up_sync(0xffffffffu, v.b, o);
        if (lane >= o) v = aff_then(Aff{pa, pb}, v);
    }
    return v;
}
__device__ __forceinline__ Aff warp_scan_incl_rev(Aff v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        float pa = __shfl_down_sync(0xffffffffu, v.a, o);
        float pb = __shfl_down_sync(0xffffffffu, v.b, o);
        if (lane + o < 32) v = aff_then(Aff{pa, pb}, v);
    }
    return v;
}

// Read raw (component y) or y-envelope (component y) at sample n from the
// owning rank's buffer (local or remote through DSMEM).
__device__ __forceinline__ float chunk_val(float2* local, float2* remote, int rank, int n) {
    int ch = n >> 13;
    int i = ((ch >> 1) << 13) | (n & 8191);
    float2* b = ((ch & 1) == rank) ? local : remote;
    return b[sx(i)].y;
}

// First-order low-pass filtfilt (the one-section case of
// SosFilter.ApplyForwardBackward / ApplyForwardBackwardFloat32,
// Core/Dsp/SosFilter.cs:178-340) of component y of the block held in buf.
// Warp w of this rank covers samples [n0, n0 + 1024) as four rows of 256; in
// each row lane l runs the recurrence over its 8 consecutive samples and a warp
// affine scan joins the lanes.  The state entering the warp's range comes from
// a 256-sample halo started at zero (for the 590 / 700 kHz filters at 40 MSPS
// the memory c^256 is below 1e-10); at the block edges the recursion starts
// from zero instead of the padded steady-state start, which only moves samples
// the overlap-save cut drops.  Component y is overwritten by the forward pass.
// emit(row_start, ms, wv) receives the final values wv[0..8) of samples
// ms..ms+7, rows in descending order.  Called by every thread of both CTAs.
template <typename Emit>
__device__ __forceinline__ void filtfilt_rows(float2* buf, float2* rbuf, int rank, int warp, int lane,
                                              float b0, float b1, float a1, cg::cluster_group& cluster,
                                              Emit emit) {
    const int lc = warp >> 3;
    const int c = 2 * lc + rank;
    const int n0 = c * 8192 + (warp & 7) * 1024;
    const float cc = -a1;
    const float gk = b1 - a1 * b0;   // state input gain
    float c8 = cc;
#pragma unroll
    for (int k = 1; k < 8; k++) c8 *= cc;
    const float* lbuf = reinterpret_cast<const float*>(buf);
    auto local_y = [&](int n) { return lbuf[2 * sx((lc << 13) | (n & 8191)) + 1]; };
    float yv[32];
    // forward: z1' = cc*z1 + gk*e ; y = b0*e + z1
    float carry = 0.0f;
    if (n0 >= 256) {
        int hs = n0 - 256 + lane * 8;
        float st = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; k++) st = fmaf(cc, st, gk * chunk_val(buf, rbuf, rank, hs + k));
        Aff inc = warp_scan_incl(Aff{c8, st}, lane);
        carry = __shfl_sync(0xffffffffu, inc.b, 31);
    }
#pragma unroll
    for (int row = 0; row < 4; row++) {
        int ms = n0 + row * 256 + lane * 8;
        float ev[8];
        float st = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            ev[k] = local_y(ms + k);
            st = fmaf(cc, st, gk * ev[k]);
        }
        Aff inc = warp_scan_incl(Aff{c8, st}, lane);
        float pb = __shfl_up_sync(0xffffffffu, inc.b, 1);
        float pa = __shfl_up_sync(0xffffffffu, inc.a, 1);
        float z = lane == 0 ? carry : fmaf(pa, carry, pb);
#pragma unroll
        for (int k = 0; k < 8; k++) {
            yv[row * 8 + k] = fmaf(b0, ev[k], z);
            z = fmaf(cc, z, gk * ev[k]);
        }
        carry = __shfl_sync(0xffffffffu, z, 31);
    }
    cluster.sync();
    {
        float* wbuf = reinterpret_cast<float*>(buf);
#pragma unroll
        for (int row = 0; row < 4; row++) {
#pragma unroll
            for (int k = 0; k < 8; k++) {
                int n = n0 + row * 256 + lane * 8 + k;
                wbuf[2 * sx((lc << 13) | (n & 8191)) + 1] = yv[row * 8 + k];
            }
        }
    }
    cluster.sync();
    // backward: w = b0*y + z1 ; z1' = cc*z1 + gk*y  (from high n to low n)
    const int nend = n0 + 1024;
    carry = 0.0f;
    if (nend + 256 <= N) {
        int hs = nend + lane * 8;  // halo samples [nend, nend+256)
        float st = 0.0f;
#pragma unroll
        for (int k = 7; k >= 0; k--) st = fmaf(cc, st, gk * chunk_val(buf, rbuf, rank, hs + k));
        Aff inc = warp_scan_incl_rev(Aff{c8, st}, lane);
        carry = __shfl_sync(0xffffffffu, inc.b, 0);
    }
#pragma unroll
    for (int row = 3; row >= 0; row--) {
        int ms = n0 + row * 256 + lane * 8;
        float st = 0.0f;
#pragma unroll
        for (int k = 7; k >= 0; k--) st = fmaf(cc, st, gk * yv[row * 8 + k]);
        Aff inc = warp_scan_incl_rev(Aff{c8, st}, lane);
        float nb = __shfl_down_sync(0xffffffffu, inc.b, 1);
        float na = __shfl_down_sync(0xffffffffu, inc.a, 1);
        float z = lane == 31 ? carry : fmaf(na, carry, nb);
        float wv[8];
#pragma unroll
        for (int k = 7; k >= 0; k--) {
            float y = yv[row * 8 + k];
            wv[k] = fmaf(b0, y, z);
            z = fmaf(cc, z, gk * y);
        }
        carry = __shfl_sync(0xffffffffu, z, 0);
        emit(n0 + row * 256, ms, wv);
    }
}

// Nonlinear gain of the low-passed sub-deemphasis amplitude
// (Core/Dsp/RfDemodulator.cs:2963-2981): max(0, amp) x scale1, ^exponent,
// x scale2, x 1 / (1 + exp(-rate (amp - mid))).  The power and the logistic
// use the hardware base-2 logarithm / exponential and a fast divide; their
// relative error (~1e-6) moves the video by ~1 Hz at most (amp = 0 gives 0).
__device__ __forceinline__ float sub_gain(float amp, const SubDeemph& s) {
    amp = fmaxf(0.0f, amp) * s.scale1;
    amp = exp2f(s.exponent * __log2f(amp)) * s.scale2;
    if (s.logistic_rate > 0.0f)
        amp = __fdividef(amp, 1.0f + __expf(-s.logistic_rate * (amp - s.logistic_mid)));
    return amp;
}

// Complex product with every operation rounded on its own (no contraction).
__device__ __forceinline__ float2 cmul_rn(float2 a, float2 b) {
    return make_float2(__fsub_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
                       __fadd_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}

// Samples 8 v .. 8 v + 7 of the block's first (ha) and second (hb) half into
// this rank's packed DIF input elements p = 4 v + e: rank 0 gets a + b, rank 1
// (a - b) W^(2p), where a / b are the complex pairs of the two halves and
// W^(2p) = W^(8v) W^(2e).  The arithmetic is spelled out rounding by rounding,
// so an int16 capture and a float capture of the same values pack to the
// same bits.
__device__ __forceinline__ void pack_rf(float2* buf, const float* ha, const float* hb, int vi, int rank,
                                        const Tw& tw) {
    float2 w8 = make_float2(1.0f, 0.0f);
    if (rank) w8 = cmul_rn(tw.hi[vi >> 4], tw.lo8[vi & 15]);
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const int pp = 4 * vi + e;
        float2 r;
        if (rank == 0) {
            r = make_float2(__fadd_rn(ha[2 * e], hb[2 * e]), __fadd_rn(ha[2 * e + 1], hb[2 * e + 1]));
        } else {
            const float2 d = make_float2(__fsub_rn(ha[2 * e], hb[2 * e]), __fsub_rn(ha[2 * e + 1], hb[2 * e + 1]));
            r = cmul_rn(d, e == 0 ? w8 : cmul_rn(w8, tw.lo[2 * e]));
        }
        buf[sx(pp)] = r;
    }
}

// One int16 RF block from the prefetch copy in shared memory.
__device__ __forceinline__ void load_rf(float2* buf, const int16_t* x, int rank, const Tw& tw, int tid) {
#pragma unroll
    for (int it = 0; it < 4; it++) {
        const int vi = tid + it * T;  // vector index in [0, 2048)
        const int4 va = reinterpret_cast<const int4*>(x)[vi];
        const int4 vb = reinterpret_cast<const int4*>(x + 16384)[vi];
        const int16_t* a16 = reinterpret_cast<const int16_t*>(&va);
        const int16_t* b16 = reinterpret_cast<const int16_t*>(&vb);
        float ha[8], hb[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            ha[k] = (float)a16[k];
            hb[k] = (float)b16[k];
        }
        pack_rf(buf, ha, hb, vi, rank, tw);
    }
}

// One float RF block (decimated or float input) from global memory; no
// prefetch: two 16-byte loads per half and vector index.
__device__ __forceinline__ void load_rf_f32(float2* buf, const float* x, int rank, const Tw& tw, int tid) {
#pragma unroll
    for (int it = 0; it < 4; it++) {
        const int vi = tid + it * T;  // vector index in [0, 2048)
        const float4* xa = reinterpret_cast<const float4*>(x) + 2 * vi;
        const float4* xb = reinterpret_cast<const float4*>(x + 16384) + 2 * vi;
        const float4 a0 = __ldg(xa), a1 = __ldg(xa + 1), b0 = __ldg(xb), b1 = __ldg(xb + 1);
        const float ha[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const float hb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
        pack_rf(buf, ha, hb, vi, rank, tw);
    }
}

// Diff-demod repair of one block (Core/Dsp/RfDemodulator.cs:966-1001,
// 2527-2582), taken when some demod sample of the block exceeds the limit:
// with the analytic signal still in buf, the demod and the spike mask go to
// cluster scratch, the diff-demod is computed only around spikes, then
// ReplaceSpikes runs in parallel (spikes.cuh) on rank 0 and the repaired demod
// returns to sh.theta.  Out of line: it is the kernel's cold path.
__device__ __noinline__ void repair_block(Shared& sh, Shared* rsh, const FastDemodParams& p, int cluster_id,
                                          int rank) {
    cg::cluster_group cluster = cg::this_cluster();
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    float2* buf = sh.buf;
    const float freq = p.fs;
    if (tid == 0 && rank == 0) atomicAdd(p.repair_count, 1);
    float* ds = reinterpret_cast<float*>(p.scratch + (int64_t)cluster_id * (2 * N));
    float* dds = ds + N;
    unsigned* maskg = reinterpret_cast<unsigned*>(dds + N);
    int* cposg = reinterpret_cast<int*>(maskg + N / 32);
#pragma unroll 4
    for (int t = 0; t < 32; t++) {
        int i = tid + t * T;
        int n = pos_to_n(i, rank);
        float d = sh.theta[i];
        ds[n] = d;
        unsigned m = __ballot_sync(0xffffffffu, d > p.diff_max);   // 32 consecutive n
        if (lane == 0) maskg[n >> 5] = m;
    }
    cluster.sync();
    // diff-demod, only where some window can reach (a spike in [n-29, n+8])
#pragma unroll 2
    for (int t = 0; t < 32; t++) {
        int i = tid + t * T;
        int n = pos_to_n(i, rank);
        int a0 = max(n - 29, 0), a1 = min(n + 8, N - 1);
        bool need = false;
        for (int w = a0 >> 5; w <= (a1 >> 5); w++) {
            int lo = max(a0 - w * 32, 0), hi = min(a1 - w * 32, 31);
            unsigned sel = (hi == 31 ? 0xffffffffu : ((2u << hi) - 1u)) & ~((1u << lo) - 1u);
            need = need || (maskg[w] & sel) != 0u;
        }
        if (!need) continue;
        float dd = 0.0f;
        if (n >= 1) {
            int il = i & 8191;
            int c = 2 * (i >> 13) + rank;
            int plc = ((c + 3) & 3) >> 1;
            float2 z0 = buf[sx(i)];
            float2 z1 = il >= 1 ? buf[sx(i - 1)] : rsh->tail_z[plc][1];
            float2 dz = csub(z0, z1);
            float th = vhs_atan2(dz.y, dz.x);
            float thp;
            if (n >= 2) {
                float2 z2 = il >= 2 ? buf[sx(i - 2)] : rsh->tail_z[plc][il == 1 ? 1 : 0];
                float2 dzp = csub(z1, z2);
                thp = vhs_atan2(dzp.y, dzp.x);
            } else {
                thp = vhs_atan2(0.0f, 0.0f);
            }
            dd = vhs_freq_diff(th, thp, freq);
        }
        dds[n] = dd;
    }
    cluster.sync();
    if (rank == 0) {
        spike_thresholds(ds, dds, maskg, cposg, N, tid, T);
        __syncthreads();
        if (warp == 0) spike_walk(maskg, cposg, sh.repl, N, lane);
        __syncthreads();
        spike_apply(ds, dds, sh.repl, N, tid, T);
    }
    cluster.sync();
#pragma unroll 4
    for (int t = 0; t < 32; t++) {
        int i = tid + t * T;
        sh.theta[i] = ds[pos_to_n(i, rank)];
    }
    __syncthreads();
}


// Bits 0..15 of x to the even bit positions of the result.
__device__ __forceinline__ unsigned spread16(unsigned x) {
    x &= 0xffffu;
    x = (x | (x << 8)) & 0x00ff00ffu;
    x = (x | (x << 4)) & 0x0f0f0f0fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}

// Pulse-scan bits of the sync reference samples base + 2 lane and base +
// 2 lane + 1 (q.x, q.y) held by the 32 lanes of a warp: condition (v <= the
// exact float threshold of the pulse scan) and hold (NaN) words for stream
// samples [sbase + base, sbase + base + 64), written where the word lies in
// the kept range.  Called by all 32 lanes.
__device__ __forceinline__ void sync_bits(float2 q, int base, int64_t sbase, const FastDemodParams& p,
                                          int lane) {
    const unsigned ce = __ballot_sync(0xffffffffu, q.x <= p.sync_thr);
    const unsigned co = __ballot_sync(0xffffffffu, q.y <= p.sync_thr);
    const unsigned he = __ballot_sync(0xffffffffu, q.x != q.x);
    const unsigned ho = __ballot_sync(0xffffffffu, q.y != q.y);
    if (lane < 2) {
        const int n = base + 32 * lane;   // first block sample of this lane's word
        if (n >= CUT + 32 && n + 32 <= CUT + 32 + S) {
            const int sh = 16 * lane;
            const unsigned c = spread16(ce >> sh) | (spread16(co >> sh) << 1);
            const unsigned h = spread16(he >> sh) | (spread16(ho >> sh) << 1);
            const int64_t w = (sbase + n) >> 5;
            p.sync_cond[w] = c;
            p.sync_hold[w] = h;
        }
    }
}

// Next block's RF (32768 int16 = 64 KB, both halves) into `dst` with
// asynchronous 16-byte copies (8 per thread), overlapping the current block's
// later stages; prefetch_wait() + a barrier make it visible.
__device__ __forceinline__ void prefetch_rf(void* dst, const int16_t* x, int tid) {
    const char* src = reinterpret_cast<const char*>(x);
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int off = (tid + i * T) * 16;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d + off), "l"(src + off) : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void prefetch_wait() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// RfVideo entries 0..16383 (64 KB, 16-byte aligned) into `dst` with
// asynchronous 16-byte copies (8 per thread): issued before the stage-1
// transform, waited for after it, so the stage-1 products read the table from
// shared memory instead of waiting for L2.
__device__ __forceinline__ void stage_rf_table(float* dst, const float* tab, int tid) {
    const char* src = reinterpret_cast<const char*>(tab);
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int off = (tid + i * T) * 16;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d + off), "l"(src + off) : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

}  // namespace fp32
}  // namespace vhsd

using namespace vhsd;
using namespace vhsd::fp32;

// Stage marks of the timed diagnostic build: thread 0 of each CTA adds the
// cycles since the previous mark to stage_cycles[rank][k].
#define VHSD_MARK(k)                                                                             \
    do {                                                                                         \
        if constexpr (TIMED) {                                                                   \
            if (tid == 0) {                                                                      \
                const long long c_ = clock64();                                                  \
                atomicAdd(p.stage_cycles + rank * kDemodStages + (k), (unsigned long long)(c_ - t_mark)); \
                t_mark = c_;                                                                     \
            }                                                                                    \
        }                                                                                        \
    } while (0)

// Window of global block g in a batched launch (the last job starting at or before g).
__device__ __forceinline__ int batch_job_of(const FastDemodParams& pk, int64_t g) {
    int lo = 0, hi = pk.batch_njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pk.batch_start[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int PLAN, bool TIMED, bool BATCHED>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(T, 1)
vhsd_demod_fp32_kernel(FastDemodParams pk) {
    long long t_mark = 0;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Shared& sh = *reinterpret_cast<Shared*>(smem_raw);
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    float2* buf = sh.buf;
    Shared* rsh = cluster.map_shared_rank(&sh, rank ^ 1);
    float2* rbuf = rsh->buf;

    for (int i = tid; i < 256; i += T) sh.tw.hi[i] = pk.tw_hi[i];
    for (int i = tid; i < 128; i += T) sh.tw.lo[i] = pk.tw_lo[i];
    for (int i = tid; i < 16; i += T) sh.tw.lo8[i] = pk.tw_lo[8 * i];
    if constexpr (BATCHED) {
        if (tid == 0) sh.cur_job = (blockIdx.x >> 1) < pk.nblocks ? batch_job_of(pk, blockIdx.x >> 1) : 0;
    }
    __syncthreads();

    const int cluster_id = blockIdx.x >> 1;
    const int nclusters = gridDim.x >> 1;
    const float inv_n = 1.0f / (float)N;
    const float inv_m = 1.0f / (float)M;
    // the RF of each block is prefetched into sh.theta (free from the demod's
    // last read until the next block's angles) while the previous block
    // finishes
    // (int16 captures only; a float capture is read from global memory)
    // (batched launches take int16 captures only)
    const int16_t* rf_smem = reinterpret_cast<const int16_t*>(sh.theta);
    const bool f32_in = !BATCHED && pk.rf_f32 != nullptr;
    if (cluster_id < pk.nblocks && !f32_in) {
        if constexpr (BATCHED) {
            const FastDemodParams& j0 = pk.batch_jobs[sh.cur_job];
            prefetch_rf(sh.theta, j0.rf + (cluster_id - pk.batch_start[sh.cur_job] + j0.first_block) * (int64_t)S,
                        tid);
        } else {
            prefetch_rf(sh.theta, pk.rf + (cluster_id + pk.first_block) * (int64_t)S, tid);
        }
    }
    // Blocks: each cluster starts on block cluster_id and then claims the next
    // unclaimed block from the launch's counter, so clusters that start late
    // (their SMs busy with other work) or take the slow repair path simply
    // take fewer blocks.  Rank 0 claims at the top of a block and publishes the
    // index to both CTAs (slot by iteration parity); both read it after the
    // next cluster barrier, so the two ranks always agree.
    int par = 0;
    int job = -1;
    for (int64_t g = cluster_id; g < pk.nblocks;) {
        // g: the block's index in the launch; blk: its index in its window
        int64_t blk = g;
        if constexpr (BATCHED) {
            const int j = sh.cur_job;
            if (j != job) {   // every thread of both CTAs is past the previous block
                const unsigned long long* src = reinterpret_cast<const unsigned long long*>(pk.batch_jobs + j);
                unsigned long long* dst = reinterpret_cast<unsigned long long*>(&sh.job);
                for (int i = tid; i < (int)(sizeof(FastDemodParams) / 8); i += T) dst[i] = src[i];
                job = j;
                __syncthreads();
            }
            blk = g - pk.batch_start[j];
        }
        const FastDemodParams& p = BATCHED ? sh.job : pk;
        const float freq = p.fs;
        if (rank == 0 && tid == 0) {
            const long long nb = pk.block_counter ? (long long)nclusters + atomicAdd(pk.block_counter, 1)
                                                  : (long long)(g + nclusters);
            sh.next_blk[par] = nb;
            rsh->next_blk[par] = nb;
            if constexpr (BATCHED) {
                const int nj = nb < pk.nblocks ? batch_job_of(pk, nb) : 0;
                sh.next_job[par] = nj;
                rsh->next_job[par] = nj;
            }
        }
        // ---------------- stage 1: RF forward FFT (packed, DIF split) -----
        prefetch_wait();
        __syncthreads();
        if constexpr (TIMED) t_mark = clock64();
        if (f32_in) load_rf_f32(buf, p.rf_f32 + (blk + p.first_block) * (int64_t)S, rank, sh.tw, tid);
        else load_rf(buf, rf_smem, rank, sh.tw, tid);
        __syncthreads();
        // theta (the RF copy) is consumed: it holds the RfVideo table until the angles
        stage_rf_table(sh.theta, p.rf_video, tid);
        VHSD_MARK(0);
        fft8192<false, 1, PLAN>(buf, sh.tw, tid);
        VHSD_MARK(1);
        prefetch_wait();
        __syncthreads();
        // X * RfVideo * Hilbert / N  (Hilbert: 1 at 0 and N/2, 2 between)
        {
            const float tab_m = __ldg(p.rf_video + M);
            post_half(sh, rank, tid, [&](int k, float2 v) {
                float g = (k < M ? sh.theta[k] : tab_m) * ((k == 0 || k == M) ? inv_n : 2.0f * inv_n);
                return make_float2(v.x * g, v.y * g);
            });
        }
        VHSD_MARK(2);
        // ---------------- stage 2: analytic inverse FFT -----------------
        if (rank == 0) {
            if (tid == 0) buf[sx(8192)] = sh.nyq;
            for (int i = 8193 + tid; i < M; i += T) buf[sx(i)] = make_float2(0.f, 0.f);
        } else {
            for (int i = 8192 + tid; i < M; i += T) buf[sx(i)] = make_float2(0.f, 0.f);
        }
        __syncthreads();
        VHSD_MARK(3);
        fft16384<true, PLAN>(buf, sh.tw, tid);
        VHSD_MARK(4);
        cluster.sync();
        VHSD_MARK(5);
        const int64_t nxt = sh.next_blk[par];
        const bool has_next = nxt < pk.nblocks && !f32_in;
        const int16_t* x_next = nullptr;
        if (has_next) {
            if constexpr (BATCHED) {
                const int nj = sh.next_job[par];
                const FastDemodParams& jn = pk.batch_jobs[nj];
                x_next = jn.rf + (nxt - pk.batch_start[nj] + jn.first_block) * (int64_t)S;
            } else {
                x_next = pk.rf + (nxt + pk.first_block) * (int64_t)S;
            }
        }
        {
            // z[n] = A[n] + W^-n B[n], z[n+16384] = A[n] - W^-n B[n]; the
            // analytic signal stays in buf (chunk rank at local 0..8191,
            // chunk rank + 2 at 8192..16383) until the demod is final
            float2 o1[16], o2[16];
#pragma unroll
            for (int t = 0; t < 16; t++) {
                int nl = tid + t * T;                 // [0, 8192)
                int n = nl + rank * 8192;             // [0, 16384)
                float2 loc = buf[sx(n)];
                float2 rem = rbuf[sx(n)];
                float2 a = rank == 0 ? loc : rem;
                float2 b = rank == 0 ? rem : loc;
                float2 wb = cmulc(b, w32k(sh.tw, n));
                o1[t] = cadd(a, wb);
                o2[t] = csub(a, wb);
                sh.theta[nl] = vhs_atan2(o1[t].y, o1[t].x);
                sh.theta[8192 + nl] = vhs_atan2(o2[t].y, o2[t].x);
            }
            cluster.sync();
#pragma unroll
            for (int t = 0; t < 16; t++) {
                int nl = tid + t * T;
                buf[sx(nl)] = o1[t];          // chunk rank
                buf[sx(8192 + nl)] = o2[t];   // chunk rank + 2
            }
        }
        __syncthreads();
        VHSD_MARK(6);
        // ---------------- stage 3: demod, spike check ----------------------
        if (tid < 2) {
            int i_last = tid * 8192 + 8191;
            sh.tail_theta[tid] = sh.theta[i_last];
            for (int k = 0; k < 4; k++) sh.tail_re[tid][k] = buf[sx(i_last - 3 + k)].x;
            sh.tail_z[tid][0] = buf[sx(i_last - 1)];
            sh.tail_z[tid][1] = buf[sx(i_last)];
        }
        cluster.sync();
        bool spike = false;
        {
            float dv[32];
#pragma unroll
            for (int t = 0; t < 32; t++) {
                int i = tid + t * T;        // local position [0, 16384)
                int n = pos_to_n(i, rank);
                int il = i & 8191;
                int c = 2 * (i >> 13) + rank;  // chunk of n
                int plc = ((c + 3) & 3) >> 1;  // predecessor chunk (other rank) slot
                float th = sh.theta[i];
                float thp = (il > 0) ? sh.theta[i - 1] : rsh->tail_theta[plc];
                float d = (n == 0) ? 0.0f : vhs_freq_diff(th, thp, freq);
                dv[t] = d;
                if (n >= 20 && n < N - 20 && d > p.diff_max) spike = true;
            }
            __syncthreads();
#pragma unroll
            for (int t = 0; t < 32; t++) sh.theta[tid + t * T] = dv[t];   // theta now holds the demod
        }
        int any = __syncthreads_or(spike ? 1 : 0);
        if (tid == 0) sh.flag = any;
        cluster.sync();
        VHSD_MARK(7);
        any = sh.flag | rsh->flag;
        if (any) repair_block(sh, rsh, p, cluster_id, rank);
        VHSD_MARK(8);
        // buf <- (demod, raw envelope |Re z[n-4]|)
        {
            float dv[32], rv[32];
#pragma unroll
            for (int t = 0; t < 32; t++) {
                int i = tid + t * T;
                int il = i & 8191;
                int c = 2 * (i >> 13) + rank;
                int plc = ((c + 3) & 3) >> 1;
                dv[t] = sh.theta[i];
                float re = (il >= 4) ? buf[sx(i - 4)].x : rsh->tail_re[plc][il];
                rv[t] = fabsf(re);
            }
            __syncthreads();
#pragma unroll
            for (int t = 0; t < 32; t++) buf[sx(tid + t * T)] = make_float2(dv[t], rv[t]);
        }
        cluster.sync();   // the envelope halos read the partner's buf
        VHSD_MARK(9);
        // ---------------- envelope: 700 kHz filtfilt of |Re z[n-4]| ----------
        {
            float* envo = p.env_out + (blk + p.first_block) * (int64_t)S - CUT;
            filtfilt_rows(buf, rbuf, rank, warp, lane, p.env_b0, p.env_b1, p.env_a1, cluster,
                          [&](int rs, int ms, const float* wv) {
                              // rows lie wholly inside or outside the kept range
                              if (rs >= CUT && rs < CUT + S) {
                                  float4* o = reinterpret_cast<float4*>(envo + ms);
                                  o[0] = make_float4(wv[0], wv[1], wv[2], wv[3]);
                                  o[1] = make_float4(wv[4], wv[5], wv[6], wv[7]);
                              }
                          });
        }
        VHSD_MARK(10);
        if (has_next && p.sub.high == nullptr) prefetch_rf(sh.theta, x_next, tid);
        // ---------------- stage 4: forward FFT of (demod - ire0) -----------
        {
            float2 uo[8], vo[8];
            int pidx[8];
#pragma unroll
            for (int t = 0; t < 8; t++) {
                int pl = tid + t * T;              // [0, 4096)
                int pp = pl + rank * 4096;         // p
                pidx[t] = pp;
                float d0 = buf[sx(2 * pl)].x - p.dc, d1 = buf[sx(2 * pl + 1)].x - p.dc;
                float e0 = buf[sx(8192 + 2 * pl)].x - p.dc, e1 = buf[sx(8192 + 2 * pl + 1)].x - p.dc;
                float2 ca = make_float2(d0, d1), cb = make_float2(e0, e1);
                uo[t] = cadd(ca, cb);
                vo[t] = cmul(csub(ca, cb), w32k(sh.tw, 2 * pp));
            }
            cluster.sync();
#pragma unroll
            for (int t = 0; t < 8; t++) {
                int pp = pidx[t];
                if (rank == 0) { buf[sx(pp)] = uo[t]; rbuf[sx(pp)] = vo[t]; }
                else { rbuf[sx(pp)] = uo[t]; buf[sx(pp)] = vo[t]; }
            }
            cluster.sync();
        }
        VHSD_MARK(11);
        fft8192<false, 1, PLAN>(buf, sh.tw, tid);
        VHSD_MARK(12);
        post_half(sh, rank, tid, [&](int k, float2 v) { return v; });
        VHSD_MARK(13);
        const bool sub = p.sub.high != nullptr;
        float2* xs = reinterpret_cast<float2*>(sh.theta);   // D kept for stage 6
        if (sub) {
            for (int q = tid; q < 8192; q += T) xs[q] = buf[sx(q)];
            __syncthreads();   // stage 5 rewrites these bins in place
        }
        // ---------------- stage 5: video and sync real inverse FFTs ---------
        {
            // F = X * H ; P[k] = (F[k] + F*[M-k])/2 + i (F[k] - F*[M-k]) W_N^-k / 2, scaled 1/M
            const float sc = 0.5f * inv_m;
            auto prep = [&](float2 fk, float2 fmk, int k) {
                float2 a = make_float2(fk.x + fmk.x, fk.y - fmk.y);
                float2 b = make_float2(fk.x - fmk.x, fk.y + fmk.y);
                float2 bw = cmulc(b, w32k(sh.tw, k));
                // a + i*bw
                return make_float2(sc * (a.x - bw.y), sc * (a.y + bw.x));
            };
            if (rank == 0) {
                for (int q = tid; q < 4096; q += T) {
                    int q2 = 8192 - q;
                    int k = 2 * q, k2 = 2 * q2;
                    float2 xk = buf[sx(q)];
                    float2 xk2 = (q == 0) ? sh.nyq : buf[sx(q2)];
                    if (q == 0) { xk.y = 0.f; xk2.y = 0.f; }
                    float2 hv = __ldg(p.video + k), hv2 = __ldg(p.video + k2);
                    float2 hs = __ldg(p.sync + k), hs2 = __ldg(p.sync + k2);
                    float2 fv = cmul(xk, hv), fv2 = cmul(xk2, hv2);
                    float2 fs = cmul(xk, hs), fs2 = cmul(xk2, hs2);
                    if (q == 0) { fv.y = 0.f; fv2.y = 0.f; fs.y = 0.f; fs2.y = 0.f; }
                    float2 pv = prep(fv, fv2, k), ps = prep(fs, fs2, k);
                    buf[sx(q)] = pv;
                    buf[sx(8192 + q)] = ps;
                    if (q != 0) {
                        buf[sx(q2)] = prep(fv2, fv, k2);
                        buf[sx(8192 + q2)] = prep(fs2, fs, k2);
                    } else {
                        // the self-paired bin 8192 (q = 4096) here, not in a ninth round
                        const float2 xm = buf[sx(4096)];
                        const float2 hvm = __ldg(p.video + 8192), hsm = __ldg(p.sync + 8192);
                        const float2 fvm = cmul(xm, hvm), fsm = cmul(xm, hsm);
                        buf[sx(4096)] = prep(fvm, fvm, 8192);
                        buf[sx(8192 + 4096)] = prep(fsm, fsm, 8192);
                    }
                }
            } else {
                for (int q = tid; q < 4096; q += T) {
                    int q2 = 8191 - q;
                    int k = 2 * q + 1, k2 = 2 * q2 + 1;
                    float2 xk = buf[sx(q)], xk2 = buf[sx(q2)];
                    float2 hv = __ldg(p.video + k), hv2 = __ldg(p.video + k2);
                    float2 hs = __ldg(p.sync + k), hs2 = __ldg(p.sync + k2);
                    float2 fv = cmul(xk, hv), fv2 = cmul(xk2, hv2);
                    float2 fs = cmul(xk, hs), fs2 = cmul(xk2, hs2);
                    buf[sx(q)] = prep(fv, fv2, k);
                    buf[sx(q2)] = prep(fv2, fv, k2);
                    buf[sx(8192 + q)] = prep(fs, fs2, k);
                    buf[sx(8192 + q2)] = prep(fs2, fs, k2);
                }
            }
            __syncthreads();
            VHSD_MARK(14);
            fft8192<true, 2, PLAN>(buf, sh.tw, tid);
            VHSD_MARK(15);
            cluster.sync();
            VHSD_MARK(16);
            float* vout = p.video_out + (blk + p.first_block) * (int64_t)S - CUT;
            float* sout = p.sync_out + (blk + p.first_block) * (int64_t)S - CUT - 32;
            // the removed DC returns through each filter's DC gain
            const float dcv = p.dc_video, dcs = p.dc_sync;
#pragma unroll 2
            for (int t = 0; t < 8; t++) {
                int ml = tid + t * T;              // [0, 4096)
                int m = ml + rank * 4096;          // [0, 8192)
                float2 w = w32k(sh.tw, 2 * m);     // W_M^m = W_N^{2m}
#pragma unroll
                for (int sig = 0; sig < 2; sig++) {
                    int off = sig * 8192;
                    float2 loc = buf[sx(off + m)], rem = rbuf[sx(off + m)];
                    float2 a = rank == 0 ? loc : rem;
                    float2 b = rank == 0 ? rem : loc;
                    float2 wb = cmulc(b, w);
                    float2 p1 = cadd(a, wb), p2 = csub(a, wb);
                    int n1 = 2 * m, n2 = 2 * m + 16384;
                    if (sig == 0) {
                        if (n1 >= CUT && n1 < CUT + S)
                            *reinterpret_cast<float2*>(vout + n1) = make_float2(p1.x + dcv, p1.y + dcv);
                        if (n2 >= CUT && n2 < CUT + S)
                            *reinterpret_cast<float2*>(vout + n2) = make_float2(p2.x + dcv, p2.y + dcv);
                    } else {
                        const float2 q1 = make_float2(p1.x + dcs, p1.y + dcs);
                        const float2 q2 = make_float2(p2.x + dcs, p2.y + dcs);
                        if (n1 >= CUT + 32 && n1 < CUT + 32 + S) *reinterpret_cast<float2*>(sout + n1) = q1;
                        if (n2 >= CUT + 32 && n2 < CUT + 32 + S) *reinterpret_cast<float2*>(sout + n2) = q2;
                        if (p.sync_cond) {
                            // the pulse scan's inputs as bits: v <= threshold and
                            // NaN, for the warp's 64 consecutive samples of each half
                            const int64_t sbase = (blk + p.first_block) * (int64_t)S - CUT - 32;
                            const int base1 = 2 * (m - lane);
                            sync_bits(q1, base1, sbase, p, lane);
                            sync_bits(q2, base1 + 16384, sbase, p, lane);
                        }
                    }
                }
            }
        }
        VHSD_MARK(17);
        if (sub) {
            // ---------------- stage 6: S-VHS sub-deemphasis -------------------
            // A[k] = D[k] Video[k] HighPass[k] (x2 for 0 < k < N/2, real part
            // at 0 and N/2, zero above): ifft(A) is the analytic signal of
            // high = irfft(D Video HighPass), whose real part is `high` and
            // whose modulus is the reference's analytic magnitude
            // (BuildAnalyticMagnitudeWithWorkspace, RfDemodulator.cs:3181-3220).
            // The video written above is corrected in place: every sample a
            // rank stores lies in its own two chunks.
            cluster.sync();   // the partner has finished reading this buf
            const float s2 = 2.0f * inv_n;
            for (int q = tid; q < 8192; q += T) {
                int k = 2 * q + rank;
                float2 v = cmul(xs[q], __ldg(p.sub.high + k));
                buf[sx(q)] = (k == 0) ? make_float2(v.x * inv_n, 0.0f) : make_float2(v.x * s2, v.y * s2);
            }
            if (rank == 0) {
                if (tid == 0) {
                    float2 v = cmul(sh.nyq, __ldg(p.sub.high + M));
                    buf[sx(8192)] = make_float2(v.x * inv_n, 0.0f);
                }
                for (int i = 8193 + tid; i < M; i += T) buf[sx(i)] = make_float2(0.f, 0.f);
            } else {
                for (int i = 8192 + tid; i < M; i += T) buf[sx(i)] = make_float2(0.f, 0.f);
            }
            __syncthreads();
            if (has_next) prefetch_rf(sh.theta, x_next, tid);   // the saved spectrum is consumed
            fft16384<true, PLAN>(buf, sh.tw, tid);
            cluster.sync();
            {
                // (high, |a| * 2 / deviation) in the time layout of the envelope
                float2 o1[16], o2[16];
#pragma unroll
                for (int t = 0; t < 16; t++) {
                    int nl = tid + t * T;
                    int n = nl + rank * 8192;
                    float2 loc = buf[sx(n)];
                    float2 rem = rbuf[sx(n)];
                    float2 a = rank == 0 ? loc : rem;
                    float2 b = rank == 0 ? rem : loc;
                    float2 wb = cmulc(b, w32k(sh.tw, n));
                    float2 z1 = cadd(a, wb), z2 = csub(a, wb);
                    o1[t] = make_float2(z1.x, sqrtf(fmaf(z1.x, z1.x, z1.y * z1.y)) * p.sub.inv_half_dev);
                    o2[t] = make_float2(z2.x, sqrtf(fmaf(z2.x, z2.x, z2.y * z2.y)) * p.sub.inv_half_dev);
                }
                cluster.sync();
#pragma unroll
                for (int t = 0; t < 16; t++) {
                    int nl = tid + t * T;
                    buf[sx(nl)] = o1[t];
                    buf[sx(8192 + nl)] = o2[t];
                }
            }
            cluster.sync();
            float* vfix = p.video_out + (blk + p.first_block) * (int64_t)S - CUT;
            const float stat = p.sub.static_factor;
            filtfilt_rows(buf, rbuf, rank, warp, lane, p.sub.b0, p.sub.b1, p.sub.a1, cluster,
                          [&](int rs, int ms, const float* wv) {
                              if (rs >= CUT && rs < CUT + S) {
                                  float4* o = reinterpret_cast<float4*>(vfix + ms);
                                  float4 va = o[0], vb = o[1];
                                  float vv[8] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
                                  const int base = ((ms >> 14) << 13) | (ms & 8191);   // local index of ms
#pragma unroll
                                  for (int k = 0; k < 8; k++) {
                                      float h = buf[sx(base + k)].x;
                                      float g = sub_gain(wv[k], p.sub);
                                      vv[k] -= h * (1.0f - g) + h * stat;
                                  }
                                  o[0] = make_float4(vv[0], vv[1], vv[2], vv[3]);
                                  o[1] = make_float4(vv[4], vv[5], vv[6], vv[7]);
                              }
                          });
        }
        VHSD_MARK(18);
        cluster.sync();
        VHSD_MARK(19);
        if constexpr (BATCHED) {
            if (tid == 0) sh.cur_job = sh.next_job[par];
            __syncthreads();
        }
        g = nxt;
        par ^= 1;
    }
}

namespace vhsd {

size_t fp32_smem_bytes() { return sizeof(fp32::Shared); }

template <int PLAN, bool TIMED = false, bool BATCHED = false>
static cudaError_t launch_plan(const FastDemodParams& p, int clusters, cudaStream_t stream, int dev) {
    static std::atomic<uint64_t> attr_set{0};
    size_t smem = sizeof(fp32::Shared);
    const uint64_t bit = dev < 64 ? (uint64_t)1 << dev : 0;
    if (!bit || !(attr_set.load() & bit)) {
        cudaError_t e = cudaFuncSetAttribute(vhsd_demod_fp32_kernel<PLAN, TIMED, BATCHED>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_set.fetch_or(bit);
    }
    if (p.nblocks <= 0) return cudaSuccess;
    vhsd_demod_fp32_kernel<PLAN, TIMED, BATCHED><<<2 * clusters, fp32::T, smem, stream>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_demod_fp32_batched(const FastDemodParams& p, int num_clusters, cudaStream_t stream) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (p.nblocks > 0 && (!p.batch_jobs || !p.batch_start || p.batch_njobs <= 0)) return cudaErrorInvalidValue;
    int clusters = num_clusters;
    if (p.nblocks > 0 && clusters > p.nblocks) clusters = (int)p.nblocks;
    if (clusters < 1) clusters = 1;
    switch (p.fft_plan) {
    case kFftPlans[0]: return launch_plan<kFftPlans[0], false, true>(p, clusters, stream, dev);
    case kFftPlans[1]: return launch_plan<kFftPlans[1], false, true>(p, clusters, stream, dev);
    case kFftPlans[2]: return launch_plan<kFftPlans[2], false, true>(p, clusters, stream, dev);
    case kFftPlans[3]: return launch_plan<kFftPlans[3], false, true>(p, clusters, stream, dev);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_demod_fp32_timed(const FastDemodParams& p, int num_clusters, cudaStream_t stream) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (!p.stage_cycles) return cudaErrorInvalidValue;
    int clusters = num_clusters;
    if (p.nblocks > 0 && clusters > p.nblocks) clusters = (int)p.nblocks;
    if (clusters < 1) clusters = 1;
    return launch_plan<0, true>(p, clusters, stream, dev);
}

// The shared-memory attribute is set once per device and plan (the first call
// on a device must not be inside a stream capture).
cudaError_t launch_demod_fp32(const FastDemodParams& p, int num_clusters, cudaStream_t stream) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    int clusters = num_clusters;
    if (p.nblocks > 0 && clusters > p.nblocks) clusters = (int)p.nblocks;
    if (clusters < 1) clusters = 1;
    static_assert(kFftPlanCount == 4, "plan list");
    switch (p.fft_plan) {
    case kFftPlans[0]: return launch_plan<kFftPlans[0]>(p, clusters, stream, dev);
    case kFftPlans[1]: return launch_plan<kFftPlans[1]>(p, clusters, stream, dev);
    case kFftPlans[2]: return launch_plan<kFftPlans[2]>(p, clusters, stream, dev);
    case kFftPlans[3]: return launch_plan<kFftPlans[3]>(p, clusters, stream, dev);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace vhsd
