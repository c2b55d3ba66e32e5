// Field-level kernels of the VHS path: sync-pulse edge extraction, hsync edge
// refinement, sinc TBC resampling to 4fSC uint16, envelope dropout runs.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "kernels.h"

namespace vhsd {

// ============================================================== pulses
// PulseDetection.FindPulses (Core/Dsp/PulseDetection.cs:45-222) as edge
// events over the whole stitched stream.  Event = 2*position + type with type
// 0 for a pulse start (value <= high entered) and 1 for a pulse end (value >
// high entered).  NaN keeps the state, as the reference's comparisons do.
namespace {
constexpr int kPWarpSamples = 1024;           // contiguous samples per warp
constexpr int kPT = kPulseChunk / kPWarpSamples * 32;  // threads per CTA (4 warps)

// Exact comparison threshold: for a float sample v and a double h,
// v <= h  <=>  v <= hf  with hf the largest float not above h.
template <typename T>
struct Cmp {
    T h;
};
template <typename T>
__host__ __device__ inline Cmp<T> make_cmp(double high);
template <>
__host__ __device__ inline Cmp<double> make_cmp<double>(double high) { return {high}; }
template <>
__host__ __device__ inline Cmp<float> make_cmp<float>(double high) {
    float f = (float)high;
    if ((double)f > high) f = nextafterf(f, -INFINITY);
    return {f};
}

template <typename T>
__device__ __forceinline__ bool state_before(const T* ref, int64_t p0, T h) {
    for (int64_t q = p0 - 1; q >= 0; q--) {
        T v = ref[q];
        if (v <= h) return true;
        if (v > h) return false;
    }
    return false;
}

// Edge bits of 32 consecutive samples given the state before the first one.
// NaN samples (and samples past the end) keep the state.
__device__ __forceinline__ unsigned edge_bits(unsigned cond, unsigned hold, unsigned& st) {
    if (hold == 0u) {
        unsigned prev = (cond << 1) | st;
        st = cond >> 31;
        return cond ^ prev;
    }
    unsigned s = st, edges = 0u;
    for (int b = 0; b < 32; b++) {
        if ((hold >> b) & 1u) continue;
        unsigned c = (cond >> b) & 1u;
        if (c != s) edges |= 1u << b;
        s = c;
    }
    st = s;
    return edges;
}

// Two passes over a stream range, 1024 samples per warp, kPT threads per CTA.
// Pass 0 counts each warp's edge events (counts[warp]) and each CTA's sum; the
// CTA that finishes last (a ticket taken after a fence, so every other CTA's
// sum is visible to it) scans the CTA sums into exclusive CTA offsets and the
// total.  No CTA waits on another.  Pass 1 recounts nothing: a warp's offset
// is its CTA's offset plus the counts of the warps before it in the CTA, and
// it writes its events in order.  offsets layout: [0] ticket (zeroed before
// pass 0), [1, 1 + nchunks) CTA offsets, [1 + nchunks, 1 + 2 nchunks) CTA sums.
// Pass-0 tail shared by the float and the bit scans: each warp's count to
// counts[warp], the CTA's sum to offsets[1 + nchunks + CTA]; the CTA that
// takes the last ticket scans the CTA sums into offsets[1 .. 1 + nchunks) and
// the total.  Called by every thread of the CTA (cnt valid on lane 0).
__device__ __forceinline__ void finish_counts(int64_t cnt, int64_t wg, int64_t* counts, int64_t* offsets,
                                              int64_t* total, int64_t nchunks) {
    constexpr int kWarps = kPT / 32;
    __shared__ int64_t wcnt[kWarps];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    if (lane == 0) {
        counts[wg] = cnt;
        wcnt[wl] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t sum = 0;
        for (int k = 0; k < kWarps; k++) sum += wcnt[k];
        offsets[1 + nchunks + blockIdx.x] = sum;
        __threadfence();
        unsigned long long t = atomicAdd(reinterpret_cast<unsigned long long*>(offsets), 1ull);
        last = t == (unsigned long long)(nchunks - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // exclusive scan of the CTA sums (read from L2: other CTAs wrote them)
    __shared__ int64_t wsum[kWarps];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < nchunks; base += kPT) {
        int64_t i = base + threadIdx.x;
        int64_t v = i < nchunks ? __ldcg(offsets + 1 + nchunks + i) : 0;
        int64_t incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) wsum[wl] = incl;
        __syncthreads();
        int64_t wb = 0, tot = 0;
        for (int k = 0; k < kWarps; k++) {
            if (k < wl) wb += wsum[k];
            tot += wsum[k];
        }
        if (i < nchunks) offsets[1 + i] = carry + wb + incl - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) total[0] = carry;
}

template <typename T, bool WRITE>
__global__ void __launch_bounds__(kPT) k_pulse_pass(const T* __restrict__ ref, int64_t begin, int64_t n,
                                                    Cmp<T> cmp, int64_t* counts, int64_t* offsets,
                                                    int64_t* events, int64_t capacity, int64_t* total,
                                                    int64_t nchunks) {
    constexpr int kWarps = kPT / 32;
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const int64_t wg = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t start = begin + wg * kPWarpSamples;
    int64_t cnt = 0;
    if (start < n) {
        unsigned st = 0u;
        if (lane == 0) st = state_before(ref, start, cmp.h) ? 1u : 0u;
        st = __shfl_sync(0xffffffffu, st, 0);
        int64_t off = 0;
        if (WRITE) {
            off = offsets[1 + blockIdx.x];
            for (int k = 0; k < wl; k++) off += counts[(int64_t)blockIdx.x * kWarps + k];
        }
        // eight loads in flight per lane, then the ballots in order
        for (int it0 = 0; it0 < kPWarpSamples / 32; it0 += 8) {
            T vv[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                int64_t p = start + (it0 + j) * 32 + lane;
                vv[j] = p < n ? ref[p] : (T)0;
            }
#pragma unroll
            for (int j = 0; j < 8; j++) {
                int64_t p = start + (it0 + j) * 32 + lane;
                bool inb = p < n;
                T v = vv[j];
                bool hold = !inb || !(v == v);
                bool c = inb && (v <= cmp.h);
                unsigned cm = __ballot_sync(0xffffffffu, c);
                unsigned hm = __ballot_sync(0xffffffffu, hold);
                unsigned e = edge_bits(cm, hm, st);
                if (WRITE && ((e >> lane) & 1u)) {
                    int64_t o = off + __popc(e & ((1u << lane) - 1u));
                    if (o < capacity) events[o] = 2 * p + (c ? 0 : 1);
                }
                int pc = __popc(e);
                off += pc;
                cnt += pc;
            }
        }
    }
    if (WRITE) return;
    finish_counts(cnt, wg, counts, offsets, total, nchunks);
}

// The same two passes over the pulse-scan bits the fused demodulator writes
// (cond: v <= threshold, hold: NaN; 32 stream samples per word, [begin, n)
// word-aligned): a warp's 32 lanes take its 32 words; the state entering each
// word is that of the last non-NaN sample before it (the warp's entering state
// from the words before `start`, walked back like state_before), found with a
// ballot of the words holding a non-NaN sample.
__device__ __forceinline__ bool bits_state_before(const unsigned* cond, const unsigned* hold, int64_t p0) {
    for (int64_t w = (p0 >> 5) - 1; w >= 0; w--) {
        const unsigned h = hold[w];
        if (h != 0xffffffffu) {
            const int b = 31 - __clz(~h);
            return (cond[w] >> b) & 1u;
        }
    }
    return false;
}

template <bool WRITE>
__global__ void __launch_bounds__(kPT) k_pulse_bits(const unsigned* __restrict__ cond,
                                                    const unsigned* __restrict__ hold, int64_t begin, int64_t n,
                                                    int64_t* counts, int64_t* offsets, int64_t* events,
                                                    int64_t capacity, int64_t* total, int64_t nchunks) {
    constexpr int kWarps = kPT / 32;
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const int64_t wg = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t start = begin + wg * kPWarpSamples;
    int64_t cnt = 0;
    if (start < n) {
        unsigned st0 = 0u;
        if (lane == 0) st0 = bits_state_before(cond, hold, start) ? 1u : 0u;
        st0 = __shfl_sync(0xffffffffu, st0, 0);
        const int64_t p0 = start + 32 * lane;   // first sample of this lane's word
        const bool inb = p0 < n;
        const unsigned c = inb ? cond[p0 >> 5] : 0u;
        const unsigned h = inb ? hold[p0 >> 5] : 0xffffffffu;
        const bool has = h != 0xffffffffu;
        const unsigned last = has ? (c >> (31 - __clz(~h))) & 1u : 0u;
        const unsigned hm = __ballot_sync(0xffffffffu, has);
        const unsigned before = hm & ((1u << lane) - 1u);
        const int src = before ? 31 - __clz(before) : 0;
        const unsigned from = __shfl_sync(0xffffffffu, last, src);
        unsigned st = before ? from : st0;
        const unsigned e = edge_bits(c, h, st);
        const int pc = __popc(e);
        int incl = pc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        cnt = __shfl_sync(0xffffffffu, incl, 31);
        if (WRITE) {
            int64_t off = offsets[1 + blockIdx.x];
            for (int k = 0; k < wl; k++) off += counts[(int64_t)blockIdx.x * kWarps + k];
            off += incl - pc;
            unsigned m = e;
            while (m) {
                const int b = __ffs(m) - 1;
                m &= m - 1;
                const int64_t p = p0 + b;
                if (off < capacity) events[off] = 2 * p + (((c >> b) & 1u) ? 0 : 1);
                off++;
            }
        }
    }
    if (WRITE) return;
    finish_counts(cnt, wg, counts, offsets, total, nchunks);
}

}  // namespace

float pulse_float_threshold(double high) { return make_cmp<float>(high).h; }

cudaError_t launch_pulse_bits_range(const unsigned* cond, const unsigned* hold, int64_t begin, int64_t end,
                                    int64_t* counts, int64_t* offsets, int64_t* events, int64_t capacity,
                                    int64_t* total, cudaStream_t s) {
    if ((begin & 31) != 0 || (end & 31) != 0) return cudaErrorInvalidValue;
    int64_t len = end > begin ? end - begin : 0;
    int64_t nchunks = (len + kPulseChunk - 1) / kPulseChunk;
    if (nchunks == 0) {
        cudaMemsetAsync(total, 0, sizeof(int64_t), s);
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(offsets, 0, sizeof(int64_t), s);   // the last-CTA ticket
    if (e != cudaSuccess) return e;
    k_pulse_bits<false><<<(unsigned)nchunks, kPT, 0, s>>>(cond, hold, begin, end, counts, offsets, nullptr, 0,
                                                         total, nchunks);
    k_pulse_bits<true><<<(unsigned)nchunks, kPT, 0, s>>>(cond, hold, begin, end, counts, offsets, events,
                                                        capacity, total, nchunks);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_pulse_events_range(const T* ref, int64_t begin, int64_t end, double high,
                                      int64_t* counts, int64_t* offsets, int64_t* events,
                                      int64_t capacity, int64_t* total, cudaStream_t s) {
    int64_t len = end > begin ? end - begin : 0;
    int64_t nchunks = (len + kPulseChunk - 1) / kPulseChunk;
    if (nchunks == 0) {
        cudaMemsetAsync(total, 0, sizeof(int64_t), s);
        return cudaGetLastError();
    }
    Cmp<T> cmp = make_cmp<T>(high);
    cudaError_t e = cudaMemsetAsync(offsets, 0, sizeof(int64_t), s);   // the last-CTA ticket
    if (e != cudaSuccess) return e;
    k_pulse_pass<T, false><<<(unsigned)nchunks, kPT, 0, s>>>(ref, begin, end, cmp, counts, offsets,
                                                            nullptr, 0, total, nchunks);
    k_pulse_pass<T, true><<<(unsigned)nchunks, kPT, 0, s>>>(ref, begin, end, cmp, counts, offsets,
                                                           events, capacity, total, nchunks);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_pulse_events(const T* ref, int64_t n, double high, int64_t* counts,
                                int64_t* offsets, int64_t* events, int64_t capacity,
                                int64_t* total, cudaStream_t s) {
    return launch_pulse_events_range<T>(ref, 0, n, high, counts, offsets, events, capacity, total, s);
}
template cudaError_t launch_pulse_events<float>(const float*, int64_t, double, int64_t*, int64_t*,
                                                int64_t*, int64_t, int64_t*, cudaStream_t);
template cudaError_t launch_pulse_events<double>(const double*, int64_t, double, int64_t*, int64_t*,
                                                 int64_t*, int64_t, int64_t*, cudaStream_t);
template cudaError_t launch_pulse_events_range<float>(const float*, int64_t, int64_t, double, int64_t*,
                                                      int64_t*, int64_t*, int64_t, int64_t*, cudaStream_t);
template cudaError_t launch_pulse_events_range<double>(const double*, int64_t, int64_t, double, int64_t*,
                                                       int64_t*, int64_t*, int64_t, int64_t*, cudaStream_t);

// ============================================================== hsync refine
// RefineLineLocationsFromHSync, VHS branch with right-edge refinement
// (Core/Decode/TbcFieldDecodePipeline.cs:4570-4679, 4807-5050) and
// PulseDetection.CalculateZeroCrossing (Core/Dsp/PulseDetection.cs:17-40,
// 224-275).  One warp per field; lines are processed in order because the
// back-porch level carries from line to line.
namespace {

__device__ __forceinline__ double round_away(double x) {
    return x >= 0.0 ? floor(x + 0.5) : -floor(-x + 0.5);
}

template <typename T>
struct Span {
    const T* d;
    int64_t n;
    __device__ double at(int64_t i) const { return (double)d[i]; }
};

// Exact sample-vs-threshold tests in the stream's own type.  For a float
// sample v and a double t: v < t <=> v < hi and v > t <=> v > lo, with hi the
// smallest float >= t and lo the largest float <= t (NaN compares false either way).
template <typename T>
struct Thr {
    T lo, hi;
};
__device__ __forceinline__ Thr<double> make_thr(double t, const double*) { return {t, t}; }
__device__ __forceinline__ Thr<float> make_thr(double t, const float*) {
    float f = __double2float_rn(t);
    float lo = f, hi = f;
    if ((double)f > t) lo = nextafterf(f, -INFINITY);
    if ((double)f < t) hi = nextafterf(f, INFINITY);
    return {lo, hi};
}

// first crossing of `target` at/after `start` within count+1 samples; NaN if none
template <typename T>
__device__ int64_t coop_first_crossing(const T* d, int64_t n, int64_t start, Thr<T> th, int edge, int count,
                                       int lane);
template <typename T>
__device__ double zero_crossing(const Span<T>& s, int64_t start, double target, int edge, int count,
                                int lane) {
    const Thr<T> th = make_thr(target, (const T*)nullptr);
    int64_t x = coop_first_crossing(s.d, s.n, start, th, edge, count, lane);
    if (x < 0) return nan("");
    double a = s.at(x - 1) - target;
    double b = s.at(x) - target;
    double y = (b - a) != 0.0 ? -a / (-a + b) : 0.0;
    return (double)(x - 1) + y;
}

template <typename T>
__device__ bool area_ok(const Span<T>& s, double crossing, int one_us, double end_us, double lo_hz,
                        double hi_hz, int lane) {
    int64_t st = (int64_t)round_away(crossing - 0.75 * one_us);
    st = st < 0 ? 0 : (st > s.n ? s.n : st);
    int64_t en = (int64_t)round_away(crossing + end_us * one_us);
    en = en < st ? st : (en > s.n ? s.n : en);
    if (en <= st) return false;
    T mn = (T)INFINITY, mx = (T)-INFINITY;
    for (int64_t i = st + lane; i < en; i += 32) {
        T v = s.d[i];
        mn = fmin(mn, v);
        mx = fmax(mx, v);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    return (double)mn >= lo_hz && (double)mx <= hi_hz;
}

// Lane partial sums: float streams accumulate as float pairs (TwoSum), which
// is exact to about 2^-48 relative; the lanes combine in double.
__device__ __forceinline__ void acc_add(double& acc, float& lo, double v) { acc += v; (void)lo; }
__device__ __forceinline__ void acc_add(float& acc, float& lo, float v) {
    float s = __fadd_rn(acc, v);
    float bb = __fsub_rn(s, acc);
    lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(acc, __fsub_rn(s, bb)), __fsub_rn(v, bb)));
    acc = s;
}

template <typename T>
__device__ bool mean_range(const Span<T>& s, double start, double end, double* mean, int lane) {
    int64_t st = (int64_t)round_away(start);
    st = st < 0 ? 0 : (st > s.n ? s.n : st);
    int64_t en = (int64_t)round_away(end);
    en = en < st ? st : (en > s.n ? s.n : en);
    if (en <= st) { *mean = 0.0; return false; }
    T acc = (T)0;
    float lo = 0.0f;
    for (int64_t i = st + lane; i < en; i += 32) acc_add(acc, lo, s.d[i]);
    double sum = (double)acc + (double)lo;
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    *mean = sum / (double)(en - st);
    return true;
}

// Per-line quantities of the refinement that do not depend on the porch
// level carried between lines (phase 1, one warp per line), the speculative
// midpoint crossing for "carried porch = previous line's right-edge porch"
// (phase 2), and the sequential carry over lines (phase 3, one warp per
// field, which repeats a search only when the speculation missed).
struct LineInfo {
    double loc;      // input location
    double crossing; // threshold crossing from round(loc - 1us), NaN if none
    double sync;     // mean sync level after the crossing
    double own_porch;
    double rc_own;   // midpoint crossing with own porch, NaN if none
    double rc_spec;  // midpoint crossing with the previous line's right porch, NaN if none
    double r_porch;  // right-edge porch level (NaN if the right refinement is invalid)
    double r_cand;   // right-edge candidate location
    int64_t ss;      // search start
    int flags;       // bit0 vsync line, bit1 usable (finite, ss in range), bit2 area+sync ok,
                     // bit3 own porch valid, bit4 right candidate valid, bit5 filled in
    int pre;         // comparisons precomputed for the chain (kPre* bits)
};

// LineInfo::pre bits: the chain's binary64 comparisons that do not depend on
// the carried porch, evaluated lane-parallel by the line and spec kernels.
constexpr int kPreCross = 1;       // crossing is a number
constexpr int kPreOwnOk = 2;       // rc_own is a number and within 1/2 us of the crossing
constexpr int kPreSpecOk = 4;      // rc_spec is a number and within 1/2 us of the crossing
constexpr int kPreNearOwn = 8;     // right candidate within 2 us of rc_own
constexpr int kPreNearSpec = 16;   // ... of rc_spec
constexpr int kPreNearCross = 32;  // ... of the crossing
constexpr int kPreNearLoc = 64;    // ... of the input location
constexpr int kPreOwnPos = 128;    // own porch > 0
constexpr int kPreRPos = 256;      // right porch > 0

// Cooperative warp primitives for the line stage: the warp works on one
// line's samples at a time (parameters broadcast from the line's lane); the
// binary64 arithmetic of all 32 lines then runs lane-parallel, one line per
// lane, so no FP64 instruction is repeated across lanes.

// index of the first crossing of `th` in (start, min(n, start + count + 1)), -1 if none
// (128 samples per step: four chunks of 32 are loaded before any is tested)
template <typename T>
__device__ int64_t coop_first_crossing(const T* d, int64_t n, int64_t start, Thr<T> th, int edge, int count,
                                       int lane) {
    if (edge == 0) edge = d[start] < th.hi ? 1 : -1;
    int64_t end = min(n, start + (int64_t)count + 1);
    int64_t len = end - start;
    for (int64_t base0 = 1; base0 < len; base0 += 128) {
        T bv[4], av[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            int64_t i = base0 + 32 * c + lane;
            bv[c] = i < len ? d[start + i] : (T)0;
            av[c] = (lane == 0 && base0 + 32 * c < len) ? d[start + base0 + 32 * c - 1] : (T)0;
        }
#pragma unroll
        for (int c = 0; c < 4; c++) {
            int64_t base = base0 + 32 * c;
            int64_t i = base + lane;
            T b = bv[c];
            T a = __shfl_up_sync(0xffffffffu, b, 1);
            if (lane == 0) a = av[c];
            bool hit = false;
            if (i < len) hit = edge == 1 ? (a < th.hi && b >= th.hi) : (a > th.lo && b <= th.lo);
            unsigned m = __ballot_sync(0xffffffffu, hit);
            if (m) return start + base + (__ffs(m) - 1);
        }
    }
    return -1;
}

// PulseDetection.CalculateZeroCrossing's interpolation at a found crossing x
template <typename T>
__device__ __forceinline__ double crossing_at(const T* d, int64_t x, double target) {
    double a = (double)d[x - 1] - target;
    double b = (double)d[x] - target;
    double y = (b - a) != 0.0 ? -a / (-a + b) : 0.0;
    return (double)(x - 1) + y;
}

template <typename T>
__device__ void coop_minmax(const T* d, int64_t st, int64_t en, T& mn, T& mx, int lane) {
    mn = (T)INFINITY;
    mx = (T)-INFINITY;
    for (int64_t i = st + lane; i < en; i += 32) {
        T v = d[i];
        mn = fmin(mn, v);
        mx = fmax(mx, v);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
}

__device__ __forceinline__ void pair_add(float& hi, float& lo, float oh, float ol) {
    float s = __fadd_rn(hi, oh);
    float bb = __fsub_rn(s, hi);
    float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(oh, bb));
    e = __fadd_rn(e, __fadd_rn(lo, ol));
    hi = __fadd_rn(s, e);
    lo = __fsub_rn(e, __fsub_rn(hi, s));
}
__device__ __forceinline__ double coop_total(const float* d, int64_t st, int64_t en, int lane) {
    float hi = 0.0f, lo = 0.0f;
    for (int64_t i = st + lane; i < en; i += 32) pair_add(hi, lo, d[i], 0.0f);
    for (int o = 16; o > 0; o >>= 1)
        pair_add(hi, lo, __shfl_xor_sync(0xffffffffu, hi, o), __shfl_xor_sync(0xffffffffu, lo, o));
    return (double)hi + (double)lo;
}
__device__ __forceinline__ double coop_total(const double* d, int64_t st, int64_t en, int lane) {
    double acc = 0.0;
    for (int64_t i = st + lane; i < en; i += 32) acc += d[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}

// [round(start), round(end)) clipped to [0, n]
__device__ __forceinline__ void range_of(double start, double end, int64_t n, int64_t& st, int64_t& en) {
    st = (int64_t)round_away(start);
    st = st < 0 ? 0 : (st > n ? n : st);
    en = (int64_t)round_away(end);
    en = en < st ? st : (en > n ? n : en);
}

// Per-line state of the line stage, shared between the line's search warp
// and the lane of warp 0 that does the line's binary64 arithmetic.
struct LineWork {
    int64_t s0, n, ss, rs;
    int64_t x[4];            // crossings found: threshold, own midpoint, right edge, right midpoint
    int64_t r[12];           // ranges: area, sync, porch (left); area, sync, porch (right)
    double sum[4];           // left sync, left porch, right sync, right porch
    float mn[2], mx[2];      // area extrema (left, right), float streams
    double mnd[2], mxd[2];   // area extrema, double streams
    float tlo[2], thi[2];    // midpoint thresholds (own, right), float form
    double tlod[2], thid[2];
    int cnt[4];
    int want;                // bit k: search / reduction k requested
};

template <typename T>
__device__ __forceinline__ void store_extrema(LineWork& w, int k, T mn, T mx);
template <>
__device__ __forceinline__ void store_extrema<float>(LineWork& w, int k, float mn, float mx) { w.mn[k] = mn; w.mx[k] = mx; }
template <>
__device__ __forceinline__ void store_extrema<double>(LineWork& w, int k, double mn, double mx) { w.mnd[k] = mn; w.mxd[k] = mx; }
__device__ __forceinline__ double ext_min(const LineWork& w, int k, const float*) { return (double)w.mn[k]; }
__device__ __forceinline__ double ext_max(const LineWork& w, int k, const float*) { return (double)w.mx[k]; }
__device__ __forceinline__ double ext_min(const LineWork& w, int k, const double*) { return w.mnd[k]; }
__device__ __forceinline__ double ext_max(const LineWork& w, int k, const double*) { return w.mxd[k]; }
__device__ __forceinline__ void store_thr(LineWork& w, int k, Thr<float> t) { w.tlo[k] = t.lo; w.thi[k] = t.hi; }
__device__ __forceinline__ void store_thr(LineWork& w, int k, Thr<double> t) { w.tlod[k] = t.lo; w.thid[k] = t.hi; }
__device__ __forceinline__ Thr<float> load_thr(const LineWork& w, int k, const float*) { return {w.tlo[k], w.thi[k]}; }
__device__ __forceinline__ Thr<double> load_thr(const LineWork& w, int k, const double*) { return {w.tlod[k], w.thid[k]}; }

// kHsyncLines lines per CTA, one warp each: warp w runs the sample searches
// and reductions of line w (the lines proceed concurrently); lanes
// 0..kHsyncLines-1 of warp 0 run the binary64 arithmetic of the CTA's lines
// lane-parallel between the phases.  16 lines per CTA keep four CTAs per SM,
// so one CTA's searches overlap another's binary64 steps.
// Per line: threshold crossing from round(loc - 1 us), area and level checks,
// own-porch midpoint crossing, and the right-edge candidate -- the per-line
// part of RefineLineLocationsFromHSync.
constexpr int kHsyncLines = 16;

template <typename T>
__global__ void __launch_bounds__(32 * kHsyncLines) k_hsync_lines(const T* stream, int64_t stream_len,
                                                                  HsyncParams p, LineInfo* info) {
    __shared__ LineWork lw[32];   // entries kHsyncLines.. are written by idle lanes of warp 0 only
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t total = (int64_t)p.nfields * p.lines;
    const int one = p.one_us, normal = p.normal_hsync;
    const int search = one * 2 > 1 ? one * 2 : 1;
    auto ire_hz = [&](double ire) { return p.ire0 + p.hz_ire * ire; };
    const Thr<T> th0 = make_thr(p.threshold, (const T*)nullptr);
    // warp 0, lane l <-> line g = kHsyncLines blockIdx + l
    const int64_t g = (int64_t)blockIdx.x * kHsyncLines + lane;
    const bool have = lane < kHsyncLines && g < total;
    LineInfo li;
    double crossing = NAN, rcx = NAN, target_own = 0.0, target_r = 0.0, r_porch = 0.0;
    int flags = 0;
    bool usable = false;
    if (warp == 0) {
        const int f = have ? (int)(g / p.lines) : 0;
        const int line = have ? (int)(g % p.lines) : 0;
        const int64_t s0 = have ? p.span_start[f] : 0;
        const int64_t n = have ? min(p.span_len[f], stream_len - s0) : 0;
        const double loc = have ? p.locs_in[g] : (double)NAN;
        li.loc = loc;
        li.crossing = li.sync = li.own_porch = li.rc_own = li.rc_spec = li.r_porch = li.r_cand = nan("");
        li.ss = 0;
        li.pre = 0;
        flags = (have && p.filled_in[g]) ? 32 : 0;
        const bool vsync_line = (line >= 3 && line <= 6) || (p.pal && line >= 1 && line <= 2);
        if (vsync_line) flags |= 1;
        const int64_t ss = isfinite(loc) ? (int64_t)round_away(loc - one) : -1;
        usable = have && !vsync_line && isfinite(loc) && ss >= 0 && ss < n - 1;
        LineWork& w = lw[lane];
        w.s0 = s0; w.n = n; w.ss = ss; w.want = 0;
        w.x[0] = w.x[1] = w.x[2] = w.x[3] = -1;
        if (usable) {
            flags |= 2;
            li.ss = ss;
            w.cnt[0] = (int)min((int64_t)search, n - ss - 1);
            w.want |= 1;
            const int64_t rs = ss + normal - one;
            w.rs = rs;
            if (rs >= 0 && rs < n - 1 && !((double)stream[s0 + rs] > p.threshold)) {
                w.cnt[2] = (int)min((int64_t)max(1, normal * 2), n - rs - 1);
                w.want |= 4;
            }
        }
    }
    __syncthreads();
    // phase A: threshold crossings (left, from ss; right edge, rising, from rs)
    {
        const LineWork& w = lw[warp];
        const T* d = stream + w.s0;
        if (w.want & 1) {
            int64_t r = coop_first_crossing(d, w.n, w.ss, th0, 0, w.cnt[0], lane);
            if (lane == 0) lw[warp].x[0] = r;
        }
        if (w.want & 4) {
            int64_t r = coop_first_crossing(d, w.n, w.rs, th0, 1, w.cnt[2], lane);
            if (lane == 0) lw[warp].x[2] = r;
        }
    }
    __syncthreads();
    // warp 0: interpolate, derive the level ranges
    if (warp == 0) {
        LineWork& w = lw[lane];
        const T* d = stream + w.s0;
        w.want &= ~(1 | 4);
        if (usable) {
            crossing = w.x[0] >= 0 ? crossing_at(d, w.x[0], p.threshold) : (double)NAN;
            li.crossing = crossing;
            if (crossing == crossing) {
                range_of(crossing - 0.75 * one, crossing + 3.5 * one, w.n, w.r[0], w.r[1]);
                range_of(crossing + one, crossing + 2.5 * one, w.n, w.r[2], w.r[3]);
                range_of(crossing - one, crossing - 0.5 * one, w.n, w.r[4], w.r[5]);
                w.want |= 16;
            }
            rcx = w.x[2] >= 0 ? crossing_at(d, w.x[2], p.threshold) : (double)NAN;
            if (rcx == rcx) {
                const double derived = rcx - normal;
                range_of(derived - 0.75 * one, derived + 8.0 * one, w.n, w.r[6], w.r[7]);
                range_of(derived + one, derived + 2.5 * one, w.n, w.r[8], w.r[9]);
                range_of(derived + normal + one, derived + normal + 2.0 * one, w.n, w.r[10], w.r[11]);
                w.want |= 32;
            }
        }
    }
    __syncthreads();
    // phase B: area extrema and level sums
    {
        const LineWork& w = lw[warp];
        const T* d = stream + w.s0;
        for (int side = 0; side < 2; side++) {
            if (!(w.want & (16 << side))) continue;
            const int64_t* r = w.r + 6 * side;
            T mn, mx;
            coop_minmax(d, r[0], r[1], mn, mx, lane);
            double s1 = coop_total(d, r[2], r[3], lane);
            double s2 = coop_total(d, r[4], r[5], lane);
            if (lane == 0) {
                store_extrema<T>(lw[warp], side, mn, mx);
                lw[warp].sum[2 * side] = s1;
                lw[warp].sum[2 * side + 1] = s2;
            }
        }
    }
    __syncthreads();
    // warp 0: level checks, midpoint thresholds
    if (warp == 0) {
        LineWork& w = lw[lane];
        const T* tp = nullptr;
        if (w.want & 16) {
            if (w.r[1] > w.r[0] && ext_min(w, 0, tp) >= ire_hz(-65.0) && ext_max(w, 0, tp) <= ire_hz(110.0) &&
                w.r[3] > w.r[2]) {
                const double sync_lv = w.sum[0] / (double)(w.r[3] - w.r[2]);
                flags |= 4;
                li.sync = sync_lv;
                if (w.r[5] > w.r[4]) {
                    const double porch = w.sum[1] / (double)(w.r[5] - w.r[4]);
                    flags |= 8;
                    li.own_porch = porch;
                    target_own = (porch + sync_lv) / 2.0;
                    store_thr(w, 0, make_thr(target_own, tp));
                    w.cnt[1] = (int)min((int64_t)400, w.n - w.ss - 1);
                    w.want |= 2;
                }
            }
        }
        if (w.want & 32) {
            if (w.r[7] > w.r[6] && ext_min(w, 1, tp) >= ire_hz(-65.0) && ext_max(w, 1, tp) <= ire_hz(30.0) &&
                w.r[9] > w.r[8] && w.r[11] > w.r[10]) {
                const double r_sync = w.sum[2] / (double)(w.r[9] - w.r[8]);
                r_porch = w.sum[3] / (double)(w.r[11] - w.r[10]);
                target_r = (r_porch + r_sync) / 2.0;
                store_thr(w, 1, make_thr(target_r, tp));
                w.cnt[3] = (int)min((int64_t)400, w.n - w.rs - 1);
                w.want |= 8;
            }
        }
    }
    __syncthreads();
    // phase C: midpoint crossings (own porch from ss; right edge from rs)
    {
        const LineWork& w = lw[warp];
        const T* d = stream + w.s0;
        if (w.want & 2) {
            int64_t r = coop_first_crossing(d, w.n, w.ss, load_thr(w, 0, (const T*)nullptr), 0, w.cnt[1], lane);
            if (lane == 0) lw[warp].x[1] = r;
        }
        if (w.want & 8) {
            int64_t r = coop_first_crossing(d, w.n, w.rs, load_thr(w, 1, (const T*)nullptr), 0, w.cnt[3], lane);
            if (lane == 0) lw[warp].x[3] = r;
        }
    }
    __syncthreads();
    if (warp == 0) {
        const LineWork& w = lw[lane];
        const T* d = stream + w.s0;
        if (w.want & 2) li.rc_own = w.x[1] >= 0 ? crossing_at(d, w.x[1], target_own) : (double)NAN;
        if (w.want & 8) {
            const double rr = w.x[3] >= 0 ? crossing_at(d, w.x[3], target_r) : (double)NAN;
            if (rr == rr && fabs(rr - rcx) < one / 2.0) {
                flags |= 16;
                li.r_porch = r_porch;
                li.r_cand = rcx - normal + 2.25 * (p.mhz32 / 40.0);
            }
        }
        li.flags = flags;
        int pre = 0;
        const double half = one / 2.0, two = one * 2.0;
        if (li.crossing == li.crossing) pre |= kPreCross;
        if (li.rc_own == li.rc_own && fabs(li.rc_own - li.crossing) < half) pre |= kPreOwnOk;
        if (li.own_porch > 0.0) pre |= kPreOwnPos;
        if (flags & 16) {
            if (fabs(li.r_cand - li.rc_own) < two) pre |= kPreNearOwn;
            if (fabs(li.r_cand - li.crossing) < two) pre |= kPreNearCross;
            if (fabs(li.r_cand - li.loc) < two) pre |= kPreNearLoc;
            if (li.r_porch > 0.0) pre |= kPreRPos;
        }
        li.pre = pre;
        if (have) info[g] = li;
    }
}

// Speculative midpoint crossing for "carried porch = previous line's
// right-edge porch": 32 lines per CTA, warp w searches line w.
template <typename T>
__global__ void __launch_bounds__(1024) k_hsync_spec(const T* stream, int64_t stream_len, HsyncParams p,
                                                     LineInfo* info) {
    __shared__ LineWork lw[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t total = (int64_t)p.nfields * p.lines;
    const int64_t g = (int64_t)blockIdx.x * 32 + lane;
    double target = 0.0;
    if (warp == 0) {
        LineWork& w = lw[lane];
        w.want = 0;
        w.x[0] = -1;
        const bool have = g < total;
        const int f = have ? (int)(g / p.lines) : 0;
        const int line = have ? (int)(g % p.lines) : 0;
        w.s0 = have ? p.span_start[f] : 0;
        w.n = have ? min(p.span_len[f], stream_len - w.s0) : 0;
        if (have && line > 0) {
            const LineInfo& li = info[g];
            const LineInfo& prev = info[g - 1];
            if ((li.flags & 4) && (prev.flags & 16) && prev.r_porch > 0.0) {
                target = (prev.r_porch + li.sync) / 2.0;
                w.ss = li.ss;
                store_thr(w, 0, make_thr(target, (const T*)nullptr));
                w.cnt[0] = (int)min((int64_t)400, w.n - w.ss - 1);
                w.want = 1;
            }
        }
    }
    __syncthreads();
    {
        const LineWork& w = lw[warp];
        if (w.want) {
            int64_t r = coop_first_crossing(stream + w.s0, w.n, w.ss, load_thr(w, 0, (const T*)nullptr), 0,
                                            w.cnt[0], lane);
            if (lane == 0) lw[warp].x[0] = r;
        }
    }
    __syncthreads();
    if (warp == 0 && lw[lane].want) {
        const LineWork& w = lw[lane];
        LineInfo& li = info[g];
        const double rc = w.x[0] >= 0 ? crossing_at(stream + w.s0, w.x[0], target) : (double)NAN;
        li.rc_spec = rc;
        int pre = li.pre;
        const int one = p.one_us;
        if (rc == rc && fabs(rc - li.crossing) < one / 2.0) pre |= kPreSpecOk;
        if ((li.flags & 16) && fabs(li.r_cand - rc) < one * 2.0) pre |= kPreNearSpec;
        li.pre = pre;
    }
}

// Carried state of the chain: the porch level carried from line to line
// (RefineLineLocationsFromHSync's previous porch), whether it is set, and the
// bits of the previous line's right porch (-1 when none).
struct ChainState {
    double pp;
    long long prev_r_bits;
    int pp_set;
    int miss;
};

__device__ __forceinline__ bool same_state(const ChainState& a, const ChainState& b) {
    return __double_as_longlong(a.pp) == __double_as_longlong(b.pp) && a.pp_set == b.pp_set &&
           a.prev_r_bits == b.prev_r_bits;
}

// One line of the carry walk (called by all 32 lanes of a warp: a porch miss
// runs a cooperative crossing search).  Every comparison that does not involve
// the carried porch level was precomputed (LineInfo::pre); the carried level
// enters only through "is it bit-identical to the previous line's right porch"
// (then the speculative crossing rc_spec applies) and, on a miss, a new
// midpoint search.  The carried level is positive once set, so its "> 0" test
// is a flag.
template <typename T>
__device__ __forceinline__ void chain_step(const LineInfo& li, ChainState& cs, const Span<T>& sp, int one,
                                           int lane, double& out, uint8_t& fo_out) {
    enum { kRefLoc, kRefCross, kRefOwn, kRefSpec, kRefMiss };
    const int flags = li.flags, pre = li.pre;
    out = li.loc;
    uint8_t fo = (flags & 32) ? 1 : 0;
    const bool filled = (flags & 32) != 0;
    if (flags & 1) {
        fo = 1;
    } else if (flags & 2) {
        int ref = kRefLoc;
        double refined = li.loc, rc_miss = 0.0;
        if ((pre & kPreCross) && !filled) {
            bool ok = false, preserve = false, porch_pos = false;
            double porch = 0.0;
            int kind = kRefLoc;
            if (flags & 4) {
                preserve = true;
                if (cs.pp_set) {
                    porch = cs.pp;
                    porch_pos = true;
                    if (__double_as_longlong(cs.pp) == cs.prev_r_bits) {
                        ok = (pre & kPreSpecOk) != 0;
                        kind = kRefSpec;
                    } else {
                        cs.miss++;
                        int c2 = (int)min((int64_t)400, sp.n - li.ss - 1);
                        rc_miss = zero_crossing(sp, li.ss, (cs.pp + li.sync) / 2.0, 0, c2, lane);
                        ok = rc_miss == rc_miss && fabs(rc_miss - li.crossing) < one / 2.0;
                        kind = kRefMiss;
                    }
                } else if (flags & 8) {
                    porch = li.own_porch;
                    porch_pos = (pre & kPreOwnPos) != 0;
                    ok = (pre & kPreOwnOk) != 0;
                    kind = kRefOwn;
                }
            }
            if (ok) {
                refined = kind == kRefSpec ? li.rc_spec : (kind == kRefOwn ? li.rc_own : rc_miss);
                ref = kind;
                fo = filled ? 1 : 0;
                if (porch_pos) { cs.pp = porch; cs.pp_set = 1; }
            } else {
                fo = 1;
                if (preserve) ref = kRefCross;
            }
        } else {
            fo = 1;
        }
        if (flags & 16) {
            bool near;
            switch (ref) {
                case kRefCross: near = (pre & kPreNearCross) != 0; break;
                case kRefOwn: near = (pre & kPreNearOwn) != 0; break;
                case kRefSpec: near = (pre & kPreNearSpec) != 0; break;
                case kRefMiss: near = fabs(li.r_cand - rc_miss) < one * 2.0; break;
                default: near = (pre & kPreNearLoc) != 0; break;
            }
            if (near) {
                refined = li.r_cand;
                fo = 0;
                if (pre & kPreRPos) { cs.pp = li.r_porch; cs.pp_set = 1; }
            }
        }
        out = refined;
    }
    cs.prev_r_bits = (flags & 16) && li.r_porch == li.r_porch ? __double_as_longlong(li.r_porch) : -1;
    fo_out = fo;
}

// The walk over a field's lines, split into kChainWarps segments walked at
// once, one warp each.  A segment's entering state is guessed by walking the
// kChainWarm lines before it from the initial state (a right-edge refinement
// resets the carried state, so the guess is almost always exact); afterwards
// warp 0 compares each guess with the state the previous segment actually
// left and re-walks the segments whose guess differed, in order.  The result
// is the sequential walk's, bit for bit.
constexpr int kChainWarps = 16;
constexpr int kChainWarm = 12;

template <typename T>
__global__ void __launch_bounds__(32 * kChainWarps) k_hsync_chain(const T* stream, int64_t stream_len,
                                                                   HsyncParams p, const LineInfo* info,
                                                                   int* misses) {
    const int f = blockIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t s0 = p.span_start[f];
    Span<T> sp{stream + s0, min(p.span_len[f], stream_len - s0)};
    extern __shared__ __align__(16) unsigned char chain_smem[];
    LineInfo* fi = reinterpret_cast<LineInfo*>(chain_smem);
    __shared__ ChainState entry[kChainWarps], leave[kChainWarps];
    {
        const int4* g = reinterpret_cast<const int4*>(info + (int64_t)f * p.lines);
        int4* d = reinterpret_cast<int4*>(fi);
        const int words = (int)(p.lines * sizeof(LineInfo) / sizeof(int4));
        for (int i = threadIdx.x; i < words; i += blockDim.x) d[i] = g[i];
    }
    __syncthreads();
    const int one = p.one_us;
    const int seg = (p.lines + kChainWarps - 1) / kChainWarps;
    double* locs = p.locs_out + (int64_t)f * p.lines;
    uint8_t* filled = p.filled_out + (int64_t)f * p.lines;
    auto walk = [&](ChainState& cs, int l0, int l1) {
        for (int line = l0; line < l1; line++) {
            double out;
            uint8_t fo;
            chain_step(fi[line], cs, sp, one, lane, out, fo);
            if (lane == 0) {
                locs[line] = out - p.ntsc_shift;
                filled[line] = fo;
            }
        }
    };
    const int l0 = min(w * seg, p.lines), l1 = min(l0 + seg, p.lines);
    ChainState cs{-1.0, -1, 0, 0};
    for (int line = max(0, l0 - kChainWarm); line < l0; line++) {
        double out;
        uint8_t fo;
        chain_step(fi[line], cs, sp, one, lane, out, fo);
    }
    cs.miss = 0;
    if (lane == 0) entry[w] = cs;
    walk(cs, l0, l1);
    if (lane == 0) leave[w] = cs;
    __syncthreads();
    if (w != 0) return;
    ChainState prev = leave[0];
    int total = prev.miss;
    for (int k = 1; k < kChainWarps; k++) {
        const int a = min(k * seg, p.lines), b = min(a + seg, p.lines);
        if (same_state(entry[k], prev)) {
            prev = leave[k];
        } else {
            ChainState c = prev;
            c.miss = 0;
            walk(c, a, b);
            prev = c;
        }
        total += prev.miss;
    }
    if (lane == 0 && misses) atomicAdd(misses, total);
}
}  // namespace

template <typename T>
cudaError_t launch_hsync_refine(const T* stream, int64_t stream_len, const HsyncParams& p,
                                cudaStream_t s) {
    if (p.nfields <= 0) return cudaSuccess;
    const int64_t lines = (int64_t)p.nfields * p.lines;   // 32 lines per CTA of 32 warps
    const int threads = 1024;
    const unsigned blocks = (unsigned)((lines + 31) / 32);
    LineInfo* info = reinterpret_cast<LineInfo*>(p.work);
    k_hsync_lines<T><<<(unsigned)((lines + kHsyncLines - 1) / kHsyncLines), 32 * kHsyncLines, 0, s>>>(
        stream, stream_len, p, info);
    k_hsync_spec<T><<<blocks, threads, 0, s>>>(stream, stream_len, p, info);
    k_hsync_chain<T><<<p.nfields, 32 * kChainWarps, p.lines * sizeof(LineInfo), s>>>(stream, stream_len, p,
                                                                                     info, p.misses);
    return cudaGetLastError();
}
size_t hsync_work_bytes(int nfields, int lines) { return (size_t)nfields * lines * sizeof(LineInfo); }
template cudaError_t launch_hsync_refine<float>(const float*, int64_t, const HsyncParams&, cudaStream_t);
template cudaError_t launch_hsync_refine<double>(const double*, int64_t, const HsyncParams&, cudaStream_t);

// ============================================================== TBC
// TbcLineResampler linear plan (Core/Tbc/TbcLineResampler.cs:732-805,
// 818-878, 997-1011, 1480-1532), SampleSinc (:1167-1234) and
// VideoOutputConverter.FastMathConversion (Core/Tbc/VideoOutputConverter.cs:9-40).
namespace {

// Per field: line factors, median / MAD outlier replacement, smoothing chain.
// level_work per field: [2 * maxl] = (adjusted factor, value before the line)
// Order-preserving int64 keys of doubles (ascending key = ascending value for
// non-NaN values; -0 sorts before +0), so the median sorts compare on the
// integer ALU instead of GB300's narrow FP64 pipe.
__device__ __forceinline__ long long dkey(double v) {
    const long long b = __double_as_longlong(v);
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double dval(long long k) {
    return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffLL));
}

// Bitonic sort of 512 entries: int64 keys, or (kDouble) raw double bits
// compared as doubles, the form that keeps NaN's no-swap behaviour.  Two
// instantiations, so the integer form issues no binary64 compare at all.
template <bool kDouble>
__device__ __forceinline__ void bitonic512_t(long long* a) {
    for (int k = 2; k <= 512; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < 512; i += blockDim.x) {
                int ixj = i ^ j;
                if (ixj > i) {
                    bool up = (i & k) == 0;
                    long long x = a[i], y = a[ixj];
                    bool gt = kDouble ? (__longlong_as_double(x) > __longlong_as_double(y)) : (x > y);
                    if (gt == up) { a[i] = y; a[ixj] = x; }
                }
            }
            __syncthreads();
        }
    }
}
__device__ __forceinline__ void bitonic512(long long* a, bool as_double) {
    if (as_double) bitonic512_t<true>(a);
    else bitonic512_t<false>(a);
}

__global__ void __launch_bounds__(512) k_tbc_levels(TbcParams p, const double* pw_outlen) {
    __shared__ double fac[512];
    __shared__ long long srt[512];
    const int f = blockIdx.x;
    const int fl = p.first_line[f];
    const int nl = fl + p.out_lines;          // lines covered by the plan incl. prefix
    const double* loc = p.locs + (int64_t)f * p.lines;
    // one binary64 division per CTA: an FP64 warp instruction costs the SM's
    // FP64 pipe the same whatever its active lanes
    __shared__ double inv_s;
    if (threadIdx.x == 0) inv_s = 1.0 / p.nominal;
    __syncthreads();
    const double inv = inv_s;
    int nan_here = 0;
    for (int l = threadIdx.x; l < 512; l += blockDim.x) {
        double v = INFINITY;
        if (l < nl) {
            int left = l < p.lines - 2 ? l : p.lines - 2;
            v = __dsub_rn(__dmul_rn(loc[left + 1], inv), __dmul_rn(loc[left], inv));
        }
        fac[l] = v;
        nan_here |= v != v;
    }
    // a NaN factor keeps the double comparisons (and their NaN behaviour)
    const bool as_double = __syncthreads_or(nan_here) != 0;
    auto enc = [&](double v) { return as_double ? __double_as_longlong(v) : dkey(v); };
    auto dec = [&](long long k) { return as_double ? __longlong_as_double(k) : dval(k); };
    for (int l = threadIdx.x; l < 512; l += blockDim.x) srt[l] = enc(fac[l]);
    __syncthreads();
    bitonic512(srt, as_double);
    __shared__ double med_s, mad_s;
    if (threadIdx.x == 0) {
        med_s = (nl & 1) ? dec(srt[nl / 2]) : (dec(srt[nl / 2 - 1]) + dec(srt[nl / 2])) / 2.0;
    }
    __syncthreads();
    double med = med_s;
    for (int l = threadIdx.x; l < 512; l += blockDim.x) srt[l] = enc(l < nl ? fabs(fac[l] - med) : INFINITY);
    __syncthreads();
    bitonic512(srt, as_double);
    if (threadIdx.x == 0) {
        mad_s = (nl & 1) ? dec(srt[nl / 2]) : (dec(srt[nl / 2 - 1]) + dec(srt[nl / 2])) / 2.0;
    }
    __syncthreads();
    double mad = mad_s;
    double thr = mad > 0.0 ? 15.0 * mad : 0.001;
    for (int l = threadIdx.x; l < nl; l += blockDim.x) {
        double v = fac[l];
        fac[l] = fabs(v - med) > thr ? med : v;
    }
    __syncthreads();
    // Line-rate smoothing chain: prev_0 = a_0, prev_l = a_l + rN (prev_{l-1} - a_l)
    // (rN = (1 - alpha)^outlen, the per-sample chain of the reference over one
    // line in closed form, like the per-sample levels in the TBC kernels), as an
    // inclusive scan of the affine maps x -> rN x + (1 - rN) a_l: 9 dependent
    // steps instead of one binary64 chain through every line (a few ulps of
    // double from the sequential order, far below the float rounding of the
    // levels' use).  One thread per line slot (512 threads).
    __shared__ double sm_m[512], sm_c[512];
    const bool smooth = p.smoothing > 0.0;
    const double rN = pw_outlen ? pw_outlen[p.outlen - 1] : 1.0;   // (1-alpha)^outlen
    const int l = threadIdx.x;
    double m = 1.0, c = 0.0;                                        // identity at l = 0 and past nl
    if (l >= 1 && l < nl) { m = rN; c = __dmul_rn(__dsub_rn(1.0, rN), fac[l]); }
    sm_m[l] = m;
    sm_c[l] = c;
    __syncthreads();
    // only the slots of lines take part (the maps past nl are never read)
    for (int d = 1; d < 512; d <<= 1) {
        double pm = 1.0, pc = 0.0;
        if (l >= d && l < nl) { pm = sm_m[l - d]; pc = sm_c[l - d]; }
        __syncthreads();
        if (l >= d && l < nl) {
            c = __fma_rn(m, pc, c);
            m = __dmul_rn(m, pm);
            sm_m[l] = m;
            sm_c[l] = c;
        }
        __syncthreads();
    }
    // prev_l = m_l a_0 + c_l (the composition of the maps 1..l applied to a_0)
    if (l < nl) {
        double* w = p.level_work + (int64_t)f * 1024;
        const double a0 = fac[0];
        double before;
        if (l == 0) before = a0;
        else if (!smooth) before = fac[l - 1];
        else before = l == 1 ? a0 : __fma_rn(sm_m[l - 1], a0, sm_c[l - 1]);
        w[2 * l] = fac[l];
        w[2 * l + 1] = before;
    }
}

__device__ __forceinline__ int wrap_idx(int i, int len) {
    if (i < 0) i += len;
    return i < 0 ? 0 : (i > len - 1 ? len - 1 : i);
}

template <typename T>
__device__ __forceinline__ double sample_sinc(const T* src, int64_t n, double position, const float* lut) {
    if (!isfinite(position)) return 0.0;
    const int taps = 16, phases = 65536;
    float coord = __double2float_rn(position);
    int ci = (int)coord;
    float fraction = __fsub_rn(coord, (float)ci);
    float pp = __fmul_rn(fraction, (float)phases);
    int ps = (int)pp;
    int pe = ps + 1;
    float alpha = __fsub_rn(pp, (float)ps);
    ps = wrap_idx(ps, phases + 1);
    pe = wrap_idx(pe, phases + 1);
    const float* ws = lut + (int64_t)ps * taps;
    const float* we = lut + (int64_t)pe * taps;
    int start = ci - (taps / 2 - 1);
    bool interior = n >= taps && (uint32_t)start <= (uint32_t)(n - taps);
    double r = 0.0;
#pragma unroll
    for (int t = 0; t < taps; t++) {
        float sw = __ldg(ws + t);
        float w = __fmaf_rn(alpha, __fsub_rn(__ldg(we + t), sw), sw);
        int64_t idx = (int64_t)start + t;
        if (!interior) {
            if (idx < 0) idx += n;
            idx = idx < 0 ? 0 : (idx > n - 1 ? n - 1 : idx);
        }
        float prod = __fmul_rn((float)src[idx], w);
        r = __dadd_rn((double)prod, r);
    }
    return r;
}

template <typename T>
__global__ void k_tbc(const T* stream, int64_t stream_len, TbcParams p, const double* pw) {
    const int f = blockIdx.y;
    const int ol = blockIdx.x;
    const int fl = p.first_line[f];
    const int line = fl + ol;
    const double* loc = p.locs + (int64_t)f * p.lines;
    const int64_t s0 = p.span_start[f];
    const int64_t n = min(p.span_len[f], stream_len - s0);
    const T* src = stream + s0;
    const double nominal = p.nominal;
    const double out_scale = __ddiv_rn(nominal, (double)p.outlen);
    const double* w = p.level_work + (int64_t)f * 1024;
    const double adj = w[2 * line], before = w[2 * line + 1];
    const double ll = loc[line];
    const double delta = __dsub_rn(loc[line + 1], ll);
    const int kx1 = p.x1 > 0 ? p.x1 : p.outlen;
    for (int k = p.x0 + threadIdx.x; k < kx1; k += blockDim.x) {
        int64_t idx = (int64_t)line * p.outlen + k;
        double scaled = __dmul_rn((double)idx, out_scale);
        double frac = __ddiv_rn(__dsub_rn(scaled, __dmul_rn((double)line, nominal)), nominal);
        frac = frac < 0.0 ? 0.0 : (frac > 1.0 ? 1.0 : frac);
        double pos = __dadd_rn(ll, __dmul_rn(delta, frac));
        double la = adj;
        if (p.smoothing > 0.0 && line > 0) la = adj + pw[k] * (before - adj);
        double v = sample_sinc(src, n, pos, p.lut);
        double outv = (double)__double2float_rn(__dmul_rn(v, la));
        int64_t o = ((int64_t)f * p.out_lines + ol) * p.outlen + k;
        if (p.out_hz) p.out_hz[o] = outv;
        if (p.out_f32) p.out_f32[((int64_t)f * p.out_lines + ol) * p.out_stride + (k - p.x0)] = (float)outv;
        if (p.out_u16) {
            double sd = __dmul_rn(p.output_scale, __dsub_rn(outv, p.ire0));
            double val = __fma_rn(sd, p.inv_hz_ire, p.offset);
            uint16_t u = val <= 0.0 ? 0 : (val >= 65535.0 ? 65535 : (uint16_t)val);
            p.out_u16[o] = u;
        }
    }
}
// Float-only rendering of a float stream to uint16.  Every quantity the
// reference keeps in binary64 is carried as an unevaluated float pair
// (hi + lo, about 48 significant bits): the line's linear position plan
// pos(k) = A + k B, the smoothed level factor, the sum of the 16 float
// products (TwoSum) and the uint16 conversion, whose floor is taken on the
// exact pair.  Results equal the binary64 ones except where a value lies
// within about 2^-46 (relative) of a float rounding boundary or of an integer.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void quick_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}
__device__ __forceinline__ float2 split_double(double d) {
    float hi = __double2float_rn(d);
    return make_float2(hi, __double2float_rn(d - (double)hi));
}
// (ah + al) * (bh + bl) as a pair
__device__ __forceinline__ float2 ff_mul(float ah, float al, float bh, float bl) {
    float m = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -m);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    float s, t;
    quick_two_sum(m, e, s, t);
    return make_float2(s, t);
}
// (ah + al) + (bh + bl) as a pair
__device__ __forceinline__ float2 ff_add(float ah, float al, float bh, float bl) {
    float s, e;
    two_sum(ah, bh, s, e);
    e = __fadd_rn(e, __fadd_rn(al, bl));
    float h, t;
    quick_two_sum(s, e, h, t);
    return make_float2(h, t);
}

struct TbcLineConsts {
    float2 a, b;        // position plan A, B
    float2 adj, dlev;   // level factor and (value before the line - factor)
    float2 ire0, k;     // conversion: (outf - ire0) * k + off
    float2 off;
    int smooth;
};

static_assert(sizeof(TbcLineConsts) <= kTbcLineConstsBytes, "line constants slot");

// The binary64 per-line plan of k_tbc_fast, one thread per output line of
// every field (lane-parallel, so no CTA of the sinc kernel waits on a serial
// FP64 preamble): position plan a + b k (TbcLineResampler's linear plan),
// the line's level factor and the uint16 conversion, each split to a float pair.
__global__ void k_tbc_consts(TbcParams p) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)p.nfields * p.out_lines) return;
    const int f = (int)(t / p.out_lines);
    const int ol = (int)(t - (int64_t)f * p.out_lines);
    const int line = p.first_line[f] + ol;
    const double* loc = p.locs + (int64_t)f * p.lines;
    const double nominal = p.nominal;
    const double out_scale = nominal / (double)p.outlen;
    const double* w = p.level_work + (int64_t)f * 1024;
    const double adj = w[2 * line];
    const double ll = loc[line];
    const double delta = loc[line + 1] - ll;
    TbcLineConsts c;
    c.a = split_double(ll + delta * (((double)line * p.outlen * out_scale - (double)line * nominal) / nominal));
    c.b = split_double(delta * out_scale / nominal);
    c.adj = split_double(adj);
    c.dlev = split_double(w[2 * line + 1] - adj);
    c.ire0 = split_double(p.ire0);
    c.k = split_double(p.output_scale * p.inv_hz_ire);
    c.off = split_double(p.offset);
    c.smooth = p.smoothing > 0.0 && line > 0;
    reinterpret_cast<TbcLineConsts*>(p.line_consts + t * kTbcLineConstsBytes)[0] = c;
}

constexpr int kTbcFastMaxThreads = 384;
// kPair: a second source (src2 -> out2_f32) summed with the same taps; its own
// instantiation, so the single-source kernel keeps its register count (two
// CTAs per SM).
template <bool kPair>
__global__ void __launch_bounds__(kTbcFastMaxThreads) k_tbc_fast(const float* stream, int64_t stream_len,
                                                                 TbcParams p) {
    const int f = blockIdx.y;
    const int ol = blockIdx.x;
    const int64_t s0 = p.span_start[f];
    const int64_t n = min(p.span_len[f], stream_len - s0);
    const int n32 = (int)n;
    const float* src = stream + s0;
    const TbcLineConsts& c = *reinterpret_cast<const TbcLineConsts*>(
        p.line_consts + ((int64_t)f * p.out_lines + ol) * kTbcLineConstsBytes);
    const float4* lut4 = reinterpret_cast<const float4*>(p.lut);
    const float4* pair4 = reinterpret_cast<const float4*>(p.lut_pair);
    uint16_t* out = p.out_u16 ? p.out_u16 + ((int64_t)f * p.out_lines + ol) * p.outlen : nullptr;
    const float* src2 = p.src2 ? p.src2 + s0 : nullptr;
    float* out2 = p.out2_f32 ? p.out2_f32 + ((int64_t)f * p.out_lines + ol) * p.outlen : nullptr;
    float* outf32 = p.out_f32 ? p.out_f32 + ((int64_t)f * p.out_lines + ol) * p.out_stride - p.x0 : nullptr;
    const int kx1 = p.x1 > 0 ? p.x1 : p.outlen;
    // Each lane owns one output sample (position, level and conversion done
    // once); the 16-tap sums are gathered cooperatively: in round r the quad
    // q of lanes works on the sample of lane 8 r + q, lane `sub` reading taps
    // 4 sub .. 4 sub + 3, so a sample's 128-byte row pair is read by one
    // quad in two coalesced accesses instead of eight scattered ones.
    const int lane = threadIdx.x & 31;
    const int q = lane >> 2, sub = lane & 3;
    for (int k0 = p.x0; k0 < kx1; k0 += blockDim.x) {
        const int k = k0 + threadIdx.x;
        const bool valid = k < kx1;
        const float kf = (float)(valid ? k : 0);
        float2 kb = ff_mul(kf, 0.0f, c.b.x, c.b.y);
        float2 pos = ff_add(c.a.x, c.a.y, kb.x, kb.y);
        float coord = __fadd_rn(pos.x, pos.y);
        int ci = (int)coord;
        float fraction = __fsub_rn(coord, (float)ci);
        float pp = __fmul_rn(fraction, 65536.0f);
        int ps = (int)pp;
        int pe = ps + 1;
        float alpha = __fsub_rn(pp, (float)ps);
        ps = wrap_idx(ps, 65537);
        pe = wrap_idx(pe, 65537);
        const int start = ci - 7;
        const int interior = (n >= 16 && (uint32_t)start <= (uint32_t)(n - 16)) ? 1 : 0;
        float hi_own = 0.0f, lo_own = 0.0f, hi2_own = 0.0f, lo2_own = 0.0f;
#pragma unroll
        for (int rnd = 0; rnd < 4; rnd++) {
            const int owner = rnd * 8 + q;
            const int ps_o = __shfl_sync(0xffffffffu, ps, owner);
            const int pe_o = __shfl_sync(0xffffffffu, pe, owner);
            const int st_o = __shfl_sync(0xffffffffu, start, owner);
            const float al_o = __shfl_sync(0xffffffffu, alpha, owner);
            const int in_o = __shfl_sync(0xffffffffu, interior, owner);
            float4 ws, we;
            if (pe_o == ps_o + 1 && pair4) {
                const float4* rs = pair4 + (int64_t)ps_o * 8;
                ws = __ldg(rs + sub);
                we = __ldg(rs + 4 + sub);
            } else {
                ws = __ldg(lut4 + (int64_t)ps_o * 4 + sub);
                we = __ldg(lut4 + (int64_t)pe_o * 4 + sub);
            }
            const float wsv[4] = {ws.x, ws.y, ws.z, ws.w};
            const float wev[4] = {we.x, we.y, we.z, we.w};
            float hi = 0.0f, lo = 0.0f, hi2 = 0.0f, lo2 = 0.0f;
#pragma unroll
            for (int r = 0; r < 4; r++) {
                float wt = __fmaf_rn(al_o, __fsub_rn(wev[r], wsv[r]), wsv[r]);
                // 32-bit tap index: a field span is far below 2^31 samples
                int idx = st_o + 4 * sub + r;
                if (!in_o) {
                    if (idx < 0) idx += n32;
                    idx = idx < 0 ? 0 : (idx > n32 - 1 ? n32 - 1 : idx);
                }
                float prod = __fmul_rn(__ldg(src + idx), wt);
                float s, e;
                two_sum(hi, prod, s, e);
                hi = s;
                lo = __fadd_rn(lo, e);
                if (kPair) {
                    float prod2 = __fmul_rn(__ldg(src2 + idx), wt);
                    two_sum(hi2, prod2, s, e);
                    hi2 = s;
                    lo2 = __fadd_rn(lo2, e);
                }
            }
#pragma unroll
            for (int o = 1; o < 4; o <<= 1) {
                float oh = __shfl_xor_sync(0xffffffffu, hi, o);
                float olo = __shfl_xor_sync(0xffffffffu, lo, o);
                float2 t = ff_add(hi, lo, oh, olo);
                hi = t.x;
                lo = t.y;
            }
            // the owners of this round (lanes 8 rnd .. 8 rnd + 7) take their sums
            const float rh = __shfl_sync(0xffffffffu, hi, 4 * (lane & 7));
            const float rl = __shfl_sync(0xffffffffu, lo, 4 * (lane & 7));
            if ((lane >> 3) == rnd) { hi_own = rh; lo_own = rl; }
            if (kPair) {
#pragma unroll
                for (int o = 1; o < 4; o <<= 1) {
                    float oh = __shfl_xor_sync(0xffffffffu, hi2, o);
                    float olo = __shfl_xor_sync(0xffffffffu, lo2, o);
                    float2 t = ff_add(hi2, lo2, oh, olo);
                    hi2 = t.x;
                    lo2 = t.y;
                }
                const float rh2 = __shfl_sync(0xffffffffu, hi2, 4 * (lane & 7));
                const float rl2 = __shfl_sync(0xffffffffu, lo2, 4 * (lane & 7));
                if ((lane >> 3) == rnd) { hi2_own = rh2; lo2_own = rl2; }
            }
        }
        if (!valid) continue;
        float2 la = c.adj;
        if (c.smooth) {
            float2 pw = p.pw_ff[k];
            float2 t = ff_mul(pw.x, pw.y, c.dlev.x, c.dlev.y);
            la = ff_add(c.adj.x, c.adj.y, t.x, t.y);
        }
        float2 v = ff_mul(hi_own, lo_own, la.x, la.y);
        float outf = __fadd_rn(v.x, v.y);
        if (kPair) {
            float2 v2 = ff_mul(hi2_own, lo2_own, la.x, la.y);
            out2[k] = __fadd_rn(v2.x, v2.y);
        }
        if (outf32) {
            outf32[k] = outf;   // float output (the chroma channel): no conversion
            continue;
        }
        if (!isfinite(outf)) {
            out[k] = outf > 0.0f ? 65535 : 0;
            continue;
        }
        // val = (outf - ire0) * k + off, floor taken on the pair
        float2 d = ff_add(outf, 0.0f, -c.ire0.x, -c.ire0.y);
        float2 sk = ff_mul(d.x, d.y, c.k.x, c.k.y);
        float2 val = ff_add(sk.x, sk.y, c.off.x, c.off.y);
        uint16_t u;
        if (!(fabsf(val.x) < 1.0e6f)) {
            u = val.x > 0.0f ? 65535 : 0;   // infinite, huge or NaN (NaN converts to 0)
        } else {
            float fl = floorf(val.x);
            float r = __fadd_rn(__fsub_rn(val.x, fl), val.y);
            int F = (int)fl + (r < 0.0f ? -1 : (r >= 1.0f ? 1 : 0));
            u = (uint16_t)(F < 0 ? 0 : (F > 65535 ? 65535 : F));
        }
        out[k] = u;
    }
}
}  // namespace

// pw must hold (1-alpha)^(k+1) for k in [0, outlen) when smoothing > 0.
// Float streams render with float-float accumulation when only uint16 output
// is asked for; double streams and float-value outputs use binary64 as the
// reference does.
template <typename T>
cudaError_t launch_tbc_pw(const T* stream, int64_t stream_len, const TbcParams& p, const double* pw,
                          cudaStream_t s) {
    if (p.nfields <= 0) return cudaSuccess;
    k_tbc_levels<<<p.nfields, 512, 0, s>>>(p, pw);   // one compare-exchange per thread per sort stage
    dim3 grid(p.out_lines, p.nfields);
    const bool one_out = (p.out_u16 != nullptr) != (p.out_f32 != nullptr);
    if (sizeof(T) == sizeof(float) && one_out && !p.out_hz && (p.smoothing <= 0.0 || p.pw_ff) &&
        p.line_consts) {
        const int64_t nl = (int64_t)p.nfields * p.out_lines;
        k_tbc_consts<<<(unsigned)((nl + 127) / 128), 128, 0, s>>>(p);
        // a line in the fewest passes of at most 384 lanes, with the fewest idle
        // lanes in the last pass (NTSC 910 samples: 3 x 320, PAL 1135: 3 x 384)
        const int width = (p.x1 > 0 ? p.x1 : p.outlen) - p.x0;
        const int passes = (width + kTbcFastMaxThreads - 1) / kTbcFastMaxThreads;
        const int threads = ((width + passes - 1) / passes + 31) / 32 * 32;
        if (p.src2)
            k_tbc_fast<true><<<grid, threads, 0, s>>>(reinterpret_cast<const float*>(stream), stream_len, p);
        else
            k_tbc_fast<false><<<grid, threads, 0, s>>>(reinterpret_cast<const float*>(stream), stream_len, p);
    } else {
        k_tbc<T><<<grid, 256, 0, s>>>(stream, stream_len, p, pw);
    }
    return cudaGetLastError();
}
template cudaError_t launch_tbc_pw<float>(const float*, int64_t, const TbcParams&, const double*, cudaStream_t);
template cudaError_t launch_tbc_pw<double>(const double*, int64_t, const TbcParams&, const double*, cudaStream_t);

// ============================================================== dropouts
// DetectTapeDropouts + RfDropoutDetector.FindDropouts + TbcDropoutMapper.MapTapeRfToTbc
// (Core/Decode/TbcFieldDecodePipeline.cs:6593-6640; Core/Decode/TbcDropoutMapping.cs:52-107, 288-370).
// threshold = float32 mean of the envelope over the field span * 0.18f; the
// device emits ordered run boundaries of (env <= thr) and starts of
// (env >= thr * hysteresis) per 16384-sample chunk, then one thread per field
// runs the merge state machine over those events and maps the ranges to
// (field line, start x, end x).
namespace {
constexpr int kDT = 256;
constexpr int kDChunk = 16384;
constexpr int kDPer = kDChunk / kDT;

__global__ void k_drop_ranges(DropoutParams p, int64_t stream_len) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= p.nfields) return;
    int64_t n = min(p.span_len[f], stream_len - p.span_start[f]);
    const double* loc = p.locs + (int64_t)f * p.lines;
    int sl = p.start_line[f], el = p.end_line[f];
    int64_t r0 = 0, r1 = 0;
    if (sl >= 0 && el > sl && sl < p.lines) {
        double a = floor(loc[sl]);
        r0 = a < 0 ? 0 : (a > (double)n ? n : (int64_t)a);
        double b = ceil(loc[el]);
        r1 = b < (double)r0 ? r0 : (b > (double)n ? n : (int64_t)b);
    }
    p.range[2 * f] = r0;
    p.range[2 * f + 1] = r1;
}

template <typename T>
__global__ void k_env_partial(const T* stream, int64_t stream_len, DropoutParams p, float* partial,
                              int nchunk) {
    __shared__ float wsum[kDT / 32];
    const int f = blockIdx.y, c = blockIdx.x;
    const int64_t s0 = p.span_start[f];
    const int64_t n = min(p.span_len[f], stream_len - s0);
    float acc = 0.0f;
    for (int k = 0; k < kDPer; k++) {
        int64_t i = (int64_t)c * kDChunk + k * kDT + threadIdx.x;
        if (i < n) acc += (float)stream[s0 + i];
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int i = 0; i < kDT / 32; i++) t += wsum[i];
        partial[(int64_t)f * nchunk + c] = t;
    }
}

__global__ void k_env_mean(DropoutParams p, const float* partial, int nchunk, int64_t stream_len) {
    int f = blockIdx.x;
    if (threadIdx.x != 0) return;
    float t = 0.0f;
    for (int c = 0; c < nchunk; c++) t += partial[(int64_t)f * nchunk + c];
    int64_t n = min(p.span_len[f], stream_len - p.span_start[f]);
    p.mean_out[f] = t / (float)n;
}

// Exact float forms of the two dropout comparisons: for a float sample v,
// v <= (double)down  <=>  v <= dn  and  v >= up  <=>  v >= upf  with upf the
// smallest float not below up.
template <typename T>
struct DropThr {
    T down, up;
};
__device__ inline DropThr<double> make_drop_thr(float thrf, double hyst, double*) {
    return {(double)thrf, (double)thrf * hyst};
}
__device__ inline DropThr<float> make_drop_thr(float thrf, double hyst, float*) {
    double up = (double)thrf * hyst;
    float u = (float)up;
    if ((double)u < up) u = nextafterf(u, INFINITY);
    return {thrf, u};
}

constexpr int kDWarp = kDChunk / (kDT / 32);   // 2048 samples per warp
constexpr int kDIter = kDWarp / 32;

// event = 4*pos + type; type 0: (env <= down) run start, 1: run end, 2: (env >= up) start.
// Each warp scans a contiguous 2048-sample slice with ballots, keeps the
// per-iteration masks in shared memory, and writes its events in order after a
// CTA scan of the warp counts.
template <typename T>
__global__ void __launch_bounds__(kDT) k_drop_events(const T* stream, int64_t stream_len,
                                                     DropoutParams p, int nchunk, int* chunk_counts) {
    __shared__ int wtot[kDT / 32];
    __shared__ unsigned masks[kDT / 32][kDIter][3];
    const int f = blockIdx.y, c = blockIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t s0 = p.span_start[f];
    const T* env = stream + s0;
    const int64_t r0 = p.range[2 * f], r1 = p.range[2 * f + 1];
    const DropThr<T> th = make_drop_thr(__fmul_rn(p.mean_out[f], p.frac), p.hyst, (T*)nullptr);
    const int64_t base = r0 + (int64_t)c * kDChunk + (int64_t)w * kDWarp;
    auto flags = [&](int64_t i, bool& a, bool& b) {
        if (i < r0 || i >= r1) { a = false; b = false; return; }
        T v = env[i];
        a = v <= th.down;
        b = v >= th.up;
    };
    bool pa, pb;
    flags(base - 1, pa, pb);
    unsigned sa = pa ? 1u : 0u, sb = pb ? 1u : 0u;
    int cnt = 0, iters = 0;
    // eight loads in flight per lane, then the ballots in order
    for (int it0 = 0; it0 < kDIter; it0 += 8) {
        if (base + it0 * 32 > r1) break;
        T v[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            int64_t i = base + (it0 + j) * 32 + lane;
            v[j] = (i >= r0 && i < r1) ? env[i] : (T)0;
        }
#pragma unroll
        for (int j = 0; j < 8; j++) {
            int it = it0 + j;
            int64_t i = base + it * 32 + lane;
            bool in = i >= r0 && i < r1;
            bool a = in && v[j] <= th.down, b = in && v[j] >= th.up;
            unsigned A = __ballot_sync(0xffffffffu, a), B = __ballot_sync(0xffffffffu, b);
            unsigned ea = A ^ ((A << 1) | sa);
            unsigned eb = B & ~((B << 1) | sb);
            sa = A >> 31;
            sb = B >> 31;
            if (lane == 0) { masks[w][it][0] = ea; masks[w][it][1] = A & ea; masks[w][it][2] = eb; }
            cnt += __popc(ea) + __popc(eb);
        }
        iters = it0 + 8;
    }
    if (lane == 0) wtot[w] = cnt;
    __syncthreads();
    int wb = 0, tot = 0;
    for (int i = 0; i < kDT / 32; i++) { if (i < w) wb += wtot[i]; tot += wtot[i]; }
    if (threadIdx.x == 0) chunk_counts[(int64_t)f * nchunk + c] = tot;
    if (cnt == 0) return;
    int64_t* ev = p.events + ((int64_t)f * nchunk + c) * p.cap;
    int off = wb;
    const unsigned lt = (1u << lane) - 1u;
    for (int it = 0; it < iters; it++) {
        unsigned ea = masks[w][it][0], ta = masks[w][it][1], eb = masks[w][it][2];
        if ((ea | eb) == 0u) continue;
        unsigned bit = 1u << lane;
        int pre = __popc(ea & lt) + __popc(eb & lt);
        int64_t i = base + it * 32 + lane;
        int o = off + pre;
        if (ea & bit) { if (o < p.cap) ev[o] = 4 * i + ((ta & bit) ? 0 : 1); o++; }
        if (eb & bit) { if (o < p.cap) ev[o] = 4 * i + 2; }
        off += __popc(ea) + __popc(eb);
    }
}

constexpr int kDropSmemEvents = 4096;

size_t drop_finish_smem(int lines, int nchunk) {
    return (size_t)lines * sizeof(double) + kDropSmemEvents * sizeof(int64_t) +
           (size_t)(nchunk + 1) * sizeof(int);
}

// One CTA per field.  The field's line locations, chunk offsets and (when they
// fit) its events are staged in shared memory, each event gathered by one
// thread (its chunk found by binary search over the chunk offsets).  Warp 0
// then runs the merge state machine, the minimum length rule and the TBC
// mapping, every lane in step (lane 0 writes): the mapping's search for the
// line holding a dropout start tests 32 lines per ballot, in line order, so it
// finds the same line as the reference's walk (MapTapeRfToTbc).
__global__ void k_drop_finish(DropoutParams p, int nchunk, const int* chunk_counts) {
    extern __shared__ __align__(16) unsigned char dsm[];
    double* sloc = reinterpret_cast<double*>(dsm);
    int64_t* sev = reinterpret_cast<int64_t*>(sloc + p.lines);
    int* soff = reinterpret_cast<int*>(sev + kDropSmemEvents);
    __shared__ int s_status;
    const int f = blockIdx.x;
    const int lane = threadIdx.x & 31;
    const double* gloc = p.locs + (int64_t)f * p.lines;
    for (int i = threadIdx.x; i < p.lines; i += blockDim.x) sloc[i] = gloc[i];
    if (threadIdx.x < 32) {
        int carry = 0, st = 0;
        for (int c0 = 0; c0 < nchunk; c0 += 32) {
            int c = c0 + lane;
            int v = c < nchunk ? chunk_counts[(int64_t)f * nchunk + c] : 0;
            if (v > p.cap) { v = p.cap; st = 2; }
            int incl = v;
            for (int o = 1; o < 32; o <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            if (c < nchunk) soff[c] = carry + incl - v;
            carry += __shfl_sync(0xffffffffu, incl, 31);
        }
        st = __reduce_max_sync(0xffffffffu, st);
        if (lane == 0) { soff[nchunk] = carry; s_status = st; }
    }
    __syncthreads();
    const int total = soff[nchunk];
    const bool fits = total <= kDropSmemEvents;
    if (fits) {
        for (int e = threadIdx.x; e < total; e += blockDim.x) {
            // the last chunk starting at or before e holds it (empty chunks share offsets)
            int lo = 0, hi = nchunk - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (soff[mid] <= e) lo = mid;
                else hi = mid - 1;
            }
            sev[e] = p.events[((int64_t)f * nchunk + lo) * p.cap + (e - soff[lo])];
        }
    }
    __syncthreads();
    if (threadIdx.x >= 32) return;
    const int64_t r1 = p.range[2 * f + 1];
    int32_t* out = p.out + (int64_t)f * p.out_cap * 3;
    int nout = 0;
    int status = s_status;
    const double* loc = sloc;
    const int sl = p.start_line[f], el = p.end_line[f], off = p.line_offset[f];
    // mapping state (MapTapeRfToTbc)
    int li = sl;
    double ls = 0.0, le = 0.0;
    bool map_ok = sl >= 0 && el > sl && el < p.lines;
    if (map_ok) { ls = loc[li]; le = loc[li + 1]; }
    bool map_done = !map_ok;
    auto emit = [&](int line, int sx, int ex) {
        if (nout < p.out_cap) {
            if (lane == 0) { out[3 * nout] = line; out[3 * nout + 1] = sx; out[3 * nout + 2] = ex; }
        } else {
            status = 1;
        }
        nout++;
    };
    auto map_range = [&](double ds, double de) {
        if (map_done) return;
        // first line k >= li whose span holds ds (the first line also takes a
        // ds before it); none: the walk ran off the field
        int k = -1;
        for (int base = li; base < el; base += 32) {
            const int kk = base + lane;
            bool hit = false;
            if (kk < el) {
                const double a = loc[kk], b = loc[kk + 1];
                hit = (ds >= a || kk == sl) && ds < b && b - a > 0.0;
            }
            const unsigned m = __ballot_sync(0xffffffffu, hit);
            if (m) { k = base + __ffs(m) - 1; break; }
        }
        if (k < 0) { li = el; map_done = true; return; }
        li = k;
        ls = loc[li];
        le = loc[li + 1];
        const int sx = (int)floor(((ds - ls) / (le - ls)) * p.outlen);
        int cur_line = li - off, cur_sx = sx > 0 ? sx : 0;
        while (li < el) {
            double ll = le - ls;
            if (de < le && ll > 0.0) {
                int ex = (int)ceil(((de - ls) / ll) * p.outlen);
                emit(cur_line, cur_sx, ex < p.outlen ? ex : p.outlen);
                break;
            }
            emit(cur_line, cur_sx, p.outlen);
            li++;
            if (li < el) {
                ls = loc[li]; le = loc[li + 1];
                cur_line = li - off;
                cur_sx = 0;
            }
        }
    };
    bool have = false, open = false, pending = false;
    int64_t start = 0, last_end = 0, cand = 0;
    auto step = [&](int64_t evv) {
        const int64_t pos = evv >> 2;
        const int type = (int)(evv & 3);
        if (type == 0) {
            if (!have) { start = pos; open = true; have = true; }
            else if (!open) {
                int64_t c2 = last_end + p.merge + 1;
                cand = pos > c2 ? pos : c2;
                pending = true;
            }
        } else if (type == 1) {
            if (pending) {
                if (cand < pos) { start = cand; open = true; }
                pending = false;
            }
        } else {
            if (have && open) {
                open = false;
                last_end = pos;
                if (pos - start > p.min_len) map_range((double)start, (double)pos);
            }
        }
    };
    if (fits) {
        for (int e = 0; e < total; e++) step(sev[e]);
    } else {
        for (int c = 0; c < nchunk; c++) {
            const int cnt = soff[c + 1] - soff[c];
            const int64_t* ev = p.events + ((int64_t)f * nchunk + c) * p.cap;
            for (int e = 0; e < cnt; e++) step(ev[e]);
        }
    }
    if (have && open && r1 - start > p.min_len) map_range((double)start, (double)r1);
    if (lane == 0) {
        p.out_count[f] = nout;
        p.status[f] = status;
    }
}
}  // namespace

int dropout_chunks(int64_t span_len) { return (int)((span_len + kDChunk - 1) / kDChunk); }

template <typename T>
cudaError_t launch_drop_mean(const T* stream, int64_t stream_len, const DropoutParams& p, float* partial,
                             cudaStream_t s) {
    if (p.nfields <= 0) return cudaSuccess;
    int nchunk = dropout_chunks(p.max_span_len);
    dim3 g(nchunk, p.nfields);
    k_env_partial<T><<<g, kDT, 0, s>>>(stream, stream_len, p, partial, nchunk);
    k_env_mean<<<p.nfields, 32, 0, s>>>(p, partial, nchunk, stream_len);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_drop_detect(const T* stream, int64_t stream_len, const DropoutParams& p, int* chunk_counts,
                               cudaStream_t s) {
    if (p.nfields <= 0) return cudaSuccess;
    int nchunk = dropout_chunks(p.max_span_len);
    k_drop_ranges<<<(p.nfields + 127) / 128, 128, 0, s>>>(p, stream_len);
    dim3 g(nchunk, p.nfields);
    k_drop_events<T><<<g, kDT, 0, s>>>(stream, stream_len, p, nchunk, chunk_counts);
    size_t smem = drop_finish_smem(p.lines, nchunk);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_drop_finish, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    k_drop_finish<<<p.nfields, 128, smem, s>>>(p, nchunk, chunk_counts);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_dropouts_full(const T* stream, int64_t stream_len, const DropoutParams& p,
                                 float* partial, int* chunk_counts, cudaStream_t s) {
    cudaError_t e = launch_drop_mean<T>(stream, stream_len, p, partial, s);
    if (e != cudaSuccess) return e;
    return launch_drop_detect<T>(stream, stream_len, p, chunk_counts, s);
}
template cudaError_t launch_dropouts_full<float>(const float*, int64_t, const DropoutParams&, float*, int*, cudaStream_t);
template cudaError_t launch_dropouts_full<double>(const double*, int64_t, const DropoutParams&, float*, int*, cudaStream_t);
template cudaError_t launch_drop_mean<float>(const float*, int64_t, const DropoutParams&, float*, cudaStream_t);
template cudaError_t launch_drop_mean<double>(const double*, int64_t, const DropoutParams&, float*, cudaStream_t);
template cudaError_t launch_drop_detect<float>(const float*, int64_t, const DropoutParams&, int*, cudaStream_t);
template cudaError_t launch_drop_detect<double>(const double*, int64_t, const DropoutParams&, int*, cudaStream_t);

}  // namespace vhsd
