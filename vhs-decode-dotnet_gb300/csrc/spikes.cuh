// ReplaceSpikes (Core/Dsp/RfDemodulator.cs:966-1001) for one block, in
// parallel on one CTA.
//
// The reference visits the spikes i_j of the unrepaired demod (demod > max)
// in ascending order; window j is [lo_j, hi_j) = [max(i_j - 8, 0),
// min(i_j + 30, n - 1)) and is overwritten with the diff-demod when
// max(diffed over it) < max(current demod over it).  Because the windows'
// starts and ends never decrease, the samples of window j that earlier
// replacements changed are exactly [lo_j, M), M being the end of the last
// replaced window, and those now hold diffed values that cannot lift the
// current max above max(diffed over the window).  So window j is replaced
// iff some original demod sample in [max(M, lo_j), hi_j) exceeds max(diffed
// over the window), i.e. iff max(M, lo_j) < c_j where c_j is one past the last
// such sample (INT_MIN if none).  The c_j are independent (phase 1, all
// threads); the ordered walk only carries M (phase 2, one warp, three
// shuffles per spike); the replacement copies are independent (phase 3).
// Maxima ignore NaN operands (fmaxf).
#pragma once
#include <climits>
#include <cuda_runtime.h>

namespace vhsd {

// c_j for every spike bit of `mask` (n / 32 words, bit k of word w = sample 32 w + k).
__device__ inline void spike_thresholds(const float* demod, const float* diffed, const unsigned* mask,
                                        int* cpos, int n, int tid, int nthreads) {
    for (int w = tid; w < n / 32; w += nthreads) {
        unsigned m = mask[w];
        while (m) {
            int b = __ffs(m) - 1;
            m &= m - 1;
            int i0 = w * 32 + b;
            int lo = max(i0 - 8, 0), hi = min(i0 + 30, n - 1);
            int cj = INT_MIN;
            if (lo < hi) {
                float mdd = -INFINITY;
                for (int k = lo; k < hi; k++) mdd = fmaxf(mdd, diffed[k]);
                for (int k = hi - 1; k >= lo; k--)
                    if (demod[k] > mdd) { cj = k + 1; break; }
            }
            cpos[i0] = cj;
        }
    }
}

// Ordered walk over the spikes by one warp; repl (n / 32 words) receives the
// replaced spikes.
__device__ inline void spike_walk(const unsigned* mask, const int* cpos, unsigned* repl, int n, int lane) {
    int mend = 0;
    const int words = n / 32;
    for (int w0 = 0; w0 < words; w0 += 32) {
        unsigned mw = (w0 + lane < words) ? mask[w0 + lane] : 0u;
        if (w0 + lane < words) repl[w0 + lane] = 0u;
        unsigned nz = __ballot_sync(0xffffffffu, mw != 0u);
        while (nz) {
            int wl = __ffs(nz) - 1;
            nz &= nz - 1;
            int w = w0 + wl;
            unsigned m = __shfl_sync(0xffffffffu, mw, wl);
            int i0 = w * 32 + lane;
            bool has = (m >> lane) & 1u;
            int cj = has ? cpos[i0] : INT_MIN;
            int lo = max(i0 - 8, 0), hi = min(i0 + 30, n - 1);
            unsigned rw = 0u;
            while (m) {
                int b = __ffs(m) - 1;
                m &= m - 1;
                int cb = __shfl_sync(0xffffffffu, cj, b);
                int lb = __shfl_sync(0xffffffffu, lo, b);
                int hb = __shfl_sync(0xffffffffu, hi, b);
                if (cb != INT_MIN && max(mend, lb) < cb) { mend = hb; rw |= 1u << b; }
            }
            if (lane == 0) repl[w] = rw;
        }
    }
}

// Copies the diff-demod over every replaced window (overlapping windows
// write equal values).
__device__ inline void spike_apply(float* demod, const float* diffed, const unsigned* repl, int n, int tid,
                                   int nthreads) {
    for (int w = tid; w < n / 32; w += nthreads) {
        unsigned m = repl[w];
        while (m) {
            int b = __ffs(m) - 1;
            m &= m - 1;
            int i0 = w * 32 + b;
            int lo = max(i0 - 8, 0), hi = min(i0 + 30, n - 1);
            for (int k = lo; k < hi; k++) demod[k] = diffed[k];
        }
    }
}

}  // namespace vhsd
