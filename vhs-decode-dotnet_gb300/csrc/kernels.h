// Device-side entry points of the VHS RF decode path and their parameter
// blocks.  All pointers are device pointers unless noted.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace vhsd {

constexpr int kBlock = 32768;
constexpr int kCut = 1024;
constexpr int kStride = 30720;
constexpr int kHalf = 16385;  // kBlock/2 + 1 spectrum bins

// ---------------------------------------------------------------- FP32 fused
// Sub-deemphasis of ApplySubDeemphasisRealCore (Core/Dsp/RfDemodulator.cs:2852-2990):
// high = irfft(D x Video x HighPass); amp = |analytic(high)| * 2 / deviation,
// first-order low-pass filtfilt, then max(0), x scale1, ^exponent, x scale2,
// x logistic; video -= high * (1 - amp) + high * static_factor.
template <typename T, typename T2>
struct SubDeemphT {
    const T2* high;            // [kHalf] Video x high-pass, nullptr = off
    T inv_half_dev;            // 2 / deviation
    T b0, b1, a1;              // amplitude low-pass
    T exponent, scale1, scale2;   // absent scales are 1
    T logistic_mid, logistic_rate;  // rate <= 0: no logistic factor
    T static_factor;
};
using SubDeemph = SubDeemphT<float, float2>;
using SubDeemph64 = SubDeemphT<double, double2>;

struct FastDemodParams {
    const int16_t* rf;         // capture, 16-byte aligned
    const float* rf_f32;       // float capture (16-byte aligned), read instead of rf when set
    unsigned* block_counter;   // zeroed before the launch: dynamic block claims (null: static schedule)
    int64_t first_block;       // first 32768-sample block to decode
    int64_t nblocks;           // number of blocks
    const float* rf_video;     // [kHalf] real RF band-pass gain
    const float2* video;       // [kHalf] video LPF x de-emphasis
    const float2* sync;        // [kHalf] video reference x 0.5 MHz FIR
    const float2* tw_hi;       // [256] exp(-2 pi i h 128 / 32768)
    const float2* tw_lo;       // [128] exp(-2 pi i l / 32768)
    float fs;                  // sample rate (Hz)
    float diff_max;            // diff-demod spike limit (Hz)
    float dc;                  // subtracted before the demod FFT (ire0) ...
    float dc_video, dc_sync;   // ... and added back as ire0 x the filters' DC gains
    float env_b0, env_b1, env_a1;
    float* video_out;          // stitched stream, stream index s = b*30720 + n - 1024
    float* sync_out;
    float* env_out;
    float2* scratch;           // repair scratch: per cluster 2*32768 float2 (demod, diff-demod, spike mask, thresholds)
    int* repair_count;         // counts blocks that took the spike-repair path
    SubDeemph sub;             // sub-deemphasis (sub.high == nullptr: off)
    int fft_plan;              // radix plans: bits 0-1 the 8192-point, bits 2-3 the 16384-point transform
    // optional pulse-scan bits of the sync stream (one bit per stream sample,
    // 32 per word): v <= sync_thr, and NaN (hold); null: not written
    unsigned* sync_cond;
    unsigned* sync_hold;
    float sync_thr;
    // diagnostics only (launch_demod_fp32_timed): per-rank cycle sums of the
    // kernel's stages, [rank * kDemodStages + stage]
    unsigned long long* stage_cycles;
    // batched launch (launch_demod_fp32_batched): the blocks of several
    // windows, each with its own parameters (capture, filters, format,
    // outputs; int16 input) in batch_jobs[j], job j owning the global blocks
    // [batch_start[j], batch_start[j + 1]); nblocks is then the total
    const FastDemodParams* batch_jobs;
    const int64_t* batch_start;
    int batch_njobs;
};
constexpr int kDemodStages = 20;
// Radix plans the fused kernel is compiled for (8192-point plan | 16384-point
// plan << 2): 16x16x32 | 16x32x32, 32x16x16 | 16x32x32, 16x16x32 | 32x32x16,
// 32x16x16 | 32x32x16.  The other plans of the transforms (16x32x16, 8x32x32;
// 32x16x32) measured 1-30 % slower on GB300.
constexpr int kFftPlanCount = 4;
constexpr int kFftPlans[kFftPlanCount] = {0, 1, 4, 5};

size_t fp32_smem_bytes();
cudaError_t launch_demod_fp32(const FastDemodParams& p, int num_clusters, cudaStream_t stream);
// The same kernel (plan 0) with clock64() stage marks summed into p.stage_cycles.
cudaError_t launch_demod_fp32_timed(const FastDemodParams& p, int num_clusters, cudaStream_t stream);
// One persistent launch over the blocks of p.batch_njobs windows (p: the
// shared twiddles, block counter, repair scratch and plan; the total in
// p.nblocks).  Each block is computed exactly as in its window's own launch.
cudaError_t launch_demod_fp32_batched(const FastDemodParams& p, int num_clusters, cudaStream_t stream);

// 2:1 half-band decimation of a capture (exactly one of src16 / src32, 16-byte
// aligned): out_len float samples, output i centred on source sample 2 i.
constexpr int kDecimateKernels = 1;
cudaError_t launch_decimate_half(const int16_t* src16, const float* src32, int64_t src_len, float* dst,
                                 int64_t out_len, cudaStream_t s);

// ---------------------------------------------------------------- FP64 plain
struct PlainDemodParams {
    const int16_t* rf;
    const float* rf_f32;       // float capture, read instead of rf when set
    int64_t block;             // block index
    const double* rf_video;    // [kHalf]
    const double2* video;      // [kHalf]
    const double2* sync;       // [kHalf]
    double fs, diff_max;
    double env_b0, env_b1, env_a1;
    double* video_out;         // stitched stream (double)
    double* sync_out;
    double* env_out;
    double2* work;             // per-block workspace: 4 * 32768 double2
    double* dwork;             // per-block workspace: 3 * 32768 double
    float* fwork;              // 32768 + 12 floats (envelope)
    int* flag;                 // spike flag
    unsigned* mask;            // 1024 words
    int64_t* blk;              // device-resident block index, advanced per replay
    SubDeemph64 sub;           // sub-deemphasis (sub.high == nullptr: off)
};
cudaError_t launch_demod_fp64_block(const PlainDemodParams& p, cudaStream_t stream);
constexpr int kPlainBlockKernels = 38;  // kernels in one plain-path block (13 + 5 FFTs x 5 passes)
constexpr int kPlainSubKernels = 10;    // added by sub-deemphasis (5 + 1 FFT x 5 passes)

// ---------------------------------------------------------------- pulses
// Sync-pulse edge events of PulseDetection.FindPulses over a whole stitched
// stream: starts (value <= high after > high) and ends (value > high after
// <= high), NaN samples hold the state.  Two passes: count per warp slice of
// 1024 samples, then ordered write.  counts / offsets_scratch hold
// pulse_count_slots(n) entries.
constexpr int kPulseChunk = 4096;
constexpr int kPulseKernels = 2;      // kernels one launch_pulse_events* call starts (plus a memset)
inline int64_t pulse_count_slots(int64_t n) { return (n + kPulseChunk - 1) / kPulseChunk * 4; }
template <typename T>
cudaError_t launch_pulse_events(const T* ref, int64_t n, double high, int64_t* counts,
                                int64_t* offsets_scratch, int64_t* events, int64_t capacity,
                                int64_t* total, cudaStream_t stream);
// Same over stream positions [begin, end) of `ref`; the state entering `begin`
// is taken from the samples before it, so consecutive ranges give exactly the
// events of one pass over their union.  Scratch holds pulse_count_slots(end - begin).
// Same events from the pulse-scan bits of FastDemodParams (cond: v <= the
// exact float threshold, hold: NaN), [begin, end) multiples of 32.
cudaError_t launch_pulse_bits_range(const unsigned* cond, const unsigned* hold, int64_t begin, int64_t end,
                                    int64_t* counts, int64_t* offsets_scratch, int64_t* events,
                                    int64_t capacity, int64_t* total, cudaStream_t stream);
// Exact float threshold of a double pulse threshold: v <= high <=> v <= it.
float pulse_float_threshold(double high);
template <typename T>
cudaError_t launch_pulse_events_range(const T* ref, int64_t begin, int64_t end, double high,
                                      int64_t* counts, int64_t* offsets_scratch, int64_t* events,
                                      int64_t capacity, int64_t* total, cudaStream_t stream);

// ---------------------------------------------------------------- hsync refine
struct HsyncParams {
    int nfields;
    int lines;                 // line locations per field
    const double* locs_in;     // [nfields * lines] span-relative
    const uint8_t* filled_in;  // [nfields * lines]
    double* locs_out;
    uint8_t* filled_out;
    const int64_t* span_start; // [nfields] stream index of each field span
    const int64_t* span_len;   // [nfields] span length
    int pal;                   // PAL vsync-line rule
    double threshold;          // sync threshold (Hz)
    int one_us, normal_hsync;  // samples
    double mhz32;              // (float)sample_rate_MHz
    double ire0, hz_ire;
    double ntsc_shift;         // subtracted after refinement (0 for PAL)
    void* work;                // hsync_work_bytes(nfields, lines) of per-line scratch
    int* misses;               // optional: counts carried-porch speculation misses
};
size_t hsync_work_bytes(int nfields, int lines);
constexpr int kHsyncKernels = 3;
template <typename T>
cudaError_t launch_hsync_refine(const T* sync_stream, int64_t stream_len, const HsyncParams& p,
                                cudaStream_t stream);

// ---------------------------------------------------------------- TBC
struct TbcParams {
    int nfields;
    int lines;                  // line locations per field
    const double* locs;         // [nfields * lines]
    const int64_t* span_start;  // [nfields]
    const int64_t* span_len;    // [nfields]
    const int* first_line;      // [nfields] output first line
    int out_lines;              // output lines per field
    int outlen;                 // samples per output line
    double nominal;             // nominal input line length (samples)
    double smoothing;           // wow level-adjust smoothing (lines)
    const float* lut;           // [(65536+1)*16] sinc LUT
    const float* lut_pair;      // optional [65536][32]: rows p and p+1 side by side
    const float2* pw_ff;        // optional [outlen] pw as (hi, lo) float pairs
    double ire0, output_scale, inv_hz_ire, offset;  // uint16 conversion
    uint16_t* out_u16;          // [nfields * out_lines * outlen] or null
    double* out_hz;             // optional float output (values rounded to float)
    float* out_f32;             // optional float output [nfields * out_lines * out_stride]:
                                // samples x0 .. x1-1 of each line at (k - x0)
    int x0, x1, out_stride;     // line window of out_f32 (x1 = 0: the whole line)
    const float* src2;          // optional second float stream rendered with the same
    float* out2_f32;            //   positions and weights (the chroma beside the luma),
                                //   [nfields * out_lines * outlen] (fast float kernel only)
    double* level_work;         // [nfields * (max_first_line + out_lines)] line factors
    unsigned char* line_consts; // [nfields * out_lines * kTbcLineConstsBytes] float-pair line plans
                                // of the fast float kernel (null: binary64 kernel)
};
constexpr int kTbcLineConstsBytes = 64;
constexpr int kTbcKernels = 2;      // levels + sinc (binary64 kernel)
constexpr int kTbcFastKernels = 3;  // levels + line plans + sinc (float kernel)
// pw[k] = (1 - alpha)^(k+1), k < outlen, alpha = 1 / (smoothing * outlen)
template <typename T>
cudaError_t launch_tbc_pw(const T* video_stream, int64_t stream_len, const TbcParams& p,
                          const double* pw, cudaStream_t stream);

// ---------------------------------------------------------------- chroma
// A float32 section cascade run forward-backward (SosFilter.ApplyForwardBackwardFloat32,
// Core/Dsp/SosFilter.cs:369-538): four sections (b0 b1 b2 a0 a1 a2), the
// steady-state initial conditions and the odd-extension length.
struct ChromaCascade {
    float sec[4][6];
    float zi[4][2];
    int edge;
};

// The odd extension of an RF block before its chroma band-pass: the default
// pad length of a 4-section filter with no zero end coefficients,
// 3 * (2 * 4 + 1).  Scratch rows of the block stage hold the extended block
// in whole 32-float chunks, the backward pass's output starting kChromaRowShift
// floats in (so its vector stores are 16-byte aligned).
constexpr int kChromaEdge = 27;
constexpr int kChromaExt = kBlock + 2 * kChromaEdge;
constexpr int kChromaRowStride = (kChromaExt + 31) / 32 * 32;
constexpr int kChromaRowShift = (4 - kChromaExt % 4) % 4;

// Chroma channel of blocks [first_block, first_block + nblocks): the RF block
// band-passed, rolled by `move` and its float mean removed, stitched like the
// demodulated channels (stream index b*30720 + n - 1024).  The capture pointer
// is 16-byte aligned.
struct ChromaBlockParams {
    const int16_t* rf16;       // capture at the decode rate (int16), or
    const float* rf32;         //   float (read when set)
    int64_t first_block, nblocks;
    ChromaCascade c;
    int move;
    float* scratch;            // [nblocks * kChromaRowStride]
    float* out;                // stitched chroma stream
};
constexpr int kChromaBlockKernels = 2;
// Kernel attributes of the chroma kernels (once per device, outside any capture).
cudaError_t prepare_chroma_kernels();
// CTAs (one per SM) of the chroma block stage for nblocks blocks.
int chroma_block_ctas(int64_t nblocks);
cudaError_t launch_chroma_blocks(const ChromaBlockParams& p, cudaStream_t stream);

// Per-field chroma stages of a field batch (every array offset to the batch).
struct ChromaFieldParams {
    int nfields;
    int lines;                  // line locations per field
    const double* locs;         // [nfields * lines] hsync-refined, before the NTSC shift
    double* locs_out;           // [nfields * lines] burst-refined, NTSC-shifted
    double ntsc_shift;          // subtracted from every location after the refinement
    int ntsc;
    int out_lines, outlen;
    int bs, be;                 // burst window of an output line
    int win0, win;              // burst-probe window of a line: [2 bs - be, bs + be)
    int input_line;             // round(nominal input line length)
    double fsc_ratio;
    int rot0, rot1;             // chroma_rotation
    ChromaCascade fin;          // final / burst-probe band-pass
    const float* het;           // [4 * field] heterodyne tables
    const float* bsin;          // [field] burst carrier tables
    const float* bcos;
    const float* ana;           // [nfields * out_lines * win] chroma TBC from line 1, probe windows
    double* probe;              // [nfields * 2 * out_lines * 5] phase, offset, magnitude, I, Q
    double* probe_nrm;          // [nfields * 2 * out_lines * 2] I / magnitude, Q / magnitude of each probe
    int* flip;                  // [nfields * 2]
    int* chosen;                // [nfields] rotation index of the kept sequence
    const int* rot_in;          // rotation index before the first field
    int* rot_out;               // rotation index after the last field
    double* summary;            // [nfields * 4] average, even, odd phase, mean magnitude
    int* status;                // nonzero: a field had no burst to average
    const int* first_line;      // [nfields] output first line
    const int* first_field;     // [nfields] 1: first field
    const int* field_number;    // [nfields] VHS field number (NTSC colour frame)
    const float* cfield;        // [nfields * field] chroma TBC of the output lines
    float* up;                  // [nfields * crow] up-converted field at offset fin.edge of each
                                //   row, then the band-passed field in the same place
    float* fwd;                 // [nfields * crow] forward pass, in reverse order
    int64_t crow;               // row stride of up and fwd: chroma_final_row(field, fin.edge)
    uint16_t* out;              // [nfields * field] uint16 chroma
    double cu_hz, fsc_mhz, burst_abs_ref;
    double ntsc_h;              // NTSC up-conversion carrier step (rad / output sample)
    const float2* ntsc_advance; // [outlen] (cos, sin) of the carrier phase advance of sample k of a line
    float2* line_cs;            // [nfields * out_lines] NTSC: (cos, sin) of the carrier phase at the line start
    double* line_scale;         // [nfields * out_lines] gain scale of the line (lines from 16)
    float2* line_scale_f;       //   the same as a float pair
};
constexpr int kChromaPhaseKernels = 5;    // probes, flips, rotation chain, averages, refinement
constexpr int kChromaDecodeKernels = 7;   // line phases, up-conversion, extension, forward, backward,
                                          // line gains, gain
// Row of the final band-pass buffers: the odd-extended field (field + 2 edge
// samples) rounded up to whole 32-float tiles, plus the tiles a pass reads
// past its end.
inline int64_t chroma_final_row(int64_t field, int edge) { return (field + 2 * edge + 31) / 32 * 32 + 64; }
cudaError_t launch_chroma_phase(const ChromaFieldParams& p, cudaStream_t stream);
cudaError_t launch_chroma_decode(const ChromaFieldParams& p, cudaStream_t stream);

// ---------------------------------------------------------------- dropouts
struct DropoutParams {
    int nfields;
    const int64_t* span_start;  // [nfields]
    const int64_t* span_len;    // [nfields]
    int64_t max_span_len;       // bound of span_len, sizes the per-chunk buffers
    const double* locs;         // [nfields * lines] refined line locations
    int lines;
    const int* start_line;      // [nfields] lineOffset + 1
    const int* end_line;        // [nfields]
    const int* line_offset;     // [nfields]
    int outlen;
    int64_t* range;             // [nfields * 2] span-relative [start, end), written on device
    float frac;                 // 0.18
    double hyst;                // 1.25
    int merge;                  // 30
    int min_len;                // 10
    float* mean_out;            // [nfields] float32 envelope mean over the span
    int64_t* events;            // [nfields * nchunk * cap] 4*pos + type, per 16384-sample chunk
    int cap;                    // events per chunk
    int32_t* out;               // [nfields * out_cap * 3] (field line, start x, end x)
    int out_cap;
    int* out_count;             // [nfields]
    int* status;                // [nfields] 0 ok, 1 output capacity, 2 event capacity
};
int dropout_chunks(int64_t span_len);
constexpr int kDropoutKernels = 5;
// partial: [nfields * nchunk] floats; chunk_counts: [nfields * nchunk]
template <typename T>
cudaError_t launch_dropouts_full(const T* env_stream, int64_t stream_len, const DropoutParams& p,
                                 float* partial, int* chunk_counts, cudaStream_t stream);
// The two halves of launch_dropouts_full: the envelope mean of each field span
// (needs only the spans: 2 kernels), then the detection and TBC mapping
// (needs the refined line locations: 3 kernels).
constexpr int kDropMeanKernels = 2;
template <typename T>
cudaError_t launch_drop_mean(const T* env_stream, int64_t stream_len, const DropoutParams& p, float* partial,
                             cudaStream_t stream);
template <typename T>
cudaError_t launch_drop_detect(const T* env_stream, int64_t stream_len, const DropoutParams& p,
                               int* chunk_counts, cudaStream_t stream);

}  // namespace vhsd
