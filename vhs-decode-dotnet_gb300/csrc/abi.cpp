// C ABI and device session of the GB300 RF decode backend.
//
// Mirrors the bridge conventions of the reference's cuda-fast library
// (src/VHSDecode.CudaFast.Native/src/vhsdecode_cuda_fast.cpp): strict
// struct_size checks (:210-214, :249-254), a thread-local last error (:23-28),
// every exception caught at the boundary (:367-377), cancellation polled
// through a monotonic latch (src/cancellation_latch.h) and the callback.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#define VHSDECODE_GB300_EXPORTS 1
#include "../../include/vhsdecode_gb300.h"
#include "control.hpp"
#include "filters.hpp"
#include "formats.hpp"
#include "kernels.h"
#include "session.hpp"

namespace vhsd {
template <typename T>
cudaError_t launch_tbc_pw(const T*, int64_t, const TbcParams&, const double*, cudaStream_t);
}

using namespace vhsd;
using namespace vhsd::detail;

namespace vhsd {
namespace detail {
thread_local std::string g_last_error;
}  // namespace detail
}  // namespace vhsd

namespace {

bool format_for(uint32_t profile, uint32_t speed, uint32_t tape_format, FormatParams& f) {
    if (speed != VHSDECODE_GB300_TAPE_SPEED_SP && speed != VHSDECODE_GB300_TAPE_SPEED_LP &&
        speed != VHSDECODE_GB300_TAPE_SPEED_EP)
        return false;
    const bool pal = profile == VHSDECODE_GB300_PROFILE_PAL, ntsc = profile == VHSDECODE_GB300_PROFILE_NTSC;
    if (!pal && !ntsc) return false;
    if (tape_format == VHSDECODE_GB300_TAPE_FORMAT_VHS) { f = vhs_format(pal, (int)speed); return true; }
    if (tape_format == VHSDECODE_GB300_TAPE_FORMAT_SVHS) { f = pal ? pal_svhs_sp() : ntsc_svhs_sp(); return true; }
    return false;
}

// Kaiser-windowed sinc LUT, TbcLineResampler.BuildKaiserSincLookup (Core/Tbc/TbcLineResampler.cs:1297-1330).
double bessel_i0(double x) {
    double sum = 1.0, y = (x * x) / 4.0, term = 1.0;
    for (int k = 1; k < 100; k++) {
        term *= y / ((double)k * (double)k);
        double next = sum + term;
        if (next == sum) break;
        sum = next;
    }
    return sum;
}
std::vector<float> build_sinc_lut() {
    const int taps = 16, phases = 65536, half = 8;
    const double beta = 5.0, pi = 3.14159265358979323846;
    std::vector<float> lut((size_t)(phases + 1) * taps);
    double i0b = bessel_i0(beta);
    double w[16];
    for (int p = 0; p < phases; p++) {
        double phase = (double)p / phases, sum = 0.0;
        for (int t = 0; t < taps; t++) {
            double x = (double)((half - 1) - t) + phase;
            double s = x == 0.0 ? 1.0 : std::sin(pi * x) / (pi * x);
            double r = x / half;
            double kw = (r < -1.0 || r > 1.0) ? 0.0 : bessel_i0(beta * std::sqrt(1.0 - r * r)) / i0b;
            w[t] = s * kw;
            sum += w[t];
        }
        for (int t = 0; t < taps; t++) lut[(size_t)p * taps + t] = (float)(w[t] / sum);
    }
    for (int t = 0; t < taps; t++) lut[(size_t)phases * taps + t] = lut[(size_t)(phases - 1) * taps + t];
    return lut;
}

}  // namespace

namespace vhsd {
namespace detail {

int64_t read_length(const SyncParams& sp) {
    int64_t line = (int64_t)std::nearbyint(sp.line_period_us * sp.mhz);
    int64_t base = sp.pal ? line * 400 : (line * 350 / 16384) * 16384;
    return (base / kBlock + 2) * kBlock;
}

void resolve_span(int64_t intended, int64_t read_len, int64_t& s0, int64_t& slen) {
    int64_t rl = std::max<int64_t>(0, intended - kCut);
    int64_t a0 = (rl / kBlock) * kBlock;
    int64_t a1 = a0 + read_len;
    int64_t first = a0 / kStride, last = a1 / kStride;
    s0 = first * kStride;
    slen = (last - first + 1) * kStride;
}

FastDemodParams fp32_params(vhsdecode_gb300_session* s, const int16_t* rf_dev);
int tuned_fft_plan(vhsdecode_gb300_session* s, FastDemodParams base);

void session_init(vhsdecode_gb300_session* s, const vhsdecode_gb300_session_config_v1& c) {
    if (!format_for(c.profile, c.tape_speed, c.tape_format, s->fmt))
        throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT,
                      "unsupported profile / tape speed / tape format (PAL or NTSC; SP, LP or EP; VHS or SVHS)");
    if (!(c.sample_rate_mhz >= 10.0 && c.sample_rate_mhz <= 100.0))
        throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "sample_rate_mhz must be within 10..100");
    if (c.precision > 1) throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "unknown precision");
    if (c.decimation > 2) throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "decimation must be 0, 1 or 2");
    s->decim = c.decimation == 2 ? 2 : 1;
    s->fs = c.sample_rate_mhz * 1e6;
    s->precision = (int)c.precision;
    s->device = c.device_id;
    s->max_samples = c.max_samples;
    s->sp = SyncParams::make(s->fmt, s->fs);
    try {
        s->filt = design_filters(s->fmt, s->fs);
    } catch (const std::runtime_error& e) {
        throw Failure(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, e.what());
    }
    s->lines = s->sp.output_lines + 10;
    s->out_lines = s->sp.output_lines;
    s->outlen = s->fmt.outlinelen;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        throw Failure(VHSDECODE_GB300_STATUS_CUDA_UNAVAILABLE, "no CUDA device available");
    if (c.device_id < 0 || c.device_id >= ndev)
        throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "device_id out of range");
    ck(cudaSetDevice(c.device_id), "cudaSetDevice");
    cudaDeviceProp prop{};
    ck(cudaGetDeviceProperties(&prop, c.device_id), "cudaGetDeviceProperties");
    s->num_sms = prop.multiProcessorCount;
    ck(cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    ck(cudaStreamCreateWithFlags(&s->aux_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    ck(cudaStreamCreateWithFlags(&s->field_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    ck(cudaEventCreateWithFlags(&s->field_end, cudaEventDisableTiming), "cudaEventCreate");
    ck(cudaStreamCreateWithFlags(&s->drop_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    for (cudaEvent_t* e : {&s->drop_fork, &s->drop_hsync, &s->drop_join})
        ck(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "cudaEventCreate");
    for (auto& e : s->stage_ev) ck(cudaEventCreate(&e), "cudaEventCreate");
    s->stage_timing = std::getenv("VHSD_STAGE_TIMING") != nullptr;
    if (std::getenv("VHSD_DEMOD_TIMING")) {
        ck(cudaMalloc(&s->demod_cycles, 2 * kDemodStages * sizeof(unsigned long long)), "cudaMalloc");
        ck(cudaMemset(s->demod_cycles, 0, 2 * kDemodStages * sizeof(unsigned long long)), "memset");
    }
    s->stream = s->own_stream;
    for (auto& ev : s->ev) ck(cudaEventCreate(&ev), "cudaEventCreate");
    s->max_blocks = block_count(c.max_samples / (uint64_t)s->decim);
    int64_t stream_cap = std::max<int64_t>(1, s->max_blocks) * kStride;
    double field_samples = s->fs / (2.0 * s->fmt.fps);
    s->max_fields = c.max_fields ? (int)c.max_fields
                                 : (int)(stream_cap / field_samples) + 4;
    s->rf.alloc(std::max<uint64_t>(c.max_samples, 16) + 8);
    const int H = kHalf;
    if (s->fp32()) {
        s->v32.alloc(stream_cap); s->s32.alloc(stream_cap); s->e32.alloc(stream_cap);
        s->sync_cond.alloc((size_t)stream_cap / 32 + 1);
        s->sync_hold.alloc((size_t)stream_cap / 32 + 1);
        std::vector<float> rv(H);
        std::vector<float2> vv(H), sv(H);
        for (int k = 0; k < H; k++) {
            rv[k] = (float)s->filt.rf_video[k];
            vv[k] = make_float2((float)s->filt.video[k].real(), (float)s->filt.video[k].imag());
            sv[k] = make_float2((float)s->filt.sync[k].real(), (float)s->filt.sync[k].imag());
        }
        s->rfv32.alloc(H); s->vid32.alloc(H); s->syn32.alloc(H);
        ck(cudaMemcpy(s->rfv32.p, rv.data(), H * sizeof(float), cudaMemcpyHostToDevice), "upload");
        ck(cudaMemcpy(s->vid32.p, vv.data(), H * sizeof(float2), cudaMemcpyHostToDevice), "upload");
        ck(cudaMemcpy(s->syn32.p, sv.data(), H * sizeof(float2), cudaMemcpyHostToDevice), "upload");
        if (!s->filt.sub_high.empty()) {
            std::vector<float2> hv(H);
            for (int k = 0; k < H; k++)
                hv[k] = make_float2((float)s->filt.sub_high[k].real(), (float)s->filt.sub_high[k].imag());
            s->sub32.alloc(H);
            ck(cudaMemcpy(s->sub32.p, hv.data(), H * sizeof(float2), cudaMemcpyHostToDevice), "upload");
        }
        std::vector<float2> hi(256), lo(128);
        const double pi = 3.14159265358979323846;
        for (int h = 0; h < 256; h++) {
            double a = -2.0 * pi * (h * 128.0) / 32768.0;
            hi[h] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
        for (int l = 0; l < 128; l++) {
            double a = -2.0 * pi * l / 32768.0;
            lo[l] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
        s->tw_hi.alloc(256); s->tw_lo.alloc(128);
        ck(cudaMemcpy(s->tw_hi.p, hi.data(), 256 * sizeof(float2), cudaMemcpyHostToDevice), "upload");
        ck(cudaMemcpy(s->tw_lo.p, lo.data(), 128 * sizeof(float2), cudaMemcpyHostToDevice), "upload");
        int clusters = s->num_sms / 2;
        // two halves: segments on the two compute streams may run at once
        s->scratch.alloc((size_t)2 * clusters * 2 * kBlock);
        s->repair.alloc(1);
        s->nseg_max = (int)((std::max<int64_t>(0, s->max_blocks - kFirstSegBlocks) + kSegBlocks - 1) / kSegBlocks) + 1;
        s->seg_cap = kSegBlocks * kStride / 64 + 4096;
        s->seg_events.alloc((size_t)s->nseg_max * s->seg_cap);
        s->pc_counts_alt.alloc(pulse_count_slots(kSegBlocks * kStride));
        s->pc_offsets_alt.alloc(pulse_count_slots(kSegBlocks * kStride));
        s->seg_total.alloc((size_t)s->nseg_max);
        s->blk_counters.alloc((size_t)s->nseg_max + 1);   // one per segment launch, the last for run_demod
        ck(cudaHostAlloc((void**)&s->h_events, (size_t)s->nseg_max * s->seg_cap * sizeof(int64_t),
                         cudaHostAllocDefault), "cudaHostAlloc");
        ck(cudaHostAlloc((void**)&s->h_totals, (size_t)s->nseg_max * sizeof(int64_t), cudaHostAllocDefault),
           "cudaHostAlloc");
        s->seg_done.resize((size_t)s->nseg_max);
        s->seg_copied.resize((size_t)s->nseg_max);
        s->seg_pulsed.resize((size_t)s->nseg_max);
        s->seg_dem.resize((size_t)s->nseg_max * 2);
        s->seg_demod_end.resize((size_t)s->nseg_max);
        for (auto& e : s->seg_demod_end) ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
        for (auto& e : s->seg_done) ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
        for (auto& e : s->seg_copied) ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
        for (auto& e : s->seg_pulsed) ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
        for (auto& e : s->seg_dem) ck(cudaEventCreate(&e), "cudaEventCreate");
        ck(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking), "cudaStreamCreate");
        ck(cudaStreamCreateWithFlags(&s->d2h_stream, cudaStreamNonBlocking), "cudaStreamCreate");
        ck(cudaStreamCreateWithFlags(&s->alt_stream, cudaStreamNonBlocking), "cudaStreamCreate");
        ck(cudaEventCreateWithFlags(&s->alt_start, cudaEventDisableTiming), "cudaEventCreate");
        ck(cudaEventCreateWithFlags(&s->alt_end, cudaEventDisableTiming), "cudaEventCreate");
        ck(cudaEventCreateWithFlags(&s->copy_end, cudaEventDisableTiming), "cudaEventCreate");
        ck(cudaEventCreateWithFlags(&s->d2h_end, cudaEventDisableTiming), "cudaEventCreate");
        ck(cudaStreamCreateWithFlags(&s->cap_stream, cudaStreamNonBlocking), "cudaStreamCreate");
        s->fft_plan = tuned_fft_plan(s, fp32_params(s, nullptr));
    } else {
        s->v64.alloc(stream_cap); s->s64.alloc(stream_cap); s->e64.alloc(stream_cap);
        std::vector<double2> vv(H), sv(H);
        for (int k = 0; k < H; k++) {
            vv[k] = make_double2(s->filt.video[k].real(), s->filt.video[k].imag());
            sv[k] = make_double2(s->filt.sync[k].real(), s->filt.sync[k].imag());
        }
        s->rfv64.alloc(H); s->vid64.alloc(H); s->syn64.alloc(H);
        ck(cudaMemcpy(s->rfv64.p, s->filt.rf_video.data(), H * sizeof(double), cudaMemcpyHostToDevice), "upload");
        ck(cudaMemcpy(s->vid64.p, vv.data(), H * sizeof(double2), cudaMemcpyHostToDevice), "upload");
        ck(cudaMemcpy(s->syn64.p, sv.data(), H * sizeof(double2), cudaMemcpyHostToDevice), "upload");
        if (!s->filt.sub_high.empty()) {
            std::vector<double2> hv(H);
            for (int k = 0; k < H; k++)
                hv[k] = make_double2(s->filt.sub_high[k].real(), s->filt.sub_high[k].imag());
            s->sub64.alloc(H);
            ck(cudaMemcpy(s->sub64.p, hv.data(), H * sizeof(double2), cudaMemcpyHostToDevice), "upload");
        }
        s->pwork.alloc(4 * (size_t)kBlock);
        s->pdwork.alloc(3 * (size_t)kBlock);
        s->pfwork.alloc(kBlock + 16);
        s->pflag.alloc(4);
        s->pmask.alloc(1024);
        s->pblk.alloc(1);
        ck(cudaMemset(s->pflag.p, 0, 4 * sizeof(int)), "memset");
    }
    int64_t pslots = pulse_count_slots(stream_cap);
    s->pc_counts.alloc(pslots);
    s->pc_offsets.alloc(pslots);
    s->pc_capacity = stream_cap / 64 + 4096;
    s->pc_events.alloc(s->pc_capacity);
    s->pc_total.alloc(1);
    size_t fl = (size_t)s->max_fields * s->lines;
    {
        // per-field inputs: locs (double), spans (int64 x 2), line indices
        // (int x 4), fill flags (uint8), each array 8-byte aligned
        const size_t mf = (size_t)s->max_fields;
        const size_t o_locs = 0, o_ss = o_locs + fl * 8, o_sl = o_ss + mf * 8, o_fl = o_sl + mf * 8;
        const size_t a4 = (mf * 4 + 7) & ~(size_t)7;
        const size_t o_st = o_fl + a4, o_el = o_st + a4, o_lo = o_el + a4;
        const size_t o_ff = o_lo + a4, o_fn = o_ff + a4, o_rot = o_fn + a4, o_fill = o_rot + 8;
        s->field_in_bytes = o_fill + ((fl + 7) & ~(size_t)7);
        s->field_in.alloc(s->field_in_bytes);
        ck(cudaHostAlloc((void**)&s->h_field_in, s->field_in_bytes, cudaHostAllocDefault), "cudaHostAlloc");
        unsigned char* b = s->field_in.p;
        s->locs_in.p = reinterpret_cast<double*>(b + o_locs);
        s->span_start_d.p = reinterpret_cast<int64_t*>(b + o_ss);
        s->span_len_d.p = reinterpret_cast<int64_t*>(b + o_sl);
        s->first_line_d.p = reinterpret_cast<int*>(b + o_fl);
        s->start_line_d.p = reinterpret_cast<int*>(b + o_st);
        s->end_line_d.p = reinterpret_cast<int*>(b + o_el);
        s->line_off_d.p = reinterpret_cast<int*>(b + o_lo);
        s->first_field_d.p = reinterpret_cast<int*>(b + o_ff);
        s->field_number_d.p = reinterpret_cast<int*>(b + o_fn);
        s->rot_in_d.p = reinterpret_cast<int*>(b + o_rot);
        s->fill_in.p = b + o_fill;
        // results: refined lines, dropout counts and status, early dropout
        // triplets, then the chroma rotation index and status
        const size_t out_bytes = fl * 8 + mf * 8 + mf * (size_t)kDropEarly * 3 * 4 + 16;
        ck(cudaHostAlloc((void**)&s->h_field_out, out_bytes, cudaHostAllocDefault), "cudaHostAlloc");
    }
    s->locs_out.alloc(fl);
    s->fill_out.alloc(fl);
    s->hsync_work.alloc(hsync_work_bytes(s->max_fields, s->lines));
    s->hsync_misses.alloc(1);
    static const std::vector<float> lut = build_sinc_lut();   // built once per process
    s->lut.alloc(lut.size());
    ck(cudaMemcpy(s->lut.p, lut.data(), lut.size() * sizeof(float), cudaMemcpyHostToDevice), "upload");
    {
        // rows p and p+1 side by side: one 128-byte line per interpolated tap set
        std::vector<float> pair((size_t)65536 * 32);
        for (size_t r = 0; r < 65536; r++)
            for (int t = 0; t < 16; t++) {
                pair[r * 32 + t] = lut[r * 16 + t];
                pair[r * 32 + 16 + t] = lut[(r + 1) * 16 + t];
            }
        s->lut_pair.alloc(pair.size());
        ck(cudaMemcpy(s->lut_pair.p, pair.data(), pair.size() * sizeof(float), cudaMemcpyHostToDevice),
           "upload");
    }
    double smoothing = s->fmt.frame_lines / 2.0;
    double alpha = 1.0 / (smoothing * s->outlen);
    std::vector<double> pw((size_t)s->outlen);
    for (int k = 0; k < s->outlen; k++) pw[(size_t)k] = std::pow(1.0 - alpha, (double)(k + 1));
    s->pw.alloc(pw.size());
    ck(cudaMemcpy(s->pw.p, pw.data(), pw.size() * sizeof(double), cudaMemcpyHostToDevice), "upload");
    std::vector<float2> pwf(pw.size());
    for (size_t k = 0; k < pw.size(); k++) {
        float hi = (float)pw[k];
        pwf[k] = make_float2(hi, (float)(pw[k] - (double)hi));
    }
    s->pw_ff.alloc(pwf.size());
    ck(cudaMemcpy(s->pw_ff.p, pwf.data(), pwf.size() * sizeof(float2), cudaMemcpyHostToDevice), "upload");
    s->level_work.alloc((size_t)s->max_fields * 1024);
    s->tbc_consts.alloc((size_t)s->max_fields * s->out_lines * kTbcLineConstsBytes);
    s->tbc.alloc((size_t)s->max_fields * s->out_lines * s->outlen);
    s->span_len = read_length(s->sp) + 2 * kStride;  // upper bound of a resolved span
    int nch = dropout_chunks(s->span_len);
    s->drop_range.alloc((size_t)s->max_fields * 2);
    s->drop_mean.alloc(s->max_fields);
    s->drop_partial.alloc((size_t)s->max_fields * nch);
    s->drop_counts.alloc((size_t)s->max_fields * nch);
    s->drop_events.alloc((size_t)s->max_fields * nch * s->drop_cap);
    s->drop_out.alloc((size_t)s->max_fields * s->drop_out_cap * 3);
    s->drop_out_count.alloc(s->max_fields);
    s->drop_status.alloc(s->max_fields);
}

// Chroma tables and buffers, made by the first decode that renders chroma.
void ensure_chroma(vhsdecode_gb300_session* s) {
    if (s->chroma_alloc) return;
    ck(prepare_chroma_kernels(), "chroma kernel attributes");
    s->cd = vhsd::design_chroma(s->fmt, s->fs);
    const vhsd::ChromaDesign& d = s->cd;
    if (2 * d.burst_start - d.burst_end < 0 || d.burst_start + d.burst_end > d.outlen ||
        d.out_lines != s->out_lines || d.outlen != s->outlen)
        throw Failure(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, "chroma burst window does not fit the line");
    if (d.rf.edge != kChromaEdge)
        throw Failure(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, "chroma band-pass pad length is not the block stage's");
    const size_t mf = (size_t)s->max_fields, field = (size_t)d.field_samples;
    const size_t win = (size_t)(2 * d.burst_end - d.burst_start);
    s->c32.alloc((size_t)std::max<int64_t>(1, s->max_blocks) * kStride);
    s->c_scratch.alloc((size_t)std::max<int64_t>(1, s->max_blocks) * kChromaRowStride);
    // Host fault injection, the counterpart of the reference build's forced
    // chroma-workspace failure (CUVHS_FORCE_CHROMA_WORKSPACE_FAILURE,
    // tools/build-cuda-fast-native.ps1:290-305): the workspace allocation
    // fails partway, and the decode must fail rather than report chroma it
    // never wrote.  A later call allocates the workspace afresh.
    if (const char* f = std::getenv("VHSD_FORCE_CHROMA_WORKSPACE_FAILURE"); f && *f && std::strcmp(f, "0") != 0)
        throw Failure(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, "chroma workspace cudaMalloc: out of memory (forced)");
    std::vector<float> het, bsin, bcos;
    vhsd::chroma_tables(d, het, bsin, bcos);
    s->c_het.alloc(het.size());
    s->c_bsin.alloc(bsin.size());
    s->c_bcos.alloc(bcos.size());
    ck(cudaMemcpy(s->c_het.p, het.data(), het.size() * sizeof(float), cudaMemcpyHostToDevice), "upload");
    ck(cudaMemcpy(s->c_bsin.p, bsin.data(), bsin.size() * sizeof(float), cudaMemcpyHostToDevice), "upload");
    ck(cudaMemcpy(s->c_bcos.p, bcos.data(), bcos.size() * sizeof(float), cudaMemcpyHostToDevice), "upload");
    s->c_ana.alloc(mf * s->out_lines * win);
    s->c_field.alloc(mf * field);
    const size_t crow = (size_t)chroma_final_row((int64_t)field, d.fin.edge);
    s->c_up.alloc(mf * crow);
    s->c_fwd.alloc(mf * crow);
    s->c_probe.alloc(mf * 2 * s->out_lines * 5);
    s->c_probe_nrm.alloc(mf * 2 * s->out_lines * 2);
    s->c_summary.alloc(mf * 4);
    s->locs_final.alloc(mf * s->lines);
    s->c_flip.alloc(mf * 2);
    s->c_chosen.alloc(mf);
    s->c_state.alloc(4);
    s->c_ones.alloc(mf);
    std::vector<int> ones(mf, 1);
    ck(cudaMemcpy(s->c_ones.p, ones.data(), mf * sizeof(int), cudaMemcpyHostToDevice), "upload");
    s->chroma.alloc(mf * field);
    s->c_line_cs.alloc(mf * s->out_lines);
    s->c_line_scale.alloc(mf * s->out_lines);
    s->c_line_scale_f.alloc(mf * s->out_lines);
    {
        // NTSC up-conversion: the phase advance of sample k of a line as the
        // reference's four lanes step theta (UpconvertChromaPhaseCompensated,
        // VhsChromaDecoder.cs:2182-2246), reduced by whole turns, as its
        // (cos, sin)
        const double h = ((d.cu_hz * 1.5707963267948965e-6) / d.fsc_mhz) + 1.5707963267948966;
        const double two_pi = 6.283185307179586, inv = 0.15915494309189535;
        const int vc = d.outlen & ~3;
        const double lane[4] = {h * 0.0, h, h * 2.0, h * 3.0};
        std::vector<float2> adv((size_t)d.outlen);
        for (int k = 0; k < d.outlen; k++) {
            double off = k < vc ? std::fma((double)(k >> 2), h * 4.0, lane[k & 3])
                                : std::fma((double)(k - vc), h, h * (double)vc);
            const double a = std::fma(-std::nearbyint(off * inv), two_pi, off);
            adv[(size_t)k] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
        s->c_advance.alloc(adv.size());
        ck(cudaMemcpy(s->c_advance.p, adv.data(), adv.size() * sizeof(float2), cudaMemcpyHostToDevice), "upload");
    }
    ck(cudaEventCreateWithFlags(&s->chroma_refined, cudaEventDisableTiming), "cudaEventCreate");
    // the block stage's stream has the highest priority: its CTAs take the
    // first SMs that a finishing demod segment frees, ahead of the next
    // segment's queued clusters
    int least = 0, greatest = 0;
    ck(cudaDeviceGetStreamPriorityRange(&least, &greatest), "cudaDeviceGetStreamPriorityRange");
    ck(cudaStreamCreateWithPriority(&s->chroma_stream, cudaStreamNonBlocking, greatest), "cudaStreamCreate");
    ck(cudaEventCreateWithFlags(&s->chroma_go, cudaEventDisableTiming), "cudaEventCreate");
    ck(cudaEventCreateWithFlags(&s->chroma_done, cudaEventDisableTiming), "cudaEventCreate");
    for (auto& e : s->chroma_t) ck(cudaEventCreate(&e), "cudaEventCreate");
    s->chroma_alloc = true;
}

// The chroma channel of blocks [b0, b1) on stream `st` (the capture must be on
// the device: rf16 or the session's float capture).
void launch_chroma_blocks_for(vhsdecode_gb300_session* s, const int16_t* rf16, int64_t nblocks, cudaStream_t st) {
    ChromaBlockParams cb{};
    cb.rf16 = s->in_f32 ? nullptr : rf16;
    cb.rf32 = s->in_f32;
    cb.first_block = 0;
    cb.nblocks = nblocks;
    std::memcpy(cb.c.sec, s->cd.rf.sec, sizeof(cb.c.sec));
    std::memcpy(cb.c.zi, s->cd.rf.zi, sizeof(cb.c.zi));
    cb.c.edge = s->cd.rf.edge;
    cb.move = s->cd.move;
    cb.scratch = s->c_scratch.p;
    cb.out = s->c32.p;
    ck(launch_chroma_blocks(cb, st), "chroma block launch");
    s->launches += kChromaBlockKernels;
}

// The chroma block band-pass of the whole capture on the chroma stream, after
// `after` (the point where the capture is on the device); the field batch
// waits for chroma_done.  The kernel needs few SMs and is latency-bound, so it
// runs beside the demodulator instead of after it.
void queue_chroma_blocks(vhsdecode_gb300_session* s, const int16_t* rf16, int64_t nblocks, cudaEvent_t after) {
    ck(cudaStreamWaitEvent(s->chroma_stream, after, 0), "wait");
    if (s->stage_timing) ck(cudaEventRecord(s->chroma_t[0], s->chroma_stream), "event");
    launch_chroma_blocks_for(s, rf16, nblocks, s->chroma_stream);
    if (s->stage_timing) ck(cudaEventRecord(s->chroma_t[1], s->chroma_stream), "event");
    ck(cudaEventRecord(s->chroma_done, s->chroma_stream), "event");
    s->chroma_pending = true;
}

void session_free(vhsdecode_gb300_session* s) {
    if (s->chroma_refined) cudaEventDestroy(s->chroma_refined);
    if (s->chroma_go) cudaEventDestroy(s->chroma_go);
    if (s->chroma_done) cudaEventDestroy(s->chroma_done);
    for (auto& e : s->chroma_t)
        if (e) cudaEventDestroy(e);
    if (s->chroma_stream) cudaStreamDestroy(s->chroma_stream);
    if (s->demod_cycles) cudaFree(s->demod_cycles);
    if (s->plain_graph) cudaGraphExecDestroy(s->plain_graph);
    for (auto& ev : s->ev) if (ev) cudaEventDestroy(ev);
    for (auto* v : {&s->seg_done, &s->seg_copied, &s->seg_pulsed, &s->seg_dem, &s->seg_demod_end})
        for (auto& ev : *v) if (ev) cudaEventDestroy(ev);
    if (s->h_events) cudaFreeHost(s->h_events);
    if (s->h_field_in) cudaFreeHost(s->h_field_in);
    if (s->h_field_out) cudaFreeHost(s->h_field_out);
    if (s->h_totals) cudaFreeHost(s->h_totals);
    if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
    if (s->d2h_stream) cudaStreamDestroy(s->d2h_stream);
    if (s->alt_stream) cudaStreamDestroy(s->alt_stream);
    if (s->alt_start) cudaEventDestroy(s->alt_start);
    if (s->alt_end) cudaEventDestroy(s->alt_end);
    if (s->copy_end) cudaEventDestroy(s->copy_end);
    if (s->d2h_end) cudaEventDestroy(s->d2h_end);
    if (s->pipe_exec) cudaGraphExecDestroy(s->pipe_exec);
    if (s->cap_stream) cudaStreamDestroy(s->cap_stream);
    if (s->aux_stream) cudaStreamDestroy(s->aux_stream);
    if (s->field_stream) cudaStreamDestroy(s->field_stream);
    if (s->field_end) cudaEventDestroy(s->field_end);
    if (s->drop_stream) cudaStreamDestroy(s->drop_stream);
    for (cudaEvent_t e : {s->drop_fork, s->drop_hsync, s->drop_join})
        if (e) cudaEventDestroy(e);
    for (auto& e : s->stage_ev) if (e) cudaEventDestroy(e);
    if (s->own_stream) cudaStreamDestroy(s->own_stream);
}

template <typename T, typename T2>
SubDeemphT<T, T2> sub_params(const FormatParams& f, const FilterSpectra& filt) {
    SubDeemphT<T, T2> d{};
    d.inv_half_dev = (T)(1.0 / (f.sub_deviation / 2.0));
    d.b0 = (T)filt.sub_b0;
    d.b1 = (T)filt.sub_b1;
    d.a1 = (T)filt.sub_a1;
    d.exponent = (T)f.sub_exp;
    d.scale1 = std::isnan(f.sub_scale1) ? (T)1 : (T)f.sub_scale1;
    d.scale2 = std::isnan(f.sub_scale2) ? (T)1 : (T)f.sub_scale2;
    d.logistic_mid = std::isnan(f.sub_logistic_mid) ? (T)0 : (T)f.sub_logistic_mid;
    d.logistic_rate = std::isnan(f.sub_logistic_rate) ? (T)0 : (T)f.sub_logistic_rate;
    d.static_factor = (T)f.sub_static;
    return d;
}

// FFT radix plan autotuner.  The fused demodulator is compiled for the
// kFftPlans radix plans of its 8192- and 16384-point transforms (same results
// up to float rounding).  The first FP32 session on a device times each on a
// synthetic FM carrier block set (four launches of 4 blocks per cluster each,
// after one warm-up) and keeps the fastest for the process; plan 0 is kept
// unless another is at least 2 % faster, so that outputs do not flip between
// runs on timing noise.  VHSD_FFT_PLAN=<n> fixes the plan (one of kFftPlans)
// and VHSD_TUNE_LOG=1 prints the timings.  Must run outside stream capture
// (session creation is).
int tuned_fft_plan(vhsdecode_gb300_session* s, FastDemodParams base) {
    static std::mutex m;
    static int plans[64];
    static bool done[64] = {};
    if (const char* env = std::getenv("VHSD_FFT_PLAN")) {
        int v = std::atoi(env);
        for (int plan : kFftPlans)
            if (plan == v) return v;
    }
    std::lock_guard<std::mutex> lk(m);
    const int dev = s->device;
    if (dev >= 0 && dev < 64 && done[dev]) return plans[dev];
    const int clusters = s->num_sms / 2;
    const int64_t nb = 4 * (int64_t)clusters;
    const int64_t n = nb * kStride + (kBlock - kStride);
    std::vector<int16_t> host((size_t)n);
    const double f = s->fmt.ire0 + 50.0 * s->fmt.hz_ire;
    uint32_t lcg = 12345u;
    double ph = 0.0;
    for (int64_t i = 0; i < n; i++) {
        lcg = lcg * 1664525u + 1013904223u;
        ph += 2.0 * 3.14159265358979323846 * (f + 300000.0 * std::sin(i * 1e-4)) / s->fs;
        host[(size_t)i] = (int16_t)std::lrint(8000.0 * std::cos(ph) + (double)((lcg >> 24) & 63) - 32.0);
    }
    DevBuf<int16_t> rf;
    DevBuf<float> v, y, e;
    rf.alloc((size_t)n + 8);
    v.alloc((size_t)nb * kStride);
    y.alloc((size_t)nb * kStride);
    e.alloc((size_t)nb * kStride);
    ck(cudaMemcpy(rf.p, host.data(), (size_t)n * sizeof(int16_t), cudaMemcpyHostToDevice), "tune upload");
    cudaStream_t st;
    ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    cudaEvent_t e0, e1;
    ck(cudaEventCreate(&e0), "cudaEventCreate");
    ck(cudaEventCreate(&e1), "cudaEventCreate");
    FastDemodParams p = base;
    p.rf = rf.p;
    p.rf_f32 = nullptr;
    p.first_block = 0;
    p.nblocks = nb;
    p.sync_cond = nullptr;   // the tuning blocks are not the session's stream
    p.sync_hold = nullptr;
    p.video_out = v.p;
    p.sync_out = y.p;
    p.env_out = e.p;
    const bool log = std::getenv("VHSD_TUNE_LOG") != nullptr;
    int best = 0;
    float best_ms = 0.0f, plan0_ms = 0.0f;
    for (int plan : kFftPlans) {
        p.fft_plan = plan;
        const int a = plan & 3, b = (plan >> 2) & 3;
        ck(launch_demod_fp32(p, clusters, st), "tune launch");
        ck(cudaEventRecord(e0, st), "event");
        for (int r = 0; r < 4; r++) ck(launch_demod_fp32(p, clusters, st), "tune launch");
        ck(cudaEventRecord(e1, st), "event");
        ck(cudaEventSynchronize(e1), "event sync");
        float ms = 0.0f;
        ck(cudaEventElapsedTime(&ms, e0, e1), "event time");
        if (log) std::fprintf(stderr, "vhsd fft plan %d (8192:%d 16384:%d): %.4f ms\n", p.fft_plan, a, b, ms / 4);
        if (p.fft_plan == 0) plan0_ms = ms;
        if (p.fft_plan == 0 || ms < best_ms) { best = p.fft_plan; best_ms = ms; }
    }
    if (best != 0 && best_ms > 0.98f * plan0_ms) best = 0;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    if (log) std::fprintf(stderr, "vhsd fft plan chosen: %d\n", best);
    if (dev >= 0 && dev < 64) { plans[dev] = best; done[dev] = true; }
    return best;
}

// The fused demodulator, or (VHSD_DEMOD_TIMING set) its timed diagnostic build.
cudaError_t launch_fused(vhsdecode_gb300_session* s, FastDemodParams p, cudaStream_t st) {
    const int clusters = s->demod_clusters > 0 ? s->demod_clusters : s->num_sms / 2;
    if (!s->demod_cycles) return launch_demod_fp32(p, clusters, st);
    p.stage_cycles = s->demod_cycles;
    return launch_demod_fp32_timed(p, clusters, st);
}

FastDemodParams fp32_params(vhsdecode_gb300_session* s, const int16_t* rf_dev) {
    FastDemodParams p{};
    p.rf = rf_dev;
    p.first_block = 0;
    p.nblocks = 0;
    p.rf_video = s->rfv32.p;
    p.video = s->vid32.p;
    p.sync = s->syn32.p;
    p.tw_hi = s->tw_hi.p;
    p.tw_lo = s->tw_lo.p;
    p.fs = (float)s->fs;
    p.diff_max = (float)((s->fmt.ire0 + s->fmt.hz_ire * 100.0) * 2.0);
    p.dc = (float)s->fmt.ire0;
    // the DC gain of Video is not exactly 1 for S-VHS (its measured luma table
    // starts at 1.0000019): 5.88 MHz x 1.9e-6 would be an 11 Hz offset
    p.dc_video = (float)((double)p.dc * s->filt.video[0].real());
    p.dc_sync = (float)((double)p.dc * s->filt.sync[0].real());
    p.env_b0 = (float)s->filt.env_b0;
    p.env_b1 = (float)s->filt.env_b1;
    p.env_a1 = (float)s->filt.env_a1;
    p.video_out = s->v32.p;
    p.sync_out = s->s32.p;
    p.env_out = s->e32.p;
    p.scratch = s->scratch.p;
    p.repair_count = s->repair.p;
    if (s->sub32.p) {
        p.sub = sub_params<float, float2>(s->fmt, s->filt);
        p.sub.high = s->sub32.p;
    }
    p.fft_plan = s->fft_plan;
    p.rf_f32 = s->in_f32;
    if (s->in_f32) p.rf = nullptr;
    p.block_counter = nullptr;
    p.sync_cond = s->sync_cond.p;
    p.sync_hold = s->sync_hold.p;
    p.sync_thr = pulse_float_threshold(s->sp.ire_to_hz(s->sp.vsync_ire / 2.0));
    return p;
}

void run_demod(vhsdecode_gb300_session* s, const int16_t* rf_dev, int64_t nblocks) {
    if (nblocks <= 0) return;
    if (s->fp32()) {
        FastDemodParams p = fp32_params(s, rf_dev);
        p.nblocks = nblocks;
        p.block_counter = s->blk_counters.p + s->nseg_max;
        ck(cudaMemsetAsync(p.block_counter, 0, sizeof(unsigned), s->stream), "memset");
        ck(cudaMemsetAsync(s->repair.p, 0, sizeof(int), s->stream), "memset");
        ck(launch_fused(s, p, s->stream), "demod fp32 launch");
    } else {
        PlainDemodParams p{};
        p.rf = s->in_f32 ? nullptr : rf_dev;
        p.rf_f32 = s->in_f32;
        p.rf_video = s->rfv64.p;
        p.video = s->vid64.p;
        p.sync = s->syn64.p;
        p.fs = s->fs;
        p.diff_max = (s->fmt.ire0 + s->fmt.hz_ire * 100.0) * 2.0;
        p.env_b0 = s->filt.env_b0;
        p.env_b1 = s->filt.env_b1;
        p.env_a1 = s->filt.env_a1;
        p.video_out = s->v64.p;
        p.sync_out = s->s64.p;
        p.env_out = s->e64.p;
        p.work = s->pwork.p;
        p.dwork = s->pdwork.p;
        p.fwork = s->pfwork.p;
        p.flag = s->pflag.p;
        p.mask = s->pmask.p;
        p.blk = s->pblk.p;
        if (s->sub64.p) {
            p.sub = sub_params<double, double2>(s->fmt, s->filt);
            p.sub.high = s->sub64.p;
        }
        // The capture lives in s->rf or a caller buffer; the graph bakes the
        // pointer, so rebuild it when the input pointer changes.
        if (!s->plain_graph || s->graph_rf != p.rf || s->graph_rf32 != p.rf_f32) {
            if (s->plain_graph) { cudaGraphExecDestroy(s->plain_graph); s->plain_graph = nullptr; }
            cudaStream_t cs;
            ck(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "stream");
            cudaGraph_t g;
            ck(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "capture");
            cudaError_t le = launch_demod_fp64_block(p, cs);
            cudaError_t ce = cudaStreamEndCapture(cs, &g);
            cudaStreamDestroy(cs);
            ck(le, "plain launch");
            ck(ce, "end capture");
            ck(cudaGraphInstantiate(&s->plain_graph, g, 0), "graph instantiate");
            cudaGraphDestroy(g);
            s->graph_rf = p.rf;
            s->graph_rf32 = p.rf_f32;
        }
        int64_t zero = 0;
        ck(cudaMemcpyAsync(s->pblk.p, &zero, sizeof(int64_t), cudaMemcpyHostToDevice, s->stream), "blk");
        for (int64_t b = 0; b < nblocks; b++) ck(cudaGraphLaunch(s->plain_graph, s->stream), "graph launch");
    }
}

// Pulse events of the stitched stream in stream order.  upto(pos) returns once
// every event before stream position pos is in `events` (the pipelined decode
// waits there for the segment that finalises pos).
struct EventFeed {
    std::vector<int64_t> events;
    std::function<void(int64_t)> upto;
};

// TbcFieldSequenceDecodeEngine order (Core/Decode/TbcFieldSequenceDecodeEngine.cs:442-560):
// resolve the next field span, take its pulses, run the control plane, step by
// the next-field offset.  The long-hsync rescue reads the sync reference of a
// finished span on the auxiliary stream, so it never waits behind queued work.
template <typename T>
void host_field_loop(vhsdecode_gb300_session* s, const T* sync, int64_t stream_len, uint32_t max_fields,
                     EventFeed& feed, uint32_t& stop_reason, const std::atomic<bool>* cancel,
                     DecodeCarry* carry) {
    const SyncParams& sp = s->sp;
    int64_t read_len = read_length(sp);
    int64_t min_len = std::max<int64_t>(0, (int64_t)std::ceil(sp.usec(sp.eq_us) / 8.0));
    int64_t max_len = std::max<int64_t>(1, (int64_t)(sp.nominal * 5.0));
    FieldState st = carry ? carry->state : FieldState{};
    s->chroma_rot_start = s->chroma_rot_end = st.chroma_rot;
    int64_t intended = carry ? std::max<int64_t>(0, carry->start) : 0;
    s->fields.clear();
    s->rescue_fetches = 0;
    s->recoveries = 0;
    stop_reason = 0;
    std::vector<T> tmp;
    while (true) {
        if (cancel && cancel->load()) throw Failure(VHSDECODE_GB300_STATUS_CANCELLED, "decode cancelled");
        if ((int)s->fields.size() >= s->max_fields) { stop_reason = 1; break; }
        if (max_fields && s->fields.size() >= max_fields) { stop_reason = 1; break; }
        int64_t s0, slen;
        resolve_span(intended, read_len, s0, slen);
        if (s0 + slen > stream_len) break;
        feed.upto(s0 + slen);
        std::vector<Pulse> raw = span_pulses(feed.events.data(), (int64_t)feed.events.size(), s0, slen,
                                             min_len, max_len);
        RefFetch fetch = [&](int64_t start, int64_t len, std::vector<double>& out) {
            tmp.resize((size_t)len);
            ck(cudaMemcpyAsync(tmp.data(), sync + s0 + start, (size_t)len * sizeof(T),
                               cudaMemcpyDeviceToHost, s->aux_stream), "rescue fetch");
            ck(cudaStreamSynchronize(s->aux_stream), "rescue fetch");
            out.assign(tmp.begin(), tmp.end());
            s->rescue_fetches++;
        };
        FieldRec rec;
        // ResolveVhsFieldNumber (TbcFieldDecodePipeline.cs:860-874)
        const int number = st.vhs_number < 0 ? 0 : (s0 > st.vhs_loc ? st.vhs_number + 1 : st.vhs_number);
        rec.sync = analyse_field(sp, raw, slen, st, fetch);
        rec.span_start = s0;
        rec.span_len = slen;
        if (!rec.sync.ok) {
            // the reference engine moves on and tries again (TbcFieldSequenceDecodeEngine.cs:804-847);
            // v0.4.0 restarts the VHS field number after an invalid field
            intended = std::max<int64_t>(0, intended + rec.sync.recover_offset);
            s->recoveries++;
            st.vhs_number = -1;
            st.vhs_loc = -1;
            continue;
        }
        st.vhs_number = number;
        st.vhs_loc = s0;
        rec.field_number = number;
        intended = s0 + std::max<int64_t>(1, (int64_t)round_away(rec.sync.next_offset));
        s->fields.push_back(std::move(rec));
    }
    if (carry) {
        carry->state = st;
        carry->next = intended;
    }
}

// Device field stage for fields [f0, f1) of s->fields: hsync refinement, TBC
// and dropouts, queued on `fs` (every per-field array is offset by f0).  The
// host must already have seen the demod of those fields' spans complete.
template <typename T>
void launch_field_batch(vhsdecode_gb300_session* s, int f0, int f1, const T* video, const T* sync,
                        const T* env, int64_t stream_len, cudaStream_t fs) {
    const SyncParams& sp = s->sp;
    const int nf = f1 - f0;
    if (nf <= 0) return;
    const size_t L = (size_t)s->lines;
    // the pinned mirror of a device view (same offset in the field_in block)
    auto host = [&](auto v) { return reinterpret_cast<decltype(v.p)>(s->h_field_in + ((unsigned char*)v.p - s->field_in.p)); };
    double* locs = host(s->locs_in) + f0 * L;
    uint8_t* fill = host(s->fill_in) + f0 * L;
    int64_t* span = host(s->span_start_d) + f0;
    int64_t* slens = host(s->span_len_d) + f0;
    int* fline = host(s->first_line_d) + f0;
    int* sline = host(s->start_line_d) + f0;
    int* eline = host(s->end_line_d) + f0;
    int* loff = host(s->line_off_d) + f0;
    int* ffirst = host(s->first_field_d) + f0;
    int* fnum = host(s->field_number_d) + f0;
    *host(s->rot_in_d) = s->chroma_rot_start;
    const bool chroma = s->want_chroma;
    for (int i = 0; i < nf; i++) {
        const FieldSync& fsy = s->fields[(size_t)(f0 + i)].sync;
        double* lr = locs + (size_t)i * L;
        uint8_t* fr = fill + (size_t)i * L;
        const size_t nl = std::min(L, fsy.locs.size()), nfl = std::min(L, fsy.filled.size());
        std::copy(fsy.locs.begin(), fsy.locs.begin() + nl, lr);
        std::fill(lr + nl, lr + L, 0.0);
        std::copy(fsy.filled.begin(), fsy.filled.begin() + nfl, fr);
        std::fill(fr + nfl, fr + L, (uint8_t)0);
        span[i] = s->fields[(size_t)(f0 + i)].span_start;
        slens[i] = s->fields[(size_t)(f0 + i)].span_len;
        fline[i] = sp.pal ? (fsy.first_field ? 3 : 4) : 1;
        loff[i] = sp.pal ? (fsy.first_field ? 2 : 3) : 0;
        sline[i] = loff[i] + 1;
        eline[i] = std::min(s->lines - 1, sp.field_lines(fsy.first_field) + sline[i] + 1);
        ffirst[i] = fsy.first_field ? 1 : 0;
        fnum[i] = s->fields[(size_t)(f0 + i)].field_number;
    }
    // with chroma the burst refinement moves the lines the TBC and the dropout
    // mapping read (and the NTSC fsc shift comes after it)
    double* final_locs = chroma ? s->locs_final.p + f0 * L : s->locs_out.p + f0 * L;
    // one asynchronous copy of the whole block from pinned memory (the mirror
    // is not written again before this decode's results are collected)
    ck(cudaMemcpyAsync(s->field_in.p, s->h_field_in, s->field_in_bytes, cudaMemcpyHostToDevice, fs), "h2d");
    const int nch = dropout_chunks(s->span_len);
    DropoutParams dp{};
    dp.nfields = nf;
    dp.span_start = s->span_start_d.p + f0;
    dp.span_len = s->span_len_d.p + f0;
    dp.max_span_len = s->span_len;
    dp.locs = final_locs;
    dp.lines = s->lines;
    dp.start_line = s->start_line_d.p + f0;
    dp.end_line = s->end_line_d.p + f0;
    dp.line_offset = s->line_off_d.p + f0;
    dp.outlen = s->outlen;
    dp.range = s->drop_range.p + 2 * (size_t)f0;
    dp.frac = 0.18f;
    dp.hyst = 1.25;
    dp.merge = 30;
    dp.min_len = 10;
    dp.mean_out = s->drop_mean.p + f0;
    dp.events = s->drop_events.p + (size_t)f0 * nch * s->drop_cap;
    dp.cap = s->drop_cap;
    dp.out = s->drop_out.p + (size_t)f0 * s->drop_out_cap * 3;
    dp.out_cap = s->drop_out_cap;
    dp.out_count = s->drop_out_count.p + f0;
    dp.status = s->drop_status.p + f0;
    // The dropout chain runs beside hsync and TBC on drop_stream: the envelope
    // means need only the spans, the detection waits for the refined lines.
    // (With per-stage timing everything stays on `fs`, in order.)
    const bool timing = s->stage_timing;
    cudaStream_t ds = timing ? fs : s->drop_stream;
    if (!timing) {
        ck(cudaEventRecord(s->drop_fork, fs), "event");
        ck(cudaStreamWaitEvent(ds, s->drop_fork, 0), "wait");
    }
    ck(launch_drop_mean<T>(env, stream_len, dp, s->drop_partial.p + (size_t)f0 * nch, ds), "dropout launch");
    HsyncParams hp{};
    hp.nfields = nf;
    hp.lines = s->lines;
    hp.locs_in = s->locs_in.p + f0 * L;
    hp.filled_in = s->fill_in.p + f0 * L;
    hp.locs_out = s->locs_out.p + f0 * L;
    hp.filled_out = s->fill_out.p + f0 * L;
    hp.span_start = s->span_start_d.p + f0;
    hp.span_len = s->span_len_d.p + f0;
    hp.pal = sp.pal ? 1 : 0;
    hp.threshold = sp.ire_to_hz(sp.vsync_ire / 2.0);
    hp.one_us = std::max(1, (int)sp.mhz);
    hp.normal_hsync = std::max(1, (int)sp.usec(sp.hsync_us));
    hp.mhz32 = (double)(float)sp.mhz;
    hp.ire0 = sp.ire0;
    hp.hz_ire = sp.hz_ire;
    const double ntsc_shift = sp.pal ? 0.0 : ((117.25 / 360.0) / sp.fsc_mhz) * sp.mhz;
    hp.ntsc_shift = chroma ? 0.0 : ntsc_shift;
    hp.work = s->hsync_work.p + hsync_work_bytes(f0, s->lines);
    hp.misses = nullptr;
    if (s->stage_timing) {
        ck(cudaMemsetAsync(s->hsync_misses.p, 0, sizeof(int), fs), "memset");
        hp.misses = s->hsync_misses.p;
    }
    if (timing) ck(cudaEventRecord(s->stage_ev[0], fs), "event");
    ck(launch_hsync_refine<T>(sync, stream_len, hp, fs), "hsync launch");
    s->launches += kHsyncKernels;
    TbcParams tp{};
    tp.nfields = nf;
    tp.lines = s->lines;
    tp.span_start = s->span_start_d.p + f0;
    tp.span_len = s->span_len_d.p + f0;
    tp.out_lines = s->out_lines;
    tp.outlen = s->outlen;
    tp.nominal = std::nearbyint(s->fmt.line_period_us * sp.mhz);
    tp.smoothing = s->fmt.frame_lines / 2.0;
    tp.lut = s->lut.p;
    tp.lut_pair = s->lut_pair.p;
    tp.pw_ff = s->pw_ff.p;
    tp.level_work = s->level_work.p + (size_t)f0 * 1024;
    tp.line_consts = s->tbc_consts.p + (size_t)f0 * s->out_lines * kTbcLineConstsBytes;
    ChromaFieldParams cp{};
    if (chroma) {
        // the line-1 chroma TBC at the probe windows, the burst phase
        // sequences and the burst refinement of the lines (then the NTSC shift)
        const vhsd::ChromaDesign& d = s->cd;
        cp.nfields = nf;
        cp.lines = s->lines;
        cp.locs = s->locs_out.p + f0 * L;
        cp.locs_out = final_locs;
        cp.ntsc_shift = ntsc_shift;
        cp.ntsc = d.ntsc ? 1 : 0;
        cp.out_lines = s->out_lines;
        cp.outlen = s->outlen;
        cp.bs = d.burst_start;
        cp.be = d.burst_end;
        cp.win0 = 2 * d.burst_start - d.burst_end;
        cp.win = 2 * d.burst_end - d.burst_start;
        cp.input_line = std::max(1, (int)std::nearbyint(sp.nominal));
        cp.fsc_ratio = d.fsc_ratio;
        cp.rot0 = d.rot[0];
        cp.rot1 = d.rot[1];
        std::memcpy(cp.fin.sec, d.fin.sec, sizeof(cp.fin.sec));
        std::memcpy(cp.fin.zi, d.fin.zi, sizeof(cp.fin.zi));
        cp.fin.edge = d.fin.edge;
        cp.het = s->c_het.p;
        cp.bsin = s->c_bsin.p;
        cp.bcos = s->c_bcos.p;
        cp.ana = s->c_ana.p + (size_t)f0 * s->out_lines * cp.win;
        cp.probe = s->c_probe.p + (size_t)f0 * 2 * s->out_lines * 5;
        cp.probe_nrm = s->c_probe_nrm.p + (size_t)f0 * 2 * s->out_lines * 2;
        cp.flip = s->c_flip.p + 2 * (size_t)f0;
        cp.chosen = s->c_chosen.p + f0;
        cp.rot_in = s->rot_in_d.p;
        cp.rot_out = s->c_state.p;
        cp.status = s->c_state.p + 1;
        cp.summary = s->c_summary.p + 4 * (size_t)f0;
        cp.first_line = s->first_line_d.p + f0;
        cp.first_field = s->first_field_d.p + f0;
        cp.field_number = s->field_number_d.p + f0;
        const size_t field = (size_t)d.field_samples;
        cp.cfield = s->c_field.p + (size_t)f0 * field;
        cp.crow = chroma_final_row((int64_t)field, d.fin.edge);
        cp.up = s->c_up.p + (size_t)f0 * (size_t)cp.crow;
        cp.fwd = s->c_fwd.p + (size_t)f0 * (size_t)cp.crow;
        cp.out = s->chroma.p + (size_t)f0 * field;
        cp.cu_hz = d.cu_hz;
        cp.fsc_mhz = d.fsc_mhz;
        cp.burst_abs_ref = d.burst_abs_ref;
        // UpconvertChromaPhaseCompensated's hetCoefficient (VhsChromaDecoder.cs:2182-2186)
        cp.ntsc_h = ((d.cu_hz * 1.5707963267948965e-6) / d.fsc_mhz) + 1.5707963267948966;
        cp.ntsc_advance = s->c_advance.p;
        cp.line_cs = s->c_line_cs.p + (size_t)f0 * s->out_lines;
        cp.line_scale = s->c_line_scale.p + (size_t)f0 * s->out_lines;
        cp.line_scale_f = s->c_line_scale_f.p + (size_t)f0 * s->out_lines;
        ck(cudaMemsetAsync(s->c_state.p + 1, 0, sizeof(int), fs), "memset");
        TbcParams ta = tp;
        ta.locs = cp.locs;
        ta.first_line = s->c_ones.p;
        ta.out_f32 = s->c_ana.p + (size_t)f0 * s->out_lines * cp.win;
        ta.x0 = cp.win0;
        ta.x1 = cp.win0 + cp.win;
        ta.out_stride = cp.win;
        ck(launch_tbc_pw<float>(s->c32.p, stream_len, ta, s->pw.p, fs), "chroma tbc launch");
        s->launches += kTbcFastKernels;
        ck(launch_chroma_phase(cp, fs), "chroma phase launch");
        s->launches += kChromaPhaseKernels;
    }
    if (timing) ck(cudaEventRecord(s->stage_ev[1], fs), "event");
    if (!timing) {
        ck(cudaEventRecord(s->drop_hsync, fs), "event");
        ck(cudaStreamWaitEvent(ds, s->drop_hsync, 0), "wait");
        ck(launch_drop_detect<T>(env, stream_len, dp, s->drop_counts.p + (size_t)f0 * nch, ds), "dropout launch");
        ck(cudaEventRecord(s->drop_join, ds), "event");
    }
    tp.locs = final_locs;
    tp.first_line = s->first_line_d.p + f0;
    tp.ire0 = s->fmt.ire0;
    tp.output_scale = output_scale(s->fmt);
    tp.inv_hz_ire = 1.0 / s->fmt.hz_ire;
    tp.offset = (s->fmt.output_zero + 0.5) - (s->fmt.vsync_ire * tp.output_scale);
    tp.out_u16 = s->tbc.p + (size_t)f0 * s->out_lines * s->outlen;
    tp.out_hz = nullptr;
    tp.line_consts = std::is_same<T, float>::value
                         ? s->tbc_consts.p + (size_t)f0 * s->out_lines * kTbcLineConstsBytes
                         : nullptr;
    const bool fused = chroma && std::is_same<T, float>::value;
    if (fused) {
        // the chroma TBC of the output lines rides on the luma's positions and weights
        tp.src2 = s->c32.p;
        tp.out2_f32 = s->c_field.p + (size_t)f0 * s->cd.field_samples;
    }
    ck(launch_tbc_pw<T>(video, stream_len, tp, s->pw.p, fs), "tbc launch");
    s->launches += tp.line_consts ? kTbcFastKernels : kTbcKernels;
    if (fused) {
        ck(launch_chroma_decode(cp, fs), "chroma decode launch");
        s->launches += kChromaDecodeKernels;
    } else if (chroma) {
        // the chroma TBC of the output lines and the field decode to uint16
        TbcParams tc = tp;
        tc.out_u16 = nullptr;
        tc.out_f32 = s->c_field.p + (size_t)f0 * s->cd.field_samples;
        tc.x0 = 0;
        tc.x1 = 0;
        tc.out_stride = s->outlen;
        tc.line_consts = s->tbc_consts.p + (size_t)f0 * s->out_lines * kTbcLineConstsBytes;
        ck(launch_tbc_pw<float>(s->c32.p, stream_len, tc, s->pw.p, fs), "chroma tbc launch");
        s->launches += kTbcFastKernels;
        ck(launch_chroma_decode(cp, fs), "chroma decode launch");
        s->launches += kChromaDecodeKernels;
    }
    if (timing) ck(cudaEventRecord(s->stage_ev[2], fs), "event");
    if (timing) {
        ck(launch_drop_detect<T>(env, stream_len, dp, s->drop_counts.p + (size_t)f0 * nch, fs), "dropout launch");
    } else {
        ck(cudaStreamWaitEvent(fs, s->drop_join, 0), "wait");
    }
    s->launches += kDropoutKernels;
    if (timing) {
        ck(cudaEventRecord(s->stage_ev[3], fs), "event");
        ck(cudaEventSynchronize(s->stage_ev[3]), "sync");
        float a = 0, b = 0, c = 0;
        cudaEventElapsedTime(&a, s->stage_ev[0], s->stage_ev[1]);
        cudaEventElapsedTime(&b, s->stage_ev[1], s->stage_ev[2]);
        cudaEventElapsedTime(&c, s->stage_ev[2], s->stage_ev[3]);
        s->stage_ms[0] += a; s->stage_ms[1] += b; s->stage_ms[2] += c;
    }
}

// The chroma rotation index and status slot at the end of the pinned results.
unsigned char* h_field_out_chroma(vhsdecode_gb300_session* s) {
    const size_t fl = (size_t)s->max_fields * s->lines, mf = (size_t)s->max_fields;
    return s->h_field_out + fl * 8 + mf * 8 + mf * (size_t)kDropEarly * 3 * 4;
}

// Refined line locations and dropout lists of every field back to the host
// once `fs` has finished the field stage.
void collect_field_results(vhsdecode_gb300_session* s, cudaStream_t fs) {
    int nf = (int)s->fields.size();
    if (nf == 0) return;
    const size_t L = (size_t)s->lines, mf = (size_t)s->max_fields;
    // pinned landing area: one round trip for the refined lines, the dropout
    // counts and status, and up to kDropEarly dropout triplets per field
    double* refined = reinterpret_cast<double*>(s->h_field_out);
    int* dcount = reinterpret_cast<int*>(refined + mf * L);
    int* dstat = dcount + mf;
    int32_t* early = dstat + mf;
    const int ke = std::min(kDropEarly, s->drop_out_cap);
    const size_t row = (size_t)s->drop_out_cap * 3 * sizeof(int32_t);
    const double* final_locs = s->want_chroma ? s->locs_final.p : s->locs_out.p;
    ck(cudaMemcpyAsync(refined, final_locs, (size_t)nf * L * sizeof(double), cudaMemcpyDeviceToHost, fs), "d2h");
    int* cstate = reinterpret_cast<int*>(h_field_out_chroma(s));
    if (s->want_chroma) ck(cudaMemcpyAsync(cstate, s->c_state.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, fs), "d2h");
    ck(cudaMemcpyAsync(dcount, s->drop_out_count.p, nf * sizeof(int), cudaMemcpyDeviceToHost, fs), "d2h");
    ck(cudaMemcpyAsync(dstat, s->drop_status.p, nf * sizeof(int), cudaMemcpyDeviceToHost, fs), "d2h");
    ck(cudaMemcpy2DAsync(early, (size_t)ke * 3 * sizeof(int32_t), s->drop_out.p, row, (size_t)ke * 3 * sizeof(int32_t),
                         (size_t)nf, cudaMemcpyDeviceToHost, fs), "d2h dropouts");
    ck(cudaStreamSynchronize(fs), "sync");
    if (s->want_chroma) {
        if (cstate[1] != 0)
            throw Failure(VHSDECODE_GB300_STATUS_DECODE_ERROR, "no valid chroma burst samples for phase averaging");
        s->chroma_rot_end = cstate[0];
    }
    int maxc = 0;
    for (int f = 0; f < nf; f++) {
        if (dstat[f] != 0)
            throw Failure(VHSDECODE_GB300_STATUS_DECODE_ERROR, "dropout event capacity exceeded");
        maxc = std::max(maxc, std::min(dcount[f], s->drop_out_cap));
    }
    // a field with more dropouts than the early copy holds: a second strided
    // copy of the first maxc triplets of every field
    std::vector<int32_t> late;
    if (maxc > ke) {
        late.resize((size_t)nf * maxc * 3);
        ck(cudaMemcpy2DAsync(late.data(), (size_t)maxc * 3 * sizeof(int32_t), s->drop_out.p, row,
                             (size_t)maxc * 3 * sizeof(int32_t), (size_t)nf, cudaMemcpyDeviceToHost, fs),
           "d2h dropouts");
        ck(cudaStreamSynchronize(fs), "sync");
    }
    for (int f = 0; f < nf; f++) {
        FieldRec& r = s->fields[(size_t)f];
        r.refined.assign(refined + (size_t)f * L, refined + (size_t)(f + 1) * L);
        int c = std::min(dcount[f], s->drop_out_cap);
        const int32_t* src = late.empty() ? early + (size_t)f * ke * 3 : late.data() + (size_t)f * maxc * 3;
        r.drop.assign(src, src + (size_t)c * 3);
    }
    if (s->stage_timing) {
        int miss = 0;
        ck(cudaMemcpy(&miss, s->hsync_misses.p, sizeof(int), cudaMemcpyDeviceToHost), "d2h");
        std::fprintf(stderr, "[gb300 stage] fields=%d hsync=%.3f ms tbc=%.3f ms dropouts=%.3f ms "
                     "rescue_fetches=%d enqueue=%.3f ms segments=%u porch_misses=%d\n", nf, s->stage_ms[0],
                     s->stage_ms[1], s->stage_ms[2], s->rescue_fetches, s->enqueue_ms, s->segments, miss);
        if (s->chroma_pending) {
            float c0 = 0, c1 = 0;
            ck(cudaEventSynchronize(s->chroma_t[1]), "sync");
            ck(cudaEventElapsedTime(&c0, s->ev[0], s->chroma_t[0]), "elapsed");
            ck(cudaEventElapsedTime(&c1, s->ev[0], s->chroma_t[1]), "elapsed");
            std::fprintf(stderr, "[gb300 stage] chroma block stage from %.3f to %.3f ms after the decode start\n",
                         c0, c1);
        }
    }
}

// Segment boundaries (in blocks) of the pipelined decode: a short first
// segment so the control plane can start early, then kSegBlocks each.
std::vector<int64_t> segment_bounds(int64_t nblocks) {
    std::vector<int64_t> b{0};
    int64_t e = std::min<int64_t>(nblocks, kFirstSegBlocks);
    while (b.back() < nblocks) {
        b.push_back(e);
        e = std::min<int64_t>(nblocks, e + kSegBlocks);
    }
    return b;
}

// FP32 decode, pipelined: the capture is demodulated in segments; after each
// segment the device writes that segment's pulse events and copies them to
// pinned host memory, so the host control plane analyses the fields of
// finished segments while later segments are still being demodulated.  With
// host input the RF of each segment is copied on a separate stream ahead of
// its demod.  Results are identical to a single pass: demod blocks are
// independent and the ranged pulse scan carries its state across segments.
// Queues the segment pipeline from `root`: RF copies on copy_stream, demod and
// pulse scans alternating between root and alt_stream, event copies on
// d2h_stream; every side stream joins back into root at the end.  When
// `capturing`, the events the host waits on or times (seg_done, seg_dem) are
// recorded as external graph nodes.
void enqueue_pipeline(vhsdecode_gb300_session* s, const int16_t* rf, uint64_t n, bool host_input,
                      bool demod_only, const std::vector<int64_t>& bounds, cudaStream_t root, bool capturing) {
    auto rec = [&](cudaEvent_t e, cudaStream_t st, bool external) {
        if (capturing && external) ck(cudaEventRecordWithFlags(e, st, cudaEventRecordExternal), "event");
        else ck(cudaEventRecord(e, st), "event");
    };
    const int nseg = (int)bounds.size() - 1;
    const int16_t* rf_dev = host_input ? s->rf.p : rf;
    FastDemodParams p = fp32_params(s, rf_dev);
    ck(cudaMemsetAsync(s->repair.p, 0, sizeof(int), root), "memset");
    rec(s->alt_start, root, false);
    ck(cudaStreamWaitEvent(s->alt_stream, s->alt_start, 0), "wait");
    ck(cudaStreamWaitEvent(s->copy_stream, s->alt_start, 0), "wait");
    ck(cudaStreamWaitEvent(s->d2h_stream, s->alt_start, 0), "wait");
    int64_t copied = 0;
    for (int k = 0; k < nseg; k++) {
        int64_t b0 = bounds[(size_t)k], b1 = bounds[(size_t)k + 1];
        cudaStream_t ks = (k & 1) ? s->alt_stream : root;
        if (host_input) {
            int64_t c1 = std::min<int64_t>((int64_t)n, (b1 - 1) * kStride + kBlock);
            if (c1 > copied) {
                ck(cudaMemcpyAsync(s->rf.p + copied, rf + copied, (size_t)(c1 - copied) * sizeof(int16_t),
                                   cudaMemcpyHostToDevice, s->copy_stream), "h2d rf");
                copied = c1;
            }
            rec(s->seg_copied[(size_t)k], s->copy_stream, false);
            ck(cudaStreamWaitEvent(ks, s->seg_copied[(size_t)k], 0), "wait");
        }
        p.first_block = b0;
        p.nblocks = b1 - b0;
        const size_t half = (size_t)(s->num_sms / 2) * kBlock;
        p.scratch = s->scratch.p + (k & 1) * 2 * half;
        p.block_counter = s->blk_counters.p + k;
        ck(cudaMemsetAsync(p.block_counter, 0, sizeof(unsigned), ks), "memset");
        rec(s->seg_dem[(size_t)(2 * k)], ks, true);
        ck(launch_fused(s, p, ks), "demod fp32 launch");
        rec(s->seg_dem[(size_t)(2 * k + 1)], ks, true);
        rec(s->seg_demod_end[(size_t)k], ks, false);   // dependency edge (the timing record above is external)
        if (!demod_only) {
            // the scan needs the previous segment's samples (state before b0)
            if (k > 0) ck(cudaStreamWaitEvent(ks, s->seg_demod_end[(size_t)k - 1], 0), "wait");
            int64_t* ev = s->seg_events.p + (size_t)k * s->seg_cap;
            int64_t* cnt = (k & 1) ? s->pc_counts_alt.p : s->pc_counts.p;
            int64_t* off = (k & 1) ? s->pc_offsets_alt.p : s->pc_offsets.p;
            // from the pulse-scan bits the demod wrote with the sync stream
            ck(launch_pulse_bits_range(s->sync_cond.p, s->sync_hold.p, b0 * kStride, b1 * kStride, cnt, off, ev,
                                       s->seg_cap, s->seg_total.p + k, ks), "pulse launch");
            rec(s->seg_pulsed[(size_t)k], ks, false);
            ck(cudaStreamWaitEvent(s->d2h_stream, s->seg_pulsed[(size_t)k], 0), "wait");
            ck(cudaMemcpyAsync(s->h_totals + k, s->seg_total.p + k, sizeof(int64_t), cudaMemcpyDeviceToHost,
                               s->d2h_stream), "d2h");
            ck(cudaMemcpyAsync(s->h_events + (size_t)k * s->seg_cap, ev, (size_t)s->seg_cap * sizeof(int64_t),
                               cudaMemcpyDeviceToHost, s->d2h_stream), "d2h events");
            rec(s->seg_done[(size_t)k], s->d2h_stream, true);
        }
    }
    // join the side streams back into root
    for (cudaStream_t side : {s->alt_stream, s->copy_stream, s->d2h_stream}) {
        cudaEvent_t j = side == s->alt_stream ? s->alt_end : (side == s->copy_stream ? s->copy_end : s->d2h_end);
        rec(j, side, false);
        ck(cudaStreamWaitEvent(root, j, 0), "wait");
    }
}

// Kernels the pipeline queues for `bounds` (demod + pulse scans).
uint32_t pipeline_launches(const std::vector<int64_t>& bounds, bool demod_only) {
    uint32_t nseg = (uint32_t)(bounds.size() - 1);
    return nseg * (1u + (demod_only ? 0u : (uint32_t)kPulseKernels));
}

// FP32 decode, pipelined: the capture is demodulated in segments; after each
// segment the device writes that segment's pulse events and copies them to
// pinned host memory, so the host control plane analyses the fields of
// finished segments while later segments are still being demodulated.  With
// host input the RF of each segment is copied on a separate stream ahead of
// its demod.  Results are identical to a single pass: demod blocks are
// independent and the ranged pulse scan carries its state across segments.
// With device input or pinned host input the queued work is captured once as
// a CUDA graph (keyed by the input pointer, length and mode) and replayed.
void decode_fp32_pipelined(vhsdecode_gb300_session* s, const int16_t* rf, uint64_t n, bool host_input,
                           bool demod_only, uint32_t max_fields, uint32_t& stop, double& host_ms,
                           float& demod_ms, const std::atomic<bool>* cancel, DecodeCarry* carry) {
    cudaStream_t cs = s->stream;
    int64_t nblocks = block_count(n);
    int64_t stream_len = nblocks * kStride;
    // with no field work to overlap, the demod runs as one launch
    std::vector<int64_t> bounds = demod_only ? std::vector<int64_t>{0, nblocks} : segment_bounds(nblocks);
    if (nblocks == 0) bounds.assign(1, 0);
    int nseg = (int)bounds.size() - 1;
    s->segments = (uint32_t)nseg;
    if (nseg > s->nseg_max) throw Failure(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, "segment table too small");
    auto tq0 = std::chrono::steady_clock::now();
    bool graphable = !host_input;
    if (host_input && n > 0) {
        cudaPointerAttributes attr{};
        graphable = cudaPointerGetAttributes(&attr, rf) == cudaSuccess && attr.type == cudaMemoryTypeHost;
        cudaGetLastError();
    }
    if (carry && carry->no_graph) graphable = false;
    s->chroma_pending = false;
    if (s->want_chroma && nblocks > 0 && host_input) {
        // The chroma block stage needs the whole capture and SMs of its own
        // for its whole run; queued behind the persistent demodulator it gets
        // them only as the demodulation ends.  Pinned input: the stage reads
        // the capture where it is (mapped host memory) from the start, beside
        // the pipeline's own copies.  Pageable input: the capture is copied
        // first and the device-input schedule follows.
        cudaPointerAttributes attr{};
        const bool mapped = cudaPointerGetAttributes(&attr, rf) == cudaSuccess &&
                            attr.type == cudaMemoryTypeHost && attr.devicePointer != nullptr &&
                            ((uintptr_t)attr.devicePointer & 15u) == 0;
        cudaGetLastError();
        if (mapped) {
            ck(cudaEventRecord(s->chroma_go, cs), "event");
            queue_chroma_blocks(s, static_cast<const int16_t*>(attr.devicePointer), nblocks, s->chroma_go);
        } else {
            ck(cudaMemcpyAsync(s->rf.p, rf, (size_t)n * sizeof(int16_t), cudaMemcpyHostToDevice, cs), "h2d rf");
            rf = s->rf.p;
            host_input = false;
            graphable = !(carry && carry->no_graph);
        }
    }
    // The chroma block stage holds an SM per CTA for its whole (latency-bound)
    // run and is queued before the demodulator, so it has its SMs first; the
    // demodulator is launched with only the clusters that find SMs beside it
    // (measured 0.05 ms faster per decode than queueing clusters that wait).
    s->demod_clusters = 0;
    if (s->want_chroma && nblocks > 0 && !demod_only) {
        const int reserve = std::min(chroma_block_ctas(nblocks), s->num_sms / 4);
        s->demod_clusters = std::max(1, (s->num_sms - reserve) / 2);
    }
    if (s->want_chroma && nblocks > 0 && !host_input) {
        // the capture is already on the device: start the chroma band-pass now
        ck(cudaEventRecord(s->chroma_go, cs), "event");
        queue_chroma_blocks(s, rf, nblocks, s->chroma_go);
    }
    if (graphable && nseg > 0) {
        PipeKey key{s->in_f32 ? (const void*)s->in_f32 : (const void*)rf, n, host_input, demod_only,
                    s->in_f32 != nullptr, s->demod_clusters};
        if (!s->pipe_exec || !(s->pipe_key == key)) {
            if (s->pipe_exec) { cudaGraphExecDestroy(s->pipe_exec); s->pipe_exec = nullptr; }
            FastDemodParams p0 = fp32_params(s, s->rf.p);
            ck(launch_fused(s, p0, s->cap_stream), "demod attribute");  // nblocks 0: sets attributes only
            ck(cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeThreadLocal), "begin capture");
            cudaGraph_t g = nullptr;
            try {
                enqueue_pipeline(s, rf, n, host_input, demod_only, bounds, s->cap_stream, true);
            } catch (...) {
                cudaStreamEndCapture(s->cap_stream, &g);
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                throw;
            }
            ck(cudaStreamEndCapture(s->cap_stream, &g), "end capture");
            cudaError_t ie = cudaGraphInstantiate(&s->pipe_exec, g, 0);
            cudaGraphDestroy(g);
            ck(ie, "graph instantiate");
            s->pipe_key = key;
        }
        ck(cudaGraphLaunch(s->pipe_exec, cs), "graph launch");
    } else {
        enqueue_pipeline(s, rf, n, host_input, demod_only, bounds, cs, false);
    }
    s->launches += pipeline_launches(bounds, demod_only);
    s->enqueue_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tq0).count();
    if (!demod_only && nblocks > 0) {
        auto t0 = std::chrono::steady_clock::now();
        EventFeed feed;
        int kdone = 0;
        int64_t ready = 0;
        feed.upto = [&](int64_t pos) {
            while (ready < pos && kdone < nseg) {
                ck(cudaEventSynchronize(s->seg_done[(size_t)kdone]), "segment wait");
                int64_t cnt = s->h_totals[kdone];
                if (cnt > s->seg_cap)
                    throw Failure(VHSDECODE_GB300_STATUS_DECODE_ERROR, "sync pulse event capacity exceeded");
                const int64_t* e = s->h_events + (size_t)kdone * s->seg_cap;
                feed.events.insert(feed.events.end(), e, e + cnt);
                ready = bounds[(size_t)kdone + 1] * kStride;
                kdone++;
            }
        };
        // The field kernels run as one batch over all fields after the host
        // loop: batches launched from the host loop while the closing segments
        // demodulate were slower (host launch and copy time lands on the
        // field analysis, and their CTAs take SMs from the demod).
        host_field_loop<float>(s, s->s32.p, stream_len, max_fields, feed, stop, cancel, carry);
        host_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        ck(cudaEventRecord(s->ev[2], cs), "event");
        if (s->chroma_pending) ck(cudaStreamWaitEvent(s->field_stream, s->chroma_done, 0), "wait");
        launch_field_batch<float>(s, 0, (int)s->fields.size(), s->v32.p, s->s32.p, s->e32.p,
                                  stream_len, s->field_stream);
        collect_field_results(s, s->field_stream);
        ck(cudaEventRecord(s->field_end, s->field_stream), "event");
        ck(cudaStreamWaitEvent(cs, s->field_end, 0), "wait");
    } else {
        ck(cudaEventRecord(s->ev[2], cs), "event");
        if (s->chroma_pending) ck(cudaStreamWaitEvent(cs, s->chroma_done, 0), "wait");
    }
    ck(cudaStreamSynchronize(s->d2h_stream), "sync");
    ck(cudaEventSynchronize(s->seg_dem[(size_t)(2 * std::max(0, nseg - 1) + 1)]), "sync");
    demod_ms = 0.0f;
    for (int k = 0; k < nseg; k++) {
        float t = 0.0f;
        ck(cudaEventElapsedTime(&t, s->seg_dem[(size_t)(2 * k)], s->seg_dem[(size_t)(2 * k + 1)]), "elapsed");
        demod_ms += t;
    }
}

// FP64 plain decode: whole capture, one block per graph replay, then the
// whole-stream pulse scan, the control plane and the field stage in order.
void decode_plain(vhsdecode_gb300_session* s, const int16_t* rf_dev, uint64_t n, bool demod_only,
                  uint32_t max_fields, uint32_t& stop, double& host_ms, float& demod_ms,
                  const std::atomic<bool>* cancel, DecodeCarry* carry) {
    cudaStream_t cs = s->stream;
    int64_t nblocks = block_count(n);
    int64_t stream_len = nblocks * kStride;
    ck(cudaEventRecord(s->ev[1], cs), "event");
    run_demod(s, rf_dev, nblocks);
    s->launches += (uint32_t)(nblocks * (kPlainBlockKernels + (s->sub64.p ? kPlainSubKernels : 0)));
    s->segments = 1;
    ck(cudaEventRecord(s->ev[2], cs), "event");
    if (!demod_only && nblocks > 0) {
        const double threshold = s->sp.ire_to_hz(s->sp.vsync_ire / 2.0);
        ck(launch_pulse_events<double>(s->s64.p, stream_len, threshold, s->pc_counts.p, s->pc_offsets.p,
                                       s->pc_events.p, s->pc_capacity, s->pc_total.p, cs), "pulse launch");
        s->launches += kPulseKernels;
        int64_t total = 0;
        ck(cudaMemcpyAsync(&total, s->pc_total.p, sizeof(int64_t), cudaMemcpyDeviceToHost, cs), "d2h");
        ck(cudaStreamSynchronize(cs), "sync");
        if (total > s->pc_capacity)
            throw Failure(VHSDECODE_GB300_STATUS_DECODE_ERROR, "sync pulse event capacity exceeded");
        EventFeed feed;
        feed.events.resize((size_t)total);
        if (total > 0)
            ck(cudaMemcpyAsync(feed.events.data(), s->pc_events.p, (size_t)total * sizeof(int64_t),
                               cudaMemcpyDeviceToHost, cs), "d2h events");
        ck(cudaStreamSynchronize(cs), "sync");
        feed.upto = [](int64_t) {};
        auto t0 = std::chrono::steady_clock::now();
        host_field_loop<double>(s, s->s64.p, stream_len, max_fields, feed, stop, cancel, carry);
        host_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (s->want_chroma) launch_chroma_blocks_for(s, rf_dev, nblocks, cs);
        launch_field_batch<double>(s, 0, (int)s->fields.size(), s->v64.p, s->s64.p, s->e64.p, stream_len, cs);
        collect_field_results(s, cs);
    } else if (s->want_chroma && nblocks > 0) {
        launch_chroma_blocks_for(s, rf_dev, nblocks, cs);
    }
    ck(cudaEventSynchronize(s->ev[2]), "sync");
    ck(cudaEventElapsedTime(&demod_ms, s->ev[1], s->ev[2]), "elapsed");
}

// Float or decimated input: the float capture at the decode rate, queued on
// the session stream.  Host input is copied in first; the decimator (cuda-fast
// reader's 20-MSPS mode, src/VHSDecode.CudaFast.Native/src/cuda_fast_decimator.cu:160-319)
// turns n source samples into n / 2.
const float* stage_float_input(vhsdecode_gb300_session* s, const void* rf, uint64_t n, bool f32_in,
                               bool host_input) {
    cudaStream_t cs = s->stream;
    const uint64_t nd = n / (uint64_t)s->decim;
    auto ensure = [&](DevBuf<float>& b, uint64_t count) {
        if (b.n < count) b.alloc(count);
    };
    if (s->decim == 1) {   // float input at the decode rate
        if (!host_input) return static_cast<const float*>(rf);
        ensure(s->rf_f32, std::max<uint64_t>(s->max_samples, 16));
        if (n > 0) ck(cudaMemcpyAsync(s->rf_f32.p, rf, n * sizeof(float), cudaMemcpyHostToDevice, cs), "h2d rf");
        return s->rf_f32.p;
    }
    ensure(s->rf_f32, std::max<uint64_t>(s->max_samples / 2, 16));
    const int16_t* src16 = nullptr;
    const float* src32 = nullptr;
    if (f32_in) {
        if (host_input) {
            ensure(s->src_f32, std::max<uint64_t>(s->max_samples, 16));
            if (n > 0)
                ck(cudaMemcpyAsync(s->src_f32.p, rf, n * sizeof(float), cudaMemcpyHostToDevice, cs), "h2d rf");
            src32 = s->src_f32.p;
        } else {
            src32 = static_cast<const float*>(rf);
        }
    } else {
        if (host_input) {
            if (n > 0)
                ck(cudaMemcpyAsync(s->rf.p, rf, n * sizeof(int16_t), cudaMemcpyHostToDevice, cs), "h2d rf");
            src16 = s->rf.p;
        } else {
            src16 = static_cast<const int16_t*>(rf);
        }
    }
    if (nd > 0) {
        ck(launch_decimate_half(src16, src32, (int64_t)n, s->rf_f32.p, (int64_t)nd, cs), "decimate launch");
        s->launches += kDecimateKernels;
    }
    return s->rf_f32.p;
}

int32_t decode_impl(vhsdecode_gb300_session* s, const void* rf_in, uint64_t n_in, uint32_t max_fields,
                    uint32_t flags, vhsdecode_gb300_decode_result_v1* res,
                    const std::atomic<bool>* cancel, DecodeCarry* carry) {
    if (n_in > s->max_samples)
        throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "sample_count exceeds the session capacity");
    ck(cudaSetDevice(s->device), "cudaSetDevice");
    cudaStream_t cs = s->stream;
    bool host_input = !(flags & VHSDECODE_GB300_DECODE_DEVICE_INPUT);
    const bool demod_only = (flags & VHSDECODE_GB300_DECODE_DEMOD_ONLY) != 0;
    const bool f32_in = (flags & VHSDECODE_GB300_DECODE_FLOAT_INPUT) != 0;
    s->want_chroma = (flags & VHSDECODE_GB300_DECODE_CHROMA) != 0;
    if (s->want_chroma) ensure_chroma(s);
    if (!host_input && ((uintptr_t)rf_in & 15u) != 0)
        throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "device rf pointer must be 16-byte aligned");
    // samples at the decode rate
    const uint64_t n = n_in / (uint64_t)s->decim;
    int64_t nblocks = block_count(n);
    uint32_t stop = 0;
    double host_ms = 0.0;
    float demod_ms = 0.0f;
    s->fields.clear();
    s->launches = 0;
    s->segments = 0;
    s->stage_ms[0] = s->stage_ms[1] = s->stage_ms[2] = 0.0f;
    ck(cudaEventRecord(s->ev[0], cs), "event");
    const int16_t* rf = static_cast<const int16_t*>(rf_in);
    s->in_f32 = nullptr;
    if (f32_in || s->decim == 2) {
        // the demodulators read the float capture from the device
        s->in_f32 = stage_float_input(s, rf_in, n_in, f32_in, host_input);
        rf = nullptr;
        host_input = false;
    }
    if (s->fp32()) {
        decode_fp32_pipelined(s, rf, n, host_input, demod_only, max_fields, stop, host_ms, demod_ms, cancel,
                              carry);
    } else {
        const int16_t* rf_dev = rf;
        if (host_input) {
            if (n > 0) ck(cudaMemcpyAsync(s->rf.p, rf, n * sizeof(int16_t), cudaMemcpyHostToDevice, cs), "h2d rf");
            rf_dev = s->rf.p;
        }
        decode_plain(s, rf_dev, n, demod_only, max_fields, stop, host_ms, demod_ms, cancel, carry);
    }
    ck(cudaEventRecord(s->ev[3], cs), "event");
    ck(cudaEventSynchronize(s->ev[3]), "sync");
    if (carry && s->want_chroma) carry->state.chroma_rot = s->chroma_rot_end;
    int rep = 0;
    if (s->fp32() && nblocks > 0)
        ck(cudaMemcpy(&rep, s->repair.p, sizeof(int), cudaMemcpyDeviceToHost), "d2h");
    s->last_blocks = nblocks;
    s->last_repairs = rep;
    if (s->demod_cycles && s->fp32() && nblocks > 0) {
        // diagnostics: the decode's per-stage demod cycles per block, to stderr
        const size_t nb = 2 * kDemodStages * sizeof(unsigned long long);
        std::vector<unsigned long long> h(2 * kDemodStages);
        ck(cudaMemcpy(h.data(), s->demod_cycles, nb, cudaMemcpyDeviceToHost), "d2h");
        ck(cudaMemset(s->demod_cycles, 0, nb), "memset");
        std::fprintf(stderr, "vhsd demod stage cycles per block (rank0 rank1), %lld blocks, %d repaired:\n",
                     (long long)nblocks, rep);
        for (int k = 0; k < kDemodStages; k++)
            std::fprintf(stderr, "  stage %2d %10.0f %10.0f\n", k, (double)h[k] / nblocks,
                         (double)h[kDemodStages + k] / nblocks);
    }
    if (res) {
        float t_all = 0, t_fld = 0;
        cudaEventElapsedTime(&t_all, s->ev[0], s->ev[3]);
        cudaEventElapsedTime(&t_fld, s->ev[2], s->ev[3]);
        res->fields = (uint32_t)s->fields.size();
        res->output_line_length = (uint32_t)s->outlen;
        res->output_field_lines = (uint32_t)s->out_lines;
        res->blocks = (uint64_t)nblocks;
        res->stream_samples = (uint64_t)(nblocks * kStride);
        res->repaired_blocks = (uint32_t)rep;
        res->stop_reason = stop;
        res->device_ms = t_all;
        res->demod_ms = demod_ms;
        res->field_ms = t_fld;
        res->host_ms = host_ms;
        res->kernel_launches = s->launches;
        res->segments = s->segments;
        res->fft_plan = (uint32_t)s->fft_plan;
    }
    return VHSDECODE_GB300_STATUS_OK;
}

// ---------------------------------------------------------------- batched windows
// Cross-stream batching for the window server: the blocks of several windows
// (each on its own session, of any format and sample rate) are demodulated by
// one persistent launch of the fused kernel, which claims blocks from one
// counter across a table of per-window parameters; then each window's pulse
// scan, field loop and field stage run on its own session.  A window's
// results equal its own decode: every block is computed by the same kernel
// code from the same samples, and the pulse scan over the whole stream gives
// the events the segmented scans give.

BatchScratch::~BatchScratch() {
    if (d_jobs) cudaFree(d_jobs);
    if (d_start) cudaFree(d_start);
    if (d_counter) cudaFree(d_counter);
    if (h_jobs) cudaFreeHost(h_jobs);
    if (h_start) cudaFreeHost(h_start);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
}

void BatchScratch::init(int max_windows) {
    cap = max_windows;
    ck(cudaEventCreate(&ev0), "cudaEventCreate");
    ck(cudaEventCreate(&ev1), "cudaEventCreate");
    ck(cudaMalloc(&d_jobs, (size_t)cap * sizeof(FastDemodParams)), "cudaMalloc");
    ck(cudaMalloc(&d_start, (size_t)(cap + 1) * sizeof(int64_t)), "cudaMalloc");
    ck(cudaMalloc(&d_counter, sizeof(unsigned)), "cudaMalloc");
    ck(cudaHostAlloc((void**)&h_jobs, (size_t)cap * sizeof(FastDemodParams), cudaHostAllocDefault), "cudaHostAlloc");
    ck(cudaHostAlloc((void**)&h_start, (size_t)(cap + 1) * sizeof(int64_t), cudaHostAllocDefault), "cudaHostAlloc");
}

bool batchable(const vhsdecode_gb300_session* s) { return s->fp32() && s->decim == 1; }

// The FP32 decode after its demod has run: pulse events over the whole
// stream, the host field loop, the field stage, the results.
void decode_after_demod(vhsdecode_gb300_session* s, uint64_t n, uint32_t max_fields, DecodeCarry* carry,
                        vhsdecode_gb300_decode_result_v1* res, float demod_ms) {
    cudaStream_t cs = s->stream;
    const int64_t nblocks = block_count(n);
    const int64_t stream_len = nblocks * kStride;
    uint32_t stop = 0;
    double host_ms = 0.0;
    s->want_chroma = false;   // batched windows render luma only
    if (nblocks > 0) {
        ck(launch_pulse_bits_range(s->sync_cond.p, s->sync_hold.p, 0, stream_len, s->pc_counts.p, s->pc_offsets.p,
                                   s->pc_events.p, s->pc_capacity, s->pc_total.p, cs), "pulse launch");
        s->launches += kPulseKernels;
        int64_t total = 0;
        ck(cudaMemcpyAsync(&total, s->pc_total.p, sizeof(int64_t), cudaMemcpyDeviceToHost, cs), "d2h");
        ck(cudaStreamSynchronize(cs), "sync");
        if (total > s->pc_capacity)
            throw Failure(VHSDECODE_GB300_STATUS_DECODE_ERROR, "sync pulse event capacity exceeded");
        EventFeed feed;
        feed.events.resize((size_t)total);
        if (total)
            ck(cudaMemcpy(feed.events.data(), s->pc_events.p, (size_t)total * sizeof(int64_t),
                          cudaMemcpyDeviceToHost), "d2h events");
        feed.upto = [](int64_t) {};
        auto t0 = std::chrono::steady_clock::now();
        host_field_loop<float>(s, s->s32.p, stream_len, max_fields, feed, stop, nullptr, carry);
        host_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        ck(cudaEventRecord(s->ev[2], cs), "event");
        launch_field_batch<float>(s, 0, (int)s->fields.size(), s->v32.p, s->s32.p, s->e32.p, stream_len,
                                  s->field_stream);
        collect_field_results(s, s->field_stream);
        ck(cudaEventRecord(s->field_end, s->field_stream), "event");
        ck(cudaStreamWaitEvent(cs, s->field_end, 0), "wait");
    } else {
        s->fields.clear();
        if (carry) carry->next = carry->start;
        ck(cudaEventRecord(s->ev[2], cs), "event");
    }
    ck(cudaEventRecord(s->ev[3], cs), "event");
    ck(cudaEventSynchronize(s->ev[3]), "sync");
    if (carry && s->want_chroma) carry->state.chroma_rot = s->chroma_rot_end;
    int rep = 0;
    if (nblocks > 0) ck(cudaMemcpy(&rep, s->repair.p, sizeof(int), cudaMemcpyDeviceToHost), "d2h");
    s->last_blocks = nblocks;
    s->last_repairs = rep;
    if (res) {
        float t_all = 0, t_fld = 0;
        cudaEventElapsedTime(&t_all, s->ev[0], s->ev[3]);
        cudaEventElapsedTime(&t_fld, s->ev[2], s->ev[3]);
        res->fields = (uint32_t)s->fields.size();
        res->output_line_length = (uint32_t)s->outlen;
        res->output_field_lines = (uint32_t)s->out_lines;
        res->blocks = (uint64_t)nblocks;
        res->stream_samples = (uint64_t)(nblocks * kStride);
        res->repaired_blocks = (uint32_t)rep;
        res->stop_reason = stop;
        res->device_ms = t_all;
        res->demod_ms = demod_ms;
        res->field_ms = t_fld;
        res->host_ms = host_ms;
        res->kernel_launches = s->launches;
        res->segments = 1;
        res->fft_plan = (uint32_t)s->fft_plan;
    }
}

void decode_batched(std::vector<BatchWindow>& wins, BatchScratch& bs, cudaStream_t st) {
    if (wins.empty()) return;
    if ((int)wins.size() > bs.cap) throw Failure(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, "batch larger than its table");
    vhsdecode_gb300_session* s0 = wins[0].s;
    ck(cudaSetDevice(s0->device), "cudaSetDevice");
    int64_t total = 0;
    for (size_t i = 0; i < wins.size(); i++) {
        BatchWindow& w = wins[i];
        vhsdecode_gb300_session* s = w.s;
        if (!batchable(s) || s->device != s0->device || s->fft_plan != s0->fft_plan)
            throw Failure(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, "window not batchable");
        if (w.n > s->max_samples)
            throw Failure(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "sample_count exceeds the session capacity");
        s->fields.clear();
        s->launches = 1;   // this window's share of the batched launch
        s->segments = 1;
        s->in_f32 = nullptr;
        // the session's own stream waits for the batch stream before its field work
        ck(cudaEventRecord(s->ev[0], st), "event");
        if (w.n > 0)
            ck(cudaMemcpyAsync(s->rf.p, w.samples, w.n * sizeof(int16_t), cudaMemcpyHostToDevice, st), "h2d rf");
        ck(cudaMemsetAsync(s->repair.p, 0, sizeof(int), st), "memset");
        const int64_t nb = block_count(w.n);
        FastDemodParams p = fp32_params(s, s->rf.p);
        p.first_block = 0;
        p.nblocks = nb;
        p.scratch = s0->scratch.p;   // per cluster of the launch
        p.block_counter = nullptr;
        bs.h_jobs[i] = p;
        bs.h_start[i] = total;
        total += nb;
    }
    bs.h_start[wins.size()] = total;
    FastDemodParams m = bs.h_jobs[0];
    m.nblocks = total;
    m.block_counter = bs.d_counter;
    m.batch_jobs = bs.d_jobs;
    m.batch_start = bs.d_start;
    m.batch_njobs = (int)wins.size();
    ck(cudaMemcpyAsync(bs.d_jobs, bs.h_jobs, wins.size() * sizeof(FastDemodParams), cudaMemcpyHostToDevice, st),
       "h2d jobs");
    ck(cudaMemcpyAsync(bs.d_start, bs.h_start, (wins.size() + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st),
       "h2d jobs");
    ck(cudaMemsetAsync(bs.d_counter, 0, sizeof(unsigned), st), "memset");
    ck(cudaEventRecord(bs.ev0, st), "event");
    ck(launch_demod_fp32_batched(m, s0->num_sms / 2, st), "batched demod launch");
    ck(cudaEventRecord(bs.ev1, st), "event");
    ck(cudaEventSynchronize(bs.ev1), "sync");
    float demod_ms = 0.0f;
    cudaEventElapsedTime(&demod_ms, bs.ev0, bs.ev1);
    for (BatchWindow& w : wins) decode_after_demod(w.s, w.n, w.max_fields, w.carry, w.res, demod_ms);
}

}  // namespace detail
}  // namespace vhsd

namespace vhsd {
int32_t set_last_error(int32_t status, const char* msg) {
    g_last_error = msg ? msg : "";
    return status;
}
std::vector<float> sinc_lut_host() { return build_sinc_lut(); }
}  // namespace vhsd

extern "C" {

VHSDECODE_GB300_API uint32_t VHSDECODE_GB300_CALL vhsdecode_gb300_get_abi_version(void) {
    return VHSDECODE_GB300_ABI_VERSION;
}

VHSDECODE_GB300_API const char* VHSDECODE_GB300_CALL vhsdecode_gb300_get_last_error(void) {
    return g_last_error.c_str();
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_get_runtime_info(
    int32_t device_id, vhsdecode_gb300_runtime_info_v1* info) {
    return guard([&]() -> int32_t {
        if (!info) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "info is null");
        if (info->struct_size != sizeof(vhsdecode_gb300_runtime_info_v1))
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "runtime_info struct_size mismatch");
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
            return fail(VHSDECODE_GB300_STATUS_CUDA_UNAVAILABLE, "no CUDA device available");
        if (device_id < 0 || device_id >= n)
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "device_id out of range");
        cudaDeviceProp p{};
        ck(cudaGetDeviceProperties(&p, device_id), "cudaGetDeviceProperties");
        ck(cudaSetDevice(device_id), "cudaSetDevice");
        size_t fr = 0, tot = 0;
        ck(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
        info->abi_version = VHSDECODE_GB300_ABI_VERSION;
        info->device_id = device_id;
        info->compute_major = p.major;
        info->compute_minor = p.minor;
        info->multiprocessor_count = p.multiProcessorCount;
        info->total_vram_bytes = tot;
        info->free_vram_bytes = fr;
        std::snprintf(info->device_name, VHSDECODE_GB300_NAME_CAPACITY, "%s", p.name);
        return VHSDECODE_GB300_STATUS_OK;
    });
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_create(
    const vhsdecode_gb300_session_config_v1* config, vhsdecode_gb300_session** session) {
    return guard([&]() -> int32_t {
        if (!config || !session) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        *session = nullptr;
        if (config->struct_size != sizeof(vhsdecode_gb300_session_config_v1))
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "session_config struct_size mismatch");
        std::unique_ptr<vhsdecode_gb300_session> s(new vhsdecode_gb300_session());
        try {
            session_init(s.get(), *config);
        } catch (...) {
            session_free(s.get());
            throw;
        }
        *session = s.release();
        return VHSDECODE_GB300_STATUS_OK;
    });
}

VHSDECODE_GB300_API void VHSDECODE_GB300_CALL vhsdecode_gb300_session_destroy(vhsdecode_gb300_session* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    session_free(s);
    delete s;
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_set_stream(
    vhsdecode_gb300_session* s, void* cuda_stream) {
    return guard([&]() -> int32_t {
        if (!s) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "session is null");
        s->stream = cuda_stream ? (cudaStream_t)cuda_stream : s->own_stream;
        return VHSDECODE_GB300_STATUS_OK;
    });
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_decode(
    vhsdecode_gb300_session* s, const void* rf, uint64_t n, uint32_t max_fields, uint32_t flags,
    vhsdecode_gb300_decode_result_v1* res) {
    return guard([&]() -> int32_t {
        if (!s || (!rf && n > 0)) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        if (res && res->struct_size != sizeof(vhsdecode_gb300_decode_result_v1))
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "decode_result struct_size mismatch");
        return decode_impl(s, rf, n, max_fields, flags, res);
    });
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_get_field(
    vhsdecode_gb300_session* s, uint32_t index, vhsdecode_gb300_field_info_v1* info) {
    return guard([&]() -> int32_t {
        if (!s || !info) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        if (info->struct_size != sizeof(vhsdecode_gb300_field_info_v1))
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "field_info struct_size mismatch");
        if (index >= s->fields.size()) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "field index out of range");
        const FieldRec& r = s->fields[index];
        info->is_first_field = r.sync.first_field ? 1 : 0;
        info->span_start = r.span_start;
        info->file_loc = (int64_t)std::floor(r.span_start + r.sync.line0 + kCut);
        info->line0 = r.sync.line0;
        info->first_hsync = r.sync.first_hsync;
        info->mean_line_length = r.sync.mean_line;
        info->next_field_offset = r.sync.next_offset;
        info->line_count = (uint32_t)r.refined.size();
        info->dropout_count = (uint32_t)(r.drop.size() / 3);
        return VHSDECODE_GB300_STATUS_OK;
    });
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_copy_tbc(
    vhsdecode_gb300_session* s, uint32_t first, uint32_t count, uint16_t* dst) {
    return guard([&]() -> int32_t {
        if (!s || (!dst && count)) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        if ((uint64_t)first + count > s->fields.size())
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "field range out of range");
        size_t per = (size_t)s->out_lines * s->outlen;
        if (count)
            ck(cudaMemcpyAsync(dst, s->tbc.p + (size_t)first * per, (size_t)count * per * sizeof(uint16_t),
                               cudaMemcpyDeviceToHost, s->stream), "d2h tbc");
        ck(cudaStreamSynchronize(s->stream), "sync");
        return VHSDECODE_GB300_STATUS_OK;
    });
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_copy_chroma(
    vhsdecode_gb300_session* s, uint32_t first, uint32_t count, uint16_t* dst) {
    return guard([&]() -> int32_t {
        if (!s || (!dst && count)) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        if (!s->want_chroma) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "the last decode rendered no chroma");
        if ((uint64_t)first + count > s->fields.size())
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "field range out of range");
        size_t per = (size_t)s->out_lines * s->outlen;
        if (count)
            ck(cudaMemcpyAsync(dst, s->chroma.p + (size_t)first * per, (size_t)count * per * sizeof(uint16_t),
                               cudaMemcpyDeviceToHost, s->stream), "d2h chroma");
        ck(cudaStreamSynchronize(s->stream), "sync");
        return VHSDECODE_GB300_STATUS_OK;
    });
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_copy_chroma_stage(
    vhsdecode_gb300_session* s, uint32_t field, uint32_t stage, double* dst, uint64_t capacity, uint64_t* count) {
    return guard([&]() -> int32_t {
        if (!s || !dst || !count) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        if (!s->want_chroma) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "the last decode rendered no chroma");
        if (field >= s->fields.size()) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "field index out of range");
        const size_t fsz = (size_t)s->cd.field_samples;
        const size_t win = (size_t)(2 * s->cd.burst_end - s->cd.burst_start);
        ck(cudaStreamSynchronize(s->stream), "sync");
        std::vector<float> tf;
        const float* fsrc = nullptr;
        size_t n = 0;
        if (stage == 0) { fsrc = s->c_field.p + field * fsz; n = fsz; }
        else if (stage == 1) {
            fsrc = s->c_up.p + field * (size_t)chroma_final_row((int64_t)fsz, s->cd.fin.edge) + s->cd.fin.edge;
            n = fsz;
        }
        else if (stage == 2) { fsrc = s->c_ana.p + field * (size_t)s->out_lines * win; n = (size_t)s->out_lines * win; }
        if (fsrc) {
            if (capacity < n) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "capacity too small");
            tf.resize(n);
            ck(cudaMemcpy(tf.data(), fsrc, n * sizeof(float), cudaMemcpyDeviceToHost), "d2h");
            for (size_t i = 0; i < n; i++) dst[i] = tf[i];
        } else if (stage == 3) {
            int c = 0;
            ck(cudaMemcpy(&c, s->c_chosen.p + field, sizeof(int), cudaMemcpyDeviceToHost), "d2h");
            n = (size_t)s->out_lines * 5 + 1;
            if (capacity < n) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "capacity too small");
            ck(cudaMemcpy(dst, s->c_probe.p + ((size_t)field * 2 + c) * s->out_lines * 5,
                          (n - 1) * sizeof(double), cudaMemcpyDeviceToHost), "d2h");
            dst[n - 1] = c;
        } else if (stage == 4) {
            n = 4;
            if (capacity < n) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "capacity too small");
            ck(cudaMemcpy(dst, s->c_summary.p + (size_t)field * 4, 4 * sizeof(double), cudaMemcpyDeviceToHost), "d2h");
        } else if (stage == 5) {
            n = (size_t)s->lines;
            if (capacity < n) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "capacity too small");
            ck(cudaMemcpy(dst, s->locs_out.p + (size_t)field * s->lines, n * sizeof(double), cudaMemcpyDeviceToHost),
               "d2h");
        } else {
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "stage must be 0..5");
        }
        *count = n;
        return VHSDECODE_GB300_STATUS_OK;
    });
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_copy_lines(
    vhsdecode_gb300_session* s, uint32_t field, double* dst, uint32_t cap) {
    return guard([&]() -> int32_t {
        if (!s || !dst) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        if (field >= s->fields.size()) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "field index out of range");
        const auto& r = s->fields[field].refined;
        if (cap < r.size()) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "capacity too small");
        std::copy(r.begin(), r.end(), dst);
        return VHSDECODE_GB300_STATUS_OK;
    });
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_copy_dropouts(
    vhsdecode_gb300_session* s, uint32_t field, int32_t* line, int32_t* sx, int32_t* ex, uint32_t cap,
    uint32_t* count) {
    return guard([&]() -> int32_t {
        if (!s || !count) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        if (field >= s->fields.size()) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "field index out of range");
        const auto& d = s->fields[field].drop;
        uint32_t n = (uint32_t)(d.size() / 3);
        *count = n;
        if (n > cap) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "capacity too small");
        if (n && (!line || !sx || !ex)) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null output");
        for (uint32_t i = 0; i < n; i++) { line[i] = d[3 * i]; sx[i] = d[3 * i + 1]; ex[i] = d[3 * i + 2]; }
        return VHSDECODE_GB300_STATUS_OK;
    });
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_copy_stream(
    vhsdecode_gb300_session* s, uint32_t channel, uint64_t start, uint64_t count, double* dst) {
    return guard([&]() -> int32_t {
        if (!s || (!dst && count)) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        if (channel > 3) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "channel must be 0..3");
        if (channel == 3 && !s->want_chroma)
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "the last decode rendered no chroma");
        uint64_t len = (uint64_t)s->last_blocks * kStride;
        if (start + count > len) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "range beyond the stream");
        ck(cudaStreamSynchronize(s->stream), "sync");
        if (channel == 3) {   // the chroma channel is float in both precisions
            std::vector<float> tmp(count);
            ck(cudaMemcpy(tmp.data(), s->c32.p + start, count * sizeof(float), cudaMemcpyDeviceToHost), "d2h");
            for (uint64_t i = 0; i < count; i++) dst[i] = tmp[i];
        } else if (s->fp32()) {
            const float* src = channel == 0 ? s->v32.p : channel == 1 ? s->s32.p : s->e32.p;
            std::vector<float> tmp(count);
            ck(cudaMemcpy(tmp.data(), src + start, count * sizeof(float), cudaMemcpyDeviceToHost), "d2h");
            for (uint64_t i = 0; i < count; i++) dst[i] = tmp[i];
        } else {
            const double* src = channel == 0 ? s->v64.p : channel == 1 ? s->s64.p : s->e64.p;
            ck(cudaMemcpy(dst, src + start, count * sizeof(double), cudaMemcpyDeviceToHost), "d2h");
        }
        return VHSDECODE_GB300_STATUS_OK;
    });
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_tbc_device(
    vhsdecode_gb300_session* s, void** ptr, uint64_t* bytes) {
    return guard([&]() -> int32_t {
        if (!s || !ptr || !bytes) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        *ptr = s->tbc.p;
        *bytes = (uint64_t)s->fields.size() * s->out_lines * s->outlen * sizeof(uint16_t);
        return VHSDECODE_GB300_STATUS_OK;
    });
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_design_filters(
    uint32_t profile, uint32_t speed, uint32_t tape_format, double mhz, double* rf_video, double* video,
    double* sync, double* sub_high, double* env) {
    return guard([&]() -> int32_t {
        if (!rf_video || !video || !sync || !env) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null output");
        FormatParams f;
        if (!format_for(profile, speed, tape_format, f))
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "unsupported profile");
        if (!(mhz > 0)) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "sample rate must be positive");
        FilterSpectra fs;
        try {
            fs = design_filters(f, mhz * 1e6);
        } catch (const std::runtime_error& e) {
            return fail(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, e.what());
        }
        if (sub_high) {
            for (int k = 0; k < kHalf; k++) {
                std::complex<double> v = fs.sub_high.empty() ? std::complex<double>() : fs.sub_high[(size_t)k];
                sub_high[2 * k] = v.real();
                sub_high[2 * k + 1] = v.imag();
            }
        }
        env[3] = fs.sub_b0;
        env[4] = fs.sub_b1;
        env[5] = fs.sub_a1;
        for (int k = 0; k < kHalf; k++) {
            rf_video[k] = fs.rf_video[(size_t)k];
            video[2 * k] = fs.video[(size_t)k].real();
            video[2 * k + 1] = fs.video[(size_t)k].imag();
            sync[2 * k] = fs.sync[(size_t)k].real();
            sync[2 * k + 1] = fs.sync[(size_t)k].imag();
        }
        env[0] = fs.env_b0;
        env[1] = fs.env_b1;
        env[2] = fs.env_a1;
        return VHSDECODE_GB300_STATUS_OK;
    });
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_design_chroma(
    uint32_t profile, uint32_t tape_speed, uint32_t tape_format, double sample_rate_mhz, double* rf_sos,
    double* final_sos, int32_t* geometry, float* heterodyne, float* burst_sin, float* burst_cos) {
    return guard([&]() -> int32_t {
        if (!rf_sos || !final_sos || !geometry) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        FormatParams f;
        if (!format_for(profile, tape_speed, tape_format, f))
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "unsupported format");
        if (!(sample_rate_mhz >= 10.0 && sample_rate_mhz <= 100.0))
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "sample_rate_mhz must be within 10..100");
        vhsd::ChromaDesign d = vhsd::design_chroma(f, sample_rate_mhz * 1e6);
        std::copy(d.rf_sos.begin(), d.rf_sos.end(), rf_sos);
        std::copy(d.final_sos.begin(), d.final_sos.end(), final_sos);
        const int32_t g[8] = {d.burst_start, d.burst_end, d.move, d.rf.edge, d.fin.edge, d.rot[0], d.rot[1],
                              (int32_t)d.field_samples};
        std::copy(g, g + 8, geometry);
        if (heterodyne || burst_sin || burst_cos) {
            std::vector<float> het, bs, bc;
            vhsd::chroma_tables(d, het, bs, bc);
            if (heterodyne) std::copy(het.begin(), het.end(), heterodyne);
            if (burst_sin) std::copy(bs.begin(), bs.end(), burst_sin);
            if (burst_cos) std::copy(bc.begin(), bc.end(), burst_cos);
        }
        return VHSDECODE_GB300_STATUS_OK;
    });
}

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_field_sync(
    uint32_t profile, double mhz, const int64_t* starts, const int64_t* lengths, uint64_t npulses,
    int64_t span_len, const double* ref, int32_t* state, double* out, double* locs, uint32_t cap,
    uint32_t* locs_count) {
    return guard([&]() -> int32_t {
        if ((!starts || !lengths) && npulses) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null pulses");
        if (!state || !out || !locs_count) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null output");
        FormatParams f;
        if (!format_for(profile, 0, VHSDECODE_GB300_TAPE_FORMAT_VHS, f))
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "unsupported profile");
        SyncParams sp = SyncParams::make(f, mhz * 1e6);
        std::vector<Pulse> raw;
        for (uint64_t i = 0; i < npulses; i++) raw.push_back({starts[i], lengths[i]});
        FieldState st;
        st.prev_first = state[0];
        st.has_prev_hsync = state[1] != 0;
        RefFetch fetch;
        if (ref)
            fetch = [&](int64_t s0, int64_t len, std::vector<double>& o) { o.assign(ref + s0, ref + s0 + len); };
        FieldSync fs = analyse_field(sp, raw, span_len, st, fetch);
        state[0] = st.prev_first;
        state[1] = st.has_prev_hsync ? 1 : 0;
        if (!fs.ok) return fail(VHSDECODE_GB300_STATUS_DECODE_ERROR, fs.error);
        out[0] = fs.first_field ? 1.0 : 0.0;
        out[1] = fs.line0;
        out[2] = fs.first_hsync;
        out[3] = fs.mean_line;
        out[4] = fs.next_offset;
        *locs_count = (uint32_t)fs.locs.size();
        if (locs) {
            if (cap < fs.locs.size()) return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "capacity too small");
            std::copy(fs.locs.begin(), fs.locs.end(), locs);
        }
        return VHSDECODE_GB300_STATUS_OK;
    });
}

}  // extern "C"
