// Internal state of a decode session and the helpers shared by the C ABI
// translation units (abi.cpp, server.cpp).  Not part of the public interface.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/vhsdecode_gb300.h"
#include "chroma.hpp"
#include "control.hpp"
#include "filters.hpp"
#include "formats.hpp"
#include "kernels.h"

namespace vhsd {
namespace detail {

extern thread_local std::string g_last_error;

struct Failure : std::runtime_error {
    int32_t status;
    Failure(int32_t s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline int32_t fail(int32_t status, const std::string& msg) {
    g_last_error = msg;
    return status;
}

inline void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        int32_t st = (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ||
                      e == cudaErrorInitializationError)
                         ? VHSDECODE_GB300_STATUS_CUDA_UNAVAILABLE
                         : VHSDECODE_GB300_STATUS_INTERNAL_ERROR;
        throw Failure(st, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

template <typename F>
int32_t guard(F&& f) {
    try {
        int32_t r = f();
        if (r == VHSDECODE_GB300_STATUS_OK) g_last_error.clear();
        return r;
    } catch (const Failure& e) {
        return fail(e.status, e.what());
    } catch (const std::bad_alloc&) {
        return fail(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, e.what());
    } catch (...) {
        return fail(VHSDECODE_GB300_STATUS_INTERNAL_ERROR, "unknown native failure");
    }
}

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    void alloc(size_t count) {
        release();
        if (count == 0) return;
        ck(cudaMalloc(&p, count * sizeof(T)), "cudaMalloc");
        n = count;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DevBuf() { release(); }
};

// A typed pointer into a DevBuf<unsigned char> owned elsewhere.
template <typename T>
struct View {
    T* p = nullptr;
};

// Identity of a captured pipeline graph: the graph bakes these in.
struct PipeKey {
    const void* rf = nullptr;
    uint64_t n = 0;
    bool host_input = false, demod_only = false, f32 = false;
    int clusters = 0;   // the fused demodulator's clusters (fewer while the chroma block stage runs)
    bool operator==(const PipeKey& o) const {
        return rf == o.rf && n == o.n && host_input == o.host_input && demod_only == o.demod_only && f32 == o.f32 &&
               clusters == o.clusters;
    }
};

struct FieldRec {
    FieldSync sync;
    int64_t span_start;
    int64_t span_len;
    int field_number = 0;       // VHS field number (NTSC chroma colour frame)
    std::vector<double> refined;
    std::vector<int32_t> drop;  // triplets
};

constexpr int64_t kFirstSegBlocks = 40;   // about 1.2 M stream samples
constexpr int64_t kSegBlocks = 128;        // about 3.9 M stream samples
constexpr int kDropEarly = 64;             // dropout triplets per field fetched with the other results

inline int64_t block_count(uint64_t n) {
    return n < (uint64_t)kBlock ? 0 : (int64_t)((n - kBlock) / kStride + 1);
}

}  // namespace detail
}  // namespace vhsd

using vhsd::detail::DevBuf;
using vhsd::detail::View;
using vhsd::detail::PipeKey;
using vhsd::detail::FieldRec;
using vhsd::FormatParams;
using vhsd::SyncParams;
using vhsd::FilterSpectra;
using vhsd::kBlock;
using vhsd::kStride;

struct vhsdecode_gb300_session {
    FormatParams fmt;
    SyncParams sp;
    FilterSpectra filt;
    double fs = 40e6;
    int precision = 0;
    int device = 0;
    uint64_t max_samples = 0;
    int64_t max_blocks = 0;
    int max_fields = 0;
    int lines = 0;       // processed lines per field
    int out_lines = 0;
    int outlen = 0;
    int num_sms = 0;
    int fft_plan = 0;    // radix plans of the fused demodulator (tuned per device)
    int decim = 1;       // 2: decode input passes the 2:1 half-band decimator
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[6] = {};
    // device data
    DevBuf<int16_t> rf;
    DevBuf<float> rf_f32;                    // float capture at the decode rate (decimated or float input)
    DevBuf<float> src_f32;                   // float source ahead of the decimator
    const float* in_f32 = nullptr;           // the current decode's float capture, if any
    DevBuf<float> v32, s32, e32;
    DevBuf<unsigned> sync_cond, sync_hold;   // pulse-scan bits of s32 (FP32 path)
    DevBuf<double> v64, s64, e64;
    DevBuf<float> rfv32;
    DevBuf<float2> vid32, syn32, sub32, tw_hi, tw_lo;
    DevBuf<double> rfv64;
    DevBuf<double2> vid64, syn64, sub64;
    DevBuf<float2> scratch;
    DevBuf<int> repair;
    DevBuf<double2> pwork;
    DevBuf<double> pdwork;
    DevBuf<float> pfwork;
    DevBuf<int> pflag;
    DevBuf<unsigned> pmask;
    DevBuf<int64_t> pblk;
    cudaGraphExec_t plain_graph = nullptr;
    const int16_t* graph_rf = nullptr;   // input pointers baked into plain_graph
    const float* graph_rf32 = nullptr;
    DevBuf<int64_t> pc_counts, pc_offsets, pc_events, pc_total;
    DevBuf<int64_t> pc_counts_alt, pc_offsets_alt;   // scan scratch of odd segments
    int64_t pc_capacity = 0;
    // the field stage's per-field inputs, carved from one device block that is
    // filled from its pinned host mirror (same layout) by one copy per decode
    DevBuf<unsigned char> field_in;
    unsigned char* h_field_in = nullptr;
    size_t field_in_bytes = 0;
    View<double> locs_in;
    View<uint8_t> fill_in;
    View<int64_t> span_start_d, span_len_d;
    View<int> first_line_d, start_line_d, end_line_d, line_off_d;
    DevBuf<double> locs_out;
    DevBuf<uint8_t> fill_out;
    // pinned landing area of the field stage's results: refined lines, dropout
    // counts and status, and the first kDropEarly dropout triplets of each field
    unsigned char* h_field_out = nullptr;
    DevBuf<unsigned char> hsync_work;
    // pipelined FP32 decode: per-segment pulse events, pinned host copies
    cudaStream_t aux_stream = nullptr;   // rescue fetches while the session stream is busy
    cudaStream_t copy_stream = nullptr;  // RF copies ahead of the demod
    cudaStream_t d2h_stream = nullptr;   // pulse events back to the host behind the demod
    cudaStream_t alt_stream = nullptr;   // odd segments, so a segment's straggler blocks overlap the next one
    cudaStream_t cap_stream = nullptr;   // origin of the pipeline graph capture
    cudaEvent_t alt_start = nullptr, alt_end = nullptr, copy_end = nullptr, d2h_end = nullptr;
    cudaEvent_t chroma_t[2] = {nullptr, nullptr};   // stage timing: the block stage's start and end
    int demod_clusters = 0;            // clusters of the pipelined demod launches (0: one per SM pair)
    cudaGraphExec_t pipe_exec = nullptr; // captured segment pipeline
    PipeKey pipe_key{};
    std::vector<cudaEvent_t> seg_done, seg_copied, seg_pulsed, seg_dem, seg_demod_end;
    int nseg_max = 0;
    int64_t seg_cap = 0;                 // pulse events per segment
    DevBuf<int64_t> seg_events, seg_total;
    DevBuf<unsigned> blk_counters;       // demod block claims, one counter per launch
    int64_t* h_events = nullptr;         // pinned [nseg_max * seg_cap]
    int64_t* h_totals = nullptr;         // pinned [nseg_max]
    int rescue_fetches = 0;
    int recoveries = 0;                  // field attempts that failed and were skipped past
    uint32_t launches = 0;               // kernels started by the current decode
    double enqueue_ms = 0.0;             // host time to queue the pipelined demod
    cudaStream_t field_stream = nullptr; // field batches, concurrent with later demod segments
    cudaEvent_t field_end = nullptr;
    cudaStream_t drop_stream = nullptr;  // a field batch's dropout chain, beside its hsync and TBC
    cudaEvent_t drop_fork = nullptr, drop_hsync = nullptr, drop_join = nullptr;
    bool stage_timing = false;           // VHSD_STAGE_TIMING set: per-stage kernel times to stderr
    unsigned long long* demod_cycles = nullptr;   // VHSD_DEMOD_TIMING set: fused-demod stage cycles
    cudaEvent_t stage_ev[4] = {};
    float stage_ms[3] = {};
    uint32_t segments = 0;
    DevBuf<int> hsync_misses;
    DevBuf<float> lut, lut_pair;
    DevBuf<float2> pw_ff;
    DevBuf<double> pw, level_work;
    DevBuf<unsigned char> tbc_consts;   // float-pair line plans of the fast TBC kernel
    DevBuf<uint16_t> tbc;
    DevBuf<int64_t> drop_range, drop_events;
    DevBuf<float> drop_mean, drop_partial;
    DevBuf<int> drop_counts, drop_out_count, drop_status;
    DevBuf<int32_t> drop_out;
    int drop_cap = 1024, drop_out_cap = 4096;
    int64_t span_len = 0;
    // colour-under chroma (allocated by the first decode that asks for it)
    bool chroma_alloc = false;
    bool want_chroma = false;            // the current decode renders chroma
    vhsd::ChromaDesign cd;
    DevBuf<float> c32;                   // stitched chroma stream
    DevBuf<float> c_scratch;             // block band-pass passes [max_blocks * (kBlock + 2 edge)]
    DevBuf<float> c_het, c_bsin, c_bcos; // field tables
    DevBuf<float> c_ana;                 // line-1 chroma TBC, probe windows
    DevBuf<float> c_field, c_up, c_fwd;  // output-line chroma TBC, up-converted / filtered, forward pass
    DevBuf<double> c_probe, c_probe_nrm, c_summary, locs_final;
    DevBuf<float2> c_advance;   // NTSC carrier advance per sample of a line: (cos, sin)
    DevBuf<float2> c_line_cs, c_line_scale_f;
    DevBuf<double> c_line_scale;
    DevBuf<int> c_flip, c_chosen, c_state, c_ones;   // c_state: rotation out, status
    DevBuf<uint16_t> chroma;             // uint16 chroma fields
    View<int> first_field_d, field_number_d, rot_in_d;
    int chroma_rot_start = 0, chroma_rot_end = 0;
    cudaEvent_t chroma_refined = nullptr;
    // the chroma block band-pass runs on its own stream beside the demod
    cudaStream_t chroma_stream = nullptr;
    cudaEvent_t chroma_go = nullptr, chroma_done = nullptr;
    bool chroma_pending = false;         // chroma blocks queued for this decode
    // host results
    std::vector<FieldRec> fields;
    int64_t last_blocks = 0;
    int last_repairs = 0;

    bool fp32() const { return precision == VHSDECODE_GB300_PRECISION_FP32_FUSED; }
};

namespace vhsd {
namespace detail {

// Decode options beyond the public flags: the server carries a stream's sync
// history from one window to the next and starts at its continuation point.
struct DecodeCarry {
    FieldState state;          // field parity / hsync history
    int64_t start = 0;         // stitched-stream index where the first field span is resolved
    int64_t next = 0;          // out: continuation point of the next field (stitched-stream index)
    bool no_graph = false;     // queue the pipeline directly (inputs change every call)
};

// One window of a batched decode (decode_batched): int16 host samples of a
// window for an FP32 session without decimation.
struct BatchWindow {
    vhsdecode_gb300_session* s;
    const int16_t* samples;
    uint64_t n;
    uint32_t max_fields;
    DecodeCarry* carry;
    vhsdecode_gb300_decode_result_v1* res;
};

// Device job table, block counter and staging of one batching thread.
struct BatchScratch {
    int cap = 0;
    FastDemodParams* d_jobs = nullptr;
    int64_t* d_start = nullptr;
    unsigned* d_counter = nullptr;
    FastDemodParams* h_jobs = nullptr;
    int64_t* h_start = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    ~BatchScratch();
    void init(int max_windows);
};

bool batchable(const vhsdecode_gb300_session* s);
// Demodulates the blocks of all `wins` in one persistent launch on `st`, then
// finishes each window on its own session (results as from decode_impl).
void decode_batched(std::vector<BatchWindow>& wins, BatchScratch& bs, cudaStream_t st);

void session_init(vhsdecode_gb300_session* s, const vhsdecode_gb300_session_config_v1& c);
void session_free(vhsdecode_gb300_session* s);
int32_t decode_impl(vhsdecode_gb300_session* s, const void* rf, uint64_t n, uint32_t max_fields,
                    uint32_t flags, vhsdecode_gb300_decode_result_v1* res,
                    const std::atomic<bool>* cancel = nullptr, DecodeCarry* carry = nullptr);

}  // namespace detail
}  // namespace vhsd
