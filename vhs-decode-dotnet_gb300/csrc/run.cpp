// Whole-run decode behind the reference's run() handoff, streamed in bounded
// windows.
//
// The reference's cuda-fast library pulls the capture through its read
// callback from a prefetch thread and decodes it in batches of fields with
// bounded memory, polling cancellation through a monotonic latch from both
// threads (src/VHSDecode.CudaFast.Native/src/vhsdecode_cuda_fast.cpp:68-91,
// 330-355; src/cancellation_latch.h; CMakeLists.txt:453-480).  Here:
//
// * a prefetch thread reads the capture in order, in chunks of kReadChunk
//   source samples (kFlacReadChunk bytes of a FLAC stream), at most
//   kPrefetchChunks ahead of the decode, and polls the cancel callback before
//   each read;
// * a watcher thread polls the cancel callback while the GPU works, so the
//   decode's field loop sees a cancellation within a field;
// * the capture is decoded in windows of a fixed number of grid steps
//   (983,040 decode samples = lcm(block stride 30,720, block length 32,768)).
//   Every window starts on that grid, counted from the start of the capture,
//   and resumes the previous window's field sequence (field parity, hsync
//   history and the continuation point of the next field), so each field is
//   decoded exactly once and bit-identically to one decode of the whole
//   capture: its span's blocks are the same blocks, with the same stream
//   indices relative to the block grid;
// * device and host memory are bounded by the window, whatever the capture's
//   length;
// * the .tbc, _chroma.tbc and .tbc.json files are written under temporary
//   names and renamed into place only when the run completes; a cancelled or
//   failed run leaves no output files.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/vhsdecode_gb300.h"
#include "flac.hpp"
#include "formats.hpp"
#include "kernels.h"
#include "session.hpp"

using namespace vhsd;
using namespace vhsd::detail;

namespace {

constexpr int64_t kGrid = 983040;              // decode samples: lcm(kStride, kBlock)
constexpr int64_t kDefaultWindowGrids = 40;    // 39.3 M decode samples (about 0.7 GB of device state)
constexpr int64_t kMinWindowGrids = 3;         // room for two fields and the continuation
constexpr size_t kReadChunk = (size_t)1 << 22; // source samples per read callback call
constexpr size_t kPrefetchChunks = 4;
constexpr size_t kFlacReadChunk = (size_t)1 << 27; // bytes per read callback call for FLAC input

// Window length in grid steps; VHSD_RUN_WINDOW_GRIDS overrides the default
// (tests use small windows to exercise many window joins on short captures).
int64_t window_grids() {
    const char* e = std::getenv("VHSD_RUN_WINDOW_GRIDS");
    int64_t g = e ? std::atoll(e) : kDefaultWindowGrids;
    return std::max<int64_t>(kMinWindowGrids, g > 0 ? g : kDefaultWindowGrids);
}

// Bytes per read of a FLAC stream; VHSD_RUN_FLAC_CHUNK overrides the default
// (tests use small chunks so that frames straddle chunk joins).
size_t flac_read_chunk() {
    const char* e = std::getenv("VHSD_RUN_FLAC_CHUNK");
    const long long v = e ? std::atoll(e) : 0;
    return v >= 4096 ? (size_t)v : kFlacReadChunk;
}

// Monotonic cancellation latch polled from the decode, watcher and prefetch
// threads (the reference's CancellationLatch).
struct Latch {
    const vhsdecode_gb300_config_v1* cfg;
    std::atomic<bool> requested{false};
    std::mutex poll_m;   // the callback is called from one thread at a time
    bool poll() {
        if (requested.load(std::memory_order_acquire)) return true;
        if (!cfg->cancel_callback) return false;
        std::lock_guard<std::mutex> lk(poll_m);
        if (cfg->cancel_callback(cfg->user_data) != 0) requested.store(true, std::memory_order_release);
        return requested.load(std::memory_order_acquire);
    }
};

// In-order reader of the capture on its own thread.
class Prefetch {
public:
    Prefetch(const vhsdecode_gb300_config_v1* cfg, size_t esz, size_t chunk, Latch& latch)
        : cfg_(cfg), esz_(esz), chunk_(chunk), latch_(latch), th_([this] { loop(); }) {}
    ~Prefetch() {
        {
            std::lock_guard<std::mutex> lk(m_);
            stop_ = true;
        }
        cv_.notify_all();
        th_.join();
    }
    // Appends the next chunk to `out`; false at the end of input (or on a
    // failure, reported by error()).
    bool next(std::vector<unsigned char>& out) {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [&] { return !q_.empty() || done_; });
        if (q_.empty()) return false;
        std::vector<unsigned char> c = std::move(q_.front());
        q_.pop_front();
        lk.unlock();
        cv_.notify_all();
        out.insert(out.end(), c.begin(), c.end());
        return true;
    }
    std::string error() {
        std::lock_guard<std::mutex> lk(m_);
        return err_;
    }

private:
    void loop() {
        uint64_t off = 0;
        const uint64_t total = cfg_->total_samples;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return stop_ || q_.size() < kPrefetchChunks; });
                if (stop_) break;
            }
            if (latch_.poll()) break;
            size_t ask = chunk_;
            if (total) {
                if (off >= total) break;
                ask = (size_t)std::min<uint64_t>(ask, total - off);
            }
            std::vector<unsigned char> c(ask * esz_);
            size_t got = cfg_->read_callback(cfg_->user_data, c.data(), off, ask);
            if (got > ask) {
                std::lock_guard<std::mutex> lk(m_);
                err_ = "read callback overran its buffer";
                break;
            }
            c.resize(got * esz_);
            off += got;
            if (got) {
                std::lock_guard<std::mutex> lk(m_);
                q_.push_back(std::move(c));
            }
            cv_.notify_all();
            if (got < ask) break;   // short read: end of input
        }
        std::lock_guard<std::mutex> lk(m_);
        done_ = true;
        cv_.notify_all();
    }

    const vhsdecode_gb300_config_v1* cfg_;
    size_t esz_, chunk_;
    Latch& latch_;
    std::mutex m_;
    std::condition_variable cv_;
    std::deque<std::vector<unsigned char>> q_;
    bool stop_ = false, done_ = false;
    std::string err_;
    std::thread th_;   // last: started after the members above exist
};

// Polls the cancel callback while the decode runs on the GPU.
class Watcher {
public:
    explicit Watcher(Latch& l) : latch_(l), th_([this] { loop(); }) {}
    ~Watcher() {
        {
            std::lock_guard<std::mutex> lk(m_);
            stop_ = true;
        }
        cv_.notify_all();
        th_.join();
    }

private:
    void loop() {
        std::unique_lock<std::mutex> lk(m_);
        while (!stop_) {
            lk.unlock();
            bool c = latch_.poll();
            lk.lock();
            if (c) break;
            cv_.wait_for(lk, std::chrono::milliseconds(2), [&] { return stop_; });
        }
    }
    Latch& latch_;
    std::mutex m_;
    std::condition_variable cv_;
    bool stop_ = false;
    std::thread th_;
};

struct FieldMeta {
    bool first_field;
    long long file_loc;          // decode-rate samples from the start of the capture
    std::vector<int32_t> drop;   // (field line, startx, endx) triplets
};

// Output files under temporary names, removed unless commit() renamed them.
struct Outputs {
    std::string tbc, chroma, json;
    FILE* ftbc = nullptr;
    FILE* fchroma = nullptr;
    bool committed = false;
    ~Outputs() {
        if (ftbc) std::fclose(ftbc);
        if (fchroma) std::fclose(fchroma);
        if (!committed) {
            std::remove((tbc + ".tmp").c_str());
            std::remove((chroma + ".tmp").c_str());
            std::remove((json + ".tmp").c_str());
        }
    }
    void open() {
        ftbc = std::fopen((tbc + ".tmp").c_str(), "wb");
        if (!ftbc) throw Failure(VHSDECODE_GB300_STATUS_OUTPUT_ERROR, "cannot open " + tbc + ".tmp");
        fchroma = std::fopen((chroma + ".tmp").c_str(), "wb");
        if (!fchroma) throw Failure(VHSDECODE_GB300_STATUS_OUTPUT_ERROR, "cannot open " + chroma + ".tmp");
    }
    void close_files() {
        int a = ftbc ? std::fclose(ftbc) : 0, b = fchroma ? std::fclose(fchroma) : 0;
        ftbc = fchroma = nullptr;
        if (a || b) throw Failure(VHSDECODE_GB300_STATUS_OUTPUT_ERROR, "cannot write " + tbc);
    }
    void commit() {
        for (const std::string* p : {&tbc, &chroma, &json})
            if (std::rename((*p + ".tmp").c_str(), p->c_str()) != 0)
                throw Failure(VHSDECODE_GB300_STATUS_OUTPUT_ERROR, "cannot rename " + *p + ".tmp");
        committed = true;
    }
};

// The cuda-fast backend's metadata file (src/VHSDecode.CudaFast.Native/src/tbc_writer.cpp:209-310):
// the same keys and number formats.  Levels carry the writer's default 10 %
// adjust; the burst window comes from the format's colorBurstUS, the active
// video window is the writer's fixed PAL/NTSC one, and fileLoc is in
// decode-rate samples for the managed rebase.
void write_json(const std::string& path, const FormatParams& fm, int outlen, int out_lines,
                const std::vector<FieldMeta>& fields) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw Failure(VHSDECODE_GB300_STATUS_OUTPUT_ERROR, "cannot open " + path);
    const double scale = output_scale(fm), rate = fm.outfreq_mhz * 1e6;
    const double level_adjust = 0.1;
    const double black16 = ((0.0 - fm.vsync_ire) * scale + fm.output_zero) * (1.0 - level_adjust);
    const double white16 = ((100.0 - fm.vsync_ire) * scale + fm.output_zero) * (1.0 + level_adjust);
    const int burst_start = (int)(fm.burst_start_us * 1e-6 * rate + 0.5);
    const int burst_end = (int)(fm.burst_end_us * 1e-6 * rate + 0.5);
    const int active_start = fm.pal ? 185 : 134, active_end = fm.pal ? 1107 : 894;
    std::fprintf(f, "{\n  \"videoParameters\": {\n");
    std::fprintf(f, "    \"system\": \"%s\",\n", fm.pal ? "PAL" : "NTSC");
    std::fprintf(f, "    \"isSubcarrierLocked\": false,\n");
    std::fprintf(f, "    \"isSourcePal\": %s,\n", fm.pal ? "true" : "false");
    std::fprintf(f, "    \"numberOfSequentialFields\": %zu,\n", fields.size());
    std::fprintf(f, "    \"black16bIre\": %.1f,\n", black16);
    std::fprintf(f, "    \"white16bIre\": %.1f,\n", white16);
    std::fprintf(f, "    \"sampleRate\": %.0f,\n", rate);
    std::fprintf(f, "    \"fieldWidth\": %d,\n", outlen);
    std::fprintf(f, "    \"fieldHeight\": %d,\n", out_lines);
    std::fprintf(f, "    \"colourBurstStart\": %d,\n", burst_start);
    std::fprintf(f, "    \"colourBurstEnd\": %d,\n", burst_end);
    std::fprintf(f, "    \"activeVideoStart\": %d,\n", active_start);
    std::fprintf(f, "    \"activeVideoEnd\": %d,\n", active_end);
    std::fprintf(f, "    \"tapeFormat\": \"%s\",\n", fm.custom_luma_table ? "SVHS" : "VHS");
    std::fprintf(f, "    \"isMapped\": false\n  },\n  \"fields\": [\n");
    for (size_t i = 0; i < fields.size(); i++) {
        const FieldMeta& r = fields[i];
        std::fprintf(f, "    {\n      \"isFirstField\": %s,\n      \"seqNo\": %zu,\n      \"fileLoc\": %lld,\n",
                     r.first_field ? "true" : "false", i + 1, r.file_loc);
        const size_t nd = r.drop.size() / 3;
        std::fprintf(f, "      \"dropOuts\": {\n        \"fieldLine\": [");
        for (size_t k = 0; k < nd; k++) std::fprintf(f, "%s%d", k ? ", " : "", r.drop[3 * k]);
        std::fprintf(f, "],\n        \"startx\": [");
        for (size_t k = 0; k < nd; k++) std::fprintf(f, "%s%d", k ? ", " : "", r.drop[3 * k + 1]);
        std::fprintf(f, "],\n        \"endx\": [");
        for (size_t k = 0; k < nd; k++) std::fprintf(f, "%s%d", k ? ", " : "", r.drop[3 * k + 2]);
        std::fprintf(f, "]\n      }\n    }%s\n", i + 1 < fields.size() ? "," : "");
    }
    std::fprintf(f, "  ]\n}\n");
    if (std::fclose(f) != 0) throw Failure(VHSDECODE_GB300_STATUS_OUTPUT_ERROR, "cannot write " + path);
}

// RAII owner of the run's session.
struct SessionHolder {
    vhsdecode_gb300_session* s = nullptr;
    ~SessionHolder() {
        if (s) {
            // a cancelled or failed decode may leave copies and kernels queued
            // on the session's streams: let them finish before freeing buffers
            cudaSetDevice(s->device);
            cudaDeviceSynchronize();
            session_free(s);
            delete s;
        }
    }
};

struct PinnedHost {
    unsigned char* p = nullptr;
    ~PinnedHost() {
        if (p) cudaFreeHost(p);
    }
};

bool file_exists(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (f) {
        std::fclose(f);
        return true;
    }
    return false;
}

}  // namespace

extern "C" {

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_run(
    const vhsdecode_gb300_config_v1* config, vhsdecode_gb300_result_v1* result) {
    return guard([&]() -> int32_t {
        if (!config || !result) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
        if (config->struct_size != sizeof(vhsdecode_gb300_config_v1) &&
            config->struct_size != sizeof(vhsdecode_gb300_config_v2))
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "config struct_size mismatch");
        const bool v2 = config->struct_size == sizeof(vhsdecode_gb300_config_v2);
        const uint32_t tape_format = v2 ? reinterpret_cast<const vhsdecode_gb300_config_v2*>(config)->tape_format
                                        : (uint32_t)VHSDECODE_GB300_TAPE_FORMAT_VHS;
        const uint32_t run_flags = v2 ? reinterpret_cast<const vhsdecode_gb300_config_v2*>(config)->decode_flags : 0u;
        if (run_flags & ~(uint32_t)VHSDECODE_GB300_DECODE_CHROMA)
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "unknown decode_flags bit");
        const bool with_chroma = (run_flags & VHSDECODE_GB300_DECODE_CHROMA) != 0;
        if (result->struct_size != sizeof(vhsdecode_gb300_result_v1))
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "result struct_size mismatch");
        if (!config->read_callback) return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "read_callback is null");
        if (!config->output_base_utf8 || !config->output_base_utf8[0])
            return fail(VHSDECODE_GB300_STATUS_NULL_POINTER, "output_base_utf8 is null");
        if (config->input_sample_format > VHSDECODE_GB300_INPUT_FLAC)
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "unknown input_sample_format");
        // vhsdecode_cuda_fast.cpp:255-275: factor 1 or 2; the source runs at
        // factor x sample_rate_mhz
        const uint32_t factor = config->device_decimation_factor;
        if (factor != 1 && factor != 2)
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "device_decimation_factor must be 1 or 2");
        if (factor == 2 && !(config->sample_rate_mhz >= 10.0 && config->sample_rate_mhz <= 50.0))
            return fail(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT,
                        "device_decimation_factor 2 needs a decode rate of 10..50 MHz");
        const bool f32_in = config->input_sample_format == VHSDECODE_GB300_INPUT_FLOAT32;
        // FLAC input: the callback reads bytes of the stream, decoded on the
        // device into int16 samples as they arrive
        const bool flac_in = config->input_sample_format == VHSDECODE_GB300_INPUT_FLAC;
        const size_t esz = f32_in ? sizeof(float) : sizeof(int16_t);
        const auto t0 = std::chrono::steady_clock::now();
        Outputs out;
        const std::string base = config->output_base_utf8;
        out.tbc = base + ".tbc";
        out.json = base + ".tbc.json";
        out.chroma = base + "_chroma.tbc";
        if (!config->overwrite && (file_exists(out.tbc) || file_exists(out.json) || file_exists(out.chroma)))
            return fail(VHSDECODE_GB300_STATUS_OUTPUT_ERROR, "output exists and overwrite is off");
        Latch latch;
        latch.cfg = config;
        if (latch.poll()) return fail(VHSDECODE_GB300_STATUS_CANCELLED, "decode cancelled before startup");

        // window geometry in source samples (decode samples x factor)
        const int64_t grid_src = kGrid * (int64_t)factor;
        const int64_t win_src = window_grids() * grid_src;
        const uint64_t total = flac_in ? 0 : config->total_samples;   // FLAC: total_samples counts bytes
        const uint64_t cap_src = total ? std::min<uint64_t>((uint64_t)win_src, total) : (uint64_t)win_src;
        if (cap_src / factor < (uint64_t)kBlock && total)
            return fail(VHSDECODE_GB300_STATUS_INPUT_ERROR, "input shorter than one block");

        // FLAC bytes come in larger chunks (about 180 M samples each): a frame
        // decodes serially on one thread, so a launch needs tens of thousands
        // of frames to keep the SMs busy
        Prefetch pre(config, flac_in ? 1 : esz, flac_in ? flac_read_chunk() : kReadChunk, latch);
        std::vector<unsigned char> buf;   // source samples [buf_off, buf_off + buf.size() / esz)
        uint64_t buf_off = 0;
        bool eof = false;
        FlacStreamDecoder flac;
        std::vector<unsigned char> fbytes;   // FLAC bytes not decoded yet
        std::vector<int16_t> pcm;
        bool flac_started = false;
        if (flac_in) flac.init(config->device_id);
        auto fill_to = [&](uint64_t end) {
            while (!eof && buf_off + buf.size() / esz < end) {
                if (!flac_in) {
                    if (!pre.next(buf)) eof = true;
                    continue;
                }
                const bool more = pre.next(fbytes);
                if (!flac_started) {
                    FlacInfo fi{};
                    if (fbytes.size() < 4096 && more) continue;   // the metadata first
                    if (flac_stream_info(fbytes.data(), fbytes.size(), fi) != VHSDECODE_GB300_STATUS_OK) {
                        if (more) continue;
                        throw Failure(VHSDECODE_GB300_STATUS_INPUT_ERROR, g_last_error);
                    }
                    if (fi.channels != 1 || fi.bits_per_sample != 16)
                        throw Failure(VHSDECODE_GB300_STATUS_INPUT_ERROR, "FLAC stream is not 16-bit mono");
                    fbytes.erase(fbytes.begin(), fbytes.begin() + (std::ptrdiff_t)fi.first_frame);
                    flac_started = true;
                }
                pcm.clear();
                const size_t used = flac.decode(fbytes.data(), fbytes.size(), !more, pcm);
                fbytes.erase(fbytes.begin(), fbytes.begin() + (std::ptrdiff_t)used);
                const unsigned char* pb = reinterpret_cast<const unsigned char*>(pcm.data());
                buf.insert(buf.end(), pb, pb + pcm.size() * sizeof(int16_t));
                if (!more) eof = true;
            }
        };
        fill_to((uint64_t)win_src);
        if (latch.requested.load()) return fail(VHSDECODE_GB300_STATUS_CANCELLED, "decode cancelled");
        if (!pre.error().empty()) return fail(VHSDECODE_GB300_STATUS_INPUT_ERROR, pre.error());
        if (buf.size() / esz / factor < (size_t)kBlock)
            return fail(VHSDECODE_GB300_STATUS_INPUT_ERROR, "input shorter than one block");

        vhsdecode_gb300_session_config_v1 sc{};
        sc.struct_size = sizeof(sc);
        sc.profile = config->profile;
        sc.tape_speed = config->tape_speed;
        sc.tape_format = tape_format;
        sc.device_id = config->device_id;
        sc.sample_rate_mhz = config->sample_rate_mhz;
        sc.max_samples = std::min<uint64_t>((uint64_t)win_src, buf.size() / esz);
        sc.precision = VHSDECODE_GB300_PRECISION_FP32_FUSED;
        sc.decimation = factor;
        PinnedHost win, tbc_host, chroma_host;   // outlive the session, whose teardown waits for the device
        SessionHolder h;
        h.s = new vhsdecode_gb300_session();
        session_init(h.s, sc);
        vhsdecode_gb300_session* s = h.s;
        const size_t per = (size_t)s->out_lines * s->outlen;
        ck(cudaMallocHost((void**)&win.p, (size_t)sc.max_samples * esz), "pinned window");
        ck(cudaMallocHost((void**)&tbc_host.p, (size_t)s->max_fields * per * sizeof(uint16_t)), "pinned tbc");
        if (with_chroma)
            ck(cudaMallocHost((void**)&chroma_host.p, (size_t)s->max_fields * per * sizeof(uint16_t)),
               "pinned chroma");
        out.open();
        const std::vector<uint16_t> neutral(per, (uint16_t)32767);
        std::vector<FieldMeta> meta;
        Watcher watch(latch);

        DecodeCarry carry;
        carry.no_graph = true;   // every window copies new samples into the same pinned buffer
        bool cont = false;
        uint64_t next_abs = 0;   // source position of the next field (continuation)
        uint64_t ws = 0;         // window start, source samples, a multiple of grid_src
        for (;;) {
            if (latch.poll()) throw Failure(VHSDECODE_GB300_STATUS_CANCELLED, "decode cancelled");
            fill_to(ws + (uint64_t)win_src);
            if (!pre.error().empty()) throw Failure(VHSDECODE_GB300_STATUS_INPUT_ERROR, pre.error());
            if (latch.requested.load()) throw Failure(VHSDECODE_GB300_STATUS_CANCELLED, "decode cancelled");
            // drop what lies before the window
            if (ws > buf_off) {
                size_t drop = (size_t)std::min<uint64_t>(ws - buf_off, buf.size() / esz);
                buf.erase(buf.begin(), buf.begin() + drop * esz);
                buf_off += drop;
            }
            const uint64_t avail = buf_off + buf.size() / esz;
            const uint64_t we = std::min<uint64_t>(ws + (uint64_t)win_src, avail);
            const uint64_t n = we > ws ? we - ws : 0;
            if (n / factor < (uint64_t)kBlock) break;
            std::memcpy(win.p, buf.data(), (size_t)n * esz);
            carry.start = cont ? (int64_t)((next_abs - ws) / factor) : 0;
            uint32_t left = 0;
            if (config->maximum_output_fields) {
                if (meta.size() >= config->maximum_output_fields) break;
                left = config->maximum_output_fields - (uint32_t)meta.size();
            }
            vhsdecode_gb300_decode_result_v1 dr{};
            dr.struct_size = sizeof(dr);
            const uint32_t dflags = (f32_in ? VHSDECODE_GB300_DECODE_FLOAT_INPUT : 0u) |
                                    (with_chroma ? VHSDECODE_GB300_DECODE_CHROMA : 0u);
            decode_impl(s, win.p, n, left, dflags, &dr, &latch.requested, &carry);
            const size_t nf = s->fields.size();
            if (nf) {
                ck(cudaMemcpy(tbc_host.p, s->tbc.p, nf * per * sizeof(uint16_t), cudaMemcpyDeviceToHost),
                   "d2h tbc");
                if (std::fwrite(tbc_host.p, sizeof(uint16_t), nf * per, out.ftbc) != nf * per)
                    throw Failure(VHSDECODE_GB300_STATUS_OUTPUT_ERROR, "cannot write " + out.tbc);
                if (with_chroma) {
                    ck(cudaMemcpy(chroma_host.p, s->chroma.p, nf * per * sizeof(uint16_t), cudaMemcpyDeviceToHost),
                       "d2h chroma");
                    if (std::fwrite(chroma_host.p, sizeof(uint16_t), nf * per, out.fchroma) != nf * per)
                        throw Failure(VHSDECODE_GB300_STATUS_OUTPUT_ERROR, "cannot write " + out.chroma);
                }
                for (size_t k = 0; k < nf; k++) {
                    // Without chroma, as cuda-fast: neutral chroma (zero chroma +
                    // 32767, VhsChromaDecoder.ChromaToU16,
                    // Core/Decode/VhsChromaDecoder.cs:455-500) in the luma
                    // geometry, which the managed finalisation truncates with the
                    // luma file (Core/Dsp/CudaFast/CudaFastDecodeRunner.cs:345,427).
                    if (!with_chroma && std::fwrite(neutral.data(), sizeof(uint16_t), per, out.fchroma) != per)
                        throw Failure(VHSDECODE_GB300_STATUS_OUTPUT_ERROR, "cannot write " + out.chroma);
                    const FieldRec& r = s->fields[k];
                    FieldMeta m;
                    m.first_field = r.sync.first_field;
                    m.file_loc = (long long)std::floor(r.span_start + r.sync.line0 + kCut) +
                                 (long long)(ws / factor);
                    m.drop = r.drop;
                    meta.push_back(std::move(m));
                }
            }
            const bool at_end = eof && we == avail;
            if (dr.stop_reason == 1 && config->maximum_output_fields &&
                meta.size() >= config->maximum_output_fields)
                break;
            if (at_end) break;
            // resume from the continuation point of the next field: the next
            // window starts on the grid at or below two blocks before it
            next_abs = ws + (uint64_t)factor * (uint64_t)std::max<int64_t>(0, carry.next);
            cont = true;
            const int64_t back = std::max<int64_t>(0, carry.next - 2 * kBlock);
            uint64_t ws_next = ws + (uint64_t)grid_src * (uint64_t)(back / kGrid);
            if (ws_next <= ws) ws_next = ws + (uint64_t)grid_src;   // no field fits: move on a step
            if (next_abs < ws_next) cont = false;
            // the previous field's read location in the next window's stream
            // (the VHS field number counts reads that move forward)
            carry.state.vhs_loc -= (int64_t)((ws_next - ws) / factor);
            ws = ws_next;
        }
        if (latch.poll()) throw Failure(VHSDECODE_GB300_STATUS_CANCELLED, "decode cancelled");
        if (!pre.error().empty()) throw Failure(VHSDECODE_GB300_STATUS_INPUT_ERROR, pre.error());
        out.close_files();
        write_json(out.json + ".tmp", s->fmt, s->outlen, s->out_lines, meta);
        out.commit();
        result->fields_written = (uint32_t)meta.size();
        result->output_line_length = (uint32_t)s->outlen;
        result->output_field_lines = (uint32_t)s->out_lines;
        result->elapsed_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return VHSDECODE_GB300_STATUS_OK;
    });
}

}  // extern "C"
